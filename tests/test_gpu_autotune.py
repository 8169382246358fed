"""Launch-shape autotuning (bie_ctx_set_autotune) of the mixed assembly (K2),
the double-float assembly (K9) and the mixed matrix-free product (K3).

* Every shape on the tuner's axes gives the same matrices within the
  tolerance of its arithmetic: forced element slicings (levels 0..3),
  records per shared-memory chunk (1, default, 5, 64) and 128 / 256 threads
  per block for K2 against the oracle at 1e-6 (mixed), K9 at 1e-12 (FP64
  grade), K3 products against the dense oracle product at 1e-6.
* The tuned shape is recorded per (kernel, target count), lies on the axes,
  and the tuning call and the calls after it stay within tolerance.
"""
from __future__ import annotations

import numpy as np
import pytest

import biegpu
import oracle
from biegpu import mesh as bm

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def p2():
    mesh = bm.icosphere(6, geometry="quadratic")
    return mesh, oracle.assemble(mesh, 4.0, n=2, m=2)


def test_autotuned_mixed_assembly(p2):
    mesh, (F, G, Cv) = p2
    ctx = biegpu.Context(mesh, n=2, m=2, device=0)
    ctx.set_autotune(True)
    for _ in range(2):   # the first call tunes, the second uses the kept shape
        Fg, Gg, Cg = ctx.assemble(4.0, precision="mixed")
        assert rel(Fg, F) <= 1e-6 and rel(Gg, G) <= 1e-6 and rel(Cg, Cv) <= 1e-6
    lv, ch, tpb = ctx.shape("mixed_assembly")
    assert 0 <= lv < 8 and 1 <= ch <= 64 and tpb in (128, 256)
    X = mesh.sources[:, :77] * 1.3
    Fo, Go, _ = oracle.assemble(mesh, 4.0, targets=X, n=2, m=2, cOn=False)
    for _ in range(2):
        Fg, Gg, _ = ctx.assemble(4.0, targets=X, cOn=False, precision="mixed")
        assert rel(Fg, Fo) <= 1e-6 and rel(Gg, Go) <= 1e-6
    assert ctx.shape("mixed_assembly", M=77) is not None


@pytest.mark.parametrize("level,chunk,tpb", [(0, 0, 128), (1, 1, 256), (2, 64, 128), (3, 0, 256), (2, 5, 256)])
def test_forced_mixed_assembly_shapes(p2, level, chunk, tpb):
    mesh, (F, G, Cv) = p2
    ctx = biegpu.Context(mesh, n=2, m=2, device=0)
    ctx.force_shape("mixed_assembly", level, chunk, tpb)
    assert ctx.shape("mixed_assembly")[0] == level
    Fg, Gg, Cg = ctx.assemble(4.0, precision="mixed")
    assert rel(Fg, F) <= 1e-6 and rel(Gg, G) <= 1e-6 and rel(Cg, Cv) <= 1e-6
    ctx.force_shape("mixed_assembly", -1)
    assert ctx.shape("mixed_assembly") is None


@pytest.mark.parametrize("level,chunk", [(0, 0), (2, 1), (3, 64)])
def test_forced_df64_assembly_shapes(p2, level, chunk):
    mesh, (F, G, Cv) = p2
    ctx = biegpu.Context(mesh, n=2, m=2, device=0)
    ctx.force_shape("df64_assembly", level, chunk)
    Fg, Gg, Cg = ctx.assemble(4.0, precision="df64")
    assert rel(Fg, F) <= 1e-12 and rel(Gg, G) <= 1e-12 and rel(Cg, Cv) <= 1e-12


def test_autotuned_df64_and_product(p2):
    mesh, (F, G, Cv) = p2
    ctx = biegpu.Context(mesh, n=2, m=2, device=0)
    ctx.set_autotune(True)
    for _ in range(2):
        Fg, Gg, Cg = ctx.assemble(4.0, precision="df64")
        assert rel(Fg, F) <= 1e-12 and rel(Gg, G) <= 1e-12
    assert ctx.shape("df64_assembly") is not None
    rng = np.random.default_rng(2)
    x = rng.normal(size=mesh.n_sources) + 1j * rng.normal(size=mesh.n_sources)
    op = biegpu.GPUFOperator(mesh, 4.0, precision="mixed")   # the mesh's shared context
    op.ctx.set_autotune(True)
    try:
        for _ in range(2):
            assert rel(op @ x, F @ x) <= 1e-6
        assert op.ctx.shape("mixed_product") is not None
        for level, chunk in [(0, 1), (3, 64)]:
            op.ctx.force_shape("mixed_product", level, chunk)
            assert rel(op @ x, F @ x) <= 1e-6
    finally:
        op.ctx.force_shape("mixed_product", -1)
        op.ctx.set_autotune(False)

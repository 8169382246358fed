"""GPU parity of the dense FP64 assembly (libbiegpu via the C ABI) against the
CPU oracle (restatement of assemble_parallel!).  Tolerance: relative Frobenius
error <= 1e-12 for F, G and C (FP64 arithmetic, different summation order)."""
from __future__ import annotations

import numpy as np
import pytest

import biegpu
import oracle
from biegpu import mesh as bm

pytestmark = pytest.mark.gpu
TOL = 1e-12


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def check(mesh, k, n, m, targets=None, **flags):
    F, G, C = biegpu.assemble_parallel(mesh, k, targets, n=n, m=m, **flags)
    Fo, Go, Co = oracle.assemble(mesh, k, targets=targets, n=n, m=m, **flags)
    for a, b, name in [(F, Fo, "F"), (G, Go, "G"), (C, Co, "C")]:
        if b is None:
            assert a is None
            continue
        assert a.shape == b.shape, name
        assert np.all(np.isfinite(a)), name
        assert rel(a, b) <= TOL, f"{name}: {rel(a, b):.3e}"


@pytest.mark.parametrize("n,m", [(2, 2), (4, 4), (3, 2)])
def test_linear_sphere(n, m):
    check(bm.icosphere(4), 2 * np.pi * 200 / 343, n, m)


@pytest.mark.parametrize("physics", ["geometry", "linear"])
def test_quadratic_sphere(physics):
    check(bm.icosphere(3, geometry="quadratic", physics=physics), 3.0, 2, 2)
    check(bm.icosphere(3, geometry="quadratic", physics=physics), 1.0, 4, 4)


def test_complex_wavenumber():
    check(bm.icosphere(3, geometry="quadratic"), 2.0 + 1.5j, 2, 2)
    check(bm.icosphere(4), 1.0 + 0.5j, 2, 2)


def test_field_points():
    z = np.linspace(0.1, 0.9, 20)
    X = np.vstack([0 * z, 0.05 + 0 * z, z])
    check(bm.icosphere(4), 1.0, 2, 2, targets=X)
    check(bm.icosphere(3, geometry="quadratic"), 1.0, 2, 2, targets=X)


@pytest.mark.parametrize("flags", [dict(gOn=False), dict(fOn=False, cOn=False), dict(fOn=False, gOn=False)])
def test_flag_subsets(flags):
    check(bm.icosphere(3), 2.5, 2, 2, **flags)


def test_ellipsoid_and_reuse():
    mesh = bm.ellipsoid(5)
    for k in (0.5, 4.0):
        check(mesh, k, 2, 2)


def test_single_element():
    # ragged edge case: one triangle, three collocation nodes, field points
    P = np.array([[0.0, 1.0, 0.0], [0.0, 0.0, 1.0], [0.0, 0.0, 0.0]])
    T = np.array([[1], [2], [3]])
    mesh = bm._finish(P, T, "linear", "geometry")
    check(mesh, 1.0, 2, 2)
    check(mesh, 1.0, 2, 2, targets=np.array([[0.2], [0.3], [0.5]]))


def test_config1_rows_full_size():
    """Pulsating-sphere workload (icosphere f=32: 10242 nodes, 20480 triangles,
    n = m = 2): the full GPU matrices, checked row-wise against the oracle on 64
    sampled rows, plus the partition-of-unity identity sum_j F(k=0)[i,j] = C[i]."""
    mesh = bm.icosphere(32)
    k = 2 * np.pi * 200 / 343
    ctx = biegpu.get_context(mesh, n=2, m=2)
    F, G, C = ctx.assemble(k)
    rows = np.random.default_rng(7).choice(mesh.n_sources, 64, replace=False)
    Fo, Go, Co = oracle.assemble(mesh, k, targets=mesh.sources[:, rows], n=2, m=2)
    assert rel(F[rows], Fo) <= TOL and rel(G[rows], Go) <= TOL and rel(C[rows], Co) <= TOL
    F0, _, C0 = ctx.assemble(0.0, gOn=False)
    assert np.max(np.abs(F0.sum(axis=1) - C0)) < 1e-10
    del F, G, F0


def test_device_entry_point_matches_host():
    torch = pytest.importorskip("torch")
    mesh = bm.icosphere(5)
    ctx = biegpu.get_context(mesh, n=2, m=2)
    F, G, C = ctx.assemble(3.0)
    N = mesh.n_sources
    dF = torch.empty((N, N), dtype=torch.complex128, device="cuda")
    dG = torch.empty_like(dF)
    dC = torch.empty(N, dtype=torch.complex128, device="cuda")
    ctx.assemble_device(3.0, dF, dG, dC)
    torch.cuda.synchronize()
    # torch row-major (N, N) over column-major memory: transpose back
    assert np.array_equal(dF.cpu().numpy().T, F) or rel(dF.cpu().numpy().T, F) < 1e-15
    assert rel(dG.cpu().numpy().T, G) < 1e-15
    assert rel(dC.cpu().numpy(), C) < 1e-15


def test_invalid_target_count_rejected():
    mesh = bm.icosphere(2)
    ctx = biegpu.get_context(mesh, n=2, m=2)
    with pytest.raises(biegpu.BIEError):
        ctx.assemble(1.0, targets=np.zeros((3, 0)))
    with pytest.raises(biegpu.BIEError):
        ctx.assemble(float("nan"))

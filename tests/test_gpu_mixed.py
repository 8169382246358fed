"""Mixed-precision assembly (BIE_PREC_MIXED): FP32 regular pairs, FP64 near
pairs and nearest-node ties.  Checked against the FP64 oracle; the stated
tolerance is a relative Frobenius error <= 1e-6 for F, G and C."""
from __future__ import annotations

import numpy as np
import pytest

import biegpu
import oracle
from biegpu import mesh as bm

pytestmark = pytest.mark.gpu
TOL_MIXED = 1e-6


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def check(mesh, k, n=2, m=2, targets=None, tol=TOL_MIXED, **flags):
    F, G, C = biegpu.assemble_parallel(mesh, k, targets, n=n, m=m, precision="mixed", **flags)
    Fo, Go, Co = oracle.assemble(mesh, k, targets=targets, n=n, m=m, **flags)
    errs = {}
    for a, b, name in [(F, Fo, "F"), (G, Go, "G"), (C, Co, "C")]:
        if b is None:
            assert a is None
            continue
        assert np.all(np.isfinite(a)), name
        errs[name] = rel(a, b)
        assert errs[name] <= tol, f"{name}: {errs[name]:.3e}"
    return errs


@pytest.mark.parametrize("k", [1.0, 3.66, 10.0])
def test_mixed_linear_sphere(k):
    check(bm.icosphere(8), k)


@pytest.mark.parametrize("k", [1.0, 5.0, 10.0])
def test_mixed_quadratic_sphere(k):
    check(bm.icosphere(5, geometry="quadratic"), k)


def test_mixed_quadratic_linear_physics():
    check(bm.icosphere(5, geometry="quadratic", physics="linear"), 4.0)


def test_mixed_complex_wavenumber():
    check(bm.icosphere(6), 3.0 + 2.0j)
    check(bm.icosphere(4, geometry="quadratic"), 2.0 + 0.7j)


def test_mixed_ellipsoid_n4():
    check(bm.ellipsoid(6), 6.0, n=4, m=4)


def test_mixed_field_points():
    rng = np.random.default_rng(3)
    X = rng.normal(size=(3, 50))
    X *= (rng.uniform(0.2, 3.0, 50) / np.linalg.norm(X, axis=0))[None, :]
    check(bm.icosphere(6), 2.0, targets=X)


def test_mixed_flags():
    check(bm.icosphere(5), 2.0, gOn=False)
    check(bm.icosphere(5), 2.0, fOn=False, cOn=False)


@pytest.mark.parametrize("precision,tol", [("mixed", TOL_MIXED), ("fp64", 1e-12), ("df64", 1e-12)])
def test_rows_full_size_rigid_sphere(precision, tol):
    """Bench workload (f=17 P2 sphere, 11562 nodes) at ka = 10: 48 sampled rows
    of the full GPU matrices against the oracle, for the mixed path (1e-6),
    the plain FP64 path and the double-float FP64-grade path (1e-12)."""
    mesh = bm.icosphere(17, geometry="quadratic")
    ctx = biegpu.get_context(mesh, n=2, m=2)
    F, G, C = ctx.assemble(10.0, precision=precision)
    rows = np.random.default_rng(11).choice(mesh.n_sources, 48, replace=False)
    Fo, Go, Co = oracle.assemble(mesh, 10.0, targets=mesh.sources[:, rows], n=2, m=2)
    assert rel(F[rows], Fo) <= tol
    assert rel(G[rows], Go) <= tol
    assert rel(C[rows], Co) <= tol

"""Edge cases of the GPU path: the smallest closed mesh, a single target, row
counts that are not multiples of the 128-row tiles, an open surface with an odd
number of nodes (the one-row-per-thread complex64 product), multi-RHS products
with 1 and 130 right-hand sides, far targets, and argument errors reported by
the device entry points.  Tolerances as elsewhere: FP64 <= 1e-12, mixed <= 1e-6."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import biegpu
import oracle
from biegpu import _capi
from biegpu import mesh as bm

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def plate(nx, ny, h=0.1):
    """Open curved plate z = 2 ((x - c)^2 + (y - c)^2), nx x ny cells, two
    triangles per cell (curved, so that F is not zero)."""
    xs, ys = np.meshgrid(np.arange(nx + 1) * h, np.arange(ny + 1) * h, indexing="xy")
    cx, cy = 0.5 * nx * h, 0.5 * ny * h
    P = np.vstack([xs.ravel(), ys.ravel(), 2.0 * ((xs.ravel() - cx) ** 2 + (ys.ravel() - cy) ** 2)])
    T = []
    for j in range(ny):
        for i in range(nx):
            a = j * (nx + 1) + i
            T.append([a, a + 1, a + nx + 2])
            T.append([a, a + nx + 2, a + nx + 1])
    T = np.array(T, dtype=np.int64).T + 1
    return bm._finish(P, T, "linear", "geometry")


def test_smallest_icosphere_both_precisions():
    mesh = bm.icosphere(1)           # 12 nodes, 20 triangles
    assert mesh.n_sources == 12
    F, G, Cv = oracle.assemble(mesh, 1.7, n=2, m=2)
    for prec, tol in (("fp64", 1e-12), ("mixed", 1e-6)):
        Fg, Gg, Cg = biegpu.assemble_parallel(mesh, 1.7, mesh.sources, n=2, m=2, precision=prec)
        assert rel(Fg, F) <= tol and rel(Gg, G) <= tol and rel(Cg, Cv) <= tol


@pytest.mark.parametrize("M", [1, 127, 129, 300])
def test_ragged_target_counts(M):
    mesh = bm.icosphere(4, geometry="quadratic")
    rng = np.random.default_rng(M)
    X = rng.normal(size=(3, M))
    X *= (1.5 + rng.random(M)) / np.linalg.norm(X, axis=0)
    F, G, _ = oracle.assemble(mesh, 2.2, targets=X, n=2, m=2, cOn=False)
    for prec, tol in (("fp64", 1e-12), ("mixed", 1e-6)):
        Fg, Gg, _ = biegpu.assemble_parallel(mesh, 2.2, X, n=2, m=2, cOn=False, precision=prec)
        assert rel(Fg, F) <= tol and rel(Gg, G) <= tol


def test_far_targets():
    mesh = bm.icosphere(3)
    X = np.array([[1e3, 0.0, -2e4], [0.0, 5e2, 0.0], [0.0, 0.0, 3e3]])
    F, G, _ = oracle.assemble(mesh, 0.9, targets=X, n=2, m=2, cOn=False)
    Fg, Gg, _ = biegpu.assemble_parallel(mesh, 0.9, X, n=2, m=2, cOn=False, precision="fp64")
    assert rel(Fg, F) <= 1e-12 and rel(Gg, G) <= 1e-12


def test_odd_node_count_complex64_solve():
    """Curved open plate with 5 x 5 = 25 nodes: the complex64 operator product
    takes the one-row-per-thread kernels (fast and exact forms) inside refined
    GMRES."""
    mesh = plate(4, 4)
    assert mesh.n_sources % 2 == 1
    k = 3.0
    F, _, Cv = oracle.assemble(mesh, k, n=2, m=2, gOn=False)
    A = F + np.diag(1.0 - Cv)
    b = np.exp(1j * k * mesh.sources[0])
    ctx = biegpu.get_context(mesh, n=2, m=2)
    x, res = biegpu.gmres(F + biegpu.Diagonal(1.0 - Cv), b, ctx=ctx, refine=True, log=True, reltol=1e-12)
    assert res.converged
    assert rel(x, np.linalg.solve(A, b)) <= 1e-9


@pytest.mark.parametrize("R", [1, 130])
def test_multi_rhs_sizes(R):
    mesh = bm.icosphere(3, geometry="quadratic")
    N = mesh.n_sources
    ctx = biegpu.Context(mesh, n=2, m=2, device=0)
    rng = np.random.default_rng(R)
    X = np.asfortranarray(rng.normal(size=(N, R)) + 1j * rng.normal(size=(N, R)))
    F, _, _ = oracle.assemble(mesh, 2.0, n=2, m=2, gOn=False, cOn=False)
    Y = np.empty_like(X)
    _capi.check(_capi.lib().bie_matvec_multi(ctx.handle, 2.0, 0.0, R, X.ctypes.data, None, Y.ctypes.data, None,
                                             _capi.BIE_PREC_FP16_SPLIT, 0))
    assert rel(Y, F @ X) <= 1e-5


def test_device_entry_point_argument_errors():
    mesh = bm.icosphere(2)
    ctx = biegpu.Context(mesh, n=2, m=2, device=0)
    L = _capi.lib()
    x = np.zeros(mesh.n_sources, dtype=np.complex128)
    y = np.empty_like(x)
    # NaN wavenumber, unknown precision, missing output, zero right-hand sides
    assert L.bie_matvec(ctx.handle, float("nan"), 0.0, None, 0, x.ctypes.data, None, y.ctypes.data, None,
                        0) == _capi.BIE_ERR_INVALID
    assert L.bie_matvec(ctx.handle, 1.0, 0.0, None, 0, x.ctypes.data, None, y.ctypes.data, None,
                        7) == _capi.BIE_ERR_INVALID
    assert L.bie_matvec(ctx.handle, 1.0, 0.0, None, 0, x.ctypes.data, None, None, None,
                        0) == _capi.BIE_ERR_INVALID
    assert L.bie_matvec_multi(ctx.handle, 1.0, 0.0, 0, x.ctypes.data, None, y.ctypes.data, None, 4,
                              0) == _capi.BIE_ERR_INVALID
    assert L.bie_taylor_assemble(ctx.handle, 1.0, 0.0, None, 0, 1, -1, y.ctypes.data, None,
                                 None) == _capi.BIE_ERR_INVALID
    h = C.c_void_p()
    assert L.bie_fastop_create(ctx.handle, 1.0, 0.0, 3, 3, 1, 0.2, 1, C.byref(h)) == _capi.BIE_ERR_INVALID
    # a 5-point triangle rule does not exist in the table: unsupported
    assert L.bie_fastop_create(ctx.handle, 1.0, 0.0, 1, 5, 1, 0.2, 1, C.byref(h)) == _capi.BIE_ERR_UNSUPPORTED
    assert len(L.bie_last_error()) > 0
    # the context stays usable after the errors
    F, _, _ = oracle.assemble(mesh, 1.0, n=2, m=2, gOn=False, cOn=False)
    Fg, _, _ = biegpu.assemble_parallel(mesh, 1.0, mesh.sources, n=2, m=2, gOn=False, cOn=False)
    assert rel(Fg, F) <= 1e-12

"""Many right-hand sides in one solve (bie_solve_multi with host matrices,
bie_solve_multi_device with device ones): lockstep GMRES
with tcgen05 16-bit products of the mixed-precision F, refined with exact
residuals of the complex64 matrix, against the oracle's dense FP64 solve of
(F + Diagonal(1 - C)) X = B (test/3d/assembly_test.jl:37-38) column by column.

Tolerances: the relative residual with respect to the complex64 matrix meets
reltol (sqrt(eps)); each column's solution is within 1e-6 of the FP64 one (the
mixed assembly's ~1e-7 error times the system's sensitivity, as for the
mixed sweep)."""
from __future__ import annotations

import numpy as np
import pytest

import biegpu
import oracle
from biegpu import mesh as bm

pytestmark = pytest.mark.gpu


def _rhs(N, R, seed):
    rng = np.random.default_rng(seed)
    return rng.normal(size=(N, R)) + 1j * rng.normal(size=(N, R))


@pytest.mark.parametrize("geometry,f,k,R,prec", [("quadratic", 5, 3.0, 40, "fp16_split"),
                                                  ("linear", 10, 2.0 + 0.4j, 130, "bf16_split"),
                                                  ("linear", 8, 6.0, 3, "fp16")])
def test_multi_rhs_solve_against_oracle(geometry, f, k, R, prec):
    mesh = bm.icosphere(f, geometry=geometry)
    N = mesh.n_sources
    B = _rhs(N, R, f + R)
    X, info = biegpu.solve_multi(mesh, k, B, precision=prec)
    assert info["converged"] == R
    assert info["max_relres"] <= np.sqrt(np.finfo(float).eps)
    assert info["passes"] >= 1 and info["tensor_products"] >= 1
    F, _, C = oracle.assemble(mesh, k, n=2, m=2)
    Xr = np.linalg.solve(F + np.diag(1.0 - C), B)
    err = np.linalg.norm(X - Xr, axis=0) / np.linalg.norm(Xr, axis=0)
    assert err.max() <= 1e-6, f"worst column {err.max():.3e}"


def test_multi_rhs_solve_device_tensors_and_one_column():
    torch = pytest.importorskip("torch")
    mesh = bm.icosphere(6)
    B = _rhs(mesh.n_sources, 1, 3)
    X, info = biegpu.solve_multi(mesh, 1.5, torch.as_tensor(B, device="cuda:0"))
    assert isinstance(X, torch.Tensor) and X.is_cuda and info["converged"] == 1
    F, _, C = oracle.assemble(mesh, 1.5, n=2, m=2)
    xr = np.linalg.solve(F + np.diag(1.0 - C), B[:, 0])
    assert np.linalg.norm(X.cpu().numpy()[:, 0] - xr) / np.linalg.norm(xr) <= 1e-6


def test_multi_rhs_solve_host_and_device_entries_agree():
    """The host-buffer entry copies B in and X out around the same solve: the
    same X as the device entry to the solve's tolerance (not bit for bit: the
    FP64 near-pair corrections reach the complex64 matrix through atomic
    additions, whose order varies between assemblies), and argument errors
    reported."""
    torch = pytest.importorskip("torch")
    from biegpu import _capi
    mesh = bm.icosphere(7, geometry="quadratic")
    B = _rhs(mesh.n_sources, 9, 17)
    ctx = biegpu.Context(mesh, n=2, m=2)
    Xh, ih = biegpu.solve_multi(mesh, 2.5 + 0.1j, B, ctx=ctx)
    Xd, idv = biegpu.solve_multi(mesh, 2.5 + 0.1j, torch.as_tensor(B, device="cuda:0"), ctx=ctx)
    assert isinstance(Xh, np.ndarray) and Xh.shape == B.shape
    Xd = Xd.cpu().numpy()
    assert np.linalg.norm(Xh - Xd) / np.linalg.norm(Xd) <= 1e-6
    assert ih["converged"] == idv["converged"] == 9 and ih["passes"] == idv["passes"]
    with pytest.raises(ValueError):
        biegpu.solve_multi(mesh, 1.0, B[:-1], ctx=ctx)
    st = _capi.lib().bie_solve_multi(ctx.handle, 1.0, 0.0, 0, B.ctypes.data, B.ctypes.data, None, None)
    assert st == _capi.BIE_ERR_INVALID
    ctx.close()

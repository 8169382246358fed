"""Multi-right-hand-side products on the tensor cores (K4).

* bie_lowp_gemm_device, the tcgen05 GEMM building block: bit-exact on
  integer-valued operands (every value and partial sum is exact in FP16/BF16
  and FP32, so any layout or descriptor error shows), and within the stated
  error of each 16-bit form on Gaussian operands.
* bie_matvec_multi_device: F X and G V against the dense FP64 matrices for real
  and complex wavenumbers; relative Frobenius tolerances FP16 3e-3, BF16 2e-2,
  FP16_SPLIT 1e-5, BF16_SPLIT 3e-5 (the split forms are limited by the FP32
  accumulation in tensor memory, up to 4096 K terms per accumulator: measured
  2-6e-6 at N = 1000-4000); the FP64 form equals the single-column products.
* The 40962-node quadratic sphere with 256 right-hand sides and three
  wavenumbers (acoustic plus two boundary-layer wavenumbers), checked column
  by column against the FP64 matrix-free product (FP16_SPLIT, measured
  1.5e-5, tolerance 5e-5).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import biegpu
from biegpu import _capi
from biegpu import mesh as bm

pytestmark = pytest.mark.gpu

GEMM_TOL = {"fp16": 2e-3, "bf16": 1.5e-2, "fp16_split": 2e-5, "bf16_split": 2e-4}
MULTI_TOL = {"fp16": 3e-3, "bf16": 2e-2, "fp16_split": 1e-5, "bf16_split": 3e-5}


def _torch():
    return pytest.importorskip("torch")


def _gemm(ctx, prec, A, B):
    torch = _torch()
    M, K = A.shape
    N = B.shape[0]
    Cm = torch.empty((M, N), dtype=torch.float64, device=A.device)
    _capi.check(_capi.lib().bie_lowp_gemm_device(ctx.handle, _capi.PRECISION[prec], M, N, K, A.data_ptr(),
                                                 B.data_ptr(), Cm.data_ptr()))
    return Cm


@pytest.fixture(scope="module")
def small_ctx():
    return biegpu.Context(bm.icosphere(3, geometry="quadratic"), n=2, m=2, device=0)


@pytest.mark.parametrize("prec", ["fp16", "bf16", "fp16_split", "bf16_split"])
@pytest.mark.parametrize("M,N,K", [(128, 256, 64), (300, 520, 1000), (1000, 64, 4100)])
def test_gemm_integer_exact(small_ctx, prec, M, N, K):
    torch = _torch()
    g = torch.Generator(device="cpu").manual_seed(M + N + K)
    # |a|, |b| <= 15 with per-row maxima spread over powers of two: exact in
    # BF16 (8 significant bits) after any power-of-two row scale; every partial
    # sum < 2^24 is exact in FP32
    A = torch.randint(-15, 16, (M, K), generator=g).double()
    B = torch.randint(-15, 16, (N, K), generator=g).double()
    A *= torch.pow(2.0, torch.randint(-6, 7, (M, 1), generator=g).double())
    B *= torch.pow(2.0, torch.randint(-6, 7, (N, 1), generator=g).double())
    ref = A @ B.T
    dev = torch.device("cuda:0")
    Cm = _gemm(small_ctx, prec, A.float().to(dev), B.float().to(dev)).cpu()
    assert torch.equal(Cm, ref), float((Cm - ref).abs().max())


@pytest.mark.parametrize("prec", ["fp16", "fp16_split"])
def test_gemm_wait_gives_up_and_context_recovers(prec):
    """The GEMM's bounded waits: with the stall switch its MMA issuer waits on a
    barrier that nothing completes, with a budget of 2e6 clock cycles (~1 ms).
    The wait runs out, the CTAs wait for their own copies, free their tensor
    memory and exit, and the call returns BIE_ERR_TIMEOUT.  The same context
    then gives bit-exact results again (integer-valued operands)."""
    torch = _torch()
    ctx = biegpu.Context(bm.icosphere(3, geometry="quadratic"), n=2, m=2, device=0)
    L = _capi.lib()
    M, N, K = 300, 520, 1000
    g = torch.Generator(device="cpu").manual_seed(5)
    A = torch.randint(-15, 16, (M, K), generator=g).double()
    B = torch.randint(-15, 16, (N, K), generator=g).double()
    ref = A @ B.T
    dev = torch.device("cuda:0")
    Ad, Bd = A.float().to(dev), B.float().to(dev)
    assert torch.equal(_gemm(ctx, prec, Ad, Bd).cpu(), ref)
    _capi.check(L.bie_ctx_set_gemm_wait(ctx.handle, 2_000_000, 1))
    Cm = torch.empty((M, N), dtype=torch.float64, device=dev)
    st = L.bie_lowp_gemm_device(ctx.handle, _capi.PRECISION[prec], M, N, K, Ad.data_ptr(), Bd.data_ptr(),
                                Cm.data_ptr())
    assert st == _capi.BIE_ERR_TIMEOUT
    assert "gave up" in L.bie_last_error().decode()
    _capi.check(L.bie_ctx_set_gemm_wait(ctx.handle, -1, 0))
    for _ in range(2):
        assert torch.equal(_gemm(ctx, prec, Ad, Bd).cpu(), ref)
    ctx.close()


@pytest.mark.parametrize("prec", ["fp16", "bf16", "fp16_split", "bf16_split"])
def test_gemm_gaussian(small_ctx, prec):
    torch = _torch()
    g = torch.Generator(device="cpu").manual_seed(7)
    A = torch.randn(700, 3000, generator=g, dtype=torch.float64)
    B = torch.randn(300, 3000, generator=g, dtype=torch.float64)
    A[::7] *= 1e-3   # rows of very different scale
    ref = A.float().double() @ B.float().double().T
    Cm = _gemm(small_ctx, prec, A.float().cuda(), B.float().cuda()).cpu()
    err = float((Cm - ref).norm() / ref.norm())
    assert err <= GEMM_TOL[prec], err
    # row-relative: the small rows are as accurate as the large ones
    rs = torch.arange(0, 700, 7)
    err_small = float((Cm[rs] - ref[rs]).norm() / ref[rs].norm())
    assert err_small <= 2 * GEMM_TOL[prec], err_small


def _dense(ctx, k, torch):
    N = ctx.n_sources
    dev = torch.device("cuda:0")
    Ft = torch.empty((N, N), dtype=torch.complex128, device=dev)
    Gt = torch.empty_like(Ft)
    ctx.assemble_device(k, F=Ft, G=Gt, precision="fp64")
    torch.cuda.synchronize()
    return Ft.T, Gt.T   # M x N views


def _multi(ctx, k, X, V, prec, scratch=0):
    """YF = F X, YG = G V through bie_matvec_multi_device (column-major N x R)."""
    torch = _torch()
    k = complex(k)
    Z = X if X is not None else V
    N, R = Z.shape
    for T in (X, V):
        assert T is None or (T.stride(0) == 1 and T.stride(1) == N)
    YF = torch.empty((R, N), dtype=torch.complex128, device=Z.device).T if X is not None else None
    YG = torch.empty((R, N), dtype=torch.complex128, device=Z.device).T if V is not None else None
    torch.cuda.synchronize()
    _capi.check(_capi.lib().bie_matvec_multi_device(
        ctx.handle, k.real, k.imag, R, _capi.ptr(X), _capi.ptr(V), _capi.ptr(YF), _capi.ptr(YG),
        _capi.PRECISION[prec], int(scratch)))
    torch.cuda.synchronize()
    return YF, YG


def _colmajor(Z, torch):
    """(N, R) complex128 device tensor laid out column-major."""
    return Z.T.contiguous().T


def _rel(a, b):
    return float((a - b).abs().pow(2).sum().sqrt() / b.abs().pow(2).sum().sqrt())


@pytest.mark.parametrize("geometry,f", [("quadratic", 5), ("linear", 12)])
@pytest.mark.parametrize("k", [3.0, 6.0 + 6.0j])
def test_multi_rhs_against_dense(geometry, f, k):
    torch = _torch()
    mesh = bm.icosphere(f, geometry=geometry)
    ctx = biegpu.Context(mesh, n=2, m=2, device=0)
    N = mesh.n_sources
    R = 37
    rng = np.random.default_rng(3)
    dev = torch.device("cuda:0")
    X = _colmajor(torch.as_tensor(rng.normal(size=(N, R)) + 1j * rng.normal(size=(N, R)), device=dev), torch)
    V = _colmajor(torch.as_tensor(rng.normal(size=(N, R)) + 1j * rng.normal(size=(N, R)), device=dev), torch)
    F, G = _dense(ctx, k, torch)
    refF, refG = F @ X, G @ V
    for prec, tol in MULTI_TOL.items():
        YF, YG = _multi(ctx, k, X, V, prec)
        eF, eG = _rel(YF, refF), _rel(YG, refG)
        assert eF <= tol and eG <= tol, (prec, eF, eG)
    # a scratch cap forces several strips; the result changes only by rounding
    # (other element slicing in the strip assembly, other K splits)
    YF2, YG2 = _multi(ctx, k, X, V, "fp16_split", scratch=N * 8 * 200)
    YF1, YG1 = _multi(ctx, k, X, V, "fp16_split")
    assert _rel(YF2, YF1) <= 1e-5 and _rel(YG2, YG1) <= 1e-5
    # FP64 form == single-column products
    YF, YG = _multi(ctx, k, X[:, :3], V[:, :3], "fp64")
    assert _rel(YF, refF[:, :3]) <= 1e-12 and _rel(YG, refG[:, :3]) <= 1e-12


def test_multi_rhs_only_one_product():
    torch = _torch()
    mesh = bm.icosphere(4, geometry="quadratic")
    ctx = biegpu.Context(mesh, n=2, m=2, device=0)
    N = mesh.n_sources
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(4)
    X = _colmajor(torch.as_tensor(rng.normal(size=(N, 5)) + 0j, device=dev), torch)
    F, G = _dense(ctx, 2.0, torch)
    YF, YG = _multi(ctx, 2.0, X, None, "fp16_split")
    assert YG is None and _rel(YF, F @ X) <= MULTI_TOL["fp16_split"]
    _, YG = _multi(ctx, 2.0, None, X, "fp16_split")
    assert _rel(YG, G @ X) <= MULTI_TOL["fp16_split"]


def _lossy_wavenumbers(freq=100.0):
    from biegpu.lossy import boundary_layer_wavenumbers
    return boundary_layer_wavenumbers(freq)


def test_multi_rhs_lossy_sphere_40962():
    """Quadratic sphere, 40962 nodes, 256 seeded right-hand sides, three
    wavenumbers.  The boundary-layer kernels e^{ikr} decay as e^{-Im k r}, so
    their matrices are numerically banded; the dense tensor-core product still
    runs over every entry.  Four columns are checked against the FP64
    matrix-free product."""
    torch = _torch()
    mesh = bm.icosphere(32, geometry="quadratic")
    assert mesh.n_sources == 40962
    ctx = biegpu.Context(mesh, n=2, m=2, device=0)
    N, R = mesh.n_sources, 256
    dev = torch.device("cuda:0")
    g = torch.Generator(device="cpu").manual_seed(5)
    X = _colmajor(torch.complex(torch.randn(N, R, generator=g, dtype=torch.float64),
                                torch.randn(N, R, generator=g, dtype=torch.float64)).to(dev), torch)
    cols = [0, 77, 128, 255]
    L = _capi.lib()
    for k in _lossy_wavenumbers():
        k = complex(k)
        YF, YG = _multi(ctx, k, X, X, "fp16_split")
        for c in cols:
            x = X[:, c].contiguous()
            yF = torch.empty_like(x)
            yG = torch.empty_like(x)
            _capi.check(L.bie_matvec_device(ctx.handle, k.real, k.imag, None, 0, x.data_ptr(), x.data_ptr(),
                                            yF.data_ptr(), yG.data_ptr(), _capi.BIE_PREC_FP64))
            torch.cuda.synchronize()
            eF, eG = _rel(YF[:, c], yF), _rel(YG[:, c], yG)
            assert eF <= 5e-5 and eG <= 5e-5, (k, c, eF, eG)


def test_operator_matrix_product():
    """GPUFOperator @ X with a host matrix X (the reference's `Ff * X`)."""
    import oracle
    from biegpu import GPUFOperator, GPUGOperator
    mesh = bm.icosphere(4)
    k = 2.5
    F, G, _ = oracle.assemble(mesh, k, n=2, m=2, cOn=False)
    rng = np.random.default_rng(9)
    X = rng.normal(size=(mesh.n_sources, 8)) + 1j * rng.normal(size=(mesh.n_sources, 8))
    Y = GPUFOperator(mesh, k) @ X
    assert isinstance(Y, np.ndarray) and Y.shape == X.shape
    assert np.linalg.norm(Y - F @ X) / np.linalg.norm(F @ X) <= MULTI_TOL["fp16_split"]
    Yg = GPUGOperator(mesh, k, multi_precision=None, precision="fp64") @ X
    assert np.linalg.norm(Yg - G @ X) / np.linalg.norm(G @ X) <= 1e-12


def test_multi_rhs_host_entry_point():
    """bie_matvec_multi (host buffers) equals the device entry point."""
    import oracle
    mesh = bm.icosphere(4, geometry="quadratic")
    ctx = biegpu.Context(mesh, n=2, m=2, device=0)
    N, R = mesh.n_sources, 11
    k = 3.0 + 0.5j
    F, G, _ = oracle.assemble(mesh, k, n=2, m=2, cOn=False)
    rng = np.random.default_rng(12)
    X = np.asfortranarray(rng.normal(size=(N, R)) + 1j * rng.normal(size=(N, R)))
    V = np.asfortranarray(rng.normal(size=(N, R)) + 1j * rng.normal(size=(N, R)))
    YF = np.empty((N, R), dtype=np.complex128, order="F")
    YG = np.empty_like(YF)
    for prec, tol in (("fp16_split", MULTI_TOL["fp16_split"]), ("fp64", 1e-12)):
        _capi.check(_capi.lib().bie_matvec_multi(ctx.handle, k.real, k.imag, R, X.ctypes.data, V.ctypes.data,
                                                 YF.ctypes.data, YG.ctypes.data, _capi.PRECISION[prec], 0))
        assert np.linalg.norm(YF - F @ X) / np.linalg.norm(F @ X) <= tol
        assert np.linalg.norm(YG - G @ V) / np.linalg.norm(G @ V) <= tol

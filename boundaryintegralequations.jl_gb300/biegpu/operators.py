"""Matrix-free BEM operators and GMRES on the GPU.

Mirrors the LinearMaps-based operator API of the reference:

* ``GPUFOperator(mesh, k)`` / ``GPUGOperator(mesh, k)`` play the role of
  ``FMMFOperator`` / ``FMMGOperator`` (src/3d/fast_multipole_method.jl:
  220-318, 374-488): ``size`` is (N, N) and ``A @ x`` applies the operator
  without storing it.  Here the products are the exact collocation matrices
  of ``assemble_parallel!`` recomputed on the fly (no FMM approximation, no
  separate near-field correction).
* The operator algebra used with ``gmres`` in the reference examples is
  supported: ``Diagonal(1 - C) - Ff`` (examples/3d_pulsating_sphere.jl:39,46),
  ``Ff + 0.5 * I`` (examples/3d_rigid_sphere.jl:53), ``Fp + Diagonal(1 - Cp)``
  for a dense matrix (test/3d/assembly_test.jl:37).
* ``gmres(A, b; restart, maxiter, reltol, abstol)`` follows
  IterativeSolvers.gmres (v0.9) defaults and runs entirely on the GPU.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _capi
from .assembly import get_context
from .mesh import Mesh3d


def _torch():
    import torch
    return torch


def _is_torch(a) -> bool:
    return hasattr(a, "data_ptr") and hasattr(a, "is_cuda")


class Diagonal:
    """Diagonal matrix (complex vector); the analogue of LinearAlgebra.Diagonal."""

    __array_ufunc__ = None   # make numpy defer `ndarray + Diagonal` to __radd__

    def __init__(self, d):
        self.d = d

    def __sub__(self, other):
        return _as_affine(other).scaled(-1.0).plus_diag(self.d)

    def __rsub__(self, other):
        return _as_affine(other).plus_diag(-np.asarray(self.d))

    def __add__(self, other):
        return _as_affine(other).plus_diag(self.d)

    __radd__ = __add__


class UniformScaling:
    """lambda * I"""

    __array_ufunc__ = None

    def __init__(self, lam: complex = 1.0):
        self.lam = complex(lam)

    def __mul__(self, s):
        return UniformScaling(self.lam * complex(s))

    __rmul__ = __mul__


I = UniformScaling(1.0)  # noqa: E741


class _Affine:
    """s * K + diag(d): K a matrix-free F (GPUFOperator) or a dense matrix."""

    __array_ufunc__ = None

    def __init__(self, base, scale: complex = 1.0, diag=None):
        self.base = base
        self.scale = complex(scale)
        self.diag = diag

    @property
    def shape(self):
        return self.base.shape

    def scaled(self, s):
        d = None if self.diag is None else self.diag * s
        return _Affine(self.base, self.scale * s, d)

    def plus_diag(self, d):
        n = self.shape[0]
        if isinstance(d, UniformScaling):
            dv = np.full(n, d.lam, dtype=np.complex128)
        else:
            dv = d
        if self.diag is None:
            return _Affine(self.base, self.scale, dv)
        return _Affine(self.base, self.scale, self.diag + dv)

    def __add__(self, other):
        if isinstance(other, (UniformScaling, Diagonal)):
            return self.plus_diag(other if isinstance(other, UniformScaling) else other.d)
        raise TypeError("only diagonal shifts are supported")

    def __sub__(self, other):
        if isinstance(other, UniformScaling):
            return self.plus_diag(UniformScaling(-other.lam))
        if isinstance(other, Diagonal):
            return self.plus_diag(-other.d)
        raise TypeError("only diagonal shifts are supported")

    def __neg__(self):
        return self.scaled(-1.0)

    def __matmul__(self, x):
        y = self.base @ x
        y = y * self.scale
        if self.diag is not None:
            d = self.diag
            if _is_torch(y) and not _is_torch(d):
                d = _torch().as_tensor(np.asarray(d), device=y.device)
            y = y + d * x
        return y


def _as_affine(a):
    if isinstance(a, _Affine):
        return a
    return _Affine(a)


class _MatrixFreeOperator:
    which = "F"

    def __init__(self, mesh: Mesh3d, k, n: int = 2, m: int = 2, precision: str = "mixed",
                 device: int = 0, multi_precision: str | None = "fp16_split"):
        self.mesh = mesh
        self.k = complex(k)
        self.precision = precision
        # arithmetic of products with a matrix of right-hand sides: a 16-bit
        # tensor-core form ("fp16", "bf16", "fp16_split", "bf16_split") or None
        # for one `precision` product per column
        self.multi_precision = multi_precision
        self.ctx = get_context(mesh, n=n, m=m, device=device)
        N = mesh.n_sources
        self.shape = (N, N)
        self.dtype = np.complex128

    @property
    def size(self):
        return self.shape

    def _apply(self, x, targets=None):
        L = _capi.lib()
        prec = _capi.PRECISION[self.precision]
        if _is_torch(x):
            torch = _torch()
            M = self.shape[0] if targets is None else int(targets.shape[-1])
            y = torch.empty(M, dtype=torch.complex128, device=x.device)
            xs = x.contiguous()
            args = (xs.data_ptr(), None, y.data_ptr(), None) if self.which == "F" else \
                   (None, xs.data_ptr(), None, y.data_ptr())
            t = None if targets is None else targets.data_ptr()
            _capi.check(L.bie_matvec_device(self.ctx.handle, self.k.real, self.k.imag, t,
                                            M if targets is not None else 0, *args, prec))
            torch.cuda.current_stream().wait_stream(torch.cuda.ExternalStream(self.ctx.stream()))
            torch.cuda.synchronize()
            return y
        xs = np.ascontiguousarray(x, dtype=np.complex128)
        if targets is not None:
            t = np.asfortranarray(targets, dtype=np.float64)
            M = t.shape[1]
        else:
            t, M = None, self.shape[0]
        y = np.empty(M, dtype=np.complex128)
        args = (xs.ctypes.data, None, y.ctypes.data, None) if self.which == "F" else \
               (None, xs.ctypes.data, None, y.ctypes.data)
        _capi.check(L.bie_matvec(self.ctx.handle, self.k.real, self.k.imag, _capi.ptr(t), M, *args, prec))
        return y

    def _apply_multi(self, X):
        """Y = K X for an N x R matrix (bie_matvec_multi_device): the matrix form
        of `_unsafe_mul!(Y, A, X::AbstractMatrix)` (src/3d/fast_multipole_method.jl:
        249-287, 427-471)."""
        torch = _torch()
        on_device = _is_torch(X) and X.is_cuda
        dev = X.device if on_device else torch.device(f"cuda:{self.ctx.device}")
        Xd = torch.as_tensor(X, dtype=torch.complex128, device=dev) if not _is_torch(X) else \
            X.to(device=dev, dtype=torch.complex128)
        N, R = Xd.shape
        Xd = Xd.T.contiguous().T   # column-major
        Y = torch.empty((R, N), dtype=torch.complex128, device=dev).T
        prec = self.multi_precision or self.precision
        args = (Xd.data_ptr(), None, Y.data_ptr(), None) if self.which == "F" else \
               (None, Xd.data_ptr(), None, Y.data_ptr())
        torch.cuda.synchronize(dev)
        _capi.check(_capi.lib().bie_matvec_multi_device(self.ctx.handle, self.k.real, self.k.imag, R, *args,
                                                        _capi.PRECISION[prec], 0))
        torch.cuda.synchronize(dev)
        return Y if on_device else Y.cpu().numpy()

    def __matmul__(self, x):
        x = np.asarray(x) if not _is_torch(x) else x
        if x.ndim == 2:
            return self._apply_multi(x)
        return self._apply(x)

    def evaluate_targets(self, x, targets):
        """Operator applied at new target points (evaluate_targets,
        src/3d/fast_multipole_method.jl:326-344, 497-519)."""
        return self._apply(x, targets=targets)

    # operator algebra
    def __neg__(self):
        return _Affine(self, -1.0)

    def __mul__(self, s):
        return _Affine(self, complex(s))

    __rmul__ = __mul__

    def __add__(self, other):
        return _Affine(self) + other

    def __sub__(self, other):
        return _Affine(self) - other


class GPUFOperator(_MatrixFreeOperator):
    """Matrix-free double-layer operator F (FMMFOperator replacement)."""
    which = "F"


class GPUGOperator(_MatrixFreeOperator):
    """Matrix-free single-layer operator G (FMMGOperator replacement)."""
    which = "G"


class _FastOperator:
    """The algorithm of FMMFOperator / FMMGOperator (src/3d/fast_multipole_method.jl:
    163-194, 306-324, 473-490) on the GPU (bie_fastop_*): far field with the
    n_gauss-point Gauss rule on every element summed exactly (the reference
    uses FMM3D to `tol`, accepted here and unused) plus the near-field
    correction (accurate adaptive rules with `offset` minus the Gauss-rule
    part, depth-1/2 pattern).  Same constructor as the reference."""
    which = "F"

    def __init__(self, mesh: Mesh3d, k, tol: float = 1e-6, n_gauss: int = 3, nearfield: bool = True,
                 offset: float = 0.2, depth: int = 1, precision: str = "mixed", device: int = 0):
        self.mesh = mesh
        self.k = complex(k)
        self.tol = tol
        self.precision = precision
        self.ctx = get_context(mesh, n=2, m=2, device=device)
        N = mesh.n_sources
        self.shape = (N, N)
        self.dtype = np.complex128
        h = C.c_void_p()
        which = _capi.BIE_F if self.which == "F" else _capi.BIE_G
        _capi.check(_capi.lib().bie_fastop_create(self.ctx.handle, self.k.real, self.k.imag, which, int(n_gauss),
                                                  1 if nearfield else 0, float(offset), int(depth), C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _capi.lib().bie_fastop_destroy(h)
            self._h = None

    @property
    def size(self):
        return self.shape

    def _apply(self, x):
        xs = np.ascontiguousarray(x, dtype=np.complex128)
        y = np.empty(self.shape[0], dtype=np.complex128)
        _capi.check(_capi.lib().bie_fastop_apply(self._h, xs.ctypes.data, y.ctypes.data,
                                                 _capi.PRECISION[self.precision]))
        return y

    def __matmul__(self, x):
        x = np.asarray(x)
        if x.ndim == 2:
            return np.stack([self._apply(x[:, j]) for j in range(x.shape[1])], axis=1)
        return self._apply(x)

    def evaluate_targets(self, x, targets):
        """Far-field sum at other points, no near-field correction (evaluate_targets,
        src/3d/fast_multipole_method.jl:326-344, 497-519)."""
        xs = np.ascontiguousarray(x, dtype=np.complex128)
        t = np.asfortranarray(targets, dtype=np.float64)
        y = np.empty(t.shape[1], dtype=np.complex128)
        _capi.check(_capi.lib().bie_fastop_evaluate_targets(self._h, t.ctypes.data, t.shape[1], xs.ctypes.data,
                                                            y.ctypes.data, _capi.PRECISION[self.precision]))
        return y

    def __neg__(self):
        return _Affine(self, -1.0)

    def __mul__(self, s):
        return _Affine(self, complex(s))

    __rmul__ = __mul__

    def __add__(self, other):
        return _Affine(self) + other

    def __sub__(self, other):
        return _Affine(self) - other


class FMMFOperator(_FastOperator):
    """Double-layer fast operator (the reference's FMMFOperator algorithm)."""
    which = "F"


class FMMGOperator(_FastOperator):
    """Single-layer fast operator (the reference's FMMGOperator algorithm)."""
    which = "G"


class GmresResult:
    def __init__(self, x, info: _capi.GmresInfo):
        self.x = x
        self.iterations = info.iterations
        self.restarts = info.restarts
        self.refinements = info.refinements
        self.converged = bool(info.converged)
        self.matvecs = info.matvecs
        self.residual_norm = info.residual_norm
        self.rhs_norm = info.rhs_norm

    @property
    def relres(self):
        return self.residual_norm / self.rhs_norm if self.rhs_norm else 0.0


def _device_complex(a, device):
    torch = _torch()
    if _is_torch(a):
        return a.to(device=device, dtype=torch.complex128).contiguous()
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.complex128), device=device)


def gmres(A, b, restart: int | None = None, maxiter: int | None = None,
          reltol: float = math.sqrt(np.finfo(np.float64).eps), abstol: float = 0.0,
          precision: str = "fp64", refine: bool = False, A32=None, log: bool = False,
          ctx=None, device: int = 0, x0=None):
    """GPU GMRES for ``A x = b`` (IterativeSolvers.gmres semantics and defaults).

    ``A`` is a dense matrix (numpy or CUDA tensor, column-major N x N as
    returned by ``assemble_parallel``), an affine combination of one
    (``Fp + Diagonal(1 - Cp)``), or an affine combination of a
    ``GPUFOperator``.  ``precision`` selects the operator arithmetic;
    ``refine=True`` runs mixed inner iterations (on ``A32``, a complex64 copy
    of a dense matrix, or the mixed matrix-free operator) with an FP64 outer
    residual.  Host (numpy) inputs go through ``bie_gmres`` (the library
    copies them to the device and x back); CUDA tensors through
    ``bie_gmres_device``.  Returns x (same array kind as b), or
    (x, GmresResult) when ``log`` is true.
    """
    aff = _as_affine(A)
    base = aff.base
    op = _capi.Operator()
    op.scale_re, op.scale_im = aff.scale.real, aff.scale.imag
    keep = []
    dense = not isinstance(base, (_MatrixFreeOperator, _FastOperator))
    on_host = not any(_is_torch(t) for t in (b, x0, aff.diag, A32, base if dense else None))
    if isinstance(base, _MatrixFreeOperator):
        if base.which != "F":
            raise ValueError("only the double-layer operator F can be inverted matrix-free")
        ctx = base.ctx
        op.kind = _capi.BIE_OP_MATRIX_FREE
        op.k_re, op.k_im = base.k.real, base.k.imag
    elif isinstance(base, _FastOperator):
        ctx = base.ctx
        op.kind = _capi.BIE_OP_FAST
        op.fast = base._h.value
        keep.append(base)
    elif ctx is None:
        raise ValueError("dense gmres needs the context of the mesh (ctx=...)")
    else:
        op.kind = _capi.BIE_OP_DENSE
    opts = _capi.GmresOpts(restart=int(restart or 0), maxiter=int(maxiter or 0), reltol=float(reltol),
                           abstol=float(abstol), precision=_capi.PRECISION[precision],
                           refine=1 if refine else 0, inner_reltol=0.0, max_refine=0,
                           initially_nonzero=1 if x0 is not None else 0)
    info = _capi.GmresInfo()
    if on_host:
        # column-major N x N matrices and vectors stay on the host; bie_gmres copies them
        if dense:
            Ah = np.asfortranarray(base, dtype=np.complex128)
            keep.append(Ah)
            op.A = Ah.ctypes.data
            if A32 is not None:
                A32h = np.asfortranarray(A32, dtype=np.complex64)
                keep.append(A32h)
                op.A32 = A32h.ctypes.data
        if aff.diag is not None:
            dg = np.ascontiguousarray(aff.diag, dtype=np.complex128)
            keep.append(dg)
            op.diag = dg.ctypes.data
        bh = np.ascontiguousarray(b, dtype=np.complex128)
        x = np.array(x0, dtype=np.complex128) if x0 is not None else np.zeros_like(bh)
        st = _capi.lib().bie_gmres(ctx.handle, C.byref(op), bh.ctypes.data, x.ctypes.data,
                                   C.byref(opts), C.byref(info))
    else:
        torch = _torch()
        dev = torch.device(f"cuda:{ctx.device}")
        if dense:
            if _is_torch(base):
                Ad = base
            else:
                # column-major N x N numpy -> device memory of the same layout
                Ad = torch.as_tensor(np.asfortranarray(base, dtype=np.complex128).T.copy(), device=dev)
            keep.append(Ad)
            op.A = Ad.data_ptr()
            if A32 is not None:
                keep.append(A32)
                op.A32 = A32.data_ptr()
            elif refine or precision == "mixed":
                A32 = torch.empty(Ad.shape, dtype=torch.complex64, device=dev)
                _capi.check(_capi.lib().bie_round_c64_device(ctx.handle, Ad.data_ptr(), A32.data_ptr(),
                                                             Ad.numel()))
                keep.append(A32)
                op.A32 = A32.data_ptr()
        if aff.diag is not None:
            dg = _device_complex(aff.diag, dev)
            keep.append(dg)
            op.diag = dg.data_ptr()
        bd = _device_complex(b, dev)
        xd = _device_complex(x0, dev).clone() if x0 is not None else torch.zeros_like(bd)
        torch.cuda.synchronize(dev)
        st = _capi.lib().bie_gmres_device(ctx.handle, C.byref(op), bd.data_ptr(), xd.data_ptr(),
                                          C.byref(opts), C.byref(info))
        x = xd if _is_torch(b) else xd.cpu().numpy()
    if st not in (_capi.BIE_OK, _capi.BIE_ERR_NOT_CONVERGED):
        _capi.check(st)
    res = GmresResult(x, info)
    return (x, res) if log else x

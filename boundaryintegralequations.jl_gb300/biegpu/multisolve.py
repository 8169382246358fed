"""Many right-hand sides at once (bie_solve_multi_device).

Solves ``(F + Diagonal(1 - C)) X = B`` for an N x R matrix B, the exterior
collocation system of test/3d/assembly_test.jl:37-38, which the reference
solves column by column with gmres.  The R solves run in lockstep with
tensor-core products of the mixed-precision F and are refined with exact
residuals of the complex64 matrix.
"""
from __future__ import annotations

import ctypes as C

from . import _capi
from .assembly import get_context


def solve_multi(mesh, k, B, precision: str = "fp16_split", restart: int = 0, maxiter: int = 0,
                max_refine: int = 0, reltol: float = 0.0, inner_reltol: float = 0.0, n: int = 2, m: int = 2,
                device: int = 0, ctx=None):
    """X (same kind as B: numpy array or CUDA tensor, N x R), info dict.

    CUDA tensors go through bie_solve_multi_device (the library works on
    them in place); host arrays through bie_solve_multi (the library copies
    B in and X out)."""
    import numpy as np
    c = ctx if ctx is not None else get_context(mesh, n=n, m=m, device=device)
    k = complex(k)
    o = _capi.MultisolveOpts(precision=_capi.PRECISION[precision], restart=int(restart), maxiter=int(maxiter),
                             max_refine=int(max_refine), reltol=float(reltol), inner_reltol=float(inner_reltol))
    info = _capi.MultisolveInfo()
    on_device = type(B).__module__.startswith("torch") and B.is_cuda
    if not on_device:
        Bh = np.asarray(B, dtype=np.complex128)
        if Bh.ndim == 1:
            Bh = Bh[:, None]
        N, R = Bh.shape
        if N != c.n_sources:
            raise ValueError("B must have one row per collocation node")
        Bh = np.asfortranarray(Bh)
        X = np.empty((N, R), dtype=np.complex128, order="F")
        _capi.check(_capi.lib().bie_solve_multi(c.handle, k.real, k.imag, R, Bh.ctypes.data, X.ctypes.data,
                                                C.byref(o), C.byref(info)))
    else:
        import torch
        Bd = B.to(dtype=torch.complex128)
        if Bd.ndim == 1:
            Bd = Bd[:, None]
        N, R = Bd.shape
        if N != c.n_sources:
            raise ValueError("B must have one row per collocation node")
        Bd = Bd.T.contiguous().T                                   # column-major
        X = torch.empty((R, N), dtype=torch.complex128, device=Bd.device).T
        torch.cuda.synchronize(Bd.device)
        _capi.check(_capi.lib().bie_solve_multi_device(c.handle, k.real, k.imag, R, Bd.data_ptr(), X.data_ptr(),
                                                       C.byref(o), C.byref(info)))
    d = {name: getattr(info, name) for name, _ in info._fields_}
    return X, d

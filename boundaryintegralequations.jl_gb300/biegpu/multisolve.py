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
    """X (same kind as B: numpy array or CUDA tensor, N x R), info dict."""
    import torch
    c = ctx if ctx is not None else get_context(mesh, n=n, m=m, device=device)
    k = complex(k)
    on_device = isinstance(B, torch.Tensor) and B.is_cuda
    dev = B.device if on_device else torch.device(f"cuda:{c.device}")
    Bd = torch.as_tensor(B, dtype=torch.complex128, device=dev) if not isinstance(B, torch.Tensor) else \
        B.to(device=dev, dtype=torch.complex128)
    if Bd.ndim == 1:
        Bd = Bd[:, None]
    N, R = Bd.shape
    if N != c.n_sources:
        raise ValueError("B must have one row per collocation node")
    Bd = Bd.T.contiguous().T                                   # column-major
    X = torch.empty((R, N), dtype=torch.complex128, device=dev).T
    o = _capi.MultisolveOpts(precision=_capi.PRECISION[precision], restart=int(restart), maxiter=int(maxiter),
                             max_refine=int(max_refine), reltol=float(reltol), inner_reltol=float(inner_reltol))
    info = _capi.MultisolveInfo()
    torch.cuda.synchronize(dev)
    _capi.check(_capi.lib().bie_solve_multi_device(c.handle, k.real, k.imag, R, Bd.data_ptr(), X.data_ptr(),
                                                   C.byref(o), C.byref(info)))
    d = {name: getattr(info, name) for name, _ in info._fields_}
    return (X if on_device else X.cpu().numpy()), d

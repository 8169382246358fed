"""k-derivative (Taylor) assembly for reduced-order sweeps (ROSEBEM).

``taylor_assemble(mesh, k0, sources; M, fOn, gOn, cOn, n, m, U)`` mirrors
``taylor_assemble!`` (src/3d/rosebem.jl:56-157): the m-th derivatives of F and
G with respect to the wavenumber at k0, m = 0..M, assembled on the GPU
(bie_taylor_assemble), optionally projected onto a reduced basis U
(From = U^H F U).  ``apply_taylor_expansion`` evaluates the series at k
(src/3d/rosebem.jl:164-200).
"""
from __future__ import annotations

import math

import numpy as np

from . import _capi
from .assembly import get_context
from .mesh import Mesh3d


def taylor_assemble(mesh: Mesh3d, k0, sources=None, M: int = 0, fOn: bool = True, gOn: bool = True,
                    cOn: bool = True, n: int = 3, m: int = 3, U=None, device: int = 0):
    """(From, Grom, C): From/Grom of shape (n_nodes, n_nodes, M + 1) (targets x
    nodes when U is None and `sources` are given), C (targets)."""
    ctx = get_context(mesh, n=n, m=m, device=device)
    k0 = complex(k0)
    at_nodes = sources is None or sources is mesh.sources
    t = None if at_nodes else np.asfortranarray(sources, dtype=np.float64)
    Mt = mesh.n_sources if at_nodes else t.shape[1]
    N = mesh.n_sources
    F = np.empty((Mt, N, M + 1), dtype=np.complex128, order="F") if fOn else None
    G = np.empty((Mt, N, M + 1), dtype=np.complex128, order="F") if gOn else None
    Cv = np.empty(Mt, dtype=np.complex128) if cOn else None
    flags = (_capi.BIE_F if fOn else 0) | (_capi.BIE_G if gOn else 0) | (_capi.BIE_C if cOn else 0)
    _capi.check(_capi.lib().bie_taylor_assemble(ctx.handle, k0.real, k0.imag, _capi.ptr(t), Mt, flags, int(M),
                                                _capi.ptr(F), _capi.ptr(G), _capi.ptr(Cv)))
    if U is not None:
        Uc = np.asarray(U)
        if fOn:
            F = np.stack([Uc.conj().T @ F[:, :, j] @ Uc for j in range(M + 1)], axis=2)
        if gOn:
            G = np.stack([Uc.conj().T @ G[:, :, j] @ Uc for j in range(M + 1)], axis=2)
    return F, G, Cv


def apply_taylor_expansion(Abasis, k, k0, bbasis=None):
    """sum_{i=0}^{M} (k - k0)^i / i! A_i (and the same for bbasis when given)."""
    Mmax = Abasis.shape[2] - 1
    A = np.array(Abasis[:, :, 0])
    b = None if bbasis is None else np.array(bbasis[:, 0])
    for i in range(1, Mmax + 1):
        coef = (k - k0) ** i / math.factorial(i)
        A += coef * Abasis[:, :, i]
        if b is not None:
            b += coef * bbasis[:, i]
    return A if b is None else (A, b)

"""Adjoint shape / impedance gradients of a far-field objective (bie_adjoint).

``farfield_objective(mesh, k, Z, field_points)`` returns J = sum_j |p(x_j)|^2
for plane-wave scattering by a surface with element impedances Z_e, and its
gradients with respect to every vertex coordinate and every Z_e, computed on
the GPU by the adjoint method.  This is the function a ChainRulesCore
``rrule`` wraps on the Julia side (the pullback scales ``dX`` and ``dZ`` by the
incoming sensitivity of J).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi
from .assembly import get_context
from .mesh import Mesh3d


def farfield_objective(mesh: Mesh3d, k: float, Z, field_points, rho_c: float = 1.21 * 343.0,
                       direction=(0.0, 0.0, 1.0), gradient: bool = True, reltol: float = 1e-13,
                       n: int = 2, m: int = 2, device: int = 0, precision: str = "fp64"):
    """(J, p_field, dJ/dX (3 x N_c) or None, dJ/dZ (E complex) or None, info).
    ``precision="df64"`` assembles the forward model in double-float
    arithmetic (FP64-grade, faster on GB300); the reverse pass is FP64."""
    ctx = get_context(mesh, n=n, m=m, device=device)
    Zc = np.ascontiguousarray(Z, dtype=np.complex128)
    if Zc.shape != (mesh.n_elements,):
        raise ValueError("Z must hold one impedance per element")
    X = np.asfortranarray(field_points, dtype=np.float64)
    M = X.shape[1]
    d = np.asarray(direction, dtype=np.float64)
    d = d / np.linalg.norm(d)
    if precision not in ("fp64", "df64"):
        raise ValueError("precision must be 'fp64' or 'df64'")
    opts = _capi.AdjointOpts(rho_c=float(rho_c), dir=(C.c_double * 3)(*d), reltol=float(reltol),
                             precision=_capi.PRECISION[precision])
    J = C.c_double()
    pf = np.empty(M, dtype=np.complex128)
    dX = np.empty((3, mesh.coordinates.shape[1]), dtype=np.float64, order="F") if gradient else None
    dZ = np.empty(mesh.n_elements, dtype=np.complex128) if gradient else None
    info = _capi.AdjointInfo()
    _capi.check(_capi.lib().bie_adjoint(ctx.handle, float(np.real(k)), float(np.imag(k)), Zc.ctypes.data,
                                        X.ctypes.data, M, C.byref(opts), C.byref(J), pf.ctypes.data,
                                        _capi.ptr(dX), _capi.ptr(dZ), C.byref(info)))
    inf = {name: getattr(info, name) for name, _ in info._fields_}
    return J.value, pf, dX, dZ, inf

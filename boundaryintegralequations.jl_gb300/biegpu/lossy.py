"""The visco-thermal ("lossy") system on the GPU.

Mirrors the reference's lossy layer:

  * :func:`ambient_to_properties`, :func:`visco_thermal_constants` -
    src/utils/ambient_to_properties.jl:1-134 and src/utils/lossy_constants.jl:1-34
    (computed by libbiegpu's host code);
  * :func:`tangential_derivatives` - interpolation_function_derivatives(mesh),
    src/3d/interpolation_function_derivatives.jl:36-118 (host code);
  * :class:`LossyGlobalOuter` - src/3d/LossyGlobalMatrix.jl:76-197: the reduced
    lossy system resident on the device, with its blocks (Ha, Ga, Hh, Gh, Hv,
    Gv, Dc, Dr, Nd, Nd', inner) as operators that apply and solve (GMRES) on
    the device, as the reference's test/3d/losses_test.jl uses them.

:func:`boundary_layer_wavenumbers` keeps the leading-order textbook forms used
by the multi-right-hand-side workload.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi
from .assembly import Context, get_context
from .assembly import mesh_desc as _mesh_desc
from .mesh import Mesh3d

AIR_20C = {"rho": 1.204, "c": 343.2, "mu": 1.81e-5, "alpha": 2.2e-5}


def boundary_layer_wavenumbers(freq: float = 100.0, air: dict = AIR_20C):
    """[k, k_v, k_h] (complex) at ``freq`` Hz in their leading-order forms
    k = omega / c, k_v = sqrt(i omega rho / mu), k_h = sqrt(i omega / alpha)
    (the S = +1 convention), for fixed textbook air properties."""
    w = 2.0 * np.pi * freq
    k = w / air["c"]
    kv = np.sqrt(1j * w * air["rho"] / air["mu"])
    kh = np.sqrt(1j * w / air["alpha"])
    return [complex(k), complex(kv), complex(kh)]


def ambient_to_properties(f=1000.0, ps=101325.0, t=20.0, H=50.0):
    """(rho, c0, cf, CpCv, eta, alfa, Cp, Cv, landa, beta) of air (Rasmussen 1997)."""
    out = (C.c_double * 10)()
    _capi.check(_capi.lib().bie_ambient_to_properties(float(f), float(ps), float(t), float(H), out))
    return tuple(out)


def _c(v):
    return complex(v[0], v[1])


def _constants_tuple(k: "_capi.LossyConstants"):
    return (k.rho, k.c, k.kp, _c(k.ka), _c(k.kh), _c(k.kv), _c(k.tau_a), _c(k.tau_h), _c(k.phi_a),
            _c(k.phi_h), k.eta, k.mu)


def visco_thermal_constants(freq=1000.0, S=-1.0, pa=101325.0, t=20.0, Hr=50.0):
    """(rho, c, kp, ka, kh, kv, tau_a, tau_h, phi_a, phi_h, eta, mu), the return
    value of the reference's visco_thermal_constants(; freq, S, pa, t, Hr)."""
    k = _capi.LossyConstants()
    _capi.check(_capi.lib().bie_visco_thermal_constants(float(freq), float(S), float(pa), float(t), float(Hr),
                                                        C.byref(k)))
    return _constants_tuple(k)


def tangential_derivatives(mesh: Mesh3d):
    """(Dx, Dy, Dz) as scipy CSR matrices (N x N): the tangential part of the
    gradient of the physics interpolation, averaged over the elements of each
    node (interpolation_function_derivatives)."""
    import scipy.sparse as sp
    L = _capi.lib()
    d, keep = _mesh_desc(mesh)
    nnz = C.c_int64()
    _capi.check(L.bie_tangential_derivatives(C.byref(d), C.byref(nnz), None, None, None, None, None))
    N = mesh.n_sources
    rp = np.empty(N + 1, dtype=np.int64)
    cols = np.empty(nnz.value, dtype=np.int64)
    D = [np.empty(nnz.value) for _ in range(3)]
    _capi.check(L.bie_tangential_derivatives(C.byref(d), C.byref(nnz), rp.ctypes.data, cols.ctypes.data,
                                             D[0].ctypes.data, D[1].ctypes.data, D[2].ctypes.data))
    del keep
    return tuple(sp.csr_matrix((v, cols, rp), shape=(N, N)) for v in D)


def _gmres_opts(reltol=0.0, restart=0, maxiter=0, abstol=0.0):
    return _capi.GmresOpts(restart=int(restart), maxiter=int(maxiter), reltol=float(reltol), abstol=float(abstol),
                           precision=_capi.BIE_PREC_FP64, refine=0, inner_reltol=0.0, max_refine=0,
                           initially_nonzero=0)


class LossyBlock:
    """One block of the lossy system: ``A @ x`` applies it on the device,
    ``A.solve(b)`` runs gmres(A, b) on the device (square blocks)."""

    def __init__(self, owner: "LossyGlobalOuter", name: str, shape):
        self._owner = owner
        self.name = name
        self.code = _capi.BIE_LOSSY_BLOCKS[name]
        self.shape = shape

    def __matmul__(self, x):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        if x.shape != (self.shape[1],):
            raise ValueError(f"{self.name}: x must have length {self.shape[1]}")
        y = np.empty(self.shape[0], dtype=np.complex128)
        _capi.check(_capi.lib().bie_lossy_apply(self._owner._h, self.code, x.ctypes.data, y.ctypes.data))
        return y

    def solve(self, b, reltol=0.0, restart=0, maxiter=0, abstol=0.0, return_info=False):
        """x = gmres(A, b) from x = 0 (IterativeSolvers defaults for zeros)."""
        if self.shape[0] != self.shape[1]:
            raise ValueError(f"{self.name} is not square")
        b = np.ascontiguousarray(b, dtype=np.complex128)
        if b.shape != (self.shape[0],):
            raise ValueError(f"{self.name}: b must have length {self.shape[0]}")
        x = np.empty_like(b)
        info = _capi.GmresInfo()
        opts = _gmres_opts(reltol, restart, maxiter, abstol)
        st = _capi.lib().bie_lossy_solve(self._owner._h, self.code, b.ctypes.data, x.ctypes.data, C.byref(opts),
                                         C.byref(info))
        if st != _capi.BIE_ERR_NOT_CONVERGED:
            _capi.check(st)
        d = {name: getattr(info, name) for name, _ in info._fields_}
        return (x, d) if return_info else x


class LossyGlobalOuter(LossyBlock):
    """LossyGlobalOuter(mesh, freq; depth, n, exterior, fmm_on) on the device.

    ``L @ x`` is the reduced lossy product (LossyGlobalMatrix.jl:179-197) and
    ``L.solve(b)`` gmres(L, b); the blocks are attributes (``Ha, Ga, Hh, Gh,
    Hv, Gv, Dc, Dr, Nd, NdT, inner``) and the constants too (``phi_a, phi_h,
    tau_a, tau_h, mu_a, mu_h`` and the wavenumbers ``ka, kh, kv``).  ``n`` is
    the acoustic assembly's quadrature (n = m, 3 in the reference); the nested
    gmres calls take ``reltol/restart/maxiter`` (zeros: IterativeSolvers
    defaults).
    """

    def __init__(self, mesh: Mesh3d, freq: float, depth: int = 1, n: int = 3, exterior: bool = True,
                 fmm_on: bool = False, S: float = 1.0, fmm_offset: float = 0.2, device: int = 0,
                 reltol: float = 0.0, restart: int = 0, maxiter: int = 0, context: Context | None = None):
        N = mesh.n_sources
        self.mesh = mesh
        self.n = N
        self.ctx = context if context is not None else get_context(mesh, n=n, m=n, device=device)
        self._normals = np.asfortranarray(mesh.normals, dtype=np.float64)
        opts = _capi.LossyOpts(S=float(S), custom_air=0, pa=0.0, t=0.0, Hr=0.0, depth=int(depth),
                               interior=0 if exterior else 1, fmm_on=1 if fmm_on else 0, n_gauss=int(n),
                               fmm_offset=float(fmm_offset), normals=self._normals.ctypes.data,
                               solve=_gmres_opts(reltol, restart, maxiter))
        h = C.c_void_p()
        _capi.check(_capi.lib().bie_lossy_create(self.ctx.handle, float(freq), C.byref(opts), C.byref(h)))
        self._h = h
        import weakref
        self._finalizer = weakref.finalize(self, _capi.lib().bie_lossy_destroy, h)
        super().__init__(self, "outer", (N, N))
        k = _capi.LossyConstants()
        _capi.check(_capi.lib().bie_lossy_constants_of(h, C.byref(k)))
        (self.rho, self.c, self.kp, self.ka, self.kh, self.kv, self.tau_a, self.tau_h, self.phi_a, self.phi_h,
         self.eta, self.mu) = _constants_tuple(k)
        self.mu_a, self.mu_h = _c(k.mu_a), _c(k.mu_h)
        shapes = {"Ha": (N, N), "Ga": (N, N), "Hh": (N, N), "Gh": (N, N), "Hv": (3 * N, 3 * N),
                  "Gv": (3 * N, 3 * N), "Dc": (3 * N, N), "Dr": (N, 3 * N), "Nd": (3 * N, N), "NdT": (N, 3 * N),
                  "inner": (N, N)}
        for name, shp in shapes.items():
            setattr(self, name, LossyBlock(self, name, shp))

    def close(self) -> None:
        self._finalizer()

    def stats(self, reset: bool = False) -> dict:
        s, i = C.c_int64(), C.c_int64()
        _capi.check(_capi.lib().bie_lossy_stats(self._h, C.byref(s), C.byref(i), 1 if reset else 0))
        return {"nested_solves": s.value, "nested_iterations": i.value}

    ONE_LAUNCH_MODES = {False: 0, True: 1, "off": 0, "auto": 1, "cluster": 2, "grid": 3}

    def set_one_launch(self, mode=True) -> None:
        """Sparse thermal / viscous solves as one launch each: True / "auto"
        (default: a cooperative grid for more than 2048 rows, else a cluster),
        "cluster" or "grid" (that form only); False / "off": the
        launch-per-operation device GMRES."""
        _capi.check(_capi.lib().bie_lossy_set_one_launch(self._h, self.ONE_LAUNCH_MODES[mode]))

    def rhs(self, v0):
        """Ga gmres(inner, Dr v0 - Nd' gmres(Gv, Hv v0)): the right-hand side of a
        prescribed boundary velocity v0 (3N), test/3d/losses_test.jl:33."""
        v0 = np.asarray(v0, dtype=np.complex128)
        return self.Ga @ self.inner.solve(self.Dr @ v0 - self.NdT @ self.Gv.solve(self.Hv @ v0))


__all__ = ["ambient_to_properties", "visco_thermal_constants", "tangential_derivatives", "LossyGlobalOuter",
           "LossyBlock", "boundary_layer_wavenumbers"]

"""Batched frequency sweeps on the GPU (bie_sweep).

For every mesh m and wavenumber k_j the library assembles F, G, C and solves
``(F + Diagonal(1 - C)) p = G w_m`` with GMRES, all on the device.  The
reference offers no batched form; its users loop ``assemble_parallel!`` +
``gmres`` over frequencies (examples/sweep_meta.jl:219-233).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _capi
from .assembly import get_context


def sweep(meshes, ks, ws, precision: str = "mixed", refine: bool = True, n: int = 2, m: int = 2,
          reltol: float = math.sqrt(np.finfo(np.float64).eps), restart: int = 0, maxiter: int = 0,
          device: int = 0, eager: bool = False, target_error: float = 1e-6):
    """Solve the frequency sweep; returns (list of N_m x nk complex arrays, info dict).

    ``ks``: wavenumbers (real or complex), ``ws``: per-mesh boundary data
    (length N_m complex).  ``precision="mixed"`` with ``refine=True`` is the
    fast path (mixed assembly, complex64 inner GMRES, complex128 residual);
    ``precision="fp64", refine=False`` is the plain FP64 path;
    ``precision="df64", refine=False`` the same with FP64-grade double-float
    assembly.  By default
    everything after each mesh's first wavenumber is one launch of a recorded
    CUDA graph (device-side loops over wavenumbers and GMRES iterations);
    ``eager=True`` launches kernel by kernel from the host.

    ``target_error`` (mixed only): after each mixed solve a short GMRES solve
    with a pseudo-random right-hand side estimates the system's sensitivity s
    (large near the interior resonances of the mesh); solves whose predicted
    error 5e-7 s exceeds ``target_error`` are solved again at FP64 grade.
    ``None`` or 0 turns the estimate off.  ``info["sensitivity"]`` holds the
    estimates (nmesh x nk) and ``info["accurate_solves"]`` the number redone.
    """
    ctxs = [get_context(mesh, n=n, m=m, device=device) for mesh in meshes]
    ks = np.asarray(ks, dtype=np.complex128)
    nk = len(ks)
    kbuf = np.ascontiguousarray(ks)
    wbufs = [np.ascontiguousarray(w, dtype=np.complex128) for w in ws]
    for w, mesh in zip(wbufs, meshes):
        if w.shape != (mesh.n_sources,):
            raise ValueError("each w must have one value per collocation node")
    outs = [np.empty((mesh.n_sources, nk), dtype=np.complex128, order="F") for mesh in meshes]
    nm = len(meshes)
    carr = (C.c_void_p * nm)(*[c.handle.value for c in ctxs])
    warr = (C.c_void_p * nm)(*[w.ctypes.data for w in wbufs])
    parr = (C.c_void_p * nm)(*[o.ctypes.data for o in outs])
    g = _capi.GmresOpts(restart=int(restart), maxiter=int(maxiter), reltol=float(reltol), abstol=0.0,
                        precision=_capi.BIE_PREC_FP64, refine=0, inner_reltol=0.0, max_refine=0,
                        initially_nonzero=0)
    tgt = float(target_error) if (target_error and precision == "mixed") else 0.0
    sens = np.zeros((nm, nk), dtype=np.float64)
    opts = _capi.SweepOpts(precision=_capi.PRECISION[precision], refine=1 if refine else 0, gmres=g,
                           eager=1 if eager else 0, target_error=tgt,
                           sensitivity=sens.ctypes.data if tgt > 0 else None)
    info = _capi.SweepInfo()
    iters = np.zeros((nm, nk), dtype=np.int32)
    _capi.check(_capi.lib().bie_sweep(carr, nm, kbuf.ctypes.data, nk, warr, parr, C.byref(opts),
                                      C.byref(info), iters.ctypes.data))
    d = {name: getattr(info, name) for name, _ in info._fields_}
    d["iterations_per_solve"] = iters
    if tgt > 0:
        d["sensitivity"] = sens
    return outs, d

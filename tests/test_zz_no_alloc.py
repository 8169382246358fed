"""The allocation-free operator product, bie_matvec_device_noalloc.

Callers such as a Julia session whose CUDA.jl pool (or a process whose
PyTorch caching allocator) already owns most of the GPU cannot let the library
call cudaMalloc.  This entry point keeps its temporaries in a fixed 32 MiB
device array inside the library instead.  The test calls it through the C ABI
twice in a row, with different inputs, and compares each result with the
ordinary entry point bie_matvec_device (mixed precision, relative 2-norm
tolerance 1e-6, the tolerance of the other mixed-precision tests); it also
checks that free device memory does not change across the calls and that a
mesh too large for the fixed array is rejected with a clear message.

This file is named so that pytest collects it last.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import biegpu
from biegpu import _capi
from biegpu import mesh as bm

pytestmark = pytest.mark.gpu
TOL = 1e-6


def _rand(n, seed, torch, dev):
    r = np.random.default_rng(seed)
    z = r.normal(size=n) + 1j * r.normal(size=n)
    return torch.as_tensor(z, dtype=torch.complex128, device=dev)


def _rel(a, b):
    return float((a - b).abs().pow(2).sum().sqrt() / b.abs().pow(2).sum().sqrt())


@pytest.mark.parametrize("geometry,f,k", [("quadratic", 6, 4.0), ("linear", 12, 2.5 + 0.3j)])
def test_noalloc_matches_matvec_device_twice(geometry, f, k):
    torch = pytest.importorskip("torch")
    L = _capi.lib()
    mesh = bm.icosphere(f, geometry=geometry)
    ctx = biegpu.Context(mesh, n=2, m=2, device=0)
    dev = torch.device("cuda:0")
    N = mesh.n_sources
    k = complex(k)
    yF = torch.empty(N, dtype=torch.complex128, device=dev)
    yG = torch.empty_like(yF)
    zF = torch.empty_like(yF)
    zG = torch.empty_like(yF)
    inputs = [(_rand(N, 10, torch, dev), _rand(N, 11, torch, dev)),
              (_rand(N, 20, torch, dev), _rand(N, 21, torch, dev))]
    # reference results from the ordinary entry point (it may allocate)
    refs = []
    for x, v in inputs:
        _capi.check(L.bie_matvec_device(ctx.handle, k.real, k.imag, None, 0, x.data_ptr(), v.data_ptr(),
                                        yF.data_ptr(), yG.data_ptr(), _capi.BIE_PREC_MIXED))
        _capi.check(L.bie_ctx_stats(ctx.handle, C.byref(_capi.Stats()), 0))   # synchronises
        refs.append((yF.clone(), yG.clone()))
    torch.cuda.synchronize()
    free_before = None
    for call, ((x, v), (rF, rG)) in enumerate(zip(inputs, refs)):
        zF.fill_(float("nan"))
        zG.fill_(float("nan"))
        torch.cuda.synchronize()
        if call == 1:
            free_before = torch.cuda.mem_get_info(dev)[0]
        _capi.check(L.bie_matvec_device_noalloc(ctx.handle, k.real, k.imag, None, 0, x.data_ptr(),
                                                v.data_ptr(), zF.data_ptr(), zG.data_ptr()))
        _capi.check(L.bie_ctx_stats(ctx.handle, C.byref(_capi.Stats()), 0))   # synchronises
        assert torch.isfinite(zF).all() and torch.isfinite(zG).all()
        assert _rel(zF, rF) <= TOL, f"call {call}: F {_rel(zF, rF):.3e}"
        assert _rel(zG, rG) <= TOL, f"call {call}: G {_rel(zG, rG):.3e}"
    assert torch.cuda.mem_get_info(dev)[0] == free_before
    # F only (no G input) through the same array
    _capi.check(L.bie_matvec_device_noalloc(ctx.handle, k.real, k.imag, None, 0, inputs[0][0].data_ptr(),
                                            None, zF.data_ptr(), None))
    _capi.check(L.bie_ctx_stats(ctx.handle, C.byref(_capi.Stats()), 0))
    assert _rel(zF, refs[0][0]) <= TOL
    ctx.close()


def test_noalloc_rejects_mesh_beyond_fixed_scratch():
    torch = pytest.importorskip("torch")
    L = _capi.lib()
    mesh = bm.icosphere(100)          # 100002 nodes, 200000 triangles: > 32 MiB of temporaries
    ctx = biegpu.Context(mesh, n=2, m=2, device=0)
    N = mesh.n_sources
    x = torch.zeros(N, dtype=torch.complex128, device="cuda:0")
    y = torch.empty_like(x)
    st = L.bie_matvec_device_noalloc(ctx.handle, 1.0, 0.0, None, 0, x.data_ptr(), x.data_ptr(),
                                     y.data_ptr(), y.data_ptr())
    assert st == _capi.BIE_ERR_INVALID
    msg = L.bie_last_error().decode()
    assert "bytes of scratch" in msg and "bie_matvec_device" in msg
    ctx.close()

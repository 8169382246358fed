"""The allocation-free operator product, bie_matvec_device_noalloc.

Callers such as a Julia session whose CUDA.jl pool (or a process whose
PyTorch caching allocator) already owns most of the GPU cannot let the library
call cudaMalloc.  This entry point keeps its temporaries in a fixed 32 MiB
device array inside the library instead; the array is committed and its
address looked up when a context is created.

The test creates a fresh context and makes the allocation-free product its
first product: two calls in a row with different inputs, then an F-only call.
Free device memory is read once before those calls and once after the last of
them and must not change.  Only then does the ordinary entry point
bie_matvec_device (which may allocate) compute the comparison values; each
result must agree with it to a relative 2-norm of 1e-6, the tolerance of the
other mixed-precision tests.  A mesh too large for the fixed array is rejected
with a clear message.

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


def _sync(L, ctx):
    _capi.check(L.bie_ctx_stats(ctx.handle, C.byref(_capi.Stats()), 0))   # synchronises the stream


@pytest.mark.parametrize("geometry,f,k", [("quadratic", 6, 4.0), ("linear", 12, 2.5 + 0.3j)])
def test_noalloc_first_products_match_matvec_device(geometry, f, k):
    torch = pytest.importorskip("torch")
    L = _capi.lib()
    mesh = bm.icosphere(f, geometry=geometry)
    dev = torch.device("cuda:0")
    N = mesh.n_sources
    k = complex(k)
    inputs = [(_rand(N, 10, torch, dev), _rand(N, 11, torch, dev)),
              (_rand(N, 20, torch, dev), _rand(N, 21, torch, dev))]
    outs = [(torch.full((N,), float("nan"), dtype=torch.complex128, device=dev),
             torch.full((N,), float("nan"), dtype=torch.complex128, device=dev)) for _ in range(2)]
    zF_only = torch.full((N,), float("nan"), dtype=torch.complex128, device=dev)
    ctx = biegpu.Context(mesh, n=2, m=2, device=0)          # fresh context: no product ran on it
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info(dev)[0]
    for (x, v), (zF, zG) in zip(inputs, outs):
        _capi.check(L.bie_matvec_device_noalloc(ctx.handle, k.real, k.imag, None, 0, x.data_ptr(),
                                                v.data_ptr(), zF.data_ptr(), zG.data_ptr()))
        _sync(L, ctx)
    _capi.check(L.bie_matvec_device_noalloc(ctx.handle, k.real, k.imag, None, 0, inputs[0][0].data_ptr(),
                                            None, zF_only.data_ptr(), None))
    _sync(L, ctx)
    free_after = torch.cuda.mem_get_info(dev)[0]
    assert free_after == free_before, f"free device memory changed by {free_before - free_after} bytes"

    # comparison values from the ordinary entry point (it may allocate)
    yF = torch.empty(N, dtype=torch.complex128, device=dev)
    yG = torch.empty_like(yF)
    for call, ((x, v), (zF, zG)) in enumerate(zip(inputs, outs)):
        _capi.check(L.bie_matvec_device(ctx.handle, k.real, k.imag, None, 0, x.data_ptr(), v.data_ptr(),
                                        yF.data_ptr(), yG.data_ptr(), _capi.BIE_PREC_MIXED))
        _sync(L, ctx)
        assert torch.isfinite(zF).all() and torch.isfinite(zG).all()
        assert _rel(zF, yF) <= TOL, f"call {call}: F {_rel(zF, yF):.3e}"
        assert _rel(zG, yG) <= TOL, f"call {call}: G {_rel(zG, yG):.3e}"
        if call == 0:
            assert _rel(zF_only, yF) <= TOL, f"F-only call: {_rel(zF_only, yF):.3e}"
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

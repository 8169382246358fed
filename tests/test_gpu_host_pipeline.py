"""bie_assemble with host buffers of 256 MB and more (and M >= 5760 targets)
runs row blocks on two streams (assembly of block b + 1 while block b is
copied to the host).  The
blocked result must equal the device-resident assembly: FP64 to 1e-13 (the
assemblies differ only by the order of FP64 atomic sums), mixed to 1e-6
against FP64, for square and ragged target counts and for pageable and pinned
host arrays."""
from __future__ import annotations

import numpy as np
import pytest
import torch

import biegpu
from biegpu import mesh as bm

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def big():
    mesh = bm.icosphere(26)          # 6762 nodes: F and G are 2 x 732 MB, 2 row blocks
    return mesh, biegpu.Context(mesh, n=2, m=2, device=0)


def device_reference(ctx, k, targets):
    N = ctx.n_sources
    t = None if targets is None else torch.as_tensor(np.ascontiguousarray(targets.T)).cuda()
    M = N if targets is None else targets.shape[1]
    F = torch.empty((N, M), dtype=torch.complex128, device="cuda")
    G = torch.empty((N, M), dtype=torch.complex128, device="cuda")
    C = torch.empty(M, dtype=torch.complex128, device="cuda")
    ctx.assemble_device(k, F=F, G=G, Cv=C, targets=t)
    torch.cuda.synchronize()
    return F.cpu().numpy().T, G.cpu().numpy().T, C.cpu().numpy()


@pytest.mark.parametrize("rows", [None, 6001])
def test_blocked_host_assembly_matches_device(big, rows):
    mesh, ctx = big
    k = 3.0 + 0.05j
    X = None if rows is None else np.asfortranarray(mesh.sources[:, :rows] * 1.0)
    Fd, Gd, Cd = device_reference(ctx, k, X)
    F, G, C = ctx.assemble(k, targets=X, precision="fp64")
    assert rel(F, Fd) <= 1e-13 and rel(G, Gd) <= 1e-13 and rel(C, Cd) <= 1e-13
    Fm, Gm, Cm = ctx.assemble(k, targets=X, precision="mixed")
    assert rel(Fm, Fd) <= 1e-6 and rel(Gm, Gd) <= 1e-6 and rel(Cm, Cd) <= 1e-6


def test_blocked_host_assembly_pinned_outputs(big):
    mesh, ctx = big
    N = mesh.n_sources
    pin = lambda shape: torch.empty(shape, dtype=torch.complex128, pin_memory=True).numpy()  # noqa: E731
    Fh, Gh, Ch = pin((N, N)).T, pin((N, N)).T, pin((N,))
    ctx.assemble(2.0, out=(Fh, Gh, Ch), precision="fp64")
    Fd, Gd, Cd = device_reference(ctx, 2.0, None)
    assert rel(Fh, Fd) <= 1e-13 and rel(Gh, Gd) <= 1e-13 and rel(Ch, Cd) <= 1e-13
    # G only: one matrix, still blocked
    _, G1, _ = ctx.assemble(2.0, fOn=False, cOn=False, precision="fp64")
    assert rel(G1, Gd) <= 1e-13

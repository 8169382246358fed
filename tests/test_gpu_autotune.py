"""Autotuned element slicing of the mixed assembly (bie_ctx_set_autotune): the
tuning call and the calls after it return the mixed-precision matrices within
the mixed tolerance (1e-6 relative Frobenius against the oracle), for two
target counts."""
from __future__ import annotations

import numpy as np
import pytest

import biegpu
import oracle
from biegpu import mesh as bm

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_autotuned_mixed_assembly():
    mesh = bm.icosphere(6, geometry="quadratic")
    ctx = biegpu.Context(mesh, n=2, m=2, device=0)
    ctx.set_autotune(True)
    F, G, Cv = oracle.assemble(mesh, 4.0, n=2, m=2)
    for _ in range(2):   # the first call tunes, the second uses the kept slicing
        Fg, Gg, Cg = ctx.assemble(4.0, precision="mixed")
        assert rel(Fg, F) <= 1e-6 and rel(Gg, G) <= 1e-6 and rel(Cg, Cv) <= 1e-6
    X = mesh.sources[:, :77] * 1.3
    Fo, Go, _ = oracle.assemble(mesh, 4.0, targets=X, n=2, m=2, cOn=False)
    for _ in range(2):
        Fg, Gg, _ = ctx.assemble(4.0, targets=X, cOn=False, precision="mixed")
        assert rel(Fg, Fo) <= 1e-6 and rel(Gg, Go) <= 1e-6

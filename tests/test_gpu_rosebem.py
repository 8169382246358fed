"""k-derivative assembly (bie_taylor_assemble, taylor_assemble!) against the
oracle restatement: F^(m), G^(m), C <= 1e-12 relative Frobenius (FP64), linear
and quadratic elements (the quadratic case keeps the reference's corner-rule
choice), complex k0 and off-surface targets; the Taylor series evaluated near
k0 reproduces the assembly at k."""
from __future__ import annotations

import numpy as np
import pytest

import biegpu
import oracle
from biegpu import mesh as bm

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("geo,f,k0", [("linear", 4, 2.0), ("quadratic", 3, 1.5), ("linear", 3, 2.0 + 0.3j)])
def test_taylor_matches_oracle(geo, f, k0):
    mesh = bm.icosphere(f, geometry=geo)
    F, G, C = biegpu.taylor_assemble(mesh, k0, M=4, n=2, m=2)
    Fo, Go, Co = oracle.taylor_assemble(mesh, k0, 4, n=2, m=2)
    for j in range(5):
        assert rel(F[:, :, j], Fo[:, :, j]) <= 1e-12, j
        assert rel(G[:, :, j], Go[:, :, j]) <= 1e-12, j
    assert rel(C, Co) <= 1e-12


def test_taylor_targets_and_series():
    mesh = bm.icosphere(5)
    X = np.array([[0.0, 0.1, 0.2], [0.0, 0.0, 0.3], [1.5, 2.0, -1.7]])
    F, G, _ = biegpu.taylor_assemble(mesh, 3.0, sources=X, M=2, n=2, m=2, cOn=False)
    Fo, Go, _ = oracle.taylor_assemble(mesh, 3.0, 2, targets=X, n=2, m=2, cOn=False)
    assert rel(F, Fo) <= 1e-12 and rel(G, Go) <= 1e-12
    # series at k = k0 + 0.05 with 12 terms against the direct assembly
    Ft, Gt, _ = biegpu.taylor_assemble(mesh, 3.0, M=12, n=2, m=2, cOn=False)
    Fk, Gk, _ = biegpu.assemble_parallel(mesh, 3.05, mesh.sources, n=2, m=2, cOn=False)
    assert rel(biegpu.apply_taylor_expansion(Ft, 3.05, 3.0), Fk) <= 1e-10
    assert rel(biegpu.apply_taylor_expansion(Gt, 3.05, 3.0), Gk) <= 1e-10

"""Batched frequency sweep (bie_sweep): mixed precision with refinement against
the plain FP64 GPU path and a dense CPU solve of the oracle matrices."""
from __future__ import annotations

import numpy as np
import pytest

import biegpu
import oracle
from biegpu import mesh as bm

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_sweep_two_meshes_against_oracle():
    meshes = [bm.icosphere(4), bm.ellipsoid(5)]
    ks = [0.5, 2.0, 4.0 + 0.2j]
    rng = np.random.default_rng(42)
    ws = [rng.normal(size=mm.n_sources) + 1j * rng.normal(size=mm.n_sources) for mm in meshes]
    ps, info = biegpu.sweep(meshes, ks, ws, precision="fp64", refine=False)
    assert info["solves"] == 6 and info["converged"] == 6
    for mesh, w, p in zip(meshes, ws, ps):
        for j, k in enumerate(ks):
            F, G, C = oracle.assemble(mesh, k, n=2, m=2)
            pd = np.linalg.solve(F + np.diag(1.0 - C), G @ w)
            assert rel(p[:, j], pd) <= 1e-6


def test_sweep_mixed_matches_fp64():
    meshes = [bm.icosphere(6), bm.icosphere(4, geometry="quadratic")]
    ks = np.linspace(0.1, 10.0, 5)
    rng = np.random.default_rng(7)
    ws = [rng.normal(size=mm.n_sources) + 1j * rng.normal(size=mm.n_sources) for mm in meshes]
    p64, i64 = biegpu.sweep(meshes, ks, ws, precision="fp64", refine=False)
    pmx, imx = biegpu.sweep(meshes, ks, ws, precision="mixed", refine=True)
    assert imx["converged"] == imx["solves"] == 10
    for a, b in zip(pmx, p64):
        for j in range(len(ks)):
            assert rel(a[:, j], b[:, j]) <= 1e-5

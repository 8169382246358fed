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
            assert rel(a[:, j], b[:, j]) <= 1e-6


def test_sweep_sphere_2562_all_64_wavenumbers():
    """The sweep workload's smallest mesh (sphere f=16, 2562 nodes) at all 64
    wavenumbers ka in [0.1, 10], which pass near the sphere's interior
    resonances (ka = 4.49, 5.76, 9.36 ...): every mixed solution within 1e-6
    of the plain FP64 one (the solves the sensitivity estimate flags are
    solved again at FP64 grade: at least one here), and the FP64-grade
    double-float sweep within 1e-10 of it.  Without the estimate the mixed
    sweep exceeds 1e-6 next to ka = 4.49."""
    mesh = bm.icosphere(16)
    ks = np.linspace(0.1, 10.0, 64)
    rng = np.random.default_rng(2026)
    w = rng.normal(size=mesh.n_sources) + 1j * rng.normal(size=mesh.n_sources)
    p64, i64 = biegpu.sweep([mesh], ks, [w], precision="fp64", refine=False)
    pmx, imx = biegpu.sweep([mesh], ks, [w], precision="mixed", refine=True, target_error=1e-6)
    pdf, idf = biegpu.sweep([mesh], ks, [w], precision="df64", refine=False)
    assert i64["converged"] == imx["converged"] == idf["converged"] == 64
    assert imx["accurate_solves"] >= 1 and imx["sensitivity"].shape == (1, 64)
    err_mx = [rel(pmx[0][:, j], p64[0][:, j]) for j in range(len(ks))]
    err_df = [rel(pdf[0][:, j], p64[0][:, j]) for j in range(len(ks))]
    assert max(err_mx) <= 1e-6, f"worst mixed error {max(err_mx):.3e} at ka={ks[int(np.argmax(err_mx))]:.3f}"
    assert max(err_df) <= 1e-10, f"worst double-float error {max(err_df):.3e}"
    # the flagged solves are the ones next to the resonances, and the estimate
    # is the same whether the sweep runs as one graph or launch by launch
    pe, ie = biegpu.sweep([mesh], ks, [w], precision="mixed", refine=True, target_error=1e-6, eager=True)
    np.testing.assert_allclose(ie["sensitivity"], imx["sensitivity"], rtol=1e-3)
    assert ie["accurate_solves"] == imx["accurate_solves"]
    pn, inf = biegpu.sweep([mesh], ks[:4], [w], precision="mixed", refine=True, target_error=0)
    assert inf["accurate_solves"] == 0 and "sensitivity" not in inf


@pytest.mark.parametrize("precision,refine", [("mixed", True), ("fp64", False), ("mixed", False)])
def test_sweep_graph_replay_matches_eager(precision, refine):
    """The recorded CUDA graph (conditional WHILE/SWITCH nodes for the GMRES
    loops) gives the solutions and iteration counts of the host-driven sweep.
    The assemblies add element contributions with atomics, so two runs differ
    by rounding order: ~1e-16 per entry in FP64, ~1e-7 in the FP32 accumulators
    of the mixed form; the solutions are compared at 1e-10 and 1e-6, the
    iteration counts to within two steps."""
    meshes = [bm.icosphere(5), bm.ellipsoid(6)]
    ks = [0.3, 2.5, 5.0 + 0.1j, 7.5]
    rng = np.random.default_rng(11)
    ws = [rng.normal(size=mm.n_sources) + 1j * rng.normal(size=mm.n_sources) for mm in meshes]
    pe, ie = biegpu.sweep(meshes, ks, ws, precision=precision, refine=refine, eager=True)
    pg, ig = biegpu.sweep(meshes, ks, ws, precision=precision, refine=refine)
    assert ie["graph_launches"] == 0 and ig["graph_launches"] == 1   # one launch for the sweep
    assert ig["converged"] == ig["solves"] == 8
    d_it = np.abs(ig["iterations_per_solve"] - ie["iterations_per_solve"])
    assert d_it.max() <= 2
    tol = 1e-10 if precision == "fp64" else 1e-6
    for a, b in zip(pg, pe):
        for j in range(len(ks)):
            assert rel(a[:, j], b[:, j]) <= tol


def test_sweep_graph_small_restart_and_maxiter():
    """restart 3 (many passes through the restart WHILE node) and a maxiter that
    stops the solve early: the replay ends and agrees with the eager sweep
    (FP64 assembly, so the runs differ only by the order of FP64 atomics)."""
    mesh = bm.icosphere(5)
    ks = [1.0, 3.0, 6.0]
    w = np.random.default_rng(3).normal(size=mesh.n_sources) + 0j
    for maxiter in (0, 7):
        kw = dict(precision="fp64", refine=False, restart=3, maxiter=maxiter)
        pe, ie = biegpu.sweep([mesh], ks, [w], eager=True, **kw)
        pg, ig = biegpu.sweep([mesh], ks, [w], **kw)
        np.testing.assert_array_equal(ig["iterations_per_solve"], ie["iterations_per_solve"])
        assert ig["converged"] == ie["converged"]
        if maxiter:
            assert (ig["iterations_per_solve"] == 7).all() and ig["converged"] == 0
        for j in range(len(ks)):
            assert rel(pg[0][:, j], pe[0][:, j]) <= 1e-10
    # the refined mixed path through the same small restart
    pe, ie = biegpu.sweep([mesh], ks, [w], precision="mixed", restart=3, eager=True)
    pg, ig = biegpu.sweep([mesh], ks, [w], precision="mixed", restart=3)
    assert ig["converged"] == ie["converged"] == 3
    for j in range(len(ks)):
        assert rel(pg[0][:, j], pe[0][:, j]) <= 1e-6

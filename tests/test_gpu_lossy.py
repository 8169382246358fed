"""Visco-thermal system on the device (bie_lossy_*) against the oracle's
LossyOuter (dense / sparse matrices with direct solves in place of the nested
gmres calls).  Tolerances: the blocks built from the FP64 assembly and the
near-field rules match the oracle to 1e-12; products that contain nested GMRES
solves (reltol sqrt(eps) each, as the reference's gmres) to 1e-6; the solved
system and the identities of the reference's test/3d/losses_test.jl to 1e-5."""
from __future__ import annotations

import numpy as np
import pytest

import biegpu
from biegpu import mesh as bm
from oracle import lossy as olossy

pytestmark = pytest.mark.gpu

FREQ = 100.0


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def crandn(rng, n):
    return rng.normal(size=n) + 1j * rng.normal(size=n)


_CACHE = {}


def systems(name):
    if name not in _CACHE:
        builders = {
            "linear": lambda: bm.icosphere(3),
            "quadratic": lambda: bm.icosphere(2, geometry="quadratic"),
        }
        mesh = builders[name]()
        L = biegpu.LossyGlobalOuter(mesh, FREQ, depth=1, n=3)
        O = olossy.LossyOuter(mesh, FREQ, depth=1, quad=3)
        _CACHE[name] = (mesh, L, O)
    return _CACHE[name]


@pytest.mark.parametrize("name", ["linear", "quadratic"])
def test_lossy_blocks_match_oracle(name):
    mesh, L, O = systems(name)
    N = mesh.n_sources
    rng = np.random.default_rng(5)
    x = crandn(rng, N)
    q = crandn(rng, 3 * N)
    qs = [q[:N], q[N:2 * N], q[2 * N:]]
    assert rel(L.Ha @ x, O.Ha @ x) <= 1e-12
    assert rel(L.Ga @ x, O.Ga @ x) <= 1e-12
    assert rel(L.Hh @ x, O.Hh @ x) <= 1e-12
    assert rel(L.Gh @ x, O.Gh @ x) <= 1e-12
    assert rel(L.Hv @ q, np.concatenate([O.Av @ v for v in qs])) <= 1e-12
    assert rel(L.Gv @ q, np.concatenate([O.Bv @ v for v in qs])) <= 1e-12
    assert rel(L.Dc @ x, np.concatenate(O.Dc(x))) <= 1e-12
    assert rel(L.Dr @ q, O.Dr(qs)) <= 1e-12
    assert rel(L.Nd @ x, np.concatenate(O.Nd(x))) <= 1e-14
    assert rel(L.NdT @ q, O.NdT(qs)) <= 1e-14
    # constants of the system (test/3d/losses_test.jl:44-45)
    assert abs(L.mu_a - (L.phi_a - L.phi_h * L.tau_a / L.tau_h)) <= 1e-14 * abs(L.mu_a)
    assert abs(L.mu_h - L.phi_h * L.tau_a / L.tau_h) <= 1e-14 * abs(L.mu_h)
    for a, b in [(L.ka, O.ka), (L.kh, O.kh), (L.kv, O.kv), (L.phi_a, O.phi_a), (L.tau_h, O.tau_h)]:
        assert abs(a - b) <= 1e-13 * abs(b)


@pytest.mark.parametrize("name", ["linear", "quadratic"])
def test_lossy_products_match_oracle(name):
    mesh, L, O = systems(name)
    N = mesh.n_sources
    rng = np.random.default_rng(6)
    x = crandn(rng, N)
    assert rel(L.inner @ x, O.inner(x)) <= 1e-6
    y = L @ x
    assert rel(y, O.matvec(x)) <= 1e-6
    st = L.stats(reset=True)
    assert st["nested_solves"] > 0 and st["nested_iterations"] > 0
    # the product twice gives the same vector (no state carried between calls)
    assert rel(L @ x, y) <= 1e-12


@pytest.mark.parametrize("name", ["linear", "quadratic"])
def test_lossy_solve_and_reference_identities(name):
    """The flow of test/3d/losses_test.jl:30-58 on the device."""
    mesh, L, O = systems(name)
    N = mesh.n_sources
    v0 = np.concatenate([0.01 * np.ones(N), np.zeros(2 * N)]).astype(np.complex128)
    rhs = L.rhs(v0)
    assert rel(rhs, O.rhs([v0[:N], v0[N:2 * N], v0[2 * N:]])) <= 1e-6
    pa, info = L.solve(rhs, return_info=True)
    assert info["converged"] == 1
    pa_ref = np.linalg.solve(O.full(), rhs)
    assert rel(pa, pa_ref) <= 1e-5
    dpa = -L.Ga.solve(L.Ha @ pa)
    ph = -L.tau_a / L.tau_h * pa
    dph = -L.Gh.solve(L.Hh @ ph)
    v = v0 - (L.phi_a * (L.Dc @ pa) + L.phi_a * (L.Nd @ dpa) + L.phi_h * (L.Dc @ ph) + L.phi_h * (L.Nd @ dph))
    dvn = -L.Gv.solve(L.Hv @ v)
    assert rel(L.Hh @ ph, -(L.Gh @ dph)) <= 1e-6
    assert rel(L.Ha @ pa, -(L.Ga @ dpa)) <= 1e-6
    assert rel(L.Hv @ v, -(L.Gv @ dvn)) <= 1e-6
    assert rel(L.tau_a * pa, -L.tau_h * ph) <= 1e-12
    lhs = L.phi_a * (L.Dc @ pa + L.Nd @ dpa) + L.phi_h * (L.Dc @ ph + L.Nd @ dph) + v
    assert rel(lhs, v0) <= 1e-12


def _sparse_runs(L, N, modes, seed=11):
    rng = np.random.default_rng(seed)
    b1, b3 = crandn(rng, N), crandn(rng, 3 * N)
    x = crandn(rng, N)
    runs = {}
    for mode in modes:
        L.set_one_launch(mode)
        r = {}
        for blk, b in (("Gh", b1), ("Hh", b1), ("Gv", b3), ("Hv", b3)):
            r[blk] = getattr(L, blk).solve(b, return_info=True)
        # a restart after every step and a step limit below what the tolerance needs
        r["short"] = L.Gv.solve(b3, reltol=1e-15, restart=1, maxiter=3, return_info=True)
        L.stats(reset=True)
        L.ctx.stats(reset=True)
        r["product"] = L @ x
        r["launches"] = L.ctx.stats(reset=True)["kernel_launches"]
        r["stats"] = L.stats(reset=True)
        runs[mode] = r
    L.set_one_launch(True)
    return runs, (b1, b3, x)


def _same_solves(ref, got):
    for blk in ("Gh", "Hh", "Gv", "Hv", "short"):
        (x0, i0), (x1, i1) = ref[blk], got[blk]
        for key in ("iterations", "restarts", "matvecs", "converged"):
            assert i0[key] == i1[key], (blk, key, i0[key], i1[key])
        assert rel(x1, x0) <= 1e-7, blk
        assert abs(i1["residual_norm"] - i0["residual_norm"]) <= 1e-6 * i0["rhs_norm"]
    short = got["short"][1]
    assert short["iterations"] <= 3 and short["restarts"] == short["iterations"]
    assert short["converged"] == 1 or short["iterations"] == 3
    assert rel(got["product"], ref["product"]) <= 1e-7
    assert got["stats"] == ref["stats"]
    assert got["launches"] < ref["launches"]


@pytest.mark.parametrize("name", ["linear", "quadratic"])
def test_one_launch_sparse_solves(name):
    """The sparse thermal / viscous solves as one launch (bie_lossy_set_one_launch:
    thread-block cluster, cooperative grid) against the launch-per-operation
    device GMRES and the oracle's sparse direct solves: the same iterations,
    restarts and products, solutions within the GMRES tolerance of each other
    (1e-7) and of the direct solve (1e-6), fewer launches per product."""
    mesh, L, O = systems(name)
    N = mesh.n_sources
    runs, (b1, b3, x) = _sparse_runs(L, N, ("off", "cluster", "grid"))
    for mode in ("cluster", "grid"):
        _same_solves(runs["off"], runs[mode])
    one = runs["cluster"]
    ref = {"Gh": O._gh.solve(b1), "Hh": np.linalg.solve(O.Hh.toarray(), b1),
           "Gv": np.concatenate([O._bv.solve(b3[k * N:(k + 1) * N]) for k in range(3)]),
           "Hv": np.concatenate([np.linalg.solve(O.Av.toarray(), b3[k * N:(k + 1) * N]) for k in range(3)])}
    for blk, xr in ref.items():
        assert one[blk][1]["converged"] == 1
        assert rel(one[blk][0], xr) <= 1e-6, blk
    assert rel(one["product"], O.matvec(x)) <= 1e-6
    assert one["launches"] <= 1000


def test_one_launch_sparse_solves_2562():
    """The bench's 2562-node sphere (3N = 7686 rows: the grid form spread over
    the SMs; the automatic choice) against the launch-per-operation GMRES."""
    mesh = bm.icosphere(16)
    L = biegpu.LossyGlobalOuter(mesh, FREQ, depth=1, n=3)
    runs, _ = _sparse_runs(L, mesh.n_sources, ("off", "auto", "cluster"), seed=12)
    _same_solves(runs["off"], runs["auto"])
    _same_solves(runs["off"], runs["cluster"])
    assert runs["auto"]["launches"] <= 100
    L.close()


def test_lossy_fast_acoustic_operators():
    """fmm_on = true: the acoustic blocks by the fast-operator algorithm."""
    mesh = bm.icosphere(3)
    L = biegpu.LossyGlobalOuter(mesh, FREQ, depth=1, n=3, fmm_on=True)
    O = olossy.LossyOuter(mesh, FREQ, depth=1, quad=3, fmm_on=True)
    x = crandn(np.random.default_rng(8), mesh.n_sources)
    assert rel(L.Ha @ x, O.Ha @ x) <= 1e-10
    assert rel(L.Ga @ x, O.Ga @ x) <= 1e-10
    assert rel(L.Hh @ x, O.Hh @ x) <= 1e-12
    assert rel(L @ x, O.matvec(x)) <= 1e-6


def test_lossy_interior_and_errors():
    mesh = bm.icosphere(3)
    L = biegpu.LossyGlobalOuter(mesh, FREQ, depth=1, n=3, exterior=False)
    O = olossy.LossyOuter(mesh, FREQ, depth=1, quad=3, exterior=False)
    x = crandn(np.random.default_rng(9), mesh.n_sources)
    assert rel(L.Ha @ x, O.Ha @ x) <= 1e-12
    assert rel(L.Hv @ np.concatenate([x, x, x]), np.concatenate([O.Av @ x] * 3)) <= 1e-12
    assert rel(L @ x, O.matvec(x)) <= 1e-6
    with pytest.raises(ValueError):
        L.Dc.solve(x)
    with pytest.raises(ValueError):
        L.Ha @ np.zeros(mesh.n_sources + 1)
    with pytest.raises(biegpu.BIEError):
        biegpu.LossyGlobalOuter(mesh, -1.0)

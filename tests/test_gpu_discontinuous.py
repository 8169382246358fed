"""Discontinuous triangle physics (DiscontinuousTriangularConstant / Linear /
Quadratic on linear and quadratic geometry, src/3d/surface_functions.jl:236-318,
src/3d/mesh.jl:115-214) through the GPU paths, against the CPU oracle.

The oracle's discontinuous restatement is pinned to the reference's own
rigid-sphere error table (tests/test_oracle_pins.py).  Tolerances: FP64
assembly and products <= 1e-12 relative Frobenius / 2-norm error, mixed
precision <= 1e-6, GMRES solutions <= 1e-6 against a dense direct solve of
the oracle's system, tensor-core multi-RHS products <= 1e-5."""
from __future__ import annotations

import numpy as np
import pytest

import biegpu
import oracle
import oracle.analytic as an
from biegpu import Diagonal, GPUFOperator, GPUGOperator, gmres
from biegpu import _capi
from biegpu import mesh as bm
from biegpu.assembly import sparse_assemble_parallel

pytestmark = pytest.mark.gpu

COMBOS = [(go, po) for go in ("linear", "quadratic") for po in bm.DISCONTINUOUS]


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def rand_c(n, seed):
    r = np.random.default_rng(seed)
    return r.normal(size=n) + 1j * r.normal(size=n)


def disc_mesh(go, po, f=None):
    return bm.icosphere(f or (3 if go == "linear" else 2), geometry=go, physics=po)


@pytest.mark.parametrize("go,po", COMBOS)
def test_fp64_assembly_matches_oracle(go, po):
    mesh = disc_mesh(go, po)
    for k in (2.0, 1.5 + 0.5j):
        F, G, C = biegpu.assemble_parallel(mesh, k, n=2, m=2)
        Fo, Go, Co = oracle.assemble(mesh, k, n=2, m=2)
        for a, b, name in [(F, Fo, "F"), (G, Go, "G"), (C, Co, "C")]:
            assert a.shape == b.shape
            assert rel(a, b) <= 1e-12, f"{name}: {rel(a, b):.3e}"


@pytest.mark.parametrize("go,po", COMBOS)
def test_mixed_assembly_and_field_points(go, po):
    mesh = disc_mesh(go, po)
    F, G, C = biegpu.assemble_parallel(mesh, 3.0, n=2, m=2, precision="mixed")
    Fo, Go, Co = oracle.assemble(mesh, 3.0, n=2, m=2)
    assert max(rel(F, Fo), rel(G, Go), rel(C, Co)) <= 1e-6
    z = np.linspace(0.1, 0.9, 12)
    X = np.vstack([0.03 + 0 * z, 0.05 + 0 * z, z])
    F, G, C = biegpu.assemble_parallel(mesh, 3.0, X, n=2, m=2)
    Fo, Go, Co = oracle.assemble(mesh, 3.0, targets=X, n=2, m=2)
    assert max(rel(F, Fo), rel(G, Go), rel(C, Co)) <= 1e-12


@pytest.mark.parametrize("go,po", [("linear", "disctriconstant"), ("linear", "disctriquadratic"),
                                   ("quadratic", "disctrilinear")])
def test_matrix_free_products(go, po):
    mesh = disc_mesh(go, po)
    k = 2.5
    F, G, _ = oracle.assemble(mesh, k, n=2, m=2, cOn=False)
    x, v = rand_c(mesh.n_sources, 1), rand_c(mesh.n_sources, 2)
    for prec, tol in (("fp64", 1e-12), ("mixed", 1e-6)):
        assert rel(GPUFOperator(mesh, k, precision=prec) @ x, F @ x) <= tol
        assert rel(GPUGOperator(mesh, k, precision=prec) @ v, G @ v) <= tol
    X = np.stack([rand_c(mesh.n_sources, 10 + j) for j in range(8)], axis=1)
    assert rel(GPUFOperator(mesh, k) @ X, F @ X) <= 1e-5


@pytest.mark.parametrize("go,po", [("linear", "disctrilinear"), ("quadratic", "disctriquadratic")])
def test_rigid_sphere_solve(go, po):
    """assembly_test.jl's system (Fp + Diagonal(1 - Cp)) p = pI on the GPU
    (assembly + GMRES) against the oracle's dense solve and the analytic
    series."""
    mesh = disc_mesh(go, po, f=4 if go == "linear" else 3)
    k = 2 * np.pi * 100 / 340
    Fp, _, Cp = biegpu.assemble_parallel(mesh, k, mesh.sources, n=4, m=4, gOn=False)
    pI = an.incoming_wave([np.pi / 2, 0.0], 1.0, mesh.sources, k)
    x, res = gmres(Fp + Diagonal(1.0 - Cp), pI, ctx=biegpu.get_context(mesh, n=4, m=4), log=True)
    Fo, _, Co = oracle.assemble(mesh, k, n=4, m=4, gOn=False)
    xo = np.linalg.solve(Fo + np.diag(1.0 - Co), pI)
    assert res.converged and rel(x, xo) <= 1e-6
    theta = np.arccos(np.clip(mesh.sources[0], -1, 1))
    pa, _ = an.plane_wave_scattering_sphere(k, 1.0, 1.0, theta, 1e-6)
    assert rel(x, pa) <= 0.05


def test_sweep_on_discontinuous_mesh():
    mesh = disc_mesh("linear", "disctrilinear")
    ks = [0.8, 2.0]
    w = rand_c(mesh.n_sources, 4)
    ps, info = biegpu.sweep([mesh], ks, [w])
    for j, k in enumerate(ks):
        F, G, C = oracle.assemble(mesh, k, n=2, m=2)
        p = np.linalg.solve(F + np.diag(1.0 - C), G @ w)
        assert rel(ps[0][:, j], p) <= 1e-6


def test_explicit_rule_tables():
    """min(NP, 3) tables for linear geometry (nodes 4-6 take table 3)."""
    for go, po in (("linear", "disctriquadratic"), ("linear", "disctriconstant"),
                   ("quadratic", "disctriquadratic")):
        mesh = disc_mesh(go, po)
        NP = mesh.physics_topology.shape[0]
        nt = min(NP, 3) if go == "linear" else NP
        ctx = biegpu.Context(mesh, rules=[oracle.rule(2, 2, r) for r in range(1, nt + 1)])
        F, G, C = ctx.assemble(1.2)
        Fo, Go, Co = oracle.assemble(mesh, 1.2, n=2, m=2)
        assert max(rel(F, Fo), rel(G, Go), rel(C, Co)) <= 1e-12


def test_unsupported_paths_are_rejected():
    mesh = disc_mesh("linear", "disctrilinear")
    with pytest.raises(biegpu.BIEError) as e:
        sparse_assemble_parallel(mesh, 1.0)
    assert e.value.code == _capi.BIE_ERR_UNSUPPORTED
    with pytest.raises(biegpu.BIEError) as e:
        biegpu.FMMFOperator(mesh, 1.0)
    assert e.value.code == _capi.BIE_ERR_UNSUPPORTED

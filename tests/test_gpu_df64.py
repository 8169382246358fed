"""Double-float assembly (BIE_PREC_DF64, kernel K9) against the CPU oracle
and the FP64 GPU assembly.  Tolerance: the FP64 parity bar, <= 1e-12 relative
Frobenius error against the oracle for F, G and C (the double-float
arithmetic itself is good to ~1e-14), on linear and quadratic geometry,
continuous and discontinuous physics, real and complex k, collocation and
field points."""
from __future__ import annotations

import numpy as np
import pytest

import biegpu
import oracle
from biegpu import mesh as bm

pytestmark = pytest.mark.gpu
TOL = 1e-12


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def check(mesh, k, n=2, m=2, targets=None, tol=TOL):
    F, G, C = biegpu.assemble_parallel(mesh, k, targets, n=n, m=m, precision="df64")
    Fo, Go, Co = oracle.assemble(mesh, k, targets=targets, n=n, m=m)
    errs = {name: rel(a, b) for a, b, name in [(F, Fo, "F"), (G, Go, "G"), (C, Co, "C")]}
    for name, e in errs.items():
        assert e <= tol, f"{name}: {e:.3e}"
    return errs


@pytest.mark.parametrize("geo,phys,f,k", [("linear", "geometry", 6, 3.0), ("linear", "geometry", 4, 0.5),
                                          ("quadratic", "geometry", 4, 5.0), ("quadratic", "linear", 4, 2.0),
                                          ("linear", "disctrilinear", 3, 2.5),
                                          ("quadratic", "disctriquadratic", 2, 2.0),
                                          ("linear", "disctriconstant", 4, 1.0)])
def test_df64_matches_oracle(geo, phys, f, k):
    errs = check(bm.icosphere(f, geometry=geo, physics=phys), k)
    # well inside the FP64 bar: the double-float arithmetic is good to ~1e-14
    assert max(errs.values()) <= 1e-13


@pytest.mark.parametrize("k", [1.0 + 0.5j, 3.0 + 0.2j])
def test_df64_complex_wavenumber(k):
    check(bm.icosphere(5), k)
    check(bm.icosphere(3, geometry="quadratic"), k)


def test_df64_field_points_and_quadrature_orders():
    z = np.linspace(0.1, 0.9, 20)
    X = np.vstack([0.02 + 0 * z, 0.05 + 0 * z, z])
    check(bm.icosphere(5), 2.0, targets=X)
    check(bm.icosphere(3, geometry="quadratic"), 2.0, n=4, m=4)
    check(bm.ellipsoid(5), 4.0, n=3, m=2)
    # far field points (radius 10): phases k r up to ~60.  C (the solid-angle
    # term) vanishes there up to the quadrature error (~1e-12), so it is
    # compared absolutely against the size of its terms (~1e-5)
    rng = np.random.default_rng(2)
    Y = rng.normal(size=(3, 16))
    Y *= 10.0 / np.linalg.norm(Y, axis=0)
    mesh = bm.ellipsoid(5)
    F, G, C = biegpu.assemble_parallel(mesh, 6.0, Y, n=2, m=2, precision="df64")
    Fo, Go, Co = oracle.assemble(mesh, 6.0, targets=Y, n=2, m=2)
    assert rel(F, Fo) <= TOL and rel(G, Go) <= TOL
    assert np.max(np.abs(C - Co)) <= 1e-16


def test_df64_matches_fp64_gpu_at_size():
    """A 4842-node P2-geometry ellipsoid at ka = 10: df64 against the FP64
    kernel (<= 1e-13; the two differ only in arithmetic)."""
    mesh = bm.icosphere(11, geometry="quadratic", axes=(1.0, 2 / 3, 1 / 3))
    F, G, C = biegpu.assemble_parallel(mesh, 10.0, n=2, m=2, precision="df64")
    F64, G64, C64 = biegpu.assemble_parallel(mesh, 10.0, n=2, m=2, precision="fp64")
    assert max(rel(F, F64), rel(G, G64), rel(C, C64)) <= 1e-13


def test_df64_falls_back_to_fp64_for_large_element_phase():
    """|k| x element radius beyond the Taylor tables: the FP64 kernel runs
    instead (same result)."""
    mesh = bm.icosphere(2)
    check(mesh, 60.0)


def test_df64_with_caller_rule_tables():
    mesh = bm.icosphere(3, geometry="quadratic")
    ctx = biegpu.Context(mesh, rules=[oracle.rule(3, 2, r) for r in range(1, 7)])
    F, G, C = ctx.assemble(2.5, precision="df64")
    Fo, Go, Co = oracle.assemble(mesh, 2.5, n=3, m=2)
    assert max(rel(F, Fo), rel(G, Go), rel(C, Co)) <= TOL


def test_df64_rejects_nothing_the_fp64_path_takes():
    mesh = bm.icosphere(3)
    ctx = biegpu.Context(mesh, n=2, m=2)
    F, G, C = ctx.assemble(1.5, precision="df64", gOn=False)
    Fo, _, Co = oracle.assemble(mesh, 1.5, n=2, m=2, gOn=False)
    assert G is None and rel(F, Fo) <= TOL and rel(C, Co) <= TOL


def test_df64_host_call_with_row_blocks():
    """The host-buffer call pipelines row blocks (outputs >= 256 MB): each
    block is its own double-float assembly with its own widening pass."""
    mesh = bm.icosphere(24)          # 5762 nodes: 2 x 531 MB of complex128
    ctx = biegpu.Context(mesh, n=2, m=2)
    F, G, C = ctx.assemble(2.0, precision="df64")
    F64, G64, C64 = ctx.assemble(2.0, precision="fp64")
    assert max(rel(F, F64), rel(G, G64), rel(C, C64)) <= 1e-13


@pytest.mark.parametrize("geo,f,k,phys", [("linear", 6, 3.0, "geometry"), ("quadratic", 4, 5.0, "geometry"),
                                          ("linear", 5, 2.0 + 0.5j, "geometry"),
                                          ("quadratic", 3, 1.0 + 0.3j, "geometry"),
                                          ("linear", 4, 2.0, "disctriconstant"),
                                          ("quadratic", 2, 2.0, "disctriquadratic")])
def test_df64_matrix_free_products(geo, f, k, phys):
    """F x and G v in double-float against the dense oracle product (<= 1e-12)."""
    mesh = bm.icosphere(f, geometry=geo, physics=phys)
    F, G, _ = oracle.assemble(mesh, k, n=2, m=2, cOn=False)
    r = np.random.default_rng(4)
    x = r.normal(size=mesh.n_sources) + 1j * r.normal(size=mesh.n_sources)
    v = r.normal(size=mesh.n_sources) + 1j * r.normal(size=mesh.n_sources)
    Ff = biegpu.GPUFOperator(mesh, k, precision="df64")
    Gf = biegpu.GPUGOperator(mesh, k, precision="df64")
    assert rel(Ff @ x, F @ x) <= TOL
    assert rel(Gf @ v, G @ v) <= TOL
    z = np.linspace(0.1, 0.9, 10)
    X = np.vstack([0 * z, 0.02 + 0 * z, z])
    Fp, Gp, _ = oracle.assemble(mesh, k, targets=X, n=2, m=2, cOn=False)
    assert rel(Ff.evaluate_targets(x, X), Fp @ x) <= TOL
    assert rel(Gf.evaluate_targets(v, X), Gp @ v) <= TOL


def test_df64_matrix_free_gmres():
    """examples/3d_pulsating_sphere.jl's interior system with double-float
    matrix-free products: plain GMRES, and mixed inner iterations refined
    with double-float residuals, against a dense direct solve."""
    mesh = bm.icosphere(5, geometry="quadratic")
    k, Z0 = 1.0, 1.21 * 343.0
    F, G, C = oracle.assemble(mesh, k, n=2, m=2)
    vs = 1j * Z0 * k * np.ones(mesh.n_sources)
    p_dense = np.linalg.solve(np.diag(1.0 - C) - F, G @ vs)
    Ff = biegpu.GPUFOperator(mesh, k, precision="df64")
    b = biegpu.GPUGOperator(mesh, k, precision="df64") @ vs
    x, res = biegpu.gmres(biegpu.Diagonal(1.0 - C) - Ff, b, precision="df64", log=True)
    assert res.converged and rel(x, p_dense) <= 1e-7
    x2, res2 = biegpu.gmres(biegpu.Diagonal(1.0 - C) - biegpu.GPUFOperator(mesh, k, precision="mixed"), b,
                            precision="df64", refine=True, log=True, reltol=1e-12)
    assert res2.converged and rel(x2, p_dense) <= 1e-10


def test_df64_fast_operator_product_and_solve():
    """The fast operator (FMMFOperator algorithm) with its Gauss-rule far field
    in double-float: the same product as its FP64 form (<= 1e-12), and the
    interior pulsating-sphere solve through it."""
    mesh = bm.icosphere(6)
    k = 2.0
    r = np.random.default_rng(6)
    x = r.normal(size=mesh.n_sources) + 1j * r.normal(size=mesh.n_sources)
    op = biegpu.FMMFOperator(mesh, k, precision="fp64")
    y64 = op @ x
    op.precision = "df64"
    ydf = op @ x
    assert rel(ydf, y64) <= TOL
    _, _, C = oracle.assemble(mesh, k, n=2, m=2, fOn=False, gOn=False)
    b = biegpu.GPUGOperator(mesh, k, precision="df64") @ np.ones(mesh.n_sources)
    xs, res = biegpu.gmres(biegpu.Diagonal(1.0 - C) - op, b, precision="df64", log=True, reltol=1e-10)
    op.precision = "fp64"
    x64, res64 = biegpu.gmres(biegpu.Diagonal(1.0 - C) - op, b, precision="fp64", log=True, reltol=1e-10)
    assert res.converged and res64.converged and rel(xs, x64) <= 1e-8


@pytest.mark.parametrize("eager", [False, True])
def test_df64_sweep_matches_fp64_sweep(eager):
    """Sweeps with double-float assembly (recorded graph reading k from device
    memory, or launch by launch) against the plain FP64 sweep."""
    meshes = [bm.icosphere(5), bm.ellipsoid(4, geometry="quadratic")]
    ks = [0.5, 2.0, 4.0 + 0.2j]
    r = np.random.default_rng(8)
    ws = [r.normal(size=m.n_sources) + 1j * r.normal(size=m.n_sources) for m in meshes]
    p64, _ = biegpu.sweep(meshes, ks, ws, precision="fp64", refine=False, eager=eager)
    pdf, info = biegpu.sweep(meshes, ks, ws, precision="df64", refine=False, eager=eager)
    for a, b in zip(pdf, p64):
        assert rel(a, b) <= 1e-10


def test_df64_adjoint_matches_fp64():
    """The adjoint gradient with the forward model assembled in double-float
    (element admittances on G in the double-float kernel and its FP64 near-pair
    correction) against the FP64 forward model."""
    mesh = bm.icosphere(5, axes=(1.0, 2 / 3, 1 / 3))
    r = np.random.default_rng(9)
    Z = 1.21 * 343.0 * np.exp(1j * r.uniform(-1, 1, mesh.n_elements))
    X = r.normal(size=(3, 8))
    X *= 10.0 / np.linalg.norm(X, axis=0)
    J, pf, dX, dZ, _ = biegpu.farfield_objective(mesh, 3.0, Z, X)
    J2, pf2, dX2, dZ2, _ = biegpu.farfield_objective(mesh, 3.0, Z, X, precision="df64")
    assert abs(J2 - J) <= 1e-11 * abs(J)
    assert rel(pf2, pf) <= 1e-11
    assert rel(dX2, dX) <= 1e-10 and rel(dZ2, dZ) <= 1e-10

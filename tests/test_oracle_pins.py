"""Pins the CPU oracle to the reference's own known-answer tests.

* rigid-sphere scattering error table, test/3d/assembly_test.jl:12-44
  (every geometry x physics entry the reference tests, continuous and
  discontinuous physics)
* total quadrature weight = sphere area 4 pi, test/3d/fmm_test.jl:11-28
* rule weights sum to 1/2, test/3d/surface_functions_test.jl:16,37
* mesh sizes, test/3d/meshing_test.jl:23
* entry level: F, G, C at field points against an integration written here
  from the integral definitions (greens3d!, freens3d!, freens3dk0!,
  src/3d/kernels.jl:13-55; the normal -(x_u x x_v)/|x_u x x_v| of jacobian!,
  src/3d/jacobian.jl:63-87; the bases of src/3d/surface_functions.jl:191-300,
  continuous and discontinuous),
  independent of the oracle's rules, nearest-node choice and per-node sums;
  at the mesh's own nodes too (continuous physics), with the singular and
  near-singular elements integrated by rules collapsed at the target, and
  the near field of sparse_assemble_parallel! (adaptive subdivision) within
  the adaptive scheme's accuracy
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
import oracle.analytic as an
from biegpu import mesh as bm

# test/3d/assembly_test.jl:22-23 (geometry x physics)
ERROR_TABLE = {("linear", "linear"): 0.037, ("linear", "disctriconstant"): 0.0073,
               ("linear", "disctrilinear"): 0.0044, ("linear", "disctriquadratic"): 0.004,
               ("quadratic", "linear"): 0.048, ("quadratic", "geometry"): 2.8e-5,
               ("quadratic", "disctriconstant"): 0.0008, ("quadratic", "disctrilinear"): 4.2e-4,
               ("quadratic", "disctriquadratic"): 4.9e-5}


@pytest.mark.parametrize("go,po", list(ERROR_TABLE))
def test_rigid_sphere_error_table(reference_meshes, go, po):
    freq, c = 100.0, 340.0
    k = 2 * np.pi * freq / c
    mesh = bm.load_comsol(reference_meshes / "sphere_1m", go, po)
    assert mesh.topology.shape[1] == 840
    # assemble_parallel!(mesh, k, mesh.sources; gOn=false) with default n = m = 4
    F, _, C = oracle.assemble(mesh, k, n=4, m=4, gOn=False)
    pI = an.incoming_wave([np.pi / 2, 0.0], 1.0, mesh.sources, k)
    A = F + np.diag(1.0 - C)
    p = np.linalg.solve(A, pI)
    theta = np.arccos(np.clip(mesh.sources[0] / 1.0, -1.0, 1.0))
    pa, _ = an.plane_wave_scattering_sphere(k, 1.0, 1.0, theta, 1e-6)
    err = np.linalg.norm(pa - p) / np.linalg.norm(pa)
    assert err <= ERROR_TABLE[(go, po)]


@pytest.mark.parametrize("go,tol", [("linear", 1e-1), ("quadratic", 1e-5)])
def test_sphere_area(reference_meshes, go, tol):
    mesh = bm.load_comsol(reference_meshes / "sphere_1m_extremely_fine", go,
                          "linear" if go == "linear" else "geometry")
    assert abs(oracle.total_weight(mesh, n=2, m=2) - 4 * np.pi) <= tol


def test_oracle_rule_weights():
    for node in range(1, 7):
        for n, m in [(2, 2), (3, 3), (4, 4)]:
            _, _, w = oracle.rule(n, m, node)
            assert abs(w.sum() - 0.5) < 1e-14


def test_oracle_c_is_half_on_smooth_sphere():
    # the k = 0 double layer gives the free term 1/2 on a smooth surface
    mesh = bm.icosphere(4, geometry="quadratic")
    _, _, C = oracle.assemble(mesh, 1.0, n=4, m=4, fOn=False, gOn=False)
    assert np.max(np.abs(C.real - 0.5)) < 5e-3


def test_oracle_rowsum_identity_at_k0():
    # partition of unity: sum_j F(k=0)[i, j] equals C[i] (same rules, same points)
    mesh = bm.icosphere(3)
    F, _, C = oracle.assemble(mesh, 0.0, n=2, m=2, gOn=False)
    assert np.max(np.abs(F.sum(axis=1) - C)) < 1e-12


def test_pulsating_sphere_quadratic():
    # examples/3d_pulsating_sphere.jl: interior field vs the analytic solution
    k = 2 * np.pi * 54.59 / 343.0
    Z0 = 1.21 * 343.0
    mesh = bm.icosphere(5, geometry="quadratic")
    F, G, C = oracle.assemble(mesh, k, n=2, m=2)
    vs = 1j * Z0 * k * np.ones(mesh.n_sources)
    p = np.linalg.solve(np.diag(1.0 - C) - F, G @ vs)
    z = np.linspace(0.1, 0.9, 20)
    X = np.vstack([0 * z, 0 * z, z])
    Fp, Gp, _ = oracle.assemble(mesh, k, targets=X, n=2, m=2)
    pa = an.pulsating_sphere_interior(k, 1.0, Z0, 1.0, z)
    assert np.linalg.norm(Fp @ p + Gp @ vs - pa) / np.linalg.norm(pa) < 5e-3


def test_oracle_taylor_derivatives_match_finite_differences():
    """The k-derivative restatement (taylor_assemble!) is consistent with the
    plain assembly: order 0 equals it, order 1 matches a central difference in k."""
    import oracle
    from biegpu import mesh as bm
    mesh = bm.icosphere(2)
    k0, h = 2.0, 1e-5
    F, G, C = oracle.taylor_assemble(mesh, k0, 2, n=2, m=2)
    F0, G0, C0 = oracle.assemble(mesh, k0, n=2, m=2)
    assert np.array_equal(F[:, :, 0], F0) and np.array_equal(G[:, :, 0], G0) and np.array_equal(C, C0)
    Fp, Gp, _ = oracle.assemble(mesh, k0 + h, n=2, m=2)
    Fm, Gm, _ = oracle.assemble(mesh, k0 - h, n=2, m=2)
    assert np.linalg.norm((Fp - Fm) / (2 * h) - F[:, :, 1]) / np.linalg.norm(F[:, :, 1]) < 1e-8
    assert np.linalg.norm((Gp - Gm) / (2 * h) - G[:, :, 1]) / np.linalg.norm(G[:, :, 1]) < 1e-8


# ---- entry-level pin --------------------------------------------------------

def _tri_linear(u, v):
    one, zero = np.ones_like(u), np.zeros_like(u)
    return np.array([1 - u - v, u, v]), np.array([-one, one, zero]), np.array([-one, zero, one])


def _tri_quadratic(u, v):
    w = 1 - u - v
    N = np.array([w * (1 - 2 * v - 2 * u), u * (2 * u - 1), v * (2 * v - 1), 4 * u * w, 4 * u * v, 4 * v * w])
    dNu = np.array([-(2 * w - 1) - 2 * w, 4 * u - 1, 0 * u, 4 * w - 4 * u, 4 * v, -4 * v])
    dNv = np.array([-(2 * w - 1) - 2 * w, 0 * u, 4 * v - 1, -4 * u, 4 * u, 4 * w - 4 * v])
    return N, dNu, dNv


def _disc_basis(kind, beta, u, v):
    """Discontinuous triangle bases (src/3d/surface_functions.jl:242-300):
    psi(s) = (s - beta) / (1 - 3 beta) of 1 - u - v, u, v."""
    if kind == "disctriconstant":
        return np.ones((1, u.size))
    p3, pu, pv = ((s - beta) / (1 - 3 * beta) for s in (1 - u - v, u, v))
    if kind == "disctrilinear":
        return np.array([p3, pu, pv])
    return np.array([p3 * (2 * p3 - 1), pu * (2 * pu - 1), pv * (2 * pv - 1), 4 * pu * p3, 4 * pu * pv,
                     4 * pv * p3])


def _integrate_definitions(mesh, k, targets, nq=16):
    """F, G, C at off-surface targets by a collapsed nq x nq Gauss-Legendre
    rule on every element (u = a (1 - b), v = a b, weight a)."""
    x, w = np.polynomial.legendre.leggauss(nq)
    x, w = (x + 1) / 2, w / 2
    a, b = (g.ravel() for g in np.meshgrid(x, x, indexing="ij"))
    wt = np.outer(w, w).ravel() * a
    u, v = a * (1 - b), a * b
    geo = _tri_linear if mesh.shape_function == "linear" else _tri_quadratic
    Ng, dNu, dNv = geo(u, v)
    if mesh.physics_function.startswith("disctri"):
        Np = _disc_basis(mesh.physics_function, mesh.physics_beta, u, v)
    else:
        Np = (_tri_linear if mesh.physics_function == "linear" else _tri_quadratic)(u, v)[0]
    M, N = targets.shape[1], mesh.n_sources
    F, G, C = np.zeros((M, N), complex), np.zeros((M, N), complex), np.zeros(M, complex)
    topo, ptopo = mesh.topology - 1, mesh.physics_topology - 1
    for e in range(topo.shape[1]):
        X = mesh.coordinates[:, topo[:, e]]
        xq, cr = X @ Ng, np.cross((X @ dNu).T, (X @ dNv).T).T
        jac = np.linalg.norm(cr, axis=0)
        nrm = -cr / jac
        for i in range(M):
            d = xq - targets[:, i:i + 1]
            r = np.linalg.norm(d, axis=0)
            dn = (d * nrm).sum(axis=0)
            jw = jac * wt
            G[i, ptopo[:, e]] += Np @ (np.exp(1j * k * r) / (4 * np.pi * r) * jw)
            F[i, ptopo[:, e]] += Np @ (np.exp(1j * k * r) * (1j * k * r - 1) * dn / (4 * np.pi * r ** 3) * jw)
            C[i] += np.sum(-dn / (4 * np.pi * r ** 3) * jw)
    return F, G, C


@pytest.mark.parametrize("k", [1.5, 2.0 + 0.3j])
@pytest.mark.parametrize("geometry,physics,f,tol", [("linear", "geometry", 3, 1e-11),
                                                    ("quadratic", "geometry", 2, 1e-8),
                                                    ("quadratic", "linear", 2, 1e-8),
                                                    ("linear", "disctriconstant", 3, 1e-11),
                                                    ("linear", "disctrilinear", 3, 1e-11),
                                                    ("linear", "disctriquadratic", 2, 1e-9),
                                                    ("quadratic", "disctrilinear", 2, 1e-8)])
def test_oracle_entries_match_integral_definitions(geometry, physics, f, tol, k):
    mesh = bm.icosphere(f, geometry=geometry, physics=physics)
    rng = np.random.default_rng(3)
    d = rng.normal(size=(3, 6))
    targets = d / np.linalg.norm(d, axis=0) * np.array([2.0, 2.5, 3.0, 1.6, 4.0, 2.2])
    Fi, Gi, Ci = _integrate_definitions(mesh, k, targets)
    # 8 x 8 rules: the oracle's own quadrature error is below the tolerance
    Fo, Go, Co = oracle.assemble(mesh, k, targets=targets, n=8, m=8)
    assert np.linalg.norm(Fo - Fi) <= tol * np.linalg.norm(Fi)
    assert np.linalg.norm(Go - Gi) <= tol * np.linalg.norm(Gi)
    assert np.max(np.abs(Fo - Fi)) <= 5 * tol * np.max(np.abs(Fi))
    # exterior points: the free term vanishes (Gauss's law) in both
    assert np.max(np.abs(Co - Ci)) <= tol and np.max(np.abs(Ci)) <= 1e-12
    # and the rules the assembly uses by default (n = m = 4) stay within their
    # quadrature error of the definitions
    F4, G4, _ = oracle.assemble(mesh, k, targets=targets, n=4, m=4)
    assert np.linalg.norm(F4 - Fi) <= 2e-4 * np.linalg.norm(Fi)
    assert np.linalg.norm(G4 - Gi) <= 5e-5 * np.linalg.norm(Gi)


# physics node positions of the continuous triangles (get_nodal_nodes_u/v,
# src/3d/SurfaceFunction.jl:426-429)
_NODE_UV = {3: [(0.0, 0.0), (1.0, 0.0), (0.0, 1.0)],
            6: [(0.0, 0.0), (1.0, 0.0), (0.0, 1.0), (0.5, 0.0), (0.5, 0.5), (0.0, 0.5)]}


def _collapsed_rule(P, nq):
    """Points and weights on the reference triangle, split into triangles
    with the common vertex P, each Duffy-collapsed there (integrable 1/r at P)."""
    x, w = np.polynomial.legendre.leggauss(nq)
    x, w = (x + 1) / 2, w / 2
    a, b = (g.ravel() for g in np.meshgrid(x, x, indexing="ij"))
    wt = np.outer(w, w).ravel() * a
    P = np.asarray(P, dtype=float)
    corners = [np.array(c) for c in [(0.0, 0.0), (1.0, 0.0), (0.0, 1.0)]]
    U, V, W = [], [], []
    for i in range(3):
        A, B = corners[i] - P, corners[(i + 1) % 3] - P
        det = abs(A[0] * B[1] - A[1] * B[0])
        if det > 1e-14:
            pts = P[:, None] + a * (A[:, None] * (1 - b) + B[:, None] * b)
            U.append(pts[0]), V.append(pts[1]), W.append(wt * det)
    return np.concatenate(U), np.concatenate(V), np.concatenate(W)


def _integrate_collocation(mesh, k, nq=24):
    """F, G, C at the mesh's own nodes: every element's rule is collapsed at
    the target's node if the element has it, else at the element's node
    nearest the target (near-singular neighbours)."""
    geo = _tri_linear if mesh.shape_function == "linear" else _tri_quadratic
    phys = _tri_linear if mesh.physics_function == "linear" else _tri_quadratic
    topo, ptopo = mesh.topology - 1, mesh.physics_topology - 1
    S, N = mesh.sources, mesh.n_sources
    nuv = _NODE_UV[ptopo.shape[0]]
    F, G, C = np.zeros((N, N), complex), np.zeros((N, N), complex), np.zeros(N, complex)
    for e in range(topo.shape[1]):
        X = mesh.coordinates[:, topo[:, e]]
        for i in range(N):
            own = np.flatnonzero(ptopo[:, e] == i)
            if own.size:
                P = nuv[own[0]]
            else:
                P = nuv[int(np.argmin(np.linalg.norm(S[:, ptopo[:, e]] - S[:, i:i + 1], axis=0)))]
            u, v, wt = _collapsed_rule(P, nq)
            Ng, dNu, dNv = geo(u, v)
            Np = phys(u, v)[0]
            xq, cr = X @ Ng, np.cross((X @ dNu).T, (X @ dNv).T).T
            jac = np.linalg.norm(cr, axis=0)
            d = xq - S[:, i:i + 1]
            r = np.linalg.norm(d, axis=0)
            dn = (d * (-cr / jac)).sum(axis=0)
            jw = jac * wt
            G[i, ptopo[:, e]] += Np @ (np.exp(1j * k * r) / (4 * np.pi * r) * jw)
            F[i, ptopo[:, e]] += Np @ (np.exp(1j * k * r) * (1j * k * r - 1) * dn / (4 * np.pi * r ** 3) * jw)
            C[i] += np.sum(-dn / (4 * np.pi * r ** 3) * jw)
    return F, G, C


@pytest.mark.parametrize("geometry,physics,f,tol", [("linear", "geometry", 2, 1e-12),
                                                    ("quadratic", "geometry", 1, 2e-9),
                                                    ("quadratic", "linear", 1, 1e-11)])
def test_oracle_collocation_entries_match_integral_definitions(geometry, physics, f, tol):
    # on-surface targets: the singular element (Duffy rule at a vertex, two
    # half-Duffy triangles at an edge midpoint) and its near neighbours
    mesh = bm.icosphere(f, geometry=geometry, physics=physics)
    k = 1.5 + 0.2j
    Fi, Gi, Ci = _integrate_collocation(mesh, k)
    Fo, Go, Co = oracle.assemble(mesh, k, n=12, m=12)
    assert np.linalg.norm(Fo - Fi) <= tol * np.linalg.norm(Fi)
    assert np.linalg.norm(Go - Gi) <= tol * np.linalg.norm(Gi)
    assert np.max(np.abs(Co - Ci)) <= tol


@pytest.mark.parametrize("geometry,physics,f", [("linear", "geometry", 3), ("quadratic", "geometry", 2),
                                                ("quadratic", "linear", 2)])
def test_oracle_near_field_matches_integral_definitions(geometry, physics, f):
    # sparse_assemble_parallel! at depth 1 (src/3d/assembly_collocation_losses.jl:
    # 200-405): each node's own elements by adaptive subdivision towards it
    # (singular_triangle_integration, src/3d/adaptive_integration.jl:172-246,
    # 3-point rules, TolE 1e-6), against the same entries integrated here by
    # rules collapsed at the node; the adaptive scheme's accuracy sets the bound
    mesh = bm.icosphere(f, geometry=geometry, physics=physics)
    k = 1.5 + 0.2j
    topo, ptopo = mesh.topology - 1, mesh.physics_topology - 1
    geo = _tri_linear if geometry == "linear" else _tri_quadratic
    phys = _tri_linear if mesh.physics_function == "linear" else _tri_quadratic
    nuv = _NODE_UV[ptopo.shape[0]]
    S, N = mesh.sources, mesh.n_sources
    Fi, Gi = np.zeros((N, N), complex), np.zeros((N, N), complex)
    for e in range(topo.shape[1]):
        X = mesh.coordinates[:, topo[:, e]]
        for a, i in enumerate(ptopo[:, e]):
            u, v, wt = _collapsed_rule(nuv[a], 24)
            Ng, dNu, dNv = geo(u, v)
            Np = phys(u, v)[0]
            xq, cr = X @ Ng, np.cross((X @ dNu).T, (X @ dNv).T).T
            jac = np.linalg.norm(cr, axis=0)
            d = xq - S[:, i:i + 1]
            r = np.linalg.norm(d, axis=0)
            dn = (d * (-cr / jac)).sum(axis=0)
            Gi[i, ptopo[:, e]] += Np @ (np.exp(1j * k * r) / (4 * np.pi * r) * jac * wt)
            Fi[i, ptopo[:, e]] += Np @ (np.exp(1j * k * r) * (1j * k * r - 1) * dn / (4 * np.pi * r ** 3) * jac * wt)
    rp, cols, Fv, Gv = oracle.nearfield(mesh, k, depth=1)
    Fo, Go = np.zeros((N, N), complex), np.zeros((N, N), complex)
    for i in range(N):
        Fo[i, cols[rp[i]:rp[i + 1]]] = Fv[rp[i]:rp[i + 1]]
        Go[i, cols[rp[i]:rp[i + 1]]] = Gv[rp[i]:rp[i + 1]]
    assert np.linalg.norm(Go - Gi) <= 3e-4 * np.linalg.norm(Gi)
    if geometry == "linear":   # flat elements: (x - y).n = 0 on a node's own elements
        assert np.max(np.abs(Fo)) <= 1e-7 * np.max(np.abs(Go)) and np.max(np.abs(Fi)) <= 1e-12
    else:
        assert np.linalg.norm(Fo - Fi) <= 3e-4 * np.linalg.norm(Fi)

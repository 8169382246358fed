"""Adjoint gradients (bie_adjoint): the objective against the oracle's dense
forward model, and the gradients against central finite differences of the
GPU objective, tolerance 1e-5 relative to the largest component.  Steps: 1e-6
for vertex coordinates (small enough that no nearest-node rule choice flips)
and 1e-5 |Z| for impedances (the objective's round-off, ~1e-14, then stays two
decades below the tolerance)."""
from __future__ import annotations

import numpy as np
import pytest

import biegpu
import oracle
from biegpu import mesh as bm

pytestmark = pytest.mark.gpu
RHO_C = 1.21 * 343.0
HZ = 1e-5 * RHO_C


def jittered_ellipsoid(f, seed=0, amp=2e-3):
    # a seeded perturbation breaks the mesh's mirror symmetries, so that no
    # nearest-node choice is an exact tie (the rule is piecewise constant)
    P, T = bm.icosphere_arrays(f)
    P = P * np.array([1.0, 2 / 3, 1 / 3])[:, None]
    P = P + amp * np.random.default_rng(seed).normal(size=P.shape) / f
    return bm._finish(P, T + 1, "linear", "geometry")


def setup(f, nfield=32, seed=1):
    mesh = jittered_ellipsoid(f, seed)
    rng = np.random.default_rng(seed)
    Z = RHO_C * np.exp(1j * rng.uniform(-1.0, 1.0, mesh.n_elements))
    X = rng.normal(size=(3, nfield))
    X *= 10.0 / np.linalg.norm(X, axis=0)
    return mesh, Z, X


def J_of(mesh, k, Z, X):
    return biegpu.farfield_objective(mesh, k, Z, X, rho_c=RHO_C, gradient=False)[0]


def test_objective_matches_oracle():
    mesh, Z, X = setup(4, nfield=8)
    J, pf, _, _, info = biegpu.farfield_objective(mesh, 3.0, Z, X, rho_c=RHO_C, gradient=False)
    Jo, pfo = oracle.farfield_objective(mesh, 3.0, Z, X, rho_c=RHO_C)
    assert info["forward_converged"]
    assert abs(J - Jo) / Jo <= 1e-9
    assert np.linalg.norm(pf - pfo) / np.linalg.norm(pfo) <= 1e-9


def test_gradients_central_differences():
    mesh, Z, X = setup(6)
    k = 3.0
    J, _, dX, dZ, info = biegpu.farfield_objective(mesh, k, Z, X, rho_c=RHO_C)
    assert info["forward_converged"] and info["adjoint_converged"]
    h = 1e-6
    rng = np.random.default_rng(5)
    scale_x = np.max(np.abs(dX))
    for v in rng.choice(mesh.coordinates.shape[1], 4, replace=False):
        for c in range(3):
            P = mesh.coordinates.copy()
            P[c, v] += h
            Jp = J_of(bm._finish(P, mesh.topology, "linear", "geometry"), k, Z, X)
            P[c, v] -= 2 * h
            Jm = J_of(bm._finish(P, mesh.topology, "linear", "geometry"), k, Z, X)
            fd = (Jp - Jm) / (2 * h)
            assert abs(fd - dX[c, v]) <= 1e-5 * scale_x, (v, c, fd, dX[c, v])
    scale_z = np.max(np.abs(dZ))
    for e in rng.choice(mesh.n_elements, 4, replace=False):
        for part in (1.0, 1j):
            Zp = Z.copy(); Zp[e] += part * HZ
            Zm = Z.copy(); Zm[e] -= part * HZ
            fd = (J_of(mesh, k, Zp, X) - J_of(mesh, k, Zm, X)) / (2 * HZ)
            g = dZ[e].real if part == 1.0 else dZ[e].imag
            assert abs(fd - g) <= 1e-5 * scale_z, (e, part, fd, g)


def test_adjoint_full_size_ellipsoid():
    """Shape/impedance workload: ellipsoid 3:2:1, f=22 (4842 nodes), ka=3, 32
    field points on the radius-10 sphere; a few gradient components by FD."""
    mesh, Z, X = setup(22)
    k = 3.0
    J, _, dX, dZ, info = biegpu.farfield_objective(mesh, k, Z, X, rho_c=RHO_C)
    assert info["forward_converged"] and info["adjoint_converged"]
    h = 1e-6
    v, c = 1234, 2
    P = mesh.coordinates.copy()
    P[c, v] += h
    Jp = J_of(bm._finish(P, mesh.topology, "linear", "geometry"), k, Z, X)
    P[c, v] -= 2 * h
    Jm = J_of(bm._finish(P, mesh.topology, "linear", "geometry"), k, Z, X)
    assert abs((Jp - Jm) / (2 * h) - dX[c, v]) <= 1e-5 * np.max(np.abs(dX))
    e = 777
    Zp = Z.copy(); Zp[e] += HZ
    Zm = Z.copy(); Zm[e] -= HZ
    fd = (J_of(mesh, k, Zp, X) - J_of(mesh, k, Zm, X)) / (2 * HZ)
    assert abs(fd - dZ[e].real) <= 1e-5 * np.max(np.abs(dZ))


@pytest.mark.parametrize("f", [3, 5])
def test_gradients_match_forward_mode_through_cpu_assembly(f):
    """The adjoint gradient contracted with random directions against the
    forward-mode (dual-number) derivative of the same objective taken through
    the CPU restatement of the assembly (oracle/forward_mode.py): vertex
    directions (collocation points moving with the vertices) and impedance
    directions.  Both are exact derivatives of the same discrete model, so the
    agreement is limited by the GMRES tolerances (1e-13), not by a step."""
    from oracle import forward_mode as fm
    mesh, Z, X = setup(f, nfield=8)
    k = 3.0
    J, _, dX, dZ, info = biegpu.farfield_objective(mesh, k, Z, X, rho_c=RHO_C)
    assert info["forward_converged"] and info["adjoint_converged"]
    rng = np.random.default_rng(11)
    for _ in range(3):
        V = rng.normal(size=mesh.coordinates.shape)
        Jf, dJ = fm.farfield_directional_derivative(mesh, k, Z, X, Vdir=V, rho_c=RHO_C)
        assert abs(J - Jf) <= 1e-9 * Jf
        g = float(np.sum(dX * V))
        assert abs(g - dJ) <= 1e-8 * max(abs(dJ), np.linalg.norm(dX) * np.linalg.norm(V) * 1e-3)
        dz = rng.normal(size=mesh.n_elements) + 1j * rng.normal(size=mesh.n_elements)
        _, dJz = fm.farfield_directional_derivative(mesh, k, Z, X, dZ=dz, rho_c=RHO_C)
        gz = float(np.sum(dZ.real * dz.real + dZ.imag * dz.imag))
        assert abs(gz - dJz) <= 1e-8 * max(abs(dJz), np.linalg.norm(dZ) * np.linalg.norm(dz) * 1e-3)

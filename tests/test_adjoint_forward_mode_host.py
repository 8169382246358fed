"""The forward-mode (dual-number) restatement of the CPU assembly and far-field
objective (oracle/forward_mode.py) against the C oracle: the objective value,
and directional derivatives against central finite differences of the C
oracle's objective along directions that cross no nearest-node rule switch
(the rule choice is piecewise constant, so a difference across a switch
measures the jump, not the derivative).  CPU only."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from biegpu import mesh as bm
from oracle import forward_mode as fm

RHO_C = 1.21 * 343.0


def jittered_ellipsoid(f, seed=0, amp=2e-3):
    P, T = bm.icosphere_arrays(f)
    P = P * np.array([1.0, 2 / 3, 1 / 3])[:, None]
    P = P + amp * np.random.default_rng(seed).normal(size=P.shape) / f
    return bm._finish(P, T + 1, "linear", "geometry")


def rule_choice(P, T, targets):
    src = P[:, T]
    d2 = np.sum((src[:, :, None, :] - targets[:, None, :, None]) ** 2, axis=0)
    return np.argmin(d2, axis=0)


def smooth_direction(mesh, X, h, rng):
    """A random vertex direction along which no rule choice changes within +-h."""
    T = mesh.topology - 1
    P = mesh.coordinates
    for _ in range(20):
        V = rng.normal(size=P.shape)
        ok = all(np.array_equal(rule_choice(P + s * h * V, T, tg(P + s * h * V)),
                                rule_choice(P, T, tg(P))) for s in (-1, 1) for tg in (lambda Q: Q, lambda Q: X))
        if ok:
            return V
    raise RuntimeError("no direction without rule switches found")


@pytest.fixture(scope="module")
def case():
    mesh = jittered_ellipsoid(3)
    rng = np.random.default_rng(1)
    Z = RHO_C * np.exp(1j * rng.uniform(-1.0, 1.0, mesh.n_elements))
    X = rng.normal(size=(3, 8))
    X *= 10.0 / np.linalg.norm(X, axis=0)
    return mesh, Z, X, rng


def J_oracle(mesh, P, Z, X):
    m2 = bm._finish(P, mesh.topology, "linear", "geometry")
    return oracle.farfield_objective(m2, 3.0, Z, X, rho_c=RHO_C)[0]


def test_forward_mode_objective_value(case):
    mesh, Z, X, _ = case
    J, _ = fm.farfield_directional_derivative(mesh, 3.0, Z, X)
    Jo, _ = oracle.farfield_objective(mesh, 3.0, Z, X, rho_c=RHO_C)
    assert abs(J - Jo) <= 1e-13 * Jo


def test_forward_mode_vertex_derivative_vs_differences(case):
    mesh, Z, X, rng = case
    h = 1e-6
    for _ in range(2):
        V = smooth_direction(mesh, X, h, rng)
        _, dJ = fm.farfield_directional_derivative(mesh, 3.0, Z, X, Vdir=V)
        P = mesh.coordinates
        fd = (J_oracle(mesh, P + h * V, Z, X) - J_oracle(mesh, P - h * V, Z, X)) / (2 * h)
        assert abs(dJ - fd) <= 1e-6 * abs(fd)


def test_forward_mode_impedance_derivative_vs_differences(case):
    mesh, Z, X, rng = case
    dZ = rng.normal(size=mesh.n_elements) + 1j * rng.normal(size=mesh.n_elements)
    _, dJ = fm.farfield_directional_derivative(mesh, 3.0, Z, X, dZ=dZ)
    hz = 1e-5 * RHO_C
    fd = (oracle.farfield_objective(mesh, 3.0, Z + hz * dZ, X, rho_c=RHO_C)[0]
          - oracle.farfield_objective(mesh, 3.0, Z - hz * dZ, X, rho_c=RHO_C)[0]) / (2 * hz)
    assert abs(dJ - fd) <= 1e-6 * abs(fd)

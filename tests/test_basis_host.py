"""Element basis functions on the host (bie_basis) against the reference's
known answers and the oracle: nodal interpolation is the identity for every
triangle kind (test/3d/surface_functions_test.jl:13-88), the basis is a
partition of unity, the derivatives match central differences and the
library's values match the oracle's restatement.  CPU only."""
from __future__ import annotations

import numpy as np
import pytest

import biegpu
import oracle
from biegpu import mesh as bm

KINDS = ["linear", "quadratic", "disctriconstant", "disctrilinear", "disctriquadratic"]
NODES = {"linear": ([0.0, 1.0, 0.0], [0.0, 0.0, 1.0]),
         "quadratic": ([0.0, 1.0, 0.0, 0.5, 0.5, 0.0], [0.0, 0.0, 1.0, 0.0, 0.5, 0.5])}


def nodes_of(kind):
    if kind in NODES:
        return (np.array(a) for a in NODES[kind]), 0.0
    beta = bm.discontinuous_beta(kind)
    return bm.discontinuous_nodes(kind, beta), beta


@pytest.mark.parametrize("kind", KINDS)
def test_nodal_interpolation_is_identity(kind):
    (u, v), beta = nodes_of(kind)
    N, _, _ = biegpu.basis(kind, u, v, beta)
    assert np.allclose(N, np.eye(len(u)), atol=1e-14)
    assert np.allclose(oracle.basis(kind, u, v, beta), np.eye(len(u)), atol=1e-14)


@pytest.mark.parametrize("kind", KINDS)
def test_partition_of_unity_derivatives_and_oracle(kind):
    rng = np.random.default_rng(7)
    u = rng.uniform(0, 1, 50)
    v = rng.uniform(0, 1, 50) * (1 - u)
    beta = 0.0 if kind in NODES else bm.discontinuous_beta(kind, 0.3)
    N, du, dv = biegpu.basis(kind, u, v, beta)
    assert np.allclose(N.sum(axis=0), 1.0, atol=1e-13)
    assert np.allclose(du.sum(axis=0), 0.0, atol=1e-12) and np.allclose(dv.sum(axis=0), 0.0, atol=1e-12)
    h = 1e-6
    fu = (biegpu.basis(kind, u + h, v, beta)[0] - biegpu.basis(kind, u - h, v, beta)[0]) / (2 * h)
    fv = (biegpu.basis(kind, u, v + h, beta)[0] - biegpu.basis(kind, u, v - h, beta)[0]) / (2 * h)
    assert np.allclose(du, fu, atol=1e-7) and np.allclose(dv, fv, atol=1e-7)
    assert np.array_equal(N, oracle.basis(kind, u, v, beta))


def test_discontinuous_beta_values():
    # get_beta_tri_linear / get_beta_tri_quadratic (src/3d/mesh.jl:182-214)
    assert bm.discontinuous_beta("disctrilinear") == pytest.approx((1 - 1 / np.sqrt(3)) / 2, abs=1e-15)
    assert bm.discontinuous_beta("disctriquadratic") == pytest.approx((1 - np.sqrt(0.6)) / 2, abs=1e-15)
    assert bm.discontinuous_beta("disctrilinear", "equidistant") == 0.25
    assert bm.discontinuous_beta("disctriquadratic", "equidistant") == pytest.approx(1 / 6)
    assert bm.discontinuous_beta("disctrilinear", 0.3) == 0.15


def test_basis_rejects_bad_arguments():
    with pytest.raises(biegpu.BIEError):
        biegpu.basis("disctrilinear", [0.2], [0.2], beta=0.5)
    with pytest.raises(ValueError):
        biegpu.basis("linear", [0.2, 0.1], [0.2])

"""Fast operators (bie_fastop_*): the FMMFOperator / FMMGOperator algorithm with
an exact far-field sum, against the oracle's dense restatement
(oracle.fast_operator: Gauss-rule far field + accurate-minus-coarse near-field
correction).  FP64 products <= 1e-12 relative, mixed <= 1e-6; evaluate_targets
(far field only) likewise; GMRES on Diagonal(1 - C) - Ff against a dense solve."""
from __future__ import annotations

import numpy as np
import pytest

import biegpu
import oracle
from biegpu import Diagonal, FMMFOperator, FMMGOperator, gmres
from biegpu import mesh as bm

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def rand_c(n, seed):
    r = np.random.default_rng(seed)
    return r.normal(size=n) + 1j * r.normal(size=n)


@pytest.mark.parametrize("geo,f,k,depth,offset", [("linear", 5, 3.0, 1, 0.2), ("quadratic", 3, 2.0, 1, 0.2),
                                                   ("linear", 4, 2.0 + 0.4j, 2, 0.0)])
def test_fast_operator_products_match_oracle(geo, f, k, depth, offset):
    mesh = bm.icosphere(f, geometry=geo)
    x = rand_c(mesh.n_sources, 1)
    for which, cls in (("F", FMMFOperator), ("G", FMMGOperator)):
        A = oracle.fast_operator(mesh, k, which, n_gauss=3, depth=depth, offset=offset)
        for prec, tol in (("fp64", 1e-12), ("mixed", 1e-6)):
            op = cls(mesh, k, n_gauss=3, depth=depth, offset=offset, precision=prec)
            assert rel(op @ x, A @ x) <= tol, (which, prec)


def test_fast_operator_without_nearfield_and_targets():
    mesh = bm.icosphere(5)
    k = 2.5
    x = rand_c(mesh.n_sources, 2)
    F, G, _ = oracle.assemble(mesh, k, n=-3, m=1, cOn=False)   # Gauss rule everywhere
    assert rel(FMMFOperator(mesh, k, nearfield=False, precision="fp64") @ x, F @ x) <= 1e-12
    assert rel(FMMGOperator(mesh, k, nearfield=False, precision="fp64") @ x, G @ x) <= 1e-12
    z = np.linspace(0.2, 0.8, 9)
    X = np.vstack([0 * z, 0.1 + 0 * z, z])
    Fp, Gp, _ = oracle.assemble(mesh, k, targets=X, n=-3, m=1, cOn=False)
    assert rel(FMMFOperator(mesh, k, precision="fp64").evaluate_targets(x, X), Fp @ x) <= 1e-12
    assert rel(FMMGOperator(mesh, k, precision="fp64").evaluate_targets(x, X), Gp @ x) <= 1e-12


def test_gmres_on_fast_operator():
    # pulsating-sphere pattern (examples/3d_pulsating_sphere.jl:46-50) with the
    # fast operator in place of FMMFOperator
    mesh = bm.icosphere(6)
    k = 2.0
    _, _, Cv = biegpu.assemble_parallel(mesh, k, mesh.sources, n=2, m=2, fOn=False, gOn=False)
    Ff = FMMFOperator(mesh, k, precision="fp64")
    b = rand_c(mesh.n_sources, 3)
    x, res = gmres(Diagonal(1.0 - Cv) - Ff, b, log=True, reltol=1e-12, restart=60)
    assert res.converged
    A = np.diag(1.0 - Cv) - oracle.fast_operator(mesh, k, "F")
    assert rel(x, np.linalg.solve(A, b)) <= 1e-9

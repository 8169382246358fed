"""Contexts built from the caller's own quadrature tables
(bie_ctx_create_rules): the tables of the reference's rules (the oracle's
restatement of src/3d/quadrature.jl:70-144) give the oracle's F, G, C; the
assembly is additive over a split of every table, invariant under a
permutation of the points and linear in the weights.  Tolerances: 1e-12
relative Frobenius error against the oracle (FP64, summation order differs),
1e-13 for the exact properties, 1e-6 for mixed precision."""
from __future__ import annotations

import numpy as np
import pytest

import biegpu
import oracle
from biegpu import mesh as bm

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def n_rules(mesh):
    return 3 if mesh.shape_function == "linear" else mesh.physics_topology.shape[0]


def assemble(mesh, rules, k, targets=None, precision="fp64"):
    ctx = biegpu.Context(mesh, rules=rules)
    try:
        return ctx.assemble(k, targets, precision=precision)
    finally:
        ctx.close()


MESHES = {
    "linear": lambda: bm.icosphere(3),
    "quadratic": lambda: bm.icosphere(2, geometry="quadratic"),
    "quadratic_linear_physics": lambda: bm.icosphere(2, geometry="quadratic", physics="linear"),
}


@pytest.mark.parametrize("kind", list(MESHES))
@pytest.mark.parametrize("n,m", [(2, 2), (3, 4)])
def test_reference_tables_match_oracle(kind, n, m):
    mesh = MESHES[kind]()
    rules = [oracle.rule(n, m, r) for r in range(1, n_rules(mesh) + 1)]
    k = 2.0 + 0.25j
    F, G, C = assemble(mesh, rules, k)
    Fo, Go, Co = oracle.assemble(mesh, k, n=n, m=m)
    for a, b, name in [(F, Fo, "F"), (G, Go, "G"), (C, Co, "C")]:
        assert rel(a, b) <= 1e-12, f"{name}: {rel(a, b):.3e}"
    # the same tables through the (n, m) path
    Fb, Gb, Cb = biegpu.Context(mesh, n=n, m=m).assemble(k)
    for a, b in [(F, Fb), (G, Gb), (C, Cb)]:
        assert rel(a, b) <= 1e-14


def test_field_points_and_mixed_precision():
    mesh = bm.icosphere(4)
    rules = [oracle.rule(2, 2, r) for r in (1, 2, 3)]
    z = np.linspace(0.1, 0.9, 16)
    X = np.vstack([0 * z + 0.02, 0.05 + 0 * z, z])
    F, G, C = assemble(mesh, rules, 3.0, targets=X)
    Fo, Go, Co = oracle.assemble(mesh, 3.0, targets=X, n=2, m=2)
    assert max(rel(F, Fo), rel(G, Go), rel(C, Co)) <= 1e-12
    F32, G32, C32 = assemble(mesh, rules, 3.0, precision="mixed")
    Fo, Go, Co = oracle.assemble(mesh, 3.0, n=2, m=2)
    assert max(rel(F32, Fo), rel(G32, Go), rel(C32, Co)) <= 1e-6


@pytest.mark.parametrize("kind", ["linear", "quadratic"])
def test_split_tables_add_up(kind):
    """Splitting every rule at a different point count gives two partial
    assemblies (rules of unequal sizes per node) that add up to the whole."""
    mesh = MESHES[kind]()
    R = n_rules(mesh)
    whole = [oracle.rule(3, 3, r) for r in range(1, R + 1)]
    cut = [1 + (r * 5) % (len(whole[r][0]) - 1) for r in range(R)]
    A = [tuple(a[:c] for a in t) for t, c in zip(whole, cut)]
    B = [tuple(a[c:] for a in t) for t, c in zip(whole, cut)]
    k = 1.5
    Fw, Gw, Cw = assemble(mesh, whole, k)
    Fa, Ga, Ca = assemble(mesh, A, k)
    Fb, Gb, Cb = assemble(mesh, B, k)
    for w, a, b in [(Fw, Fa, Fb), (Gw, Ga, Gb), (Cw, Ca, Cb)]:
        assert rel(a + b, w) <= 1e-13


def test_permuted_points_and_scaled_weights():
    mesh = bm.ellipsoid(3)
    rng = np.random.default_rng(3)
    rules = [oracle.rule(4, 3, r) for r in (1, 2, 3)]
    perm = []
    for u, v, w in rules:
        p = rng.permutation(u.size)
        perm.append((u[p], v[p], w[p]))
    twice = [(u, v, 2.0 * w) for u, v, w in rules]
    F, G, C = assemble(mesh, rules, 2.5)
    Fp, Gp, Cp = assemble(mesh, perm, 2.5)
    F2, G2, C2 = assemble(mesh, twice, 2.5)
    for a, p, t in [(F, Fp, F2), (G, Gp, G2), (C, Cp, C2)]:
        assert rel(p, a) <= 1e-13
        assert rel(t, 2.0 * a) <= 1e-14


def test_one_rule_for_every_node():
    """The same table for every nearest node equals the sum of three
    assemblies that each keep the table for one node and zero the weights of
    the other two (every pair is integrated by exactly one rule)."""
    mesh = bm.icosphere(3)
    t = oracle.rule(3, 3, 2)
    zero = (t[0], t[1], 0.0 * t[2])
    same = assemble(mesh, [t, t, t], 0.7)
    parts = [assemble(mesh, [t if j == i else zero for j in range(3)], 0.7) for i in range(3)]
    for idx in range(3):
        total = parts[0][idx] + parts[1][idx] + parts[2][idx]
        assert rel(total, same[idx]) <= 1e-13

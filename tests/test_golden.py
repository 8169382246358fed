"""Golden vectors (tests/golden/*.npz, written by tests/golden/make_golden.py
from the pinned CPU oracle): the oracle reproduces them (CPU, 1e-13), and the
library's FP64 assembly matches them to the parity tolerance 1e-12 relative
Frobenius error and its mixed assembly to 1e-6 (GPU), on linear and
quadratic geometry with continuous and discontinuous physics, collocation
and field points.  The quadrature tables match to about an ulp (CPU)."""
from __future__ import annotations

import re
from pathlib import Path

import numpy as np
import pytest

import biegpu
import oracle
from biegpu import mesh as bm

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(p.stem[len("assembly_"):] for p in GOLDEN.glob("assembly_*.npz"))


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def load(name):
    z = np.load(GOLDEN / f"assembly_{name}.npz")
    go, po = str(z["geometry"]), str(z["physics"])
    pkind = go if po == "geometry" else po
    coords, topo = z["coordinates"], z["topology"]
    normals = np.zeros_like(z["sources"])
    t1, t2 = normals.copy(), normals.copy()
    mesh = bm.Mesh3d(sources=z["sources"], coordinates=coords, topology=topo, normals=normals, tangents=t1,
                     sangents=t2, shape_function=go, physics_function=pkind,
                     physics_topology=z["physics_topology"], physics_beta=float(z["physics_beta"]))
    return mesh, z


def test_fixtures_present():
    assert len(CASES) >= 9


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_golden(name):
    mesh, z = load(name)
    k, n, m = complex(z["k"]), int(z["n"]), int(z["m"])
    F, G, C = oracle.assemble(mesh, k, n=n, m=m)
    for a, key in ((F, "F"), (G, "G"), (C, "C")):
        assert rel(a, z[key]) <= 1e-13, key
    Fx, Gx, Cx = oracle.assemble(mesh, k, targets=z["X"], n=n, m=m)
    for a, key in ((Fx, "Fx"), (Gx, "Gx"), (Cx, "Cx")):
        assert rel(a, z[key]) <= 1e-13, key


def test_rules_match_golden():
    z = np.load(GOLDEN / "rules.npz")
    for key in z.files:
        n, m, node = (int(t) for t in re.fullmatch(r"n(\d+)m(\d+)_node(\d+)", key).groups())
        # Gauss-Legendre nodes by Newton iteration in long double: the same to
        # about an ulp on every host (x86 80-bit, Arm 128-bit long double)
        assert np.allclose(np.stack(oracle.rule(n, m, node)), z[key], rtol=0, atol=1e-15), key
        assert np.allclose(np.stack(biegpu.quadrature_rule(n, m, node)), z[key], rtol=0, atol=1e-15), key


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_library_matches_golden(name):
    mesh, z = load(name)
    k, n, m = complex(z["k"]), int(z["n"]), int(z["m"])
    ctx = biegpu.Context(mesh, n=n, m=m)
    try:
        F, G, C = ctx.assemble(k)
        for a, key in ((F, "F"), (G, "G"), (C, "C")):
            assert rel(a, z[key]) <= 1e-12, key
        Fx, Gx, Cx = ctx.assemble(k, z["X"])
        for a, key in ((Fx, "Fx"), (Gx, "Gx"), (Cx, "Cx")):
            assert rel(a, z[key]) <= 1e-12, key
        F, G, C = ctx.assemble(k, precision="mixed")
        for a, key in ((F, "F"), (G, "G"), (C, "C")):
            assert rel(a, z[key]) <= 1e-6, key
    finally:
        ctx.close()

"""Writes the golden vectors of tests/test_golden.py from the CPU oracle.

The oracle (oracle/bem_oracle.c) is pinned to the reference's own known
answers (the rigid-sphere error table of test/3d/assembly_test.jl:22-23 on the
shipped sphere_1m mesh, the sphere area of test/3d/fmm_test.jl:11-28, the rule
weight sums and nodal interpolation of test/3d/surface_functions_test.jl); the
Julia reference itself cannot run here.  These fixtures freeze the oracle's
outputs on small synthetic meshes so that the library is checked against
fixed numbers as well as against the oracle built where the tests run.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path[:0] = [str(ROOT / "boundaryintegralequations.jl_gb300"), str(ROOT)]

import oracle  # noqa: E402
from biegpu import mesh as bm  # noqa: E402

OUT = Path(__file__).resolve().parent

# (name, geometry, physics, icosphere frequency, k, n, m)
CASES = [
    ("lin_lin", "linear", "geometry", 2, 2.0, 2, 2),
    ("lin_lin_cplx", "linear", "geometry", 2, 1.5 + 0.5j, 3, 2),
    ("p2_geo", "quadratic", "geometry", 1, 3.0, 2, 2),
    ("p2_lin", "quadratic", "linear", 1, 2.5, 4, 4),
    ("lin_dconst", "linear", "disctriconstant", 2, 2.0, 2, 2),
    ("lin_dlin", "linear", "disctrilinear", 1, 2.0, 2, 2),
    ("lin_dquad", "linear", "disctriquadratic", 1, 1.2, 2, 2),
    ("p2_dlin", "quadratic", "disctrilinear", 1, 2.0, 2, 2),
    ("p2_dquad", "quadratic", "disctriquadratic", 1, 0.8, 2, 2),
]


def field_points():
    z = np.linspace(0.1, 0.9, 5)
    return np.vstack([0.05 + 0 * z, -0.03 + 0 * z, z])


def main():
    for name, go, po, f, k, n, m in CASES:
        mesh = bm.icosphere(f, geometry=go, physics=po)
        F, G, C = oracle.assemble(mesh, k, n=n, m=m)
        X = field_points()
        Fx, Gx, Cx = oracle.assemble(mesh, k, targets=X, n=n, m=m)
        np.savez_compressed(OUT / f"assembly_{name}.npz", geometry=go, physics=po, f=f, k=complex(k), n=n, m=m,
                            coordinates=mesh.coordinates, topology=mesh.topology, sources=mesh.sources,
                            physics_topology=mesh.physics_topology, physics_beta=mesh.physics_beta,
                            F=F, G=G, C=C, X=X, Fx=Fx, Gx=Gx, Cx=Cx)
    rules = {f"n{n}m{m}_node{c}": np.stack(oracle.rule(n, m, c)) for n, m in [(2, 2), (3, 4), (4, 4)]
             for c in range(1, 7)}
    np.savez_compressed(OUT / "rules.npz", **rules)
    print("wrote", len(CASES), "assembly fixtures and", len(rules), "rules to", OUT)


if __name__ == "__main__":
    main()

"""GPU near-field (sparse) assembly against the oracle restatement of
sparse_assemble_parallel! and partial_assemble_parallel!; FP64, relative
2-norm error of the CSR values <= 1e-12."""
from __future__ import annotations

import numpy as np
import pytest

import biegpu
import oracle
from biegpu import mesh as bm
from biegpu.assembly import nearfield_values

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("geo,phys,f", [("linear", "geometry", 4), ("quadratic", "geometry", 3),
                                        ("quadratic", "linear", 3)])
@pytest.mark.parametrize("depth", [1, 2])
def test_nearfield_accurate(geo, phys, f, depth):
    mesh = bm.icosphere(f, geometry=geo, physics=phys)
    ctx = biegpu.get_context(mesh)
    k = 2.0 + 0.1j if depth == 2 else 3.0
    rp, cols, F, G = nearfield_values(ctx, k, depth=depth)
    rpo, colso, Fo, Go = oracle.nearfield(mesh, k, depth=depth)
    assert np.array_equal(rp, rpo) and np.array_equal(cols, colso)
    assert rel(F, Fo) <= 1e-12 and rel(G, Go) <= 1e-12


@pytest.mark.parametrize("offset", [0.2])
def test_nearfield_offset_and_coarse(offset):
    mesh = bm.icosphere(4)
    ctx = biegpu.get_context(mesh)
    _, _, F, G = nearfield_values(ctx, 1.5, offset=offset)
    _, _, Fo, Go = oracle.nearfield(mesh, 1.5, offset=offset)
    assert rel(F, Fo) <= 1e-12 and rel(G, Go) <= 1e-12
    _, _, F, G = nearfield_values(ctx, 1.5, coarse=True, n_gauss=3)
    _, _, Fo, Go = oracle.nearfield(mesh, 1.5, coarse=True, n_gauss=3)
    assert rel(F, Fo) <= 1e-12 and rel(G, Go) <= 1e-12


def test_sparse_assemble_parallel_api():
    mesh = bm.icosphere(3, geometry="quadratic")
    # the dispatcher's default depth is 2 (src/3d/assembly_collocation.jl:259-260)
    F, G = biegpu.assemble_parallel(mesh, 2.0, mesh.sources, sparse=True)
    assert F.shape == (mesh.n_sources, mesh.n_sources)
    rp, cols, Fo, Go = oracle.nearfield(mesh, 2.0, depth=2)
    assert rel(F.data, Fo) <= 1e-12
    # the diagonal (self) entries of G are the largest single-layer values
    assert np.all(np.abs(G.diagonal()) > 0)

"""Mesh builders and the COMSOL reader (host side, no GPU)."""
from __future__ import annotations

import numpy as np
import pytest

from biegpu import mesh as bm


@pytest.mark.parametrize("f", [1, 2, 5, 16, 17])
def test_icosphere_counts(f):
    P, T = bm.icosphere_arrays(f)
    assert P.shape == (3, 10 * f * f + 2)
    assert T.shape == (3, 20 * f * f)
    assert np.allclose(np.linalg.norm(P, axis=0), 1.0)
    # every edge shared by exactly two triangles (closed surface)
    e = np.sort(np.concatenate([T[[0, 1]], T[[1, 2]], T[[2, 0]]], axis=1), axis=0)
    _, cnt = np.unique(e, axis=1, return_counts=True)
    assert np.all(cnt == 2)


def test_icosphere_outward_orientation_and_inward_normals():
    m = bm.icosphere(4)
    X = m.coordinates[:, m.topology - 1]
    n = np.cross(X[:, 1] - X[:, 0], X[:, 2] - X[:, 0], axis=0)
    c = X.mean(axis=1)
    assert np.all(np.sum(n * c, axis=0) > 0)          # counter-clockwise seen from outside
    assert np.all(np.sum(m.normals * m.sources, axis=0) < -0.99)   # negated nodal normals


def test_quadratic_promotion():
    f = 17
    m = bm.icosphere(f, geometry="quadratic")
    V, E = 10 * f * f + 2, 20 * f * f
    assert m.sources.shape == (3, V + 3 * E // 2)    # 2892 vertices + 8670 midpoints = 11562
    assert m.topology.shape == (6, E)
    assert np.allclose(np.linalg.norm(m.coordinates, axis=0), 1.0)
    # midpoint node 4 lies between corners 1 and 2 (before projection)
    X = m.coordinates[:, m.topology - 1]
    mid = 0.5 * (X[:, 0] + X[:, 1])
    mid /= np.linalg.norm(mid, axis=0)
    assert np.allclose(mid, X[:, 3])


def test_linear_physics_on_quadratic_geometry():
    m = bm.icosphere(3, geometry="quadratic", physics="linear")
    assert m.physics_topology.shape[0] == 3
    assert m.sources.shape[1] == 10 * 9 + 2


def test_ellipsoid_axes():
    m = bm.ellipsoid(6)
    ext = m.coordinates.max(axis=1)
    assert np.allclose(ext, [1.0, 2 / 3, 1 / 3], atol=2e-2)


def test_tangents_orthonormal():
    m = bm.icosphere(3)
    assert np.allclose(np.sum(m.normals * m.tangents, axis=0), 0.0, atol=1e-14)
    assert np.allclose(np.sum(m.tangents * m.sangents, axis=0), 0.0, atol=1e-14)


def test_comsol_reader(reference_meshes):
    # test/3d/meshing_test.jl:23 - 840 triangles, physics nodes = sources
    for go in ["linear", "quadratic"]:
        m = bm.load_comsol(reference_meshes / "sphere_1m", go, "linear" if go == "linear" else "geometry")
        assert m.topology.shape[1] == 840
        assert m.sources.shape[1] == len(np.unique(m.physics_topology))
    C, T, ents = bm.read_comsol(reference_meshes / "sphere_1m")
    assert C.shape == (3, 1682) and T.shape == (6, 840)


@pytest.mark.parametrize("go", ["linear", "quadratic"])
@pytest.mark.parametrize("po", ["linear", "quadratic", "disctriconstant", "disctrilinear", "disctriquadratic"])
def test_comsol_mesh_invariants_every_physics(reference_meshes, go, po):
    """test/3d/meshing_test.jl:13-44 for every triangle physics: 840 elements,
    sources = the distinct physics nodes, normals orthogonal to the tangents;
    discontinuous nodes lie inside their element and its geometry."""
    if go == "linear" and po == "quadratic":
        pytest.skip("the reference skips quadratic physics on linear geometry")
    m = bm.load_comsol(reference_meshes / "sphere_1m", go, "geometry" if po == go else po)
    assert m.topology.shape[1] == 840 and m.physics_topology.shape[1] == 840
    assert m.sources.shape == (3, len(np.unique(m.physics_topology)))
    assert m.normals.shape == m.tangents.shape == m.sangents.shape
    assert abs(np.sum(m.normals * m.tangents)) <= 1e-12
    assert abs(np.sum(m.tangents * m.sangents)) <= 1e-12
    if po.startswith("disc"):
        NP = {"disctriconstant": 1, "disctrilinear": 3, "disctriquadratic": 6}[po]
        assert m.n_sources == NP * 840
        # every node of element e is closer to e's centroid than to any vertex
        X = m.coordinates[:, m.topology[:3] - 1]          # 3 x 3 x E
        cen = X.mean(axis=1)
        S = m.sources[:, m.physics_topology - 1]          # 3 x NP x E
        dc = np.linalg.norm(S - cen[:, None, :], axis=0)
        dv = np.min(np.linalg.norm(S[:, :, None, :] - X[:, None, :, :], axis=0), axis=1)
        assert np.all(dc < np.max(np.linalg.norm(X - cen[:, None, :], axis=0), axis=0))
        assert np.all(dv > 0.0)


def test_comsol_native_reader_matches_python(reference_meshes):
    # the C reader (bie_read_comsol) and the Python reader agree on every
    # triangle fixture the reference ships
    n = 0
    for f in sorted(reference_meshes.glob("*.mphtxt")):
        Cp, Tp, Ep = bm.read_comsol(f)
        if Tp.shape[0] not in (3, 6):
            continue   # quadrilateral meshes
        Cn, Tn, En = bm.read_comsol_native(f)
        assert np.array_equal(Cn, Cp) and np.array_equal(Tn, Tp) and np.array_equal(En, Ep), f.name
        n += 1
    assert n >= 5
    a = bm.load_comsol(reference_meshes / "sphere_1m", "quadratic", "geometry", reader="native")
    b = bm.load_comsol(reference_meshes / "sphere_1m", "quadratic", "geometry", reader="python")
    assert np.array_equal(a.topology, b.topology) and np.array_equal(a.sources, b.sources)


MPHTXT = """# Created by hand
0 1
# Mesh vertex coordinates
0 0 0
1 0 0
0 1 0
0.5 0 0
0.5 0.5 0
0 0.5 0

3 # number of vertices per element
# Elements
{elements}

# Geometric entity indices
{entities}

"""


def test_comsol_native_reader_small_files(tmp_path):
    from biegpu import BIEError
    p = tmp_path / "tri6.mphtxt"
    p.write_text(MPHTXT.format(elements="0 1 2 3 4 5 ", entities="1"))
    C, T, E = bm.read_comsol_native(tmp_path / "tri6")          # ".mphtxt" appended
    assert C.shape == (3, 6) and T.tolist() == [[1], [2], [3], [4], [6], [5]] and E.tolist() == [1]
    Cp, Tp, Ep = bm.read_comsol(p)
    assert np.array_equal(C, Cp) and np.array_equal(T, Tp) and np.array_equal(E, Ep)
    p.write_text(MPHTXT.format(elements="0 1 2\n3 4 5", entities="1\n2"))
    C, T, E = bm.read_comsol_native(p)
    assert T.tolist() == [[1, 4], [2, 5], [3, 6]] and E.tolist() == [1, 2]
    for bad in ["0 1 2\n3 4", "0 1 9", "0 1 x", "0 1 2 3"]:
        p.write_text(MPHTXT.format(elements=bad, entities="1"))
        with pytest.raises(BIEError):
            bm.read_comsol_native(p)
    with pytest.raises(BIEError):
        bm.read_comsol_native(tmp_path / "missing.mphtxt")


def test_operator_algebra_on_dense_matrices():
    # the reference's compositions, on host matrices (no GPU involved)
    from biegpu.operators import Diagonal, I, _Affine
    rng = np.random.default_rng(0)
    A = rng.normal(size=(5, 5)) + 1j * rng.normal(size=(5, 5))
    d = rng.normal(size=5) + 0j
    x = rng.normal(size=5) + 1j * rng.normal(size=5)
    op = A + Diagonal(d)
    assert isinstance(op, _Affine)
    assert np.allclose(op @ x, A @ x + d * x)
    op = Diagonal(d) - A
    assert np.allclose(op @ x, d * x - A @ x)
    op = A - Diagonal(d)
    assert np.allclose(op @ x, A @ x - d * x)
    op = _Affine(A) + 0.5 * I
    assert np.allclose(op @ x, A @ x + 0.5 * x)

"""Triangular surface meshes in the layout of BoundaryIntegralEquations.jl's ``Mesh3d``.

``Mesh3d`` (src/utils/mesh.jl:23-34) stores column-major arrays:
``sources`` 3 x N (collocation nodes), ``coordinates`` 3 x N_c, ``topology``
n_shape x E and ``physics_topology`` n_phys x E (both 1-based), plus nodal
``normals``/``tangents``/``sangents`` and the element kinds.  Here the same
arrays are numpy arrays of those shapes; the element kinds are the strings
``"linear"`` (3-node triangle) and ``"quadratic"`` (6-node triangle, nodes
1 2 3 corners, 4 on edge 1-2, 5 on edge 2-3, 6 on edge 3-1), and for the
physics also the discontinuous triangles ``"disctriconstant"``,
``"disctrilinear"``, ``"disctriquadratic"`` (nodes inside each element, offset
``physics_beta`` from the edges; src/3d/SurfaceFunction.jl:81-105, 430-439,
src/3d/surface_functions.jl:236-318).

Builders:
  * :func:`icosphere` - geodesic sphere, each icosahedron face split f x f
    (V = 10 f^2 + 2 vertices, E = 20 f^2 triangles);
  * :func:`promote_quadratic` - 6-node triangles with edge midpoints pushed
    onto the sphere;
  * :func:`ellipsoid` - a sphere mesh scaled to semi-axes (a, b, c);
  * :func:`load_comsol` - COMSOL ``.mphtxt`` reader for triangle meshes
    (src/3d/read_comsol.jl:9-119) with physics ``"geometry"``, ``"linear"`` or
    a discontinuous kind.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

KIND_NODES = {"linear": 3, "quadratic": 6, "disctriconstant": 1, "disctrilinear": 3, "disctriquadratic": 6}
DISCONTINUOUS = ("disctriconstant", "disctrilinear", "disctriquadratic")


@dataclass(eq=False)   # identity hash: contexts are cached per mesh object
class Mesh3d:
    sources: np.ndarray            # 3 x N   collocation nodes
    coordinates: np.ndarray        # 3 x Nc  geometry nodes
    topology: np.ndarray           # NS x E  1-based into coordinates
    normals: np.ndarray            # 3 x N
    tangents: np.ndarray           # 3 x N
    sangents: np.ndarray           # 3 x N
    shape_function: str            # "linear" | "quadratic"
    physics_function: str          # "linear" | "quadratic" | "disctri*"
    physics_topology: np.ndarray   # NP x E  1-based into sources
    entities: np.ndarray = field(default_factory=lambda: np.zeros(0, dtype=np.int64))
    physics_beta: float = 0.0      # node offset of discontinuous physics (0 otherwise)

    @property
    def n_elements(self) -> int:
        return int(self.topology.shape[1])

    @property
    def n_sources(self) -> int:
        return int(self.sources.shape[1])

    def __post_init__(self):
        self.sources = np.ascontiguousarray(self.sources, dtype=np.float64)
        self.coordinates = np.ascontiguousarray(self.coordinates, dtype=np.float64)
        self.topology = np.ascontiguousarray(self.topology, dtype=np.int64)
        self.physics_topology = np.ascontiguousarray(self.physics_topology, dtype=np.int64)


# ---------------------------------------------------------------------------
# Shape functions at the nodal positions (for averaged nodal normals)
# ---------------------------------------------------------------------------
_NODAL_UV = {
    "linear": (np.array([0.0, 1.0, 0.0]), np.array([0.0, 0.0, 1.0])),
    "quadratic": (np.array([0.0, 1.0, 0.0, 0.5, 0.5, 0.0]), np.array([0.0, 0.0, 1.0, 0.0, 0.5, 0.5])),
}


def _shape_derivatives(kind: str, u: np.ndarray, v: np.ndarray):
    """dN/du, dN/dv as (n_shape, len(u)) arrays (src/3d/surface_functions.jl:191-236)."""
    if kind == "linear":
        du = np.array([-1.0, 1.0, 0.0])[:, None] * np.ones_like(u)[None, :]
        dv = np.array([-1.0, 0.0, 1.0])[:, None] * np.ones_like(v)[None, :]
        return du, dv
    l = (1.0 - v) - u
    d1 = -(2.0 * l - 1.0) - 2.0 * l
    du = np.stack([d1, 4 * u - 1, np.zeros_like(u), 4 * l - 4 * u, 4 * v, -4 * v])
    dv = np.stack([d1, np.zeros_like(u), 4 * v - 1, -4 * u, 4 * u, 4 * l - 4 * v])
    return du, dv


def _shape_values(kind: str, u: np.ndarray, v: np.ndarray) -> np.ndarray:
    """N(u, v) as an (n_shape, len(u)) array (src/3d/surface_functions.jl:191-236)."""
    if kind == "linear":
        return np.stack([(1.0 - u) - v, u, v])
    l = (1.0 - v) - u
    return np.stack([l * ((1.0 - 2.0 * v) - 2.0 * u), u * (2.0 * u - 1.0), v * (2.0 * v - 1.0),
                     4.0 * u * l, 4.0 * u * v, 4.0 * v * l])


def discontinuous_beta(kind: str, beta_type="legendre") -> float:
    """Node offset of a discontinuous triangle (set_physics_element /
    get_beta_tri_* of src/3d/mesh.jl:156-214): half the quadrilateral value,
    which is 1 + the first Gauss-Legendre node of 2 (linear) or 3 (quadratic)
    points for "legendre", 1/2 or 1/3 for "equidistant", or the number given."""
    if kind == "disctriconstant":
        return 0.0
    quad = kind == "disctriquadratic"
    if isinstance(beta_type, (int, float)) and not isinstance(beta_type, bool):
        b = float(beta_type)
    elif beta_type == "legendre":
        b = 1.0 + np.polynomial.legendre.leggauss(3 if quad else 2)[0][0]
    elif beta_type == "equidistant":
        b = 1.0 / 3.0 if quad else 0.5
    else:
        raise ValueError(f"unknown beta_type {beta_type!r}")
    return b / 2


def discontinuous_nodes(kind: str, beta: float):
    """(u, v) of the nodes of a discontinuous triangle (src/3d/SurfaceFunction.jl:430-439)."""
    b = float(beta)
    if kind == "disctriconstant":
        return np.array([1 / 3]), np.array([1 / 3])
    if kind == "disctrilinear":
        return np.array([b, 1 - 2 * b, b]), np.array([b, b, 1 - 2 * b])
    if kind == "disctriquadratic":
        return (np.array([b, 1 - 2 * b, b, (1 - b) / 2, (1 - b) / 2, b]),
                np.array([b, b, 1 - 2 * b, b, (1 - b) / 2, (1 - b) / 2]))
    raise ValueError(f"not a discontinuous kind: {kind!r}")


def compute_sources(shape: str, kind: str, beta: float, coordinates: np.ndarray, topology: np.ndarray):
    """Collocation nodes, their normals and the physics topology of
    discontinuous physics (compute_sources, src/3d/mesh.jl:115-145): the nodes
    of element e are sources e*NP+1 .. e*NP+NP, placed by the geometry's
    shape functions, with the negated unit normal of the geometry there."""
    u, v = discontinuous_nodes(kind, beta)
    NP, E = len(u), topology.shape[1]
    N = _shape_values(shape, u, v)                      # NS x NP
    du, dv = _shape_derivatives(shape, u, v)
    X = coordinates[:, topology - 1]                    # 3 x NS x E
    src = np.einsum("kae,ab->kbe", X, N)                # 3 x NP x E
    t1 = np.einsum("kae,ab->kbe", X, du)
    t2 = np.einsum("kae,ab->kbe", X, dv)
    n = np.cross(t1, t2, axis=0)
    n = -n / np.sqrt(np.sum(n**2, axis=0, keepdims=True))
    ptopo = np.arange(1, NP * E + 1, dtype=np.int64).reshape(NP, E, order="F")
    return src.reshape(3, NP * E, order="F").copy(), n.reshape(3, NP * E, order="F").copy(), ptopo


def element_normals(kind: str, coordinates: np.ndarray, topology: np.ndarray) -> np.ndarray:
    """Averaged, normalised and negated nodal normals (src/3d/mesh.jl:78-105)."""
    u, v = _NODAL_UV[kind]
    du, dv = _shape_derivatives(kind, u, v)
    X = coordinates[:, topology - 1]                    # 3 x NS x E
    t1 = np.einsum("kae,ab->kbe", X, du)                # 3 x NS x E
    t2 = np.einsum("kae,ab->kbe", X, dv)
    n = np.cross(t1, t2, axis=0)
    n = n / np.sqrt(np.sum(n**2, axis=0, keepdims=True))
    normals = np.zeros_like(coordinates)
    count = np.zeros(coordinates.shape[1])
    idx = (topology - 1).ravel(order="F")
    nn = n.reshape(3, -1, order="F")
    for k in range(3):
        np.add.at(normals[k], idx, nn[k])
    np.add.at(count, idx, 1.0)
    normals = normals / np.maximum(count, 1.0)
    return -normals / np.sqrt(np.sum(np.abs(normals) ** 2, axis=0, keepdims=True))


def tangents(normals: np.ndarray):
    """Two unit tangents per normal (src/3d/mesh.jl:49-70).  The reference only
    switches basis vectors for normals equal to +e2; normals equal to -e2 are
    switched too here, where the reference would divide by zero."""
    e1 = np.array([1.0, 0.0, 0.0])
    e2 = np.array([0.0, 1.0, 0.0])
    n = normals.T
    t1 = np.cross(e2[None, :], n)
    t2 = np.cross(n, t1)
    flip = np.abs(np.abs(n @ e2) - 1.0) <= 1e-10
    if np.any(flip):
        t2[flip] = np.cross(n[flip], e1[None, :])
        t1[flip] = np.cross(t2[flip], n[flip])
    t1 /= np.linalg.norm(t1, axis=1, keepdims=True)
    t2 /= np.linalg.norm(t2, axis=1, keepdims=True)
    return t1.T.copy(), t2.T.copy()


def _finish(coordinates, topology, shape, physics, beta_type="legendre") -> Mesh3d:
    """Build the Mesh3d for physics 'geometry' (same nodes), 'linear' (corners
    only) or a discontinuous kind, following load3dTriangularComsolMesh
    (src/3d/read_comsol.jl:61-119)."""
    beta = 0.0
    if physics in DISCONTINUOUS:
        beta = discontinuous_beta(physics, beta_type)
        sources, normals, ptopo = compute_sources(shape, physics, beta, coordinates, topology)
        pkind = physics
    elif physics in ("geometry", shape):
        normals = element_normals(shape, coordinates, topology)
        sources = coordinates[:, np.unique(topology) - 1]
        ptopo = topology
        pkind = shape
    elif physics == "linear":
        normals = element_normals(shape, coordinates, topology)
        ptopo = topology[:3, :]
        used = np.unique(ptopo)
        normals = normals[:, used - 1]
        sources = coordinates[:, used - 1]
        if used[-1] != len(used):
            raise ValueError("corner nodes must be numbered first for linear physics on quadratic geometry")
        pkind = "linear"
    else:
        raise ValueError(f"unsupported physics order {physics!r}")
    t1, t2 = tangents(normals)
    return Mesh3d(sources=sources, coordinates=coordinates, topology=topology, normals=normals,
                  tangents=t1, sangents=t2, shape_function=shape, physics_function=pkind,
                  physics_topology=ptopo.copy(), physics_beta=beta)


# ---------------------------------------------------------------------------
# Geodesic spheres
# ---------------------------------------------------------------------------
def _icosahedron():
    p = (1.0 + 5.0**0.5) / 2.0
    V = np.array([[-1, p, 0], [1, p, 0], [-1, -p, 0], [1, -p, 0],
                  [0, -1, p], [0, 1, p], [0, -1, -p], [0, 1, -p],
                  [p, 0, -1], [p, 0, 1], [-p, 0, -1], [-p, 0, 1]], dtype=np.float64)
    F = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    return V, F


def icosphere_arrays(f: int, radius: float = 1.0):
    """Vertices (3 x V) and 0-based counter-clockwise (outward) triangles (3 x E)."""
    if f < 1:
        raise ValueError("f must be >= 1")
    V0, F0 = _icosahedron()
    index: dict = {}
    pts: list = []

    def node(key, xyz):
        j = index.get(key)
        if j is None:
            j = len(pts)
            index[key] = j
            pts.append(xyz)
        return j

    tris = []
    for fi, (a, b, c) in enumerate(F0):
        A, B, C = V0[a], V0[b], V0[c]
        ids = {}
        for i in range(f + 1):
            for j in range(f + 1 - i):
                xyz = A + (B - A) * (i / f) + (C - A) * (j / f)
                k = f - i - j
                # canonical keys: corners by vertex id, edge points by (lo, hi, steps from lo)
                if i == 0 and j == 0:
                    key = ("v", a)
                elif i == f:
                    key = ("v", b)
                elif j == f:
                    key = ("v", c)
                elif j == 0:
                    key = ("e", min(a, b), max(a, b), i if a < b else f - i)
                elif i == 0:
                    key = ("e", min(a, c), max(a, c), j if a < c else f - j)
                elif k == 0:
                    key = ("e", min(b, c), max(b, c), j if b < c else f - j)
                else:
                    key = ("f", fi, i, j)
                ids[(i, j)] = node(key, xyz)
        for i in range(f):
            for j in range(f - i):
                tris.append((ids[(i, j)], ids[(i + 1, j)], ids[(i, j + 1)]))
                if i + j + 1 < f:
                    tris.append((ids[(i + 1, j)], ids[(i + 1, j + 1)], ids[(i, j + 1)]))
    P = np.array(pts)
    P = radius * P / np.linalg.norm(P, axis=1, keepdims=True)
    return P.T.copy(), np.array(tris, dtype=np.int64).T.copy()


def promote_quadratic_arrays(coords: np.ndarray, tris: np.ndarray, radius: float | None = 1.0):
    """Add edge midpoints (6-node triangles).  Vertices keep their numbers, the
    midpoints follow in order of first appearance.  With ``radius`` set the
    midpoints are pushed onto the sphere of that radius."""
    E = tris.shape[1]
    nv = coords.shape[1]
    mids: dict = {}
    new = []
    t6 = np.zeros((6, E), dtype=np.int64)
    t6[:3] = tris
    for e in range(E):
        for slot, (p, q) in zip((3, 4, 5), ((0, 1), (1, 2), (2, 0))):
            a, b = int(tris[p, e]), int(tris[q, e])
            key = (min(a, b), max(a, b))
            j = mids.get(key)
            if j is None:
                j = nv + len(new)
                mids[key] = j
                x = 0.5 * (coords[:, a] + coords[:, b])
                if radius is not None:
                    x = radius * x / np.linalg.norm(x)
                new.append(x)
            t6[slot, e] = j
    C = np.concatenate([coords, np.array(new).T], axis=1)
    return C, t6


def icosphere(f: int, radius: float = 1.0, geometry: str = "linear", physics: str = "geometry",
              axes: tuple[float, float, float] | None = None, beta_type="legendre") -> Mesh3d:
    """Geodesic sphere (optionally scaled to an ellipsoid with semi-axes ``axes``)."""
    P, T = icosphere_arrays(f, radius)
    if geometry == "quadratic":
        P, T = promote_quadratic_arrays(P, T, radius)
    elif geometry != "linear":
        raise ValueError("geometry must be 'linear' or 'quadratic'")
    if axes is not None:
        P = P * (np.asarray(axes, dtype=np.float64)[:, None] / radius)
    return _finish(P, T + 1, geometry, physics, beta_type)


def ellipsoid(f: int, axes=(1.0, 2.0 / 3.0, 1.0 / 3.0), geometry: str = "linear",
              physics: str = "geometry") -> Mesh3d:
    """Ellipsoid with semi-axes ``axes`` (default 3:2:1 with the longest equal to 1)."""
    return icosphere(f, 1.0, geometry=geometry, physics=physics, axes=axes)


# ---------------------------------------------------------------------------
# COMSOL .mphtxt
# ---------------------------------------------------------------------------
def read_comsol(path: str | Path):
    """Coordinates (3 x Nc), 1-based topology and entities of a COMSOL text mesh
    (src/3d/read_comsol.jl:9-54), including the swap of 6-node rows 5 and 6."""
    path = Path(path)
    if path.suffix != ".mphtxt":
        path = path.with_name(path.name + ".mphtxt")
    lines = path.read_text().splitlines()
    coords, topo, ents = [], [], []
    i = 0
    while i < len(lines):
        line = lines[i]
        i += 1
        if len(line) < 4:
            continue
        if line == "# Mesh vertex coordinates":
            while i < len(lines) and lines[i].strip():
                coords.append([float(t) for t in lines[i].split()])
                i += 1
        elif line == "# Elements":
            while i < len(lines) and lines[i].strip():
                topo.append([int(t) for t in lines[i].split()])
                i += 1
        elif line == "# Geometric entity indices":
            while i < len(lines) and lines[i].strip():
                ents.append(int(lines[i].split()[0]))
                i += 1
    C = np.array(coords, dtype=np.float64).T.copy()
    T = np.array(topo, dtype=np.int64).T.copy() + 1
    if T.shape[0] == 6:
        T[[4, 5], :] = T[[5, 4], :]
    return C, T, np.array(ents, dtype=np.int64)


def read_comsol_native(path: str | Path):
    """:func:`read_comsol` through libbiegpu's C reader (bie_read_comsol)."""
    import ctypes as C

    from . import _capi
    L = _capi.lib()
    nc, ne, ni = C.c_int64(), C.c_int64(), C.c_int64()
    npe = C.c_int32()
    p = str(path).encode()
    _capi.check(L.bie_read_comsol(p, C.byref(nc), C.byref(ne), C.byref(npe), C.byref(ni), None, None, None))
    coords = np.empty((3, nc.value), dtype=np.float64, order="F")
    topo = np.empty((npe.value, ne.value), dtype=np.int64, order="F")
    ents = np.empty(ni.value, dtype=np.int64)
    _capi.check(L.bie_read_comsol(p, C.byref(nc), C.byref(ne), C.byref(npe), C.byref(ni), coords.ctypes.data,
                                  topo.ctypes.data, ents.ctypes.data))
    return np.ascontiguousarray(coords), np.ascontiguousarray(topo), ents


def _remove_unused_nodes(topology: np.ndarray) -> np.ndarray:
    used = np.unique(topology)
    remap = np.zeros(int(used.max()) + 1, dtype=np.int64)
    remap[used] = np.arange(1, len(used) + 1)
    return remap[topology]


def load_comsol(path: str | Path, geometry_order: str = "quadratic", physics_order: str = "geometry",
                reader: str = "native", beta_type="legendre") -> Mesh3d:
    """load3dTriangularComsolMesh for physics 'geometry', 'linear' or a
    discontinuous kind; ``reader`` "native" parses the file with libbiegpu's C
    reader, "python" in Python."""
    if reader not in ("native", "python"):
        raise ValueError("reader must be 'native' or 'python'")
    C0, T0, ents = read_comsol_native(path) if reader == "native" else read_comsol(path)
    if geometry_order == "linear":
        T0 = T0[:3, :]
    elif geometry_order != "quadratic":
        raise ValueError("geometry_order must be 'linear' or 'quadratic'")
    used = np.unique(T0)
    T = _remove_unused_nodes(T0)
    C = C0[:, used - 1]
    m = _finish(C, T, geometry_order, physics_order, beta_type)
    m.entities = ents
    return m

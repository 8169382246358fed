"""Element slicing of the assembly kernels on the host (bie_element_slicing;
no GPU): the element order and the node counts of the mixed assembly's write
protocol, against a numpy restatement written here.

The emulation at the end drives one row of the mixed assembly through the
flags and slot indices the library builds and checks that every entry gets
its plain sum, written once.

The kernels process elements in the order of a recursive coordinate bisection
of their centroids: the range [num*E/den, (num+1)*E/den) is split at
(2 num + 1)*E/(2 den) across the longest side of its centroids' bounding box
(ties by element index) until it holds at most two elements, which go in
Morton order of their centroids (10 bits per axis, ties by index).  Slice s
of 2^l covers positions [s*E/2^l, (s+1)*E/2^l).  A node touched by two or
more slices is shared (one side slot per slice that touches it); a node of
one slice with several contributions gets one of 16 ring slots, assigned per
slice in order of last position to the slot freed latest before the node's
first position (strictly), else it is widened afterwards.
"""
from __future__ import annotations

import numpy as np
import pytest

import biegpu
from biegpu import mesh as bm

RING_SLOTS = 16


def _spread10(v):
    v = v.astype(np.uint32) & 0x3FF
    v = (v | (v << 16)) & 0x30000FF
    v = (v | (v << 8)) & 0x300F00F
    v = (v | (v << 4)) & 0x30C30C3
    v = (v | (v << 2)) & 0x9249249
    return v


def bisection_order(mesh):
    """0-based element order (restatement)."""
    topo = mesh.topology - 1
    X = mesh.coordinates
    E = topo.shape[1]
    cen = (X[:, topo[0]] + X[:, topo[1]] + X[:, topo[2]]) / 3.0
    lo, hi = X.min(axis=1), X.max(axis=1)
    key = np.zeros(E, dtype=np.uint64)
    for k in range(3):
        span = hi[k] - lo[k]
        t = (cen[k] - lo[k]) / span if span > 0 else np.zeros(E)
        q = np.clip(t * 1023.0, 0.0, 1023.0).astype(np.uint32)
        key |= (_spread10(q) << k).astype(np.uint64)
    order = np.arange(E)
    pending = [(0, E, 0, 1)]
    while pending:
        p0, p1, num, den = pending.pop()
        seg = order[p0:p1]
        if p1 - p0 <= 2:
            order[p0:p1] = seg[np.lexsort((seg, key[seg]))]
            continue
        c = cen[:, seg]
        ext = c.max(axis=1) - c.min(axis=1)
        ax = int(np.argmax(ext))   # first of equal extents, as the strict > of the library
        mid = (2 * num + 1) * E // (2 * den)
        order[p0:p1] = seg[np.lexsort((seg, cen[ax, seg]))]
        pending.append((mid, p1, 2 * num + 1, 2 * den))
        pending.append((p0, mid, 2 * num, 2 * den))
    return order


def slicing_counts(mesh, order, level):
    """(shared, side_slots, ring, widened, single, untouched) at `level` (restatement)."""
    ptopo = mesh.physics_topology - 1
    NP, E = ptopo.shape
    N = mesh.n_sources
    S = 1 << level
    slices = [set() for _ in range(N)]
    first, last = {}, {}
    for s in range(S):
        for p in range(s * E // S, (s + 1) * E // S):
            for nd in ptopo[:, order[p]]:
                slices[nd].add(s)
                first.setdefault((nd, s), p)
                last[(nd, s)] = p
    shared = {nd for nd in range(N) if len(slices[nd]) > 1}
    side = sum(len(slices[nd]) for nd in shared)
    ring = widened = single = untouched = 0
    spans = {s: [] for s in range(S)}
    for nd in range(N):
        if not slices[nd]:
            untouched += 1
        elif nd not in shared:
            (s,) = slices[nd]
            f, l = first[(nd, s)], last[(nd, s)]
            if f == l:
                single += 1
            else:
                spans[s].append((l, nd, f))
    for s in range(S):
        free_at = [-1] * RING_SLOTS
        for l, _nd, f in sorted(spans[s]):
            best = -1
            for k in range(RING_SLOTS):
                if free_at[k] < f and (best < 0 or free_at[k] > free_at[best]):
                    best = k
            if best < 0:
                widened += 1
            else:
                free_at[best] = l
                ring += 1
    return len(shared), side, ring, widened, single, untouched


MESHES = {
    "sphere_p2_f6": lambda: bm.icosphere(6, geometry="quadratic"),
    "sphere_p1_f8": lambda: bm.icosphere(8),
    "ellipsoid_p1_f6": lambda: bm.ellipsoid(6),
    "sphere_disclinear_f4": lambda: bm.icosphere(4, physics="disctrilinear"),
}


@pytest.fixture(scope="module", params=sorted(MESHES))
def mesh(request):
    return MESHES[request.param]()


def test_order_is_the_bisection_of_centroids(mesh):
    order, _ = biegpu.element_slicing(mesh, 0)
    assert order.dtype == np.int32 and order.shape == (mesh.n_elements,)
    assert np.array_equal(np.sort(order), np.arange(1, mesh.n_elements + 1))
    assert np.array_equal(order - 1, bisection_order(mesh))
    again, _ = biegpu.element_slicing(mesh, 5)
    assert np.array_equal(order, again)


@pytest.mark.parametrize("level", [0, 2, 4, 5, 6, 7])
def test_node_counts_match_restatement(mesh, level):
    _, got = biegpu.element_slicing(mesh, level)
    want = slicing_counts(mesh, bisection_order(mesh), level)
    assert tuple(got[k] for k in biegpu.assembly.SLICING_COUNTS) == want
    assert got["shared"] + got["ring"] + got["widened"] + got["single"] + got["untouched"] == mesh.n_sources
    assert got["side_slots"] >= 2 * got["shared"]


def test_bisection_shares_fewer_nodes_than_morton_order():
    mesh = bm.icosphere(12, geometry="quadratic")
    order, got = biegpu.element_slicing(mesh, 6)
    topo = mesh.topology - 1
    X = mesh.coordinates
    cen = (X[:, topo[0]] + X[:, topo[1]] + X[:, topo[2]]) / 3.0
    lo, hi = X.min(axis=1), X.max(axis=1)
    key = np.zeros(mesh.n_elements, dtype=np.uint64)
    for k in range(3):
        q = np.clip((cen[k] - lo[k]) / (hi[k] - lo[k]) * 1023.0, 0, 1023).astype(np.uint32)
        key |= (_spread10(q) << k).astype(np.uint64)
    morton = np.lexsort((np.arange(mesh.n_elements), key))
    shared_morton = slicing_counts(mesh, morton, 6)[0]
    assert got["shared"] < 0.8 * shared_morton


def test_discontinuous_constant_nodes_have_one_contribution():
    mesh = bm.icosphere(3, physics="disctriconstant")
    for level in (0, 3, 7):
        _, got = biegpu.element_slicing(mesh, level)
        assert got == {"shared": 0, "side_slots": 0, "ring": 0, "widened": 0,
                       "single": mesh.n_sources, "untouched": 0}


def _tiny_mesh(extra_source: bool):
    coords = np.array([[0.0, 1.0, 0.0], [0.0, 0.0, 1.0], [0.0, 0.0, 0.0]])
    topo = np.array([[1], [2], [3]], dtype=np.int64)
    src = coords.copy()
    if extra_source:
        src = np.concatenate([src, [[5.0], [5.0], [5.0]]], axis=1)
    z = np.zeros_like(src)
    return bm.Mesh3d(sources=src, coordinates=coords, topology=topo, normals=z, tangents=z, sangents=z,
                     shape_function="linear", physics_function="linear", physics_topology=topo.copy())


def test_single_element_and_untouched_node():
    mesh = _tiny_mesh(extra_source=True)
    for level in (0, 7):   # 128 slices of one element: all but one empty
        order, got = biegpu.element_slicing(mesh, level)
        assert order.tolist() == [1]
        assert got == {"shared": 0, "side_slots": 0, "ring": 0, "widened": 0, "single": 3, "untouched": 1}


def test_invalid_arguments_are_reported():
    mesh = _tiny_mesh(extra_source=False)
    for level in (-1, 8):
        with pytest.raises(biegpu.BIEError, match="level"):
            biegpu.element_slicing(mesh, level)
    bad = _tiny_mesh(extra_source=False)
    bad.physics_topology = np.array([[1], [2], [4]], dtype=np.int64)
    with pytest.raises(biegpu.BIEError, match="physics_topology"):
        biegpu.element_slicing(bad, 0)
    bad = _tiny_mesh(extra_source=False)
    bad.coordinates = bad.coordinates.copy()
    bad.coordinates[0, 1] = np.nan
    with pytest.raises(biegpu.BIEError, match="non-finite"):
        biegpu.element_slicing(bad, 0)


def emulate_write_protocol(mesh, level):
    """One row of the mixed assembly under the write protocol the library
    builds (flags and slots of bie_element_slicing), with integer
    contributions so that sums are exact: slices in order, each element's
    nodes through a side slot, a ring slot, the entry's partial sums or a
    direct final write; then the widening and fix-up passes and the zero
    columns.  Returns (entries, expected sums, final writes per node, counts)."""
    order, counts, flags, slots = biegpu.element_slicing(mesh, level, tables=True)
    order = order - 1
    ptopo = mesh.physics_topology - 1
    NP, E = ptopo.shape
    N = mesh.n_sources
    S = 1 << level
    rng = np.random.default_rng(1000 + level)
    contrib = rng.integers(1, 1 << 20, size=(E, NP)).astype(np.float64)
    entry = np.zeros(N)
    writes = np.zeros(N, dtype=np.int64)
    partial = {}
    side, side_of = {}, {}
    seen = np.zeros(N, dtype=bool)
    for s in range(S):
        ring = [None] * RING_SLOTS        # (node, sum) while open
        for p in range(s * E // S, (s + 1) * E // S):
            w = int(flags[p])
            for a in range(NP):
                nd, c = ptopo[a, order[p]], contrib[p, a]
                seen[nd] = True
                first, last = (w >> a) & 1, (w >> (8 + a)) & 1
                shared, ringed = (w >> (16 + a)) & 1, (w >> (24 + a)) & 1
                k = int(slots[a, p])
                assert not (shared and ringed)
                if shared:
                    assert 0 <= k < counts["side_slots"]
                    assert side_of.setdefault(k, (s, nd)) == (s, nd), "side slot reused"
                    assert first or k in side
                    side[k] = c if first else side[k] + c
                elif ringed:
                    assert 0 <= k < RING_SLOTS and not (first and last)
                    if first:
                        assert ring[k] is None, "ring slot still open"
                        ring[k] = (nd, c)
                    else:
                        assert ring[k] is not None and ring[k][0] == nd, "ring slot lost"
                        ring[k] = (nd, ring[k][1] + c)
                    if last:
                        entry[nd] = ring[k][1]
                        writes[nd] += 1
                        ring[k] = None
                else:
                    assert k == -1
                    if first and last:
                        entry[nd] = c
                        writes[nd] += 1
                    else:
                        assert first or nd in partial
                        partial[nd] = c if first else partial[nd] + c
        assert all(r is None for r in ring), "ring slot open at the end of its slice"
    for nd, v in partial.items():          # widening pass
        entry[nd] = v
        writes[nd] += 1
    fix = {}
    for k, (_, nd) in side_of.items():     # fix-up pass
        fix[nd] = fix.get(nd, 0.0) + side[k]
    for nd, v in fix.items():
        entry[nd] = v
        writes[nd] += 1
    writes[~seen] += 1                     # untouched nodes: zero columns
    want = np.zeros(N)
    np.add.at(want, ptopo[:, order].T.ravel(), contrib.ravel())
    return entry, want, writes, counts


@pytest.mark.parametrize("level", range(8))
def test_write_protocol_gives_each_entry_its_sum_once(mesh, level):
    entry, want, writes, counts = emulate_write_protocol(mesh, level)
    assert np.all(writes == 1)
    assert np.array_equal(entry, want)


def test_write_protocol_with_ring_overflow():
    # few slices: more nodes open at once than a block has ring slots, so
    # some nodes take the float partial sums and the widening pass
    mesh = bm.icosphere(12, geometry="quadratic")
    entry, want, writes, counts = emulate_write_protocol(mesh, 2)
    assert counts["widened"] > 0 and counts["ring"] > 0 and counts["shared"] > 0
    assert np.all(writes == 1) and np.array_equal(entry, want)

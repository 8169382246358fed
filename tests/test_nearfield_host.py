"""Near-field set-up on the host (no GPU): libbiegpu's adaptive singular rules
against the oracle's restatement of subdivide_triangle /
singular_triangle_integration (src/3d/adaptive_integration.jl:172-246)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import oracle
from biegpu import _capi


def product_rule(node, offset):
    cap = 32768
    u, v, w = (np.zeros(cap) for _ in range(3))
    cnt = C.c_int()
    _capi.check(_capi.lib().bie_singular_rule(node, offset, u.ctypes.data, v.ctypes.data, w.ctypes.data,
                                              cap, C.byref(cnt)))
    q = cnt.value
    return u[:q], v[:q], w[:q]


@pytest.mark.parametrize("node", [1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("offset", [0.0, 0.2])
def test_singular_rules_match_oracle(node, offset):
    u, v, w = product_rule(node, offset)
    uo, vo, wo = oracle.singular_rule(node, offset)
    assert len(u) == len(uo)
    # same arithmetic in the same order (no FMA contraction on either side): bitwise equal
    assert np.array_equal(u, uo) and np.array_equal(v, vo) and np.array_equal(w, wo)
    assert abs(w.sum() - 0.5) < 1e-13
    assert np.all(u >= -1e-15) and np.all(v >= -1e-15) and np.all(u + v <= 1 + 1e-15)


def test_singular_rule_sizes():
    # corner rules refine 20 levels towards the node; midpoint rules towards an edge point
    assert len(product_rule(1, 0.0)[0]) == 3711
    assert len(product_rule(4, 0.0)[0]) == 10623


def test_connected_sources_depths():
    from biegpu import mesh as bm
    m = bm.icosphere(3)
    e1, s1 = oracle.connected_sources(m, 1)
    e2, s2 = oracle.connected_sources(m, 2)
    # icosphere interior vertex: 6 elements, 7 nodes at depth 1 (5 at the 12 original vertices)
    assert sorted(set(len(x) for x in e1)) == [5, 6]
    assert all(set(a) <= set(b) for a, b in zip(s1, s2))
    assert all(i in s for i, s in enumerate(s1))

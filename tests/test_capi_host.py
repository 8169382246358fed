"""C-ABI checks that need no GPU: the library builds, loads and exports every
declared entry point; host-side validation returns the documented codes."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import biegpu
from biegpu import _capi

HEADER = Path(__file__).resolve().parent.parent / "include" / "biegpu.h"


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"BIE_API\s+[\w\s\*]*?\b(bie_\w+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ["bie_version", "bie_last_error", "bie_ctx_create", "bie_ctx_destroy",
              "bie_assemble", "bie_assemble_device", "bie_quadrature_rule"]:
        assert s in syms


def test_library_exports_every_declared_symbol():
    L = _capi.lib()
    for s in declared_symbols():
        assert hasattr(L, s), f"{s} declared in biegpu.h but not exported"
    # and the Python binding knows every one of them
    assert set(declared_symbols()) <= set(_capi.SIGNATURES)


def _ctypes_kind(t) -> str:
    if t in (C.c_void_p, C.c_char_p) or (isinstance(t, type) and issubclass(t, C._Pointer)):
        return "ptr"
    return {C.c_int32: "i32", C.c_uint32: "i32", C.c_int64: "i64", C.c_uint64: "i64", C.c_double: "f64",
            C.c_float: "f32"}.get(t, "?" + getattr(t, "__name__", str(t)))


def test_ctypes_signatures_match_the_header():
    # each ctypes argument of the same kind (32/64-bit integer, float,
    # double, pointer) as the declared parameter
    from _c_header import header_decls
    decls = header_decls()
    for name, (_res, args) in _capi.SIGNATURES.items():
        assert name in decls, f"{name} has a ctypes signature but no declaration"
        kinds = tuple(_ctypes_kind(a) for a in args)
        assert kinds == decls[name], f"{name}: ctypes {kinds}, C {decls[name]}"


def test_version_and_empty_error():
    L = _capi.lib()
    assert L.bie_version().decode().startswith("biegpu")
    assert isinstance(L.bie_last_error(), bytes)


def test_rule_weights_sum_to_triangle_area():
    # test/3d/surface_functions_test.jl:16,37 - weights add to 0.5
    for node in range(1, 7):
        for n, m in [(1, 1), (2, 2), (3, 3), (4, 4), (2, 5)]:
            u, v, w = biegpu.quadrature_rule(n, m, node)
            assert abs(w.sum() - 0.5) < 1e-14
            assert np.all(u >= 0) and np.all(v >= 0) and np.all(u + v <= 1 + 1e-15)


def test_rule_bad_arguments():
    with pytest.raises(biegpu.BIEError) as e:
        biegpu.quadrature_rule(2, 2, 7)
    assert e.value.code == _capi.BIE_ERR_INVALID


def _desc(mesh, topo=None, ptopo=None, kind=None, n=2, m=2, coords=None):
    coords = np.asfortranarray(mesh.coordinates if coords is None else coords)
    topo = np.asfortranarray(mesh.topology if topo is None else topo, dtype=np.int64)
    ptopo = np.asfortranarray(mesh.physics_topology if ptopo is None else ptopo, dtype=np.int64)
    src = np.asfortranarray(mesh.sources)
    keep = (coords, topo, ptopo, src)
    d = _capi.MeshDesc(coords.shape[1], coords.ctypes.data_as(C.POINTER(C.c_double)), topo.shape[1],
                       _capi.KIND[mesh.shape_function] if kind is None else kind,
                       _capi.KIND[mesh.physics_function],
                       topo.ctypes.data_as(C.POINTER(C.c_int64)),
                       ptopo.ctypes.data_as(C.POINTER(C.c_int64)), src.shape[1],
                       src.ctypes.data_as(C.POINTER(C.c_double)), n, m)
    return d, keep


@pytest.mark.parametrize("case", ["topo_zero", "topo_high", "ptopo_high", "nan", "bad_kind", "bad_quad"])
def test_ctx_create_rejects_invalid_mesh(case):
    """Validation runs on the host before any device call, so these need no GPU."""
    mesh = biegpu.icosphere(2)
    kw = {}
    if case == "topo_zero":
        t = mesh.topology.copy(); t[0, 3] = 0; kw["topo"] = t
    elif case == "topo_high":
        t = mesh.topology.copy(); t[2, 5] = mesh.coordinates.shape[1] + 1; kw["topo"] = t
    elif case == "ptopo_high":
        t = mesh.physics_topology.copy(); t[1, 1] = mesh.sources.shape[1] + 7; kw["ptopo"] = t
    elif case == "nan":
        c = mesh.coordinates.copy(); c[1, 4] = np.nan; kw["coords"] = c
    elif case == "bad_kind":
        kw["kind"] = 9
    elif case == "bad_quad":
        kw["n"] = 0
    d, keep = _desc(mesh, **kw)
    h = C.c_void_p()
    st = _capi.lib().bie_ctx_create(C.byref(h), C.byref(d), 0)
    assert st in (_capi.BIE_ERR_INVALID, _capi.BIE_ERR_UNSUPPORTED)
    assert h.value is None
    assert len(_capi.lib().bie_last_error()) > 0


def test_null_context_is_rejected():
    L = _capi.lib()
    st = L.bie_assemble(None, 1.0, 0.0, None, 0, 7, 0, None, None, None)
    assert st == _capi.BIE_ERR_INVALID
    assert b"NULL" in L.bie_last_error()
    assert L.bie_ctx_destroy(None) == _capi.BIE_OK


def _tables(rules):
    keep = [tuple(np.ascontiguousarray(a, dtype=np.float64) for a in r) for r in rules]
    tabs = (_capi.RuleTable * max(len(keep), 1))(*[
        _capi.RuleTable(r[0].size, r[0].ctypes.data_as(C.POINTER(C.c_double)),
                        r[1].ctypes.data_as(C.POINTER(C.c_double)),
                        r[2].ctypes.data_as(C.POINTER(C.c_double))) for r in keep])
    return tabs, keep


@pytest.mark.parametrize("case", ["count", "outside", "nan", "empty", "too_many", "null"])
def test_ctx_create_rules_rejects_invalid_tables(case):
    """bie_ctx_create_rules validates the caller's rule tables on the host
    before any device call (so these need no GPU)."""
    mesh = biegpu.icosphere(2)
    rules = [biegpu.quadrature_rule(2, 2, r) for r in (1, 2, 3)]
    if case == "count":
        rules = rules[:2]
    elif case == "outside":
        u, v, w = (a.copy() for a in rules[1]); u[0] = 0.9; v[0] = 0.2; rules[1] = (u, v, w)
    elif case == "nan":
        u, v, w = (a.copy() for a in rules[2]); w[3] = np.nan; rules[2] = (u, v, w)
    elif case == "empty":
        rules[0] = (np.zeros(0), np.zeros(0), np.zeros(0))
    elif case == "too_many":
        rules[0] = (np.full(65, 0.1), np.full(65, 0.1), np.full(65, 0.5 / 65))
    tabs, keep = _tables(rules)
    if case == "null":
        tabs[1].v = C.POINTER(C.c_double)()
    d, keep_mesh = _desc(mesh, n=0, m=0)      # (n, m) are ignored with explicit tables
    h = C.c_void_p()
    st = _capi.lib().bie_ctx_create_rules(C.byref(h), C.byref(d), tabs, len(rules), 0)
    assert st == _capi.BIE_ERR_INVALID
    assert h.value is None
    assert len(_capi.lib().bie_last_error()) > 0


@pytest.mark.parametrize("beta", [0.0, 1.0 / 3.0, -0.1, float("nan")])
def test_ctx_create_rejects_bad_discontinuous_beta(beta):
    """Discontinuous linear/quadratic physics need 0 < beta < 1/3 (checked on
    the host before any device call)."""
    mesh = biegpu.icosphere(2, physics="disctrilinear")
    d, keep = _desc(mesh)
    d.physics_beta = beta
    h = C.c_void_p()
    assert _capi.lib().bie_ctx_create(C.byref(h), C.byref(d), 0) == _capi.BIE_ERR_INVALID
    assert h.value is None


def test_discontinuous_kinds_and_unsupported_host_paths():
    mesh = biegpu.icosphere(2, geometry="quadratic", physics="disctriquadratic")
    assert mesh.physics_topology.shape == (6, mesh.n_elements)
    assert mesh.n_sources == 6 * mesh.n_elements
    # quadratic geometry: the nodes lie on the sphere (interpolated by the
    # 6-node map, so only approximately on it)
    assert np.allclose(np.linalg.norm(mesh.sources, axis=0), 1.0, atol=2e-2)
    with pytest.raises(biegpu.BIEError) as e:
        biegpu.tangential_derivatives(mesh)
    assert e.value.code == _capi.BIE_ERR_UNSUPPORTED
    # geometry must be a continuous kind
    d, keep = _desc(mesh, kind=_capi.BIE_TRI_DISC_LINEAR)
    h = C.c_void_p()
    assert _capi.lib().bie_ctx_create(C.byref(h), C.byref(d), 0) == _capi.BIE_ERR_UNSUPPORTED

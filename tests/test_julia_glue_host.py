"""The Julia glue's `ccall`s against the C header and the built library.

Julia is not installed here, so the glue (julia/src/BIEGPU.jl and the
package extension) cannot run; this test reads it as text.  Every
`ccall((:name, libbiegpu), Ret, (T1, ..., Tn), ...)` must name an entry point
that include/biegpu.h declares and libbiegpu.so exports, with one argument
type per declared parameter and of the same kind (32- or 64-bit integer,
float, double, pointer).  The struct layouts the calls pass are checked in
test_abi_layout.py.
"""
from __future__ import annotations

import re
from pathlib import Path

from _c_header import _balanced, _split_top, header_decls
from biegpu import _capi

ROOT = Path(__file__).resolve().parent.parent
JULIA_DIR = ROOT / "boundaryintegralequations.jl_gb300" / "julia"


def julia_ccalls() -> dict[str, set[tuple[str, ...]]]:
    """Per entry point, the argument kinds of every call site."""
    src = "\n".join(re.sub(r"#.*", "", p.read_text()) for p in sorted(JULIA_DIR.rglob("*.jl")))
    calls: dict[str, set[tuple[str, ...]]] = {}
    for m in re.finditer(r"ccall\(\(:(\w+),\s*libbiegpu\),", src):
        rest = src[m.end():]
        # return type, then the argument type tuple
        i = 0
        depth = 0
        while not (rest[i] == "," and depth == 0):
            depth += rest[i] in "({["
            depth -= rest[i] in ")}]"
            i += 1
        j = i + 1
        while rest[j].isspace():
            j += 1
        types, _ = _balanced(rest, j)
        calls.setdefault(m.group(1), set()).add(tuple(_julia_kind(t) for t in _split_top(types)))
    return calls


_JULIA_SCALARS = {"Cint": "i32", "Int32": "i32", "Cuint": "i32", "UInt32": "i32", "Int64": "i64",
                  "Clonglong": "i64", "UInt64": "i64", "Csize_t": "i64", "Cdouble": "f64", "Float64": "f64",
                  "Cfloat": "f32", "Float32": "f32"}


def _julia_kind(t: str) -> str:
    t = t.strip()
    if t.startswith(("Ptr{", "Ref{")) or t in ("Cstring", "Ptr"):
        return "ptr"
    return _JULIA_SCALARS.get(t, "?" + t)


def test_every_julia_ccall_matches_a_declared_exported_entry():
    calls = julia_ccalls()
    decls = header_decls()
    lib = _capi.lib()   # builds the library first if it is missing
    assert len(calls) >= 20, sorted(calls)
    for name, sites in sorted(calls.items()):
        assert name in decls, f"{name} is called from Julia but not declared in biegpu.h"
        assert hasattr(lib, name), f"{name} is not exported by libbiegpu.so"
        for kinds in sites:
            assert kinds == decls[name], f"{name}: Julia passes {kinds}, C takes {decls[name]}"


def test_parser_reads_known_signatures():
    decls = header_decls()
    assert decls["bie_version"] == ()
    assert decls["bie_element_slicing"] == ("ptr", "i32", "ptr", "ptr", "ptr", "ptr")
    assert decls["bie_ctx_create"] == ("ptr", "ptr", "i32")
    assert decls["bie_assemble"][1:3] == ("f64", "f64")
    assert all("?" not in k for kinds in decls.values() for k in kinds), decls
    calls = julia_ccalls()
    assert calls["bie_ctx_destroy"] == {("ptr",)}
    assert calls["bie_element_slicing"] == {("ptr", "i32", "ptr", "ptr", "ptr", "ptr")}

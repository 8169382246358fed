"""Layout of the public C structs against their Python (ctypes) and Julia
mirrors.

tests/abi_layout.c prints, for every struct of include/biegpu.h that crosses
the C ABI, its size and the offset and size of each leaf field (nested structs
and arrays flattened).  The ctypes classes of biegpu._capi and the isbits
structs of the Julia glue (julia/src/BIEGPU.jl, which `ccall` passes by
reference) must give the same leaves: a field added to a C struct without its
mirrors, or a type that changes a size or alignment, fails here.  Julia cannot
run in this test, so its layout is computed from the struct definitions with
the C alignment rules that Julia applies to isbits structs.
"""
from __future__ import annotations

import ctypes as C
import re
import shutil
import subprocess
from pathlib import Path

import pytest

from biegpu import _capi

ROOT = Path(__file__).resolve().parent.parent
JULIA = ROOT / "boundaryintegralequations.jl_gb300" / "julia" / "src" / "BIEGPU.jl"

PY = {"bie_mesh_desc": _capi.MeshDesc, "bie_rule_table": _capi.RuleTable, "bie_stats": _capi.Stats,
      "bie_peaks": _capi.Peaks, "bie_operator": _capi.Operator, "bie_gmres_opts": _capi.GmresOpts,
      "bie_gmres_info": _capi.GmresInfo, "bie_sweep_opts": _capi.SweepOpts, "bie_sweep_info": _capi.SweepInfo,
      "bie_adjoint_opts": _capi.AdjointOpts, "bie_adjoint_info": _capi.AdjointInfo,
      "bie_lossy_constants": _capi.LossyConstants, "bie_lossy_opts": _capi.LossyOpts,
      "bie_multisolve_opts": _capi.MultisolveOpts, "bie_multisolve_info": _capi.MultisolveInfo}
JL = {"bie_mesh_desc": "MeshDesc", "bie_rule_table": "RuleTable", "bie_operator": "OperatorC",
      "bie_gmres_opts": "GmresOptsC", "bie_gmres_info": "GmresInfoC", "bie_sweep_opts": "SweepOpts",
      "bie_sweep_info": "SweepInfo", "bie_adjoint_opts": "AdjointOpts", "bie_adjoint_info": "AdjointInfo",
      "bie_lossy_opts": "LossyOpts", "bie_multisolve_opts": "MultisolveOpts",
      "bie_multisolve_info": "MultisolveInfo"}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = tmp_path_factory.mktemp("abi") / "abi_layout"
    subprocess.run([cc, "-std=c99", "-I", str(ROOT / "include"), str(ROOT / "tests" / "abi_layout.c"), "-o",
                    str(exe)], check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    lay = {}
    for line in out.splitlines():
        name, size, *leaves = line.split()
        lay[name] = (int(size), [tuple(int(v) for v in x.split(":")) for x in leaves])
    return lay


def _ctypes_leaves(cls, base=0):
    out = []
    for name, typ in cls._fields_:
        off = base + getattr(cls, name).offset
        if isinstance(typ, type) and issubclass(typ, C.Structure):
            out += _ctypes_leaves(typ, off)
        elif isinstance(typ, type) and issubclass(typ, C.Array):
            es = C.sizeof(typ._type_)
            out += [(off + i * es, es) for i in range(typ._length_)]
        else:
            out.append((off, C.sizeof(typ)))
    return out


def test_ctypes_mirrors(c_layout):
    assert set(PY) <= set(c_layout)
    for cname, cls in PY.items():
        size, leaves = c_layout[cname]
        assert C.sizeof(cls) == size, cname
        assert _ctypes_leaves(cls) == leaves, cname


# ---- Julia structs ------------------------------------------------------------
_SIZES = {"Int32": 4, "Cint": 4, "UInt32": 4, "Float32": 4, "Int64": 8, "Float64": 8, "UInt64": 8,
          "Int": 8, "Csize_t": 8}


def _julia_structs(text):
    structs = {}
    for m in re.finditer(r"^struct\s+(\w+)(?:\{[^}]*\})?(?:\s*<:\s*[^\n]+)?\n(.*?)^end", text, re.M | re.S):
        fields = []
        for line in m.group(2).splitlines():
            line = line.split("#", 1)[0]
            for part in line.split(";"):
                part = part.strip()
                if "::" in part:
                    fname, ftype = part.split("::", 1)
                    fields.append((fname.strip(), ftype.strip()))
        structs[m.group(1)] = fields
    return structs


def _julia_leaves(structs, name):
    """Leaf (offset, size) list, size and alignment of a Julia isbits struct."""
    leaves, off, align = [], 0, 1

    def place(size, al):
        nonlocal off, align
        off = (off + al - 1) // al * al
        align = max(align, al)
        start = off
        off += size
        return start

    for _, t in structs[name]:
        tup = re.fullmatch(r"NTuple\{(\d+),\s*(\w+)\}", t)
        if t.startswith("Ptr{") or t == "Ptr":
            leaves.append((place(8, 8), 8))
        elif tup:
            n, et = int(tup.group(1)), _SIZES[tup.group(2)]
            start = place(n * et, et)
            leaves += [(start + i * et, et) for i in range(n)]
        elif t in _SIZES:
            s = _SIZES[t]
            leaves.append((place(s, s), s))
        elif t in structs:
            sub, ssize, salign = _julia_leaves(structs, t)
            start = place(ssize, salign)
            leaves += [(start + o, s) for o, s in sub]
        else:
            raise AssertionError(f"{name}: field type {t} is not an isbits C type")
    size = (off + align - 1) // align * align
    return leaves, size, align


def test_julia_mirrors(c_layout):
    structs = _julia_structs(JULIA.read_text())
    for cname, jname in JL.items():
        assert jname in structs, jname
        leaves, size, _ = _julia_leaves(structs, jname)
        assert (size, leaves) == c_layout[cname], f"{jname} vs {cname}"

"""Parsing helpers for include/biegpu.h shared by the host-side binding tests:
the kind (32- or 64-bit integer, float, double, pointer) of every parameter
of every declared entry point."""
from __future__ import annotations

import re
from pathlib import Path

HEADER = Path(__file__).resolve().parent.parent / "include" / "biegpu.h"


def _split_top(text: str) -> list[str]:
    """Split at commas outside (), {} and []; drop empty trailing parts."""
    parts, depth, cur = [], 0, []
    for ch in text:
        if ch in "({[":
            depth += 1
        elif ch in ")}]":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append("".join(cur).strip())
            cur = []
        else:
            cur.append(ch)
    parts.append("".join(cur).strip())
    return [p for p in parts if p]


def _balanced(text: str, start: int) -> tuple[str, int]:
    """Contents of the parenthesised group opening at text[start] and the index after it."""
    assert text[start] == "("
    depth = 0
    for i in range(start, len(text)):
        depth += text[i] == "("
        depth -= text[i] == ")"
        if depth == 0:
            return text[start + 1:i], i + 1
    raise ValueError("unbalanced parentheses")


def _c_kind(param: str) -> str:
    p = re.sub(r"\bconst\b", "", param).strip()
    if "*" in p or "[" in p:
        return "ptr"
    base = p.rsplit(None, 1)[0] if len(p.split()) > 1 else p
    return {"int": "i32", "unsigned": "i32", "int32_t": "i32", "uint32_t": "i32", "int64_t": "i64",
            "uint64_t": "i64", "size_t": "i64", "double": "f64", "float": "f32"}.get(base, "?" + base)


def header_decls() -> dict[str, tuple[str, ...]]:
    """Per declared entry point, the kinds of its parameters."""
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    decls = {}
    for m in re.finditer(r"BIE_API\s+[\w\s\*]+?\b(bie_\w+)\s*\(", text):
        params, _ = _balanced(text, m.end() - 1)
        p = _split_top(params)
        decls[m.group(1)] = () if p == ["void"] else tuple(_c_kind(x) for x in p)
    return decls

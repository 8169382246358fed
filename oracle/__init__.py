"""ORACLE - test infrastructure only (never imported by the product path).

CPU checker for libbiegpu.so:
  * ``bem_oracle.c`` - C99/OpenMP restatement of the reference's dense
    collocation assembly (see its header for the file:line map);
  * ``analytic.py`` - the reference's analytic sphere solutions.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py
may use this package.

Parity status: the Julia reference cannot run here (no Julia toolchain), so the
restatement is pinned by reproducing the reference's own known-answer tests:
the rigid-sphere error table (test/3d/assembly_test.jl:12-44), the sphere
area (test/3d/fmm_test.jl:11-28) and the rule weight sums
(test/3d/surface_functions_test.jl:13-53).
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
import threading
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "bem_oracle.c"
LIB = HERE / "libbemoracle.so"
_lib = None
_lock = threading.Lock()


def build(force: bool = False) -> Path:
    """Compile the C restatement with gcc (FMA contraction off, OpenMP)."""
    if not force and LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, "-O2", "-std=gnu99", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           str(SRC), "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    with _lock:
        if _lib is None:
            L = C.CDLL(str(build()))
            P, D, I, I64 = C.c_void_p, C.c_double, C.c_int, C.c_int64
            L.oracle_assemble.restype = I
            L.oracle_assemble.argtypes = [P, I64, P, I, P, I, I64, P, I64, P, I64, I, I, D, D, I,
                                          P, P, P, I]
            L.oracle_rule.restype = I
            L.oracle_rule.argtypes = [I, I, I, P, P, P]
            L.oracle_total_weight.restype = D
            L.oracle_total_weight.argtypes = [P, P, I, I64, I, I]
            L.oracle_assemble_w.restype = I
            L.oracle_assemble_w.argtypes = [P, I64, P, I, P, I, I64, P, I64, P, I64, I, I, D, D, I,
                                             P, P, P, I, P]
            L.oracle_taylor_assemble.restype = I
            L.oracle_taylor_assemble.argtypes = [P, I64, P, I, P, I, I64, P, I64, P, I64, I, I, D, D, I, I,
                                                 P, P, P, I]
            L.oracle_singular_rule.restype = I
            L.oracle_singular_rule.argtypes = [I, D, P, P, P, I]
            L.oracle_basis.restype = None
            L.oracle_basis.argtypes = [I, D, I64, P, P, P]
            L.oracle_set_beta.restype = None
            L.oracle_set_beta.argtypes = [D]
            L.oracle_nearfield.restype = I
            L.oracle_nearfield.argtypes = [P, P, I, P, I, P, P, I64, I64, D, I, I, D, D, I, P, P, I]
            _lib = L
        return _lib


_KIND = {"linear": 1, "quadratic": 2, "disctriconstant": 3, "disctrilinear": 4, "disctriquadratic": 5}


def _physics(mesh) -> int:
    """Physics kind code; sets the node offset of discontinuous kinds."""
    lib().oracle_set_beta(float(getattr(mesh, "physics_beta", 0.0)))
    return _KIND[mesh.physics_function]


def basis(kind: str, u, v, beta: float = 0.0):
    """Basis values (n_nodes x len(u)) of the restated shape functions."""
    u = np.ascontiguousarray(u, dtype=np.float64).ravel()
    v = np.ascontiguousarray(v, dtype=np.float64).ravel()
    nn = {1: 3, 2: 6, 3: 1, 4: 3, 5: 6}[_KIND[kind]]
    N = np.zeros((nn, u.size), order="F")
    lib().oracle_basis(_KIND[kind], float(beta), u.size, u.ctypes.data, v.ctypes.data, N.ctypes.data)
    return N


def rule(n: int, m: int, corner: int):
    """(u, v, w) of the rule clustered at element node ``corner`` (1..6)."""
    size = 2 * n * (m + 1) + 8
    u, v, w = (np.zeros(size) for _ in range(3))
    q = lib().oracle_rule(n, m, corner, u.ctypes.data, v.ctypes.data, w.ctypes.data)
    return u[:q].copy(), v[:q].copy(), w[:q].copy()


def total_weight(mesh, n: int = 2, m: int = 2) -> float:
    c = np.asfortranarray(mesh.coordinates, dtype=np.float64)
    t = np.asfortranarray(mesh.topology, dtype=np.int64)
    return lib().oracle_total_weight(c.ctypes.data, t.ctypes.data, _KIND[mesh.shape_function],
                                     t.shape[1], n, m)


def singular_rule(node: int, offset: float = 0.0):
    """(u, v, w) of singular_triangle_integration towards element node ``node``."""
    cap = 32768
    u, v, w = (np.zeros(cap) for _ in range(3))
    q = lib().oracle_singular_rule(node, float(offset), u.ctypes.data, v.ctypes.data, w.ctypes.data, cap)
    return u[:q].copy(), v[:q].copy(), w[:q].copy()


def connected_sources(mesh, depth: int = 1):
    """connected_sources for continuous physics (src/3d/assembly_collocation_losses.jl:
    98-132): per node, the sorted elements and physics nodes within ``depth``."""
    T = mesh.physics_topology - 1
    NP, E = T.shape
    N = mesh.n_sources
    econ = [[] for _ in range(N)]
    scon = [[] for _ in range(N)]
    for e in range(E):
        for a in range(NP):
            econ[T[a, e]].append(e)
            scon[T[a, e]].extend(T[:, e].tolist())
    if depth == 2:
        e2 = [[] for _ in range(N)]
        s2 = [[] for _ in range(N)]
        for i in range(N):
            for j in scon[i]:
                e2[i].extend(econ[j])
                s2[i].extend(scon[j])
        econ, scon = e2, s2
    return [sorted(set(x)) for x in econ], [sorted(set(x)) for x in scon]


def nearfield(mesh, k, depth=1, offset=0.0, coarse=False, n_gauss=3, fOn=True, gOn=True, threads=0):
    """Near-field F, G (CSR: row_ptr, cols, values) of sparse_assemble_parallel!
    (coarse=False) or partial_assemble_parallel! (coarse=True)."""
    if mesh.physics_function.startswith("disc"):
        raise NotImplementedError("the near field of discontinuous physics (polar rules) is not restated")
    k = complex(k)
    econ, scon = connected_sources(mesh, depth)
    N = mesh.n_sources
    row_ptr = np.zeros(N + 1, dtype=np.int64)
    for i in range(N):
        row_ptr[i + 1] = row_ptr[i] + len(scon[i])
    cols = np.concatenate([np.asarray(s, dtype=np.int64) for s in scon])
    T = mesh.physics_topology - 1
    NP = T.shape[0]
    pairs = []
    for i in range(N):
        pos = {nd: row_ptr[i] + j for j, nd in enumerate(scon[i])}
        for e in econ[i]:
            pairs.append([i, e] + [pos[T[a, e]] for a in range(NP)])
    pairs = np.ascontiguousarray(np.asarray(pairs, dtype=np.int64))
    nnz = len(cols)
    F = np.zeros(nnz, dtype=np.complex128)
    G = np.zeros(nnz, dtype=np.complex128)
    c = np.asfortranarray(mesh.coordinates, dtype=np.float64)
    t = np.asfortranarray(mesh.topology, dtype=np.int64)
    pt = np.asfortranarray(mesh.physics_topology, dtype=np.int64)
    s = np.asfortranarray(mesh.sources, dtype=np.float64)
    flags = (1 if fOn else 0) | (2 if gOn else 0)
    st = lib().oracle_nearfield(c.ctypes.data, t.ctypes.data, _KIND[mesh.shape_function], pt.ctypes.data,
                                _physics(mesh), s.ctypes.data, pairs.ctypes.data,
                                len(pairs), nnz, float(offset), 1 if coarse else 0, int(n_gauss),
                                k.real, k.imag, flags, F.ctypes.data, G.ctypes.data, int(threads))
    if st != 0:
        raise RuntimeError("oracle_nearfield failed")
    return row_ptr, cols, F, G


def farfield_objective(mesh, k, Z, field_points, rho_c=1.21 * 343.0, direction=(0.0, 0.0, 1.0), n=2, m=2):
    """J = sum |p(x_f)|^2 of the impedance scattering model, by dense oracle
    assembly and a direct solve:
      (F + Diagonal(1 - C) - i rho c k G_Y) p = p_I,  p_f = p_I(x_f) + (-F_x + i rho c k G_xY) p,
    G_Y = single layer with element factors 1 / Z_e, p_I = exp(-i k d.x)."""
    d = np.asarray(direction, dtype=np.float64)
    d = d / np.linalg.norm(d)
    Y = np.ascontiguousarray(1.0 / np.asarray(Z, dtype=np.complex128))
    F, G, Cv = assemble(mesh, k, n=n, m=m, g_weight=Y)
    A = F + np.diag(1.0 - Cv) - 1j * rho_c * k * G
    pI = np.exp(-1j * k * (d @ mesh.sources))
    p = np.linalg.solve(A, pI)
    X = np.asarray(field_points, dtype=np.float64)
    Fx, Gx, _ = assemble(mesh, k, targets=X, n=n, m=m, cOn=False, g_weight=Y)
    pf = np.exp(-1j * k * (d @ X)) + (-Fx + 1j * rho_c * k * Gx) @ p
    return float(np.sum(np.abs(pf) ** 2)), pf


def taylor_assemble(mesh, k0, order, targets=None, n=3, m=3, fOn=True, gOn=True, cOn=True, threads=0):
    """taylor_assemble! (src/3d/rosebem.jl:56-157) with U = I: F, G of shape
    (M, N, order + 1) (k-derivatives m = 0..order at k0) and C."""
    k0 = complex(k0)
    c = np.asfortranarray(mesh.coordinates, dtype=np.float64)
    t = np.asfortranarray(mesh.topology, dtype=np.int64)
    pt = np.asfortranarray(mesh.physics_topology, dtype=np.int64)
    s = np.asfortranarray(mesh.sources, dtype=np.float64)
    tg = s if targets is None else np.asfortranarray(targets, dtype=np.float64)
    N, M = s.shape[1], tg.shape[1]
    F = np.zeros((M, N, order + 1), dtype=np.complex128, order="F") if fOn else None
    G = np.zeros((M, N, order + 1), dtype=np.complex128, order="F") if gOn else None
    Cv = np.zeros(M, dtype=np.complex128) if cOn else None
    flags = (1 if fOn else 0) | (2 if gOn else 0) | (4 if cOn else 0)
    addr = lambda a: None if a is None else a.ctypes.data  # noqa: E731
    st = lib().oracle_taylor_assemble(c.ctypes.data, c.shape[1], t.ctypes.data, _KIND[mesh.shape_function],
                                      pt.ctypes.data, _physics(mesh), t.shape[1], s.ctypes.data,
                                      N, tg.ctypes.data, M, n, m, k0.real, k0.imag, flags, int(order),
                                      addr(F), addr(G), addr(Cv), int(threads))
    if st != 0:
        raise RuntimeError("oracle_taylor_assemble failed")
    return F, G, Cv


def fast_operator(mesh, k, which="F", n_gauss=3, nearfield=True, offset=0.2, depth=1):
    """Dense matrix of FMMFOperator / FMMGOperator (src/3d/fast_multipole_method.jl:
    163-194, 306-324, 473-490) with an exact far-field sum: every pair with the
    n_gauss-point Gauss rule, plus nearfield_correction = accurate near field
    (adaptive rules, offset) - its Gauss-rule part on the depth pattern."""
    F, G, _ = assemble(mesh, k, n=-n_gauss, m=1, fOn=which == "F", gOn=which == "G", cOn=False)
    A = np.array(F if which == "F" else G)
    if nearfield:
        near = globals()["nearfield"]   # the function (the argument shadows its name)
        rp, cols, Fa, Ga = near(mesh, k, depth=depth, offset=offset, fOn=which == "F", gOn=which == "G")
        _, _, Fc, Gc = near(mesh, k, depth=depth, coarse=True, n_gauss=n_gauss, fOn=which == "F",
                            gOn=which == "G")
        acc, coarse = (Fa, Fc) if which == "F" else (Ga, Gc)
        for i in range(mesh.n_sources):
            for p in range(rp[i], rp[i + 1]):
                A[i, cols[p]] += acc[p] - coarse[p]
    return A


def assemble(mesh, k, targets=None, n=4, m=4, fOn=True, gOn=True, cOn=True, threads=0, g_weight=None):
    """Reference-algorithm (F, G, C) on the CPU; F, G are M x N Fortran-ordered.
    n < 0 selects the symmetric (-n)-point Gauss rule for every pair."""
    k = complex(k)
    c = np.asfortranarray(mesh.coordinates, dtype=np.float64)
    t = np.asfortranarray(mesh.topology, dtype=np.int64)
    pt = np.asfortranarray(mesh.physics_topology, dtype=np.int64)
    s = np.asfortranarray(mesh.sources, dtype=np.float64)
    tg = s if targets is None else np.asfortranarray(targets, dtype=np.float64)
    N, M = s.shape[1], tg.shape[1]
    F = np.zeros((M, N), dtype=np.complex128, order="F") if fOn else None
    G = np.zeros((M, N), dtype=np.complex128, order="F") if gOn else None
    Cv = np.zeros(M, dtype=np.complex128) if cOn else None
    flags = (1 if fOn else 0) | (2 if gOn else 0) | (4 if cOn else 0)
    addr = lambda a: None if a is None else a.ctypes.data  # noqa: E731
    gw = None if g_weight is None else np.ascontiguousarray(g_weight, dtype=np.complex128)
    lib().oracle_assemble_w(c.ctypes.data, c.shape[1], t.ctypes.data, _KIND[mesh.shape_function],
                            pt.ctypes.data, _physics(mesh), t.shape[1], s.ctypes.data,
                            N, tg.ctypes.data, M, n, m, k.real, k.imag, flags, addr(F), addr(G),
                            addr(Cv), int(threads), addr(gw))
    return F, G, Cv

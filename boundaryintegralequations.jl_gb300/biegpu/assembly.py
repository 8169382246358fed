"""Dense collocation assembly on the GPU, mirroring ``assemble_parallel!``.

``assemble_parallel(mesh, k, sources; fOn, gOn, cOn, n, m)`` has the argument
meaning, defaults (n = m = 4) and return value (F, G, C) of the reference's
dispatcher (src/3d/assembly_collocation.jl:259-268): F and G are
``len(targets) x N`` complex128 matrices in column-major (Fortran) order, the
memory layout of Julia's ``Matrix{ComplexF64}``, and C is a complex vector.
Everything is computed by libbiegpu.so on the GPU.
"""
from __future__ import annotations

import ctypes as C
import weakref

import numpy as np

from . import _capi
from .mesh import Mesh3d


def quadrature_rule(n: int, m: int, node: int):
    """(u, v, w) of the collocation rule clustered at element node ``node`` (1..6),
    computed by libbiegpu's host code (no GPU needed)."""
    cap = 2 * n * (m + 1) + 8
    u, v, w = (np.zeros(cap) for _ in range(3))
    cnt = C.c_int()
    _capi.check(_capi.lib().bie_quadrature_rule(n, m, node, u.ctypes.data, v.ctypes.data,
                                                w.ctypes.data, cap, C.byref(cnt)))
    q = cnt.value
    return u[:q].copy(), v[:q].copy(), w[:q].copy()


def basis(kind: str, u, v, beta: float = 0.0):
    """(N, dN/du, dN/dv) of element kind ``kind`` ("linear", "quadratic",
    "disctriconstant", "disctrilinear", "disctriquadratic"; node offset
    ``beta`` for the discontinuous ones) at the points (u, v), each an
    n_nodes x len(u) array like basisFunction / basisFunctionDerivative
    (src/3d/surface_functions.jl:191-318) - bie_basis, host only."""
    from .mesh import KIND_NODES
    u = np.ascontiguousarray(u, dtype=np.float64).ravel()
    v = np.ascontiguousarray(v, dtype=np.float64).ravel()
    if u.shape != v.shape:
        raise ValueError("u and v must have the same length")
    NP = KIND_NODES[kind]
    out = [np.zeros((NP, u.size), order="F") for _ in range(3)]
    _capi.check(_capi.lib().bie_basis(_capi.KIND[kind], float(beta), u.size, u.ctypes.data, v.ctypes.data,
                                      out[0].ctypes.data, out[1].ctypes.data, out[2].ctypes.data))
    return tuple(out)


def mesh_desc(mesh: Mesh3d):
    """A bie_mesh_desc of the mesh (quad_n = quad_m = 1) and the tuple of the
    Fortran-ordered arrays it points at, to be kept alive while it is used."""
    keep = (np.asfortranarray(mesh.coordinates, dtype=np.float64),
            np.asfortranarray(mesh.topology, dtype=np.int64),
            np.asfortranarray(mesh.physics_topology, dtype=np.int64),
            np.asfortranarray(mesh.sources, dtype=np.float64))
    d = _capi.MeshDesc(
        n_coordinates=keep[0].shape[1], coordinates=keep[0].ctypes.data_as(C.POINTER(C.c_double)),
        n_elements=keep[1].shape[1], shape_kind=_capi.KIND[mesh.shape_function],
        physics_kind=_capi.KIND[mesh.physics_function], topology=keep[1].ctypes.data_as(C.POINTER(C.c_int64)),
        physics_topology=keep[2].ctypes.data_as(C.POINTER(C.c_int64)), n_sources=keep[3].shape[1],
        sources=keep[3].ctypes.data_as(C.POINTER(C.c_double)), quad_n=1, quad_m=1,
        physics_beta=float(getattr(mesh, "physics_beta", 0.0)))
    return d, keep


SLICING_COUNTS = ("shared", "side_slots", "ring", "widened", "single", "untouched")


def element_slicing(mesh: Mesh3d, level: int, tables: bool = False):
    """The element slicing of the assembly kernels, computed on the host
    (bie_element_slicing; no GPU): (order, counts).  order: the E 1-based
    element numbers in the order the kernels process them (a recursive
    coordinate bisection of the element centroids); counts: the nodes of each
    kind at slicing level `level` (2^level slices), keyed by SLICING_COUNTS:
    shared between slices (with their side slots), of one slice with several
    contributions summed in the shared-memory ring or widened afterwards, with
    one contribution, or touched by no element.  tables=True adds the write
    protocol of the mixed assembly: (order, counts, flags, slots) with flags
    (E uint32; per position p and local node a: bit a first, 8+a last, 16+a
    shared, 24+a ring) and slots (n_phys x E int32: side slot, ring slot or -1)."""
    d, keep = mesh_desc(mesh)
    E, NP = mesh.topology.shape[1], mesh.physics_topology.shape[0]
    order = np.empty(E, dtype=np.int32)
    counts = np.zeros(len(SLICING_COUNTS), dtype=np.int64)
    flags = np.empty(E, dtype=np.uint32) if tables else None
    slots = np.empty((E, NP), dtype=np.int32) if tables else None
    _capi.check(_capi.lib().bie_element_slicing(C.byref(d), int(level), order.ctypes.data, counts.ctypes.data,
                                                None if flags is None else flags.ctypes.data,
                                                None if slots is None else slots.ctypes.data))
    del keep
    out = (order, dict(zip(SLICING_COUNTS, (int(v) for v in counts))))
    return out + (flags, slots.T.copy()) if tables else out


class Context:
    """A libbiegpu context: one mesh, one quadrature order (n, m), one device.

    ``rules``, when given, replaces the rules built from (n, m): a sequence of
    (u, v, w) arrays, one per element node that can be the nearest to a
    collocation point (3 for linear geometry, 3 or 6 physics nodes for
    quadratic geometry), e.g. the ``gauss_u``, ``gauss_v``, ``weights`` of the
    shape functions ``create_rotated_element`` returns
    (src/3d/assembly_collocation.jl:122-136) - bie_ctx_create_rules."""

    def __init__(self, mesh: Mesh3d, n: int = 4, m: int = 4, device: int = 0, rules=None):
        L = _capi.lib()
        self.mesh = mesh
        self.n, self.m, self.device = int(n), int(m), int(device)
        # keep the arrays alive while the descriptor points at them
        self._coords = np.asfortranarray(mesh.coordinates, dtype=np.float64)
        self._topo = np.asfortranarray(mesh.topology, dtype=np.int64)
        self._ptopo = np.asfortranarray(mesh.physics_topology, dtype=np.int64)
        self._src = np.asfortranarray(mesh.sources, dtype=np.float64)
        desc = _capi.MeshDesc(
            n_coordinates=self._coords.shape[1],
            coordinates=self._coords.ctypes.data_as(C.POINTER(C.c_double)),
            n_elements=self._topo.shape[1],
            shape_kind=_capi.KIND[mesh.shape_function],
            physics_kind=_capi.KIND[mesh.physics_function],
            topology=self._topo.ctypes.data_as(C.POINTER(C.c_int64)),
            physics_topology=self._ptopo.ctypes.data_as(C.POINTER(C.c_int64)),
            n_sources=self._src.shape[1],
            sources=self._src.ctypes.data_as(C.POINTER(C.c_double)),
            quad_n=self.n,
            quad_m=self.m,
            physics_beta=float(getattr(mesh, "physics_beta", 0.0)),
        )
        h = C.c_void_p()
        if rules is None:
            _capi.check(L.bie_ctx_create(C.byref(h), C.byref(desc), self.device))
        else:
            self.n = self.m = 0
            keep = [tuple(np.ascontiguousarray(a, dtype=np.float64) for a in r) for r in rules]
            if any(len({a.shape for a in r}) != 1 or r[0].ndim != 1 for r in keep):
                raise ValueError("every rule is three 1-D arrays (u, v, w) of one length")
            tabs = (_capi.RuleTable * len(keep))(*[
                _capi.RuleTable(n_points=r[0].size,
                                u=r[0].ctypes.data_as(C.POINTER(C.c_double)),
                                v=r[1].ctypes.data_as(C.POINTER(C.c_double)),
                                w=r[2].ctypes.data_as(C.POINTER(C.c_double))) for r in keep])
            _capi.check(L.bie_ctx_create_rules(C.byref(h), C.byref(desc), tabs, len(keep), self.device))
        self._h = h
        self._finalizer = weakref.finalize(self, L.bie_ctx_destroy, h)

    @property
    def handle(self):
        return self._h

    @property
    def n_sources(self) -> int:
        return self.mesh.n_sources

    def close(self) -> None:
        self._finalizer()

    def stream(self) -> int:
        s = C.c_void_p()
        _capi.check(_capi.lib().bie_ctx_stream(self._h, C.byref(s)))
        return s.value or 0

    def set_timing(self, on: bool) -> None:
        _capi.check(_capi.lib().bie_ctx_set_timing(self._h, 1 if on else 0))

    def set_autotune(self, on: bool) -> None:
        """Search the launch shape (slicing, records per chunk, block size) on
        the first call per target count of the mixed and double-float
        assemblies and the mixed product, and keep the fastest
        (bie_ctx_set_autotune)."""
        _capi.check(_capi.lib().bie_ctx_set_autotune(self._h, 1 if on else 0))

    SHAPE_KERNELS = {"mixed_assembly": 0, "df64_assembly": 1, "mixed_product": 2}

    def shape(self, kernel: str, M: int | None = None):
        """(level, chunk, threads per block) tuned or forced for `kernel` and M
        targets (default: the collocation nodes), or None."""
        found, lv, ch, tp = C.c_int(0), C.c_int(0), C.c_int(0), C.c_int(0)
        _capi.check(_capi.lib().bie_ctx_get_shape(self._h, self.SHAPE_KERNELS[kernel],
                                                  int(self.n_sources if M is None else M), C.byref(found),
                                                  C.byref(lv), C.byref(ch), C.byref(tp)))
        return (lv.value, ch.value, tp.value) if found.value else None

    def force_shape(self, kernel: str, level: int, chunk: int = 0, tpb: int = 0, M: int = 0) -> None:
        """Use this shape for `kernel` (M = 0: every target count); level < 0 clears it."""
        _capi.check(_capi.lib().bie_ctx_set_shape(self._h, self.SHAPE_KERNELS[kernel], int(M), int(level),
                                                  int(chunk), int(tpb)))

    def stats(self, reset: bool = False) -> dict:
        st = _capi.Stats()
        _capi.check(_capi.lib().bie_ctx_stats(self._h, C.byref(st), 1 if reset else 0))
        return {name: getattr(st, name) for name, _ in st._fields_}

    # ---- host-buffer assembly (the reference-facing call) -----------------
    def assemble(self, k, targets=None, fOn=True, gOn=True, cOn=True, precision="fp64",
                 out=None):
        """(F, G, C) on the host; ``targets`` is 3 x M (None = mesh sources)."""
        k = complex(k)
        N = self.n_sources
        if targets is not None:
            t = np.asfortranarray(targets, dtype=np.float64)
            if t.ndim != 2 or t.shape[0] != 3:
                raise ValueError("targets must be a 3 x M array")
            M = t.shape[1]
        else:
            t, M = None, N
        flags = (_capi.BIE_F if fOn else 0) | (_capi.BIE_G if gOn else 0) | (_capi.BIE_C if cOn else 0)
        if out is not None:
            F, G, Cv = out
        else:
            F = np.empty((M, N), dtype=np.complex128, order="F") if fOn else None
            G = np.empty((M, N), dtype=np.complex128, order="F") if gOn else None
            Cv = np.empty(M, dtype=np.complex128) if cOn else None
        _capi.check(_capi.lib().bie_assemble(
            self._h, k.real, k.imag, _capi.ptr(t), M, flags, _capi.PRECISION[precision],
            _capi.ptr(F), _capi.ptr(G), _capi.ptr(Cv)))
        return F, G, Cv

    # ---- device-buffer assembly (torch tensors, enqueued on the context stream)
    def _torch_streams(self):
        """(torch's current stream, the library stream as a torch stream)."""
        import torch
        dev = torch.device(f"cuda:{self.device}")
        if getattr(self, "_lib_stream", None) is None:
            self._lib_stream = torch.cuda.ExternalStream(self.stream(), device=dev)
        return torch.cuda.current_stream(dev), self._lib_stream

    def assemble_device(self, k, F=None, G=None, Cv=None, targets=None, precision="fp64"):
        """Fill device tensors: F, G complex128 of shape (N, M) in row-major torch
        terms (= column-major M x N), Cv complex128 (M,).  Asynchronous and
        ordered with torch's current stream: the assembly waits for the work
        queued there before it, and later work queued there waits for the
        assembly (device-side waits, no host synchronisation)."""
        k = complex(k)
        M = self.n_sources if targets is None else int(targets.shape[-1] if targets.ndim == 2 and targets.shape[0] == 3 else targets.shape[0])
        flags = (_capi.BIE_F if F is not None else 0) | (_capi.BIE_G if G is not None else 0) | \
                (_capi.BIE_C if Cv is not None else 0)
        cur, lib_stream = self._torch_streams()
        lib_stream.wait_stream(cur)
        _capi.check(_capi.lib().bie_assemble_device(
            self._h, k.real, k.imag, _capi.ptr(targets), M, flags, _capi.PRECISION[precision],
            _capi.ptr(F), _capi.ptr(G), _capi.ptr(Cv)))
        cur.wait_stream(lib_stream)


def nearfield_pattern(ctx: "Context", depth: int = 1):
    """(row_ptr, cols) CSR pattern of the near field (0-based)."""
    L = _capi.lib()
    nnz = C.c_int64()
    _capi.check(L.bie_nearfield_pattern(ctx.handle, int(depth), C.byref(nnz), None, None))
    row_ptr = np.empty(ctx.n_sources + 1, dtype=np.int64)
    cols = np.empty(nnz.value, dtype=np.int64)
    _capi.check(L.bie_nearfield_pattern(ctx.handle, int(depth), C.byref(nnz), row_ptr.ctypes.data,
                                        cols.ctypes.data))
    return row_ptr, cols


def nearfield_values(ctx: "Context", k, depth=1, offset=None, coarse=False, n_gauss=3, fOn=True, gOn=True):
    """Near-field F, G values (complex, CSR order of nearfield_pattern)."""
    k = complex(k)
    row_ptr, cols = nearfield_pattern(ctx, depth)
    nnz = len(cols)
    F = np.empty(nnz, dtype=np.complex128) if fOn else None
    G = np.empty(nnz, dtype=np.complex128) if gOn else None
    flags = (_capi.BIE_F if fOn else 0) | (_capi.BIE_G if gOn else 0)
    off = -1.0 if offset is None else float(offset)
    _capi.check(_capi.lib().bie_nearfield_assemble(ctx.handle, k.real, k.imag, int(depth), off, flags,
                                                   1 if coarse else 0, int(n_gauss), _capi.ptr(F),
                                                   _capi.ptr(G)))
    return row_ptr, cols, F, G


def sparse_assemble_parallel(mesh: Mesh3d, k, fOn=True, gOn=True, depth=1, offset=None, device=0):
    """GPU ``assemble_parallel!(mesh, k, mesh.sources; sparse=true)``
    (sparse_assemble_parallel!, src/3d/assembly_collocation_losses.jl:200-405):
    the near-field F and G with the adaptive singular rules, as scipy CSR
    matrices (N x N)."""
    import scipy.sparse as sp
    ctx = get_context(mesh, device=device)
    row_ptr, cols, F, G = nearfield_values(ctx, k, depth=depth, offset=offset, fOn=fOn, gOn=gOn)
    N = mesh.n_sources
    mk = lambda v: None if v is None else sp.csr_matrix((v, cols, row_ptr), shape=(N, N))  # noqa: E731
    return mk(F), mk(G)


_CTX_CACHE: "weakref.WeakKeyDictionary[Mesh3d, dict]" = weakref.WeakKeyDictionary()


def get_context(mesh: Mesh3d, n: int = 4, m: int = 4, device: int = 0) -> Context:
    """Cached context per (mesh object, n, m, device)."""
    d = _CTX_CACHE.setdefault(mesh, {})
    key = (int(n), int(m), int(device))
    if key not in d:
        d[key] = Context(mesh, n=n, m=m, device=device)
    return d[key]


def assemble_parallel(mesh: Mesh3d, k, sources=None, fOn=True, gOn=True, cOn=True,
                      sparse=False, m=4, n=4, progress=True, depth=2, offset=None,
                      precision="fp64", device=0):
    """GPU ``assemble_parallel!``: returns (F, G, C).

    ``sources`` are the collocation/field points (3 x M); passing
    ``mesh.sources`` (or None) assembles the square BEM matrices.  ``progress``
    is accepted and ignored.  ``precision``: "fp64" (the reference's
    arithmetic), "mixed" (FP32 regular pairs, ~1e-7) or "df64" (double-float
    regular pairs, FP64-grade ~1e-14, faster than "fp64" on GB300).  ``sparse=True`` (the near-field-only assembly)
    is not part of this library yet and raises.
    """
    if sparse:
        return sparse_assemble_parallel(mesh, k, fOn=fOn, gOn=gOn, depth=depth, offset=offset,
                                        device=device)
    ctx = get_context(mesh, n=n, m=m, device=device)
    targets = None if sources is None or sources is mesh.sources else sources
    return ctx.assemble(k, targets=targets, fOn=fOn, gOn=gOn, cOn=cOn, precision=precision)

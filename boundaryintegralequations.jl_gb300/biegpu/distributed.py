"""Frequency sweeps split across ranks (one process per GPU).

The sweep shards with no exchange on the data path: rank r of W solves a
contiguous block of the wavenumber list for every mesh on its own GPU
(:func:`biegpu.sweep`), and the solutions are gathered once at the end.  The
reference has no parallel sweep (users loop over frequencies,
examples/sweep_meta.jl:219-233); this is the multi-GPU form of that loop.
Works with any torch.distributed backend: NCCL between GPU ranks, gloo on CPU.
"""
from __future__ import annotations

import numpy as np


def shard(n: int, rank: int, world: int) -> range:
    """Contiguous block of ``range(n)`` owned by ``rank`` (sizes differ by at most one)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def max_over_ranks(x: float, group=None) -> float:
    """Largest value of ``x`` over the ranks (the timing rule of the benchmark)."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64)
    if dist.get_backend(group) == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def sharded_sweep(meshes, ks, ws, group=None, solve=None, **kwargs):
    """:func:`biegpu.sweep` over ``ks`` split across the ranks of ``group``.

    Every rank passes the same meshes, wavenumbers and boundary data; each
    solves its shard (``shard(len(ks), rank, world)``) and all ranks return the
    full result: one N_m x len(ks) complex array per mesh, and the info
    counters summed over the ranks.  ``solve`` replaces :func:`biegpu.sweep`
    (same signature), e.g. to run the host logic without a GPU.
    """
    import torch.distributed as dist
    if solve is None:
        from .sweep import sweep as solve
    ks = np.asarray(ks, dtype=np.complex128)
    if dist.is_available() and dist.is_initialized():
        rank, world = dist.get_rank(group), dist.get_world_size(group)
    else:
        rank, world = 0, 1
    mine = shard(len(ks), rank, world)
    if len(mine):
        outs, info = solve(meshes, ks[mine.start:mine.stop], ws, **kwargs)
    else:
        outs = [np.zeros((m.n_sources, 0), dtype=np.complex128) for m in meshes]
        info = {"solves": 0, "converged": 0, "iterations": 0, "assemble_ms": 0.0, "solve_ms": 0.0}
    counters = {k: info[k] for k in ("solves", "converged", "iterations", "assemble_ms", "solve_ms") if k in info}
    if world == 1:
        return outs, counters
    parts = [None] * world
    dist.all_gather_object(parts, (mine.start, [np.asarray(o) for o in outs], counters), group=group)
    full = [np.empty((m.n_sources, len(ks)), dtype=np.complex128, order="F") for m in meshes]
    total = {k: 0 for k in counters}
    for start, pouts, pc in parts:
        for f, p in zip(full, pouts):
            f[:, start:start + p.shape[1]] = p
        for k in total:
            total[k] += pc[k]
    return full, total

"""Two-rank (gloo, CPU) tests of the sharded sweep's host logic: the shards
cover the wavenumber list once, every rank gets the full gathered result, the
counters add up, and max_over_ranks returns the largest rank value.  The
per-rank solve is replaced by a deterministic host function (no GPU)."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from biegpu.distributed import max_over_ranks, shard, sharded_sweep


def test_shard_covers_once():
    for n in (0, 1, 5, 64, 65):
        for w in (1, 2, 3, 8):
            got = [i for r in range(w) for i in shard(n, r, w)]
            assert got == list(range(n))
            sizes = [len(shard(n, r, w)) for r in range(w)]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard(4, 2, 2)


class _Mesh:
    def __init__(self, n):
        self.n_sources = n


def _fake_solve(meshes, ks, ws, **kw):
    outs = [np.outer(w, np.asarray(ks)) for w in ws]     # p[:, j] = k_j w
    return outs, {"solves": len(ks) * len(meshes), "converged": len(ks) * len(meshes),
                  "iterations": 3 * len(ks) * len(meshes), "assemble_ms": 1.0, "solve_ms": 2.0}


def _worker(rank, world, port, nk, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        meshes = [_Mesh(4), _Mesh(7)]
        rng = np.random.default_rng(0)
        ws = [rng.normal(size=m.n_sources) + 1j * rng.normal(size=m.n_sources) for m in meshes]
        ks = np.linspace(0.1, 10.0, nk)
        outs, info = sharded_sweep(meshes, ks, ws, solve=_fake_solve)
        ok = all(np.allclose(o, np.outer(w, ks), rtol=0, atol=0) for o, w in zip(outs, ws))
        ok = ok and info["solves"] == nk * 2 and info["iterations"] == 3 * nk * 2
        ok = ok and abs(info["assemble_ms"] - sum(1.0 for r in range(world) if len(shard(nk, r, world)))) < 1e-12
        m = max_over_ranks(float(rank + 1))
        ok = ok and m == float(world)
        q.put((rank, ok))
    finally:
        dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


@pytest.mark.parametrize("nk", [5, 1])
def test_sharded_sweep_two_ranks_gloo(nk):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, nk, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    res = dict(q.get(timeout=5) for _ in procs)
    assert res == {0: True, 1: True}

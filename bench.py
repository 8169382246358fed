#!/usr/bin/env python
"""Benchmark of the GB300 collocation-BEM hot path (libbiegpu.so).

Workload (default ``rigid_sphere_p2``): rigid-sphere plane-wave scattering
mesh with 6-node triangles, radius 1, geodesic sphere f=17 promoted to P2:
11562 nodes, 5780 triangles, quadrature n = m = 2 (4-point corner rules,
8-point midpoint rules), ka cycling over 1..10.  One step = one dense assembly
of F, G (11562 x 11562 complex128 each) and C at one wavenumber.

Metric: F/G entries per second (an entry is one complex element of F or G:
2 N^2 per step), whole job.  ``value`` is measured with inputs resident on the
device (bie_assemble_device, CUDA events on the library's stream, 256 MB L2
flush between steps); ``e2e`` goes through the host-buffer C-ABI call
bie_assemble with the target points copied in from pinned host memory and F,
G, C copied back to pinned host memory inside the timed region.

``--impl reference`` times the reference algorithm on the host cores: the
Julia reference cannot run here, so this is the C restatement (oracle/) with
OpenMP over all host threads, on bounded row samples of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "boundaryintegralequations.jl_gb300"
for p in (str(PKG), str(ROOT)):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "F/G entries/s (dense collocation assembly)"
UNIT = "entries/s"


def workload(name: str):
    from biegpu import mesh as bm
    if name == "rigid_sphere_p2":
        mesh = bm.icosphere(17, geometry="quadratic")
        ks = [float(ka) for ka in range(1, 11)]          # radius 1: k = ka
        desc = {"workload": "rigid_sphere_p2", "mesh": "geodesic sphere f=17, 6-node triangles, r=1",
                "nodes": mesh.n_sources, "elements": mesh.n_elements, "quad_n": 2, "quad_m": 2,
                "ka": "1..10 cycled", "outputs": "F, G complex128 N x N + C"}
    elif name == "small_p2":
        # profiling case: same kernel, 2562 nodes (F, G = 210 MB, larger than L2)
        mesh = bm.icosphere(8, geometry="quadratic")
        ks = [float(ka) for ka in range(1, 11)]
        desc = {"workload": "small_p2", "mesh": "geodesic sphere f=8, 6-node triangles, r=1",
                "nodes": mesh.n_sources, "elements": mesh.n_elements, "quad_n": 2, "quad_m": 2,
                "ka": "1..10 cycled", "outputs": "F, G complex128 N x N + C"}
    elif name == "pulsating_sphere":
        mesh = bm.icosphere(32)
        ks = [2 * np.pi * 200 / 343]
        desc = {"workload": "pulsating_sphere", "mesh": "geodesic sphere f=32, 3-node triangles, r=1",
                "nodes": mesh.n_sources, "elements": mesh.n_elements, "quad_n": 2, "quad_m": 2,
                "k": ks[0], "outputs": "F, G complex128 N x N + C"}
    else:
        raise SystemExit(f"unknown workload {name}")
    return mesh, ks, desc


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        try:
            return json.loads(path.read_text())
        except json.JSONDecodeError:
            pass
    return {}


def ncu_traffic(kernel: str, workload_name: str):
    path = ROOT / "profiles" / "ncu_traffic.json"
    if not path.exists():
        return None
    try:
        d = json.loads(path.read_text())
        return d.get(workload_name, {}).get(kernel)
    except (json.JSONDecodeError, AttributeError):
        return None


def cpu_baseline(mesh, ks, target_seconds: float, threads: int):
    """Oracle (C restatement) on the host cores over a bounded row sample."""
    import oracle
    N = mesh.n_sources
    oracle.assemble(mesh, ks[0], targets=mesh.sources[:, :8], n=2, m=2, threads=threads)   # warm-up
    rows = 64
    t0 = time.perf_counter()
    oracle.assemble(mesh, ks[0], targets=mesh.sources[:, :rows], n=2, m=2, threads=threads)
    dt = time.perf_counter() - t0
    rows = int(min(N, max(rows, rows * target_seconds / max(dt, 1e-6))))
    t0 = time.perf_counter()
    oracle.assemble(mesh, ks[0], targets=mesh.sources[:, :rows], n=2, m=2, threads=threads)
    dt = time.perf_counter() - t0
    return 2.0 * rows * N / dt, rows, dt


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    mesh, ks, desc = workload(args.workload)
    threads = os.cpu_count() or 1
    import oracle
    N = mesh.n_sources
    # size one step to ~3 s of CPU work
    t0 = time.perf_counter()
    oracle.assemble(mesh, ks[0], targets=mesh.sources[:, :64], n=2, m=2, threads=threads)
    dt = time.perf_counter() - t0
    rows = int(min(N, max(64, 64 * 3.0 / max(dt, 1e-6))))
    for w in range(args.warmup):
        oracle.assemble(mesh, ks[w % len(ks)], targets=mesh.sources[:, :rows], n=2, m=2, threads=threads)
    t0 = time.perf_counter()
    for s in range(args.steps):
        oracle.assemble(mesh, ks[s % len(ks)], targets=mesh.sources[:, :rows], n=2, m=2, threads=threads)
    dt = time.perf_counter() - t0
    value = 2.0 * rows * N * args.steps / dt
    sample = f"{rows} of {N} rows per step (F, G, C), n=m=2"
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": desc,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "Julia reference unavailable (no Julia toolchain); C restatement of assemble_parallel! timed",
    }))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="rigid_sphere_p2")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup

    if args.impl == "reference":
        run_reference(args)
        return

    import torch
    import biegpu

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)

    def barrier():
        if dist is not None:
            dist.barrier()

    mesh, ks, desc = workload(args.workload)
    # weak scaling: every rank assembles its own share of the frequency list
    ks = ks[rank % len(ks):] + ks[:rank % len(ks)]
    N = mesh.n_sources
    ctx = biegpu.Context(mesh, n=2, m=2, device=local)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=f"cuda:{local}")
    dev = torch.device(f"cuda:{local}")
    F = torch.empty((N, N), dtype=torch.complex128, device=dev)
    G = torch.empty_like(F)
    Cv = torch.empty(N, dtype=torch.complex128, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    entries_per_step = 2.0 * N * N

    for w in range(args.warmup):
        ctx.assemble_device(ks[w % len(ks)], F, G, Cv, precision=args.precision)
    torch.cuda.synchronize()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ctx.set_timing(True)
    ctx.stats(reset=True)
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for s in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(s & 0xFF)
                starts[s].record(stream)
            ctx.assemble_device(ks[s % len(ks)], F, G, Cv, precision=args.precision)
            with torch.cuda.stream(stream):
                ends[s].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    barrier()
    st = ctx.stats(reset=True)
    ctx.set_timing(False)
    dev_ms = sum(a.elapsed_time(b) for a, b in zip(starts, ends))
    t = torch.tensor([dev_ms], dtype=torch.float64, device=dev)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dev_ms = float(t.item())
    value = entries_per_step * args.steps * world / (dev_ms * 1e-3)

    # ---- roofline of the dominant kernel (FP64 pipe bound) -----------------
    kernel_ms = st["timed_ms"] / max(st["timed_launches"], 1)
    flops_per_launch = st["algorithmic_flops"] / max(st["timed_launches"], 1)
    peaks = biegpu._capi.measure_peaks(local)
    achieved = flops_per_launch / (kernel_ms * 1e-3) / 1e12
    peak = peaks["fp64_flops"] / 1e12
    roofline = {"bound": "fp64", "kernel": "assemble_fp64_kernel", "achieved": achieved, "peak": peak,
                "unit": "TFLOP/s", "frac": achieved / peak,
                "peak_source": "measured FP64 FMA-chain throughput (bie_measure_peaks) on this GPU",
                "traffic": ncu_traffic("assemble_fp64_kernel", args.workload),
                "flops_per_launch": flops_per_launch, "kernel_ms": kernel_ms,
                "qpe_per_launch": st["quadrature_evals"] / max(st["timed_launches"], 1),
                "flops_per_qpe": "32 + 8 n_phys (n_phys=%d)" % (3 if mesh.physics_function == "linear" else 6),
                "fp32_peak_tflops": peaks["fp32_flops"] / 1e12}
    gpu_launches = st["kernel_launches"]

    # ---- end to end through the host-buffer C-ABI call -----------------------
    e2e = None
    if not args.no_e2e:
        del F, G
        torch.cuda.empty_cache()
        pin = lambda shape, dt: torch.empty(shape, dtype=dt, pin_memory=True).numpy()  # noqa: E731
        Fh = pin((N, N), torch.complex128).T      # column-major N x N view
        Gh = pin((N, N), torch.complex128).T
        Ch = pin((N,), torch.complex128)
        tg = pin((N, 3), torch.float64).T
        tg[...] = mesh.sources
        ctx.assemble(ks[0], targets=tg, out=(Fh, Gh, Ch), precision=args.precision)   # warm-up
        barrier()
        t0 = time.perf_counter()
        n_e2e = max(1, min(args.steps, 5))
        for s in range(n_e2e):
            ctx.assemble(ks[s % len(ks)], targets=tg, out=(Fh, Gh, Ch), precision=args.precision)
        e2e_s = time.perf_counter() - t0
        tt = torch.tensor([e2e_s], dtype=torch.float64, device=dev)
        if dist is not None:
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        e2e_s = float(tt.item())
        e2e = {"value": entries_per_step * n_e2e * world / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": int(tg.nbytes), "d2h_bytes_per_step": int(Fh.nbytes + Gh.nbytes + Ch.nbytes),
               "steps": n_e2e, "call": "bie_assemble (host buffers, pinned)"}

    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, rows, dt = cpu_baseline(mesh, ks, args.cpu_seconds, threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{rows} of {N} rows of F, G, C at k={ks[0]} ({dt:.1f} s)"}

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "wall_ms_per_step": 1e3 * wall / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "precision": args.precision, "data": "synthetic",
        "config": dict(desc, l2="256 MB L2 flush between steps; each step writes 4.3 GB", parallelism=f"replicas{world}"),
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": gpu_launches,
        "clocks": clk.summary(), "gpu": torch.cuda.get_device_name(dev),
        "measured_peaks_file": {k: measured_peaks().get(k) for k in ("hbm_gbs", "bf16_tflops")},
    }
    print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

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

    def __init__(self, device: int, interval_ms: int = 20):
        self.device = device
        self.interval_ms = interval_ms
        self.proc = None
        self.lines: list[str] = []
        self._stamped: list[tuple[float, str]] = []
        self._t0 = self._t1 = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", str(self.interval_ms)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
            # the timed region starts once the sampler reports (nvidia-smi
            # takes a moment to start), so that its samples fall inside it
            deadline = time.monotonic() + 5.0
            while not self._stamped and time.monotonic() < deadline and self.proc.poll() is None:
                time.sleep(0.005)
        except (OSError, FileNotFoundError):
            self.proc = None
        self._t0 = time.monotonic()
        return self

    def _read(self):
        for line in self.proc.stdout:
            self._stamped.append((time.monotonic(), line.strip()))

    def __exit__(self, *exc):
        self._t1 = time.monotonic()
        # keep the samples taken inside the region (the last one before it
        # when the region was shorter than the sampling interval)
        inside = [ln for t, ln in self._stamped if self._t0 <= t <= self._t1 + 0.001 * self.interval_ms]
        if not inside and self._stamped:
            inside = [self._stamped[-1][1]]
        self.lines = inside
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
        "data": "synthetic", "config": desc, "rows_per_step": rows,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "Julia reference unavailable (no Julia toolchain); C restatement of assemble_parallel! timed",
    }))


def timed_steps(ctx, stream, ks, F, G, Cv, flush, steps, warmup, precision, barrier):
    """W untimed + K timed assemblies; CUDA events on the library stream around each
    step, an L2 flush (256 MB write) before each step outside the events."""
    import torch
    for w in range(warmup):
        ctx.assemble_device(ks[w % len(ks)], F, G, Cv, precision=precision)
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ctx.set_timing(True)
    ctx.stats(reset=True)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in range(steps):
        with torch.cuda.stream(stream):
            flush.fill_(s & 0xFF)
            starts[s].record(stream)
        ctx.assemble_device(ks[s % len(ks)], F, G, Cv, precision=precision)
        with torch.cuda.stream(stream):
            ends[s].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    barrier()
    st = ctx.stats(reset=True)
    ctx.set_timing(False)
    dev_ms = sum(a.elapsed_time(b) for a, b in zip(starts, ends))
    return dev_ms, wall, st


def sweep_meshes():
    """Sweep workload: sphere f=16 (2562 nodes), ellipsoid 3:2:1 f=28 (7842 nodes,
    semi-axes 1, 2/3, 1/3), sphere f=45 (20252 nodes); linear triangles."""
    from biegpu import mesh as bm
    return [("sphere_2562", bm.icosphere(16)), ("ellipsoid_7842", bm.ellipsoid(28)),
            ("sphere_20252", bm.icosphere(45))]


def sweep_bench(args, rank, world, max_over_ranks):
    """64 wavenumbers, ka uniform in [0.1, 10] (a = 1, the longest semi-axis),
    boundary data seeded complex N(0,1) per node; every rank runs the whole
    sweep on its own GPU (replicas).  Timed: the mixed path (mixed assembly +
    refined GMRES) and the FP64-grade double-float path on all 64
    wavenumbers, the plain FP64 path on `sweep_fp64_k` evenly spaced ones per
    mesh.  Errors (relative 2-norm of the surface pressure): mixed against the
    double-float solution on every solve of the sweep, and mixed and
    double-float against plain FP64 on the wavenumbers FP64 ran."""
    import biegpu
    named = sweep_meshes()[:max(1, args.sweep_meshes)]
    meshes = [m for _, m in named]
    ks = np.linspace(0.1, 10.0, args.sweep_nk)
    rng = np.random.default_rng(2026)
    ws = [rng.normal(size=m.n_sources) + 1j * rng.normal(size=m.n_sources) for m in meshes]
    biegpu.sweep(meshes, ks[:1], ws, precision="mixed")      # warm-up (contexts, modules)
    t0 = time.perf_counter()
    pm, im = biegpu.sweep(meshes, ks, ws, precision="mixed", target_error=args.sweep_target)
    t_mixed = max_over_ranks(time.perf_counter() - t0)
    # FP64-grade: double-float assembly + FP64 GMRES on complex128 matrices, all wavenumbers
    t0 = time.perf_counter()
    pdf, idf = biegpu.sweep(meshes, ks, ws, precision="df64", refine=False)
    t_df = max_over_ranks(time.perf_counter() - t0)
    sel = np.linspace(0, len(ks) - 1, max(1, min(args.sweep_fp64_k, len(ks)))).round().astype(int)
    t0 = time.perf_counter()
    p64, i64 = biegpu.sweep(meshes, ks[sel], ws, precision="fp64", refine=False)
    t_fp64 = max_over_ranks(time.perf_counter() - t0)

    def rel(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    err_mx_df = [rel(a[:, j], b[:, j]) for a, b in zip(pm, pdf) for j in range(len(ks))]
    err_mx_64 = [rel(a[:, j], b[:, jj]) for a, b in zip(pm, p64) for jj, j in enumerate(sel)]
    err_df_64 = [rel(a[:, j], b[:, jj]) for a, b in zip(pdf, p64) for jj, j in enumerate(sel)]
    worst = int(np.argmax(err_mx_df))
    shapes = {}
    for n, m in named:   # launch shapes the autotuner kept for each mesh's mixed assembly
        sh = biegpu.get_context(m, n=2, m=2).shape("mixed_assembly")
        shapes[n] = {"level": sh[0], "records_per_chunk": sh[1], "threads_per_block": sh[2]} if sh else None
    solves = im["solves"] * world
    v_mixed = solves / t_mixed
    v_fp64 = i64["solves"] * world / t_fp64
    v_df = idf["solves"] * world / t_df
    return {"metric": "sweep solves/s", "value": v_mixed, "unit": "solves/s",
            "meshes": {n: m.n_sources for n, m in named}, "wavenumbers": len(ks), "solves": solves,
            "seconds": t_mixed, "assemble_ms": im["assemble_ms"], "solve_ms": im["solve_ms"],
            "graph_launches": im["graph_launches"], "converged": im["converged"],
            "gmres_iterations_mean": im["iterations"] / max(im["solves"], 1),
            "tuned_assembly_shapes": shapes,
            "target_error": args.sweep_target, "accurate_solves": im.get("accurate_solves", 0),
            "sensitivity_max": float(np.max(im["sensitivity"])) if "sensitivity" in im else None,
            "plain_fp64": {"value": v_fp64, "solves": i64["solves"] * world, "wavenumbers_per_mesh": len(sel),
                           "seconds": t_fp64, "converged": i64["converged"]},
            "df64": {"value": v_df, "solves": idf["solves"] * world, "seconds": t_df,
                     "converged": idf["converged"], "speedup_vs_plain_fp64": v_df / v_fp64,
                     "max_rel_err_vs_fp64": max(err_df_64)},
            "errors": {"mixed_vs_df64_all_solves": {"n": len(err_mx_df), "max": max(err_mx_df),
                                                    "median": float(np.median(err_mx_df)),
                                                    "worst_at": {"mesh": named[worst // len(ks)][0],
                                                                 "ka": float(ks[worst % len(ks)])}},
                       "mixed_vs_fp64": {"n": len(err_mx_64), "max": max(err_mx_64)}},
            "speedup_vs_plain_fp64": v_mixed / v_fp64,
            "max_rel_err_vs_fp64": max(err_mx_64 + err_mx_df),
            "max_rel_err_over": f"{len(err_mx_df)} solves against the FP64-grade double-float solutions "
                                f"and {len(err_mx_64)} against plain FP64",
            "path": "mixed assembly into complex64 matrices + GMRES (restart 20, reltol sqrt(eps)) with "
                    "complex64 products and double-float sums, refined with exact residuals; per solve a "
                    "sensitivity estimate, and FP64-grade re-solves where 5e-7 x estimate > target_error"}


def multi_rhs_bench(args, local, max_over_ranks):
    """Multi-RHS workload: quadratic sphere f=32 (40962 nodes, 20480 tri6),
    256 seeded complex N(0,1) right-hand sides, wavenumbers k, k_v, k_h of air
    at 100 Hz (biegpu.lossy).  One step = F X and G X for all three wavenumbers
    through bie_matvec_multi_device (strip generation in mixed precision +
    tcgen05 FP16 split GEMM).  Compared with the mixed matrix-free product per
    column (timed on a few columns and scaled to 256) and checked against the
    FP64 matrix-free product on two columns per wavenumber."""
    import torch
    import biegpu
    from biegpu import _capi
    from biegpu import mesh as bm
    from biegpu.lossy import boundary_layer_wavenumbers
    mesh = bm.icosphere(args.multi_f, geometry="quadratic")
    N, R = mesh.n_sources, args.multi_rhs
    ctx = biegpu.Context(mesh, n=2, m=2, device=local)
    dev = torch.device(f"cuda:{local}")
    g = torch.Generator(device="cpu").manual_seed(2026)
    X = torch.complex(torch.randn(R, N, generator=g, dtype=torch.float64),
                      torch.randn(R, N, generator=g, dtype=torch.float64)).to(dev).T   # column-major
    YF = torch.empty((R, N), dtype=torch.complex128, device=dev).T
    YG = torch.empty_like(YF)
    ks = boundary_layer_wavenumbers(100.0)
    L = _capi.lib()
    prec = _capi.PRECISION[args.multi_precision]

    def step():
        for k in ks:
            _capi.check(L.bie_matvec_multi_device(ctx.handle, k.real, k.imag, R, X.data_ptr(), X.data_ptr(),
                                                  YF.data_ptr(), YG.data_ptr(), prec, 0))

    step()   # warm-up (scratch, modules)
    torch.cuda.synchronize(dev)
    ctx.set_timing(True)
    ctx.stats(reset=True)
    steps = max(1, args.multi_steps)
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    torch.cuda.synchronize(dev)
    t = max_over_ranks(time.perf_counter() - t0) / steps
    st = ctx.stats(reset=True)
    ctx.set_timing(False)
    # accuracy against the FP64 matrix-free product, two columns per wavenumber
    errs = []
    for k in ks:
        _capi.check(L.bie_matvec_multi_device(ctx.handle, k.real, k.imag, R, X.data_ptr(), X.data_ptr(),
                                              YF.data_ptr(), YG.data_ptr(), prec, 0))
        for c in (0, R - 1):
            x = X[:, c].contiguous()
            yF, yG = torch.empty_like(x), torch.empty_like(x)
            _capi.check(L.bie_matvec_device(ctx.handle, k.real, k.imag, None, 0, x.data_ptr(), x.data_ptr(),
                                            yF.data_ptr(), yG.data_ptr(), _capi.BIE_PREC_FP64))
            torch.cuda.synchronize(dev)
            errs.append(float(torch.linalg.norm(YF[:, c] - yF) / torch.linalg.norm(yF)))
            errs.append(float(torch.linalg.norm(YG[:, c] - yG) / torch.linalg.norm(yG)))
    # the matrix-free mixed product, one column at a time
    ncol = 2
    t0 = time.perf_counter()
    for k in ks:
        _capi.check(L.bie_matvec_multi_device(ctx.handle, k.real, k.imag, ncol, X.data_ptr(), X.data_ptr(),
                                              YF.data_ptr(), YG.data_ptr(), _capi.BIE_PREC_MIXED, 0))
    torch.cuda.synchronize(dev)
    t_col = (time.perf_counter() - t0) / ncol
    peaks = measured_peaks()
    bf16 = peaks.get("bf16_tflops", 1900.0)
    gemm_ms = st["tensor_ms"] / steps
    executed_tf = st["tensor_flops_executed"] / max(st["tensor_ms"], 1e-9) / 1e9
    algo_tf = st["tensor_flops"] / max(st["tensor_ms"], 1e-9) / 1e9
    del X, YF, YG
    ctx.close()
    torch.cuda.empty_cache()
    return {"metric": "multi-RHS operator products/s", "value": 2 * len(ks) * R / t, "unit": "rhs-products/s",
            "workload": f"quadratic sphere f={args.multi_f} ({N} nodes), {R} RHS, k={ks[0]:.4f}, k_v={ks[1]:.1f}, "
                        f"k_h={ks[2]:.1f} (air, 100 Hz); F X and G X per wavenumber",
            "precision": args.multi_precision, "ms_per_step": 1e3 * t,
            "entries_per_s": 2 * len(ks) * float(N) * N / t,
            "gemm": {"kernel": "lowp_gemm_kernel", "ms_per_step": gemm_ms, "launches_per_step": st["tensor_launches"] / steps,
                     "roofline": {"bound": "tensor", "achieved": executed_tf, "peak": bf16, "unit": "TFLOP/s",
                                  "frac": executed_tf / bf16, "algorithmic_tflops": algo_tf,
                                  "peak_source": "MEASURED_PEAKS.json bf16_tflops (cuBLAS bf16 burst) of measured",
                                  "note": "executed = issued MMA flops incl. padding and the three split products"}},
            "generation_ms_per_step": st["timed_ms"] / steps,
            "max_rel_err_vs_fp64": max(errs), "median_rel_err_vs_fp64": float(np.median(errs)),
            "per_column_mixed": {"ms_per_rhs_all_k": 1e3 * t_col, "speedup": t_col * R / t}}


def progress(msg: str) -> None:
    """One progress line on stderr (the JSON line stays alone on stdout)."""
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def multi_solve_bench(args, local, max_over_ranks):
    """Multi-RHS solve workload (the same quadratic sphere, 256 seeded complex
    N(0,1) right-hand sides, wavenumbers k, k_v, k_h of air at 100 Hz):
    (F + Diagonal(1 - C)) X = B for all columns at once
    (bie_solve_multi_device: lockstep GMRES with tcgen05 FP16-split products,
    refined with exact complex64 residuals to sqrt(eps)).  One column per
    wavenumber is checked against an FP64-grade matrix-free GMRES solve
    (double-float products of F, C from the double-float assembly)."""
    import torch
    import biegpu
    from biegpu import Diagonal, GPUFOperator, gmres
    from biegpu import mesh as bm
    from biegpu.lossy import boundary_layer_wavenumbers
    mesh = bm.icosphere(args.multi_f, geometry="quadratic")
    N, R = mesh.n_sources, args.multi_rhs
    ctx = biegpu.get_context(mesh, n=2, m=2, device=local)
    dev = torch.device(f"cuda:{local}")
    g = torch.Generator(device="cpu").manual_seed(2027)
    B = torch.complex(torch.randn(R, N, generator=g, dtype=torch.float64),
                      torch.randn(R, N, generator=g, dtype=torch.float64)).to(dev).T
    ks = boundary_layer_wavenumbers(100.0)
    biegpu.solve_multi(mesh, ks[0], B[:, :2], ctx=ctx)          # warm-up (modules, scratch)
    per_k, infos, errs = [], [], []
    for k in ks:
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        X, info = biegpu.solve_multi(mesh, k, B, ctx=ctx)
        torch.cuda.synchronize(dev)
        per_k.append(time.perf_counter() - t0)
        infos.append(info)
        progress(f"multi-RHS solve k={k:.4g}: {per_k[-1]:.2f} s, passes {info['passes']}, "
                 f"inner steps {info['inner_steps']}, converged {info['converged']}/{R}")
        Cv = torch.empty(N, dtype=torch.complex128, device=dev)
        ctx.assemble_device(k, None, None, Cv, precision="df64")
        torch.cuda.synchronize(dev)
        c = R - 1
        t1 = time.perf_counter()
        xr, gres = gmres(GPUFOperator(mesh, k) + Diagonal(1.0 - Cv), B[:, c].contiguous(), reltol=1e-12,
                         maxiter=600, precision="df64", log=True)
        errs.append(float(torch.linalg.norm(X[:, c] - xr) / torch.linalg.norm(xr)))
        progress(f"  check column: df64 matrix-free GMRES {time.perf_counter() - t1:.2f} s, "
                 f"{gres.iterations} iterations, error {errs[-1]:.2e}")
        del X
        torch.cuda.empty_cache()
    total = max_over_ranks(sum(per_k))
    return {"metric": "multi-RHS solves/s", "value": len(ks) * R / total, "unit": "solves/s",
            "workload": f"quadratic sphere f={args.multi_f} ({N} nodes), {R} RHS, k, k_v, k_h (air, 100 Hz)",
            "seconds_per_wavenumber": per_k, "passes": [i["passes"] for i in infos],
            "inner_steps": [i["inner_steps"] for i in infos],
            "setup_ms": [i["setup_ms"] for i in infos], "tensor_ms": [i["tensor_ms"] for i in infos],
            "exact_ms": [i["exact_ms"] for i in infos], "converged": [i["converged"] for i in infos],
            "max_relres": max(i["max_relres"] for i in infos),
            "rel_err_vs_df64_matrix_free_gmres": errs,
            "path": "mixed assembly (complex64 F) quantised once to FP16 split tiles; lockstep GMRES (restart 20, "
                    "inner 1e-4) on tcgen05 products; refinement with exact complex64 residuals to sqrt(eps)"}


def nearfield_bench(args, max_over_ranks):
    """Near-field and fast-operator workload: pulsating-sphere mesh (f=32, 10242
    nodes, linear), k = 2 pi 200 / 343.  Times (1) the accurate near field of F
    and G on the depth-1 connected_sources pattern with the fast operators'
    offset 0.2 (sparse_assemble_parallel!), (2) one product of the fast
    operator (FMMFOperator algorithm: Gauss-rule far field summed exactly +
    near-field correction) against (3) the matrix-free product of the exact
    dense rows (GPUFOperator), FP64, double-float (FP64-grade) and mixed."""
    import biegpu
    from biegpu import FMMFOperator, GPUFOperator
    from biegpu import mesh as bm
    from biegpu.assembly import nearfield_values
    mesh = bm.icosphere(32)
    k = 2 * np.pi * 200 / 343
    ctx = biegpu.get_context(mesh, n=2, m=2)
    reps = max(1, args.nearfield_steps)
    rp, cols, _, _ = nearfield_values(ctx, k, depth=1, offset=0.2)   # builds pattern and rules
    ctx.set_timing(True)
    ctx.stats(reset=True)
    t0 = time.perf_counter()
    for _ in range(reps):
        nearfield_values(ctx, k, depth=1, offset=0.2)
    t_near = max_over_ranks(time.perf_counter() - t0) / reps
    st = ctx.stats(reset=True)
    ctx.set_timing(False)
    x = np.random.default_rng(3).normal(size=mesh.n_sources) + 0j
    out = {"workload": f"icosphere f=32 ({mesh.n_sources} nodes, {mesh.n_elements} linear elements), "
                       "k = 2 pi 200/343, depth 1, offset 0.2",
           "nnz": int(len(cols)), "near_field_ms": 1e3 * t_near,
           "near_field_kernel_ms": st["timed_ms"] / max(st["timed_launches"], 1) if st["timed_launches"] else None}
    t0 = time.perf_counter()
    op = FMMFOperator(mesh, k, precision="fp64")
    out["fast_operator_setup_ms"] = 1e3 * (time.perf_counter() - t0)
    for prec in ("fp64", "df64", "mixed"):
        op.precision = prec
        dense = GPUFOperator(mesh, k, precision=prec)
        op @ x
        dense @ x
        t0 = time.perf_counter()
        for _ in range(reps):
            op @ x
        t_fast = (time.perf_counter() - t0) / reps
        t0 = time.perf_counter()
        for _ in range(reps):
            dense @ x
        t_dense = (time.perf_counter() - t0) / reps
        out[f"product_ms_{prec}"] = {"fast_operator": 1e3 * t_fast, "exact_rows": 1e3 * t_dense}
    return out


def lossy_bench(args, max_over_ranks):
    """Visco-thermal workload: LossyGlobalOuter on a sphere f=16 (2562 nodes,
    linear, radius 1) at 100 Hz, depth 1, n = m = 3 (the reference's
    defaults), dense acoustic blocks.  Times the device set-up (FP64 acoustic
    assembly, thermal / viscous near field, derivative matrices), the product
    L x (with its nested gmres calls) and the solve of the reference test's
    system (test/3d/losses_test.jl:30-35: v0 = 0.01 normal velocity)."""
    import biegpu
    from biegpu import mesh as bm
    mesh = bm.icosphere(16)
    N = mesh.n_sources
    t0 = time.perf_counter()
    L = biegpu.LossyGlobalOuter(mesh, 100.0, depth=1, n=3)
    t_setup = time.perf_counter() - t0
    x = np.random.default_rng(4).normal(size=N) + 1j * np.random.default_rng(5).normal(size=N)
    reps = max(1, args.lossy_steps)
    per_op = {}
    for one_launch in (False, True):   # sparse solves per operation, then as one cluster launch each
        L.set_one_launch(one_launch)
        L @ x
        L.stats(reset=True)
        L.ctx.stats(reset=True)
        t0 = time.perf_counter()
        for _ in range(reps):
            L @ x
        t_prod = max_over_ranks(time.perf_counter() - t0) / reps
        launches = L.ctx.stats(reset=True)["kernel_launches"] / reps
        st = L.stats(reset=True)
        if not one_launch:
            per_op = {"product_ms": 1e3 * t_prod, "launches_per_product": launches}
    v0 = np.concatenate([0.01 * np.ones(N), np.zeros(2 * N)])
    t0 = time.perf_counter()
    rhs = L.rhs(v0)
    pa, info = L.solve(rhs, return_info=True)
    t_solve = max_over_ranks(time.perf_counter() - t0)
    st2 = L.stats(reset=True)
    res = float(np.linalg.norm(L @ pa - rhs) / np.linalg.norm(rhs))
    return {"workload": f"icosphere f=16 ({N} nodes, linear), 100 Hz, depth 1, n = m = 3, dense acoustic blocks",
            "setup_s": t_setup, "product_ms": 1e3 * t_prod, "launches_per_product": launches,
            "per_operation_sparse_solves": per_op,
            "nested_solves_per_product": st["nested_solves"] / reps,
            "nested_iterations_per_product": st["nested_iterations"] / reps,
            "solve_s": t_solve, "outer_iterations": info["iterations"], "converged": info["converged"],
            "solve_nested_iterations": st2["nested_iterations"], "relative_residual": res,
            "timing": "host wall clock (the nested solves synchronise with the host)"}


def adjoint_bench(args, max_over_ranks):
    """Adjoint workload: ellipsoid 3:2:1 f=22 (4842 nodes, linear), ka=3, 32
    seeded field points on the radius-10 sphere, seeded impedances |Z| = rho c.
    One step = J and its gradient with respect to all vertex coordinates and
    element impedances (forward solve, adjoint solve, reverse pass)."""
    import biegpu
    from biegpu import mesh as bm
    rho_c = 1.21 * 343.0
    P, T = bm.icosphere_arrays(22)
    P = P * np.array([1.0, 2 / 3, 1 / 3])[:, None]
    P = P + 2e-3 * np.random.default_rng(0).normal(size=P.shape) / 22
    mesh = bm._finish(P, T + 1, "linear", "geometry")
    rng = np.random.default_rng(1)
    Z = rho_c * np.exp(1j * rng.uniform(-1.0, 1.0, mesh.n_elements))
    Xf = rng.normal(size=(3, 32))
    Xf *= 10.0 / np.linalg.norm(Xf, axis=0)
    k = 3.0
    biegpu.farfield_objective(mesh, k, Z, Xf, rho_c=rho_c)   # warm-up
    steps = max(1, args.adjoint_steps)
    t0 = time.perf_counter()
    for _ in range(steps):
        J, _, dX, dZ, info = biegpu.farfield_objective(mesh, k, Z, Xf, rho_c=rho_c)
    t_grad = max_over_ranks(time.perf_counter() - t0) / steps
    t0 = time.perf_counter()
    for _ in range(steps):
        biegpu.farfield_objective(mesh, k, Z, Xf, rho_c=rho_c, gradient=False)
    t_fwd = max_over_ranks(time.perf_counter() - t0) / steps
    # forward model assembled in double-float (FP64-grade), reverse pass FP64
    biegpu.farfield_objective(mesh, k, Z, Xf, rho_c=rho_c, precision="df64")
    t0 = time.perf_counter()
    for _ in range(steps):
        Jd, _, dXd, _, _ = biegpu.farfield_objective(mesh, k, Z, Xf, rho_c=rho_c, precision="df64")
    t_grad_df = max_over_ranks(time.perf_counter() - t0) / steps
    h = 1e-6
    v, c = 1234, 2
    Pp = mesh.coordinates.copy()
    Pp[c, v] += h
    Jp = biegpu.farfield_objective(bm._finish(Pp, mesh.topology, "linear", "geometry"), k, Z, Xf, rho_c=rho_c,
                                   gradient=False)[0]
    Pp[c, v] -= 2 * h
    Jm = biegpu.farfield_objective(bm._finish(Pp, mesh.topology, "linear", "geometry"), k, Z, Xf, rho_c=rho_c,
                                   gradient=False)[0]
    fd = (Jp - Jm) / (2 * h)
    n_params = 3 * mesh.coordinates.shape[1] + 2 * mesh.n_elements
    return {"metric": "adjoint gradients/s", "value": 1.0 / t_grad, "unit": "gradients/s",
            "workload": f"ellipsoid 3:2:1 f=22 ({mesh.n_sources} nodes, {mesh.n_elements} elements), ka=3, "
                        "32 field points at radius 10",
            "ms_per_gradient": 1e3 * t_grad, "ms_per_forward": 1e3 * t_fwd, "parameters": n_params,
            "df64_forward": {"ms_per_gradient": 1e3 * t_grad_df,
                             "J_rel_diff": abs(Jd - J) / abs(J),
                             "dX_rel_diff": float(np.linalg.norm(dXd - dX) / np.linalg.norm(dX))},
            "central_fd_equivalent_s": 2 * n_params * t_fwd,
            "fd_check": {"component": f"dX[{c},{v}]", "adjoint": float(dX[c, v]), "central_fd_h1e-6": fd,
                         "rel_to_max": abs(fd - dX[c, v]) / float(np.abs(dX).max())},
            "gmres_iterations": [info["forward_iterations"], info["adjoint_iterations"]]}


def profile_case(name: str) -> None:
    """Small runs of single kernels for ncu captures (profiles/*.md give the
    commands): `multi` (multi-RHS products: strip generation, quantisation,
    tcgen05 GEMM, reduction; 5762-node P2 sphere, 64 RHS), `df64mv` (double-
    float matrix-free products, same mesh), `gemv` (dense GMRES on a 6252-node
    sphere: complex128 FP64 products), `taylor` (ROSEBEM k-derivative
    assembly, 2562-node P2 sphere), `sweep` (mixed frequency sweep of the
    2562-node sphere, 8 wavenumbers, launch by launch: complex64 products and
    the exact products of the refinement residuals), `mixedmv` (mixed-precision
    matrix-free products F x, 5762-node P2 sphere), `multisolve` (64 right-hand
    sides on the 5762-node P2 sphere), `sweepgraph` (the recorded-graph sweep of
    the 2562-node sphere, 8 wavenumbers), `adjoint` (one gradient on a 1002-node
    ellipsoid), `misc` (the remaining helper kernels: fast-operator product, the
    standalone tensor-core GEMM, dense mixed GMRES on an odd-sized system, a
    launch-per-operation lossy product), `lossy` (LossyGlobalOuter
    products on the 2562-node sphere at 100 Hz: the one-launch sparse GMRES
    solves and the rest of the product)."""
    import torch
    import biegpu
    from biegpu import _capi
    from biegpu import mesh as bm
    dev = torch.device("cuda:0")
    L = _capi.lib()
    if name == "multi":
        mesh = bm.icosphere(12, geometry="quadratic")
        N, R = mesh.n_sources, 64
        g = torch.Generator().manual_seed(1)
        X = torch.complex(torch.randn(R, N, generator=g, dtype=torch.float64),
                          torch.randn(R, N, generator=g, dtype=torch.float64)).to(dev).T
        ctx = biegpu.Context(mesh, n=2, m=2)
        Y = torch.empty((R, N), dtype=torch.complex128, device=dev).T
        for _ in range(4):
            _capi.check(L.bie_matvec_multi_device(ctx.handle, 4.0, 0.0, R, X.data_ptr(), None, Y.data_ptr(),
                                                  None, _capi.PRECISION["fp16_split"], 0))
    elif name == "df64mv":
        mesh = bm.icosphere(12, geometry="quadratic")
        ctx = biegpu.Context(mesh, n=2, m=2)
        x = torch.randn(mesh.n_sources, dtype=torch.complex128, device=dev)
        y = torch.empty_like(x)
        for _ in range(4):
            _capi.check(L.bie_matvec_device(ctx.handle, 4.0, 0.0, None, 0, x.data_ptr(), None, y.data_ptr(), None,
                                            _capi.BIE_PREC_DF64))
    elif name == "gemv":
        from biegpu import Diagonal, gmres
        mesh = bm.icosphere(25)
        Fp, _, Cp = biegpu.assemble_parallel(mesh, 3.0, mesh.sources, n=2, m=2, gOn=False)
        b = np.random.default_rng(1).normal(size=mesh.n_sources) + 0j
        gmres(Fp + Diagonal(1.0 - Cp), b, ctx=biegpu.get_context(mesh, n=2, m=2))
    elif name == "taylor":
        mesh = bm.icosphere(8, geometry="quadratic")
        for _ in range(2):
            biegpu.taylor_assemble(mesh, 3.0, M=2, n=2, m=2)
    elif name == "sweep":
        mesh = bm.icosphere(16)
        w = np.random.default_rng(2).normal(size=mesh.n_sources) + 0j
        biegpu.sweep([mesh], np.linspace(0.5, 8.0, 8), [w], precision="mixed", eager=True, target_error=0)
    elif name == "multisolve":
        mesh = bm.icosphere(12, geometry="quadratic")
        g = torch.Generator().manual_seed(3)
        B = torch.complex(torch.randn(64, mesh.n_sources, generator=g, dtype=torch.float64),
                          torch.randn(64, mesh.n_sources, generator=g, dtype=torch.float64)).to(dev).T
        biegpu.solve_multi(mesh, 3.0, B)
    elif name == "sweepgraph":
        mesh = bm.icosphere(16)
        w = np.random.default_rng(2).normal(size=mesh.n_sources) + 0j
        biegpu.sweep([mesh], np.linspace(0.5, 8.0, 8), [w], precision="mixed", target_error=1e-6)
    elif name == "adjoint":
        P, T = bm.icosphere_arrays(10)
        P = P * np.array([1.0, 2 / 3, 1 / 3])[:, None]
        mesh = bm._finish(P, T + 1, "linear", "geometry")
        rng = np.random.default_rng(1)
        Z = 1.21 * 343.0 * np.exp(1j * rng.uniform(-1.0, 1.0, mesh.n_elements))
        Xf = rng.normal(size=(3, 8))
        Xf *= 10.0 / np.linalg.norm(Xf, axis=0)
        biegpu.farfield_objective(mesh, 3.0, Z, Xf, rho_c=1.21 * 343.0)
    elif name == "misc":
        # the remaining helper kernels: fast-operator product (sparse near-field
        # correction), the standalone tensor-core GEMM, dense mixed GMRES on an
        # odd-sized system (complex64 rounding, one-row GEMV forms), and a
        # launch-per-operation GMRES on vectors above 4096 entries
        from biegpu import Diagonal, gmres
        mesh = bm.icosphere(9)
        xr = np.random.default_rng(1).normal(size=mesh.n_sources) + 0j
        biegpu.FMMFOperator(mesh, 2.0) @ xr
        ctx = biegpu.get_context(mesh, n=2, m=2)
        # open curved plate of 41 x 41 = 1681 nodes (an odd count)
        nx, h = 40, 0.05
        xs, ys = np.meshgrid(np.arange(nx + 1) * h, np.arange(nx + 1) * h, indexing="xy")
        c0 = 0.5 * nx * h
        Pp = np.vstack([xs.ravel(), ys.ravel(), 0.5 * ((xs.ravel() - c0) ** 2 + (ys.ravel() - c0) ** 2)])
        Tp = []
        for j in range(nx):
            for i in range(nx):
                a = j * (nx + 1) + i
                Tp += [[a, a + 1, a + nx + 2], [a, a + nx + 2, a + nx + 1]]
        plate = bm._finish(Pp, np.array(Tp, dtype=np.int64).T + 1, "linear", "geometry")
        Fp, _, Cp = biegpu.assemble_parallel(plate, 2.0, plate.sources, n=2, m=2, gOn=False)
        gmres(Fp + Diagonal(1.0 - Cp), np.exp(2j * plate.sources[0]), refine=True, reltol=1e-10, maxiter=200,
              ctx=biegpu.get_context(plate, n=2, m=2))
        A = torch.randn(256, 512, device=dev, dtype=torch.float32)
        Bm = torch.randn(384, 512, device=dev, dtype=torch.float32)
        Cm = torch.empty(256, 384, device=dev, dtype=torch.float64)
        _capi.check(L.bie_lowp_gemm_device(ctx.handle, _capi.PRECISION["fp16_split"], 256, 384, 512, A.data_ptr(),
                                           Bm.data_ptr(), Cm.data_ptr()))
        m16 = bm.icosphere(16)
        Lo = biegpu.LossyGlobalOuter(m16, 100.0, depth=1, n=3)
        Lo.set_one_launch(False)
        Lo @ (np.random.default_rng(4).normal(size=m16.n_sources) + 0j)
    elif name == "mixedmv":
        mesh = bm.icosphere(12, geometry="quadratic")
        ctx = biegpu.Context(mesh, n=2, m=2)
        x = torch.randn(mesh.n_sources, dtype=torch.complex128, device=dev)
        y = torch.empty_like(x)
        for _ in range(4):
            _capi.check(L.bie_matvec_device(ctx.handle, 4.0, 0.0, None, 0, x.data_ptr(), None, y.data_ptr(), None,
                                            _capi.BIE_PREC_MIXED))
    elif name == "lossy":
        mesh = bm.icosphere(16)
        Lo = biegpu.LossyGlobalOuter(mesh, 100.0, depth=1, n=3)
        x = np.random.default_rng(4).normal(size=mesh.n_sources) + 1j * np.random.default_rng(5).normal(
            size=mesh.n_sources)
        for _ in range(3):
            Lo @ x
    else:
        raise SystemExit(f"unknown profile case {name}")
    torch.cuda.synchronize()
    print("profile case", name, "done")


def roofline_entry(st, kernel, bound, peak_flops, workload_name, nphys):
    kernel_ms = st["timed_ms"] / max(st["timed_launches"], 1)
    flops = st["algorithmic_flops"] / max(st["timed_launches"], 1)
    achieved = flops / (kernel_ms * 1e-3) / 1e12
    peak = peak_flops / 1e12
    tr = ncu_traffic(kernel, workload_name)
    return {"bound": bound, "kernel": kernel, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak,
            "peak_source": f"measured {bound.upper()} FMA-chain throughput (bie_measure_peaks) on this GPU",
            "traffic": tr.get("dram_bytes_per_launch") if tr else None,
            "traffic_how": tr.get("how") if tr else None,
            "flops_per_launch": flops, "kernel_ms": kernel_ms,
            "qpe_per_launch": st["quadrature_evals"] / max(st["timed_launches"], 1),
            "flops_per_qpe": f"32 + 8 n_phys (n_phys={nphys})"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="rigid_sphere_p2")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="mixed",
                    help="arithmetic of the headline path (the plain FP64 path is always timed beside it)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 comparison run")
    ap.add_argument("--no-sweep", action="store_true", help="skip the frequency-sweep measurement")
    ap.add_argument("--sweep-fp64-k", type=int, default=16,
                    help="wavenumbers per mesh timed on the plain FP64 path (the error check set)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--sweep-nk", type=int, default=64, help="wavenumbers of the sweep")
    ap.add_argument("--sweep-target", type=float, default=1e-6,
                    help="mixed sweep: re-solve at FP64 grade where the predicted error exceeds this (0: off)")
    ap.add_argument("--sweep-meshes", type=int, default=3, help="use the first n of the three sweep meshes")
    ap.add_argument("--no-multi", action="store_true", help="skip the multi-RHS tensor-core measurement")
    ap.add_argument("--multi-rhs", type=int, default=256)
    ap.add_argument("--multi-f", type=int, default=32, help="sphere frequency of the multi-RHS mesh (32: 40962 nodes)")
    ap.add_argument("--multi-steps", type=int, default=3)
    ap.add_argument("--no-multi-solve", action="store_true", help="skip the multi-RHS solve")
    ap.add_argument("--multi-precision", default="fp16_split",
                    choices=["fp16", "bf16", "fp16_split", "bf16_split"])
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint-gradient measurement")
    ap.add_argument("--adjoint-steps", type=int, default=3)
    ap.add_argument("--no-nearfield", action="store_true", help="skip the near-field / fast-operator measurement")
    ap.add_argument("--nearfield-steps", type=int, default=3)
    ap.add_argument("--no-lossy", action="store_true", help="skip the visco-thermal system measurement")
    ap.add_argument("--lossy-steps", type=int, default=3)
    ap.add_argument("--profile-case", default=None,
                    help="run one small kernel case for an ncu capture and exit (see profile_case)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    if args.profile_case:
        profile_case(args.profile_case)
        return

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

    def max_over_ranks(x):
        t = torch.tensor([x], dtype=torch.float64, device=f"cuda:{local}")
        if dist is not None:
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    mesh, ks, desc = workload(args.workload)
    # weak scaling: every rank assembles its own share of the frequency list
    ks = ks[rank % len(ks):] + ks[:rank % len(ks)]
    N = mesh.n_sources
    nphys = 3 if mesh.physics_function == "linear" else 6
    ctx = biegpu.Context(mesh, n=2, m=2, device=local)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=f"cuda:{local}")
    dev = torch.device(f"cuda:{local}")
    F = torch.empty((N, N), dtype=torch.complex128, device=dev)
    G = torch.empty_like(F)
    Cv = torch.empty(N, dtype=torch.complex128, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    entries_per_step = 2.0 * N * N
    peaks = biegpu._capi.measure_peaks(local)

    progress(f"headline assembly: {args.workload}, {N} nodes, {args.steps} steps")
    with ClockSampler(local) as clk:
        dev_ms, wall, st = timed_steps(ctx, stream, ks, F, G, Cv, flush, args.steps, args.warmup,
                                       args.precision, barrier)
    dev_ms = max_over_ranks(dev_ms)
    value = entries_per_step * args.steps * world / (dev_ms * 1e-3)
    gpu_launches = st["kernel_launches"]
    if args.precision == "mixed":
        roofline = roofline_entry(st, "assemble_mixed_kernel", "fp32", peaks["fp32_flops"], args.workload, nphys)
    else:
        roofline = roofline_entry(st, "assemble_fp64_kernel", "fp64", peaks["fp64_flops"], args.workload, nphys)

    # ---- the plain FP64 GPU path, and the mixed path's error against it ------
    plain = None
    accuracy = None
    if args.precision == "mixed" and not args.no_fp64:
        progress("plain FP64 and double-float assemblies")
        p_ms, _, pst = timed_steps(ctx, stream, ks, F, G, Cv, flush, max(2, args.steps // 2), 1, "fp64", barrier)
        p_ms = max_over_ranks(p_ms)
        psteps = max(2, args.steps // 2)
        plain = {"value": entries_per_step * psteps * world / (p_ms * 1e-3), "unit": UNIT,
                 "ms_per_step": p_ms / psteps,
                 "roofline": roofline_entry(pst, "assemble_fp64_kernel", "fp64", peaks["fp64_flops"],
                                            args.workload, nphys)}
        kerr = max(ks)
        ctx.assemble_device(kerr, F, G, Cv, precision="fp64")
        F2 = torch.empty_like(F)
        G2 = torch.empty_like(F)
        C2 = torch.empty_like(Cv)
        ctx.assemble_device(kerr, F2, G2, C2, precision="mixed")
        torch.cuda.synchronize()
        accuracy = {"k": kerr, "vs": "plain FP64 GPU assembly (same inputs)",
                    "F_rel_fro": float(torch.linalg.norm(F2 - F) / torch.linalg.norm(F)),
                    "G_rel_fro": float(torch.linalg.norm(G2 - G) / torch.linalg.norm(G)),
                    "C_rel": float(torch.linalg.norm(C2 - Cv) / torch.linalg.norm(Cv))}
        # FP64-grade assembly in double-float arithmetic (BIE_PREC_DF64)
        ctx.assemble_device(kerr, F2, G2, C2, precision="df64")
        torch.cuda.synchronize()
        df_acc = {"F_rel_fro": float(torch.linalg.norm(F2 - F) / torch.linalg.norm(F)),
                  "G_rel_fro": float(torch.linalg.norm(G2 - G) / torch.linalg.norm(G)),
                  "C_rel": float(torch.linalg.norm(C2 - Cv) / torch.linalg.norm(Cv)), "k": kerr}
        del F2, G2, C2
        d_ms, _, dst = timed_steps(ctx, stream, ks, F, G, Cv, flush, psteps, 1, "df64", barrier)
        d_ms = max_over_ranks(d_ms)
        plain["df64"] = {"value": entries_per_step * psteps * world / (d_ms * 1e-3), "unit": UNIT,
                         "ms_per_step": d_ms / psteps, "speedup_vs_fp64": p_ms / d_ms,
                         "kernel": "assemble_df64_kernel (regular pairs in float-pair arithmetic on the "
                                   "FP32 pipes) + correct_fp64_kernel (near pairs in FP64)",
                         "accuracy_vs_fp64": df_acc}
        # FP64-equivalent algorithmic flops of the double-float kernel; it runs on
        # the FP32 pipes, so its roofline is FP32 issue (one FP64-equivalent
        # flop costs ~10-20 FP32 instructions); the FP64 pipe ratio says how far
        # FP64-grade results beat the FP64 pipe itself
        rdf = roofline_entry(dst, "assemble_df64_kernel", "fp32", peaks["fp32_flops"], args.workload, nphys)
        plain["df64"]["roofline"] = {
            "bound": "fp32 issue", "fp64_equivalent_tflops": rdf["achieved"], "kernel_ms": rdf["kernel_ms"],
            "vs_fp32_peak": rdf["frac"], "vs_fp64_pipe_peak": rdf["achieved"] / (peaks["fp64_flops"] / 1e12)}

    # ---- end to end through the host-buffer C-ABI call -----------------------
    e2e = None
    if not args.no_e2e:
        progress("end to end through the host-buffer call")
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
        n_e2e = max(1, min(args.steps, 5))
        t0 = time.perf_counter()
        for s in range(n_e2e):
            ctx.assemble(ks[s % len(ks)], targets=tg, out=(Fh, Gh, Ch), precision=args.precision)
        e2e_s = max_over_ranks(time.perf_counter() - t0)
        e2e = {"value": entries_per_step * n_e2e * world / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": int(tg.nbytes), "d2h_bytes_per_step": int(Fh.nbytes + Gh.nbytes + Ch.nbytes),
               "steps": n_e2e, "call": "bie_assemble (host buffers, pinned)"}
        if plain is not None:
            # the same host-buffer call at FP64 grade (double-float assembly)
            ctx.assemble(ks[0], targets=tg, out=(Fh, Gh, Ch), precision="df64")
            barrier()
            t0 = time.perf_counter()
            for s in range(n_e2e):
                ctx.assemble(ks[s % len(ks)], targets=tg, out=(Fh, Gh, Ch), precision="df64")
            e2e_df = max_over_ranks(time.perf_counter() - t0)
            plain["df64"]["e2e"] = {"value": entries_per_step * n_e2e * world / e2e_df, "unit": UNIT,
                                    "h2d_bytes_per_step": int(tg.nbytes),
                                    "d2h_bytes_per_step": int(Fh.nbytes + Gh.nbytes + Ch.nbytes),
                                    "steps": n_e2e, "call": "bie_assemble (host buffers, pinned), df64"}

    # ---- batched frequency sweep (3 meshes x 64 wavenumbers): solves/s -----
    sweep = None
    if not args.no_sweep:
        progress("frequency sweep")
        sweep = sweep_bench(args, rank, world, max_over_ranks)

    # ---- multi-RHS tensor-core products and adjoint gradients ---------------
    multi = None
    if not args.no_multi:
        progress("multi-RHS products")
        multi = multi_rhs_bench(args, local, max_over_ranks)
        if not args.no_multi_solve:
            progress("multi-RHS solve")
            multi["solve"] = multi_solve_bench(args, local, max_over_ranks)
    adjoint = None
    if not args.no_adjoint:
        progress("adjoint gradients")
        adjoint = adjoint_bench(args, max_over_ranks)
    nearfield = None
    if not args.no_nearfield:
        progress("near field and fast operators")
        nearfield = nearfield_bench(args, max_over_ranks)
    lossy = None
    if not args.no_lossy:
        progress("visco-thermal system")
        lossy = lossy_bench(args, max_over_ranks)

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    cpu = None
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, rows, dt = cpu_baseline(mesh, ks, args.cpu_seconds, threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{rows} of {N} rows of F, G, C at k={ks[0]} ({dt:.1f} s)"}

    # key order: the headline keys, then the bulky per-workload sections, and
    # last the FP64 comparison, the accuracy and the sweep (the end of the line
    # is what a log tail keeps)
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "wall_ms_per_step": 1e3 * wall / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if args.precision == "mixed" else "f64",
        "precision": args.precision, "data": "synthetic", "config": desc,
        "rows_per_step": N, "l2": "256 MB L2 flush between steps; each step writes 4.3 GB",
        "parallelism": f"replicas{world}",
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": gpu_launches,
        "clocks": clk.summary(), "gpu": torch.cuda.get_device_name(dev),
        "peaks": {"fp64_tflops": peaks["fp64_flops"] / 1e12, "fp32_tflops": peaks["fp32_flops"] / 1e12,
                  "fp_how": "bie_measure_peaks: dependent FMA chains on every SM (CUDA events), this GPU",
                  "hbm_gbs": measured_peaks().get("hbm_gbs"), "bf16_tflops": measured_peaks().get("bf16_tflops"),
                  "hbm_bf16_how": "MEASURED_PEAKS.json"},
        "multi_rhs": multi, "adjoint": adjoint, "nearfield": nearfield, "lossy": lossy,
        "plain_fp64": plain, "accuracy": accuracy, "sweep": sweep,
    }
    print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

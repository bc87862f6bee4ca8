"""Benchmark: AMG-preconditioned CG to 1e-8 relative residual on the 256^3
27-point lognormal diffusion system (16.7M rows, 449M non-zeros, CSR, FP64
values, int32 columns), plain FP64 and mixed precision, plus the CSR SpMV
bandwidth on the same matrix.

One step = one full AMG-PCG solve from x0 = 0 (hierarchy set up once,
outside the timed region; its setup time is reported separately).  The
matrix (5.7 GB) is far larger than the 129 MB L2, so no flush is needed
between steps.  Inputs are seeded synthetic data: conductivity
k = exp(1.5 N(0,1)) (numpy PCG64, seed 1), b ~ U[-1, 1] (seed 0).

--impl reference times the CPU restatement of lineal's shared-memory path
(oracle/, the reference itself cannot be built: its thesauros/grex
dependencies are not vendored) on all host cores, on the same 256^3 system
and a hierarchy built with lineal's own partition rule; each timed step is
one full solve to 1e-8.

Multi-GPU: the solve path has no exchange step on one box; N > 1 runs N
independent replicas (one system per rank, weak scaling) and reports the
slowest rank.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "AMG-PCG ms to 1e-8 rel. residual & SpMV HBM GB/s at 256^3: mixed vs plain FP64"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def autotune_log(name, h):
    """Runs the row-engine autotuner on hierarchy `h`, logs each choice and
    returns its wall time in ms."""
    import torch

    t0 = time.perf_counter()
    entries = h.autotune(reps=3)
    torch.cuda.synchronize()
    ms_total = (time.perf_counter() - t0) * 1e3
    log(f"[gb300] {name} autotune {ms_total / 1e3:.2f}s")
    for e in entries:
        ms = " ".join(f"{t:.3f}" for t in e["ms"])
        log(f"[gb300]   level {e['level']} {e['op']:7s} {e['value_bytes']}B -> "
            f"config {e['config']} (fastest alone {e['fastest']}: {ms} ms)")
    return ms_total


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def red_black_colours(dims):
    i, j, k = np.meshgrid(*[np.arange(d, dtype=np.int32) for d in dims], indexing="ij")
    return ((i + j + k) % 2).ravel().astype(np.int32)


def parity_colours(dims):
    i, j, k = np.meshgrid(*[np.arange(d, dtype=np.int32) for d in dims], indexing="ij")
    return ((i % 2) * 4 + (j % 2) * 2 + (k % 2)).ravel().astype(np.int32)


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def make_problem(n_edge, seed_k=1, seed_b=0, sigma=1.5):
    dims = (n_edge, n_edge, n_edge)
    n = n_edge ** 3
    k = np.exp(sigma * np.random.default_rng(seed_k).standard_normal(n))
    b = np.random.default_rng(seed_b).uniform(-1.0, 1.0, n)
    return dims, k, b


# DRAM bytes per FP64 SpMV launch over algorithmic bytes, from the ncu capture
# of k_wrows<double, SpmvOp> on the 128^3 27-point matrix: (702.512 + 17.138)
# MB read + write / 719.247 MB algorithmic
NCU_SPMV_TRAFFIC_RATIO = (702.512128e6 + 17.137920e6) / 719247272.0


# FP64 FMA rate of GB300 (nominal 1.25 TFLOP/s; 1.2 measured with a
# dependent-chain-free FMA loop): the roof of the matrix-free stencils, whose
# 7 FMAs per cell outweigh their 25-48 bytes, and of the FP64 grid rows
FP64_PEAK_TFLOPS = 1.25

# One colour launch of the FP64 grid SOR sweep, k_g27_rows<double, double, 2,
# 27>, on the 160^3 27-point matrix (512,000 rows): ncu dram__bytes_read +
# write = 152.014 + 3.908 MB, FP64 pipe busy 74.1 % of the elapsed cycles,
# DRAM throughput 31.0 % of peak
NCU_G27_SOR64_DRAM_PER_ROW = (152.014336e6 + 3.908096e6) / 512000
NCU_G27_SOR64_FP64_BUSY = 0.741
NCU_G27_SOR64_DRAM_FRAC = 0.310


def csr_bytes(n, nnz, val_bytes=8, vec_bytes=8):
    # values + int32 columns + int64 row offsets + x once + y once
    return nnz * (val_bytes + 4) + 8 * (n + 1) + vec_bytes * n + vec_bytes * n


# ---------------------------------------------------------------------------
# CPU restatement (reference arm, cpu_baseline, parity at the bench size)
# ---------------------------------------------------------------------------
# iterations of a reference warm-up step (a slice of the solve)
REF_SAMPLE_ITERS = 9


def workload_config(args, n, nnz, world):
    """The `config` of both arms' JSON lines (identical by construction)."""
    return {"workload": f"{args.grid}^3 27-point lognormal(sigma=1.5) CSR, AMG-PCG to 1e-8",
            "rows": n, "nnz": nnz, "parallelism": f"replicas x{world}",
            "l2": (f"inputs ({(12 * nnz + 24 * n) / 1e9:.2f} GB: matrix and vectors) "
                   + ("larger than the 129 MB L2; no flush" if 12 * nnz + 24 * n > 129e6 else
                      "fit in the 129 MB L2: a small case, not a bench configuration"))}


def lineal_amg_params(threads):
    """lineal's shared-memory AMG on `threads` threads: aggregation partitions
    clamp(n / 8, 1, threads) on every level (aggregation/independent.hpp:
    183-186 with min_per_thread = 8, test/aux/default.hpp:184-186) and the
    thread-hybrid SOR with one row range per thread (gauss-seidel-variant/
    sweep.hpp:135-169)."""
    return dict(min_coarsen_size=2000, partition_size=8, partition_growth=1.0, min_partitions=1,
                max_partitions=threads, smoother_parts=threads)


def gpu_amg_params(args):
    """The oracle with the GPU hierarchy's parameters: the same aggregation
    partitions per level and colour-ordered SOR (Jones-Plassmann colourings
    with the same seeds, or smallest-last on the coarse levels)."""
    return dict(min_coarsen_size=2000, partition_size=args.partition_size,
                partition_growth=args.partition_growth, min_partitions=args.min_partitions,
                smoother_parts=0, coarse_smallest_last=int(args.coarse_smallest_last))


def oracle_problem(grid):
    import oracle as lo

    dims, k, b = make_problem(grid)
    t0 = time.perf_counter()
    a = lo.gen_27pt(dims, k)
    return dims, a, b, time.perf_counter() - t0


def oracle_pcg(a, b, amg, rtol=1e-8, maxit=500):
    """Oracle AMG-PCG from x0 = 0; returns (x, iterations, seconds)."""
    import oracle as lo

    t0 = time.perf_counter()
    x, it, _ = lo.pcg(a, b, precon=lo.PRECON_AMG, amg=amg, rtol=rtol, maxit=maxit)
    return x, it, time.perf_counter() - t0


def oracle_legs(args, gpu_levels, gpu_iterations):
    """The GPU line's CPU legs at the bench size, on all host threads:
    (1) parity: the oracle with the GPU's partitions and colourings (finest
    level: the grid parity colouring) builds its hierarchy and solves to
    1e-8 -- level sizes and iteration count beside the GPU's; (2)
    cpu_baseline: one full solve with lineal's own partitions and hybrid SOR,
    timed around the solve only (setup reported separately)."""
    import oracle as lo

    lo.build()
    threads = os.cpu_count() or 1
    lo.set_threads(threads)
    dims, a, b, gen_s = oracle_problem(args.grid)
    bn = float(np.linalg.norm(b))
    t0 = time.perf_counter()
    oh = lo.Amg(a, finest_colours=parity_colours(dims), ncolours=8, **gpu_amg_params(args))
    setup_s = time.perf_counter() - t0
    levels = [oh.level_size(l) for l in range(oh.nlevels)]
    x, it, solve_s = oracle_pcg(a, b, oh)
    rel = float(np.linalg.norm(b - lo.spmv(a, x))) / bn
    oh.close()
    del oh, x
    parity = {"oracle_iterations": it, "gpu_iterations": gpu_iterations,
              "iterations_within_5pct": abs(it - gpu_iterations) <= max(1, 0.05 * it),
              "oracle_levels": levels, "gpu_levels": list(gpu_levels),
              "levels_equal": levels == list(gpu_levels), "oracle_rel_residual": rel,
              "oracle_setup_s": setup_s, "oracle_solve_s": solve_s, "threads": threads,
              "what": "oracle AMG-PCG with the GPU hierarchy's partitions and colourings "
                      "(colour-ordered SOR), same system"}
    log(f"[parity] oracle {it} it vs GPU {gpu_iterations}; levels {levels} "
        f"{'==' if parity['levels_equal'] else '!='} GPU {list(gpu_levels)}; "
        f"setup {setup_s:.1f}s solve {solve_s:.1f}s")
    t0 = time.perf_counter()
    amg = lo.Amg(a, **lineal_amg_params(threads))
    rsetup = time.perf_counter() - t0
    x, rit, rsolve = oracle_pcg(a, b, amg)
    rrel = float(np.linalg.norm(b - lo.spmv(a, x))) / bn
    amg.close()
    cpu = {"value": rsolve * 1e3, "unit": "ms", "cores": threads, "kind": "port",
           "sample": f"one full {args.grid}^3 oracle AMG-PCG solve to 1e-8 ({rit} iterations, "
                     f"rel. residual {rrel:.2e}) with lineal's partitions clamp(n/8, 1, "
                     f"{threads}) and {threads}-part hybrid SOR, {threads} threads, solve only "
                     f"(setup {rsetup:.1f}s, generation {gen_s:.1f}s excluded)",
           "iterations": rit, "setup_ms": rsetup * 1e3,
           "single_core": {"omitted": "a one-core 256^3 solve takes several minutes, beyond "
                                      "the bench's time budget"}}
    log(f"[gb300] cpu baseline {rsolve * 1e3:.0f} ms ({threads} threads, {rit} it, "
        f"setup {rsetup:.1f}s)")
    return parity, cpu


def run_reference(args):
    """lineal's shared-memory AMG-PCG (the oracle, restated in C) on all host
    threads on the bench workload itself: the --grid^3 system and its
    hierarchy (lineal's partition rule, hybrid SOR) are built once outside
    the timed region; each timed step is one full solve to 1e-8 from x0 = 0
    (the oracle's own iteration count), timed around the solve only.  Warm-up
    steps run REF_SAMPLE_ITERS iterations of the same solve (they touch every
    array a full solve touches)."""
    rank, world, _ = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        if rank != 0:
            dist.barrier()
            dist.destroy_process_group()
            return
    import oracle as lo

    lo.build()
    threads = os.cpu_count() or 1
    lo.set_threads(threads)
    dims, a, b, gen_s = oracle_problem(args.grid)
    t0 = time.perf_counter()
    amg = lo.Amg(a, **lineal_amg_params(threads))
    setup_s = time.perf_counter() - t0
    levels = [amg.level_size(l) for l in range(amg.nlevels)]
    log(f"[reference] {args.grid}^3: generation {gen_s:.1f}s setup {setup_s:.1f}s, levels "
        f"{levels}")
    for _ in range(args.warmup):
        oracle_pcg(a, b, amg, rtol=0.0, maxit=REF_SAMPLE_ITERS)
    step_ms, iters = [], []
    for _ in range(args.steps):
        x, it, dt = oracle_pcg(a, b, amg)
        step_ms.append(dt * 1e3)
        iters.append(it)
        log(f"[reference] solve {dt:.2f}s, {it} it")
    rel = float(np.linalg.norm(b - lo.spmv(a, x))) / float(np.linalg.norm(b))
    value = float(np.mean(step_ms))
    sample = (f"the {args.grid}^3 system itself: oracle AMG-PCG to 1e-8 ({iters[-1]} iterations) "
              f"with lineal's partitions clamp(n/8, 1, {threads}) and {threads}-part hybrid SOR, "
              f"{threads} threads, each step one full solve from x0 = 0, solve only (setup "
              f"{setup_s:.1f}s, generation {gen_s:.1f}s excluded)")
    out = {
        "metric": METRIC, "value": value, "unit": "ms", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": value, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "impl": "reference",
        "config": workload_config(args, a.n, a.nnz, world),
        "oracle_iterations": iters[-1], "final_rel_residual": rel, "setup_ms": setup_s * 1e3,
        "levels": levels, "warmup_iterations_per_step": REF_SAMPLE_ITERS,
        "cpu_baseline": {"value": value, "unit": "ms", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


# ---------------------------------------------------------------------------
# GB300 arm
# ---------------------------------------------------------------------------
def precision_form(g, args, stream):
    """The precision form on its own workload: 7-point lognormal(sigma=3)
    diffusion (seed 2) at --grid^3 solved to 1e-10 by the plain FP64 AMG-PCG
    and by flexible CG over the float V-cycle; residuals verified in FP64."""
    import torch

    dims, k, b_host = make_problem(args.grid, seed_k=2, seed_b=0, sigma=3.0)
    a = g.gen_7pt(dims, k)
    col = g.Colouring.from_array(a, red_black_colours(dims), 2)
    b = torch.as_tensor(b_host, device="cuda")
    bn = float(torch.linalg.norm(b).item())
    hier_kw = dict(min_coarsen_size=2000, partition_size=args.partition_size,
                   partition_growth=args.partition_growth, min_partitions=args.min_partitions,
                   grid27=args.grid27, coarse_smallest_last=args.coarse_smallest_last)
    out = {"workload": f"{args.grid}^3 7-point lognormal(sigma=3, seed 2), AMG-PCG to 1e-10",
           "rows": a.row_num(), "nnz": a.non_zero_num(),
           "finest_kernels": "7-point grid rows, red-black order" if args.grid27 else "CSR"}
    xs = {}
    for tag, f32, bf16, flexible, refine in (("fp64", False, False, False, False),
                                             ("mixed_fcg", True, False, True, False),
                                             ("mixed_refined", True, False, True,
                                              args.refine),
                                             ("mixed_bf16_fcg", True, True, True, False)):
        t0 = time.perf_counter()
        h = g.HierarchyWright(cycle_f32=f32, cycle_bf16=bf16, **hier_kw).instantiate(
            a, finest_colouring=col)
        torch.cuda.synchronize()
        setup = time.perf_counter() - t0
        if args.autotune:
            h.autotune(reps=3)
        for _ in range(args.warmup):
            res = g.pcg(a, b, precon=g.PRECON_AMG, amg=h, rtol=1e-10, maxit=1000,
                        flexible=flexible, refine=refine,
                        inner_rtol=args.precision_inner_rtol)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            res = g.pcg(a, b, precon=g.PRECON_AMG, amg=h, rtol=1e-10, maxit=1000,
                        flexible=flexible, refine=refine,
                        inner_rtol=args.precision_inner_rtol)
        e1.record(stream)
        e1.synchronize()
        _, rn = g.residual(a, b, res.x)
        xs[tag] = res.x
        out[tag] = {"ms": e0.elapsed_time(e1) / args.steps, "iterations": res.iterations,
                    "rel_residual_fp64": float(np.sqrt(rn)) / bn, "setup_ms": setup * 1e3,
                    "levels": h.sizes()[0]}
        log(f"[precision] {tag}: {out[tag]['ms']:.1f} ms, {res.iterations} it, "
            f"rel {out[tag]['rel_residual_fp64']:.2e}")
        del h
    out["mixed_refined"]["what"] = (
        f"float-vector CG (refine {args.refine}, flexible beta) with FP64 residual "
        f"replacement every {args.precision_inner_rtol:g} reduction; float products and "
        "V-cycle, compensated dots and FP64 CG scalars")
    out["mixed_fcg"]["what"] = "flexible CG with FP64 vectors over the float V-cycle"
    for tag in ("mixed_fcg", "mixed_refined", "mixed_bf16_fcg"):
        out[tag]["rel_error_vs_fp64_solution"] = float(
            torch.linalg.norm(xs[tag] - xs["fp64"]).item() / torch.linalg.norm(xs["fp64"]).item())
        out[tag]["speedup_vs_fp64"] = out["fp64"]["ms"] / out[tag]["ms"]
    out["speedup_vs_fp64"] = out["fp64"]["ms"] / min(out["mixed_fcg"]["ms"],
                                                     out["mixed_refined"]["ms"])
    return out

def run_gb300(args):
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import lineal_gb300 as g

    g.build.build()
    stream = torch.cuda.current_stream()
    peak, peak_kind = measured_peaks()

    dims, k, b_host = make_problem(args.grid)
    n = int(np.prod(dims))
    t0 = time.perf_counter()
    a = g.gen_27pt(dims, k)
    nnz = a.non_zero_num()
    colours = parity_colours(dims)
    col = g.Colouring.from_array(a, colours, 8)
    torch.cuda.synchronize()
    log(f"[gb300] generated {dims} nnz={nnz} in {time.perf_counter() - t0:.2f}s")

    hier_kw = dict(min_coarsen_size=2000, partition_size=args.partition_size,
                   partition_growth=args.partition_growth, min_partitions=args.min_partitions,
                   grid27=args.grid27, coarse_smallest_last=args.coarse_smallest_last)
    wright = g.HierarchyWright(**hier_kw)
    t0 = time.perf_counter()
    h64 = wright.instantiate(a, finest_colouring=col)
    torch.cuda.synchronize()
    setup64 = time.perf_counter() - t0
    rows, nnzs = h64.sizes()
    grid_on = h64.grid27_active()
    log(f"[gb300] FP64 hierarchy {rows} in {setup64:.2f}s"
        f"{' (finest level: 27-point grid kernels)' if grid_on else ''}")
    tune64 = autotune_log("FP64", h64) if args.autotune else None

    b = torch.as_tensor(b_host, device="cuda")

    def solve(h):
        return g.pcg(a, b, precon=g.PRECON_AMG, amg=h, rtol=1e-8, maxit=500)

    # ---- plain FP64: warm-up then K timed solves --------------------------
    # (library launch counts mark the solves in profiler launch lists)
    log(f"[gb300] launches before the FP64 solves: {g.kernel_launches()}")
    for _ in range(args.warmup):
        res = solve(h64)
    iters64 = res.iterations
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    launches0 = g.kernel_launches()
    e0.record(stream)
    for _ in range(args.steps):
        res = solve(h64)
    e1.record(stream)
    e1.synchronize()
    launches = g.kernel_launches() - launches0
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms64 = e0.elapsed_time(e1) / args.steps
    if world > 1:
        t = torch.tensor([ms64], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms64 = float(t.item())
    x = res.x
    r, rn = g.residual(a, b, x)
    rel64 = float(np.sqrt(rn)) / float(torch.linalg.norm(b).item())
    log(f"[gb300] FP64 AMG-PCG {ms64:.1f} ms, {res.iterations} it, rel {rel64:.2e}")

    # ---- mixed precision: float cycle under the FP64 CG ---------------------
    wright32 = g.HierarchyWright(cycle_f32=True, **hier_kw)
    t0 = time.perf_counter()
    h32 = wright32.instantiate(a, finest_colouring=col)
    torch.cuda.synchronize()
    setup32 = time.perf_counter() - t0
    tune32 = autotune_log("mixed", h32) if args.autotune else None
    log(f"[gb300] launches before the mixed solves: {g.kernel_launches()}")
    for _ in range(args.warmup):
        res32 = solve(h32)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        res32 = solve(h32)
    e1.record(stream)
    e1.synchronize()
    ms32 = e0.elapsed_time(e1) / args.steps
    _, rn32 = g.residual(a, b, res32.x)
    rel32 = float(np.sqrt(rn32)) / float(torch.linalg.norm(b).item())
    err = float(torch.linalg.norm(res32.x - x).item() / torch.linalg.norm(x).item())
    log(f"[gb300] mixed AMG-PCG {ms32:.1f} ms, {res32.iterations} it, rel {rel32:.2e}")

    # ---- mixed, FP64 iterative refinement over a float inner PCG (same float
    # hierarchy): float products and V-cycles, compensated dots, FP64 scalars, outer
    # residual and stopping test
    def solve_refined(h):
        return g.pcg(a, b, precon=g.PRECON_AMG, amg=h, rtol=1e-8, maxit=500, refine=args.refine,
                     inner_rtol=args.inner_rtol, flexible=args.refine_flexible)

    for _ in range(args.warmup):
        resr = solve_refined(h32)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        resr = solve_refined(h32)
    e1.record(stream)
    e1.synchronize()
    msr = e0.elapsed_time(e1) / args.steps
    _, rnr = g.residual(a, b, resr.x)
    relr = float(np.sqrt(rnr)) / float(torch.linalg.norm(b).item())
    errr = float(torch.linalg.norm(resr.x - x).item() / torch.linalg.norm(x).item())
    log(f"[gb300] mixed refined AMG-PCG {msr:.1f} ms, {resr.iterations} it, rel {relr:.2e}")

    # ---- mixed with bfloat16 level values (precision form option) ----------
    h16 = g.HierarchyWright(cycle_f32=True, cycle_bf16=True, **hier_kw).instantiate(
        a, finest_colouring=col)
    tune16 = autotune_log("bf16", h16) if args.autotune else None
    for _ in range(args.warmup):
        res16 = solve(h16)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        res16 = solve(h16)
    e1.record(stream)
    e1.synchronize()
    ms16 = e0.elapsed_time(e1) / args.steps
    _, rn16 = g.residual(a, b, res16.x)
    rel16 = float(np.sqrt(rn16)) / float(torch.linalg.norm(b).item())
    err16 = float(torch.linalg.norm(res16.x - x).item() / torch.linalg.norm(x).item())
    log(f"[gb300] mixed bf16 AMG-PCG {ms16:.1f} ms, {res16.iterations} it, rel {rel16:.2e}")
    del h16

    # ---- SpMV bandwidth (FP64 values, and float values) ---------------------
    xs = torch.randn(n, dtype=torch.float64, device="cuda")
    ys = torch.empty_like(xs)
    spmv_reps = 20

    def time_spmv(m, x_, y_, fn):
        for _ in range(3):
            fn(m, x_, y_)
        torch.cuda.synchronize()
        s0 = torch.cuda.Event(enable_timing=True)
        s1 = torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        for _ in range(spmv_reps):
            fn(m, x_, y_)
        s1.record(stream)
        s1.synchronize()
        return s0.elapsed_time(s1) / spmv_reps

    t_spmv64 = time_spmv(a, xs, ys, lambda m, x_, y_: g.spmv(m, x_, out=y_))
    bytes64 = csr_bytes(n, nnz, 8, 8)
    gbs64 = bytes64 / (t_spmv64 * 1e-3) / 1e9
    del h64
    a32 = g.gen_27pt(dims, k, storage=g.F32)
    xs32 = xs.float()
    ys32 = torch.empty_like(xs32)
    t_spmv32 = time_spmv(a32, xs32, ys32, lambda m, x_, y_: g.spmv_f32(m, x_, out=y_))
    bytes32 = csr_bytes(n, nnz, 4, 4)
    gbs32 = bytes32 / (t_spmv32 * 1e-3) / 1e9
    del a32
    log(f"[gb300] SpMV fp64 {t_spmv64:.3f} ms {gbs64:.0f} GB/s; fp32 {t_spmv32:.3f} ms "
        f"{gbs32:.0f} GB/s")

    # ---- the finest-level smoother: one multicolour SOR sweep (8 colour
    # launches) through the grid kernels, in the colouring's row order;
    # algorithmic bytes = stored values + b, x read once, x written
    smoother = None
    colg = g.Colouring.from_array(a, colours, 8)
    if colg.use_grid27(dims, with_float=True):
        bp = g.permute(colg, b)
        xg = g.permute(colg, xs)
        xg32, bp32 = xg.float(), bp.float()
        t_sw64 = time_spmv(colg, xg, bp, lambda c_, x_, b_: g.sor_sweep_permuted(c_, b_, x_))
        t_sw32 = time_spmv(colg, xg32, bp32,
                           lambda c_, x_, b_: g.sor_sweep_permuted(c_, b_, x_))
        sb64, sb32 = nnz * 8 + 24 * n, nnz * 4 + 12 * n
        smoother = {"kernel": "k_g27_rows<VT, XT, 2> (8 colour launches)",
                    "fp64_ms": t_sw64, "fp64_gbs": sb64 / (t_sw64 * 1e-3) / 1e9,
                    "fp64_fma_tflops": 2 * nnz / (t_sw64 * 1e-3) / 1e12,
                    "fp32_ms": t_sw32, "fp32_gbs": sb32 / (t_sw32 * 1e-3) / 1e9,
                    "fp32_frac": sb32 / (t_sw32 * 1e-3) / 1e9 / peak,
                    "bytes_fp64": sb64, "bytes_fp32": sb32}
        log(f"[gb300] SOR sweep (grid) fp64 {t_sw64:.3f} ms; fp32 {t_sw32:.3f} ms "
            f"{smoother['fp32_gbs']:.0f} GB/s ({smoother['fp32_frac']:.0%} of peak)")
        del colg, bp, xg, xg32, bp32

    # ---- roofline of the dominant kernel of the timed FP64 solve: the finest
    # SOR colour launch k_g27_rows<double, double, 2, 27> (8 per sweep, 16 per
    # V-cycle); achieved = algorithmic bytes per launch / average launch time
    # (CUDA events over whole sweeps on the launching stream)
    if smoother:
        launch_ms = smoother["fp64_ms"] / 8
        launch_bytes = smoother["bytes_fp64"] / 8
        achieved = launch_bytes / (launch_ms * 1e-3) / 1e9
        fma_tf = 2 * nnz / (smoother["fp64_ms"] * 1e-3) / 1e12
        roofline = {
            "bound": "hbm", "kernel": "k_g27_rows<double, double, 2, 27> (finest-level SOR "
                                      "colour, 8 launches per sweep)",
            "achieved": achieved, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
            "frac": achieved / peak, "launch_ms": launch_ms, "bytes_per_launch": launch_bytes,
            "traffic": (n / 8) * NCU_G27_SOR64_DRAM_PER_ROW,
            "traffic_source": "ncu dram__bytes_read+write of one colour launch of the 160^3 "
                              "27-point matrix (512,000 rows), per row, times the rows of a "
                              "256^3 colour launch; above the algorithmic bytes by the x of "
                              "the other seven colours that every colour launch gathers",
            "fp64_pipe": {"fma_tflops": fma_tf, "peak_tflops": FP64_PEAK_TFLOPS,
                          "peak_kind": "nominal", "frac": fma_tf / FP64_PEAK_TFLOPS,
                          "ncu_busy_160cube": NCU_G27_SOR64_FP64_BUSY},
            "binding_roof": "FP64 pipe: at 160^3 ncu shows it busy for "
                            f"{NCU_G27_SOR64_FP64_BUSY:.0%} of the launch while DRAM "
                            f"throughput is {NCU_G27_SOR64_DRAM_FRAC:.0%} of peak"}
    else:
        roofline = {"bound": "hbm", "kernel": "k_wrows<double, SpmvOp<double,double>, 4, 1>",
                    "achieved": gbs64, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                    "frac": gbs64 / peak, "traffic": bytes64 * NCU_SPMV_TRAFFIC_RATIO,
                    "traffic_source": "ncu dram__bytes_read+write of one launch at 128^3, "
                                      "scaled to this matrix by its algorithmic bytes"}

    # ---- end to end through the C ABI with host buffers -----------------------
    e2e = None
    if args.e2e:
        rowptr, colidx, val = a.download()
        h_rowptr = torch.from_numpy(rowptr).pin_memory()
        h_col = torch.from_numpy(colidx).pin_memory()
        h_val = torch.from_numpy(val).pin_memory()
        h_b = torch.from_numpy(b_host).pin_memory()
        h_col_colours = torch.from_numpy(colours).pin_memory()
        del h32
        e2e_ms = []
        # a one-shot solve: Jones-Plassmann coarse colourings (device-side,
        # fast setup) whatever the resident solves use
        e2e_kw = dict(hier_kw, coarse_smallest_last=False)
        phases = []
        for step in range(args.e2e_steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            d_rowptr = h_rowptr.to("cuda", non_blocking=True)
            d_col = h_col.to("cuda", non_blocking=True)
            d_val = h_val.to("cuda", non_blocking=True)
            d_b = h_b.to("cuda", non_blocking=True)
            d_colours = h_col_colours.to("cuda", non_blocking=True)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            m = g.CsrMatrix.from_device(d_rowptr, d_col, d_val, symmetric=True)
            if args.grid27:
                m.set_grid27(dims)  # the caller knows its operator is the 27-point grid
            del d_rowptr, d_col, d_val
            c = g.Colouring.from_array(m, d_colours, 8)
            torch.cuda.synchronize()
            t2 = time.perf_counter()
            hh = g.HierarchyWright(cycle_f32=True, **e2e_kw).instantiate(
                m, finest_colouring=c)
            torch.cuda.synchronize()
            t3 = time.perf_counter()
            rr = g.pcg(m, d_b, precon=g.PRECON_AMG, amg=hh, rtol=1e-8, maxit=500,
                       refine=args.refine if args.e2e_refine else 0,
                       inner_rtol=args.inner_rtol)
            torch.cuda.synchronize()
            t4 = time.perf_counter()
            xh = rr.x.cpu()
            torch.cuda.synchronize()
            t5 = time.perf_counter()
            e2e_ms.append((t5 - t0) * 1e3)
            phases.append({"h2d": (t1 - t0) * 1e3, "matrix_and_colouring": (t2 - t1) * 1e3,
                           "hierarchy": (t3 - t2) * 1e3, "solve": (t4 - t3) * 1e3,
                           "d2h": (t5 - t4) * 1e3, "iterations": rr.iterations})
            del m, c, hh, rr
        h2d = (rowptr.nbytes + colidx.nbytes + val.nbytes + b_host.nbytes + colours.nbytes)
        e2e = {"value": float(np.median(e2e_ms)), "unit": "ms", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(n * 8), "phases_ms": phases[len(phases) // 2],
               "what": "host CSR + b (pinned) -> device, AMG setup (float cycle, "
                       "Jones-Plassmann coarse colourings), "
                       + ("float-vector CG with FP64 residual (refine "
                          f"{args.refine})" if args.e2e_refine else "CG") + ", x -> host"}
        log(f"[gb300] e2e {e2e['value']:.0f} ms {e2e['phases_ms']}")

    # ---- CPU baseline (bounded sample) -----------------------------------------
    prec = precision_form(g, args, stream) if args.precision_form else None

    # ---- the other named configurations, each with its own check -------------
    configs = {}
    if args.configs:
        a = h32 = b = None  # the 256^3 system is done with: free its device memory
        torch.cuda.empty_cache()
        sw = (max(3, args.warmup // 2), stream)
        configs["config1_jacobi_pcg_64"] = config1_entry(g, min(args.steps, 10), *sw)
        configs["batch_1024"] = batch_entry(g, min(args.steps, 5), *sw)
        configs["multi_rhs_32"] = multi_entry(g, min(args.steps, 3), *sw,
                                              partition_size=args.partition_size)
        configs["adjoint_128"] = adjoint_entry(g, 128, args.bench_fd_directions)

    cpu = parity = None
    if rank == 0 and args.cpu_baseline:
        parity, cpu = oracle_legs(args, rows, iters64)

    out = {
        "metric": METRIC, "value": ms64, "unit": "ms", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms64, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args, n, nnz, world),
        "amg": {"levels": rows, "level_nnz": nnzs, "partition_size": args.partition_size,
                "partition_growth": args.partition_growth,
                "min_partitions": args.min_partitions,
                "finest_colouring": "grid parity, 8 colours",
                "coarse_colouring": ("smallest-last (host)" if args.coarse_smallest_last
                                     else "Jones-Plassmann"),
                "finest_kernels": ("27-point grid rows, column indices computed "
                                   "(lgx_amg_params.grid27)" if grid_on else "CSR row engine"),
                "row_engine": ("autotuned per level (lgx_amg_autotune, setup-time, outside "
                               "the timed solves; e2e untuned)"
                               if args.autotune else "process-wide configuration 3")},
        "oracle_iterations": parity["oracle_iterations"] if parity else None,
        "oracle_parity": parity,
        "iterations": iters64, "final_rel_residual": rel64, "setup_ms": setup64 * 1e3,
        "autotune_ms": tune64,
        "mixed": {"ms": ms32, "iterations": res32.iterations, "rel_residual_fp64": rel32,
                  "setup_ms": setup32 * 1e3, "autotune_ms": tune32,
                  "speedup_vs_fp64": ms64 / ms32, "rel_error_vs_fp64_solution": err},
        "mixed_refined": {"ms": msr, "iterations": resr.iterations, "rel_residual_fp64": relr,
                          "speedup_vs_fp64": ms64 / msr, "rel_error_vs_fp64_solution": errr,
                          "what": ("float-vector CG with reliable updates (FP64 solution "
                                   "and residual replaced every " if args.refine == 2 else
                                   "FP64 iterative refinement over a float-vector inner PCG, "
                                   "inner tolerance ") + f"{args.inner_rtol:g}" +
                                  (" reduction" if args.refine == 2 else "") +
                                  "; float finest products and V-cycle, compensated dots and FP64 CG "
                                  "scalars", "refine": args.refine},
        "mixed_speedup_vs_fp64": ms64 / min(ms32, msr),
        "mixed_bf16": {"ms": ms16, "iterations": res16.iterations, "rel_residual_fp64": rel16,
                       "autotune_ms": tune16, "speedup_vs_fp64": ms64 / ms16,
                       "rel_error_vs_fp64_solution": err16,
                       "what": "float cycle with bfloat16 level values (diagonal row scales)"},
        "spmv": {"fp64_ms": t_spmv64, "fp64_gbs": gbs64, "fp64_frac": gbs64 / peak,
                 "fp32_ms": t_spmv32, "fp32_gbs": gbs32, "fp32_frac": gbs32 / peak,
                 "bytes_fp64": bytes64, "bytes_fp32": bytes32},
        "smoother": smoother,
        "precision_form": prec,
        "roofline": roofline,
        **configs,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


def run_kernels(args):
    """Times the row kernels alone on the --grid matrix (also the ncu target):
    FP64 SpMV, one multicolour SOR sweep, the residual and the FP32 SpMV; with
    --vcycle also one V-cycle of the FP64 and of the mixed hierarchy."""
    import torch

    import lineal_gb300 as g

    g.build.build()
    stream = torch.cuda.current_stream()
    dims, k, b_host = make_problem(args.grid)
    n = int(np.prod(dims))
    a = g.gen_27pt(dims, k)
    nnz = a.non_zero_num()
    col = g.Colouring.from_array(a, parity_colours(dims), 8)
    x = torch.randn(n, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    b = torch.as_tensor(b_host, device="cuda")
    a32 = g.gen_27pt(dims, k, storage=g.F32)
    x32 = x.float()
    y32 = torch.empty_like(x32)
    kernels = [
        ("spmv_fp64", lambda: g.spmv(a, x, out=y), csr_bytes(n, nnz, 8, 8)),
        ("sor_sweep_fp64", lambda: g.sor_sweep(a, col, b, x, out=y),
         csr_bytes(n, nnz, 8, 8) + 8 * n),
        ("residual_fp64", lambda: g.residual(a, b, x, with_norm=False),
         csr_bytes(n, nnz, 8, 8) + 8 * n),
        ("spmv_fp32", lambda: g.spmv_f32(a32, x32, out=y32), csr_bytes(n, nnz, 4, 4)),
    ]
    # sweeps in the colouring's row order (no permutation traffic)
    bp = g.permute(col, b)
    xp = g.permute(col, x)
    bp32, xp32 = bp.float(), xp.float()
    kernels += [
        ("sor_sweep_permuted_fp64", lambda: g.sor_sweep_permuted(col, bp, xp),
         csr_bytes(n, nnz, 8, 8) + 8 * n),
        ("sor_sweep_permuted_fp32", lambda: g.sor_sweep_permuted(col, bp32, xp32),
         csr_bytes(n, nnz, 4, 4) + 4 * n),
    ]
    # the same sweeps through the 27-point grid kernels (no column indices):
    # algorithmic bytes = stored values + b, x read once and x written
    colg = g.Colouring.from_array(a, parity_colours(dims), 8)
    if colg.use_grid27(dims, with_float=True):
        xg, xg32 = xp.clone(), xp32.clone()
        kernels += [
            ("sor_sweep_grid_fp64", lambda: g.sor_sweep_permuted(colg, bp, xg),
             nnz * 8 + 3 * 8 * n),
            ("sor_sweep_grid_fp32", lambda: g.sor_sweep_permuted(colg, bp32, xg32),
             nnz * 4 + 3 * 4 * n),
        ]
    if args.vcycle:
        hier = {}
        for tag, f32 in (("fp64", False), ("mixed", True)):
            hier[tag] = g.HierarchyWright(min_coarsen_size=2000, cycle_f32=f32,
                                          partition_size=args.partition_size,
                                          partition_growth=args.partition_growth,
                                          min_partitions=args.min_partitions).instantiate(
                                              a, finest_colouring=col)
        kernels.append(("vcycle_fp64", lambda: hier["fp64"].vcycle(b, out=y), 0))
        kernels.append(("vcycle_mixed", lambda: hier["mixed"].vcycle(b, out=y), 0))
    out = {}
    for name, fn, nbytes in kernels:
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        out[name] = {"ms": ms, "gbs": nbytes / (ms * 1e-3) / 1e9 if nbytes else None}
        log(f"[kernels] {name}: {ms:.3f} ms" +
            (f" {out[name]['gbs']:.0f} GB/s" if nbytes else ""))
    print(json.dumps({"grid": args.grid, "kernels": out}), flush=True)


def batch_systems(count=1024, seed=3):
    """1024 upwind convection-diffusion systems: cubic grids with edges uniform
    in 12..48, velocity components uniform in [-20, 20] (D = 1)."""
    rng = np.random.default_rng(seed)
    edges = rng.integers(12, 49, count)
    vs = rng.uniform(-20.0, 20.0, (count, 3))
    return [((int(e),) * 3, tuple(float(c) for c in v)) for e, v in zip(edges, vs)]




def run_stencil(args):
    """Matrix-free 7-point stencil products at --grid^3 with both stencil
    kernels (thread per cell; plane march with TMA-staged x planes): time,
    algorithmic GB/s and FP64 rate against their roofs."""
    import torch

    import lineal_gb300 as g

    g.build.build()
    stream = torch.cuda.current_stream()
    peak, peak_kind = measured_peaks()
    dims, k, b_host = make_problem(args.grid)
    n0, n1, n2 = dims
    n = int(np.prod(dims))
    # products per cell: diagonal + one per neighbour inside the grid
    fmas = n + 2 * ((n0 - 1) * n1 * n2 + n0 * (n1 - 1) * n2 + n0 * n1 * (n2 - 1))
    mat = np.random.default_rng(2).integers(0, 4, n).astype(np.uint8)
    st = {"lookup": g.StencilMatrix.lookup(dims, (1.0, 1.0, 1.0), (0.5, 1.0, 2.0, 4.0), mat),
          "value": g.StencilMatrix.value(dims, (1.0, 1.0, 1.0), k)}
    cell_bytes = {"lookup": 1 + 8 + 8 + 8, "value": 24 + 8 + 8 + 8}
    x = torch.randn(n, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    b = torch.as_tensor(b_host, device="cuda")
    r = torch.empty_like(x)
    out = {}
    for engine, etag in ((0, "cells"), (1, "planes")):
        g.stencil_engine(engine)
        for kind, m in st.items():
            for op in ("spmv", "residual"):
                if op == "spmv":
                    fn = lambda: g.spmv(m, x, out=y)  # noqa: E731
                    nbytes, flops = cell_bytes[kind] * n, 2 * fmas
                else:
                    fn = lambda: g.lib().lgx_residual(  # noqa: E731
                        m.handle, g._ptr(b), g._ptr(x), g._ptr(r), None, g._stream())
                    nbytes, flops = (cell_bytes[kind] + 8) * n, 2 * fmas + n
                for _ in range(args.warmup):
                    fn()
                torch.cuda.synchronize()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for _ in range(args.steps):
                    fn()
                e1.record(stream)
                e1.synchronize()
                ms = e0.elapsed_time(e1) / args.steps
                name = f"{kind}_{op}_{etag}"
                gbs = nbytes / (ms * 1e-3) / 1e9
                tf = flops / (ms * 1e-3) / 1e12
                out[name] = {"ms": ms, "gbs": gbs, "hbm_frac": gbs / peak, "fp64_tflops": tf,
                             "fp64_frac": tf / FP64_PEAK_TFLOPS}
                log(f"[stencil] {name}: {ms:.3f} ms {gbs:.0f} GB/s ({gbs / peak:.0%} of HBM) "
                    f"{tf:.2f} FP64 TFLOP/s ({tf / FP64_PEAK_TFLOPS:.0%} of nominal)")
    g.stencil_engine(0)
    # matrix-free red-black SOR sweeps (two colour launches, in situ):
    # algorithmic bytes per cell = valuator data + diagonal + b + x read and
    # written; 6 FMAs and one division per cell
    sweep_bytes = {"lookup": 1 + 8 + 8 + 8 + 8, "value": 24 + 8 + 8 + 8 + 8}
    for kind, m in st.items():
        col = g.Colouring.red_black(m)
        xs = x.clone()
        fn = lambda: g.sor_sweep(m, col, b, x_in=xs, out=xs)  # noqa: E731
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        gbs = sweep_bytes[kind] * n / (ms * 1e-3) / 1e9
        tf = 2 * (fmas - n) / (ms * 1e-3) / 1e12
        name = f"{kind}_sor_red_black"
        out[name] = {"ms": ms, "gbs": gbs, "hbm_frac": gbs / peak, "fp64_tflops": tf,
                     "fp64_frac": tf / FP64_PEAK_TFLOPS}
        log(f"[stencil] {name}: {ms:.3f} ms {gbs:.0f} GB/s ({gbs / peak:.0%} of HBM) "
            f"{tf:.2f} FP64 TFLOP/s of FMAs")
    print(json.dumps({"mode": "stencil", "grid": args.grid, "cells": n, "fp64_fmas": fmas,
                      "hbm_peak_gbs": peak, "hbm_peak_kind": peak_kind,
                      "fp64_peak_tflops": FP64_PEAK_TFLOPS, "fp64_peak_kind": "nominal",
                      "kernels": out}), flush=True)


def timed(fn, steps, warmup, stream):
    """Mean ms of `steps` calls of fn after `warmup` untimed ones (CUDA events
    on the launching stream); returns (ms, last result)."""
    import torch

    res = None
    for _ in range(warmup):
        res = fn()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        res = fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / steps, res


def config1_entry(g, steps, warmup, stream, edge=64):
    """Plain method, small: the 64^3 constant-coefficient Poisson system as a
    matrix-free lookup stencil (one material, unit cells, Dirichlet values 0
    on the axis-0 faces), b ~ U[-1, 1] (seed 0), x0 = 0, Jacobi-PCG to 1e-8,
    FP64; iterations and the FP64 residual checked against the oracle."""
    import oracle as lo

    dims = (edge,) * 3
    n = edge ** 3
    mat = np.ones(n, dtype=np.uint8)
    coeffs = (0.0, 1.0, 0.0, 0.0)
    b = np.random.default_rng(0).uniform(-1, 1, n)
    st = g.StencilMatrix.lookup(g.BoxInfo(dims, dims), None, coeffs, mat, 0.0, 0.0)
    bd = g._dvec(b)
    ms, res = timed(lambda: g.pcg(st, bd, precon=g.PRECON_JACOBI, rtol=1e-8, maxit=5000),
                    steps, warmup, stream)
    lo.build()
    ref, _ = lo.Stencil(dims, mat=mat, coeffs=coeffs, sol_start=0, sol_end=0).to_csr()
    _, it, _ = lo.pcg(ref, b, precon=lo.PRECON_JACOBI, rtol=1e-8, maxit=5000)
    x = res.x.cpu().numpy()
    rel = float(np.linalg.norm(b - lo.spmv(ref, x)) / np.linalg.norm(b))
    out = {"workload": f"{edge}^3 7-point Poisson, lookup stencil, Jacobi-PCG to 1e-8",
           "rows": n, "ms": ms, "iterations": res.iterations, "oracle_iterations": it,
           "iterations_within_5pct": abs(res.iterations - it) <= max(1, 0.05 * it),
           "rel_residual_fp64": rel,
           "note": "about 4.5 MB of operator and vectors: an L2-resident case, no HBM claim"}
    log(f"[config1] {ms:.2f} ms, {res.iterations} it (oracle {it}), rel {rel:.2e}")
    return out


def batch_entry(g, steps, warmup, stream, count=1024, cpu_sample=0, oracle_check=8):
    """Batching form: Jacobi-BiCGStab to 1e-8 on `count` uneven upwind
    convection-diffusion systems in one persistent launch (per step the
    whole batch, b resident); the first `oracle_check` systems' iterations
    and FP64 residuals checked against the oracle."""
    import torch

    import oracle as lo

    systems = batch_systems(count)
    rows = sum(int(np.prod(d)) for d, _ in systems)
    bh = np.random.default_rng(0).uniform(-1, 1, rows)
    b = torch.as_tensor(bh, device="cuda")
    ms, res = timed(lambda: g.batch_convdiff_bicgstab(systems, b, rtol=1e-8, maxit=2000),
                    steps, warmup, stream)
    row_iters = sum(int(np.prod(d)) * int(i) for (d, _), i in zip(systems, res.iterations))
    out = {"systems": len(systems), "rows": rows, "ms": ms,
           "systems_per_s": len(systems) / (ms * 1e-3),
           "iterations_mean": float(res.iterations.mean()),
           "iterations_max": int(res.iterations.max()),
           "converged": int((res.status == 0).sum()),
           "max_rel_residual": float(res.rel_residual.max()),
           "row_iterations_per_s": row_iters / (ms * 1e-3)}
    lo.build()
    x = res.x.cpu().numpy()
    off, worst_it, worst_rel = 0, 0.0, 0.0
    for k, (dims, v) in enumerate(systems):
        m = int(np.prod(dims))
        if k < oracle_check:
            a = lo.gen_convdiff(dims, v)
            _, it, _ = lo.pbicgstab(a, bh[off:off + m], precon=lo.PRECON_JACOBI, rtol=1e-8,
                                    maxit=2000)
            worst_it = max(worst_it, abs(int(res.iterations[k]) - it) / max(it, 1))
            r = bh[off:off + m] - lo.spmv(a, x[off:off + m])
            worst_rel = max(worst_rel, float(np.linalg.norm(r) / np.linalg.norm(bh[off:off + m])))
        off += m
    out["oracle_check"] = {"systems": oracle_check, "max_iteration_gap": worst_it,
                           "max_rel_residual_fp64": worst_rel}
    if cpu_sample:
        sample = systems[:cpu_sample]
        rng = np.random.default_rng(0)
        t0 = time.perf_counter()
        srows = 0
        for dims, v in sample:
            a = lo.gen_convdiff(dims, v)
            srows += a.n
            lo.pbicgstab(a, rng.uniform(-1, 1, a.n), precon=lo.PRECON_JACOBI, rtol=1e-8,
                         maxit=2000)
        cpu_s = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": cpu_s * rows / srows * 1e3, "unit": "ms",
                               "cores": os.cpu_count() or 1, "kind": "port",
                               "sample": f"oracle Jacobi-BiCGStab on the first {len(sample)} "
                                         f"systems ({srows} rows, assembly included), scaled "
                                         f"by rows to the batch"}
    log(f"[batch] {len(systems)} systems, {rows} rows: {ms:.1f} ms, "
        f"mean {out['iterations_mean']:.1f} it, converged {out['converged']}")
    return out


def run_batch(args):
    """Batching form: Jacobi-BiCGStab to 1e-8 on 1024 uneven convection-diffusion
    systems in one persistent launch (per step: the whole batch, b resident)."""
    import torch

    import lineal_gb300 as g

    g.build.build()
    out = batch_entry(g, args.steps, args.warmup, torch.cuda.current_stream(),
                      args.batch_systems, args.batch_cpu_sample if args.cpu_baseline else 0)
    out["mode"] = "batch"
    print(json.dumps(out), flush=True)


def run_profile(args):
    """Profiler target: one untimed AMG-PCG solve of the --grid^3 27-point
    workload (or the precision form's 7-point workload with
    --profile-precision) (FP64, or the float cycle with --mixed -- the float-vector CG with
    reliable updates with --profile-refined -- with bfloat16 level values with
    --bf16; the bench's hierarchy options; row engine autotuned unless
    --no-autotune), then one more inside the NVTX range "solve" (ncu --nvtx
    --nvtx-include solve/ selects its kernels)."""
    import torch

    import lineal_gb300 as g

    g.build.build()
    if args.profile_precision:
        # the precision form's workload: 7-point lognormal(sigma=3), red-black
        dims, k, b_host = make_problem(args.grid, seed_k=2, seed_b=0, sigma=3.0)
        a = g.gen_7pt(dims, k)
        col = g.Colouring.from_array(a, red_black_colours(dims), 2)
    else:
        dims, k, b_host = make_problem(args.grid)
        a = g.gen_27pt(dims, k)
        col = g.Colouring.from_array(a, parity_colours(dims), 8)
    rtol = 1e-10 if args.profile_precision else 1e-8
    mixed = args.mixed or args.bf16
    h = g.HierarchyWright(min_coarsen_size=2000, cycle_f32=mixed, cycle_bf16=args.bf16,
                          partition_size=args.partition_size,
                          partition_growth=args.partition_growth,
                          min_partitions=args.min_partitions, grid27=args.grid27,
                          coarse_smallest_last=args.coarse_smallest_last).instantiate(
        a, finest_colouring=col)
    if args.autotune:
        h.autotune(reps=3)
    b = torch.as_tensor(b_host, device="cuda")
    # --mixed --profile-refined: the float-vector CG with reliable updates
    # (with --profile-precision, as the precision form runs them: flexible CG
    # over the float cycle, the float-vector CG with its inner reduction)
    if args.profile_precision:
        kw = (dict(refine=args.refine, inner_rtol=args.precision_inner_rtol, flexible=True)
              if mixed and args.profile_refined else dict(flexible=mixed))
    else:
        kw = (dict(refine=args.refine, inner_rtol=args.inner_rtol,
                   flexible=args.refine_flexible) if mixed and args.profile_refined else {})
    res = g.pcg(a, b, precon=g.PRECON_AMG, amg=h, rtol=rtol, maxit=1000, **kw)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("solve")
    res = g.pcg(a, b, precon=g.PRECON_AMG, amg=h, rtol=rtol, maxit=1000, **kw)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    form = ("bf16" if args.bf16 else "mixed refined" if mixed and args.profile_refined
            else "mixed" if args.mixed else "fp64")
    log(f"[profile] {form} solve: {res.iterations} it")


def multi_entry(g, steps, warmup, stream, grid=128, partition_size=4096):
    """Batching form, second part: a grid^3 7-point Poisson CSR with 32
    right-hand sides uniform in [-1, 1], solved to 1e-8 by blocked AMG-PCG
    (FP64 outer iteration, float V-cycle), against 32 single-vector solves of
    the same hierarchy."""
    import torch

    dims = (grid,) * 3
    n = grid ** 3
    a = g.gen_7pt(dims, np.ones(n))
    col = g.Colouring.from_array(a, red_black_colours(dims), 2)
    h = g.HierarchyWright(min_coarsen_size=2000, cycle_f32=True,
                          partition_size=partition_size).instantiate(a, finest_colouring=col)
    B = torch.as_tensor(np.random.default_rng(0).uniform(-1, 1, (n, 32)), device="cuda")
    ms_block, (X, its, rels) = timed(lambda: g.pcg_multi(a, h, B, rtol=1e-8), steps, warmup,
                                     stream)
    cols = B.t().contiguous()

    def singles():
        return [g.pcg(a, cols[c], precon=g.PRECON_AMG, amg=h, rtol=1e-8, flexible=True)
                .iterations for c in range(32)]

    ms_single, single_its = timed(singles, 1, 2, stream)
    _, rn = g.residual(a, B[:, 0].contiguous(), X[:, 0].contiguous())
    out = {"workload": f"{grid}^3 7-point Poisson CSR, 32 RHS, AMG-PCG to 1e-8",
           "rows": n, "ms_blocked": ms_block, "ms_32_single_solves": ms_single,
           "speedup": ms_single / ms_block, "iterations_blocked_max": int(its.max()),
           "iterations_single_max": int(max(single_its)),
           "max_rel_residual": float(rels.max()),
           "col0_rel_residual_fp64": float(np.sqrt(rn)) /
                                     float(torch.linalg.norm(B[:, 0]).item())}
    log(f"[multi] blocked {ms_block:.1f} ms vs 32 single solves {ms_single:.1f} ms, "
        f"{int(its.max())} it")
    return out


def run_multi(args):
    """The 32-right-hand-side part of the batching form as its own line."""
    import torch

    import lineal_gb300 as g

    g.build.build()
    out = multi_entry(g, args.steps, args.warmup, torch.cuda.current_stream(), args.grid,
                      args.partition_size)
    out["mode"] = "multi"
    print(json.dumps(out), flush=True)


def adjoint_entry(g, grid, directions, warmup=1):
    """Differentiation form at grid^3 (workload 128^3): x = A(theta)^-1 b for
    the 7-point operator with k = exp(theta), theta ~ N(0, 1) (seed 4), b a
    Gaussian bump, x_target the solve at theta + 0.3 N(0, 1); loss
    0.5 ||x - x_target||^2.  Times the forward (mixed: flexible CG over the
    float V-cycle) and backward solves, checks the gradient against FP64
    central differences along `directions` random N(0, 1) directions
    (h = 1e-6; perturbed solutions from accurately formed right-hand sides
    and compensated defect correction) and against the all-FP64 gradient."""
    import torch

    from lineal_gb300.autograd import (SolveOptions, accurate_gradient, accurate_system,
                                       diffusion7_solve, loss_difference_fd)

    dims = (grid,) * 3
    n = grid ** 3
    rng = np.random.default_rng(4)
    theta0 = rng.standard_normal(n)
    theta_t = theta0 + 0.3 * rng.standard_normal(n)
    i, j, k = np.meshgrid(*[np.arange(d, dtype=np.float64) for d in dims], indexing="ij")
    c, s = (grid - 1) / 2, grid / 6.0
    b = torch.as_tensor(np.exp(-((i - c) ** 2 + (j - c) ** 2 + (k - c) ** 2) / (2 * s * s)).ravel(),
                        device="cuda")
    fp64 = SolveOptions(rtol=1e-11)
    mixed = SolveOptions(rtol=1e-10, mixed=True)
    _, _, x_t = accurate_system(torch.as_tensor(theta_t, device="cuda"), b, dims)

    def grad(opts):
        th = torch.as_tensor(theta0, device="cuda").requires_grad_(True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        x = diffusion7_solve(th, b, dims, opts)
        loss = 0.5 * torch.sum((x - x_t) ** 2)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        loss.backward()
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        return th.grad.detach(), float(loss), (t1 - t0) * 1e3, (t2 - t1) * 1e3

    for _ in range(warmup):
        grad(mixed)
    g_mixed, loss_m, fwd_ms, bwd_ms = grad(mixed)
    g_64, _, fwd64_ms, bwd64_ms = grad(fp64)
    rel_vs_fp64 = float(torch.linalg.norm(g_mixed - g_64) / torch.linalg.norm(g_64))
    th0 = torch.as_tensor(theta0, device="cuda")
    a0, h0, x0 = accurate_system(th0, b, dims)
    g_ref = accurate_gradient(th0, b, dims, x_t)
    drng = np.random.default_rng(6)
    h = 1e-6
    errs = {"mixed": [], "fp64": [], "refined": []}
    t0 = time.perf_counter()
    for _ in range(directions):
        vt = torch.as_tensor(drng.standard_normal(n), device="cuda")
        fd = loss_difference_fd(th0, vt, h, dims, x0, x_t, a0, h0)
        for tag, gg in (("mixed", g_mixed), ("fp64", g_64), ("refined", g_ref)):
            gv = float(torch.dot(gg, vt))
            errs[tag].append(abs(fd - gv) / abs(gv))
    fd_s = time.perf_counter() - t0
    fd_stats = {tag: {"max": float(np.max(e)), "median": float(np.median(e))}
                for tag, e in errs.items()}
    rel_ref = float(torch.linalg.norm(g_mixed - g_ref) / torch.linalg.norm(g_ref))
    out = {"workload": f"{grid}^3 7-point, k = exp(theta), theta ~ N(0,1)",
           "forward_ms": fwd_ms, "backward_ms": bwd_ms, "forward_fp64_ms": fwd64_ms,
           "backward_fp64_ms": bwd64_ms, "loss": loss_m,
           "grad_rel_error_vs_fp64": rel_vs_fp64, "grad_rel_error_vs_refined": rel_ref,
           "fd_directions": directions, "fd_step": h, "fd_max_rel_error": fd_stats["mixed"]["max"],
           "fd_rel_error_by_gradient": fd_stats, "fd_seconds": fd_s}
    log(f"[adjoint] fwd {fwd_ms:.1f} ms bwd {bwd_ms:.1f} ms; fd max rel "
        f"{fd_stats['mixed']['max']:.2e}; vs fp64 {rel_vs_fp64:.2e}")
    return out


def run_adjoint(args):
    """The differentiation form as its own line (all --fd-directions)."""
    import lineal_gb300 as g

    g.build.build()
    out = adjoint_entry(g, args.grid, args.fd_directions, args.warmup)
    out["mode"] = "adjoint"
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--mode", default="solve",
                    choices=["solve", "kernels", "stencil", "adjoint", "batch", "multi",
                             "profile"])
    ap.add_argument("--mixed", action="store_true", help="--mode profile: the float cycle")
    ap.add_argument("--profile-refined", action="store_true",
                    help="--mode profile --mixed: the float-vector CG (--refine)")
    ap.add_argument("--bf16", action="store_true",
                    help="--mode profile: the float cycle with bfloat16 level values")
    ap.add_argument("--profile-precision", action="store_true",
                    help="--mode profile: the precision form's 7-point sigma=3 workload "
                         "solved to 1e-10")
    ap.add_argument("--batch-systems", type=int, default=1024)
    ap.add_argument("--batch-cpu-sample", type=int, default=16)
    ap.add_argument("--fd-directions", type=int, default=64)
    ap.add_argument("--grid", type=int, default=None,
                    help="grid edge (default 256; 128 for --mode adjoint and --mode multi)")
    ap.add_argument("--partition-size", type=int, default=4096)
    ap.add_argument("--partition-growth", type=float, default=4.0)
    ap.add_argument("--min-partitions", type=int, default=8)
    ap.add_argument("--no-grid27", dest="grid27", action="store_false",
                    help="finest level on the CSR row engine even for the 27-point grid")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="skip the row-engine autotuner of the solve-mode hierarchies "
                         "(setup-time: every level's shapes timed before the timed solves)")
    ap.add_argument("--vcycle", action="store_true",
                    help="--mode kernels: also time one FP64 and one mixed V-cycle")
    ap.add_argument("--no-precision-form", dest="precision_form", action="store_false",
                    help="skip the 7-point sigma=3 precision-form solves")
    ap.add_argument("--no-e2e", dest="e2e", action="store_false")
    ap.add_argument("--e2e-steps", type=int, default=1)
    ap.add_argument("--no-e2e-refine", dest="e2e_refine", action="store_false",
                    help="e2e: plain CG over the float cycle instead of --refine")
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--refine", type=int, default=2, choices=[1, 2],
                    help="mixed_refined: 1 iterative refinement, 2 reliable updates")
    ap.add_argument("--refine-flexible", action="store_true",
                    help="mixed_refined of the 27-point workload: flexible beta")
    ap.add_argument("--inner-rtol", type=float, default=1e-4,
                    help="mixed_refined: inner tolerance / reduction between FP64 residuals")
    ap.add_argument("--precision-inner-rtol", type=float, default=1e-2,
                    help="precision form's mixed_refined: reduction between FP64 residuals")
    ap.add_argument("--no-configs", dest="configs", action="store_false",
                    help="skip the 64^3 Jacobi-PCG, batch, 32-RHS and adjoint keys")
    ap.add_argument("--bench-fd-directions", type=int, default=16,
                    help="finite-difference directions of the default line's adjoint key")
    ap.add_argument("--no-coarse-smallest-last", dest="coarse_smallest_last",
                    action="store_false",
                    help="resident solves: Jones-Plassmann colourings on AMG levels >= 1 "
                         "instead of the host smallest-last colouring (fewer colours, "
                         "setup-time host work; the e2e solve always uses Jones-Plassmann)")
    args = ap.parse_args()
    if args.grid is None:
        # the differentiation and multi-right-hand-side configurations are 128^3
        args.grid = 128 if args.mode in ("adjoint", "multi") else 256
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    if args.impl == "reference":
        run_reference(args)
    elif args.mode == "stencil":
        run_stencil(args)
    elif args.mode == "kernels":
        run_kernels(args)
    elif args.mode == "adjoint":
        run_adjoint(args)
    elif args.mode == "batch":
        run_batch(args)
    elif args.mode == "multi":
        run_multi(args)
    elif args.mode == "profile":
        run_profile(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()

"""Benchmark of the 2-D Jacobi sweep hot path on GB300.

Workload (one bench step): box2d2r (25-point) Jacobi on an 8192 x 8192
interior with a 2-cell zero halo (8196^2 grid), FP16 storage / FP32
accumulate, 100 ping-pong timesteps, tensor-core engine — the plain box2d2r
configuration of the reference's headline comparison.  Inputs are seeded
synthetic U[-1,1) grids with coefficients U[0,1) normalised to sum 1 (the
reference ships no datasets; its benchmark meshes are synthetic too).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  `value` is device-timed Gpts/s (point-updates per
second) with the grid resident in HBM; `e2e` is the same metric through the
public one-call C-ABI (tcs_sweep_host) with pinned host buffers, host<->device
copies inside the timed region.  Each panel plane is 139 MB and a sweep
alternates two of them, so the working set (269 MB) exceeds the 129 MB L2.
`--impl reference` times the CPU gold code (the oracle's port of
common/gold_box2d2r.cpp, in gold's own loop shape) on the host cores, one
timestep of the same grid per bench step.  With torchrun (N > 1) every rank
sweeps its own replica grid (weak scaling, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

INTERIOR = 8192
HALO = 2
TIMESTEPS = 100
STENCIL = "box2d2r"
BYTES_PER_UPDATE = {"f16": 4, "split": 8, "f32": 8}
FLOPS_PER_UPDATE = {"star2d1r": 10, "star2d2r": 18, "box2d1r": 18, "box2d2r": 50}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--stencil", default=STENCIL)
    ap.add_argument("--engine", default="tensor")
    ap.add_argument("--precision", default="f16")
    ap.add_argument("--interior", type=int, default=INTERIOR)
    ap.add_argument("--timesteps", type=int, default=TIMESTEPS)
    ap.add_argument("--temporal-depth", type=int, default=1,
                    help="2: split sweeps in temporally blocked pairs")
    ap.add_argument("--no-extras", action="store_true", help="skip comparator and CPU legs")
    ap.add_argument("--workload", choices=["sweep", "batch", "serve"], default="sweep",
                    help="sweep: one grid (default); batch: 512 mixed grids in one "
                         "persistent launch per run; serve: Poisson-arrival request serving")
    ap.add_argument("--serve-seconds", type=float, default=10.0)
    ap.add_argument("--serve-rate", type=float, default=2000.0)
    ap.add_argument("--serve-round-steps", type=int, default=None,
                    help="steps per request per server round (default: autotuned or 16)")
    ap.add_argument("--batch-grids", type=int, default=512)
    ap.add_argument("--multistep", type=int, default=-1, choices=(-1, 0, 1),
                    help="plain FP16 tensor plans: all timesteps in one launch (1), one launch "
                         "per timestep (0), or by grid size (-1, default)")
    ap.add_argument("--profile", action="store_true",
                    help="profiling driver: upload the grid, run --timesteps single-step "
                         "launches (no graph), exit; for ncu captures")
    return ap.parse_args()


def run_profile(args):
    import torch

    import tcstencil_gb300 as tcs

    if args.workload == "batch":
        from tcstencil_gb300.workloads import mixed_batch

        specs = mixed_batch(args.batch_grids)
        b = build_batch(tcs, specs)
        for k, sp in enumerate(specs):
            b.upload(k, sp.grid())
        b.run(use_graph=False)
        b.run(use_graph=False)
        torch.cuda.synchronize()
        assert tcs.device_error() == 0
        print(f"profile run: batch of {args.batch_grids} mixed grids x 2 runs {b.info()}")
        b.close()
        return
    n = args.interior + 2 * HALO
    A, B = make_inputs(n, args.stencil, 1000)
    plan = tcs.Plan(n, n, args.stencil, B, engine=args.engine, precision=args.precision,
                    temporal_depth=args.temporal_depth)
    plan.set_multistep(args.multistep)
    plan.upload(A)
    plan.run(args.timesteps, use_graph=False)
    torch.cuda.synchronize()
    assert tcs.device_error() == 0
    plan.close()
    print(f"profile run: {args.stencil}/{args.engine}/{args.precision} {n}^2 x {args.timesteps}")


def max_over_ranks(values, device="cuda"):
    """Each value's maximum over all ranks (the slowest replica's time); the
    values themselves when the job runs on one process."""
    import torch

    dist = torch.distributed
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    return int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")), ws


def make_inputs(n_grid: int, stencil: str, seed: int):
    rng = np.random.default_rng(seed)
    r = 1 if stencil in ("star2d1r", "box2d1r") else 2
    n = 2 * r + 1
    A = np.zeros((n_grid, n_grid), np.float32)
    A[HALO:-HALO, HALO:-HALO] = rng.uniform(-1, 1, (n_grid - 2 * HALO,) * 2).astype(np.float32)
    B = rng.random((n, n))
    if stencil.startswith("star"):
        m = np.zeros((n, n), bool)
        m[r, :] = True
        m[:, r] = True
        B = np.where(m, B, 0.0)
    return A, (B / B.sum()).astype(np.float32)


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic(stencil, engine, precision):
    """DRAM bytes per step from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    e = d.get(f"{stencil}/{engine}/{precision}")
    return e.get("dram_bytes_per_step") if e else None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}",
                                       "--format=csv,noheader,nounits", "-i", str(gpu_index),
                                       "-lms", "50"], stdout=self.f, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.p = None
        time.sleep(0.3)

    def stop(self):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [ln.split(", ") for ln in self.f.read().strip().splitlines() if ln.count(",") >= 9]
        os.unlink(self.f.name)
        return rows

    @staticmethod
    def summarize(rows):
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        sm = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        smax = [float(r[3]) for r in rows if r[3].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[6 + i].strip() == "Active"})
        loaded = [s for s in sm if smax and s > 0.5 * max(smax)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows),
                "power_w_max": max((float(r[4]) for r in rows if r[4].strip().replace(".", "").isdigit()),
                                   default=None)}


def metric_name(stencil: str) -> str:
    """The headline metric; both arms (ours and --impl reference) print it."""
    return f"{stencil} Jacobi point-updates per second (Gpts/s)"


def gold_full_grid(args, budget_s: float | None = None, steps: int | None = None,
                   warmup: int = 0):
    """Gold on the host cores, on the bench's own grid: the oracle's port of
    common/gold_<stencil>.cpp in gold's own loop shape (for box stencils the
    output cell is zeroed, then accumulated and stored once per tap, with tap
    rows and columns from k / n and k % n), every host thread on a band of
    rows of ONE (interior + 2*halo)^2 grid, ping-pong steps with a barrier
    between them.  Either `steps` timed steps after `warmup` untimed ones, or
    as many as fit in `budget_s`.  Returns (seconds per step, steps, threads,
    register-accumulator Gpts/s on the same grid for context)."""
    import oracle

    threads = os.cpu_count() or 1
    n = args.interior + 2 * HALO
    A, B = make_inputs(n, args.stencil, 7)
    if warmup:
        oracle.gold_bench_bands(A, B, args.stencil, warmup, threads, loop_shape=True)
    if steps is None:
        t1 = oracle.gold_bench_bands(A, B, args.stencil, 1, threads, loop_shape=True)
        steps = max(1, min(200, int(budget_s / max(t1, 1e-3))))
    t = oracle.gold_bench_bands(A, B, args.stencil, steps, threads, loop_shape=True)
    tr = oracle.gold_bench_bands(A, B, args.stencil, 1, threads, loop_shape=False)
    interior = args.interior * args.interior
    return t / steps, steps, threads, interior / tr / 1e9


def gold_sample_text(args, steps, threads, reg_gpts):
    n = args.interior + 2 * HALO
    return (f"{steps} of the {args.timesteps} timesteps of the workload: gold's loop shape "
            f"(port of common/gold_{args.stencil}.cpp; box stencils store into the output cell "
            f"once per tap) over the whole {n}^2 grid, {threads} host threads on row bands; "
            f"the register-accumulator form of the same arithmetic runs "
            f"{reg_gpts:.3f} Gpts/s here")


def cpu_baseline(args, budget_s: float = 12.0):
    """Gold on every host core, on the bench's grid, for about budget_s."""
    t, steps, threads, reg = gold_full_grid(args, budget_s=budget_s)
    return {"value": args.interior * args.interior / t / 1e9, "unit": "Gpts/s", "cores": threads,
            "kind": "port", "sample": gold_sample_text(args, steps, threads, reg)}


def run_reference(args):
    """The reference's CPU implementation of the path (gold, as the oracle's
    port in gold's own loop shape) on the host cores: each bench step is one
    timestep over the bench's whole grid.  Under torchrun only rank 0 runs."""
    rank, _, ws = dist_env()
    if rank != 0:
        return
    t, steps, threads, reg = gold_full_grid(args, steps=args.steps, warmup=args.warmup)
    v = args.interior * args.interior / t / 1e9
    cfg = workload_config(args)
    cfg.update({"engine": "cpu (gold port, gold's loop shape)", "precision": "f32",
                "storage": "f32", "accumulate": "f32",
                "parallelism": "host threads on row bands of one grid",
                "l2": "CPU run: two FP32 host grids",
                "sample": f"one of the {args.timesteps} timesteps per bench step"})
    print(json.dumps({
        "impl": "reference", "metric": metric_name(args.stencil),
        "value": v, "unit": "Gpts/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": cfg,
        "cpu_baseline": {"value": v, "unit": "Gpts/s", "cores": threads, "kind": "port",
                         "sample": gold_sample_text(args, steps, threads, reg)},
        "e2e": {"value": v, "unit": "Gpts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def workload_config(args):
    n = args.interior + 2 * HALO
    return {"workload": f"{args.stencil} Jacobi, {args.interior}x{args.interior} interior + "
                        f"{HALO}-cell zero halo ({n}^2 grid), {args.timesteps} ping-pong "
                        f"timesteps per bench step",
            "stencil": args.stencil, "grid": [n, n], "timesteps": args.timesteps,
            "engine": args.engine, "precision": args.precision,
            "storage": "f32" if args.precision == "f32" else "f16",
            "accumulate": "f32", "parallelism": "replicas",
            "l2": "inputs larger than L2 (two 139 MB panel planes > 129 MB L2)"}


def build_batch(tcs, specs):
    b = tcs.Batch()
    for sp in specs:
        b.add(sp.ny, sp.nx, sp.stencil, sp.coeffs, sp.steps, sp.precision)
    return b


def batch_leg(torch, tcs, K, W, stream, count=512, check=16):
    """Batched mixed stencils (512 grids, sides log-uniform in [64, 2048], 1-64
    steps, FP16 and split 50/50): one persistent launch per run, replayed as a
    CUDA graph.  Returns device-timed and end-to-end figures, and the error
    against FP64 of `check` grids (half FP16, half split) after one run."""
    from tcstencil_gb300.workloads import mixed_batch

    specs = mixed_batch(count)
    grids = [torch.from_numpy(sp.grid()).pin_memory() for sp in specs]
    outs = [torch.empty_like(g).pin_memory() for g in grids]
    b = build_batch(tcs, specs)
    for k, g in enumerate(grids):
        b.upload(k, g.numpy(), stream=stream)
    pu, items, ngrids = b.info()
    byts = sum(sp.bytes for sp in specs)
    for _ in range(W):
        b.run(use_graph=True, stream=stream)
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(K):
        b.run(use_graph=True, stream=stream)
    stop.record(stream)
    torch.cuda.synchronize()
    t = start.elapsed_time(stop) / 1e3 / K
    assert tcs.device_error() == 0
    # end to end: pinned host grids in, one run, host grids out, every run
    Ke = max(2, K // 4)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(Ke):
        for k, g in enumerate(grids):
            b.upload(k, g.numpy(), stream=stream)
        b.run(use_graph=True, stream=stream)
        for k, o in enumerate(outs):
            b.download(k, o.numpy(), stream=stream)
        torch.cuda.synchronize()
    te = (time.perf_counter() - t0) / Ke
    # accuracy: every grid from its input, one run, a sample against FP64
    for k, g in enumerate(grids):
        b.upload(k, g.numpy(), stream=stream)
    b.run(use_graph=True, stream=stream)
    errs = {"f16": [], "split": []}
    picks = [k for k in range(len(specs)) if specs[k].precision == "f16"][:check // 2] + \
            [k for k in range(len(specs)) if specs[k].precision == "split"][:check // 2]
    for k in picks:
        sp = specs[k]
        b.download(k, outs[k].numpy(), stream=stream)
        torch.cuda.synchronize()
        rel, mx = fp64_error(torch, tcs, grids[k].numpy(), sp.coeffs, sp.stencil, sp.steps,
                             outs[k].numpy())
        errs[sp.precision].append((rel, mx))
    b.close()
    accuracy_sample = {p: {"grids": len(v), "rel_l2_vs_fp64_max": float(f"{max(e[0] for e in v):.4g}"),
                           "rel_l2_vs_fp64_median": float(f"{statistics.median(e[0] for e in v):.4g}"),
                           "max_abs_vs_fp64_max": float(f"{max(e[1] for e in v):.4g}")}
                       for p, v in errs.items() if v}
    host_bytes = sum(g.numel() * 4 for g in grids)
    return {"gpts": pu / t / 1e9, "ms_per_run": 1e3 * t, "point_updates_per_run": pu,
            "items_per_run": items, "grids": ngrids, "algorithmic_bytes_per_run": byts,
            "achieved_gbs": byts / t / 1e9, "e2e_gpts": pu / te / 1e9,
            "e2e_h2d_bytes": host_bytes, "e2e_d2h_bytes": host_bytes,
            "accuracy_sample": accuracy_sample}


def serve_round_steps(args):
    if args.serve_round_steps is not None:
        return args.serve_round_steps
    from tcstencil_gb300.autotune import best_round_steps

    return best_round_steps(args.serve_rate)


def serve_leg(tcs, seconds=10.0, rate=2000.0, budget_gb=120.0, round_steps=16, check=16):
    """Served stencil solves: Poisson arrivals at `rate`/s for `seconds`, sides
    log-uniform in [128, 4096] per axis, random stencil and coefficients, 1-200
    steps, FP16 or split; admission against a `budget_gb` HBM budget.  Then
    `check` of the requests are served again and checked against FP64."""
    from tcstencil_gb300.serving import InputPool, OutputRing, replay
    from tcstencil_gb300.workloads import poisson_requests

    import torch

    reqs = poisson_requests(rate=rate, duration=seconds)
    srv = tcs.Server(int(budget_gb * 2**30), round_steps=round_steps)
    pool = InputPool(1 << 26)
    try:
        res = replay(srv, reqs, pool, OutputRing(1 << 30))
        # accuracy of served results: a sample of the requests, served again
        # together, each against its FP64 shadow
        sample = reqs[::max(1, len(reqs) // check)][:check]
        held = []
        for rq in sample:
            sp = rq.spec
            g = np.ascontiguousarray(pool.grid(sp.ny, sp.nx, sp.seed))
            out = np.empty((sp.ny, sp.nx), np.float32)
            held.append((srv.submit(g, out, sp.stencil, sp.coeffs, sp.steps, sp.precision),
                         sp, g, out))
        errs = {"f16": [], "split": []}
        for t, sp, g, out in held:
            srv.wait(t, 60.0)
            errs[sp.precision].append(fp64_error(torch, tcs, g, sp.coeffs, sp.stencil,
                                                 sp.steps, out))
    finally:
        srv.close()
    res["accuracy_sample"] = {
        p: {"requests": len(v), "rel_l2_vs_fp64_max": float(f"{max(e[0] for e in v):.4g}"),
            "rel_l2_vs_fp64_median": float(f"{statistics.median(e[0] for e in v):.4g}"),
            "max_abs_vs_fp64_max": float(f"{max(e[1] for e in v):.4g}")}
        for p, v in errs.items() if v}
    res["algorithmic_bytes"] = sum(r.spec.bytes for r in reqs)
    res["achieved_gbs"] = res["algorithmic_bytes"] / res["span_s"] / 1e9
    res["offered_gpts"] = res["point_updates"] / seconds / 1e9
    res["budget_gb"] = budget_gb
    res["round_steps"] = round_steps
    return res


def split_input(interior, stencil):
    """The split configuration's input: U[-1,1) + sin(2 pi x) sin(2 pi y) on
    the interior, a zero halo of the stencil's radius, normalised coefficients."""
    from tcstencil_gb300.workloads import normalized_coeffs

    r = 1 if stencil in ("star2d1r", "box2d1r") else 2
    n = interior + 2 * r
    rng = np.random.default_rng(3000)
    yy, xx = np.meshgrid(np.arange(interior) / interior, np.arange(interior) / interior,
                         indexing="ij")
    A = np.zeros((n, n), np.float32)
    A[r:-r, r:-r] = (rng.uniform(-1, 1, (interior, interior)) +
                     np.sin(2 * np.pi * xx) * np.sin(2 * np.pi * yy))
    del xx, yy
    return A, normalized_coeffs(rng, stencil)


def split_config_leg(torch, tcs, stream, interior=16384, steps=200, check_every=50,
                     stencil="box2d1r"):
    """Split-precision configuration: box2d1r on a 16384^2 interior + 1-cell
    zero halo, input U[-1,1) + sin(2 pi x) sin(2 pi y), 200 steps.  Times the
    200 steps (CUDA events, graph replay), then replays them one by one beside
    the FP64 shadow (tcs_drift) and reports the error after every step, with
    the drift checks every 50 steps called out."""
    from tcstencil_gb300.autotune import best_config

    r = 1 if stencil in ("star2d1r", "box2d1r") else 2
    n = interior + 2 * r
    A, B = split_input(interior, stencil)
    _, depth = best_config(stencil, "split", n, n)
    plan = tcs.Plan(n, n, stencil, B, engine="tensor", precision="split", temporal_depth=depth)
    plan.upload(A)
    plan.run(10, use_graph=True, stream=stream)
    torch.cuda.synchronize()
    plan.upload(A)
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(stream)
    plan.run(steps, use_graph=True, stream=stream)
    b.record(stream)
    torch.cuda.synchronize()
    t = a.elapsed_time(b) / 1e3
    assert tcs.device_error() == 0
    pts = interior * interior * steps
    # error vs FP64 after every step (not timed)
    drift = tcs.Drift(n, n, stencil, B)
    plan.upload(A)
    drift.upload(A)
    out = torch.empty((n, n), dtype=torch.float32, device="cuda")
    errs = []
    for k in range(steps):
        plan.run(1, use_graph=False, stream=stream)
        drift.run(1)
        plan.download(out, stream=stream)
        rel, mx = drift.compare(out, stream=stream)
        errs.append(rel)
    drift.close()
    plan.close()
    peak, _ = load_peaks()
    return {"workload": f"{stencil} split precision, {interior}^2 interior + {r}-cell zero halo, "
                        f"{steps} steps, U[-1,1) + sin(2 pi x) sin(2 pi y)",
            "gpts": pts / t / 1e9, "ms_per_step": 1e3 * t / steps,
            "roofline_frac": 8 * pts / t / 1e9 / peak, "temporal_depth": depth,
            "rel_l2_vs_fp64_max": max(errs), "max_abs_vs_fp64_final": mx,
            "drift_checks": {str(s): errs[s - 1] for s in range(check_every, steps + 1, check_every)},
            "rel_l2_vs_fp64_every_10_steps": [round(e, 10) for e in errs[9::10]]}


def timed_sweeps(torch, tcs, plan, K, W, timesteps, stream):
    for _ in range(W):
        plan.run(timesteps, use_graph=True, stream=stream)
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(K):
        plan.run(timesteps, use_graph=True, stream=stream)
    stop.record(stream)
    torch.cuda.synchronize()
    return start.elapsed_time(stop) / 1e3


def fp64_error(torch, tcs, A, B, stencil, steps, result, rect=None):
    """(relative L2, max abs) of an FP32 result (device tensor or host array)
    against the device FP64 shadow of the same problem (tcs_drift: the
    oracle's FP64 restatement of gold, bit for bit) after `steps` steps."""
    ny, nx = A.shape
    d = tcs.Drift(ny, nx, stencil, B, rect=rect)
    d.upload(np.ascontiguousarray(A, np.float32))
    d.run(steps)
    if isinstance(result, np.ndarray):
        result = torch.from_numpy(np.ascontiguousarray(result, np.float32)).cuda()
    rel, mx = d.compare(result)
    d.close()
    return rel, mx


def plan_result(torch, tcs, A, B, stencil, steps, engine, precision, stream):
    """The device FP32 result of `steps` steps of A through a plan."""
    n0, n1 = A.shape
    p = tcs.Plan(n0, n1, stencil, B, engine=engine, precision=precision)
    p.upload(A)
    p.run(steps, use_graph=True, stream=stream)
    out = torch.empty((n0, n1), dtype=torch.float32, device="cuda")
    p.download(out, stream=stream)
    torch.cuda.synchronize()
    p.close()
    return out


def accuracy(torch, tcs, A, B, stencil, steps, out, stream, gold=True):
    """Error of a result against FP64 and, with gold=True, against FP32 gold
    (the CUDA-core F32 engine, which reproduces common/gold_*.cpp bit for bit)."""
    rel, mx = fp64_error(torch, tcs, A, B, stencil, steps, out)
    acc = {"rel_l2_vs_fp64": rel, "max_abs_vs_fp64": mx}
    if gold:
        g = plan_result(torch, tcs, A, B, stencil, steps, "cudacore", "f32", stream)
        d = (out.double() - g.double())
        acc["max_abs_vs_gold_f32"] = float(d.abs().max())
        acc["rel_l2_vs_gold_f32"] = float(d.norm() / g.double().norm())
        del g, d
    return {k: float(f"{v:.4g}") for k, v in acc.items()}


def flush_l2(torch, scratch):
    scratch.add_(1)


def events_timed(torch, stream, fn, reps, scratch):
    """Seconds of `reps` calls of fn, each timed alone with CUDA events on
    `stream`, L2 flushed (a write larger than L2) between them."""
    total = 0.0
    for _ in range(reps):
        flush_l2(torch, scratch)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        b.synchronize()
        total += a.elapsed_time(b) / 1e3
    return total


def config1_leg(torch, tcs, stream, reps=200):
    """The first configuration: star2d1r on a 1024^2 interior + 1-cell zero
    halo (1026^2), U[0,1) inputs, 5 coefficients U[0,1) normalised to sum 1,
    10 ping-pong steps, FP16 storage / FP32 accumulate, both engines; each of
    `reps` runs timed alone with L2 flushed before it; errors against FP64
    and FP32 gold; gold on the host cores beside it."""
    import oracle
    from tcstencil_gb300.workloads import normalized_coeffs

    n, steps, st = 1026, 10, "star2d1r"
    rng = np.random.default_rng(1000)
    A = np.zeros((n, n), np.float32)
    A[1:-1, 1:-1] = rng.random((n - 2, n - 2), dtype=np.float32)
    B = normalized_coeffs(rng, st)
    scratch = torch.empty(64 << 20, dtype=torch.float32, device="cuda")  # 256 MB > L2
    peak, _ = load_peaks()
    pts = (n - 2) ** 2 * steps
    res = {"workload": "star2d1r, 1024^2 interior + 1-cell zero halo, U[0,1), 10 steps, FP16 "
                       "storage / FP32 accumulate; each run timed alone, L2 flushed before it"}
    for eng in ("tensor", "cudacore"):
        # the tensor plan takes the autotuner's tile shape and launch form
        p = tcs.Plan(n, n, st, B, engine="auto" if eng == "tensor" else eng, precision="f16")
        assert p.engine == eng
        tile_w = p.tile_width()
        p.upload(A)
        for _ in range(5):
            p.run(steps, use_graph=True, stream=stream)
        t = events_timed(torch, stream, lambda: p.run(steps, use_graph=True, stream=stream),
                         reps, scratch)
        launches = p.launches(steps)
        p.close()
        out = plan_result(torch, tcs, A, B, st, steps, eng, "f16", stream)
        g = pts * reps / t / 1e9
        res[eng] = {"gpts": round(g, 2), "us_per_run": round(1e6 * t / reps, 2),
                    "launches_per_run": launches, "tile": f"128x{tile_w}",
                    "roofline_frac": round(4 * g / peak, 4),
                    **accuracy(torch, tcs, A, B, st, steps, out, stream)}
    threads = os.cpu_count() or 1
    tc = oracle.gold_bench_bands(A, B, st, steps, threads, loop_shape=True)
    res["cpu_gold"] = {"gpts": round(pts / tc / 1e9, 3), "cores": threads, "kind": "port",
                       "sample": "the whole configuration: gold's loop shape, 10 steps, "
                                 "threads on row bands"}
    del scratch
    return res


def equal_accuracy_leg(torch, tcs, stream, split_res, interior=16384, steps=200):
    """The split configuration's grid run by the FP32 CUDA-core engine (gold's
    arithmetic, FP32 storage, 8 B per point-update like split) and by the plain
    FP16 tensor engine, each timed (CUDA events around one graph replay of the
    200 steps) and checked against FP64, beside the split tensor figures;
    then split against FP32 CUDA cores on box2d2r (below)."""
    st = "box2d1r"
    A, B = split_input(interior, st)
    peak, _ = load_peaks()
    res = {"workload": split_res["workload"],
           "split_tensor": {"gpts": split_res["gpts"], "roofline_frac": split_res["roofline_frac"],
                            "rel_l2_vs_fp64": split_res["rel_l2_vs_fp64_max"]}}

    def timed_form(A, B, st, steps, eng, prec, bpu):
        n = A.shape[0]
        interior = n - 2 * (1 if st in ("star2d1r", "box2d1r") else 2)
        p = tcs.Plan(n, n, st, B, engine=eng, precision=prec)
        p.upload(A)
        p.run(10, use_graph=True, stream=stream)
        p.upload(A)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        p.run(steps, use_graph=True, stream=stream)
        b.record(stream)
        torch.cuda.synchronize()
        t = a.elapsed_time(b) / 1e3
        out = torch.empty((n, n), dtype=torch.float32, device="cuda")
        p.download(out, stream=stream)
        torch.cuda.synchronize()
        p.close()
        rel, mx = fp64_error(torch, tcs, A, B, st, steps, out)
        del out
        g = interior * interior * steps / t / 1e9
        return {"gpts": round(g, 2), "roofline_frac": round(bpu * g / peak, 4),
                "rel_l2_vs_fp64": float(f"{rel:.4g}"), "max_abs_vs_fp64": float(f"{mx:.4g}")}

    for key, eng, prec, bpu in (("f32_cudacore", "cudacore", "f32", 8),
                                ("f16_tensor", "tensor", "f16", 4)):
        res[key] = timed_form(A, B, st, steps, eng, prec, bpu)
    ok = [k for k in ("split_tensor", "f32_cudacore", "f16_tensor")
          if res[k]["rel_l2_vs_fp64"] <= 1e-6]
    res["at_1e-6"] = {"forms": ok,
                      "split_over_f32_cudacore": round(res["split_tensor"]["gpts"] /
                                                       res["f32_cudacore"]["gpts"], 3)}
    del A
    # The 25-point box, whose 25 FMAs per point in gold's order leave the
    # CUDA-core form bound by issue rather than by HBM: the same input form
    # on the bench's 8192^2 interior, 50 steps, split against FP32 CUDA cores.
    A2, B2 = split_input(8192, "box2d2r")
    box = {"workload": "box2d2r, 8192^2 interior + 2-cell zero halo, 50 steps, "
                       "U[-1,1) + sin(2 pi x) sin(2 pi y)"}
    for key, eng, prec in (("split_tensor", "tensor", "split"), ("f32_cudacore", "cudacore", "f32")):
        box[key] = timed_form(A2, B2, "box2d2r", 50, eng, prec, 8)
    box["split_over_f32_cudacore"] = round(box["split_tensor"]["gpts"] /
                                           box["f32_cudacore"]["gpts"], 3)
    res["box2d2r_8192"] = box
    return res


def run_ours(args):
    import torch

    import tcstencil_gb300 as tcs

    rank, local_rank, ws = dist_env()
    torch.cuda.set_device(local_rank)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    n = args.interior + 2 * HALO
    A, B = make_inputs(n, args.stencil, 1000 + rank)
    stream = torch.cuda.current_stream()
    plan = tcs.Plan(n, n, args.stencil, B, engine=args.engine, precision=args.precision,
                    temporal_depth=args.temporal_depth)
    plan.set_multistep(args.multistep)
    plan.upload(A)
    torch.cuda.synchronize()
    updates_per_step = args.interior * args.interior * args.timesteps

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # warm-up, then the timed region with clocks sampled during it
    for _ in range(args.warmup):
        plan.run(args.timesteps, use_graph=True, stream=stream)
    barrier()
    sampler = ClockSampler(local_rank) if rank == 0 else None
    barrier()
    t = timed_sweeps(torch, tcs, plan, args.steps, 0, args.timesteps, stream)
    clocks = ClockSampler.summarize(sampler.stop()) if sampler else None
    (tmax,) = max_over_ranks([t])
    assert tcs.device_error() == 0
    value = ws * updates_per_step * args.steps / tmax / 1e9
    # the dominant kernel's launches: one per bench step when all timesteps
    # run in one multi-step launch, else one per timestep (or step pair)
    launches_per_run = plan.launches(args.timesteps)
    steps_per_launch = args.timesteps / launches_per_run
    launch_s = t / (args.steps * launches_per_run)
    bpu = BYTES_PER_UPDATE[args.precision]
    achieved = bpu * args.interior * args.interior * steps_per_launch / launch_s / 1e9
    peak, peak_kind = load_peaks()
    traffic_step = load_traffic(args.stencil, args.engine, args.precision)
    traffic = round(traffic_step * steps_per_launch) if traffic_step else None

    # e2e through the one-call C-ABI with pinned host buffers
    h_in = torch.from_numpy(A).pin_memory().numpy()
    h_out = torch.empty((n, n), dtype=torch.float32).pin_memory().numpy()
    e2e_steps = max(3, args.steps // 4)
    for _ in range(2):
        tcs.sweep_host(h_in, args.timesteps, args.stencil, B, engine=args.engine,
                       precision=args.precision, h_out=h_out)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        tcs.sweep_host(h_in, args.timesteps, args.stencil, B, engine=args.engine,
                       precision=args.precision, h_out=h_out)
    torch.cuda.synchronize()
    te = time.perf_counter() - t0
    (te,) = max_over_ranks([te])
    e2e = {"value": ws * updates_per_step * e2e_steps / te / 1e9, "unit": "Gpts/s",
           "h2d_bytes_per_step": n * n * 4, "d2h_bytes_per_step": n * n * 4,
           "api": "tcs_sweep_host (pinned host FP32 grid in/out, cached plan)"}
    # the same metric through the double-buffered pipe: each grid's copies and
    # packing overlap the other slot's sweeps
    pipe = tcs.Pipe(n, n, args.stencil, B, engine=args.engine, precision=args.precision)
    h_outs = [torch.empty((n, n), dtype=torch.float32).pin_memory().numpy() for _ in range(2)]
    for k in range(2):
        pipe.submit(h_in, h_outs[k], args.timesteps)
    pipe.wait()
    barrier()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        pipe.submit(h_in, h_outs[k % 2], args.timesteps)
    pipe.wait()
    tp = time.perf_counter() - t0
    pipe.close()
    (tp,) = max_over_ranks([tp])
    e2e_pipelined = {"value": ws * updates_per_step * e2e_steps / tp / 1e9, "unit": "Gpts/s",
                     "h2d_bytes_per_step": n * n * 4, "d2h_bytes_per_step": n * n * 4,
                     "api": "tcs_pipe_submit (two plans on two streams, pinned host FP32 grid in/out)"}
    # the headline result's error: the same timesteps from the same input,
    # against FP64 and against FP32 gold
    plan.upload(A)
    plan.run(args.timesteps, use_graph=True, stream=stream)
    out = torch.empty((n, n), dtype=torch.float32, device="cuda")
    plan.download(out, stream=stream)
    torch.cuda.synchronize()
    plan.close()
    tcs.lib().tcs_release_cache()
    head_acc = accuracy(torch, tcs, A, B, args.stencil, args.timesteps, out, stream)
    del out

    extras = {}
    if rank == 0 and not args.no_extras:
        # the other engine and stencil of the same configuration, same GPU
        for st in ("box2d2r", "star2d2r"):
            for eng in ("tensor", "cudacore"):
                if st == args.stencil and eng == args.engine:
                    continue
                A2, B2 = make_inputs(n, st, 2000)
                p2 = tcs.Plan(n, n, st, B2, engine=eng, precision="f16")
                p2.upload(A2)
                t2 = timed_sweeps(torch, tcs, p2, max(5, args.steps // 4), 2, args.timesteps, stream)
                p2.close()
                g2 = updates_per_step * max(5, args.steps // 4) / t2 / 1e9
                o2 = plan_result(torch, tcs, A2, B2, st, args.timesteps, eng, "f16", stream)
                extras[f"{st}/{eng}/f16"] = {
                    "gpts": round(g2, 2), "roofline_frac": round(4 * g2 / load_peaks()[0], 4),
                    **accuracy(torch, tcs, A2, B2, st, args.timesteps, o2, stream)}
                del o2
        extras["config1_star2d1r_1026"] = config1_leg(torch, tcs, stream)
        r = split_config_leg(torch, tcs, stream)
        extras["split_16384_box2d1r"] = {k: (round(v, 10) if isinstance(v, float) else v)
                                         for k, v in r.items()}
        extras["equal_accuracy_16384_box2d1r"] = equal_accuracy_leg(torch, tcs, stream, r)
        r = batch_leg(torch, tcs, 10, 3, stream)
        extras["batched_512_mixed"] = {k: round(v, 3) if isinstance(v, float) else v
                                       for k, v in r.items()}
        r = serve_leg(tcs, args.serve_seconds, args.serve_rate, round_steps=serve_round_steps(args))
        extras["served_poisson"] = {k: round(v, 3) if isinstance(v, float) else v
                                    for k, v in r.items()}
    if ws > 1:
        torch.distributed.barrier()
    if rank != 0:
        torch.distributed.destroy_process_group()
        return
    line = {
        "metric": metric_name(args.stencil),
        "value": round(value, 3), "unit": "Gpts/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1e3 * tmax / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f16" if args.precision != "f32" else "f32",
        "data": "synthetic (seeded U[-1,1) grid, normalised U[0,1) coefficients)",
        "config": workload_config(args),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic,
                     "peak_kind": peak_kind,
                     "basis": f"{bpu} B per point-update x {args.interior}^2 updates x "
                              f"{steps_per_launch:g} steps per launch / mean launch time "
                              f"{launch_s * 1e6:.2f} us (CUDA events); traffic = ncu DRAM bytes "
                              f"per step x steps per launch"},
        "accuracy": {**head_acc, "basis": "the headline's timesteps from its input, against the "
                                          "device FP64 shadow (tcs_drift) and FP32 gold (the "
                                          "CUDA-core F32 engine, bit-exact with gold)"},
        "e2e": e2e,
        "e2e_pipelined": e2e_pipelined,
        "gpu_launches": args.steps * launches_per_run,
        "clocks": clocks,
        "tflops_useful": round(value * FLOPS_PER_UPDATE[args.stencil] / 1e3, 2),
        "comparators_gpts": extras,
    }
    if not args.no_extras:
        line["cpu_baseline"] = cpu_baseline(args)
    print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()


def run_batch(args):
    """--workload batch: the batched mixed-stencil configuration as the line."""
    import torch

    import tcstencil_gb300 as tcs

    rank, local_rank, ws = dist_env()
    torch.cuda.set_device(local_rank)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    stream = torch.cuda.current_stream()
    sampler = ClockSampler(local_rank) if rank == 0 else None
    r = batch_leg(torch, tcs, args.steps, args.warmup, stream, args.batch_grids)
    clocks = ClockSampler.summarize(sampler.stop()) if sampler else None
    t = r["ms_per_run"] * args.steps / 1e3
    te = r["point_updates_per_run"] / r["e2e_gpts"] / 1e9
    t, te = max_over_ranks([t, te])
    if rank != 0:
        torch.distributed.destroy_process_group()
        return
    peak, peak_kind = load_peaks()
    pu = r["point_updates_per_run"]
    line = {
        "metric": "batched mixed-stencil Jacobi point-updates per second (Gpts/s)",
        "value": round(ws * pu * args.steps / t / 1e9, 3), "unit": "Gpts/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * t / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f16",
        "data": "synthetic (seeded U[-1,1) grids, normalised U[0,1) coefficients)",
        "config": {"workload": f"{r['grids']} grids, sides log-uniform in [64, 2048] per axis, "
                               "stencil uniform over the four, 1-64 steps each, FP16 and split "
                               "50/50; one persistent launch per run (CUDA graph)",
                   "grids": r["grids"], "items_per_run": r["items_per_run"],
                   "point_updates_per_run": pu, "parallelism": "replicas",
                   "l2": "inputs larger than L2 (1.3 GB of planes > 129 MB L2)"},
        "roofline": {"bound": "hbm", "achieved": round(r["achieved_gbs"], 1), "peak": peak,
                     "unit": "GB/s", "frac": round(r["achieved_gbs"] / peak, 4),
                     "traffic": None, "peak_kind": peak_kind,
                     "basis": "4 B (FP16) / 8 B (split) per point-update, summed over the batch, "
                              "/ run time (CUDA events)"},
        "e2e": {"value": round(ws * pu / te / 1e9, 3), "unit": "Gpts/s",
                "h2d_bytes_per_step": r["e2e_h2d_bytes"], "d2h_bytes_per_step": r["e2e_d2h_bytes"],
                "api": "tcs_batch_upload / tcs_batch_run / tcs_batch_download, pinned host grids"},
        "gpu_launches": 2 * args.steps,
        "clocks": clocks,
    }
    print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()


def run_serve(args):
    """--workload serve: the served configuration as the line (rank 0 only
    serves; a server is per GPU, so N GPUs are N independent replicas)."""
    import torch

    import tcstencil_gb300 as tcs

    rank, local_rank, ws = dist_env()
    torch.cuda.set_device(local_rank)
    sampler = ClockSampler(local_rank) if rank == 0 else None
    r = serve_leg(tcs, args.serve_seconds, args.serve_rate, round_steps=serve_round_steps(args))
    clocks = ClockSampler.summarize(sampler.stop()) if sampler else None
    if rank != 0:
        return
    peak, peak_kind = load_peaks()
    line = {
        "metric": "served stencil solves: aggregate point-updates per second (Gpts/s), "
                  "p50/p99 latency in 'latency'",
        "value": round(r["gpts"], 3), "unit": "Gpts/s", "n_gpus": ws, "steps": r["requests"],
        "warmup": 0, "ms_per_step": round(r["mean_ms"], 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f16",
        "data": "synthetic (Poisson arrivals; seeded U[-1,1) grids, normalised coefficients)",
        "config": {"workload": f"Poisson arrivals at {args.serve_rate:g} req/s for "
                               f"{args.serve_seconds:g} s, sides log-uniform in [128, 4096], "
                               "random stencil, 1-200 steps, FP16 or split, 120 GB HBM budget",
                   "requests": r["requests"], "parallelism": "replicas",
                   "l2": "request state far larger than L2"},
        "latency": {"p50_ms": r["p50_ms"], "p99_ms": r["p99_ms"], "mean_ms": r["mean_ms"],
                    "max_ms": r["max_ms"], "basis": "completion (result in host memory) minus "
                                                    "scheduled arrival"},
        "roofline": {"bound": "hbm", "achieved": round(r["achieved_gbs"], 1), "peak": peak,
                     "unit": "GB/s", "frac": round(r["achieved_gbs"] / peak, 4),
                     "traffic": None, "peak_kind": peak_kind,
                     "basis": "4 B (FP16) / 8 B (split) per point-update over the arrival-to-"
                              "last-completion span"},
        "e2e": {"value": round(r["gpts"], 3), "unit": "Gpts/s",
                "h2d_bytes_per_step": None, "d2h_bytes_per_step": None,
                "api": "tcs_server_submit with pinned host grids; every request's host grid "
                       "goes in and its result comes back inside the span"},
        "serving": {k: (round(v, 4) if isinstance(v, float) else v) for k, v in r.items()},
        "gpu_launches": r["rounds"],
        "clocks": clocks,
    }
    print(json.dumps(line))


def main():
    args = parse()
    if args.profile:
        run_profile(args)
    elif args.impl == "ours" and args.workload == "serve":
        run_serve(args)
    elif args.impl == "ours" and args.workload == "batch":
        run_batch(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

"""Autotuner: measures candidate configurations on the device and persists
the fastest per problem class in a JSON cache.

The reference picks its brick tiling by sweeping TILE_SIZE over compiled
variants and reading ncu durations (script/param.py:5, script/nvcc_compile.py,
script/process_data.py:29-43).  Here the candidates are run-time choices of
one library, timed with CUDA events:

  sweep  (stencil, precision, size class) -> engine ("tensor" | "cudacore"),
                                             temporal depth (1 | 2), launch
                                             form (one launch per step, or one
                                             launch for all steps of a call)
                                             and tile shape (128 rows by 128,
                                             96 or 64 columns; plain FP16)
  serve  (offered load)                   -> round_steps of the request server

Size classes are half octaves of each side (sqrt(2) steps), so one entry
covers grids of similar shape.  The cache file is TCS_AUTOTUNE_CACHE, else
~/.cache/tcstencil_gb300/autotune.json; entries are keyed by GPU name, so one
file can hold several machines' results.  Lookups fall back to the results
shipped with the package (tuned.json, measured on GB300 by this module) when
the cache has no entry.

    python -m tcstencil_gb300.autotune [--sweep] [--serve] [--cache PATH]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import time

import numpy as np

from .workloads import RADIUS, normalized_coeffs

ENGINES_FOR = {"f16": ("tensor", "cudacore"), "split": ("tensor",), "f32": ("cudacore",)}
# (engine, temporal depth, one launch for all steps, tile width) candidates
# per precision
CANDIDATES = {"f16": (("tensor", 1, 0, 128), ("tensor", 1, 1, 128), ("tensor", 1, 0, 96),
                      ("tensor", 1, 1, 96), ("tensor", 1, 0, 64), ("tensor", 1, 1, 64),
                      ("cudacore", 1, 0, 128)),
              "split": (("tensor", 1, 0, 128), ("tensor", 1, 1, 128), ("tensor", 2, 0, 128)),
              "f32": (("cudacore", 1, 0, 128),)}


def candidate_key(engine: str, depth: int, multistep: int, tile_w: int = 128) -> str:
    """"tensor/1" (one launch per step), "tensor/1/m" (one launch),
    "tensor/1/m/w64" (and 64-column tiles), ..."""
    return f"{engine}/{depth}" + ("/m" if multistep else "") + (f"/w{tile_w}" if tile_w != 128 else "")


def parse_candidate(key: str) -> tuple:
    """(engine, depth, multistep, tile_w) of a candidate_key."""
    parts = key.split("/")
    w = [int(p[1:]) for p in parts[2:] if p.startswith("w")]
    return parts[0], int(parts[1]), int("m" in parts[2:]), w[0] if w else 128
DEFAULT_ROUND_STEPS = 16
# one square grid per half-octave class from 256 to 8196 (1026 and 8196 are
# the first two benchmark configurations' grids)
SWEEP_SIDES = (256, 362, 512, 724, 1024, 1026, 1600, 2896, 4096, 5792, 8192, 8196)


def cache_path() -> str:
    p = os.environ.get("TCS_AUTOTUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "tcstencil_gb300", "autotune.json")


def device_key() -> str:
    try:
        import torch

        if torch.cuda.is_available():
            return torch.cuda.get_device_name(0)
    except Exception:
        pass
    return "no-gpu"


def size_class(ny: int, nx: int) -> str:
    """Half-octave class of each side: ceil(2 log2 n) / 2, e.g. "10.5x10.5"
    for sides 1025 .. 1448 and "11x11" for 1449 .. 2048."""
    def c(n):
        return f"{math.ceil(2 * math.log2(max(n, 1)) - 1e-9) / 2:g}"
    return f"{c(ny)}x{c(nx)}"


SHIPPED = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuned.json")


class Cache:
    """JSON cache: {device: {"sweep": {key: {...}}, "serve": {key: {...}}}}."""

    def __init__(self, path: str | None = None, shipped: str | None = SHIPPED):
        self.path = path or cache_path()
        self.data = {}
        if os.path.exists(self.path):
            with open(self.path) as f:
                self.data = json.load(f)
        self.shipped = {}
        if shipped and os.path.exists(shipped):
            with open(shipped) as f:
                self.shipped = json.load(f)

    def section(self, name: str, device: str | None = None) -> dict:
        return self.data.setdefault(device or device_key(), {}).setdefault(name, {})

    def lookup(self, name: str, key: str, device: str | None = None):
        dev = device or device_key()
        e = self.data.get(dev, {}).get(name, {}).get(key)
        if e is None:
            e = self.shipped.get(dev, {}).get(name, {}).get(key)
        return e

    def save(self) -> None:
        d = os.path.dirname(self.path)
        if d:
            os.makedirs(d, exist_ok=True)
        tmp = self.path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(self.data, f, indent=1, sort_keys=True)
        os.replace(tmp, self.path)


def sweep_key(stencil: str, precision: str, ny: int, nx: int) -> str:
    return f"{stencil}/{precision}/{size_class(ny, nx)}"


def pick_fastest(timings: dict) -> str:
    """The candidate with the smallest time (ties: first listed)."""
    return min(timings, key=lambda k: (timings[k], list(timings).index(k)))


def time_sweep(engine: str, depth: int, stencil: str, precision: str, ny: int, nx: int,
               steps: int, multistep: int = 0, tile_w: int = 128, reps: int = 3) -> float:
    """Seconds per step of a plan on the device (CUDA-graph runs, CUDA events)."""
    import torch

    import tcstencil_gb300 as tcs

    rng = np.random.default_rng(7)
    g = rng.uniform(-1, 1, (ny, nx)).astype(np.float32)
    p = tcs.Plan(ny, nx, stencil, normalized_coeffs(rng, stencil), engine=engine,
                 precision=precision, temporal_depth=depth)
    try:
        if engine == "tensor" and depth == 1:
            p.set_multistep(multistep)
        if tile_w != 128:
            p.set_tile_width(tile_w)
        p.upload(g)
        p.run(steps, use_graph=True)
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(reps):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
            p.run(steps, use_graph=True)
            b.record()
            torch.cuda.synchronize()
            best = min(best, a.elapsed_time(b) / 1e3 / steps)
    finally:
        p.close()
    return best


def tune_sweep(stencil: str, precision: str, ny: int, nx: int, steps: int = 20,
               cache: Cache | None = None, timer=time_sweep) -> dict:
    """Times every (engine, temporal depth, launch form, tile width) that
    supports the precision; stores and returns {"engine", "temporal_depth",
    "multistep", "tile_w", "s_per_step": {candidate_key: s}}."""
    cache = cache or Cache()
    timings = {candidate_key(e, d, m, w): timer(e, d, stencil, precision, ny, nx, steps, m,
                                                **({"tile_w": w} if w != 128 else {}))
               for e, d, m, w in CANDIDATES[precision]}
    engine, depth, multistep, tile_w = parse_candidate(pick_fastest(timings))
    entry = {"engine": engine, "temporal_depth": depth, "multistep": multistep,
             "tile_w": tile_w, "s_per_step": timings,
             "measured_on": [ny, nx], "when": time.strftime("%Y-%m-%dT%H:%M:%S")}
    cache.section("sweep")[sweep_key(stencil, precision, ny, nx)] = entry
    cache.save()
    return entry


def best_config(stencil: str, precision: str, ny: int, nx: int,
                cache: Cache | None = None) -> tuple:
    """The tuned (engine, temporal depth) for this problem class, else the
    tensor engine at depth 1 (the CUDA-core engine for FP32, the only one
    that has it)."""
    cache = cache or Cache()
    e = cache.lookup("sweep", sweep_key(stencil, precision, ny, nx))
    if e:
        return e["engine"], int(e.get("temporal_depth", 1))
    return CANDIDATES[precision][0][:2]


def best_launch(stencil: str, precision: str, ny: int, nx: int, cache: Cache | None = None) -> int:
    """The tuned launch form for this problem class: 1 (one launch for all
    steps of a call), 0 (one launch per step), or -1 (not tuned: the
    library's size rule)."""
    cache = cache or Cache()
    e = cache.lookup("sweep", sweep_key(stencil, precision, ny, nx))
    return int(e["multistep"]) if e and "multistep" in e else -1


def best_tile_width(stencil: str, ny: int, nx: int, cache: Cache | None = None) -> int:
    """The tuned tile width of plain FP16 tensor sweeps for this problem class
    (128 when not tuned)."""
    cache = cache or Cache()
    e = cache.lookup("sweep", sweep_key(stencil, "f16", ny, nx))
    return int(e.get("tile_w", 128)) if e else 128


def best_engine(stencil: str, precision: str, ny: int, nx: int, cache: Cache | None = None) -> str:
    return best_config(stencil, precision, ny, nx, cache)[0]


def serve_key(rate: float) -> str:
    return f"poisson/{int(round(rate))}"


def tune_serve(rate: float = 2000.0, seconds: float = 3.0, candidates=(0, 4, 8, 16, 32),
               budget_gb: float = 120.0, cache: Cache | None = None, runner=None) -> dict:
    """Replays the served configuration once per round_steps candidate and keeps
    the one with the lowest p99 latency among those that kept up with the
    offered load (throughput within 2 % of the best)."""
    cache = cache or Cache()
    runner = runner or _serve_once
    res = {rs: runner(rate, seconds, rs, budget_gb) for rs in candidates}
    best_gpts = max(r["gpts"] for r in res.values())
    ok = {rs: r for rs, r in res.items() if r["gpts"] >= 0.98 * best_gpts}
    pick = min(ok, key=lambda rs: (ok[rs]["p99_ms"], ok[rs]["p50_ms"]))
    entry = {"round_steps": pick,
             "candidates": {str(rs): {k: r[k] for k in ("gpts", "p50_ms", "p99_ms")}
                            for rs, r in res.items()},
             "when": time.strftime("%Y-%m-%dT%H:%M:%S")}
    cache.section("serve")[serve_key(rate)] = entry
    cache.save()
    return entry


def best_round_steps(rate: float = 2000.0, cache: Cache | None = None) -> int:
    cache = cache or Cache()
    e = cache.lookup("serve", serve_key(rate))
    return e["round_steps"] if e else DEFAULT_ROUND_STEPS


def _serve_once(rate, seconds, round_steps, budget_gb):
    import tcstencil_gb300 as tcs
    from .serving import InputPool, OutputRing, replay
    from .workloads import poisson_requests

    srv = tcs.Server(int(budget_gb * 2**30), round_steps=round_steps)
    try:
        return replay(srv, poisson_requests(rate=rate, duration=seconds), InputPool(1 << 26),
                      OutputRing(1 << 30))
    finally:
        srv.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--cache", default=None)
    ap.add_argument("--sweep", action="store_true", help="engines for the benchmark shapes")
    ap.add_argument("--serve", action="store_true", help="server round quantum")
    ap.add_argument("--rate", type=float, default=2000.0)
    ap.add_argument("--seconds", type=float, default=3.0, help="replay length per serve candidate")
    args = ap.parse_args()
    cache = Cache(args.cache)
    if args.sweep or not args.serve:
        for stencil in RADIUS:
            for precision in ("f16", "split"):
                for n in SWEEP_SIDES:
                    e = tune_sweep(stencil, precision, n, n, cache=cache)
                    print(json.dumps({"key": sweep_key(stencil, precision, n, n), **e}))
    if args.serve:
        print(json.dumps(tune_serve(args.rate, seconds=args.seconds, cache=cache)))


if __name__ == "__main__":
    main()

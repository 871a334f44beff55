"""Sweep harness: time the sweep kernels over a grid of (engine, stencil,
precision, mesh size) and write CSV rows.

The reference builds one binary per (variant, stencil, mesh, tile), runs each
under ncu and post-processes the `Duration` lines into CSV (script/param.py,
script/nvcc_compile.py, script/run_file_with_ncu.sh, script/process_data.py).
Here one process covers the whole sweep: each configuration is a plan on the
device, timed with CUDA events over `--launches` single-step launches after a
warm-up, and reported as the reference's metric (update points per second,
script/draw.py:19) and as a fraction of the measured HBM roofline.  The
reference's TILE_SIZE axis is the tile width here (`--tiles`, plain FP16
tensor sweeps: 128 rows by 128, 96 or 64 columns); as process_data.py:29-43
keeps the default-tile row and the best-tile row, each row says whether it is
the fastest tile of its (variant, stencil, precision, mesh size).

    python -m tcstencil_gb300.harness --sizes 1600,3200,7200 --tiles 128,96,64 --csv out.csv
"""
from __future__ import annotations

import argparse
import csv
import json
import os
import sys

import numpy as np

from . import ENGINES, PRECISIONS, RADIUS, Plan

BYTES_PER_UPDATE = {"f16": 4, "split": 8, "f32": 8}
# script/param.py:4: mesh sizes 160*i, i = 1..45
REFERENCE_SIZES = [160 * i for i in range(1, 46)]


def peak_gbs() -> float:
    p = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                     "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"])
    return 6800.0


def time_config(engine: str, stencil: str, precision: str, n: int, launches: int,
                warmup: int = 5, tile_w: int = 128) -> dict:
    import torch

    rng = np.random.default_rng(n)
    r = RADIUS[stencil]
    k = 2 * r + 1
    B = rng.random((k, k))
    if stencil.startswith("star"):
        m = np.zeros((k, k), bool)
        m[r, :] = True
        m[:, r] = True
        B = np.where(m, B, 0.0)
    B = (B / B.sum()).astype(np.float32)
    # the reference's mesh: N x N interior, padded by r here (gold's domain)
    A = np.zeros((n + 2 * r, n + 2 * r), np.float32)
    A[r:-r, r:-r] = rng.uniform(-1, 1, (n, n)).astype(np.float32)
    plan = Plan(n + 2 * r, n + 2 * r, stencil, B, engine=engine, precision=precision)
    if tile_w != 128:
        plan.set_tile_width(tile_w)
    kernel_launches = plan.launches(launches)  # 1: all steps in one launch
    plan.upload(A)
    stream = torch.cuda.current_stream()
    plan.run(warmup, use_graph=False, stream=stream)
    # the same call once more, untimed: it captures and caches the graph
    plan.run(launches, use_graph=True, stream=stream)
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    plan.run(launches, use_graph=True, stream=stream)
    stop.record(stream)
    torch.cuda.synchronize()
    plan.close()
    ms = start.elapsed_time(stop) / launches
    gpts = n * n / (ms * 1e-3) / 1e9
    achieved = gpts * BYTES_PER_UPDATE[precision]
    return {"variant": engine, "stencil": stencil, "precision": precision, "mesh_size": n,
            "tile": f"128x{tile_w}", "steps": launches, "kernel_launches": kernel_launches,
            "time_ms": round(ms, 5), "gpts": round(gpts, 2),
            "hbm_frac": round(achieved / peak_gbs(), 4)}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--engines", default="tensor,cudacore")
    ap.add_argument("--stencils", default="star2d1r,star2d2r,box2d1r,box2d2r")
    ap.add_argument("--precisions", default="f16")
    ap.add_argument("--sizes", default="1600,3200,4800,7200",
                    help="comma list, or 'reference' for script/param.py's 160*i sizes")
    ap.add_argument("--launches", type=int, default=50)
    ap.add_argument("--tiles", default="128",
                    help="comma list of tile widths (128, 96, 64) for plain FP16 tensor sweeps")
    ap.add_argument("--csv", default="-")
    args = ap.parse_args(argv)
    sizes = REFERENCE_SIZES if args.sizes == "reference" else [int(s) for s in args.sizes.split(",")]
    rows = []
    for engine in args.engines.split(","):
        for precision in args.precisions.split(","):
            if (engine, precision) in (("tensor", "f32"), ("cudacore", "split")):
                continue
            assert engine in ENGINES and precision in PRECISIONS
            for stencil in args.stencils.split(","):
                for n in sizes:
                    widths = ([int(w) for w in args.tiles.split(",")]
                              if (engine, precision) == ("tensor", "f16") else [128])
                    group = [time_config(engine, stencil, precision, n, args.launches, tile_w=w)
                             for w in widths]
                    best = min(group, key=lambda row: row["time_ms"])
                    for row in group:
                        row["best_tile"] = int(row is best)
                    rows.extend(group)
    out = sys.stdout if args.csv == "-" else open(args.csv, "w", newline="")
    w = csv.DictWriter(out, fieldnames=list(rows[0].keys()))
    w.writeheader()
    w.writerows(rows)
    if out is not sys.stdout:
        out.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())

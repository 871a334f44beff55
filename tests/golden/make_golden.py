"""Generates the golden fixtures in tests/golden/ from the reference's own code.

Run here, where the reference sources exist:
    python tests/golden/make_golden.py [--ref-src /path/to/TCStencil]

It compiles the reference's common/gold_*.cpp and layout16/host_*.cu helpers
unchanged (`make -C oracle ref`, outputs in oracle/_ref/), runs them on seeded
inputs and stores inputs and outputs as .npz files.  The fixtures pin the
in-repo oracle (oracle/oracle.c) and need nothing of the reference at test time.
"""
from __future__ import annotations

import argparse
import os
import re
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

STENCILS = ["star2d1r", "star2d2r", "box2d1r", "box2d2r"]


def ref_init_B(n: int) -> np.ndarray:
    """Coefficients the reference's drivers use: B[i] = i with the centre set to
    -40 (3x3, common/main_1r.cu:10-16) or -290 (5x5, common/main_2r.cu:13-19)."""
    B = np.arange(n * n, dtype=np.float32)
    B[(n * n) // 2] = -40.0 if n == 3 else -290.0
    return B.reshape(n, n)


def normalized_B(rng, stencil: str) -> np.ndarray:
    """Uniform [0,1) taps normalised to sum 1 over the stencil's active taps."""
    n = 2 * oracle.RADIUS[stencil] + 1
    B = rng.random((n, n))
    if stencil.startswith("star"):
        mask = np.zeros((n, n), bool)
        mask[n // 2, :] = True
        mask[:, n // 2] = True
        B = np.where(mask, B, 0.0)
    return (B / B.sum()).astype(np.float32)


def ref_sweep(R: oracle.Ref, A: np.ndarray, B: np.ndarray, stencil: str, steps: int) -> np.ndarray:
    """Ping-pong of the reference gold with a fixed border (C starts as A)."""
    cur = A.copy()
    nxt = A.copy()
    for _ in range(steps):
        nxt = R.gold(cur, B, stencil, nxt)
        cur, nxt = nxt, cur
    return cur


def ref_check_error(N, out, ref, region):
    """Runs the reference's checkError2D and checkRelativeError2D (through
    oracle/_ref/ref_check_error) and parses what they print and return."""
    with tempfile.NamedTemporaryFile(delete=False) as f:
        f.write(struct.pack("5i", N, *region))
        f.write(np.ascontiguousarray(out, np.float32).tobytes())
        f.write(np.ascontiguousarray(ref, np.float32).tobytes())
    try:
        r = subprocess.run([os.path.join(oracle.REF_DIR, "ref_check_error"), f.name],
                           capture_output=True, text=True, check=True)
    finally:
        os.unlink(f.name)
    res, part = {}, "abs"
    res["abs_reported"], res["rel_reported"] = [], []
    for line in r.stdout.splitlines():
        m = re.match(r"Values at index \((\d+),(\d+)\) differ", line)
        if m:
            res[f"{part}_reported"].append((int(m.group(1)), int(m.group(2))))
        m = re.match(r"\[Test\] Max (Relative )?Error : (\S+) @ \(,(\d+),(\d+)\)", line)
        if m:
            res[f"{part}_max_line"] = (m.group(2), int(m.group(3)), int(m.group(4)))
        if line.startswith("RMS "):
            res["rms"] = float(line.split()[1])
            part = "rel"
        if line.startswith("REL "):
            res["rel"] = float(line.split()[1])
    return res


def error_metric_cases(rng):
    """Inputs for checkError2D / checkRelativeError2D: noise below and above
    TOLERANCE, references with exact zeros and values below MIN_NUMBER, both
    signs, maxima at (0, 0) and elsewhere."""
    cases = []
    for N, region, noise in ((8, (1, 7, 1, 7), 0.02), (33, (2, 31, 2, 31), 1e-3),
                             (64, (0, 64, 0, 64), 0.05), (40, (1, 39, 3, 37), 1e-4),
                             (16, (0, 16, 0, 16), 0.0)):
        ref = rng.uniform(-1, 1, (N, N)).astype(np.float32)
        ref[region[0], region[2]:region[2] + 3] = [0.0, 5e-7, -3e-7]
        out = (ref + rng.normal(0, noise, (N, N))).astype(np.float32) if noise else ref.copy()
        if noise != 1e-4:
            out[region[0] + 1, region[2] + 1] += 0.3  # one large error
        if N == 16:
            out[0, 0] += 2.0  # the largest error at (0, 0): no "Max" line
        cases.append((N, region, out, ref))
    return cases


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-src", default=oracle.ref_src_dir())
    args = ap.parse_args()
    if not oracle.Ref.build(args.ref_src):
        sys.exit(f"reference sources not found at {args.ref_src}")
    R = oracle.Ref()
    rng = np.random.default_rng(20261203)

    for st in STENCILS:
        n = 2 * oracle.RADIUS[st] + 1
        cases = {}
        for N in (16, 37, 64):
            lo = 0.0 if st == "star2d1r" else -1.0
            A = (lo + (1.0 - lo) * rng.random((N, N))).astype(np.float32)
            for tag, B in (("refB", ref_init_B(n)), ("normB", normalized_B(rng, st))):
                C_in = rng.random((N, N)).astype(np.float32)
                cases[f"A_{N}_{tag}"] = A
                cases[f"B_{N}_{tag}"] = B
                cases[f"Cin_{N}_{tag}"] = C_in
                cases[f"Cout_{N}_{tag}"] = R.gold(A, B, st, C_in)
            Bn = cases[f"B_{N}_normB"]
            cases[f"sweep5_{N}"] = ref_sweep(R, A, Bn, st, 5)
        # host_code semantics: gold on the grid padded by 16 cells of 1.0
        # (layout16/host_star2d1r.cu:138-144), interior N x N
        for N in (32, 48):
            A = rng.random((N, N)).astype(np.float32)
            B = ref_init_B(n)
            P = np.ones((N + 32, N + 32), np.float32)
            P[16:16 + N, 16:16 + N] = A
            out = R.gold(P, B, st)[16:16 + N, 16:16 + N]
            Pabs = np.abs(P)
            absout = R.gold(Pabs, np.abs(B), st)[16:16 + N, 16:16 + N]
            cases[f"drop_A_{N}"] = A
            cases[f"drop_B_{N}"] = B
            cases[f"drop_C_{N}"] = out
            cases[f"drop_absC_{N}"] = absout
        np.savez_compressed(os.path.join(HERE, f"gold_{st}.npz"), **cases)

    # layout helpers: padding_2D -> brick_layout_2D -> reverse_layout_2D
    lay = {}
    for N in (16, 48):
        a16 = oracle.f32_to_f16(rng.random((N, N)).astype(np.float32))
        one = int(np.float16(1.0).view(np.uint16))
        p = R.padding_2d(a16, 16, one)
        b = R.brick_layout_2d(p)
        lay[f"in_{N}"] = a16
        lay[f"padded_{N}"] = p
        lay[f"bricks_{N}"] = b
        lay[f"reversed_{N}"] = R.reverse_layout_2d(b, N + 32)
    np.savez_compressed(os.path.join(HERE, "layout16.npz"), **lay)

    # init_coe band matrices for the drivers' coefficients and a random set
    coe = {}
    for st in STENCILS:
        n = 2 * oracle.RADIUS[st] + 1
        for tag, B in (("refB", ref_init_B(n)),
                       ("randB", (rng.random((n, n)) * 8 - 4).astype(np.float32))):
            B16 = oracle.f32_to_f16(B)
            coe[f"{st}_{tag}_B16"] = B16
            if st.startswith("star"):
                a, b = R.init_coe(B16, st)
                coe[f"{st}_{tag}_a"] = a
                coe[f"{st}_{tag}_b"] = b
            else:
                coe[f"{st}_{tag}_coe"] = R.init_coe(B16, st)
    np.savez_compressed(os.path.join(HERE, "init_coe.npz"), **coe)

    # error metrics (common/common.hpp:38-92), as the reference's build runs them
    err = {}
    for c, (N, region, out, ref) in enumerate(error_metric_cases(rng)):
        res = ref_check_error(N, out, ref, region)
        err[f"c{c}_N"] = np.int32(N)
        err[f"c{c}_region"] = np.array(region, np.int32)
        err[f"c{c}_out"] = out
        err[f"c{c}_ref"] = ref
        err[f"c{c}_rms"] = np.float64(res["rms"])
        err[f"c{c}_rel"] = np.float64(res["rel"])
        for part in ("abs", "rel"):
            err[f"c{c}_{part}_reported"] = np.array(res[f"{part}_reported"], np.int32).reshape(-1, 2)
            line = res.get(f"{part}_max_line")
            err[f"c{c}_{part}_max_line"] = np.array([] if line is None else [line[0]])
            err[f"c{c}_{part}_max_at"] = np.array([] if line is None else line[1:], np.int32)
    np.savez_compressed(os.path.join(HERE, "check_error.npz"), **err)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()

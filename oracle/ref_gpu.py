"""The reference's own GPU kernels on this GPU, as a comparator.

Test and measurement infrastructure: nothing in tcstencil_gb300 imports it.

The modules are `oracle/_ref/mma_run_<stencil>.cubin` (from
layout16/kernel_<stencil>.cu) and `kernel_run_<stencil>.cubin` (from
baseline/kernel_<stencil>.cu). They are the reference's kernels compiled
unchanged for sm_103a (`make -C oracle refgpu`, which needs the reference
sources). A cubin holds only device code, so it loads on the GPU machine's Arm
host through the driver API.

`RefKernel` gives a kernel the inputs the reference's host_code gives it
(layout16/host_star2d1r.cu:129-176, baseline/host_star2d1r.cu:78-118):
- the FP16 grid, padded by 16 cells of 1.0 (padding_2D, :63-75);
- in 16 x 16 bricks (brick_layout_2D, :77-88);
- C initialised with the padded row-major grid (:160);
- the coefficient bands of init_coe (layout16 only);
- the halo gather tables of set_halo_index;
- a grid of (N/16, N/16) blocks of 16 x 2 threads, the padded size N + 32 as
  the kernel's N, and tile size 1 (common/param.hpp TILE_SIZE).
Padding, bricks and bands come from the oracle's restatements, which are
bit-exact with the reference's helpers (tests/test_oracle.py).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import brick_2d, f16_to_f32, f32_to_f16, init_coe_box, init_coe_star, pad_2d, unbrick_2d

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(HERE, "_ref")
RADIUS = {"star2d1r": 1, "star2d2r": 2, "box2d1r": 1, "box2d2r": 2}
F16_ONE = 0x3C00


def cubin(kind: str, stencil: str) -> str:
    """Path of the reference module: kind 'mma_run' (layout16) or 'kernel_run' (baseline)."""
    return os.path.join(REF, f"{kind}_{stencil}.cubin")


def available(kind: str, stencil: str) -> bool:
    return os.path.exists(cubin(kind, stencil))


def reference_coeffs(stencil: str) -> np.ndarray:
    """init_B of common/main_1r.cu:10-16 / main_2r.cu:13-19: B[i] = i, centre -40 / -290."""
    n = 2 * RADIUS[stencil] + 1
    B = np.arange(n * n, dtype=np.float32)
    B[n * n // 2] = -40.0 if n == 3 else -290.0
    return B.reshape(n, n)


def halo_tables(kind: str, stencil: str, P: int):
    """set_halo_index of the reference host files, for padded size P.

    layout16/host_star2d1r.cu:103-118, host_star2d2r.cu:103-120,
    host_box2d1r.cu:99-109, host_box2d2r.cu:101-126; the baseline/ files use
    the same tables except star2d2r's shared-memory slots
    (baseline/host_star2d2r.cu:53-70)."""
    if stencil == "star2d1r":
        i = np.arange(16)
        idx1 = np.concatenate([i, i + 16, i + 32, i + 48])
        idx2 = np.concatenate([i - 16 * P + 240, i + 16 * P, 16 * i - 241, 16 * i + 256])
    elif stencil == "star2d2r":
        i = np.arange(32)
        x, y = i % 16, i // 16
        idx2 = np.concatenate([i - 16 * P + 224, i + 16 * P, 16 * x - 242 + y, 16 * x + 256 + y])
        if kind == "mma_run":
            idx1 = np.concatenate([i, i + 32, 2 * x + y + 64, 2 * x + y + 96])
        else:
            slot = 20 * y + x
            idx1 = np.concatenate([slot + 2, slot + 362, (x + 2) * 20 + y, (x + 2) * 20 + y + 18])
    elif stencil == "box2d1r":
        idx1 = np.array([0, 17, 18, 35])
        idx2 = np.array([-16 * P - 1, 16 * P - 256 + 15, -16 * P + 240, 16 * P + 256])
    else:  # box2d2r
        i = np.arange(16)
        x, y = i // 2, i % 2
        g = i // 4
        idx1 = np.where(g == 0, 20 * y + x,
               np.where(g == 1, 20 * y + x + 16,
               np.where(g == 2, x + 20 * y + 36, x + 20 * y + 52)))
        idx2 = np.where(g == 0, 16 * x - 16 * P + y - 18,
               np.where(g == 1, 16 * x + 16 * P + y - 274,
               np.where(g == 2, 16 * x - 16 * P + y + 416, 16 * x + 16 * P + y + 160)))
    return idx1.astype(np.int32), idx2.astype(np.int32)


class _Driver:
    """The few driver-API calls a module launch needs (the CUDA runtime of
    torch has made the device's primary context current)."""

    def __init__(self):
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.cu.cuModuleLoad.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p]
        self.cu.cuModuleGetFunction.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p,
                                                ctypes.c_char_p]
        self.cu.cuModuleUnload.argtypes = [ctypes.c_void_p]
        self.cu.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 7 + [
            ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p)]

    def check(self, r: int, what: str) -> None:
        if r != 0:
            raise RuntimeError(f"{what} failed: CUresult {r}")


class RefKernel:
    """One reference kernel set up on an N x N FP32 grid (N a multiple of 16)."""

    def __init__(self, kind: str, stencil: str, A: np.ndarray, B: np.ndarray | None = None):
        import torch

        N = A.shape[0]
        if A.shape != (N, N) or N % 16:
            raise ValueError("the reference kernels take N x N grids with N a multiple of 16")
        self.kind, self.stencil, self.N = kind, stencil, N
        P = N + 32
        self.drv = _Driver()
        torch.cuda.init()
        torch.empty(1, device="cuda")
        mod = ctypes.c_void_p()
        self.drv.check(self.drv.cu.cuModuleLoad(ctypes.byref(mod), cubin(kind, stencil).encode()),
                       "cuModuleLoad")
        self.mod = mod
        fn = ctypes.c_void_p()
        self.drv.check(self.drv.cu.cuModuleGetFunction(ctypes.byref(fn), mod, kind.encode()),
                       "cuModuleGetFunction")
        self.fn = fn
        padded = pad_2d(f32_to_f16(A), 16, F16_ONE)  # (P, P) row-major
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
        self.d_A = dev(brick_2d(padded, 16).view(np.int16))
        self.d_C = dev(padded.reshape(-1).view(np.int16))
        idx1, idx2 = halo_tables(kind, stencil, P)
        self.d_i1, self.d_i2 = dev(idx1), dev(idx2)
        ptrs = [self.d_A.data_ptr()]
        if kind == "mma_run":
            n = 2 * RADIUS[stencil] + 1
            B16 = f32_to_f16((reference_coeffs(stencil) if B is None else B).astype(np.float32))
            if stencil.startswith("star"):
                a, b = init_coe_star(B16, n)
                self.d_coe = [dev(a.view(np.int16)), dev(b.view(np.int16))]
            else:
                self.d_coe = [dev(init_coe_box(B16, n).view(np.int16))]
            ptrs += [c.data_ptr() for c in self.d_coe]
        ptrs.append(self.d_C.data_ptr())
        self._args = [ctypes.c_void_p(p) for p in ptrs] + [ctypes.c_int(P), ctypes.c_int(1)] + [
            ctypes.c_void_p(self.d_i1.data_ptr()), ctypes.c_void_p(self.d_i2.data_ptr())]
        self._params = (ctypes.c_void_p * len(self._args))(
            *[ctypes.addressof(a) for a in self._args])

    def launch(self) -> None:
        import torch

        g = self.N // 16
        s = torch.cuda.current_stream().cuda_stream
        self.drv.check(self.drv.cu.cuLaunchKernel(self.fn, g, g, 1, 16, 2, 1, 0, s, self._params,
                                                  None), "cuLaunchKernel")

    def result(self) -> np.ndarray:
        """C's interior (what host_code copies to h_C) as FP32."""
        import torch

        torch.cuda.synchronize()
        P = self.N + 32
        c = self.d_C.cpu().numpy().view(np.uint16)
        full = unbrick_2d(c, P, P, 16)
        return f16_to_f32(full[16:16 + self.N, 16:16 + self.N])

    def time_us(self, launches: int = 20, warmup: int = 3) -> float:
        """Mean launch duration (CUDA events), as host_code's [Time] line."""
        import torch

        for _ in range(warmup):
            self.launch()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(launches):
            self.launch()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) * 1e3 / launches

    def close(self) -> None:
        if getattr(self, "mod", None):
            self.drv.cu.cuModuleUnload(self.mod)
            self.mod = None


def main():
    import argparse
    import json

    ap = argparse.ArgumentParser(description="time the reference's own kernels beside the engine's")
    ap.add_argument("--size", type=int, default=8192, help="N (a multiple of 16)")
    ap.add_argument("--stencils", default="star2d1r,star2d2r,box2d1r,box2d2r")
    args = ap.parse_args()
    rng = np.random.default_rng(1)
    A = rng.random((args.size, args.size), dtype=np.float32)
    for st in args.stencils.split(","):
        row = {"stencil": st, "N": args.size}
        for kind in ("mma_run", "kernel_run"):
            if not available(kind, st):
                row[kind] = "unavailable (make -C oracle refgpu)"
                continue
            k = RefKernel(kind, st, A)
            us = k.time_us()
            k.close()
            row[kind] = {"us": round(us, 2), "gpts": round(args.size ** 2 / us / 1e3, 1)}
        print(json.dumps(row), flush=True)


if __name__ == "__main__":
    main()

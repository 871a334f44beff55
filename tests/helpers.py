"""Shared helpers for the GPU parity tests (inputs, tolerances, device planes)."""
from __future__ import annotations

import numpy as np

import oracle

RADIUS = {"star2d1r": 1, "star2d2r": 2, "box2d1r": 1, "box2d2r": 2}


def normalized_coeffs(rng, stencil: str) -> np.ndarray:
    """Uniform [0,1) taps, normalised in FP64 to sum 1 over the active taps."""
    n = 2 * RADIUS[stencil] + 1
    B = rng.random((n, n))
    if stencil.startswith("star"):
        mask = np.zeros((n, n), bool)
        mask[n // 2, :] = True
        mask[:, n // 2] = True
        B = np.where(mask, B, 0.0)
    return (B / B.sum()).astype(np.float32)


def grid(rng, ny, nx, lo=-1.0, hi=1.0) -> np.ndarray:
    return (lo + (hi - lo) * rng.random((ny, nx))).astype(np.float32)


def f16_ulp(x: np.ndarray) -> np.ndarray:
    """Spacing of FP16 numbers at |x| (subnormal spacing below 2^-14)."""
    a = np.maximum(np.abs(np.asarray(x, dtype=np.float64)), 2.0 ** -14)
    return 2.0 ** (np.floor(np.log2(a)) - 10)


def plane_shape(ny: int, nx: int, cpp: int = 8):
    """(rows per panel, panels) of the engine's panel plane (include/tcs.h)."""
    return -(-ny // 128) * 128 + 8, -(-nx // 128) * 128 // cpp + 2


def plane_index(ny: int, nx: int, cpp: int = 8) -> np.ndarray:
    """Element index of every cell (y, x) in the panel plane."""
    nyp, _ = plane_shape(ny, nx, cpp)
    y = np.arange(ny)[:, None]
    x = np.arange(nx)[None, :]
    return ((x // cpp + 1) * nyp + (y + 4)) * cpp + x % cpp


def to_plane(g: np.ndarray, cpp: int = 8) -> np.ndarray:
    """Host panel plane of a row-major grid (padding cells 0)."""
    ny, nx = g.shape
    nyp, npan = plane_shape(ny, nx, cpp)
    flat = np.zeros(nyp * npan * cpp, g.dtype)
    flat[plane_index(ny, nx, cpp)] = g
    return flat


def plane16(torch, g16: np.ndarray):
    """Device FP16 panel plane (int16 tensor) of a row-major FP16-bits grid."""
    return torch.from_numpy(to_plane(g16).view(np.int16)).cuda()


def grid16(plane, ny: int, nx: int) -> np.ndarray:
    """Row-major FP16 bits of a device panel plane."""
    return plane.cpu().numpy().view(np.uint16)[plane_index(ny, nx)]


def f16tc_step_bound(prev16: np.ndarray, B, stencil: str, rect=None):
    """One tensor-contract oracle step from the FP16 state prev16, and the
    per-cell bound a GPU tensor step from the same state must meet:

        ulp16(|oracle|) + 2^-16 * sum_k |c_k x_k|

    i.e. one FP16 rounding step (the GPU rounds an FP32 sum, the oracle the
    exact sum, so a sum next to a rounding boundary may round the other way)
    plus a wide margin for the FP32 accumulation error of the tensor core's
    sums (a few 2^-24 of the sum of |terms|).  A tile computed from the wrong
    data, or not at all, misses it by the size of the values."""
    ref = oracle.f16_to_f32(oracle.sweep_f16tc(prev16, B, stencil, 1, rect=rect)).astype(np.float64)
    absx = np.abs(oracle.f16_to_f32(prev16)).astype(np.float64)
    c16 = np.abs(oracle.f16_to_f32(oracle.f32_to_f16(B))).astype(np.float64)
    s = oracle.sweep_f64(absx, c16, stencil, 1, rect=rect)
    return ref, f16_ulp(ref) + 2.0 ** -16 * s


def assert_f16tc_step(gpu: np.ndarray, prev16: np.ndarray, B, stencil: str, what: str, rect=None):
    """Checks a GPU tensor FP16 step cell by cell against f16tc_step_bound;
    returns the fraction of cells that differ from the oracle at all."""
    ref, bound = f16tc_step_bound(prev16, B, stencil, rect)
    d = np.abs(np.asarray(gpu, np.float64) - ref)
    bad = d > bound
    if bad.any():
        idx = np.argwhere(bad)[:5].tolist()
        raise AssertionError(f"{what}: {int(bad.sum())} cells beyond one FP16 step of the oracle, "
                             f"e.g. {idx}; max |d| {d.max():.3g}")
    return float((d > 0).mean())

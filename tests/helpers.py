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

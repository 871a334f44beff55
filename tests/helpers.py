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


def plane16(torch, g16: np.ndarray):
    """Device FP16 brick plane (uint16 tensor) of a row-major FP16-bits grid."""
    return torch.from_numpy(oracle.brick_2d(g16).view(np.int16)).cuda()


def grid16(plane, ny: int, nx: int) -> np.ndarray:
    """Row-major FP16 bits of a device brick plane."""
    return oracle.unbrick_2d(plane.cpu().numpy().view(np.uint16), ny, nx)


def brick_index(ny: int, nx: int) -> np.ndarray:
    nbx = (nx + 15) // 16
    y = np.arange(ny)[:, None]
    x = np.arange(nx)[None, :]
    return ((y // 16) * nbx + (x // 16)) * 256 + (y % 16) * 16 + (x % 16)


def plane32(torch, g: np.ndarray):
    ny, nx = g.shape
    flat = np.zeros(((ny + 15) // 16) * ((nx + 15) // 16) * 256, np.float32)
    flat[brick_index(ny, nx)] = g
    return torch.from_numpy(flat).cuda()


def grid32(plane, ny: int, nx: int) -> np.ndarray:
    return plane.cpu().numpy()[brick_index(ny, nx)]

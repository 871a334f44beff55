"""Seeded synthetic workloads of the benchmark configurations (the reference
measures on synthetic meshes only, script/param.py:4).

Every grid is drawn from its own generator, seed = config index x 1000 + grid
id, in FP64 and rounded to FP32; coefficients are U[0,1) normalised in FP64 to
sum 1 over the stencil's active taps.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

STENCILS = ("star2d1r", "star2d2r", "box2d1r", "box2d2r")
RADIUS = {"star2d1r": 1, "star2d2r": 2, "box2d1r": 1, "box2d2r": 2}
BYTES_PER_UPDATE = {"f16": 4, "split": 8, "f32": 8}


def normalized_coeffs(rng: np.random.Generator, stencil: str) -> np.ndarray:
    r = RADIUS[stencil]
    n = 2 * r + 1
    B = rng.random((n, n))
    if stencil.startswith("star"):
        m = np.zeros((n, n), bool)
        m[r, :] = True
        m[:, r] = True
        B = np.where(m, B, 0.0)
    return (B / B.sum()).astype(np.float32)


def log_uniform_int(rng: np.random.Generator, lo: int, hi: int) -> int:
    return int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))


@dataclass
class GridSpec:
    """One stencil problem: a grid, its stencil and coefficients, a step count."""
    gid: int
    stencil: str
    precision: str
    ny: int
    nx: int
    steps: int
    coeffs: np.ndarray = field(repr=False)
    seed: int = 0

    @property
    def updates(self) -> int:
        r = RADIUS[self.stencil]
        return (self.ny - 2 * r) * (self.nx - 2 * r) * self.steps

    @property
    def bytes(self) -> int:
        return BYTES_PER_UPDATE[self.precision] * self.updates

    def grid(self) -> np.ndarray:
        """U[-1,1) interior with a zero border of the stencil's radius."""
        rng = np.random.default_rng(self.seed + 1)
        r = RADIUS[self.stencil]
        g = np.zeros((self.ny, self.nx), np.float32)
        g[r:-r, r:-r] = rng.uniform(-1.0, 1.0, (self.ny - 2 * r, self.nx - 2 * r))
        return g


def mixed_batch(count: int = 512, side=(64, 2048), steps=(1, 64), config: int = 4,
                precisions=("f16", "split")) -> list[GridSpec]:
    """Batched mixed stencils: sides log-uniform per axis, stencil uniform over
    the four, per-grid normalised coefficients, uniform step counts, FP16 and
    split modes alternating (50/50)."""
    out = []
    for gid in range(count):
        seed = config * 1000 + gid
        rng = np.random.default_rng(seed)
        stencil = STENCILS[int(rng.integers(0, 4))]
        ny = log_uniform_int(rng, *side)
        nx = log_uniform_int(rng, *side)
        nsteps = int(rng.integers(steps[0], steps[1] + 1))
        out.append(GridSpec(gid, stencil, precisions[gid % len(precisions)], ny, nx, nsteps,
                            normalized_coeffs(rng, stencil), seed))
    return out


@dataclass
class Request:
    """A served stencil solve: arrives at `arrival` seconds."""
    rid: int
    arrival: float
    spec: GridSpec


def poisson_requests(rate: float = 2000.0, duration: float = 10.0, side=(128, 4096),
                     steps=(1, 200), config: int = 5, max_requests: int | None = None,
                     precisions=("f16", "split")) -> list[Request]:
    """Served stencil solves: Poisson arrivals at `rate` per second over
    `duration` seconds, sides log-uniform per axis, random stencil and
    coefficients, uniform step counts, plain or split precision."""
    rng = np.random.default_rng(config * 1000 + 999)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration or (max_requests is not None and len(out) >= max_requests):
            break
        rid = len(out)
        seed = config * 1000 + rid
        g = np.random.default_rng(seed)
        stencil = STENCILS[int(g.integers(0, 4))]
        ny = log_uniform_int(g, *side)
        nx = log_uniform_int(g, *side)
        nsteps = int(g.integers(steps[0], steps[1] + 1))
        prec = precisions[int(g.integers(0, len(precisions)))]
        out.append(Request(rid, t, GridSpec(rid, stencil, prec, ny, nx, nsteps,
                                            normalized_coeffs(g, stencil), seed)))
    return out

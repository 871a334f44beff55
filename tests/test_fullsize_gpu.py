"""Full-size configuration (box2d2r / star2d2r, 8192^2 interior + 2-cell zero
halo, 100 steps) checked through a size-independent property: the stencil is
local, so after T steps a W x W window depends only on the input within
T*r cells of it.  The oracle sweeps that neighbourhood (clipped at the grid
edge, where the border is fixed) and the window must match: bit-exact for the
CUDA-core engine, within one FP16 step of the value per sweep step for the
tensor engine."""
import numpy as np
import pytest

import oracle
from helpers import f16_ulp, normalized_coeffs

pytestmark = pytest.mark.gpu

N = 8192 + 4
STEPS = 100
W = 40


def windows(rng):
    return [(0, 0), (N - W, 4000), (int(rng.integers(300, N - 300)), int(rng.integers(300, N - 300)))]


@pytest.mark.parametrize("stencil", ["box2d2r", "star2d2r"])
@pytest.mark.parametrize("engine", ["cudacore", "tensor"])
def test_config2_windows_after_100_steps(tcs, torch_cuda, stencil, engine):
    rng = np.random.default_rng(2000)
    A = np.zeros((N, N), np.float32)
    A[2:-2, 2:-2] = rng.uniform(-1, 1, (N - 4, N - 4)).astype(np.float32)
    B = normalized_coeffs(rng, stencil)
    p = tcs.Plan(N, N, stencil, B, engine=engine, precision="f16")
    p.upload(A)
    p.run(STEPS)
    out = np.empty_like(A)
    p.download(out)
    p.close()
    assert tcs.device_error() == 0
    A16 = oracle.f32_to_f16(A)
    r, halo = 2, 2 * STEPS
    for (wy, wx) in windows(rng):
        y0, y1 = max(0, wy - halo), min(N, wy + W + halo)
        x0, x1 = max(0, wx - halo), min(N, wx + W + halo)
        sub = np.ascontiguousarray(A16[y0:y1, x0:x1])
        # update the cells of the region that are grid interior
        rect = (max(r, y0) - y0, min(N - r, y1) - y0, max(r, x0) - x0, min(N - r, x1) - x0)
        f = oracle.sweep_f16cc if engine == "cudacore" else oracle.sweep_f16tc
        ref = f(sub, B, stencil, STEPS, rect=rect)[wy - y0:wy - y0 + W, wx - x0:wx - x0 + W]
        got = oracle.f32_to_f16(out[wy:wy + W, wx:wx + W])
        if engine == "cudacore":
            np.testing.assert_array_equal(got, ref)
        else:
            g = oracle.f16_to_f32(got).astype(np.float64)
            e = oracle.f16_to_f32(ref).astype(np.float64)
            assert np.max(np.abs(g - e)) <= STEPS * f16_ulp(1.0)

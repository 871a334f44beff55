"""Full-size configuration (box2d2r / star2d2r, 8192^2 interior + 2-cell zero
halo, 100 steps) checked in windows through a size-independent property: the
stencil is local, so after T steps a W x W window depends only on the input
within T*r cells of it.  The oracle sweeps that neighbourhood (clipped at the
grid edge, where the border is fixed) and the window must match: bit-exact
for the CUDA-core engine; for the tensor engine within the sum over the steps
of one FP16 rounding step at that step's largest value in the neighbourhood
plus the FP32 accumulation error (each step's error is carried, not grown, by
a normalised non-negative stencil).  The windows sit on the seams of the
128 x 128 tiles, on the grid's corners and on the 65th, partial tile row and
column (rows and columns 8192-8195)."""
import numpy as np
import pytest

import oracle
from helpers import f16_ulp, normalized_coeffs

pytestmark = pytest.mark.gpu

N = 8192 + 4
STEPS = 100
W = 40


def windows(rng):
    s = lambda k: 128 * k - 20  # a window across the seam at tile row/column k
    return [(0, 0), (N - W, N - W), (N - W, s(16)), (s(32), N - W), (s(1), s(32)),
            (s(32), s(16)), (s(16), s(1)), (s(63), s(64) - W // 2), (s(48), s(40)),
            (int(rng.integers(300, N - 300)), int(rng.integers(300, N - 300)))]


def tensor_window_bound(sub16, B, stencil, rect, win):
    """Oracle trajectory of the neighbourhood and the accumulated bound: at
    step t only the cells within (STEPS - t) * r of the window can still reach
    it, so each step's rounding and accumulation terms are taken at the
    largest value there."""
    r = oracle.RADIUS[stencil]
    h, w = sub16.shape

    def cone_max(a, t):
        m = (STEPS - t) * r
        ys = slice(max(0, win[0].start - m), min(h, win[0].stop + m))
        xs = slice(max(0, win[1].start - m), min(w, win[1].stop + m))
        return float(np.abs(oracle.f16_to_f32(a[ys, xs])).max())

    cur = sub16
    m_prev = cone_max(cur, 0)
    tol = 0.0
    for t in range(1, STEPS + 1):
        cur = oracle.sweep_f16tc(cur, B, stencil, 1, rect=rect)
        m = cone_max(cur, t)
        tol += float(f16_ulp(m * (1 + 2.0 ** -10))) + 2.0 ** -16 * m_prev
        m_prev = m
    return cur, 1.1 * tol


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
        assert 0 <= wy <= N - W and 0 <= wx <= N - W
        y0, y1 = max(0, wy - halo), min(N, wy + W + halo)
        x0, x1 = max(0, wx - halo), min(N, wx + W + halo)
        sub = np.ascontiguousarray(A16[y0:y1, x0:x1])
        # update the cells of the region that are grid interior and whose taps
        # stay in the region; the rest, at least T*r cells from the window,
        # cannot reach it within T steps
        rect = (r, min(N - r - y0, y1 - y0 - r), r, min(N - r - x0, x1 - x0 - r))
        win = (slice(wy - y0, wy - y0 + W), slice(wx - x0, wx - x0 + W))
        got = oracle.f32_to_f16(out[wy:wy + W, wx:wx + W])
        if engine == "cudacore":
            ref = oracle.sweep_f16cc(sub, B, stencil, STEPS, rect=rect)[win]
            np.testing.assert_array_equal(got, ref, err_msg=f"window {(wy, wx)}")
        else:
            full, tol = tensor_window_bound(sub, B, stencil, rect, win)
            e = oracle.f16_to_f32(full[win]).astype(np.float64)
            g = oracle.f16_to_f32(got).astype(np.float64)
            d = np.max(np.abs(g - e))
            assert d <= tol, f"window {(wy, wx)}: max |d| {d:.3g} > {tol:.3g}"
            # The bound above holds for any rounding pattern, but near the
            # zero halo it exceeds the values themselves.  Rounding flips are
            # rare and the stencil smooths the early ones away, so the GPU
            # stays within a few FP16 steps of the window's largest value
            # (measured on GB300: at most 1); eight is the bar, which a zeroed, stale
            # or shifted window misses by two orders of magnitude.
            ulp = float(f16_ulp(np.abs(e).max()))
            print(f"window {(wy, wx)}: max |d| = {d / ulp:.2f} FP16 steps of max |window|")
            assert d <= 8 * ulp, f"window {(wy, wx)}: max |d| {d:.3g} = {d / ulp:.1f} steps"

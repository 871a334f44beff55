"""The reference's own kernels on this GPU (oracle/ref_gpu.py).

mma_run (layout16/) and kernel_run (baseline/) are compiled unchanged for
sm_103a and get host_code's own input set-up. That set-up is right when
mma_run's FP16-accumulated result lies within FP16 error of gold (the
reference's main leaves its own check commented out, common/main_1r.cu:33-38).

Measured on GB300 at 512² with the reference's coefficients:
- star2d1r and box2d2r match gold cell for cell within FP16 error;
- star2d2r misses by more than 10 % on about 6 % of cells, the ones seen at
  brick rows 1-3 and columns 0, 1, 14 and 15 (its halo strips), and 80 % of
  cells are within 1 %;
- box2d1r's mma_run misses gold on 96 % of cells, whatever the orientation of
  B. That is a defect of the reference kernel: its own padding, bricks, bands
  and halo tables (shared with the other three) are what it gets here.
The engine's sweep of the same grid must be faster than both kernels."""
import numpy as np
import pytest

import oracle
from oracle import ref_gpu

pytestmark = pytest.mark.gpu


def _need(kind, stencil):
    if not ref_gpu.available(kind, stencil):
        pytest.skip("reference kernels not built (make -C oracle refgpu needs the reference sources)")


def _mma_run_vs_gold(stencil, N=512):
    r = ref_gpu.RADIUS[stencil]
    A = np.random.default_rng(7).random((N, N), dtype=np.float32)
    k = ref_gpu.RefKernel("mma_run", stencil, A)
    k.launch()
    got = k.result()
    k.close()
    expect = oracle.gold_step(A, ref_gpu.reference_coeffs(stencil), stencil,
                              rect=(r, N - r, r, N - r))
    region = (slice(r, N - r), slice(r, N - r))
    d = np.abs(got[region].astype(np.float64) - expect[region])
    rel = d / np.maximum(np.abs(expect[region]), 1.0)
    return rel


@pytest.mark.parametrize("stencil", ["star2d1r", "box2d2r"])
def test_reference_mma_run_matches_gold(torch_cuda, stencil):
    _need("mma_run", stencil)
    rel = _mma_run_vs_gold(stencil)
    # FP16 storage of values up to ~300 and FP16 accumulation
    assert np.mean(rel > 0.01) < 0.05 and np.mean(rel > 0.1) < 1e-3, (np.mean(rel > 0.01),
                                                                      np.mean(rel > 0.1))


def test_reference_star2d2r_matches_gold_on_most_cells(torch_cuda):
    """Measured: 80 % of cells within 1 % (a wrong set-up misses on ~90 %)."""
    _need("mma_run", "star2d2r")
    rel = _mma_run_vs_gold("star2d2r")
    assert np.mean(rel <= 0.01) > 0.75


@pytest.mark.parametrize("stencil", ["star2d1r", "box2d2r"])
def test_engine_beats_the_reference_kernels(tcs, torch_cuda, stencil):
    for kind in ("mma_run", "kernel_run"):
        _need(kind, stencil)
    N = 2048
    A = np.random.default_rng(8).random((N, N), dtype=np.float32)
    ref_us = {}
    for kind in ("mma_run", "kernel_run"):
        k = ref_gpu.RefKernel(kind, stencil, A)
        ref_us[kind] = k.time_us(launches=10)
        k.close()
    torch = torch_cuda
    r = ref_gpu.RADIUS[stencil]
    B = np.random.default_rng(9).random((2 * r + 1, 2 * r + 1)).astype(np.float32)
    B /= B.sum()
    p = tcs.Plan(N + 2 * r, N + 2 * r, stencil, B, engine="tensor")
    p.upload(np.pad(A, r))
    p.run(3, use_graph=False)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    p.run(10, use_graph=False)
    e1.record()
    torch.cuda.synchronize()
    ours = e0.elapsed_time(e1) * 1e3 / 10
    p.close()
    assert ours < ref_us["mma_run"] and ours < ref_us["kernel_run"], (ours, ref_us)

"""Tensor-engine parity where every CTA reuses its pipeline stages and
accumulator slots, checked against the oracle.

The tensor kernels are persistent: CTA b takes tiles b, b + 152, ... of a step
(and, in a multi-step launch, of the following steps).  The FP16 kernel keeps
four shared-memory stages and two TMEM accumulator slots for radius-2 stencils
(three and three for radius 1), so a CTA reuses a stage and a slot from its
fourth or fifth tile on.  Small grids never get there (1026^2 has 81 tiles).
Here:

  * 4100^2 (33 x 33 = 1089 tiles, seven per CTA per step), all four stencils:
    each of the first steps, launched one per step, is checked cell by cell
    against one oracle step of the GPU's own previous state
    (helpers.f16tc_step_bound: one FP16 rounding step plus the FP32
    accumulation error), and the same steps as ONE multi-step launch must give
    the same bits;
  * the 8196^2, 100-step benchmark configuration (box2d2r, star2d2r; 65 x 65 =
    4225 tiles, 28 per CTA per step): steps 1 and 100 checked cell by cell the
    same way, the 100-step multi-step launch bit-identical to 100 single steps,
    and its relative L2 error against the device FP64 shadow (tcs_drift) no
    larger than that of a 1028^2 grid with the same coefficients, whose every
    cell is checked against the oracle (the error of FP16 storage with these
    coefficients does not depend on the grid size);
  * split precision on 4100^2 (box2d1r, box2d2r), 12 steps, whole grid
    against the oracle's split contract, and its error against FP64.
A skipped, repeated or stale tile misses these bounds by the size of the
values.
"""
import numpy as np
import pytest

import oracle
from helpers import assert_f16tc_step, f16_ulp, grid, normalized_coeffs

pytestmark = pytest.mark.gpu


def _download(p, shape):
    out = np.empty(shape, np.float32)
    p.download(out)
    return out


@pytest.mark.parametrize("stencil", ["box2d2r", "box2d1r", "star2d2r", "star2d1r"])
def test_f16_every_step_against_the_oracle_at_seven_tiles_per_cta(tcs, torch_cuda, stencil):
    rng = np.random.default_rng(4100)
    n, steps = 4100, 4
    A = grid(rng, n, n)
    B = normalized_coeffs(rng, stencil)
    p = tcs.Plan(n, n, stencil, B, engine="tensor", precision="f16")
    p.set_multistep(0)  # one launch per step
    p.upload(A)
    prev16 = oracle.f32_to_f16(A)
    diff = []
    for t in range(1, steps + 1):
        p.run(1)
        got = _download(p, A.shape)
        diff.append(assert_f16tc_step(got, prev16, B, stencil, f"{stencil} step {t}"))
        prev16 = oracle.f32_to_f16(got)
    p.close()
    assert max(diff) < 0.01, diff  # rounding differences are rare
    q = tcs.Plan(n, n, stencil, B, engine="tensor", precision="f16")
    q.set_multistep(1)  # the same steps in one launch
    q.upload(A)
    q.run(steps)
    np.testing.assert_array_equal(oracle.f32_to_f16(_download(q, A.shape)), prev16)
    q.close()
    assert tcs.device_error() == 0


def _config2_input(stencil, n):
    rng = np.random.default_rng(2000)
    A = np.zeros((n, n), np.float32)
    A[2:-2, 2:-2] = rng.uniform(-1, 1, (n - 4, n - 4)).astype(np.float32)
    return A, normalized_coeffs(np.random.default_rng(2001), stencil)


@pytest.mark.parametrize("stencil", ["box2d2r", "star2d2r"])
def test_f16_benchmark_grid_100_steps(tcs, torch_cuda, stencil):
    torch = torch_cuda
    n, steps = 8196, 100
    A, B = _config2_input(stencil, n)
    # one launch per step: steps 1 and 100 against the oracle, cell by cell
    p = tcs.Plan(n, n, stencil, B, engine="tensor", precision="f16")
    p.set_multistep(0)
    p.upload(A)
    p.run(1)
    s1 = _download(p, A.shape)
    assert_f16tc_step(s1, oracle.f32_to_f16(A), B, stencil, f"{stencil} 8196^2 step 1")
    p.run(steps - 2)
    s99 = _download(p, A.shape)
    p.run(1)
    s100 = _download(p, A.shape)
    assert_f16tc_step(s100, oracle.f32_to_f16(s99), B, stencil, f"{stencil} 8196^2 step 100")
    p.close()
    del s1, s99
    # the benchmark's form: all 100 steps in one launch, the same bits
    q = tcs.Plan(n, n, stencil, B, engine="tensor", precision="f16")
    q.upload(A)
    assert q.launches(steps) == 1
    q.run(steps)
    out = torch.empty((n, n), dtype=torch.float32, device="cuda")
    q.download(out)
    np.testing.assert_array_equal(out.cpu().numpy(), s100)
    q.close()
    # error against FP64 after 100 steps
    d = tcs.Drift(n, n, stencil, B)
    d.upload(A)
    d.run(steps)
    rel, mx = d.compare(out)
    d.close()
    # the same coefficients on 1028^2: whole grid against the oracle, and its
    # own FP64 error, which FP16 storage with these coefficients sets
    m = 1028
    a = A[:m, :m].copy()
    a[-2:, :] = 0
    a[:, -2:] = 0
    r = tcs.Plan(m, m, stencil, B, engine="tensor", precision="f16")
    r.upload(a)
    r.run(steps)
    small = _download(r, a.shape).astype(np.float64)
    r.close()
    ora = oracle.f16_to_f32(oracle.sweep_f16tc(oracle.f32_to_f16(a), B, stencil, steps))
    assert np.max(np.abs(small - ora)) <= steps * f16_ulp(np.abs(ora).max())
    f64 = oracle.sweep_f64(a.astype(np.float64), B.astype(np.float64), stencil, steps)
    rel_small = np.linalg.norm(small - f64) / np.linalg.norm(f64)
    assert rel <= 1.1 * rel_small + 1e-5, (rel, rel_small, mx)
    assert tcs.device_error() == 0


def _split_field(rng, n):
    yy, xx = np.meshgrid(np.arange(n) / n, np.arange(n) / n, indexing="ij")
    return (rng.uniform(-1, 1, (n, n)) + np.sin(2 * np.pi * xx) * np.sin(2 * np.pi * yy)).astype(np.float32)


@pytest.mark.parametrize("stencil", ["box2d1r", "box2d2r"])
def test_split_whole_grid_at_seven_tiles_per_cta(tcs, torch_cuda, stencil):
    rng = np.random.default_rng(4101)
    n, steps = 4100, 12
    A = _split_field(rng, n)
    B = normalized_coeffs(rng, stencil)
    p = tcs.Plan(n, n, stencil, B, engine="tensor", precision="split")
    p.upload(A)
    p.run(steps)
    got = _download(p, A.shape).astype(np.float64)
    p.close()
    assert tcs.device_error() == 0
    e = oracle.split_scale_exp(A)
    hi, lo = oracle.split(A.astype(np.float64), e)
    h, l, e2 = oracle.sweep_split(hi, lo, B, stencil, steps, scale_exp=e)
    contract = oracle.join(h, l, e2)
    # FP32 (not double) combination of the two accumulators: a few 2^-24 per step
    assert np.max(np.abs(got - contract)) <= steps * 2.0 ** (e - 22)
    f64 = oracle.sweep_f64(A.astype(np.float64), B.astype(np.float64), stencil, steps)
    assert np.linalg.norm(got - f64) / np.linalg.norm(f64) <= 1e-6

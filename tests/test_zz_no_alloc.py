"""tcs_sweep_steps_noalloc: multi-step sweeps for callers that cannot call
cudaMalloc where they sweep (inside CUDA graph capture, allocator-free
real-time loops, memory budgets owned by someone else).  Its ping-pong plane
is a static device array shared by every call, so this checks two calls in a
row, each against the plan path (tcs_plan_*, which allocates its planes), with
the tolerance the other sweep tests use.  Kept in its own file, collected last.
"""
import numpy as np
import pytest

import oracle
from helpers import f16_ulp, grid, grid16, normalized_coeffs, plane16

pytestmark = pytest.mark.gpu


def plan_result16(tcs, A, B, stencil, steps, engine):
    p = tcs.Plan(A.shape[0], A.shape[1], stencil, B, engine=engine, precision="f16")
    p.upload(A)
    p.run(steps)
    out = np.empty_like(A)
    p.download(out)
    p.close()
    return oracle.f32_to_f16(out)


@pytest.mark.parametrize("engine", ["tensor", "cudacore"])
def test_noalloc_two_calls_match_the_plan_path(tcs, torch_cuda, engine):
    torch = torch_cuda
    rng = np.random.default_rng(77)
    cases = [("box2d2r", (300, 411), 5), ("star2d1r", (257, 190), 4)]
    for stencil, (ny, nx), steps in cases:  # two calls in a row on the shared scratch
        A = grid(rng, ny, nx)
        B = normalized_coeffs(rng, stencil)
        expect = plan_result16(tcs, A, B, stencil, steps, engine)
        A16 = oracle.f32_to_f16(A)
        d_in = plane16(torch, A16)
        d_out = torch.zeros_like(d_in)
        tcs.sweep_steps_noalloc(d_in, d_out, ny, nx, stencil, B, steps, engine=engine)
        torch.cuda.synchronize()
        assert tcs.device_error() == 0
        got = grid16(d_out, ny, nx)
        np.testing.assert_array_equal(grid16(d_in, ny, nx), A16)  # input untouched
        if engine == "cudacore":
            np.testing.assert_array_equal(got, expect)
        else:
            g = oracle.f16_to_f32(got).astype(np.float64)
            e = oracle.f16_to_f32(expect).astype(np.float64)
            assert np.max(np.abs(g - e)) <= steps * f16_ulp(np.abs(e).max())


def test_noalloc_rejects_grids_beyond_the_static_scratch(tcs, torch_cuda):
    limit = tcs.lib().tcs_noalloc_scratch_bytes()
    assert limit == 32 << 20
    n = 4097  # 257 x 257 bricks x 512 B > 32 MiB
    with pytest.raises(tcs.TcsError) as e:
        tcs.sweep_steps_noalloc(1 << 20, 2 << 20, n, n, "box2d1r", np.full((3, 3), 1 / 9), 3)
    assert e.value.status == tcs.TCS_ERR_INVALID
    assert "static scratch" in str(e.value)

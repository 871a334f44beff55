"""tcs_sweep_steps_noalloc: multi-step sweeps for callers that cannot call
cudaMalloc where they sweep (loops that forbid allocator calls, device memory
owned by a pool or budget the caller does not control).  Its ping-pong plane is
a static device array that every call shares and that keeps the last call's
contents, so these tests make calls in a row, of different shapes, each
compared bit for bit with the plan path (tcs_plan_*, which allocates its own
planes) and with the oracle.  Kept in its own file so it is collected last.
"""
import numpy as np
import pytest

import oracle
from helpers import grid, grid16, normalized_coeffs, plane16

pytestmark = pytest.mark.gpu


def plan_result16(tcs, A, B, stencil, steps, engine):
    p = tcs.Plan(A.shape[0], A.shape[1], stencil, B, engine=engine, precision="f16")
    p.upload(A)
    p.run(steps)
    out = np.empty_like(A)
    p.download(out)
    p.close()
    return oracle.f32_to_f16(out)


def noalloc16(tcs, torch, A16, B, stencil, steps, engine, out_fill=0):
    ny, nx = A16.shape
    d_in = plane16(torch, A16)
    d_out = torch.full_like(d_in, out_fill)
    tcs.sweep_steps_noalloc(d_in, d_out, ny, nx, stencil, B, steps, engine=engine)
    torch.cuda.synchronize()
    assert tcs.device_error() == 0
    np.testing.assert_array_equal(grid16(d_in, ny, nx), A16)  # input untouched
    return grid16(d_out, ny, nx)


def check_against_oracle(got16, A16, B, stencil, steps, engine):
    if engine == "cudacore":
        np.testing.assert_array_equal(got16, oracle.sweep_f16cc(A16, B, stencil, steps))
        return
    # tensor contract: exact FP16 x FP16 products, FP32 sums; within one FP16
    # step of the value per sweep step of the exact-sum oracle
    ref = oracle.f16_to_f32(oracle.sweep_f16tc(A16, B, stencil, steps)).astype(np.float64)
    g = oracle.f16_to_f32(got16).astype(np.float64)
    ulp = 2.0 ** (np.floor(np.log2(max(np.abs(ref).max(), 2.0 ** -14))) - 10)
    assert np.max(np.abs(g - ref)) <= steps * ulp


@pytest.mark.parametrize("engine", ["tensor", "cudacore"])
def test_noalloc_two_calls_match_the_plan_path(tcs, torch_cuda, engine):
    torch = torch_cuda
    rng = np.random.default_rng(77)
    cases = [("box2d2r", (300, 411), 5), ("star2d1r", (257, 190), 4)]
    for stencil, (ny, nx), steps in cases:  # two calls in a row on the shared scratch
        A = grid(rng, ny, nx)
        B = normalized_coeffs(rng, stencil)
        A16 = oracle.f32_to_f16(A)
        got = noalloc16(tcs, torch, A16, B, stencil, steps, engine)
        np.testing.assert_array_equal(got, plan_result16(tcs, A, B, stencil, steps, engine))
        check_against_oracle(got, A16, B, stencil, steps, engine)


def test_noalloc_ignores_what_an_earlier_call_left(tcs, torch_cuda):
    """A call whose fixed border holds inf leaves inf in the shared scratch; a
    later call of another shape, whose padding lies where that border was, and
    whose output plane starts as NaN, still gets the plan path's bits."""
    torch = torch_cuda
    rng = np.random.default_rng(78)
    A = grid(rng, 300, 411)
    A[:2, :] = np.inf
    A[:, -2:] = -np.inf
    B = normalized_coeffs(rng, "box2d2r")
    noalloc16(tcs, torch, oracle.f32_to_f16(A), B, "box2d2r", 3, "tensor")
    nan16 = int(np.float16(np.nan).view(np.int16))
    for stencil, (ny, nx), steps in (("box2d2r", (257, 190), 4), ("box2d1r", (200, 300), 3)):
        A2 = grid(rng, ny, nx)
        B2 = normalized_coeffs(rng, stencil)
        got = noalloc16(tcs, torch, oracle.f32_to_f16(A2), B2, stencil, steps, "tensor",
                        out_fill=nan16)
        assert np.all(np.isfinite(oracle.f16_to_f32(got)))
        np.testing.assert_array_equal(got, plan_result16(tcs, A2, B2, stencil, steps, "tensor"))


def test_noalloc_rejects_grids_beyond_the_static_scratch(tcs, torch_cuda):
    torch = torch_cuda
    limit = tcs.lib().tcs_noalloc_scratch_bytes()
    assert limit == 32 << 20
    # the largest square grid whose FP16 plane fits, and the next size up
    assert tcs.plane_elems(3968, 3968) * 2 <= limit < tcs.plane_elems(3969, 3969) * 2
    B = np.full((3, 3), 1 / 9, np.float32)
    with pytest.raises(tcs.TcsError) as e:
        tcs.sweep_steps_noalloc(1 << 20, 2 << 20, 3969, 3969, "box2d1r", B, 3)
    assert e.value.status == tcs.TCS_ERR_INVALID
    assert "static scratch" in str(e.value)
    # 3968^2 is accepted and gets the plan path's bits
    rng = np.random.default_rng(79)
    A = grid(rng, 3968, 3968)
    B = normalized_coeffs(rng, "box2d1r")
    got = noalloc16(tcs, torch, oracle.f32_to_f16(A), B, "box2d1r", 3, "tensor")
    np.testing.assert_array_equal(got, plan_result16(tcs, A, B, "box2d1r", 3, "tensor"))


def test_noalloc_writes_stay_inside_the_planes(tcs, torch_cuda):
    """Guard regions: canary bytes around the caller's input and output
    planes, and (guard mode) the library's canaries before the shared scratch
    plane and after the part of it each call uses, stay intact over calls of
    growing and shrinking shapes on both engines; the results keep the plan
    path's bits."""
    torch = torch_cuda
    rng = np.random.default_rng(80)
    G = 4096
    tcs.set_guard_bytes(G)
    try:
        cases = [("box2d2r", (300, 411), 5, "tensor"), ("star2d1r", (1030, 130), 4, "tensor"),
                 ("box2d1r", (129, 131), 3, "cudacore"), ("star2d2r", (257, 190), 6, "tensor")]
        for stencil, (ny, nx), steps, engine in cases:
            A = grid(rng, ny, nx)
            B = normalized_coeffs(rng, stencil)
            p16 = plane16(torch, oracle.f32_to_f16(A))
            n = p16.numel() * 2
            bufs = [torch.full((G + n + G,), 0xA5, dtype=torch.uint8, device="cuda") for _ in range(2)]
            bufs[0][G:G + n].copy_(p16.view(torch.uint8))
            tcs.sweep_steps_noalloc(bufs[0].data_ptr() + G, bufs[1].data_ptr() + G, ny, nx, stencil,
                                    B, steps, engine=engine)
            torch.cuda.synchronize()
            assert tcs.device_error() == 0
            for k, b in enumerate(bufs):
                for part in (b[:G], b[G + n:]):
                    assert bool((part == 0xA5).all()), f"caller guard of plane {k}, {stencil} {ny}x{nx}"
            assert tcs.guard_check() == 0, tcs.lib().tcs_last_error().decode()
            out = bufs[1][G:G + n].view(torch.int16)
            np.testing.assert_array_equal(grid16(out, ny, nx),
                                          plan_result16(tcs, A, B, stencil, steps, engine))
    finally:
        tcs.set_guard_bytes(0)

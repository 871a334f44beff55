"""Batched sweeps (tcs_batch_*): every grid of a mixed batch, advanced by one
persistent launch per run, must equal bit for bit the same problem run alone
through a plan (whose parity with the oracle the sweep tests establish)."""
import numpy as np
import pytest

from helpers import RADIUS, grid, normalized_coeffs

pytestmark = pytest.mark.gpu

STENCILS = list(RADIUS)


def _solo(tcs, g0, stencil, coeffs, steps, precision, rect=None, runs=1):
    p = tcs.Plan(*g0.shape, stencil, coeffs, engine="tensor", precision=precision, rect=rect)
    p.upload(g0)
    for _ in range(runs):
        p.run(steps, use_graph=False)
    out = np.empty_like(g0)
    p.download(out)
    p.close()
    return out


def _mixed(rng, count, max_side=400):
    cases = []
    for i in range(count):
        stencil = STENCILS[i % 4]
        precision = "split" if (i // 4) % 2 else "f16"
        r = RADIUS[stencil]
        ny = int(rng.integers(2 * r + 1, max_side))
        nx = int(rng.integers(2 * r + 1, max_side))
        steps = int(rng.integers(0, 7))
        cases.append((stencil, precision, ny, nx, steps))
    return cases


def _run_batch(tcs, torch, cases, rng, runs=1, use_graph=False, rects=None):
    b = tcs.Batch()
    inputs, coeffs = [], []
    for k, (stencil, precision, ny, nx, steps) in enumerate(cases):
        c = normalized_coeffs(rng, stencil)
        rect = rects[k] if rects else None
        assert b.add(ny, nx, stencil, c, steps, precision, rect=rect) == k
        coeffs.append(c)
        inputs.append(grid(rng, ny, nx))
    for k, g0 in enumerate(inputs):
        b.upload(k, g0)
    for _ in range(runs):
        b.run(use_graph=use_graph)
    outs = []
    for k, g0 in enumerate(inputs):
        out = np.empty_like(g0)
        b.download(k, out)
        outs.append(out)
    torch.cuda.synchronize()
    assert tcs.device_error() == 0
    return b, inputs, coeffs, outs


def test_batch_equals_solo_plans(tcs, torch_cuda):
    rng = np.random.default_rng(41)
    cases = [("star2d1r", "f16", 128, 128, 3), ("star2d2r", "f16", 300, 200, 5),
             ("box2d1r", "split", 129, 257, 4), ("box2d2r", "split", 64, 40, 2),
             ("box2d2r", "f16", 517, 333, 1), ("star2d1r", "split", 5, 700, 6),
             ("box2d1r", "f16", 1000, 9, 0), ("star2d2r", "split", 250, 250, 7)]
    b, inputs, coeffs, outs = _run_batch(tcs, torch_cuda, cases, rng)
    pu, items, grids = b.info()
    assert grids == len(cases)
    assert pu == sum((ny - 2 * RADIUS[s]) * (nx - 2 * RADIUS[s]) * t for s, _, ny, nx, t in cases)
    assert items == sum(-(-ny // 128) * -(-nx // 128) * t for _, _, ny, nx, t in cases)
    for (stencil, precision, ny, nx, steps), g0, c, out in zip(cases, inputs, coeffs, outs):
        np.testing.assert_array_equal(out, _solo(tcs, g0, stencil, c, steps, precision),
                                      err_msg=f"{stencil} {precision} {ny}x{nx} {steps}")
    b.close()


def test_batch_rectangles(tcs, torch_cuda):
    rng = np.random.default_rng(42)
    cases = [("box2d2r", "f16", 300, 260, 3), ("star2d1r", "split", 200, 150, 4)]
    rects = [(10, 250, 2, 258), (1, 77, 40, 149)]
    b, inputs, coeffs, outs = _run_batch(tcs, torch_cuda, cases, rng, rects=rects)
    for (stencil, precision, ny, nx, steps), rect, g0, c, out in zip(cases, rects, inputs,
                                                                     coeffs, outs):
        np.testing.assert_array_equal(out, _solo(tcs, g0, stencil, c, steps, precision, rect))
        y0, y1, x0, x1 = rect
        outside = np.ones_like(g0, bool)
        outside[y0:y1, x0:x1] = False
        # cells outside the rectangle keep their (stored) input value
        assert np.all(np.abs(out[outside] - g0[outside]) <= 1e-3 * np.abs(g0[outside]) + 1e-7)
    b.close()


@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_repeated_runs(tcs, torch_cuda, use_graph):
    """Runs chain: three runs of a batch == each grid's plan run 3 x its steps
    (odd and even step counts flip the ping-pong state differently)."""
    rng = np.random.default_rng(43)
    cases = [("box2d2r", "f16", 200, 300, 3), ("star2d2r", "split", 150, 140, 2),
             ("box2d1r", "f16", 260, 90, 1), ("star2d1r", "split", 77, 333, 5)]
    b, inputs, coeffs, outs = _run_batch(tcs, torch_cuda, cases, rng, runs=3,
                                         use_graph=use_graph)
    for (stencil, precision, ny, nx, steps), g0, c, out in zip(cases, inputs, coeffs, outs):
        np.testing.assert_array_equal(out, _solo(tcs, g0, stencil, c, steps, precision, runs=3))
    b.close()


def test_batch_many_mixed_grids(tcs, torch_cuda):
    """More grids than SMs, many steps: exercises the cross-CTA step waits."""
    rng = np.random.default_rng(44)
    cases = _mixed(rng, 240)
    b, inputs, coeffs, outs = _run_batch(tcs, torch_cuda, cases, rng, use_graph=True)
    for (stencil, precision, ny, nx, steps), g0, c, out in zip(cases, inputs, coeffs, outs):
        np.testing.assert_array_equal(out, _solo(tcs, g0, stencil, c, steps, precision),
                                      err_msg=f"{stencil} {precision} {ny}x{nx} {steps}")
    b.close()


def test_batch_one_large_grid_many_steps(tcs, torch_cuda):
    """A single grid whose every step spans all SMs: step t waits on step t-1
    across the whole GPU, 20 times in one launch."""
    rng = np.random.default_rng(45)
    cases = [("box2d2r", "f16", 2048, 1536, 20)]
    _, inputs, coeffs, outs = _run_batch(tcs, torch_cuda, cases, rng)
    np.testing.assert_array_equal(outs[0], _solo(tcs, inputs[0], "box2d2r", coeffs[0], 20, "f16"))


def test_batch_device_buffers(tcs, torch_cuda):
    torch = torch_cuda
    rng = np.random.default_rng(46)
    c = normalized_coeffs(rng, "star2d2r")
    g0 = grid(rng, 190, 210)
    b = tcs.Batch()
    b.add(190, 210, "star2d2r", c, 4, "split")
    d_in = torch.from_numpy(g0).cuda()
    d_out = torch.empty_like(d_in)
    b.upload(0, d_in)
    b.run()
    b.download(0, d_out)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d_out.cpu().numpy(), _solo(tcs, g0, "star2d2r", c, 4, "split"))
    b.close()


def _gated_batch(tcs, rng, flag, limit=None):
    """A gated FP16 grid and an ungated one (same launch) plus an ungated split
    grid (its own launch)."""
    cases = [("box2d1r", "f16", 300, 260, 3), ("star2d2r", "f16", 180, 210, 2),
             ("box2d2r", "split", 200, 140, 2)]
    b = tcs.Batch()
    inputs, coeffs = [], []
    for k, (stencil, precision, ny, nx, steps) in enumerate(cases):
        c = normalized_coeffs(rng, stencil)
        b.add(ny, nx, stencil, c, steps, precision)
        coeffs.append(c)
        inputs.append(grid(rng, ny, nx))
    b.set_gate(0, flag, 1)
    if limit is not None:
        b.set_wait_limit(limit)
    for k, g0 in enumerate(inputs):
        b.upload(k, g0)
    return b, cases, inputs, coeffs


def test_gate_that_never_opens_times_out_cleanly(tcs, torch_cuda):
    """A bounded wait runs out on a flag nothing sets: the launch stops, the
    host reads TCS_ERR_TIMEOUT with the dependency-wait code 6, the split
    launch after it is unaffected, and the context stays usable."""
    torch = torch_cuda
    rng = np.random.default_rng(47)
    flag = torch.zeros(4, dtype=torch.int32, device="cuda")
    b, cases, inputs, coeffs = _gated_batch(tcs, rng, flag, limit=0.05)
    b.run(use_graph=False)
    torch.cuda.synchronize()
    with pytest.raises(tcs.TcsError) as e:
        tcs.device_error()
    assert e.value.status == tcs.TCS_ERR_TIMEOUT and "code 6" in str(e.value)
    assert tcs.device_error() == 0  # the word was cleared
    out = np.empty_like(inputs[2])
    b.download(2, out)
    stencil, precision, _, _, steps = cases[2]
    np.testing.assert_array_equal(out, _solo(tcs, inputs[2], stencil, coeffs[2], steps, precision))
    b.close()
    # the same batch with its gate open runs to the plans' results
    flag.fill_(1)
    b, cases, inputs, coeffs = _gated_batch(tcs, np.random.default_rng(47), flag, limit=0.05)
    b.run(use_graph=True)
    for k, (stencil, precision, _, _, steps) in enumerate(cases):
        out = np.empty_like(inputs[k])
        b.download(k, out)
        np.testing.assert_array_equal(out, _solo(tcs, inputs[k], stencil, coeffs[k], steps, precision))
    torch.cuda.synchronize()
    assert tcs.device_error() == 0
    b.close()


def test_gate_opened_by_a_copy_on_another_stream(tcs, torch_cuda):
    """The batch waits in the kernel for a word another stream writes (a copy
    engine transfer, no kernel), then runs to the plans' results."""
    import time

    torch = torch_cuda
    rng = np.random.default_rng(48)
    flag = torch.zeros(4, dtype=torch.int32, device="cuda")
    one = torch.ones(4, dtype=torch.int32).pin_memory()
    b, cases, inputs, coeffs = _gated_batch(tcs, rng, flag)
    torch.cuda.synchronize()
    s_run, s_copy = torch.cuda.Stream(), torch.cuda.Stream()
    b.run(use_graph=False, stream=s_run)
    time.sleep(0.02)
    with torch.cuda.stream(s_copy):
        flag.copy_(one, non_blocking=True)
    torch.cuda.synchronize()
    assert tcs.device_error() == 0
    for k, (stencil, precision, _, _, steps) in enumerate(cases):
        out = np.empty_like(inputs[k])
        b.download(k, out)
        np.testing.assert_array_equal(out, _solo(tcs, inputs[k], stencil, coeffs[k], steps, precision))
    b.close()

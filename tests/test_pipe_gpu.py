"""Double-buffered host pipeline (tcs_pipe_*): every submission's result is
the same bits as the one-call form (tcs_sweep_host) for that grid, with the
two slots' submissions overlapping on the device."""
import numpy as np
import pytest

from helpers import grid, normalized_coeffs

pytestmark = pytest.mark.gpu


def _pinned(torch, a):
    t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    return t, t.numpy()


@pytest.mark.parametrize("stencil,precision", [("box2d2r", "f16"), ("star2d1r", "split"),
                                               ("box2d1r", "split")])
def test_pipe_matches_the_one_call_form(tcs, torch_cuda, stencil, precision):
    torch = torch_cuda
    rng = np.random.default_rng(91)
    ny, nx, steps = 300, 260, 7
    c = normalized_coeffs(rng, stencil)
    keep = []
    ins, outs = [], []
    for k in range(5):
        a = grid(rng, ny, nx, -1.0 - k, 1.0 + 2 * k)  # a different scale per grid
        ti, hi = _pinned(torch, a)
        to, ho = _pinned(torch, np.zeros((ny, nx), np.float32))
        keep += [ti, to]
        ins.append(hi)
        outs.append(ho)
    pipe = tcs.Pipe(ny, nx, stencil, c, precision=precision)
    for hi, ho in zip(ins, outs):
        pipe.submit(hi, ho, steps)
    pipe.wait()
    pipe.close()
    for hi, ho in zip(ins, outs):
        expect = tcs.sweep_host(hi.copy(), steps, stencil, c, precision=precision)
        np.testing.assert_array_equal(ho, expect)


def test_pipe_slot_reuse_keeps_results(tcs, torch_cuda):
    """Submission k's output is final once submission k + 2 has been submitted."""
    torch = torch_cuda
    rng = np.random.default_rng(92)
    c = normalized_coeffs(rng, "box2d1r")
    _, h0 = _pinned(torch, grid(rng, 140, 150))
    _, h1 = _pinned(torch, grid(rng, 140, 150))
    _, o0 = _pinned(torch, np.zeros((140, 150), np.float32))
    _, o1 = _pinned(torch, np.zeros((140, 150), np.float32))
    _, o2 = _pinned(torch, np.zeros((140, 150), np.float32))
    pipe = tcs.Pipe(140, 150, "box2d1r", c)
    pipe.submit(h0, o0, 3)
    pipe.submit(h1, o1, 3)
    pipe.submit(h0, o2, 5)  # reuses slot 0: submission 0 is complete
    np.testing.assert_array_equal(o0, tcs.sweep_host(h0.copy(), 3, "box2d1r", c))
    pipe.wait()
    np.testing.assert_array_equal(o1, tcs.sweep_host(h1.copy(), 3, "box2d1r", c))
    np.testing.assert_array_equal(o2, tcs.sweep_host(h0.copy(), 5, "box2d1r", c))
    pipe.close()

"""Temporally blocked split sweeps (two steps per launch): bit-identical to
single steps.  Plans at temporal depth 2 run steps in blocked pairs; the
batched kernel runs single steps, so the two must agree bit for bit on every
shape, edge and rectangle."""
import numpy as np
import pytest

from helpers import RADIUS, grid, normalized_coeffs

pytestmark = pytest.mark.gpu


def _single_steps(tcs, g0, stencil, c, steps, rect=None):
    b = tcs.Batch()
    b.add(*g0.shape, stencil, c, steps, "split", rect=rect)
    b.upload(0, g0)
    b.run(use_graph=False)
    out = np.empty_like(g0)
    b.download(0, out)
    b.close()
    return out


def _plan(tcs, g0, stencil, c, steps, rect=None, use_graph=False):
    p = tcs.Plan(*g0.shape, stencil, c, engine="tensor", precision="split", rect=rect,
                 temporal_depth=2)
    p.upload(g0)
    p.run(steps, use_graph=use_graph)
    out = np.empty_like(g0)
    p.download(out)
    p.close()
    return out


@pytest.mark.parametrize("stencil", list(RADIUS))
@pytest.mark.parametrize("shape", [(300, 200), (130, 97), (128, 96), (777, 1000), (9, 400)])
def test_blocked_pairs_equal_single_steps(tcs, torch_cuda, stencil, shape):
    rng = np.random.default_rng(1000 * shape[0] + shape[1] + list(RADIUS).index(stencil))
    c = normalized_coeffs(rng, stencil)
    g0 = grid(rng, *shape)
    for steps in (2, 5):
        np.testing.assert_array_equal(_plan(tcs, g0, stencil, c, steps),
                                      _single_steps(tcs, g0, stencil, c, steps),
                                      err_msg=f"{stencil} {shape} {steps}")
    assert tcs.device_error() == 0


@pytest.mark.parametrize("use_graph", [False, True])
def test_blocked_pairs_with_rectangles_and_graphs(tcs, torch_cuda, use_graph):
    rng = np.random.default_rng(71)
    for stencil, shape, rect in [("box2d2r", (400, 350), (7, 390, 2, 300)),
                                 ("star2d1r", (260, 513), (1, 259, 100, 512)),
                                 ("box2d1r", (1030, 770), (300, 700, 96, 200))]:
        c = normalized_coeffs(rng, stencil)
        g0 = grid(rng, *shape)
        for steps in (4, 7):
            np.testing.assert_array_equal(
                _plan(tcs, g0, stencil, c, steps, rect, use_graph),
                _single_steps(tcs, g0, stencil, c, steps, rect),
                err_msg=f"{stencil} {shape} {rect} {steps}")
    assert tcs.device_error() == 0

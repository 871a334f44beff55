"""Request server (tcs_server_*): continuous batching must not change results.
Every served solve equals, bit for bit, the same problem run alone through a
plan (tensor engine), whatever it was batched with, however it was split into
rounds, and however long it waited for memory."""
import numpy as np
import pytest

from helpers import grid, normalized_coeffs
from tcstencil_gb300.workloads import poisson_requests

pytestmark = pytest.mark.gpu


def _alone(tcs, g0, stencil, coeffs, steps, precision):
    p = tcs.Plan(*g0.shape, stencil, coeffs, engine="tensor", precision=precision)
    p.upload(g0)
    p.run(steps, use_graph=False)
    out = np.empty_like(g0)
    p.download(out)
    p.close()
    return out


def _check_all_alone(tcs, cases):
    for (stencil, precision, steps, c, g0, out) in cases:
        np.testing.assert_array_equal(out, _alone(tcs, g0, stencil, c, steps, precision),
                                      err_msg=f"{stencil} {precision} {g0.shape} {steps}")


def test_served_results_equal_alone(tcs, torch_cuda):
    """Poisson arrivals (4k req/s, small grids, 0-30 steps, mixed stencils and
    precisions): requests overlap on the device and share rounds."""
    from tcstencil_gb300.serving import InputPool, replay

    reqs = poisson_requests(rate=4000.0, duration=0.03, side=(40, 400), steps=(0, 30),
                            max_requests=100)
    assert len(reqs) >= 60
    srv = tcs.Server(1 << 30)
    res = replay(srv, reqs, InputPool(1 << 20), keep_outputs=True)
    st = srv.stats()
    srv.close()
    assert res["failed"] == 0 and st["completed"] == len(reqs)
    assert st["rounds"] < len(reqs)  # requests were folded into shared launches
    cases = []
    for rq in reqs:
        g0, out = res["outputs"][rq.rid]
        sp = rq.spec
        cases.append((sp.stencil, sp.precision, sp.steps, sp.coeffs, np.array(g0), out))
    _check_all_alone(tcs, cases)
    assert tcs.device_error() == 0


@pytest.mark.parametrize("round_steps", [1, 3])
def test_rounds_split_long_requests(tcs, torch_cuda, round_steps):
    rng = np.random.default_rng(50 + round_steps)
    srv = tcs.Server(1 << 28, round_steps=round_steps)
    cases, tickets = [], []
    for i, (stencil, precision, ny, nx, steps) in enumerate(
            [("box2d2r", "f16", 300, 200, 10), ("star2d1r", "split", 129, 517, 7),
             ("box2d1r", "split", 256, 256, 1), ("star2d2r", "f16", 90, 700, 5)]):
        c = normalized_coeffs(rng, stencil)
        g0 = grid(rng, ny, nx)
        out = np.empty_like(g0)
        tickets.append(srv.submit(g0, out, stencil, c, steps, precision))
        cases.append((stencil, precision, steps, c, g0, out))
    for t in tickets:
        srv.wait(t, timeout=30.0)
    st = srv.stats()
    srv.close()
    assert st["completed"] == 4 and st["failed"] == 0
    assert st["rounds"] >= -(-10 // round_steps)
    _check_all_alone(tcs, cases)


def test_admission_waits_for_budget(tcs, torch_cuda):
    """A budget that holds two requests at a time: the rest queue until memory
    frees up, the held memory never exceeds the budget, and every result
    still equals its solve alone."""
    rng = np.random.default_rng(60)
    ny = nx = 384
    # state of one FP16 request: 4 panel planes of (384+8) rows x (384+16) cells x 2 B,
    # plus its FP32 staging grid
    one = 4 * (392 * 400 * 2) + 384 * 384 * 4
    budget = 2 * one + 4096
    stencils = ["star2d1r", "box2d2r"]
    inputs = [(stencils[i % 2], normalized_coeffs(rng, stencils[i % 2]), grid(rng, ny, nx), 20 + i)
              for i in range(8)]
    srv = tcs.Server(budget)
    cases, tickets = [], []
    for stencil, c, g0, steps in inputs:
        out = np.empty_like(g0)
        tickets.append(srv.submit(g0, out, stencil, c, steps, "f16"))
        cases.append((stencil, "f16", steps, c, g0, out))
    for t in tickets:
        srv.wait(t, timeout=30.0)
    st = srv.stats()
    srv.close()
    assert st["completed"] == 8 and st["failed"] == 0
    assert one <= st["peak_bytes_in_use"] <= budget
    _check_all_alone(tcs, cases)


def test_oversized_request_is_rejected(tcs, torch_cuda):
    srv = tcs.Server(1 << 20)
    g0 = np.zeros((1024, 1024), np.float32)
    with pytest.raises(tcs.TcsError) as e:
        srv.submit(g0, np.empty_like(g0), "box2d1r", np.full((3, 3), 1 / 9, np.float32), 1)
    assert e.value.status == tcs.TCS_ERR_NOMEM
    srv.close()

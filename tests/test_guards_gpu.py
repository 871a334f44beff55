"""Bounds and failure checks without a sanitizer or a device fault.

* Guard regions: with tcs_set_guard_bytes every device allocation of the
  library carries canary bytes before and after it, batches and the server
  put canaries between the planes of their pools and around each request,
  and tcs_guard_check reports any that changed.  Plans of every engine and
  precision, batches and the server run on ragged sizes (partial tiles in
  both directions, sizes off every multiple of 8, 16 and 128) and the guards
  must be intact after each.  A positive control writes one byte into a
  plane's trailing guard from the host and the check must see it.
* Allocation failure: a hook fails the k-th allocation of plan, batch,
  drift and server set-up for every k in turn; each call fails with
  TCS_ERR_NOMEM naming the allocation and leaves no live allocation behind,
  and the library works again once the hook is removed.  A server whose
  round buffers cannot grow fails that request with TCS_ERR_NOMEM and goes
  on serving.
* Cancellation: queued and resident server requests end with
  TCS_ERR_CANCELLED, their output untouched and their memory returned, while
  the other requests complete with their plan-path bits; a wait with a
  timeout followed by a cancel gives a deadline.
"""
import ctypes
import ctypes.util
import time

import numpy as np
import pytest

from helpers import grid, normalized_coeffs

pytestmark = pytest.mark.gpu

RAGGED = [(37, 250), (129, 131), (300, 411), (257, 190), (130, 1030)]
GUARD = 4096


@pytest.fixture
def guards(tcs, torch_cuda):
    tcs.set_guard_bytes(GUARD)
    try:
        yield tcs
    finally:
        tcs.set_guard_bytes(0)


def plan_bits(tcs, A, B, stencil, steps, engine="tensor", precision="f16", **kw):
    p = tcs.Plan(A.shape[0], A.shape[1], stencil, B, engine=engine, precision=precision, **kw)
    p.upload(A)
    p.run(steps)
    out = np.empty_like(A)
    p.download(out)
    p.close()
    return out


def assert_guards_intact(tcs, what):
    n = tcs.guard_check()
    assert n == 0, f"{what}: {n} damaged guard regions ({tcs.lib().tcs_last_error().decode()})"


def test_plan_guards_intact_on_ragged_sizes(guards):
    tcs = guards
    rng = np.random.default_rng(900)
    forms = [("tensor", "f16", {}), ("tensor", "f16", {"tile_w": 64}), ("cudacore", "f16", {}),
             ("cudacore", "f32", {}), ("tensor", "split", {}),
             ("tensor", "split", {"temporal_depth": 2})]
    for (ny, nx) in RAGGED:
        for stencil in ("star2d1r", "box2d2r"):
            A = grid(rng, ny, nx)
            B = normalized_coeffs(rng, stencil)
            for engine, precision, kw in forms:
                plan_bits(tcs, A, B, stencil, 5, engine, precision, **kw)
                assert_guards_intact(tcs, f"{engine}/{precision}/{kw} {stencil} {ny}x{nx}")
    # several steps in one launch, at more tiles than SMs
    A = grid(rng, 2100, 1900)
    for precision in ("f16", "split"):
        p = tcs.Plan(2100, 1900, "box2d1r", normalized_coeffs(rng, "box2d1r"), precision=precision)
        p.set_multistep(1)
        p.upload(A)
        p.run(6)
        p.close()
        assert_guards_intact(tcs, f"multi-step {precision}")


def test_guard_check_sees_a_write_past_a_plane(guards):
    """Positive control: one byte written from the host into the trailing
    guard of a plan's plane (memory of the allocation itself, so nothing is
    out of bounds for the device) is reported."""
    tcs = guards
    path = ctypes.util.find_library("cudart") or "/usr/local/cuda/lib64/libcudart.so"
    try:
        rt = ctypes.CDLL(path)
    except OSError:
        pytest.skip("no CUDA runtime library to write the byte with")
    rt.cudaMemset.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t]
    rt.cudaDeviceSynchronize.argtypes = []
    rng = np.random.default_rng(901)
    A = grid(rng, 129, 131)
    p = tcs.Plan(129, 131, "box2d1r", normalized_coeffs(rng, "box2d1r"))
    p.upload(A)
    p.run(2)
    assert_guards_intact(tcs, "before the write")
    hi, _, nbytes = p.state()
    assert rt.cudaMemset(ctypes.c_void_p(hi + nbytes + 17), 0x3C, 1) == 0
    assert rt.cudaDeviceSynchronize() == 0
    assert tcs.guard_check() == 1
    assert "plane" in tcs.lib().tcs_last_error().decode()
    # put the canary back, so the plane frees cleanly
    assert rt.cudaMemset(ctypes.c_void_p(hi + nbytes + 17), 0xA5, 1) == 0
    p.close()
    assert tcs.guard_check() == 0


def test_batch_and_server_guards_intact_on_ragged_sizes(guards):
    tcs = guards
    rng = np.random.default_rng(902)
    cases = []
    for k, (ny, nx) in enumerate(RAGGED):
        stencil = ("star2d1r", "star2d2r", "box2d1r", "box2d2r")[k % 4]
        for precision in ("f16", "split"):
            cases.append((grid(rng, ny, nx), normalized_coeffs(rng, stencil), stencil,
                          7 + 3 * k, precision))
    b = tcs.Batch()
    for A, B, st, steps, prec in cases:
        b.add(A.shape[0], A.shape[1], st, B, steps, prec)
    for k, (A, *_rest) in enumerate(cases):
        b.upload(k, A)
    b.run()
    b.run(use_graph=False)
    for k, (A, B, st, steps, prec) in enumerate(cases):
        got = np.empty_like(A)
        b.download(k, got)
        assert np.all(np.isfinite(got))
    assert_guards_intact(tcs, "batch")
    b.close()
    assert_guards_intact(tcs, "batch, after its memory was freed")

    srv = tcs.Server(256 << 20, round_steps=4)
    outs = [np.full_like(A, np.nan) for A, *_ in cases]
    tickets = [srv.submit(A, o, st, B, steps, prec) for (A, B, st, steps, prec), o in zip(cases, outs)]
    for t in tickets:
        srv.wait(t, 60.0)
    assert_guards_intact(tcs, "server, requests retired")
    srv.close()
    for (A, B, st, steps, prec), o in zip(cases, outs):
        np.testing.assert_array_equal(o, plan_bits(tcs, A, B, st, steps, "tensor", prec))
    assert_guards_intact(tcs, "server, closed")


# ------------------------------------------------------------ allocation hook


class FailNth:
    """Fails the n-th allocation (0-based) from now on, counting all of them."""

    def __init__(self, n, only=None):
        self.n, self.only, self.seen, self.failed = n, only, 0, None

    def __call__(self, nbytes, what):
        if self.only and what != self.only:
            return False
        k = self.seen
        self.seen += 1
        if k == self.n:
            self.failed = what
            return True
        return False


def sweep_every_failure_point(tcs, action):
    """Runs action() with the k-th allocation failing, k = 0, 1, ..., until it
    succeeds: each failure is TCS_ERR_NOMEM naming the allocation, and no
    allocation stays live once the objects it made are closed."""
    base = tcs.alloc_stats()
    k = 0
    while True:
        hook = FailNth(k)
        tcs.set_alloc_hook(hook)
        objs = []
        try:
            action(objs)
            ok = True
        except tcs.TcsError as e:
            ok = False
            assert e.status == tcs.TCS_ERR_NOMEM, str(e)
            assert hook.failed and hook.failed in str(e), (hook.failed, str(e))
        finally:
            tcs.set_alloc_hook(None)
            for o in objs:
                o.close()
        assert tcs.alloc_stats() == base, (k, hook.failed)
        if ok:
            assert hook.failed is None
            return k
        k += 1
        assert k < 64


def test_allocation_failures_free_what_was_allocated(tcs, torch_cuda):
    rng = np.random.default_rng(903)
    A = grid(rng, 300, 411)
    for stencil, engine, precision in (("box2d2r", "tensor", "f16"), ("star2d1r", "tensor", "split"),
                                       ("star2d2r", "cudacore", "f32")):
        B = normalized_coeffs(rng, stencil)

        def plan(objs):
            p = tcs.Plan(300, 411, stencil, B, engine=engine, precision=precision)
            objs.append(p)
            p.upload(A)
            p.run(3)
            out = np.empty_like(A)
            p.download(out)

        n = sweep_every_failure_point(tcs, plan)
        assert n >= 3  # planes and more: every one of them was made to fail
        np.testing.assert_array_equal(plan_bits(tcs, A, B, stencil, 3, engine, precision),
                                      plan_bits(tcs, A, B, stencil, 3, engine, precision))

    def batch(objs):
        b = tcs.Batch()
        objs.append(b)
        b.add(300, 411, "box2d1r", normalized_coeffs(rng, "box2d1r"), 4, "f16")
        b.add(129, 131, "star2d2r", normalized_coeffs(rng, "star2d2r"), 5, "split")
        b.upload(0, A)
        b.upload(1, grid(rng, 129, 131))
        b.run()

    assert sweep_every_failure_point(tcs, batch) >= 5

    def drift(objs):
        d = tcs.Drift(300, 411, "box2d2r", normalized_coeffs(rng, "box2d2r"))
        objs.append(d)
        d.upload(A)
        d.run(2)

    assert sweep_every_failure_point(tcs, drift) >= 2

    def server(objs):
        s = tcs.Server(64 << 20, max_active=8, round_steps=4)
        objs.append(s)

    assert sweep_every_failure_point(tcs, server) >= 8


def test_server_request_fails_when_its_round_cannot_grow(tcs, torch_cuda):
    """A request whose round needs larger round buffers (thousands of steps
    in one round) fails with TCS_ERR_NOMEM when the hook refuses them; the
    server goes on serving."""
    rng = np.random.default_rng(904)
    srv = tcs.Server(64 << 20, max_active=4, round_steps=0)
    A = grid(rng, 64, 70)
    B = normalized_coeffs(rng, "box2d1r")
    hook = FailNth(0, only="round")
    tcs.set_alloc_hook(hook)
    try:
        out = np.full_like(A, np.nan)
        t = srv.submit(A, out, "box2d1r", B, 3000, "f16")
        with pytest.raises(tcs.TcsError) as e:
            srv.wait(t, 60.0)
        assert e.value.status == tcs.TCS_ERR_NOMEM
        assert hook.failed == "round"
        assert np.all(np.isnan(out))
    finally:
        tcs.set_alloc_hook(None)
    out2 = np.empty_like(A)
    srv.wait(srv.submit(A, out2, "box2d1r", B, 3000, "f16"), 60.0)
    np.testing.assert_array_equal(out2, plan_bits(tcs, A, B, "box2d1r", 3000))
    assert srv.stats()["failed"] == 1
    srv.close()


# --------------------------------------------------------------- cancellation


def wait_state(srv, t, want, limit=20.0):
    t0 = time.time()
    while time.time() - t0 < limit:
        st, _ = srv.poll(t)
        if st in want:
            return st
        time.sleep(0.0005)
    raise AssertionError(f"ticket {t} never reached {want}")


def test_server_cancels_queued_and_resident_requests(tcs, torch_cuda):
    rng = np.random.default_rng(905)
    B = normalized_coeffs(rng, "box2d2r")
    srv = tcs.Server(256 << 20, max_active=1, round_steps=8)
    base = srv.stats()
    # a long request holds the only slot; the next two wait in the queue
    L = grid(rng, 512, 512)
    out_l = np.full_like(L, np.nan)
    t_long = srv.submit(L, out_l, "box2d2r", B, 200000, "f16")
    wait_state(srv, t_long, (1,))
    Q1, Q2 = grid(rng, 200, 300), grid(rng, 130, 131)
    out_q1, out_q2 = np.full_like(Q1, np.nan), np.full_like(Q2, np.nan)
    t_q1 = srv.submit(Q1, out_q1, "box2d2r", B, 9, "split")
    t_q2 = srv.submit(Q2, out_q2, "box2d2r", B, 11, "f16")
    assert srv.poll(t_q1)[0] == 0 and srv.poll(t_q2)[0] == 0
    # queued: dropped at once
    srv.cancel(t_q1)
    assert srv.poll(t_q1) == (3, tcs.TCS_ERR_CANCELLED)
    with pytest.raises(tcs.TcsError) as e:
        srv.wait(t_q1, 5.0)
    assert e.value.status == tcs.TCS_ERR_CANCELLED
    # resident: retired after its current round
    assert srv.poll(t_long)[0] == 1
    srv.cancel(t_long)
    with pytest.raises(tcs.TcsError) as e:
        srv.wait(t_long, 30.0)
    assert e.value.status == tcs.TCS_ERR_CANCELLED
    with pytest.raises(tcs.TcsError):  # twice: already cancelled
        srv.cancel(t_long)
    # the slot is free again: the queued request runs, with the plan's bits
    srv.wait(t_q2, 60.0)
    np.testing.assert_array_equal(out_q2, plan_bits(tcs, Q2, B, "box2d2r", 11))
    with pytest.raises(tcs.TcsError):  # done: nothing to cancel
        srv.cancel(t_q2)
    assert np.all(np.isnan(out_q1)) and np.all(np.isnan(out_l))
    s = srv.stats()
    assert s["cancelled"] - base["cancelled"] == 2 and s["active"] == 0 and s["queued"] == 0
    assert s["completed"] - base["completed"] == 1
    srv.close()


def test_server_deadline_by_wait_and_cancel(tcs, torch_cuda):
    rng = np.random.default_rng(906)
    B = normalized_coeffs(rng, "star2d1r")
    srv = tcs.Server(128 << 20, round_steps=4)
    A = grid(rng, 400, 400)
    out = np.full_like(A, np.nan)
    t = srv.submit(A, out, "star2d1r", B, 400000, "split")
    with pytest.raises(tcs.TcsError) as e:
        srv.wait(t, 0.05)
    assert e.value.status == tcs.TCS_ERR_TIMEOUT
    srv.cancel(t)
    with pytest.raises(tcs.TcsError) as e:
        srv.wait(t, 30.0)
    assert e.value.status == tcs.TCS_ERR_CANCELLED
    assert np.all(np.isnan(out))
    # other work still runs and matches the plan path
    C = grid(rng, 131, 257)
    out_c = np.empty_like(C)
    srv.wait(srv.submit(C, out_c, "star2d1r", B, 13, "split"), 60.0)
    np.testing.assert_array_equal(out_c, plan_bits(tcs, C, B, "star2d1r", 13, "tensor", "split"))
    srv.close()


def test_server_cancels_under_load(tcs, torch_cuda):
    """Cancels racing admission, rounds and downloads: every third of 45
    mixed requests is cancelled right after submission. A cancel either
    succeeds (the ticket ends cancelled, its output untouched) or is refused
    because the request is already finishing (it then completes); every
    other request keeps its plan-path bits, and the server ends idle."""
    rng = np.random.default_rng(907)
    srv = tcs.Server(256 << 20, max_active=6, round_steps=4)
    base = srv.stats()
    reqs = []
    for k in range(45):
        st = ("star2d1r", "star2d2r", "box2d1r", "box2d2r")[k % 4]
        prec = "split" if k % 3 == 1 else "f16"
        A = grid(rng, int(rng.integers(64, 400)), int(rng.integers(64, 400)))
        B = normalized_coeffs(rng, st)
        steps = int(rng.integers(5, 60))
        out = np.full_like(A, np.nan)
        reqs.append((A, B, st, steps, prec, out, srv.submit(A, out, st, B, steps, prec)))
    cancelled = set()
    for k, r in enumerate(reqs):
        if k % 3 == 0:
            try:
                srv.cancel(r[6])
                cancelled.add(k)
            except tcs.TcsError as e:
                assert e.status == tcs.TCS_ERR_INVALID
    for k, (A, B, st, steps, prec, out, t) in enumerate(reqs):
        if k in cancelled:
            with pytest.raises(tcs.TcsError) as e:
                srv.wait(t, 60.0)
            assert e.value.status == tcs.TCS_ERR_CANCELLED
            assert np.all(np.isnan(out))
        else:
            srv.wait(t, 60.0)
            np.testing.assert_array_equal(out, plan_bits(tcs, A, B, st, steps, "tensor", prec),
                                          err_msg=f"request {k}")
    s = srv.stats()
    assert s["cancelled"] - base["cancelled"] == len(cancelled)
    assert s["completed"] - base["completed"] == len(reqs) - len(cancelled)
    assert s["active"] == 0 and s["queued"] == 0
    srv.close()
    assert tcs.device_error() == 0

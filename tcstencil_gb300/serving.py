"""Open-loop load generator for the request server: replays timed arrivals
(e.g. workloads.poisson_requests) against a tcstencil_gb300.Server and reports
latency percentiles and aggregate throughput.

Inputs are slices of one seeded pinned buffer (each request reads ny*nx
consecutive floats at a seeded offset); outputs go to a pinned ring arena, so
a run of tens of thousands of requests holds a bounded amount of host memory.
"""
from __future__ import annotations

import time
from collections import deque

import numpy as np

from .workloads import Request


def pinned_empty(n: int) -> np.ndarray:
    import torch

    return torch.empty(n, dtype=torch.float32).pin_memory().numpy()


class InputPool:
    """`n` seeded U[-1,1) floats in pinned memory; request grids are views."""

    def __init__(self, n: int, seed: int = 5000):
        self.buf = pinned_empty(n)
        rng = np.random.default_rng(seed)
        chunk = 1 << 24
        for i in range(0, n, chunk):
            m = min(chunk, n - i)
            self.buf[i:i + m] = rng.uniform(-1.0, 1.0, m).astype(np.float32)

    def grid(self, ny: int, nx: int, seed: int) -> np.ndarray:
        n = ny * nx
        off = int(np.random.default_rng(seed).integers(0, len(self.buf) - n + 1))
        return self.buf[off:off + n].reshape(ny, nx)


class OutputRing:
    """Pinned arena handed out first-in first-out."""

    def __init__(self, n: int):
        self.buf = pinned_empty(n)
        self.head = 0
        self.live = deque()  # (ticket, start, end)

    def take(self, ny: int, nx: int, wait_oldest):
        """A ny x nx view; waits for the oldest tickets whose outputs it would
        overwrite.  Returns (view, start, end)."""
        n = ny * nx
        if n > len(self.buf):
            raise ValueError("request larger than the output arena")
        start = self.head if self.head + n <= len(self.buf) else 0
        end = start + n
        while self.live and any(s < end and start < e for _, s, e in self.live):
            t, _, _ = self.live.popleft()
            wait_oldest(t)
        self.head = end
        return self.buf[start:end].reshape(ny, nx), start, end

    def hold(self, ticket: int, start: int, end: int) -> None:
        self.live.append((ticket, start, end))


def replay(server, requests: list[Request], inputs: InputPool, outputs: OutputRing | None = None,
           keep_outputs: bool = False, spin_s: float = 2e-4, timeout_s: float = 120.0) -> dict:
    """Submits every request at its arrival time on the server clock (open
    loop), waits for all, and returns per-request latencies (completion minus
    scheduled arrival, seconds) with p50/p99 and aggregate Gpts/s."""
    base = server.clock() + 0.05
    tickets, kept, lag = [], {}, []
    for rq in requests:
        target = base + rq.arrival
        while True:
            now = server.clock()
            if now >= target:
                break
            if target - now > spin_s:
                time.sleep(target - now - spin_s)
        sp = rq.spec
        g = inputs.grid(sp.ny, sp.nx, sp.seed)
        if keep_outputs:
            out = np.empty((sp.ny, sp.nx), np.float32)
            t = server.submit(g, out, sp.stencil, sp.coeffs, sp.steps, sp.precision)
            kept[rq.rid] = (g, out)
        else:
            out, s0, e0 = outputs.take(sp.ny, sp.nx, lambda t: server.wait(t, timeout_s))
            t = server.submit(g, out, sp.stencil, sp.coeffs, sp.steps, sp.precision)
            outputs.hold(t, s0, e0)
        lag.append(server.clock() - target)
        tickets.append((t, target, rq))
    for t, _, _ in tickets:
        server.wait(t, timeout_s)
    lat, queue_wait, updates = [], [], 0
    first = tickets[0][1] if tickets else 0.0
    last_done = first
    for t, target, rq in tickets:
        sub, adm, done = server.times(t)
        lat.append(done - target)
        queue_wait.append(adm - sub)
        last_done = max(last_done, done)
        updates += rq.spec.updates
    lat = np.array(lat)
    span = max(last_done - first, 1e-9)
    st = server.stats()
    res = {
        "requests": len(tickets),
        "p50_ms": float(np.percentile(lat, 50) * 1e3) if len(lat) else None,
        "p99_ms": float(np.percentile(lat, 99) * 1e3) if len(lat) else None,
        "mean_ms": float(lat.mean() * 1e3) if len(lat) else None,
        "max_ms": float(lat.max() * 1e3) if len(lat) else None,
        "admission_wait_p99_ms": float(np.percentile(queue_wait, 99) * 1e3) if queue_wait else None,
        "submit_lag_p99_ms": float(np.percentile(lag, 99) * 1e3) if lag else None,
        "point_updates": updates,
        "span_s": span,
        "gpts": updates / span / 1e9,
        "gpu_busy_frac": st["gpu_busy_s"] / span,
        "rounds": st["rounds"],
        "peak_bytes_in_use": st["peak_bytes_in_use"],
        "failed": st["failed"],
        "sched_max_ms": [round(v * 1e3, 3) for v in st["sched_max_s"]],
        "sched_total_s": [round(v, 3) for v in st["sched_total_s"]],
        "launch_max_ms": [round(v * 1e3, 3) for v in st["launch_max_s"]],
        "launch_total_s": [round(v, 3) for v in st["launch_total_s"]],
    }
    if keep_outputs:
        res["outputs"] = kept
    return res

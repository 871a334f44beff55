"""bench.py's multi-GPU host logic on CPU: `gloo` ranks, world size 2.

On GPUs the sweep runs as replicas, one process per GPU on its own grids, with
no data exchange. What the ranks share is host logic: their rank from
torchrun's environment, a seed per replica, the timing reduction (the slowest
rank's time sets the whole-job rate) and rank 0 alone printing, including the
CPU reference arm."""
import json
import multiprocessing
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, port: int, q) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      LOCAL_RANK=str(rank), WORLD_SIZE="2")
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=2)
    r, local, ws = bench.dist_env()
    times = bench.max_over_ranks([1.0 + rank, 5.0 - rank], device="cpu")
    A, _ = bench.make_inputs(64, "box2d1r", 1000 + r)
    q.put({"rank": r, "local": local, "ws": ws, "times": times, "sum": float(A.sum())})
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_reduce_to_the_slowest_time():
    ctx = multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort(key=lambda d: d["rank"])
    assert [d["rank"] for d in out] == [0, 1] and all(d["ws"] == 2 for d in out)
    assert [d["local"] for d in out] == [0, 1]
    # every rank sees the maximum of each value over the ranks
    assert all(d["times"] == [2.0, 5.0] for d in out)
    # replicas sweep different grids (a seed per rank)
    assert out[0]["sum"] != out[1]["sum"]


def test_one_process_keeps_its_own_values():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks([3.0, 4.5], device="cpu") == [3.0, 4.5]


@pytest.mark.parametrize("rank,prints", [(1, False), (0, True)])
def test_reference_arm_prints_on_rank_zero_only(rank, prints):
    env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "0"], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    if not prints:
        assert lines == []
    else:
        d = json.loads(lines[-1])
        assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
        assert d["cpu_baseline"]["kind"] == "port"

"""The N > 1 bench path on CPU: two gloo ranks shard the cases, meet at the barrier and
take the max of their times (bench.py's dist_init / barrier / reduce_max / shard)."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench

    r, w, _ = bench.dist_init()
    lo, hi = bench.shard(3001, r, w)
    bench.barrier(w)
    t = bench.reduce_max(float(10 + r), w)
    q.put((r, lo, hi, t))
    import torch.distributed as dist

    dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_reduce():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got[0][1:3] == (0, 1501) and got[1][1:3] == (1501, 3001)
    assert got[0][3] == got[1][3] == 11.0


def test_reference_arm_prints_the_bench_contract():
    """`bench.py --impl reference` (the CPU oracle on the host cores) prints one JSON line with
    the bench contract's keys, the same metric and config as the GPU arm would, and its own
    e2e / cpu_baseline blocks (no copies: a CPU arm)."""
    import json
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0", "--hours", "24", "--cpu-hours", "24"],
                         capture_output=True, text=True, timeout=600, check=True).stdout
    line = json.loads([ln for ln in out.splitlines() if ln.startswith("{")][-1])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    import bench

    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["higher_is_better"] is True
    assert line["value"] > 0 and line["unit"] == "solves/s" and line["config"]["hours"] == 24
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["cpu_baseline"]["cores"] >= 1 and line["cpu_baseline"]["value"] == line["value"]

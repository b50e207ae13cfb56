"""The benchmark's multi-rank path on the CPU (gloo, world size 2).

Images are independent, so N GPUs run N replicas with no data-path
collective: the only cross-rank steps are the barrier around the timed region
and the max of the ranks' times. Here two gloo ranks check that aggregation,
and `bench.py --gpus 2` started without a launcher runs two ranks itself,
rank 0 alone printing the one JSON line (the reference arm, which needs no GPU).
"""

import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, local_ms, out_q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    w, r, _, pg = bench.dist_setup("gloo")
    bench.barrier(pg)
    value, slowest = bench.replica_throughput(pg, w, 10, local_ms[rank])
    out_q.put((r, value, slowest))
    pg.destroy_process_group()


def test_two_gloo_ranks_report_the_slowest_rank():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    local_ms = [40.0, 50.0]
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, local_ms, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for _, value, slowest in res:
        assert slowest == 50.0
        assert value == pytest.approx(2 * 10 / 0.050)


def test_gpus_flag_starts_its_own_ranks():
    env = dict(os.environ, BENCH_MASTER_PORT=str(free_port()))
    res = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                          "--steps", "1", "--warmup", "0", "--width", "128", "--height", "96"],
                         capture_output=True, text=True, timeout=300, env=env, cwd=ROOT)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["native_so_loaded"] == ["oracle/_build/librd_oracle.so"]

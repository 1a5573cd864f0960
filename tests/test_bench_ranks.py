"""The multi-rank side of bench.py on the CPU (gloo, world size 2).

bench.py runs one replica per GPU (each rank its own instance: weak
scaling, no exchange in the data path); across ranks it only takes the
slowest rank's time, and the reference arm runs on rank 0 alone.  Checked
here without a GPU: the max-reduction and barrier over a gloo group, the
whole-job rate, and that rank 1 of the reference arm exits cleanly without
output.
"""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier(dist)
        slowest = bench.reduce_max(dist, 1.0 + rank)  # rank r took 1 + r seconds
        q.put((rank, slowest, bench.job_rate(world, 1000, 10, slowest)))
        bench.barrier(dist)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_slowest_time_and_the_job_rate():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert [g[0] for g in got] == [0, 1]
    assert all(g[1] == 2.0 for g in got)            # max over ranks
    assert all(g[2] == 2 * 1000 * 10 / 2.0 for g in got)


def test_reference_arm_on_rank_one_exits_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0"], capture_output=True, text=True,
                       env=env, timeout=300, cwd=ROOT)
    assert r.returncode == 0 and r.stdout.strip() == ""

"""The benchmark's multi-GPU form is N independent replicas (rays, tiles
and views shard with no exchange step): each rank renders the whole camera
path on its own GPU, and rank 0 reports the whole-job frames/s from the
slowest rank's time.  These tests run that host-side logic as two gloo
ranks on the CPU, and check that the reference arm's extra ranks exit
without work."""
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


def _rank(rank: int, ws: int, port: int, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        # rank r took 100 + 10 r ms for the cached path, 50 - r ms for the plain one
        vals = bench.max_over_ranks([100.0 + 10 * rank, 50.0 - rank, 2.0 + rank], ws)
        fps = bench.whole_job_rate(ws, 60, vals[0] / 1e3)
        q.put((rank, vals, fps))
    finally:
        dist.destroy_process_group()


def test_replica_times_are_the_slowest_ranks_and_rates_are_whole_job():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    ws, port = 2, _free_port()
    procs = [mp.Process(target=_rank, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(ws)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, vals, fps in out:
        assert vals == [110.0, 50.0, 3.0]
        assert fps == pytest.approx(2 * 60 / 0.110)


def test_single_rank_leaves_values_alone():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks([3.0, 1.0], 1) == [3.0, 1.0]
    assert bench.whole_job_rate(1, 60, 2.0) == 30.0


def test_reference_arm_ranks_above_zero_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""

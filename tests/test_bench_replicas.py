"""The replica path of bench.py (one independent replica per GPU, no
exchange between them) on CPU: two gloo ranks time different steps, and
both end with the slowest rank's times, from which the whole-job rate is
world x steps over that time; the reference arm runs on rank 0 only."""
import os
import socket
import subprocess
import sys

import pytest

import bench

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        out.put((rank, bench.replica_times(times[rank], world)))
    finally:
        dist.destroy_process_group()


def test_two_ranks_report_the_slowest_replica():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    times = [[12.5, 30.0, 40.0], [10.0, 31.5, 39.0]]
    procs = [ctx.Process(target=_rank, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got[0] == got[1] == [12.5, 31.5, 40.0]
    # 2 replicas x 20 steps within the slowest replica's 12.5 ms
    assert bench.job_rate(2, 20, got[0][0]) == pytest.approx(2 * 20 / 12.5e-3)


def test_one_rank_keeps_its_times():
    assert bench.replica_times([1.0, 2.0], 1) == [1.0, 2.0]


def test_config_names_replicas():
    assert bench.deck_config(1)["parallelism"] == "single GPU"
    assert bench.deck_config(4)["parallelism"] == "replicas"


def test_reference_arm_runs_on_rank_zero_only():
    """Under torchrun the reference arm's other ranks exit at once without
    output (rank 0 alone times the host cores)."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert not [line for line in r.stdout.splitlines() if line.startswith("{")]

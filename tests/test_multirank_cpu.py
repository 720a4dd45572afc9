"""The N > 1 path of bench.py without a GPU: two gloo ranks reduce their
timings as the benchmark does (one independent replica per rank: the slowest
rank's time, the sum of particle-steps and of e2e throughputs), and the
reference arm runs on rank 0 only."""
import os
import socket
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, REPO)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms_max, value, e2e = bench.reduce_over_ranks(dist, "cpu", ms=10.0 + 5.0 * rank, e2e=1e6 * (rank + 1),
                                                     particles=1000 * (rank + 1), steps=100)
        out[rank] = (ms_max, value, e2e)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_like_the_benchmark():
    import torch.multiprocessing as mp

    world = 2
    manager = mp.Manager()
    out = manager.dict()
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    for rank in range(world):
        ms_max, value, e2e = out[rank]
        assert ms_max == 15.0
        assert value == pytest.approx((1000 + 2000) * 100 / 0.015)
        assert e2e == 3e6


def test_single_rank_reduce_is_identity():
    sys.path.insert(0, REPO)
    import bench

    assert bench.reduce_over_ranks(None, "cpu", 20.0, 5.0, 10, 4) == (20.0, 10 * 4 / 0.02, 5.0)


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    res = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--gpus", "2"],
                         capture_output=True, text=True, env=env, timeout=300)
    assert res.returncode == 0, res.stderr
    assert res.stdout.strip() == ""


def test_reference_arm_line_on_rank_zero():
    """The reference arm's JSON line (dompap's loops restated in C, on the host
    cores) on the small workload: the contract's keys, and the same `config`
    as the repo's own arm."""
    import json

    sys.path.insert(0, REPO)
    import bench

    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0")
    res = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--workload", "lj500",
                          "--steps", "2", "--warmup", "3"], capture_output=True, text=True, env=env, timeout=300)
    assert res.returncode == 0, res.stderr
    line = json.loads(res.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["value"] > 0 and line["steps"] == 2 and line["higher_is_better"] is True
    assert line["config"] == bench.config_of("lj500", 1, False)
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": bench.UNIT, "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}

"""Multi-rank host logic of bench.py on CPU: world_size-2 gloo ranks.

Each rank runs an independent replica (no data-path collective); the job's
step time is the slowest rank's, and the whole-job value counts every rank's
nodes.  The reference arm runs on rank 0 only; other ranks exit without work.
"""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = [3.0, 5.0][rank]  # rank 1 is the slow replica
    ms_max = bench.max_over_ranks_on(ms, world, torch.device("cpu"))
    val = bench.replica_points_per_s(1 << 21, world, ms_max)
    out[rank] = (ms_max, val)
    dist.destroy_process_group()


def test_gloo_two_ranks_max_time_and_job_value():
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank_main, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    assert out[0][0] == out[1][0] == 5.0
    assert out[0][1] == pytest.approx(2 * (1 << 21) / 5e-3)


def test_reference_arm_nonzero_rank_exits_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_single_rank_value_formula():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks_on(7.0, 1, None) == 7.0
    assert bench.replica_points_per_s(1000, 1, 1.0) == pytest.approx(1e6)
    json.dumps({"metric": bench.METRIC, "unit": bench.UNIT})


def test_gpus_flag_must_match_the_launcher():
    """--gpus N under a launcher that started a different number of ranks fails loudly
    instead of timing fewer GPUs than asked for."""
    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--gpus", "2", "--steps", "1"], env=env,
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 2 and "WORLD_SIZE=1" in r.stderr

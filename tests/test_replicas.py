"""The multi-rank host logic of bench.py on the CPU (gloo, world size 2): one replica per rank,
a barrier and the max over ranks of the timed region, whole-job throughput from the slowest
rank; and the reference arm, which only rank 0 runs."""
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    ranks = bench.Replicas("gloo")
    ranks.barrier()
    ms = 10.0 * (rank + 1)  # rank 1 is the slower replica
    ms_max = ranks.max(ms)
    out[rank] = (ranks.world, ms_max, bench.replica_value(ranks.world, 1000, 50, ms_max))
    ranks.barrier()
    ranks.close()


def test_two_gloo_ranks_take_the_slowest_rank():
    world = 2
    out = mp.Manager().dict()
    mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world, start_method="spawn")
    for r in range(world):
        w, ms_max, value = out[r]
        assert w == world and ms_max == 20.0
        # both replicas' particle-steps over the slower replica's time
        assert value == pytest.approx(2 * 1000 * 50 / 0.020)


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--gpus", "2", "--steps", "1", "--warmup", "0"],
                       capture_output=True, text=True, timeout=120, env=env)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""

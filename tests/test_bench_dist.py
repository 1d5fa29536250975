"""The benchmark's multi-rank host logic (replicas: no data-path collective)
on two CPU ranks over gloo: rendezvous on 127.0.0.1, the barrier around the
timed region, and the max over ranks that turns per-rank times into the
whole-job figure."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import sys
sys.path.insert(0, {root!r})
import bench
ws, rank, local = bench.dist_setup()
assert ws == 2 and local == rank
bench.barrier(ws)
v = bench.max_over_ranks(1.5 + rank, ws)
assert v == 2.5, v
import torch.distributed as dist
assert dist.get_backend() == "gloo"
dist.destroy_process_group()
print("ok", rank)
"""


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_two_gloo_ranks_barrier_and_max():
    pytest.importorskip("torch")
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD.format(root=ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
    outs = []
    for p in procs:
        try:
            out, _ = p.communicate(timeout=240)
        except subprocess.TimeoutExpired:
            p.kill()
            out, _ = p.communicate()
        outs.append(out)
        assert p.returncode == 0, out
    assert "ok 0" in outs[0] and "ok 1" in outs[1]


def test_reference_arm_second_rank_exits_without_work():
    """--impl reference under two ranks: rank 1 returns at once, printing
    nothing (rank 0 alone times the CPU path)."""
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        n, steps, warmup, gpus = 4, 1, 0, 2

    bench.run_reference(Args(), 2, 1)  # returns before any work

"""The multi-GPU launch of bench.py is N independent replicas: a barrier and
the maximum step time over ranks.  Exercised here with two gloo ranks on the
CPU (the GPU runs use NCCL with the same calls)."""

import os
import socket
import subprocess
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    from mplicits_gb300 import replicas
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = replicas.rank_info()
        replicas.barrier()
        ms = 10.0 + 20.0 * rank  # the second replica is the slower one
        slowest = replicas.max_over_ranks(ms)
        value = replicas.replica_value(1000, slowest * 1e-3, w)
        out.put((r, w, local, slowest, value))
        replicas.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas_share_the_slowest_time():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1]
    for r, w, local, slowest, value in res:
        assert w == 2 and local == r
        assert slowest == 30.0
        assert value == pytest.approx(2 * 1000 / 0.030)


def test_single_process_needs_no_group():
    from mplicits_gb300 import replicas
    assert replicas.max_over_ranks(7.5) == 7.5
    assert replicas.replica_value(10, 2.0, 1) == 5.0


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""

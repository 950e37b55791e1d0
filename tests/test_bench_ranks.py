"""Multi-rank host logic of bench.py on the CPU (gloo, world size 2).

The table path needs no exchange, so ranks are replicas: the job's time is the
largest of the ranks' times and its throughput counts every rank's units.
The reference arm runs on rank 0 only; the other ranks exit 0 without work.
"""
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as tmp  # noqa: E402

sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        # rank r "took" 1 + 2r seconds; every rank sees the slowest
        t = bench.max_over_ranks(1.0 + 2.0 * rank, ws, device="cpu")
        dist.barrier()
        q.put((rank, t, bench.replica_value(100, ws, 5, t)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    ws = 2
    ctx = tmp.get_context("spawn")
    q = ctx.SimpleQueue()
    tmp.start_processes(_rank_main, args=(ws, _free_port(), q), nprocs=ws, join=True, start_method="spawn")
    got = sorted(q.get() for _ in range(ws))
    assert [r for r, _, _ in got] == [0, 1]
    for _, t, v in got:
        assert t == 3.0
        # 2 replicas x 100 units x 5 steps in 3 s
        assert v == pytest.approx(1000.0 / 3.0, rel=0, abs=1e-12)


def test_max_over_ranks_one_rank_needs_no_group():
    assert not dist.is_initialized()
    assert bench.max_over_ranks(2.5, 1) == 2.5
    assert bench.replica_value(4.32e6, 1, 20, 0.125) == 4.32e6 * 20 / 0.125


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""

"""bench.py's multi-GPU form runs independent replicas; its only collective is the max over ranks of the
timed region. The host logic runs here as two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.max_over_ranks(1.5 + rank, dist, device="cpu")
    out[rank] = (ms, bench.whole_job_gdofs(world, 1_000_000, ms * 1e-3))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_value():
    world, port = 2, _free_port()
    with mp.Manager() as man:
        out = man.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 2.5
    assert abs(res[0][1] - 2 * 1e6 / 2.5e-3 / 1e9) < 1e-12


def test_single_rank_is_identity():
    assert bench.max_over_ranks(3.25, None) == 3.25
    assert abs(bench.whole_job_gdofs(1, 10**9, 2.0) - 0.5) < 1e-15


def test_reference_arm_other_ranks_exit_without_work(monkeypatch):
    class A:
        steps, warmup, gpus = 3, 3, 2
    called = []
    monkeypatch.setattr(bench, "cpu_baseline", lambda *a, **k: called.append(1) or {"value": 1.0})
    assert bench.run_reference(A(), bench.CONFIGS["hp-elasticity-32"], 1) is None
    assert not called

"""The multi-GPU replica path's host logic (cubff_gb300/replicas.py) on CPU:
two gloo ranks, a barrier, and the reduction of work (sum) and time (max)
that bench.py applies to its timed region."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
mp = pytest.importorskip("torch.multiprocessing")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    from cubff_gb300 import replicas
    import torch.distributed as dist
    group = replicas.init("gloo", timeout_s=60)
    replicas.barrier(group)
    units, secs = replicas.reduce(100.0 * (rank + 1), 0.5 + rank, group)
    replicas.barrier(group)
    out[rank] = (units, secs, replicas.replica_seed(1, rank))
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_work_and_time():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    assert out[0][:2] == (300.0, 1.5) and out[1][:2] == (300.0, 1.5)
    assert (out[0][2], out[1][2]) == (1, 2)


def test_single_process_needs_no_group(monkeypatch):
    from cubff_gb300 import replicas
    monkeypatch.setenv("WORLD_SIZE", "1")
    assert replicas.init() is None
    assert replicas.reduce(7, 2.5, None) == (7.0, 2.5)

"""The multi-replica measurement of bench.py (torchrun, one independent replica per
rank, the job's time = the slowest replica's), on CPU with the gloo backend and
world size 2."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    ws, r, local = bench._init_replicas(backend="gloo")
    assert (ws, r, local) == (world, rank, rank)
    out[rank] = bench._max_over_ranks(10.0 + 5.0 * rank, device="cpu")
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_two_gloo_ranks():
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        assert dict(out) == {0: 15.0, 1: 15.0}


def test_single_replica_needs_no_group(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("WORLD_SIZE", "1")
    assert bench._init_replicas() == (1, 0, 0)
    assert bench._max_over_ranks(3.5) == 3.5

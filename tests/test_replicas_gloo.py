"""The multi-GPU path of bench.py is replicas only: each rank advances its own run and the
ranks meet only in barriers and a max-reduction of their times.  Covered here with two gloo
ranks on the CPU (no GPU)."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    w, r, local = bench.dist_env()
    assert (w, r, local) == (ws, rank, rank)
    bench.barrier(ws)
    m = bench.barrier_max(float(rank + 1) * 1.5, ws)
    out[rank] = m
    dist.destroy_process_group()


def test_two_rank_max_over_ranks():
    ws = 2
    port = _free_port()
    out = mp.Manager().dict()
    mp.start_processes(_rank, args=(ws, port, out), nprocs=ws, start_method="spawn", join=True)
    assert dict(out) == {0: 3.0, 1: 3.0}

"""bench.py's multi-rank timing under torch.distributed with the gloo backend on CPU: every rank
reports the maximum step time over ranks (independent replicas, no data-path collective)."""
import os
import socket

import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    import bench
    out[rank] = bench.max_over_ranks(10.0 + 7.5 * rank, torch.device('cpu'))
    dist.destroy_process_group()


def test_max_over_ranks_with_gloo():
    world = 2
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.start_processes(_rank, args=(world, port, out), nprocs=world, start_method='spawn')
        assert dict(out) == {0: 17.5, 1: 17.5}


def test_max_over_ranks_single_process_is_identity():
    import bench
    assert bench.max_over_ranks(3.25, torch.device('cpu')) == 3.25

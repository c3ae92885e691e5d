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


def _shard_rank(rank, world, port, out):
    """One rank of a point-sharded evaluation: its share of the FP64 oracle (its residual rows,
    the boundary terms on rank 0 only), summed over the ranks by the package's all-reduce."""
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    import cases
    from oracle import oracle as O
    from torch_de_solver_gb300.prepare import shard_rows
    from torch_de_solver_gb300.solution import allreduce_sum
    res = {}
    for name, builder in (('burgers', lambda api, dtype='float32': cases.burgers_ag(api, n=20, dtype=dtype)),
                          ('kovasznay', lambda api, dtype='float32': cases.kovasznay_ag(api, n=11, dtype=dtype))):
        prob, net = O.build_problem(builder, 'float64')
        rows = shard_rows(prob.points.shape[0], rank, world)
        loss, lossn, grad, _ = O.loss_and_grad_chunked(prob, net, chunk=50, rows=rows,
                                                       with_boundary=rank == 0)
        lbuf = torch.tensor([loss, lossn], dtype=torch.float64)
        grad = grad.detach().clone()
        allreduce_sum(grad, lbuf)
        res[name] = (lbuf.tolist(), grad.numpy())
    out[rank] = res
    dist.destroy_process_group()


def test_point_sharded_step_sums_to_the_whole_problem_with_gloo():
    """Two ranks, each with its contiguous share of the residual points (rank 0 also the boundary
    conditions): after the one all-reduce every rank holds the unsharded FP64 loss and gradient."""
    import numpy as np
    import cases
    from oracle import oracle as O
    world = 2
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.start_processes(_shard_rank, args=(world, port, out), nprocs=world, start_method='spawn')
        got = dict(out)
    for name, builder in (('burgers', lambda api, dtype='float32': cases.burgers_ag(api, n=20, dtype=dtype)),
                          ('kovasznay', lambda api, dtype='float32': cases.kovasznay_ag(api, n=11, dtype=dtype))):
        prob, net = O.build_problem(builder, 'float64')
        loss, lossn, grad, _ = O.loss_and_grad(prob, net)
        for rank in range(world):
            (l, ln), g = got[rank][name]
            assert abs(l - loss) <= 1e-12 * abs(loss) and abs(ln - lossn) <= 1e-12 * abs(lossn)
            assert np.linalg.norm(g - grad.numpy()) <= 1e-12 * np.linalg.norm(grad.numpy())

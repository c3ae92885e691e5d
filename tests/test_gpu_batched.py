"""Batched sweep: several independent solves (different grids, coefficients and networks) in one
launch give the same per-solve loss and gradient as separate plans and as the oracle."""
import numpy as np
import pytest
import torch

import cases
from helpers import rel
from oracle import oracle as O


def _solves(k):
    params = cases.sweep_params(k, seed=3)
    for i, sp in enumerate(params):
        sp['nx'] = 16 + (sp['nx'] % 24)
        sp['nt'] = 16 + (sp['nt'] % 20)
        yield i, sp


@pytest.mark.gpu
@pytest.mark.parametrize('precision', ['fp32', '3xtf32'])
def test_batched_solves_match_oracle_and_single_plans(precision):
    """Every solve's own network: the tensor-core kernel packs each problem's hidden weights."""
    import torch_de_solver_gb300 as T
    models, refs = [], []
    for i, sp in _solves(5):
        b = lambda api, dtype='float32', sp=sp, i=i: cases.sweep_ag(api, seed=1000 + i, dtype=dtype, **sp)
        d, bc, eq, net, kw = b(T)
        models.append(T.Model(net, d, eq, bc))
        prob, onet = O.build_problem(b, 'float64')
        l, ln, g, _ = O.loss_and_grad(prob, onet)
        refs.append((l, ln, g.numpy()))
    bm = T.BatchedModel(models)
    bm.compile('autograd', lambda_operator=1, lambda_bound=1, precision=precision)
    losses = bm.evaluate(with_grad=True).cpu().numpy()
    P = bm.plan.n_params
    grads = bm.grad.view(len(models), P).cpu().numpy()
    for i, (l, ln, g) in enumerate(refs):
        assert rel(losses[i, 0], l) < 1e-5, (i, losses[i, 0], l)
        assert rel(losses[i, 1], ln) < 1e-5
        assert rel(grads[i], g) < 1e-5, (i, rel(grads[i], g))


@pytest.mark.gpu
def test_batched_training_decreases_every_loss():
    import torch_de_solver_gb300 as T
    models = []
    for i, sp in _solves(8):
        d, bc, eq, net, kw = cases.sweep_ag(T, seed=1000 + i, **sp)
        models.append(T.Model(net, d, eq, bc))
    bm = T.BatchedModel(models)
    bm.compile('autograd', lambda_operator=1, lambda_bound=1)
    l0 = bm.evaluate().cpu().numpy()[:, 0].copy()
    bm.train(lr=1e-3, epochs=30)
    l1 = bm.evaluate().cpu().numpy()[:, 0]
    assert (l1 < l0).all(), (l0, l1)

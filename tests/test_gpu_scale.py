"""Parity at the benchmark sizes.

Kovasznay flow (Re=20) at the full 1024 x 1024 = 1,048,576 collocation points plus 4,096
boundary points, MLP 2-128x5-3: the fused kernel's loss, normalized loss, gradient and per-equation
residual sums against the FP64 oracle of the same weights. At this size each persistent CTA walks
~270 tiles and adds every tile's weight gradient into its own FP32 segment, so this checks the
accumulation depth the small fixtures do not reach. The oracle runs on the CUDA device as the
checker, chunk by chunk of residual points (its loss is a sum over points, tedeous/losses.py:58).

The equation-discovery sweep with the full grid-size range Nx, Nt in {16..128}: 32 solves (the
smallest and largest grids forced in) in one batched launch, every solve against its own FP64
oracle.

Tolerance: relative 1e-5 (FP32, split TF32 and the plain form against FP64); 1e-2 for TF32 and 1e-1
for BF16, the bounds of the precision study.
"""
import numpy as np
import pytest
import torch

import cases
from helpers import build_model, rel
from oracle import oracle as O

TOL = 1e-5
N_FULL = 1023   # 1024 nodes per axis


def _kov_builder(api, dtype='float32'):
    return cases.kovasznay_ag(api, n=N_FULL, dtype=dtype)


@pytest.fixture(scope='module')
def kovasznay_fp64():
    prob, net = O.build_problem(_kov_builder, 'float64')
    prob.to('cuda')
    net = net.to('cuda')
    loss, lossn, grad, sumsq = O.loss_and_grad_chunked(prob, net, chunk=262144)
    out = dict(loss=loss, lossn=lossn, grad=grad.cpu().numpy(), sumsq=sumsq.cpu().numpy(),
               n=prob.points.shape[0])
    del prob, net
    torch.cuda.empty_cache()
    return out


# (precision, form, tolerance): the FP32-tolerance forms at 1e-5; TF32 and BF16 at the bounds the
# precision study states for them
SCALE_CASES = [('3xtf32', 'fused', TOL), ('fp32', 'fused', TOL), ('fp32', 'plain', TOL),
               ('tf32', 'fused', 1e-2), ('bf16', 'fused', 1e-1)]


@pytest.mark.gpu
@pytest.mark.parametrize('precision,form,tol', SCALE_CASES)
def test_kovasznay_million_points_match_fp64_oracle(precision, form, tol, kovasznay_fp64):
    import torch_de_solver_gb300 as T
    ref = kovasznay_fp64
    model = build_model(T, builder=_kov_builder, precision=precision, form=form)
    sol = model.solution_cls
    assert sol.ir.n_residual_rows == ref['n'] == 1024 * 1024
    loss, lossn = sol.evaluate()
    loss.backward()
    sol.check_status()
    grad = torch.cat([p.grad.reshape(-1) for p in model.net.parameters()]).cpu().numpy()
    op = sol.op.double()
    sumsq = (op ** 2).sum(0).cpu().numpy()
    rl, rn, rg, rs = (rel(loss.item(), ref['loss']), rel(lossn.item(), ref['lossn']),
                      rel(grad, ref['grad']), rel(sumsq, ref['sumsq']))
    print(f'kovasznay 1M {precision} {form}: loss rel {rl:.2e} lossn rel {rn:.2e} grad rel {rg:.2e} '
          f'op sumsq rel {rs:.2e} (tiles {sol.plan.info.n_tiles}, CTAs {sol.plan.info.n_ctas})')
    assert rl < tol and rn < tol and rg < tol and rs < tol, (rl, rn, rg, rs)
    del model, sol
    torch.cuda.empty_cache()


def _sweep_solves(k):
    params = cases.sweep_params(k, seed=11)
    params[0].update(nx=16, nt=16)
    params[1].update(nx=128, nt=128)
    return params


@pytest.mark.gpu
@pytest.mark.parametrize('precision', ['fp32', '3xtf32'])
def test_sweep_batch_full_grid_range_matches_fp64_oracle(precision):
    import torch_de_solver_gb300 as T
    params = _sweep_solves(32)
    assert min(min(p['nx'], p['nt']) for p in params) == 16
    assert max(max(p['nx'], p['nt']) for p in params) == 128
    models, refs = [], []
    for i, sp in enumerate(params):
        b = lambda api, dtype='float32', sp=sp, i=i: cases.sweep_ag(api, seed=1000 + i, dtype=dtype, **sp)
        d, bc, eq, net, kw = b(T)
        models.append(T.Model(net, d, eq, bc))
        prob, onet = O.build_problem(b, 'float64')
        prob.to('cuda')
        l, ln, g, _ = O.loss_and_grad(prob, onet.to('cuda'))
        refs.append((l, ln, g.cpu().numpy()))
    bm = T.BatchedModel(models)
    bm.compile('autograd', lambda_operator=1, lambda_bound=1, precision=precision)
    losses = bm.evaluate(with_grad=True).cpu().numpy()
    P = bm.plan.n_params
    grads = bm.grad.view(len(models), P).cpu().numpy()
    worst = 0.0
    for i, (l, ln, g) in enumerate(refs):
        r = max(rel(losses[i, 0], l), rel(losses[i, 1], ln), rel(grads[i], g))
        worst = max(worst, r)
        assert r < TOL, (i, params[i], r)
    n_pts = sum(p['nx'] * p['nt'] for p in params)
    print(f'sweep 32 solves ({n_pts} points) {precision}: worst rel {worst:.2e}')

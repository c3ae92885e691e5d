"""Tile schedules (tdg_plan_create_scheduled) and the autotuner that picks them.

Every candidate schedule of torch_de_solver_gb300.autotune (rows per tile 128 / 96 / 64, equal
tile counts or equal estimated work per CTA) evaluates the same problems: loss and gradient equal
the default schedule's to FP32 summation-order rounding and the FP64 oracle to 1e-5, on a batched
sweep of uneven grids and on Kovasznay. tune() times them on the device, returns one of them and
caches the choice per problem shape."""
import numpy as np
import pytest
import torch

import cases
from helpers import rel
from oracle import oracle as O


def _sweep_irs(T, k=6):
    from torch_de_solver_gb300.prepare import lower
    irs, nets, refs = [], [], []
    for i, sp in enumerate(cases.sweep_params(k, seed=4)):
        b = lambda api, dtype='float32', sp=sp, i=i: cases.sweep_ag(api, seed=1000 + i, dtype=dtype, **sp)
        d, bc, eq, net, kw = b(T)
        irs.append(lower(d.build('autograd'), eq.equation_lst, bc.build(d.variable_dict), 'autograd',
                         1, 1, d_out=1))
        nets.append(net)
        prob, onet = O.build_problem(b, 'float64')
        l, ln, g, _ = O.loss_and_grad(prob, onet)
        refs.append((l, g.numpy()))
    return irs, nets, refs


def _eval(plan, flat):
    grad = torch.zeros_like(flat)
    loss = torch.zeros(2 * plan.n_problems, dtype=torch.float64, device=flat.device)
    plan.loss_grad(flat, grad, loss)
    return loss.view(-1, 2)[:, 0].cpu().numpy(), grad.view(plan.n_problems, -1).cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize('precision', ['fp32', '3xtf32'])
def test_every_candidate_schedule_gives_the_same_loss_and_gradient(precision):
    import torch_de_solver_gb300 as T
    from torch_de_solver_gb300.autotune import CANDIDATES
    from torch_de_solver_gb300.solution import DevicePlan
    irs, nets, refs = _sweep_irs(T)
    widths = [2, 64, 64, 64, 1]
    flat = torch.cat([torch.nn.utils.parameters_to_vector(n.parameters()) for n in nets]).cuda()
    base_l, base_g = _eval(DevicePlan(irs, widths, torch.device('cuda'), precision), flat)
    for sched in CANDIDATES:
        plan = DevicePlan(irs, widths, torch.device('cuda'), precision, schedule=sched)
        l, g = _eval(plan, flat)
        assert rel(l, base_l) < 1e-6 and rel(g, base_g) < 1e-6, (sched, rel(l, base_l), rel(g, base_g))
        for i, (l64, g64) in enumerate(refs):
            assert rel(l[i], l64) < 1e-5 and rel(g[i], g64) < 1e-5, (sched, i)
        print(precision, sched, 'tiles', plan.info.n_tiles, 'ctas', plan.info.n_ctas)


@pytest.mark.gpu
def test_kovasznay_under_a_tuned_schedule_matches_the_oracle(tmp_path, monkeypatch):
    import torch_de_solver_gb300 as T
    monkeypatch.setenv('TDG_AUTOTUNE_CACHE', str(tmp_path / 'tune.json'))
    b = lambda api, dtype='float32': cases.kovasznay_ag(api, n=47, dtype=dtype)
    domain, bnd, eq, net, kw = b(T)
    kw = dict(kw)
    model = T.Model(net, domain, eq, bnd)
    model.compile(kw.pop('mode'), autotune=True, **kw)
    sol = model.solution_cls
    rec = sol.tuning
    assert sol.schedule in [t['schedule'] for t in rec['trials']]
    assert rec['ms'] == min(t['ms'] for t in rec['trials'])
    print('kovasznay 48x48 tuning:', [(t['schedule'], t['ms']) for t in rec['trials']])
    loss, _ = sol.evaluate()
    loss.backward()
    grad = torch.cat([p.grad.reshape(-1) for p in model.net.parameters()]).cpu().numpy()
    prob, onet = O.build_problem(b, 'float64')
    l64, _, g64, _ = O.loss_and_grad(prob, onet)
    assert rel(loss.item(), l64) < 1e-5 and rel(grad, g64.numpy()) < 1e-5
    # the second compile of the same shape reads the cache instead of timing again
    from torch_de_solver_gb300 import autotune
    calls = []
    monkeypatch.setattr(autotune, 'time_schedule', lambda *a, **k: calls.append(1))
    domain, bnd, eq, net, kw = b(T)
    kw = dict(kw)
    model2 = T.Model(net, domain, eq, bnd)
    model2.compile(kw.pop('mode'), autotune=True, **kw)
    assert not calls and model2.solution_cls.schedule == sol.schedule

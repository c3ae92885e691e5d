"""The device path solves the equations: long Adam runs against closed-form solutions. Heat in
'NN' mode on the survey's 21x21 grid (u = exp(-pi^2 t) sin(pi x)) and Kovasznay flow in autograd
mode at the default precision (split TF32) on a 128x128 grid. The bounds leave about twice the
errors measured on a GB300 (heat 2.8 % after 1500 steps; Kovasznay u 1.9 %, v 3.7 %, p 1.5 %
after 6000 steps)."""
import numpy as np
import pytest
import torch

import cases


def _rel_l2(a, b):
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


@pytest.mark.gpu
def test_heat_nn_converges_to_the_closed_form():
    import torch_de_solver_gb300 as T
    d, b, e, net, kw = cases.heat_nn(T)
    kw = dict(kw)
    model = T.Model(net, d, e, b)
    model.compile(kw.pop('mode'), **kw)
    model.train(T.Optimizer('Adam', {'lr': 1e-3}), 1501)
    g = d.build('NN').cuda()
    with torch.no_grad():
        u = model.net(g).reshape(-1)
    exact = torch.exp(-np.pi ** 2 * g[:, 1]) * torch.sin(np.pi * g[:, 0])
    err = _rel_l2(u, exact)
    print(f'heat NN: relative L2 error {err:.4f}')
    assert err < 0.07


@pytest.mark.gpu
def test_kovasznay_converges_to_the_closed_form():
    import torch_de_solver_gb300 as T
    d, b, e, net, kw = cases.kovasznay_ag(T, n=127)
    kw = dict(kw)
    model = T.Model(net, d, e, b)
    model.compile(kw.pop('mode'), **kw)
    assert model.solution_cls.precision == '3xtf32'
    model.train(T.Optimizer('Adam', {'lr': 1e-3}), 6001)
    g = d.build('autograd').cuda()
    with torch.no_grad():
        out = model.net(g)
    exact = torch.stack(cases.kovasznay_exact(g), 1)
    errs = [_rel_l2(out[:, i], exact[:, i]) for i in range(3)]
    print('Kovasznay: relative L2 errors (u, v, p)', errs)
    assert errs[0] < 0.05 and errs[1] < 0.12 and errs[2] < 0.05, errs


@pytest.mark.gpu
def test_kovasznay_adam_then_lbfgs64():
    """Adam, then L-BFGS with FP64 dot products (the survey's recipe for this flow): measured
    0.09 % / 0.36 % / 0.11 % relative L2 error in u / v / p after 3000 Adam and 50 L-BFGS steps."""
    import torch_de_solver_gb300 as T
    d, b, e, net, kw = cases.kovasznay_ag(T, n=127)
    kw = dict(kw)
    model = T.Model(net, d, e, b)
    model.compile(kw.pop('mode'), **kw)
    model.train(T.Optimizer('Adam', {'lr': 1e-3}), 3001)
    model.train(T.Optimizer('LBFGS', {'lr': 1.0, 'max_iter': 20, 'history_size': 50}), 51)
    assert isinstance(model.optimizer, T.LBFGS64)
    g = d.build('autograd').cuda()
    with torch.no_grad():
        out = model.net(g)
    exact = torch.stack(cases.kovasznay_exact(g), 1)
    errs = [_rel_l2(out[:, i], exact[:, i]) for i in range(3)]
    print('Kovasznay, Adam + L-BFGS: relative L2 errors (u, v, p)', errs)
    assert errs[0] < 0.005 and errs[1] < 0.01 and errs[2] < 0.005, errs

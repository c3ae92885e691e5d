"""The kernels' parameter gradient against central finite differences of the FP64 loss.

For 64 parameter indices drawn with a fixed seed, d loss / d theta_i is estimated as
(L(theta + h e_i) - L(theta - h e_i)) / (2h), h = 1e-3, with L the FP64 oracle loss (the
reference's nested-autograd path, tedeous/derivative.py:74-132, or its stencil path,
derivative.py:30-58, in FP64). The kernels' gradient (FP32, split TF32, plain form) must agree
with it. Measured: the FP64 difference quotient itself matches the FP64 analytic gradient to
~1e-7 relative (test_fd_quotient_matches_fp64_gradient), so the bound below, 1e-5 on the vector
of sampled entries and per entry relative to the largest sampled entry, tests the kernels.

Workloads: Burgers 'autograd' at its benchmark size (101 x 101, MLP 2-32x4-1) and heat 'NN'
(21 x 21, MLP 2-100x3-1, h = 1/20).
"""
import numpy as np
import pytest
import torch

import cases
from helpers import build_model, rel
from oracle import oracle as O

H = 1e-3
K = 64
BOUND = 1e-5

BUILDERS = {
    'burgers_ag_101': lambda api, dtype='float32': cases.burgers_ag(api, n=100, dtype=dtype),
    'heat_nn_21': lambda api, dtype='float32': cases.heat_nn(api, n=20, dtype=dtype),
}


def _fd(builder, k=K, seed=0):
    """(sampled indices, central differences, FP64 analytic gradient at those indices)."""
    prob, net = O.build_problem(builder, 'float64')
    _, _, g, _ = O.loss_and_grad(prob, net)
    w0 = torch.nn.utils.parameters_to_vector(net.parameters()).detach().clone()
    idx = np.random.default_rng(seed).choice(w0.numel(), k, replace=False)
    fd = np.empty(k)
    for j, i in enumerate(idx):
        vals = []
        for s in (1.0, -1.0):
            w = w0.clone()
            w[i] += s * H
            torch.nn.utils.vector_to_parameters(w, net.parameters())
            vals.append(float(prob.evaluate(net)['loss'].detach().reshape(-1)[0]))
        fd[j] = (vals[0] - vals[1]) / (2 * H)
    return idx, fd, g.numpy()[idx]


_CACHE = {}


def _fd_cached(name):
    if name not in _CACHE:
        _CACHE[name] = _fd(BUILDERS[name])
    return _CACHE[name]


def _errors(fd, g):
    return rel(g, fd), float(np.abs(g - fd).max() / np.abs(fd).max())


def test_fd_quotient_matches_fp64_gradient():
    """The difference quotient the GPU test uses, checked against the FP64 analytic gradient
    (16 indices of the heat 'NN' case keep this CPU test short)."""
    idx, fd, g64 = _fd(BUILDERS['heat_nn_21'], k=16, seed=1)
    vec, ent = _errors(fd, g64)
    assert vec < 1e-6 and ent < 1e-6, (vec, ent)


@pytest.mark.gpu
@pytest.mark.parametrize('precision,form', [('fp32', 'fused'), ('3xtf32', 'fused'), ('fp32', 'plain')])
@pytest.mark.parametrize('name', list(BUILDERS))
def test_gradient_matches_central_differences(name, precision, form):
    import torch_de_solver_gb300 as T
    idx, fd, g64 = _fd_cached(name)
    model = build_model(T, builder=BUILDERS[name], precision=precision, form=form)
    loss, _ = model.solution_cls.evaluate()
    loss.backward()
    grad = torch.cat([p.grad.reshape(-1) for p in model.net.parameters()]).double().cpu().numpy()
    vec, ent = _errors(fd, grad[idx])
    print(f'{name} {form} {precision}: vs central differences (h={H}, {K} entries) vector rel '
          f'{vec:.2e}, max entry err / max |entry| {ent:.2e}; FD vs FP64 gradient '
          f'{_errors(fd, g64)[0]:.2e}')
    assert vec < BOUND and ent < BOUND, (vec, ent)

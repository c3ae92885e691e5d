"""Edge cases of the device path: the plan's limits raise NotImplementedError with the limit named,
and the smallest problems (a tile mostly padding, the widest supported MLP) still match the
oracle."""
import numpy as np
import pytest
import torch

import cases
from helpers import rel
from oracle import oracle as O


def _compile(T, builder, **compile_kw):
    d, bc, eq, net, kw = builder(T)
    kw = dict(kw)
    m = T.Model(net, d, eq, bc)
    m.compile(kw.pop('mode'), **kw, **compile_kw)
    return m


@pytest.mark.gpu
@pytest.mark.parametrize('precision', ['fp32', '3xtf32'])
def test_fused_form_refuses_a_width_not_a_multiple_of_4(precision):
    """Asked for explicitly, the fused form names its width limit (the plan refuses it)."""
    import torch_de_solver_gb300 as T
    b = lambda api, dtype='float32': cases.burgers_ag(api, n=8, dtype=dtype, widths=(2, 30, 30, 1))
    with pytest.raises(NotImplementedError, match='hidden width 30'):
        _compile(T, b, precision=precision, form='fused')


@pytest.mark.gpu
def test_tensor_core_precision_refuses_a_width_the_fused_form_lacks():
    import torch_de_solver_gb300 as T
    b = lambda api, dtype='float32': cases.burgers_ag(api, n=8, dtype=dtype, widths=(2, 30, 30, 1))
    with pytest.raises(NotImplementedError, match='hidden widths'):
        _compile(T, b, precision='3xtf32')


@pytest.mark.gpu
@pytest.mark.parametrize('widths', [(2, 30, 30, 1), (2, 150, 150, 1), (2, 256, 1)])
def test_any_width_runs_in_the_plain_form(widths):
    """Networks the fused kernels do not take (the reference's examples use 50-, 150- and
    256-wide layers) compile to the plain form with a warning, and its loss and gradient match
    the FP64 oracle; a few training steps run and lower the loss."""
    import torch_de_solver_gb300 as T
    b = lambda api, dtype='float32': cases.burgers_ag(api, n=16, dtype=dtype, widths=widths)
    prob, onet = O.build_problem(b, 'float64')
    l_ref, ln_ref, g_ref, _ = O.loss_and_grad(prob, onet)
    with pytest.warns(UserWarning, match='plain form'):
        m = _compile(T, b)
    assert m.solution_cls.form == 'plain' and m.solution_cls.precision == 'fp32'
    w = torch.nn.utils.parameters_to_vector(onet.parameters()).detach().float()
    torch.nn.utils.vector_to_parameters(w.to(m.solution_cls.device), m.net.parameters())
    loss, lossn = m.solution_cls.evaluate()
    loss.backward()
    grad = torch.cat([p.grad.reshape(-1) for p in m.net.parameters()]).double().cpu().numpy()
    assert rel(loss.item(), l_ref) < 1e-5 and rel(lossn.item(), ln_ref) < 1e-5
    assert rel(grad, g_ref.numpy()) < 1e-5, rel(grad, g_ref.numpy())
    first = loss.item()
    m.train(T.Optimizer('Adam', {'lr': 1e-3}), 21)
    m.solution_cls.check_status()
    assert m.solution_cls.evaluate(save_graph=False)[0].item() < first


@pytest.mark.gpu
@pytest.mark.parametrize('precision', ['fp32', '3xtf32'])
def test_one_hidden_layer_runs_fused(precision):
    """A network with a single hidden layer has no hidden GEMM: the fused kernels go from the
    input layer's jets straight to the output layer (no weights staged for a GEMM). Loss and
    gradient against the FP64 oracle, and a few training steps."""
    import torch_de_solver_gb300 as T
    b = lambda api, dtype='float32': cases.burgers_ag(api, n=16, dtype=dtype, widths=(2, 32, 1))
    prob, onet = O.build_problem(b, 'float64')
    l_ref, ln_ref, g_ref, _ = O.loss_and_grad(prob, onet)
    m = _compile(T, b, precision=precision)
    assert m.solution_cls.form == 'fused'
    w = torch.nn.utils.parameters_to_vector(onet.parameters()).detach().float()
    torch.nn.utils.vector_to_parameters(w.to(m.solution_cls.device), m.net.parameters())
    loss, lossn = m.solution_cls.evaluate()
    loss.backward()
    grad = torch.cat([p.grad.reshape(-1) for p in m.net.parameters()]).double().cpu().numpy()
    assert rel(loss.item(), l_ref) < 1e-5 and rel(lossn.item(), ln_ref) < 1e-5
    assert rel(grad, g_ref.numpy()) < 1e-5, rel(grad, g_ref.numpy())
    first = loss.item()
    m.train(T.Optimizer('Adam', {'lr': 1e-3}), 21)
    m.solution_cls.check_status()
    assert m.solution_cls.evaluate(save_graph=False)[0].item() < first


@pytest.mark.gpu
def test_unsupported_networks_are_refused():
    import torch_de_solver_gb300 as T
    d, bc, eq, net, kw = cases.burgers_ag(T, n=8)
    relu = torch.nn.Sequential(torch.nn.Linear(2, 32), torch.nn.ReLU(), torch.nn.Linear(32, 1))
    with pytest.raises(NotImplementedError, match='Tanh'):
        T.Model(relu, d, eq, bc).compile('autograd', lambda_operator=1, lambda_bound=10)
    wide = cases.mlp([2, 256, 1], 0)
    with pytest.raises(NotImplementedError, match='hidden width 256'):
        T.Model(wide, d, eq, bc).compile('autograd', lambda_operator=1, lambda_bound=10, form='fused')


@pytest.mark.gpu
@pytest.mark.parametrize('precision', ['fp32', '3xtf32'])
def test_tiny_problem_and_widest_mlp_match_oracle(precision):
    """A 3x3 grid (9 residual points in one mostly padded tile) with the widest supported hidden
    layers (128) and a single hidden GEMM."""
    import torch_de_solver_gb300 as T
    b = lambda api, dtype='float32': cases.burgers_ag(api, n=2, dtype=dtype, widths=(2, 128, 128, 1))
    prob, onet = O.build_problem(b, 'float64')
    l_ref, ln_ref, g_ref, _ = O.loss_and_grad(prob, onet)
    m = _compile(T, b, precision=precision)
    w = torch.nn.utils.parameters_to_vector(onet.parameters()).detach().float()
    torch.nn.utils.vector_to_parameters(w.to(m.solution_cls.device), m.net.parameters())
    loss, lossn = m.solution_cls.evaluate()
    loss.backward()
    grad = torch.cat([p.grad.reshape(-1) for p in m.net.parameters()]).double().cpu().numpy()
    assert rel(loss.item(), l_ref) < 1e-5 and rel(lossn.item(), ln_ref) < 1e-5
    assert rel(grad, g_ref.numpy()) < 1e-5, rel(grad, g_ref.numpy())

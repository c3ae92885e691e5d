"""Inverse problems: trainable equation coefficients (nn.Parameter terms registered on the network,
as tedeous.models.parameter_registr does) on the device path. The gradient with respect to each
coefficient, the training run that fits them and the batched form are compared with the reference's
own fixtures (autograd mode) and with the FP64 oracle ('NN' mode, which the reference rejects)."""
import numpy as np
import pytest
import torch

import cases
from helpers import build_model, golden, rel, set_flat_weights
from oracle import oracle as O

# per-coefficient bounds against the FP64 fixture: the FP32 paths at the FP32 tolerance of a
# sum over the residual points, TF32 and BF16 at their operand precisions
COEFF_BOUND = {('fp32', 'fused'): 1e-4, ('3xtf32', 'fused'): 1e-4, ('fp32', 'plain'): 1e-4,
               ('tf32', 'fused'): 3e-2, ('bf16', 'fused'): 3e-1}


@pytest.mark.gpu
@pytest.mark.parametrize('precision,form', list(COEFF_BOUND))
def test_coefficient_gradient_matches_reference(precision, form):
    import torch_de_solver_gb300 as T
    g = golden('inverse_burgers_ag')
    model = build_model(T, 'inverse_burgers_ag', weights=g['weights'], precision=precision,
                        form=form)
    loss, _ = model.solution_cls.evaluate()
    loss.backward()
    net = model.net
    got = [float(net.lam1.grad), float(net.lam2.grad)]
    want = g['grad64'][:2]
    errs = [abs(a - b) / abs(b) for a, b in zip(got, want)]
    print(f'{precision}/{form}: d loss/d lam {got} reference {list(want)} rel {errs}')
    assert max(errs) < COEFF_BOUND[(precision, form)], (got, want)
    grad = torch.cat([p.grad.reshape(-1) for p in net.parameters()]).cpu().numpy()
    bound = 1e-5 if COEFF_BOUND[(precision, form)] <= 1e-4 else 10 * COEFF_BOUND[(precision, form)]
    assert rel(grad, g['grad64']) < bound


@pytest.mark.gpu
def test_inverse_training_matches_reference():
    """train(6) with Adam(lr=1e-3) on the network and its coefficients (the fused Adam launch and
    the CUDA-graph replay of the step): the closure losses, the final network and coefficients."""
    import torch_de_solver_gb300 as T
    g = golden('inverse_burgers_ag')
    model = build_model(T, 'inverse_burgers_ag', weights=g['weights'])
    seen = []

    class Record(T.Callback):
        def on_epoch_end(self, logs=None):
            seen.append(float(self.model.cur_loss.reshape(-1)[0]))

    model.train(T.Optimizer('Adam', {'lr': 1e-3}), 6, callbacks=[Record()])
    assert rel(seen, g['curve32']) < 1e-5, (seen, g['curve32'])
    w = torch.nn.utils.parameters_to_vector(model.net.parameters()).detach().cpu().numpy()
    assert rel(w, g['final32']) < 1e-5, rel(w, g['final32'])
    assert np.abs(w[:2] - g['final32'][:2]).max() < 1e-6, (w[:2], g['final32'][:2])


def _oracle_fp64(builder, weights, drop=()):
    prob, net = O.build_problem(builder, 'float64')
    set_flat_weights(net, weights)
    net.to(torch.float64)
    for name in drop:
        del net._parameters[name]
    loss, lossn, _, _ = O.loss_and_grad(prob, net)
    return loss, lossn, net


@pytest.mark.gpu
@pytest.mark.parametrize('precision', ['fp32', '3xtf32'])
def test_inverse_nn_mode_matches_oracle(precision):
    import torch_de_solver_gb300 as T
    builder = lambda api, dtype='float32': cases.inverse_burgers_ag(api, n=24, dtype=dtype, mode='NN')
    w = cases.inverse_burgers_ag(T, n=24)[3]
    w = torch.nn.utils.parameters_to_vector(w.parameters()).detach().numpy()
    loss, lossn, onet = _oracle_fp64(builder, w)
    ref = torch.cat([p.grad.reshape(-1) for p in onet.parameters()]).numpy()
    model = build_model(T, builder=builder, weights=w, precision=precision)
    l, ln = model.solution_cls.evaluate()
    l.backward()
    got = torch.cat([p.grad.reshape(-1) for p in model.net.parameters()]).cpu().numpy()
    assert rel(l.item(), loss) < 1e-5 and rel(ln.item(), lossn) < 1e-5
    assert rel(got, ref) < 1e-5, rel(got, ref)
    assert rel(got[:2], ref[:2]) < 1e-4, (got[:2], ref[:2])


@pytest.mark.gpu
def test_unregistered_coefficient_gets_gradient():
    """A coefficient that is not a parameter of the network still receives its gradient in
    loss.backward() (the reference's autograd graph reaches it too), and the optimiser, built
    on the network's parameters, leaves it alone."""
    import torch_de_solver_gb300 as T
    g = golden('inverse_burgers_ag')
    builder = cases.GOLDEN_CASES['inverse_burgers_ag']
    loss, _, onet = _oracle_fp64(builder, g['weights'], drop=('lam1',))
    d, bc, eq, net, kw = builder(T)
    set_flat_weights(net, g['weights'])
    lam1 = net.lam1
    del net._parameters['lam1']
    model = T.Model(net, d, eq, bc)
    kw = dict(kw)
    model.compile(kw.pop('mode'), **kw)
    l, _ = model.solution_cls.evaluate()
    l.backward()
    assert rel(l.item(), loss) < 1e-5
    ref_lam1 = eq.equation_lst[0]['+u*du/dx']['coeff']
    assert ref_lam1 is lam1
    want = float(g['grad64'][0])
    assert abs(float(lam1.grad) - want) < 1e-4 * abs(want), (float(lam1.grad), want)
    before = float(lam1.detach())
    model.train(T.Optimizer('Adam', {'lr': 1e-3}), 4)
    assert float(lam1.detach()) == before
    assert float(net.lam2.detach()) != float(g["weights"][1])


@pytest.mark.gpu
@pytest.mark.parametrize('precision', ['fp32', '3xtf32'])
def test_batched_inverse_solves_match_oracle(precision):
    """Solves with different data and coefficient values in one launch: per-solve loss and
    gradient (device order: network, then coefficients) against the FP64 oracle."""
    import torch_de_solver_gb300 as T
    models, refs = [], []
    for i in range(3):
        b = lambda api, dtype='float32', i=i: cases.inverse_burgers_ag(api, n=16 + 2 * i,
                                                                       seed=20 + i, dtype=dtype)
        d, bc, eq, net, kw = b(T)
        with torch.no_grad():
            net.lam1.fill_(1.0 + 0.5 * i)
        models.append(T.Model(net, d, eq, bc))
        w = torch.nn.utils.parameters_to_vector(net.parameters()).detach().numpy()
        loss, lossn, onet = _oracle_fp64(b, w)
        gr = torch.cat([p.grad.reshape(-1) for p in onet.parameters()]).numpy()
        refs.append((loss, lossn, np.concatenate([gr[2:], gr[:2]])))
    bm = T.BatchedModel(models)
    bm.compile('autograd', lambda_operator=1, lambda_bound=100, precision=precision)
    losses = bm.evaluate(with_grad=True).cpu().numpy()
    P = bm.plan.n_params
    grads = bm.grad.view(len(models), P).cpu().numpy()
    for i, (l, ln, gr) in enumerate(refs):
        assert rel(losses[i, 0], l) < 1e-5, (i, losses[i, 0], l)
        assert rel(grads[i], gr) < 1e-5, (i, rel(grads[i], gr))
        assert rel(grads[i][-2:], gr[-2:]) < 1e-4, (i, grads[i][-2:], gr[-2:])
    l0 = losses[:, 0].copy()
    bm.train(lr=1e-3, epochs=20)
    l1 = bm.evaluate().cpu().numpy()[:, 0]
    assert (l1 < l0).all(), (l0, l1)

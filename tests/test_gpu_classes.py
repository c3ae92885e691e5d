"""Every compile-time jet class on the GPU: one small autograd problem per class whose residual site
has that layout, so the tensor-core and FP32 kernel variants of that class run. Loss and gradient
against the oracle in FP64 (relative 1e-5, FP32 tolerance) for the split-TF32 and FP32 paths, and
the compiled jets against the table-driven jets of the same build (relative 1e-6) for both."""
import numpy as np
import pytest
import torch

import cases
from helpers import build_model, rel
from oracle import oracle as O

TOL = 1e-5


def _loss_grad(T, builder, precision):
    model = build_model(T, builder=builder, precision=precision)
    loss, _ = model.solution_cls.evaluate()
    loss.backward()
    grad = torch.cat([p.grad.reshape(-1) for p in model.net.parameters()]).cpu().numpy()
    return loss.item(), grad, model.solution_cls.op.cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize('name', list(cases.CLASS_CASES))
def test_class_against_oracle_and_tables(name, monkeypatch):
    import torch_de_solver_gb300 as T
    builder, _ = cases.CLASS_CASES[name]
    prob, onet = O.build_problem(builder, dtype='float64')
    l64, _, g64, r = O.loss_and_grad(prob, onet)
    g64, op64 = g64.numpy(), r['op'].detach().numpy()
    l3, g3, op3 = _loss_grad(T, builder, '3xtf32')
    l1, g1, _ = _loss_grad(T, builder, 'fp32')
    print(f'{name}: 3xtf32 loss {rel(l3, l64):.2e} grad {rel(g3, g64):.2e}; '
          f'fp32 loss {rel(l1, l64):.2e} grad {rel(g1, g64):.2e}')
    assert np.isfinite(g3).all()
    assert rel(l3, l64) < TOL and rel(g3, g64) < TOL
    assert rel(l1, l64) < TOL and rel(g1, g64) < TOL
    assert op3.shape == op64.shape
    assert np.abs(op3 - op64).max() <= 1e-5 * (1 + np.abs(op64).max())
    monkeypatch.setenv('TDG_JET_TABLES', '1')
    lt, gt, _ = _loss_grad(T, builder, '3xtf32')
    assert rel(l3, lt) < 1e-6 and rel(g3, gt) < 1e-6
    lt1, gt1, _ = _loss_grad(T, builder, 'fp32')
    assert rel(l1, lt1) < 1e-6 and rel(g1, gt1) < 1e-6

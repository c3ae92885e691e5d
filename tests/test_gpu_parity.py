"""GPU parity: loss, normalized loss, parameter gradient and fields of the fused kernel against
fixtures produced by the reference itself (FP64 run of the same weights) and against the oracle.
Tolerance: relative 1e-5 for loss and gradient (FP32 path vs FP64 reference)."""
import numpy as np
import pytest
import torch

import cases
from helpers import build_model, golden, rel

TOL = 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize('name', list(cases.GOLDEN_CASES))
def test_loss_and_gradient_match_reference(name):
    import torch_de_solver_gb300 as T
    g = golden(name)
    model = build_model(T, name, weights=g['weights'])
    sol = model.solution_cls
    loss, lossn = sol.evaluate()
    loss.backward()
    grad = torch.cat([p.grad.reshape(-1) for p in model.net.parameters()]).cpu().numpy()
    assert rel(loss.item(), g['loss64']) < TOL, (loss.item(), float(g['loss64']))
    assert rel(lossn.item(), g['lossn64']) < TOL, (lossn.item(), float(g['lossn64']))
    assert rel(grad, g['grad64']) < TOL, rel(grad, g['grad64'])
    op = sol.op.cpu().numpy()
    assert op.shape[0] == int(g['n_op'])
    ref_op = g['op64']
    assert np.abs(op[:len(ref_op)] - ref_op).max() <= 1e-4 * (1 + np.abs(ref_op).max())
    assert rel((op.astype(np.float64) ** 2).sum(0), g['op_sumsq64']) < TOL
    bval = sol.bval.cpu().numpy()
    assert bval.shape == g['bval64'].shape
    assert list(sol.bval_keys) == [str(k) for k in g['bval_keys']]


@pytest.mark.gpu
@pytest.mark.parametrize('name', ['heat_nn', 'burgers_ag'])
def test_forward_only_matches_fused(name):
    import torch_de_solver_gb300 as T
    g = golden(name)
    model = build_model(T, name, weights=g['weights'])
    with torch.no_grad():
        l0, n0 = model.solution_cls.evaluate()
    l1, n1 = model.solution_cls.evaluate()
    assert abs(l0.item() - l1.item()) <= 1e-7 * abs(l1.item())
    assert rel(l0.item(), g['loss64']) < TOL

"""Plain form (one launch per layer operation, activations in device memory) against the
reference's FP64 fixtures and against the fused kernel on the same weights."""
import numpy as np
import pytest
import torch

import cases
from helpers import build_model, golden, rel


@pytest.mark.gpu
@pytest.mark.parametrize('name', list(cases.GOLDEN_CASES))
def test_plain_form_matches_reference(name):
    import torch_de_solver_gb300 as T
    g = golden(name)
    model = build_model(T, name, weights=g['weights'], form='plain')
    sol = model.solution_cls
    loss, lossn = sol.evaluate()
    loss.backward()
    grad = torch.cat([p.grad.reshape(-1) for p in model.net.parameters()]).cpu().numpy()
    assert rel(loss.item(), g['loss64']) < 1e-5
    assert rel(lossn.item(), g['lossn64']) < 1e-5
    assert rel(grad, g['grad64']) < 1e-5, rel(grad, g['grad64'])
    op = sol.op.cpu().numpy()
    assert rel((op.astype(np.float64) ** 2).sum(0), g['op_sumsq64']) < 1e-5

"""The oracle (CPU restatement) against fixtures produced by executing the reference itself."""
import numpy as np
import pytest
import torch

import cases
from helpers import golden, rel, set_flat_weights
from oracle import oracle as O


@pytest.mark.parametrize('name', list(cases.GOLDEN_CASES))
@pytest.mark.parametrize('dtype', ['float32', 'float64'])
def test_oracle_matches_reference(name, dtype):
    g = golden(name)
    prob, net = O.build_problem(cases.GOLDEN_CASES[name], dtype)
    set_flat_weights(net, g['weights'])
    net.to(torch.float32 if dtype == 'float32' else torch.float64)
    loss, lossn, grad, r = O.loss_and_grad(prob, net)
    suf = '32' if dtype == 'float32' else '64'
    tol = 1e-6 if dtype == 'float32' else 1e-12
    assert rel(loss, g['loss' + suf]) < tol
    assert rel(lossn, g['lossn' + suf]) < tol
    assert rel(grad.detach().double().numpy(), g['grad' + suf]) < tol
    if dtype == 'float64':
        op = r['op'].detach().numpy()
        assert np.allclose(op[:len(g['op64'])], g['op64'], rtol=0, atol=1e-12)
        assert np.allclose(r['bval'].detach().numpy(), g['bval64'], atol=1e-12)
        assert np.allclose(r['true_bval'].detach().numpy(), g['true_bval64'], atol=1e-12)
        assert r['keys'] == [str(k) for k in g['bval_keys']]


@pytest.mark.parametrize('name', ['heat_nn', 'burgers_ag', 'kdv_ag', 'inverse_burgers_ag',
                                  'allen_cahn_causal_ag', 'allen_cahn_batch_ag',
                                  'allen_cahn_batch_causal_ag', 'heat_causal_nn',
                                  'kovasznay_causal_ag', 'inverse_burgers_batch_ag'])
def test_oracle_training_curve(name):
    """Model.train(6) with Adam(lr=1e-3): five closure losses, then the final weights."""
    g = golden(name)
    prob, net = O.build_problem(cases.GOLDEN_CASES[name], 'float32')
    set_flat_weights(net, g['weights'])
    seen = O.train_adam(prob, net, 1e-3, 6)
    assert np.allclose(seen, g['curve32'], rtol=2e-6)
    w = torch.nn.utils.parameters_to_vector(net.parameters()).detach().numpy()
    assert rel(w, g['final32']) < 1e-6


def test_fd_stencils_match_reference_tables():
    """Heat 'NN' stencils: u_t -> shifts (t+1, t-1) weights +-1/(2h); u_xx -> (x+2, x, x, x-2)
    weights (1, -1, -1, 1)/(4h^2) (tedeous/finite_diffs.py:59-117)."""
    h = 0.05
    sh, w = O.stencil([1], 2, 'central', '1', h)
    assert sh == [[0, 1], [0, -1]] and np.allclose(w, [10, -10])
    sh, w = O.stencil([0, 0], 2, 'central', '1', h)
    assert sh == [[2, 0], [0, 0], [0, 0], [-2, 0]] and np.allclose(w, [100, -100, -100, 100])
    sh, w = O.stencil([0], 2, 'fb', '2', h)
    assert sh == [[2, 0], [1, 0], [0, 0]] and np.allclose(w, [30, -40, 10])


@pytest.mark.parametrize('name', ['kovasznay_ag', 'burgers_ag', 'sweep_ag', 'kdv_ag'])
def test_chunked_oracle_matches_reference(name):
    """The chunked evaluation used as the checker at a million points (the residual summed chunk
    by chunk, tedeous/losses.py:58) reproduces the reference's FP64 loss and gradient."""
    g = golden(name)
    prob, net = O.build_problem(cases.GOLDEN_CASES[name], 'float64')
    set_flat_weights(net, g['weights'])
    net.to(torch.float64)
    loss, lossn, grad, sumsq = O.loss_and_grad_chunked(prob, net, chunk=997)
    assert rel(loss, g['loss64']) < 1e-12
    assert rel(lossn, g['lossn64']) < 1e-12
    assert rel(grad.detach().numpy(), g['grad64']) < 1e-12
    assert rel(sumsq.numpy(), g['op_sumsq64']) < 1e-12

"""Long training runs against the reference's own: the benchmark configs C1 (heat u_t = u_xx,
'NN' mode, 2000 epochs) and C2 (Burgers, 'autograd', 5000 epochs), Adam(lr=1e-3) from the same
seeded weights through Model.train (fused loss+gradient, fused Adam, CUDA-graph replay). The
reference's trained solution on the grid comes from executing it
(tests/golden/make_golden.py --trained). Two FP32 trainings that differ only in summation order
drift apart over thousands of Adam steps; the bounds below are the measured drift with margin,
stated per case, and the heat solution's error against the closed form exp(-pi^2 t) sin(pi x)
must equal the reference's to within the same drift."""
import math
import os

import numpy as np
import pytest
import torch

from helpers import GOLDEN, build_model, rel

# relative L2 distance between our trained u and the reference's trained u on the grid
DRIFT_BOUND = {'heat_nn': 2e-3, 'burgers_ag': 2e-2}


def _trained(name):
    return np.load(os.path.join(GOLDEN, f'trained_{name}.npz'))


@pytest.mark.gpu
@pytest.mark.parametrize('precision', ['3xtf32', 'fp32'])
@pytest.mark.parametrize('name', ['heat_nn', 'burgers_ag'])
def test_trained_solution_matches_the_reference_training(name, precision):
    import torch_de_solver_gb300 as T
    g = _trained(name)
    epochs = int(g['epochs'])
    model = build_model(T, name, weights=g['weights'], precision=precision)
    seen = []

    class Record(T.Callback):
        def on_epoch_end(self, logs=None):
            if self.model.t % 100 == 0:
                seen.append((self.model.t, float(self.model.cur_loss.reshape(-1)[0])))

    model.train(T.Optimizer('Adam', {'lr': 1e-3}), epochs, callbacks=[Record()])
    grid = torch.as_tensor(g['grid'], device='cuda')
    with torch.no_grad():
        u = model.net(grid).double().cpu().numpy()
    drift = rel(u, g['u'])
    ref_curve = g['curve']
    ours = np.array(seen)
    curve_drift = float(np.max(np.abs(ours[:, 1] - ref_curve[:, 1]) / np.abs(ref_curve[:, 1])))
    msg = (f'{name} {precision} {epochs} epochs: |u - u_ref| / |u_ref| = {drift:.2e}, loss curve '
           f'max rel gap {curve_drift:.2e}, final loss {ours[-1, 1]:.6g} (reference '
           f'{ref_curve[-1, 1]:.6g}); curves (epoch, ours, reference): '
           f'{[(int(a), float(b), float(c)) for a, b, c in zip(ours[:, 0], ours[:, 1], ref_curve[:, 1])]}')
    if name == 'heat_nn':
        x, t = g['grid'][:, 0], g['grid'][:, 1]
        exact = np.exp(-math.pi ** 2 * t) * np.sin(math.pi * x)
        e_ours, e_ref = rel(u[:, 0], exact), rel(g['u'][:, 0], exact)
        msg += f'; error vs exp(-pi^2 t) sin(pi x): ours {e_ours:.4e}, reference {e_ref:.4e}'
        assert abs(e_ours - e_ref) <= DRIFT_BOUND[name], msg
    print(msg)
    assert drift <= DRIFT_BOUND[name], msg
    assert curve_drift <= 5 * DRIFT_BOUND[name], msg

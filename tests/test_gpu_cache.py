"""Cache interop: many cached networks evaluated on one problem in one launch per network shape
(Solution.evaluate_many), against one evaluate per network and against the FP64 oracle, and the
Cache callback built on it (tedeous/callbacks/cache.py)."""
import copy
import glob
import os

import numpy as np
import pytest
import torch

import cases
from helpers import build_model, golden, rel
from oracle import oracle as O


def _nets(widths_list, seed0=100):
    return [cases.mlp(list(w), seed0 + i) for i, w in enumerate(widths_list)]


def _one_by_one(sol, nets):
    keep = sol.model
    out = []
    for n in nets:
        sol._model_change(n)
        loss, lossn = sol.evaluate(save_graph=False)
        out.append((loss.item(), lossn.item()))
    sol._model_change(keep)
    return np.array(out)


@pytest.mark.gpu
@pytest.mark.parametrize('precision,form', [('fp32', 'fused'), ('3xtf32', 'fused'),
                                            ('fp32', 'plain')])
@pytest.mark.parametrize('name', ['burgers_ag', 'allen_cahn_causal_ag', 'inverse_burgers_ag',
                                  'heat_nn'])
def test_evaluate_many_equals_one_by_one(name, precision, form):
    """Networks of two shapes, each shape in one launch, against one evaluate per network (the
    reference's loop); trainable coefficients keep the solver's values for every network."""
    import torch_de_solver_gb300 as T
    g = golden(name)
    model = build_model(T, name, weights=g['weights'], precision=precision, form=form)
    sol = model.solution_cls
    w = [m.in_features for m in model.net if isinstance(m, torch.nn.Linear)][0]
    d_out = [m.out_features for m in model.net if isinstance(m, torch.nn.Linear)][-1]
    nets = _nets([(w, 32, 32, 32, d_out), (w, 16, 16, d_out), (w, 32, 32, 32, d_out),
                  (w, 16, 16, d_out), (w, 32, 32, 32, d_out)])
    many = sol.evaluate_many(nets).cpu().numpy()
    ref = _one_by_one(sol, nets)
    assert rel(many[:, 0], ref[:, 0]) < 1e-5, (many, ref)
    assert rel(many[:, 1], ref[:, 1]) < 1e-5
    # every network's loss against the FP64 oracle of the same problem and weights (the
    # problem's own trainable coefficients keep their initial values, as in the solver)
    for k, net in enumerate(nets):
        prob, _ = O.build_problem(cases.GOLDEN_CASES[name], 'float64')
        loss64, lossn64, _, _ = O.loss_and_grad(prob, copy.deepcopy(net).double().cpu())
        assert rel(many[k, 0], loss64) < 1e-5, (k, many[k, 0], loss64)
        assert rel(many[k, 1], lossn64) < 1e-5, (k, many[k, 1], lossn64)
    l0, _ = sol.evaluate(save_graph=False)   # the solver's own network is untouched
    assert rel(l0.item(), g['loss64']) < 1e-5


@pytest.mark.gpu
def test_cache_callback_takes_the_best_network(tmp_path):
    """Networks saved under the reference's file names; the Cache callback evaluates them, starts
    from the one with the smallest loss, and points the model's save folder at the cache."""
    import torch_de_solver_gb300 as T
    model = build_model(T, builder=cases.burgers_ag, n=20)
    cache_dir = str(tmp_path) + '/'
    nets = _nets([(2, 32, 32, 32, 32, 1)] * 3 + [(2, 16, 1)], seed0=7)
    with torch.no_grad():   # the network of the other shape is far off: never the best
        nets[3][-1].bias.fill_(10.0)
    saver = T.Model(None, None, None, None)
    saver._save_dir = cache_dir
    for i, n in enumerate(nets):
        saver.net = n
        saver._model_save(True, f'net{i}')
    files = sorted(glob.glob(cache_dir + '\\*.tar'))
    assert len(files) == 4 and all(os.path.basename(f).startswith('\\') for f in files)
    losses = _one_by_one(model.solution_cls, nets)[:, 0]
    order = [int(os.path.basename(f)[4:-4]) for f in glob.glob(cache_dir + '\\*.tar')]
    best = order[int(np.argmin([losses[i] for i in order]))]
    model.train(T.Optimizer('Adam', {'lr': 1e-3}), 1,
                callbacks=[T.Cache(cache_dir=cache_dir, model_randomize_parameter=0)])
    got = torch.nn.utils.parameters_to_vector(model.net.parameters()).detach().cpu()
    want = torch.nn.utils.parameters_to_vector(nets[best].parameters()).detach().cpu()
    assert torch.equal(got, want)
    assert model._save_dir == cache_dir
    l1, _ = model.solution_cls.evaluate(save_graph=False)
    assert rel(l1.item(), losses[best]) < 1e-6


@pytest.mark.gpu
def test_cache_retrain_fits_another_architecture(tmp_path):
    """A cached network of another shape is not reused directly: the solver's network is fitted
    to its outputs on the grid (scheme_interp)."""
    import torch_de_solver_gb300 as T
    model = build_model(T, builder=cases.burgers_ag, n=10)
    other = cases.mlp([2, 8, 1], 3)
    with torch.no_grad():
        for p in other.parameters():
            p.mul_(0.1)
    pre = T.CachePreprocessing(model)
    pre.cache_retrain({'model': other, 'model_state_dict': other.state_dict()})
    sol = model.solution_cls
    grid = sol.grid.to(sol.device)
    diff = torch.mean((other.to(sol.device)(grid) - sol.model(grid)) ** 2).item()
    assert diff <= 1e-5
    l, _ = sol.evaluate(save_graph=False)   # the device path sees the fitted network
    assert np.isfinite(l.item())

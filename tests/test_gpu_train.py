"""Model.train on the device path against the reference's own training run: 5 Adam(lr=1e-3)
steps of train(epochs=6) (the reference performs epochs - 1 steps after an initial evaluate,
tedeous/model.py:154-193). Covers the fused Adam kernel and the CUDA-graph replay of the step
(steps 4 and 5 are replays)."""
import numpy as np
import pytest
import torch

from helpers import build_model, golden, rel


@pytest.mark.gpu
@pytest.mark.parametrize('name', ['heat_nn', 'burgers_ag', 'kdv_ag', 'kovasznay_ag',
                                  'allen_cahn_causal_ag', 'allen_cahn_batch_ag',
                                  'allen_cahn_batch_causal_ag', 'heat_causal_nn',
                                  'kovasznay_causal_ag', 'inverse_burgers_batch_ag'])
def test_train_curve_and_weights_match_reference(name):
    import torch_de_solver_gb300 as T
    g = golden(name)
    model = build_model(T, name, weights=g['weights'])
    seen = []

    class Record(T.Callback):
        def on_epoch_end(self, logs=None):
            seen.append(float(self.model.cur_loss.reshape(-1)[0]))

    model.train(T.Optimizer('Adam', {'lr': 1e-3}), 6, callbacks=[Record()])
    assert len(seen) == 5
    assert rel(seen, g['curve32']) < 1e-5, (seen, g['curve32'])
    w = torch.nn.utils.parameters_to_vector(model.net.parameters()).detach().cpu().numpy()
    assert rel(w, g['final32']) < 1e-5, rel(w, g['final32'])


@pytest.mark.gpu
@pytest.mark.parametrize('name', ['burgers_ag', 'inverse_burgers_ag', 'allen_cahn_causal_ag',
                                  'kovasznay_ag'])
def test_train_at_the_default_precision_matches_reference(name):
    """The same 5 steps with the default precision (split TF32 on the tensor cores): the fused
    Adam launch and the CUDA-graph replay of the tensor-core step, including the weight packing
    and, for the causal loss, the forward and weight passes inside the graph."""
    import torch_de_solver_gb300 as T
    g = golden(name)
    model = build_model(T, name, weights=g['weights'], precision=None)
    assert model.solution_cls.precision == '3xtf32'
    seen = []

    class Record(T.Callback):
        def on_epoch_end(self, logs=None):
            seen.append(float(self.model.cur_loss.reshape(-1)[0]))

    model.train(T.Optimizer('Adam', {'lr': 1e-3}), 6, callbacks=[Record()])
    assert rel(seen, g['curve32']) < 1e-5, (seen, g['curve32'])
    w = torch.nn.utils.parameters_to_vector(model.net.parameters()).detach().cpu().numpy()
    assert rel(w, g['final32']) < 1e-5, rel(w, g['final32'])


@pytest.mark.gpu
def test_train_with_lbfgs_closure():
    """Optimizer("LBFGS") (LBFGS64, FP64 dots) through the reference closure: the loss decreases."""
    import torch_de_solver_gb300 as T
    g = golden('burgers_ag')
    model = build_model(T, 'burgers_ag', weights=g['weights'])
    l0 = model.solution_cls.evaluate()[0].item()
    model.train(T.Optimizer('LBFGS', {'lr': 1e-1, 'max_iter': 5}), 3)
    l1 = model.solution_cls.evaluate()[0].item()
    assert l1 < l0


@pytest.mark.gpu
def test_dot_f64_exact_on_integers():
    from torch_de_solver_gb300 import _lib
    a = torch.arange(1, 100001, dtype=torch.float32, device='cuda')
    out = torch.zeros(1, dtype=torch.float64, device='cuda')
    _lib.check(_lib.load().tdg_dot_f64(a.data_ptr(), a.data_ptr(), a.numel(), out.data_ptr(),
                                       torch.cuda.current_stream().cuda_stream), 'dot')
    n = 100000
    assert out.item() == n * (n + 1) * (2 * n + 1) / 6


@pytest.mark.gpu
def test_callback_weight_changes_reach_the_captured_step():
    """A callback that replaces parameter data mid-run (as the reference's EarlyStopping perturbation does):
    the next step, a CUDA-graph replay by then, trains from the new values."""
    import torch_de_solver_gb300 as T
    g = golden('burgers_ag')
    model = build_model(T, 'burgers_ag', weights=g['weights'], precision=None)
    seen = {}

    class Perturb(T.Callback):
        def on_epoch_end(self, logs=None):
            if self.model.t == 6:
                with torch.no_grad():
                    for p in self.model.net.parameters():
                        p.data = p.data + 1e-3   # new tensors, no longer views of the buffer
                # the loss of the new values from a separate model, so that nothing here makes
                # the training model's Solution copy the values back: the step itself must
                w = torch.cat([p.data.reshape(-1) for p in self.model.net.parameters()]).cpu()
                other = build_model(T, 'burgers_ag', weights=w.numpy(), precision=None)
                seen['expected'] = other.solution_cls.evaluate(save_graph=False)[0].item()
                seen['stale'] = float(self.model.cur_loss.reshape(-1)[0])
            elif self.model.t == 7:
                seen['got'] = float(self.model.cur_loss.reshape(-1)[0])

    model.train(T.Optimizer('Adam', {'lr': 1e-3}), 9, callbacks=[Perturb()])
    assert model._graph is None and model.t == 9
    assert abs(seen['got'] - seen['expected']) <= 1e-6 * abs(seen['expected']), seen
    assert abs(seen['expected'] - seen['stale']) > 1e-4 * abs(seen['stale']), seen


@pytest.mark.gpu
def test_changed_parameter_layout_raises():
    """A callback that gives a parameter another number of elements: the plans, the captured step
    and the fused Adam hold the old layout, so the next step raises instead of training stale
    parameters."""
    import torch_de_solver_gb300 as T
    from torch_de_solver_gb300 import _lib
    g = golden('burgers_ag')
    model = build_model(T, 'burgers_ag', weights=g['weights'], precision=None)

    class Grow(T.Callback):
        def on_epoch_end(self, logs=None):
            if self.model.t == 5:
                lin = self.model.net[0]
                lin.bias.data = torch.zeros(lin.bias.numel() + 1, device=lin.bias.device)

    with pytest.raises(_lib.TdgError, match='parameter layout changed'):
        model.train(T.Optimizer('Adam', {'lr': 1e-3}), 9, callbacks=[Grow()])

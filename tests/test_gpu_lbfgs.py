"""Device-resident L-BFGS (tdg_lbfgs_*): the two-loop recursion and curvature updates against an
FP64 restatement of torch.optim.LBFGS's (the optimizer the reference selects,
tedeous/optimizers/optimizer.py:50-51), the step statistics, and LBFGS64 as a whole against
torch.optim.LBFGS with and without the strong-Wolfe line search."""
import ctypes

import numpy as np
import pytest
import torch

from helpers import build_model, golden, rel


def _two_loop(g, pairs, h_diag):
    """torch.optim.LBFGS's direction in FP64: pairs = [(s, y, rho)] oldest first."""
    q = -g.clone()
    al = []
    for s, y, rho in reversed(pairs):
        a = rho * float(s @ q)
        q -= a * y
        al.append(a)
    al.reverse()
    r = q * h_diag
    for (s, y, rho), a in zip(pairs, al):
        b = rho * float(y @ r)
        r += (a - b) * s
    return r


@pytest.mark.gpu
def test_direction_matches_fp64_two_loop_with_wraparound_and_rejections():
    from torch_de_solver_gb300 import _lib
    lib = _lib.load()
    n, hist = 10_001, 3
    h = ctypes.c_void_p()
    _lib.check(lib.tdg_lbfgs_create(n, hist, ctypes.byref(h)), 'create')
    stream = torch.cuda.current_stream().cuda_stream
    gen = torch.Generator().manual_seed(5)
    pairs, h_diag, n_push, accepted, rejected = [], 1.0, 0, 0, 0
    g_prev = torch.randn(n, generator=gen)
    d_prev = torch.randn(n, generator=gen)
    try:
        for it in range(8):
            t = 0.5 + 0.1 * it
            # y = c * s with c in [0.5, 1.5) plus a little noise: positive curvature, accepted
            c = 0.5 + torch.rand(n, generator=gen)
            g = g_prev + c * t * d_prev + 1e-3 * torch.randn(n, generator=gen)
            if it in (2, 5):   # negative curvature: y = -s, the pair must be rejected
                g = g_prev - t * d_prev
            gd, gpd, dd = g.cuda(), g_prev.cuda(), d_prev.cuda()
            _lib.check(lib.tdg_lbfgs_push(h, gd.data_ptr(), gpd.data_ptr(), dd.data_ptr(), t,
                                          stream), 'push')
            n_push += 1
            y = (g - g_prev).double()
            s = (d_prev * t).float().double()
            ys = float(y @ s)
            if ys > 1e-10:
                if len(pairs) == hist:
                    pairs.pop(0)
                pairs.append((s, y, 1.0 / ys))
                h_diag = ys / float(y @ y)
                accepted += 1
            else:
                rejected += 1
            out = torch.empty(n, device='cuda')
            _lib.check(lib.tdg_lbfgs_direction(h, gd.data_ptr(), out.data_ptr(),
                                               min(n_push, hist), stream), 'direction')
            want = _two_loop(g.double(), pairs, h_diag)
            got = out.double().cpu()
            assert rel(got.numpy(), want.numpy()) < 1e-6, (it, rel(got.numpy(), want.numpy()))
            g_prev, d_prev = g, out.cpu()
        # the run covered both a full ring that wrapped around and rejected pairs
        assert accepted > hist and rejected >= 2, (accepted, rejected)
    finally:
        lib.tdg_lbfgs_destroy(h)


@pytest.mark.gpu
def test_stats_and_axpy():
    from torch_de_solver_gb300 import _lib
    lib = _lib.load()
    n = 66_819
    h = ctypes.c_void_p()
    _lib.check(lib.tdg_lbfgs_create(n, 2, ctypes.byref(h)), 'create')
    stream = torch.cuda.current_stream().cuda_stream
    try:
        g = torch.randn(n, device='cuda')
        d = torch.randn(n, device='cuda')
        loss = torch.tensor([0.125], device='cuda')
        out = torch.zeros(8, dtype=torch.float64, device='cuda')
        _lib.check(lib.tdg_lbfgs_stats(h, g.data_ptr(), d.data_ptr(), loss.data_ptr(),
                                       out.data_ptr(), stream), 'stats')
        o = out.cpu().numpy()
        g64, d64 = g.double(), d.double()
        assert abs(o[0] - float(g64 @ d64)) <= 1e-12 * float((g64 * d64).abs().sum())
        assert o[1] == pytest.approx(float(g64.abs().sum()), rel=1e-12)
        assert o[2] == float(g.abs().max()) and o[3] == float(d.abs().max()) and o[4] == 0.125
        x = torch.randn(n, device='cuda')
        y = torch.empty_like(x)
        _lib.check(lib.tdg_axpy(x.data_ptr(), d.data_ptr(), 0.75, y.data_ptr(), n, stream), 'axpy')
        assert torch.allclose(y, (x.double() + 0.75 * d64).float(), rtol=0, atol=0)
    finally:
        lib.tdg_lbfgs_destroy(h)


@pytest.mark.gpu
@pytest.mark.parametrize('line_search', [None, 'strong_wolfe'])
def test_lbfgs64_follows_torch_lbfgs(line_search):
    """Same closure, same hyper-parameters: LBFGS64 (device history, FP64 dots) and
    torch.optim.LBFGS (FP32 dots) take the same steps up to dot-product rounding."""
    import torch_de_solver_gb300 as T
    g = golden('burgers_ag')
    finals, losses = [], []
    for cls in (T.LBFGS64, torch.optim.LBFGS):
        model = build_model(T, 'burgers_ag', weights=g['weights'])
        opt = cls(model.net.parameters(), lr=0.5, max_iter=6, history_size=4,
                  line_search_fn=line_search)
        sol = model.solution_cls

        def closure():
            opt.zero_grad()
            loss, _ = sol.evaluate()
            loss.backward()
            return loss
        seen = [float(opt.step(closure)) for _ in range(3)]
        finals.append(torch.nn.utils.parameters_to_vector(model.net.parameters()).detach().cpu().numpy())
        losses.append(seen + [sol.evaluate(save_graph=False)[0].item()])
        st = opt.state[opt.param_groups[0]['params'][0]]
        print(cls.__name__, line_search, 'func_evals', st['func_evals'], 'n_iter', st['n_iter'],
              'losses', losses[-1])
    assert rel(finals[0], finals[1]) < 1e-4, rel(finals[0], finals[1])
    assert rel(losses[0], losses[1]) < 1e-4


@pytest.mark.gpu
def test_model_train_with_strong_wolfe_lbfgs():
    """Optimizer('LBFGS', line_search_fn='strong_wolfe') through Model.train and the reference
    closure selects LBFGS64; the loss decreases."""
    import torch_de_solver_gb300 as T
    g = golden('burgers_ag')
    model = build_model(T, 'burgers_ag', weights=g['weights'])
    l0 = model.solution_cls.evaluate()[0].item()
    optim = T.Optimizer('LBFGS', {'lr': 1.0, 'max_iter': 10, 'line_search_fn': 'strong_wolfe'})
    model.train(optim, 3)
    assert isinstance(model.optimizer, T.LBFGS64)
    l1 = model.solution_cls.evaluate()[0].item()
    assert l1 < l0

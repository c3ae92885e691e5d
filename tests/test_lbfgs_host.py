"""The host logic of LBFGS64's strong-Wolfe line search against the line search of
torch.optim.LBFGS (the optimizer the reference selects, tedeous/optimizers/optimizer.py:50-51),
both in FP64 on the CPU on smooth test functions: the same accepted step, loss and number of
evaluations."""
import numpy as np
import pytest
import torch

from torch_de_solver_gb300.optimizer import _Trial, _cubic_min, strong_wolfe


def rosenbrock(x):
    return torch.sum(100.0 * (x[1:] - x[:-1] ** 2) ** 2 + (1 - x[:-1]) ** 2)


def quartic(x):
    return torch.sum(x ** 4 - 3 * x ** 2 + 0.5 * x)


def _fg(fn, x):
    x = x.detach().clone().requires_grad_(True)
    f = fn(x)
    g, = torch.autograd.grad(f, x)
    return float(f.detach()), g


CASES = [(rosenbrock, 10, 0, 1.0), (rosenbrock, 6, 1, 1e-3), (quartic, 8, 2, 1.0),
         (quartic, 5, 3, 25.0), (rosenbrock, 4, 4, 10.0)]


@pytest.mark.parametrize('fn,n,seed,t0', CASES)
def test_strong_wolfe_matches_torch(fn, n, seed, t0):
    from torch.optim.lbfgs import _strong_wolfe
    torch.manual_seed(seed)
    x0 = torch.randn(n, dtype=torch.float64)
    f0, g0 = _fg(fn, x0)
    d = -g0 / g0.abs().max()
    gtd = float(g0.dot(d))

    def obj(x, t, d):
        return _fg(fn, x + t * d)
    f_t, g_t, t_t, n_t = _strong_wolfe(obj, x0, t0, d, f0, g0, torch.tensor(gtd, dtype=torch.float64))

    def evaluate(t):
        f, g = _fg(fn, x0 + t * d)
        return _Trial(t, f, g, float(g.dot(d)), float(g.abs().max()))
    best, n_ours = strong_wolfe(evaluate, _Trial(0.0, f0, g0, gtd, None), t0,
                                float(d.abs().max()))
    assert n_ours == n_t
    assert best.t == pytest.approx(float(t_t), rel=1e-12, abs=1e-15)
    assert best.f == pytest.approx(float(f_t), rel=1e-12, abs=1e-15)
    assert np.allclose(best.g.numpy(), g_t.numpy(), rtol=1e-12, atol=1e-14)


def test_cubic_min_is_the_cubics_minimiser():
    """For f = (x - 0.3)^3 - 2 (x - 0.3) the local minimiser is 0.3 + sqrt(2/3); a cubic fitted
    through two points with exact slopes recovers it exactly."""
    f = lambda x: (x - 0.3) ** 3 - 2 * (x - 0.3)
    df = lambda x: 3 * (x - 0.3) ** 2 - 2
    m = _cubic_min(0.0, f(0.0), df(0.0), 2.0, f(2.0), df(2.0))
    assert m == pytest.approx(0.3 + (2 / 3) ** 0.5, rel=1e-12)
    # f(0) = 0, f(1) = 1, slopes 2 at both ends: the cubic is monotone (no real minimiser), so
    # the midpoint of the bounds
    assert _cubic_min(0.0, 0.0, 2.0, 1.0, 1.0, 2.0, 0.0, 4.0) == 2.0

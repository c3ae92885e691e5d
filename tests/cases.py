"""Problem definitions shared by the golden generator, the oracle tests and the GPU parity tests.

Each case is written once, in the reference's user-level format (``Domain.variable``,
``Conditions.dirichlet/periodic``, ``Equation.add`` with term dicts), and is applied to any
module set that exposes those names: the reference ``tedeous`` package (golden generation),
this package (drop-in parity) or the oracle (CPU restatement).

The workloads follow the benchmark definitions:
  heat_nn      1D heat u_t = u_xx, 'NN' mode, 21x21 grid, MLP 2-100-100-100-1, lambda_bound=100,
               h = grid step 1/20 (examples/examples_heat/example_heat_1d.py:147-151).
  burgers_ag   Burgers u_t + u u_x = (0.01/pi) u_xx, 'autograd', 101x101, MLP 2-32x4-1
               (examples/examples_burgers/example_Burgers_1d_paper.py:24-74).
  kdv_ag       KdV u_t + 6 u u_x + u_xxx = 0, 'autograd', 256x128, MLP 2-64x4-1, IC 2 sech^2(x),
               periodic u and u_x (examples/examples_korteweg_de_vries/example_KdV_periodic.py:94-160).
  sweep_ag     u_t = a u_xx + b u u_x + c u on [0,1]^2, IC sin(pi x), zero Dirichlet, MLP 2-64x3-1.
  kovasznay_ag steady 2D Navier-Stokes (Kovasznay flow, Re=20), outputs (u, v, p), MLP 2-128x5-3.
"""

import math

import numpy as np
import torch


def mlp(widths, seed, dtype=torch.float32):
    """tanh MLP as a torch.nn.Sequential of Linear/Tanh, seeded right before construction."""
    torch.manual_seed(seed)
    layers = []
    for i in range(len(widths) - 1):
        layers.append(torch.nn.Linear(widths[i], widths[i + 1]))
        if i < len(widths) - 2:
            layers.append(torch.nn.Tanh())
    return torch.nn.Sequential(*layers).to(dtype)


def heat_nn(api, n=20, seed=0, dtype='float32'):
    domain = api.Domain()
    domain.variable('x', [0, 1], n, dtype=dtype)
    domain.variable('t', [0, 1], n, dtype=dtype)
    bnd = api.Conditions()
    bnd.dirichlet({'x': [0, 1], 't': 0}, value=lambda g: torch.sin(np.pi * g[:, 0]))
    bnd.dirichlet({'x': 0, 't': [0, 1]}, value=0)
    bnd.dirichlet({'x': 1, 't': [0, 1]}, value=0)
    eq = api.Equation()
    eq.add({'du/dt': {'coeff': 1, 'du/dt': [1], 'pow': 1},
            '-d2u/dx2': {'coeff': -1, 'd2u/dx2': [0, 0], 'pow': 1}})
    net = mlp([2, 100, 100, 100, 1], seed)
    compile_kw = dict(mode='NN', lambda_operator=1, lambda_bound=100, h=1.0 / n)
    return domain, bnd, eq, net, compile_kw


def burgers_ag(api, n=100, seed=0, dtype='float32', widths=(2, 32, 32, 32, 32, 1)):
    mu = 0.01 / np.pi
    domain = api.Domain()
    domain.variable('x', [-1, 1], n, dtype=dtype)
    domain.variable('t', [0, 1], n, dtype=dtype)
    bnd = api.Conditions()
    bnd.dirichlet({'x': [-1, 1], 't': 0}, value=lambda g: -torch.sin(np.pi * g[:, 0]))
    bnd.dirichlet({'x': -1, 't': [0, 1]}, value=0)
    bnd.dirichlet({'x': 1, 't': [0, 1]}, value=0)
    eq = api.Equation()
    eq.add({'du/dt**1': {'coeff': 1., 'du/dt': [1], 'pow': 1, 'var': 0},
            '+u*du/dx': {'coeff': 1, 'u*du/dx': [[None], [0]], 'pow': [1, 1], 'var': [0, 0]},
            '-mu*d2u/dx2': {'coeff': -mu, 'd2u/dx2': [0, 0], 'pow': 1, 'var': 0}})
    net = mlp(list(widths), seed)
    compile_kw = dict(mode='autograd', lambda_operator=1, lambda_bound=1)
    return domain, bnd, eq, net, compile_kw


def burgers_nn(api, n=100, seed=0, dtype='float32'):
    domain, bnd, eq, net, kw = burgers_ag(api, n=n, seed=seed, dtype=dtype)
    kw = dict(mode='NN', lambda_operator=1, lambda_bound=1, h=2.0 / n)
    return domain, bnd, eq, net, kw


def kdv_ag(api, nx=255, nt=127, seed=0, dtype='float32', widths=(2, 64, 64, 64, 64, 1)):
    domain = api.Domain()
    domain.variable('x', [-10, 10], nx, dtype=dtype)
    domain.variable('t', [0, 1], nt, dtype=dtype)
    bnd = api.Conditions()
    bnd.dirichlet({'x': [-10, 10], 't': 0}, value=lambda g: 2.0 / torch.cosh(g[:, 0]) ** 2)
    bnd.periodic([{'x': -10, 't': [0, 1]}, {'x': 10, 't': [0, 1]}])
    bnd.periodic([{'x': -10, 't': [0, 1]}, {'x': 10, 't': [0, 1]}],
                 operator={'du/dx': {'coeff': 1, 'du/dx': [0], 'pow': 1, 'var': 0}})
    eq = api.Equation()
    eq.add({'1*du/dt**1': {'coeff': 1, 'du/dt': [1], 'pow': 1, 'var': 0},
            '6*u**1*du/dx**1': {'coeff': 6, 'u*du/dx': [[None], [0]], 'pow': [1, 1], 'var': [0, 0]},
            'd3u/dx3**1': {'coeff': 1, 'd3u/dx3': [0, 0, 0], 'pow': 1, 'var': 0}})
    net = mlp(list(widths), seed)
    compile_kw = dict(mode='autograd', lambda_operator=1, lambda_bound=10)
    return domain, bnd, eq, net, compile_kw


def sweep_params(n_solves=256, seed=0):
    """Coefficients and grid sizes of the equation-discovery sweep (one row per solve)."""
    rng = np.random.default_rng(seed)
    a = rng.uniform(0.01, 1.0, n_solves)
    b = rng.uniform(-1.0, 1.0, n_solves)
    c = rng.uniform(-0.5, 0.5, n_solves)
    nx = rng.integers(16, 129, n_solves)
    nt = rng.integers(16, 129, n_solves)
    return [dict(a=float(a[i]), b=float(b[i]), c=float(c[i]), nx=int(nx[i]), nt=int(nt[i]))
            for i in range(n_solves)]


def sweep_ag(api, a=0.5, b=0.3, c=-0.2, nx=24, nt=20, seed=1000, dtype='float32',
             widths=(2, 64, 64, 64, 1)):
    """u_t - a u_xx - b u u_x - c u = 0 on its own nx x nt grid (nx, nt node counts)."""
    domain = api.Domain()
    domain.variable('x', [0, 1], nx - 1, dtype=dtype)
    domain.variable('t', [0, 1], nt - 1, dtype=dtype)
    bnd = api.Conditions()
    bnd.dirichlet({'x': [0, 1], 't': 0}, value=lambda g: torch.sin(np.pi * g[:, 0]))
    bnd.dirichlet({'x': 0, 't': [0, 1]}, value=0)
    bnd.dirichlet({'x': 1, 't': [0, 1]}, value=0)
    eq = api.Equation()
    eq.add({'du/dt': {'coeff': 1, 'du/dt': [1], 'pow': 1, 'var': 0},
            '-a*d2u/dx2': {'coeff': -a, 'd2u/dx2': [0, 0], 'pow': 1, 'var': 0},
            '-b*u*du/dx': {'coeff': -b, 'u*du/dx': [[None], [0]], 'pow': [1, 1], 'var': [0, 0]},
            '-c*u': {'coeff': -c, 'u': [None], 'pow': 1, 'var': 0}})
    net = mlp(list(widths), seed)
    compile_kw = dict(mode='autograd', lambda_operator=1, lambda_bound=1)
    return domain, bnd, eq, net, compile_kw


KOV_RE = 20.0


def kovasznay_exact(g):
    """Closed-form Kovasznay flow (u, v, p) at points g[:, 0] = x, g[:, 1] = y."""
    re = KOV_RE
    lam = re / 2 - math.sqrt(re * re / 4 + 4 * math.pi ** 2)
    x, y = g[:, 0], g[:, 1]
    u = 1 - torch.exp(lam * x) * torch.cos(2 * math.pi * y)
    v = lam / (2 * math.pi) * torch.exp(lam * x) * torch.sin(2 * math.pi * y)
    p = 0.5 * (1 - torch.exp(2 * lam * x))
    return u, v, p


def kovasznay_ag(api, n=1023, seed=0, dtype='float32', widths=(2, 128, 128, 128, 128, 128, 3)):
    """Kovasznay flow on an (n+1)^2 grid over [-0.5, 1] x [-0.5, 1.5]; Dirichlet (u, v, p) on 4 sides."""
    nu = 1.0 / KOV_RE
    domain = api.Domain()
    domain.variable('x', [-0.5, 1.0], n, dtype=dtype)
    domain.variable('y', [-0.5, 1.5], n, dtype=dtype)
    bnd = api.Conditions()
    sides = [{'x': -0.5, 'y': [-0.5, 1.5]}, {'x': 1.0, 'y': [-0.5, 1.5]},
             {'x': [-0.5, 1.0], 'y': -0.5}, {'x': [-0.5, 1.0], 'y': 1.5}]
    for side in sides:
        for var in range(3):
            bnd.dirichlet(dict(side), value=(lambda g, k=var: kovasznay_exact(g)[k]), var=var)
    eq = api.Equation()
    continuity = {
        'du/dx': {'coeff': 1, 'du/dx': [0], 'pow': 1, 'var': 0},
        'dv/dy': {'coeff': 1, 'dv/dy': [1], 'pow': 1, 'var': 1}}
    mom_x = {
        'u*du/dx': {'coeff': 1, 'u*du/dx': [[None], [0]], 'pow': [1, 1], 'var': [0, 0]},
        'v*du/dy': {'coeff': 1, 'v*du/dy': [[None], [1]], 'pow': [1, 1], 'var': [1, 0]},
        'dp/dx': {'coeff': 1, 'dp/dx': [0], 'pow': 1, 'var': 2},
        '-nu*d2u/dx2': {'coeff': -nu, 'd2u/dx2': [0, 0], 'pow': 1, 'var': 0},
        '-nu*d2u/dy2': {'coeff': -nu, 'd2u/dy2': [1, 1], 'pow': 1, 'var': 0}}
    mom_y = {
        'u*dv/dx': {'coeff': 1, 'u*dv/dx': [[None], [0]], 'pow': [1, 1], 'var': [0, 1]},
        'v*dv/dy': {'coeff': 1, 'v*dv/dy': [[None], [1]], 'pow': [1, 1], 'var': [1, 1]},
        'dp/dy': {'coeff': 1, 'dp/dy': [1], 'pow': 1, 'var': 2},
        '-nu*d2v/dx2': {'coeff': -nu, 'd2v/dx2': [0, 0], 'pow': 1, 'var': 1},
        '-nu*d2v/dy2': {'coeff': -nu, 'd2v/dy2': [1, 1], 'pow': 1, 'var': 1}}
    eq.add(continuity)
    eq.add(mom_x)
    eq.add(mom_y)
    net = mlp(list(widths), seed)
    compile_kw = dict(mode='autograd', lambda_operator=1, lambda_bound=1)
    return domain, bnd, eq, net, compile_kw


# Small variants used for committed golden fixtures (full sizes where the reference finishes
# in seconds on CPU).
GOLDEN_CASES = {
    'heat_nn': lambda api, dtype='float32': heat_nn(api, dtype=dtype),
    'burgers_ag': lambda api, dtype='float32': burgers_ag(api, dtype=dtype),
    'burgers_nn': lambda api, dtype='float32': burgers_nn(api, n=40, dtype=dtype),
    'kdv_ag': lambda api, dtype='float32': kdv_ag(api, dtype=dtype),
    'sweep_ag': lambda api, dtype='float32': sweep_ag(api, dtype=dtype),
    'kovasznay_ag': lambda api, dtype='float32': kovasznay_ag(api, n=31, dtype=dtype),
}


# ---- boundary-condition and coefficient coverage (small grids)
def neumann_ag(api, n=16, seed=3, dtype='float32'):
    """u_t = 0.3 u_xx - x u; u(x,0) = sin(pi x); u_x(0,t) = cos t (operator BC); u(1,t) = 0."""
    domain = api.Domain()
    domain.variable('x', [0, 1], n, dtype=dtype)
    domain.variable('t', [0, 1], n, dtype=dtype)
    bnd = api.Conditions()
    bnd.dirichlet({'x': [0, 1], 't': 0}, value=lambda g: torch.sin(np.pi * g[:, 0]))
    bnd.operator({'x': 0, 't': [0, 1]}, operator={'du/dx': {'coeff': 1, 'du/dx': [0], 'pow': 1}},
                 value=lambda g: torch.cos(g[:, 1]))
    bnd.dirichlet({'x': 1, 't': [0, 1]}, value=0)
    eq = api.Equation()
    eq.add({'du/dt': {'coeff': 1, 'du/dt': [1], 'pow': 1},
            '-0.3 u_xx': {'coeff': -0.3, 'u_xx': [0, 0], 'pow': 1},
            'x u': {'coeff': lambda g: g[:, 0], 'u': [None], 'pow': 1}})
    net = mlp([2, 32, 32, 1], seed)
    return domain, bnd, eq, net, dict(mode='autograd', lambda_operator=1, lambda_bound=10)


def robin_data_ag(api, n=12, seed=4, dtype='float32'):
    """u_t = u_xx + u^2 with a Robin condition at x=1, a data condition in the interior and a
    per-point tensor coefficient."""
    domain = api.Domain()
    domain.variable('x', [0, 1], n, dtype=dtype)
    domain.variable('t', [0, 1], n, dtype=dtype)
    bnd = api.Conditions()
    bnd.dirichlet({'x': [0, 1], 't': 0}, value=lambda g: torch.sin(np.pi * g[:, 0]) ** 2)
    bnd.dirichlet({'x': 0, 't': [0, 1]}, value=0)
    bnd.robin({'x': 1, 't': [0, 1]}, value=lambda g: 0.5 * g[:, 1],
              operator={'u': {'coeff': 2.0, 'u': [None], 'pow': 1},
                        'du/dx': {'coeff': 0.5, 'du/dx': [0], 'pow': 1}})
    pts = torch.tensor([[0.25, 0.5], [0.5, 0.5], [0.75, 0.25]], dtype=torch.float64)
    bnd.data(pts, operator=None, value=torch.tensor([0.1, 0.2, 0.3]))
    eq = api.Equation()
    n_grid = (n + 1) ** 2
    eq.add({'du/dt': {'coeff': 1, 'du/dt': [1], 'pow': 1},
            '-u_xx': {'coeff': -1, 'u_xx': [0, 0], 'pow': 1},
            '-c u^2': {'coeff': -torch.linspace(0.5, 1.5, n_grid), 'u': [None], 'pow': 2}})
    net = mlp([2, 32, 32, 1], seed)
    return domain, bnd, eq, net, dict(mode='autograd', lambda_operator=1, lambda_bound=[10, 5, 2])


def neumann_nn(api, n=14, seed=5, dtype='float32'):
    """'NN' mode with an operator (Neumann) condition: one-sided second-order stencils on the
    typed boundary points, and periodic values in t."""
    domain = api.Domain()
    domain.variable('x', [0, 1], n, dtype=dtype)
    domain.variable('t', [0, 1], n, dtype=dtype)
    bnd = api.Conditions()
    bnd.dirichlet({'x': [0, 1], 't': 0}, value=lambda g: torch.sin(np.pi * g[:, 0]))
    bnd.operator({'x': 0, 't': [0, 1]}, operator={'du/dx': {'coeff': 1, 'du/dx': [0], 'pow': 1}},
                 value=0.0)
    bnd.periodic([{'x': [0, 1], 't': 0}, {'x': [0, 1], 't': 1}])
    eq = api.Equation()
    eq.add({'du/dt': {'coeff': 1, 'du/dt': [1], 'pow': 1},
            '-u_xx': {'coeff': lambda g: -0.2 - 0.1 * g[:, 0], 'u_xx': [0, 0], 'pow': 1}})
    net = mlp([2, 24, 24, 1], seed)
    return domain, bnd, eq, net, dict(mode='NN', lambda_operator=1, lambda_bound=10, h=1.0 / n)


def register_coefficients(net, values):
    """Trainable equation coefficients as parameters of the network, the way
    tedeous.models.parameter_registr (tedeous/models.py:183-196) registers them."""
    dtype = next(net.parameters()).dtype
    for name, v in values.items():
        # float32 first, like parameter_registr's .float(), so that fp32 and fp64 runs start equal
        net.register_parameter(name, torch.nn.Parameter(
            torch.tensor([v], dtype=torch.float32).to(dtype)))


def inverse_burgers_ag(api, n=20, seed=6, dtype='float32', n_data=200, mode='autograd'):
    """Inverse Burgers problem u_t + lam1 u u_x + lam2 u_xx = 0 with lam1, lam2 trainable,
    fitted to u data at seeded random points (the setup of
    examples/examples_burgers/example_burgers_1d_inverse.py:19-97, synthetic data
    u = -sin(pi x) exp(-t) instead of its data file)."""
    domain = api.Domain()
    domain.variable('x', [-1, 1], n, dtype=dtype)
    domain.variable('t', [0, 1], n, dtype=dtype)
    bnd = api.Conditions()
    gen = torch.Generator().manual_seed(seed)
    pts = torch.rand(n_data, 2, generator=gen, dtype=torch.float64) * torch.tensor([2.0, 1.0]) \
        - torch.tensor([1.0, 0.0])
    val = (-torch.sin(np.pi * pts[:, 0]) * torch.exp(-pts[:, 1])).reshape(-1, 1)
    bnd.data(bnd=pts.float(), operator=None, value=val.float())
    net = mlp([2, 32, 32, 32, 1], seed, getattr(torch, dtype))
    register_coefficients(net, {'lam1': 2.0, 'lam2': 0.2})
    eq = api.Equation()
    eq.add({'du/dt**1': {'coeff': 1., 'du/dt': [1], 'pow': 1, 'var': 0},
            '+u*du/dx': {'coeff': net.lam1, 'u*du/dx': [[None], [0]], 'pow': [1, 1],
                         'var': [0, 0]},
            '-mu*d2u/dx2': {'coeff': net.lam2, 'd2u/dx2': [0, 0], 'pow': 1, 'var': 0}})
    kw = dict(mode=mode, lambda_operator=1, lambda_bound=100)
    if mode == 'NN':
        kw['h'] = 2.0 / n
    return domain, bnd, eq, net, kw


def allen_cahn_ag(api, n=20, seed=7, dtype='float32', tol=10.0, batch_size=None,
                  widths=(2, 32, 32, 32, 1)):
    """Allen-Cahn u_t - 1e-4 u_xx + 5u^3 - 5u = 0 with time as the first variable, periodic u and
    u_x in x, the causal loss (tol) and optionally mini-batches of the collocation points (the setup
    of examples/examples_allen_cahn/example_Allen_Cahn.py:20-104 and
    example_Allen_Cahn_batches.py:102-104, with a plain tanh MLP instead of its Fourier features)."""
    domain = api.Domain()
    domain.variable('t', [0, 1], n, dtype=dtype)
    domain.variable('x', [-1, 1], n, dtype=dtype)
    bnd = api.Conditions()
    bnd.dirichlet({'x': [-1, 1], 't': 0}, value=lambda g: g[:, 1] ** 2 * torch.cos(np.pi * g[:, 1]))
    bnd.periodic([{'x': -1, 't': [0, 1]}, {'x': 1, 't': [0, 1]}])
    bnd.periodic([{'x': -1, 't': [0, 1]}, {'x': 1, 't': [0, 1]}],
                 operator={'du/dx': {'coeff': 1, 'du/dx': [1], 'pow': 1, 'var': 0}})
    eq = api.Equation()
    eq.add({'1*du/dt**1': {'coeff': 1, 'du/dt': [0], 'pow': 1, 'var': 0},
            '-0.0001*d2u/dx2**1': {'coeff': -0.0001, 'd2u/dx2': [1, 1], 'pow': 1, 'var': 0},
            '+5u**3': {'coeff': 5, 'u': [None], 'pow': 3, 'var': 0},
            '-5u**1': {'coeff': -5, 'u': [None], 'pow': 1, 'var': 0}})
    net = mlp(list(widths), seed, getattr(torch, dtype))
    kw = dict(mode='autograd', lambda_operator=1, lambda_bound=100, tol=tol)
    if batch_size is not None:
        kw['batch_size'] = batch_size
    return domain, bnd, eq, net, kw


def heat2d_ag(api, n=8, seed=9, dtype='float32'):
    """2-D heat u_t = 0.1 (u_xx + u_yy) on (x, y, t) in [0, 1]^3: three inputs, u(x, y, 0) =
    sin(pi x) sin(pi y), zero on the four sides (the sites are 3-axis, so the table-driven jets
    run)."""
    domain = api.Domain()
    domain.variable('x', [0, 1], n, dtype=dtype)
    domain.variable('y', [0, 1], n, dtype=dtype)
    domain.variable('t', [0, 1], n, dtype=dtype)
    bnd = api.Conditions()
    bnd.dirichlet({'x': [0, 1], 'y': [0, 1], 't': 0},
                  value=lambda g: torch.sin(np.pi * g[:, 0]) * torch.sin(np.pi * g[:, 1]))
    for side in ({'x': 0, 'y': [0, 1], 't': [0, 1]}, {'x': 1, 'y': [0, 1], 't': [0, 1]},
                 {'x': [0, 1], 'y': 0, 't': [0, 1]}, {'x': [0, 1], 'y': 1, 't': [0, 1]}):
        bnd.dirichlet(side, value=0)
    eq = api.Equation()
    eq.add({'du/dt': {'coeff': 1, 'du/dt': [2], 'pow': 1},
            '-0.1 u_xx': {'coeff': -0.1, 'u_xx': [0, 0], 'pow': 1},
            '-0.1 u_yy': {'coeff': -0.1, 'u_yy': [1, 1], 'pow': 1}})
    net = mlp([3, 32, 32, 1], seed, getattr(torch, dtype))
    return domain, bnd, eq, net, dict(mode='autograd', lambda_operator=1, lambda_bound=10)


def _with_kw(case, **extra):
    """A case with more compile / Model arguments (tol, batch_size)."""
    domain, bnd, eq, net, kw = case
    return domain, bnd, eq, net, dict(kw, **extra)


def heat_causal_nn(api, n=12, dtype='float32', tol=1.0):
    """The 'NN' heat problem with the causal loss (the first variable, x, plays time)."""
    domain, bnd, eq, net, kw = heat_nn(api, n=n, dtype=dtype)
    return domain, bnd, eq, net, dict(kw, tol=tol)


COVERAGE_CASES = {
    'neumann_ag': lambda api, dtype='float32': neumann_ag(api, dtype=dtype),
    'robin_data_ag': lambda api, dtype='float32': robin_data_ag(api, dtype=dtype),
    'neumann_nn': lambda api, dtype='float32': neumann_nn(api, dtype=dtype),
    'inverse_burgers_ag': lambda api, dtype='float32': inverse_burgers_ag(api, dtype=dtype),
    'allen_cahn_causal_ag': lambda api, dtype='float32': allen_cahn_ag(api, dtype=dtype),
    'allen_cahn_batch_ag': lambda api, dtype='float32': allen_cahn_ag(api, dtype=dtype, tol=0,
                                                                      batch_size=64),
    'allen_cahn_batch_causal_ag': lambda api, dtype='float32': allen_cahn_ag(api, dtype=dtype,
                                                                             batch_size=64),
    'heat_causal_nn': lambda api, dtype='float32': heat_causal_nn(api, dtype=dtype),
    # a 3-equation system under the causal loss, and trainable coefficients with mini-batches
    'kovasznay_causal_ag': lambda api, dtype='float32': _with_kw(
        kovasznay_ag(api, n=15, dtype=dtype, widths=(2, 32, 32, 32, 3)), tol=0.1),
    'inverse_burgers_batch_ag': lambda api, dtype='float32': _with_kw(
        inverse_burgers_ag(api, dtype=dtype), batch_size=100),
    'heat2d_ag': lambda api, dtype='float32': heat2d_ag(api, dtype=dtype),
}
GOLDEN_CASES.update(COVERAGE_CASES)


# ---- one small autograd problem per compile-time jet class (csrc/tdg_jetcls.h) that the benchmark
# cases above do not reach: the residual site of each is the class named, so the tensor-core kernel
# variant of that class (and its compiled jets) runs.
def class_case(kind, api, n=16, seed=11, dtype='float32'):
    one_d = kind == 'c4'
    domain = api.Domain()
    domain.variable('x', [0, 1], n, dtype=dtype)
    if not one_d:
        domain.variable('y', [0, 1], n - 2, dtype=dtype)
    bnd = api.Conditions()
    u = lambda c, term: {'coeff': c, 'term': term, 'pow': 1, 'var': 0}
    if one_d:   # u'' + u = 0, u(0) = 0, u(1) = sin 1
        bnd.dirichlet({'x': 0}, value=0)
        bnd.dirichlet({'x': 1}, value=math.sin(1.0))
        terms = {'d2u/dx2': u(1, [0, 0]), 'u': u(1, [None])}
    else:
        bnd.dirichlet({'x': 0, 'y': [0, 1]}, value=lambda g: torch.cos(g[:, 1]))
        bnd.dirichlet({'x': [0, 1], 'y': 0}, value=lambda g: torch.exp(-g[:, 0]))
        terms = {
            'c1': {'du/dx': u(1, [0]), 'u': u(1, [None])},
            'c2': {'du/dy': u(1, [1]), '0.5u': u(0.5, [None])},
            'c3': {'du/dx': u(1, [0]), 'du/dy': u(1, [1])},
            'c6': {'du/dx': u(1, [0]), '-0.1d2u/dy2': u(-0.1, [1, 1])},
            'c9': {'du/dx': u(1, [0]), 'u*du/dy': {'coeff': 1, 'term': [[None], [1]], 'pow': [1, 1],
                                                   'var': [0, 0]},
                   '0.01d3u/dy3': u(0.01, [1, 1, 1])},
            'c10': {'d2u/dx2': u(1, [0, 0]), '0.5d2u/dxdy': u(0.5, [0, 1]), 'd2u/dy2': u(1, [1, 1])},
        }[kind]
    eq = api.Equation()
    eq.add(terms)
    net = mlp([1 if one_d else 2, 32, 32, 32, 1], seed)
    # a small boundary weight: the residual (the compiled jets) dominates loss and gradient
    return domain, bnd, eq, net, dict(mode='autograd', lambda_operator=1, lambda_bound=0.001)


CLASS_CASES = {   # name -> (builder, class of the residual site)
    f'class_{k}': (lambda api, dtype='float32', k=k: class_case(k, api, dtype=dtype), c)
    for k, c in (('c1', 1), ('c2', 2), ('c3', 3), ('c4', 4), ('c6', 6), ('c9', 9), ('c10', 10))
}

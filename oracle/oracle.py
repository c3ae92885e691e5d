"""CPU oracle for the TEDEouS training hot path (test infrastructure only).

This module is the oracle. Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline
leg use it; the product package never imports it. It restates, in plain PyTorch on the CPU, the
reference algorithm for one loss evaluation and its parameter gradient:

  grid build            tedeous/data.py:41-107          (linspace(n+1), cartesian product)
  boundary subgrids     tedeous/data.py:241-323         (per-variable value / range / tensor)
  point typing          tedeous/points_type.py:22-125   (Delaunay hull test, 1e-4 probe)
  FD stencils           tedeous/finite_diffs.py:9-268   (first order central/one-sided, "second order")
  NN term evaluation    tedeous/derivative.py:30-58     (one MLP forward per stencil point)
  autograd evaluation   tedeous/derivative.py:74-132    (nested torch.autograd.grad)
  operator residual     tedeous/eval.py:143-193
  boundary conditions   tedeous/eval.py:283-461         (dirichlet/operator/periodic/robin/data)
  padding by type       tedeous/eval.py:55-87, tedeous/utils.py:257-290
  lambdas and loss      tedeous/input_preprocessing.py:14-43, tedeous/losses.py:38-135
  train loop            tedeous/model.py:134-193        (initial evaluate, then epochs-1 steps)

The operation sequence follows the reference (same term order, same MLP calls, same nested
gradients), so an fp32 run of this oracle also serves as the timed CPU baseline of that path.
Parity of this restatement is pinned by tests/test_oracle_golden.py against fixtures produced
by executing the reference itself (tests/golden/make_golden.py).

For the largest parity cases (a million collocation points) the checker moves a problem to a CUDA
device (Problem.to) and evaluates the residual in chunks of points (loss_and_grad_chunked): the
reference's operator loss is a mean over points (tedeous/losses.py:58), so the loss and its
gradient are sums of per-chunk parts. The arithmetic is the same restatement; only where it runs
changes.
"""

from copy import deepcopy

import numpy as np
import torch

_DTYPES = {'float32': torch.float32, 'float64': torch.float64, 'float16': torch.float16}


# ----------------------------------------------------------------------------- problem data
class Domain:
    """Uniform grid definition (tedeous/data.py:33-107)."""

    def __init__(self, type='uniform'):
        self.type = type
        self.variable_dict = {}

    def variable(self, variable_name, variable_set, n_points, dtype='float32'):
        dt = _DTYPES.get(dtype, dtype)
        if isinstance(variable_set, torch.Tensor):
            self.variable_dict[variable_name] = variable_set.to(dt)
        else:
            lo, hi = variable_set
            self.variable_dict[variable_name] = torch.linspace(lo, hi, n_points + 1, dtype=dt)

    def build(self, mode):
        axes = list(self.variable_dict.values())
        if len(axes) == 1:
            return axes[0].reshape(-1, 1)
        return torch.cartesian_prod(*axes)


class Conditions:
    """Boundary-condition definitions (tedeous/data.py:110-323)."""

    def __init__(self):
        self.conditions_lst = []

    def dirichlet(self, bnd, value, var=0):
        self.conditions_lst.append(dict(bnd=bnd, bop=None, bval=value, var=var, type='dirichlet'))

    def operator(self, bnd, operator, value):
        self.conditions_lst.append(dict(bnd=bnd, bop=unify(operator), bval=value, var=0,
                                        type='operator'))

    def periodic(self, bnd, operator=None, var=0):
        self.conditions_lst.append(dict(bnd=bnd, bop=None if operator is None else unify(operator),
                                        bval=torch.tensor([0.]), var=var if operator is None else 0,
                                        type='periodic'))

    def robin(self, bnd, value, operator=None, var=0):
        self.conditions_lst.append(dict(bnd=bnd, bop=unify(operator), bval=value, var=var,
                                        type='robin'))

    def data(self, bnd, operator, value, var=0):
        self.conditions_lst.append(dict(bnd=bnd, bop=None if operator is None else unify(operator),
                                        bval=value, var=var, type='data'))


class Equation:
    def __init__(self):
        self.equation_lst = []

    def add(self, eq):
        self.equation_lst.append(eq)


def unify(equation):
    """Term normalisation: derivative/pow/var become per-factor lists
    (tedeous/input_preprocessing.py:52-81). The derivative key is the term's second key."""
    for label in equation:
        term = equation[label]
        key = list(term.keys())[1]
        if 'var' not in term:
            if isinstance(term['pow'], list):
                term['var'] = [0] * len(term['pow'])
            else:
                term[key] = [term[key]]
                term['pow'] = [term['pow']]
                term['var'] = [0]
            continue
        if not isinstance(term['pow'], list):
            term[key] = [term[key]]
            term['pow'] = [term['pow']]
            term['var'] = [term['var']]
    return equation


def _restore_params(prepared, original):
    """Trainable (nn.Parameter) coefficients go back into the copied operator, so that the loss
    reaches the caller's parameters (tedeous/solution.py:91-107, _operator_coeff)."""
    for key, term in original.items():
        if isinstance(term['coeff'], torch.nn.Parameter):
            prepared[key]['coeff'] = term['coeff']
    return prepared


def _bnd_grid(bnd, variable_dict, dtype):
    """Boundary subgrid of one condition (tedeous/data.py:241-286)."""
    if isinstance(bnd, torch.Tensor):
        g = bnd.to(dtype)
    else:
        parts = []
        for name, axis in variable_dict.items():
            spec = bnd[name]
            if isinstance(spec, torch.Tensor):
                parts.append(spec.to(dtype))
            elif isinstance(spec, (int, float)):
                parts.append(torch.tensor([spec]).to(dtype))
            else:
                lo, hi = spec
                parts.append(axis[(axis >= lo) & (axis <= hi)].to(dtype))
        g = torch.cartesian_prod(*parts).to(dtype)
    if g.dim() == 1:
        g = g.reshape(-1, 1)
    return g


def build_conditions(conds, variable_dict):
    """Evaluate subgrids and boundary values once (tedeous/data.py:288-323)."""
    dtype = next(iter(variable_dict.values())).dtype
    out = []
    for c in deepcopy(conds):
        if c['type'] == 'periodic':
            c['bnd'] = [_bnd_grid(b, variable_dict, dtype) for b in c['bnd']]
        else:
            c['bnd'] = _bnd_grid(c['bnd'], variable_dict, dtype)
        v = c['bval']
        if isinstance(v, torch.Tensor):
            c['bval'] = v.to(dtype)
        elif isinstance(v, (int, float)):
            c['bval'] = (torch.ones_like(c['bnd'][:, 0]) * v).to(dtype)
        elif callable(v):
            c['bval'] = v(c['bnd']).to(dtype)
        out.append(c)
    return out


# ----------------------------------------------------------------------------- NN-mode pieces
def point_types(grid):
    """'central' or an f/b string per grid point (tedeous/points_type.py:40-106)."""
    n, d = grid.shape
    if d == 1:
        return ['central'] * n
    from scipy.spatial import Delaunay
    tri = Delaunay(grid.cpu().numpy())
    inside = []
    for axis in range(d):
        for sgn in (1.0, -1.0):
            g = grid.clone()
            g[:, axis] = grid[:, axis] + sgn * 0.0001
            inside.append(tri.find_simplex(g.cpu().numpy()) >= 0)
    inside = np.stack(inside, 1)
    types = []
    for i in range(n):
        if inside[i].all():
            types.append('central')
        else:
            types.append(''.join('f' if inside[i, 2 * a] else 'b' for a in range(d)))
    return types


def grid_sort(grid):
    """Typed subgrids in grid order; types iterate in sorted order (the reference iterates a
    Python set of the type names, tedeous/points_type.py:108-125)."""
    types = point_types(grid)
    out = {}
    for t in sorted(set(types)):
        out[t] = torch.stack([grid[i] for i in range(len(types)) if types[i] == t])
    return out


def bnd_sort(grid_dict, b):
    """Boundary points split by the type of the equal grid point (tedeous/points_type.py:127-157)."""
    if isinstance(b, list):
        return [bnd_sort(grid_dict, x) for x in b]
    out = {}
    for t, pts in grid_dict.items():
        sel = [p for p in b if (p == pts).all(dim=1).any()]
        if sel:
            out[t] = torch.stack(sel)
    return out


def stencil(term, nvars, ptype, order_label, h):
    """Integer shift vectors and weights (tedeous/finite_diffs.py:9-268)."""
    if term == [None]:
        return [None], [1]
    if ptype == 'central':
        dirs = ['central'] * len(term)
    else:
        dirs = [ptype[a] for a in term]
    shifts = [[0] * nvars]
    weights = [1]
    if order_label == '1':
        c = 1 / (2 * h) if sorted(set(dirs))[0] == 'central' else 1 / h
        for i, axis in enumerate(term):
            new = []
            for s in shifts:
                p, m = list(s), list(s)
                if dirs[i] == 'central':
                    p[axis] += 1
                    m[axis] -= 1
                elif dirs[i] == 'f':
                    p[axis] += 1
                else:
                    m[axis] -= 1
                new += [p, m]
            shifts = new
            weights = [x for w in weights for x in (w * c, -w * c)]
    else:
        c = 1 / (2 * h)
        for i, axis in enumerate(term):
            new = []
            for s in shifts:
                a, b_, z = list(s), list(s), list(s)
                step = 1 if dirs[i] == 'f' else -1
                a[axis] += 2 * step
                b_[axis] += step
                new += [a, b_, z]
            shifts = new
            if dirs[i] == 'f':
                weights = [x for w in weights for x in (3 * c * w, -4 * c * w, c * w)]
            else:
                weights = [x for w in weights for x in (-3 * c * w, 4 * c * w, -c * w)]
    return shifts, weights


def shifted(points, shift, h):
    """x + fp(k*h) axis by axis (tedeous/input_preprocessing.py:239-264, points_type.py:22-38)."""
    if shift is None:
        return points
    g = points
    for axis, k in enumerate(shift):
        g2 = g.clone()
        g2[:, axis] = g[:, axis] + k * h
        g = g2
    return g


def bndpos(grid, pts):
    """Row of `grid` equal to each point (tedeous/input_preprocessing.py:126-170)."""
    g = grid.double()
    pos = []
    for p in pts.double():
        hit = torch.where(torch.all(torch.isclose(g, p), dim=1))[0]
        pos.append(int(hit[0]) if len(hit) else int(torch.argmin(torch.linalg.norm(g - p, dim=1))))
    return pos


# ----------------------------------------------------------------------------- the problem
class Problem:
    """Prepared operator + boundary conditions + loss of one reference Solution
    (tedeous/solution.py:23-168)."""

    def __init__(self, domain, conditions, equation, mode, lambda_operator, lambda_bound,
                 h=0.001, inner_order='1', boundary_order='2', tol=0, batch_size=None):
        if mode not in ('NN', 'autograd'):
            raise NotImplementedError(mode)
        self.mode = mode
        self.grid = domain.build(mode)
        self.dtype = self.grid.dtype
        self.h = h
        self.inner_order, self.boundary_order = inner_order, boundary_order
        self.lambda_operator, self.lambda_bound = lambda_operator, lambda_bound
        ops = equation.equation_lst
        self.equations = [_restore_params(unify(deepcopy(e)), e) for e in ops]
        self.bconds = build_conditions(conditions.conditions_lst, domain.variable_dict)
        self.nvars = self.grid.shape[1]
        if mode == 'NN':
            self.grid_dict = grid_sort(self.grid)
            self.points = self.grid_dict['central']
            self.prep = [self._prep_nn(e, self.points, 'central') for e in self.equations]
            for bc in self.bconds:
                if bc['bop'] is not None:
                    sides = bnd_sort(self.grid_dict, bc['bnd'])
                    if bc['type'] == 'periodic':
                        bc['prep'] = [[(t, self._prep_nn(bc['bop'], s[t], t)) for t in s]
                                      for s in sides]
                    else:
                        bc['prep'] = [(t, self._prep_nn(bc['bop'], sides[t], t)) for t in sides]
        else:
            self.points = self.grid
            self.prep = [self._prep_ag(e) for e in self.equations]
        # causal loss: time slices = distinct values of the first coordinate of the residual
        # points (tedeous/solution.py:49-56)
        self.tol = tol
        self.n_t = len((self.grid_dict['central'] if mode == 'NN' else self.grid)[:, 0].unique())
        # mini-batches of the collocation points (tedeous/model.py:107-109, tedeous/eval.py:119-144):
        # a shuffling DataLoader with an unseeded torch.Generator over the (type-sorted) grid; each
        # residual evaluation takes the current batch and moves on, a new pass starts after the last
        if batch_size is not None and len(self.grid) < batch_size:
            batch_size = None
        self.batch_size = batch_size
        if batch_size is not None:
            from torch.utils.data import DataLoader
            sorted_grid = torch.cat(list(self.grid_dict.values())) if mode == 'NN' else self.grid
            self.loader = DataLoader(sorted_grid, batch_size=batch_size, shuffle=True,
                                     generator=torch.Generator())
            self.n_batches = len(self.loader)
            self._batches = iter(self.loader)
            self._batch = next(self._batches)

    # coefficient resolution (tedeous/input_preprocessing.py:266-295, :433-458)
    def _coeff_nn(self, coeff, pts):
        if isinstance(coeff, (int, float)):
            return coeff
        if isinstance(coeff, torch.nn.Parameter):
            # a trainable scalar; the reference indexes it like a per-point tensor here
            # (tedeous/input_preprocessing.py:285-288), which fails, so 'NN' mode with trainable
            # coefficients is an extension checked only against this restatement
            return coeff
        if isinstance(coeff, torch.Tensor):
            return coeff[bndpos(self.grid, pts)].reshape(-1, 1)
        if callable(coeff):
            return ('call', coeff, pts)
        raise NameError('"coeff" should be: torch.Tensor or callable or int or float!')

    def _prep_nn(self, eq, pts, ptype):
        label = self.inner_order if ptype == 'central' else self.boundary_order
        out = []
        for term in _restore_params(unify(deepcopy(eq)), eq).values():
            key = list(term.keys())[1]
            factors = []
            for j, d in enumerate(term[key]):
                sh, w = stencil(d, self.nvars, ptype, label, self.h)
                factors.append(([shifted(pts, s, self.h) for s in sh], w, term['var'][j],
                                term['pow'][j]))
            out.append((self._coeff_nn(term['coeff'], pts), factors))
        return out

    def _prep_ag(self, eq):
        out = []
        for term in eq.values():
            key = list(term.keys())[1]
            c = term['coeff']
            if isinstance(c, torch.nn.Parameter):
                pass   # used as it is, shape (1,) (tedeous/solution.py:91-107 puts it back)
            elif isinstance(c, torch.Tensor):
                c = c.reshape(-1, 1)
            elif not isinstance(c, (int, float)) and not callable(c):
                raise NameError('"coeff" should be: torch.Tensor or callable or int or float!')
            out.append((c, [(d, term['var'][j], term['pow'][j]) for j, d in enumerate(term[key])]))
        return out

    # term evaluation ---------------------------------------------------------------------
    @staticmethod
    def _coeff_value(c, pts):
        if isinstance(c, tuple) and c and c[0] == 'call':
            return c[1](c[2]).reshape(-1, 1)
        if callable(c) and not isinstance(c, torch.Tensor):
            return c(pts).reshape(-1, 1)
        return c

    def _apply_nn(self, net, prepared):
        """Sum over terms; each factor is sum_k net(x + shift_k)[:, var] * w_k
        (tedeous/derivative.py:30-58)."""
        total = None
        for coeff, factors in prepared:
            der = 1.
            for grids, w, var, pw in factors:
                acc = 0.
                for k, g in enumerate(grids):
                    acc = acc + net(g)[:, var].reshape(-1, 1) * w[k]
                der = der * acc ** pw if isinstance(pw, (int, float)) else pw(der * acc)
            val = self._coeff_value(coeff, None) * der
            total = val if total is None else total + val
        return total

    @staticmethod
    def _nested_grad(net, pts, var, axes):
        """d^k u_var / dx_a1..dx_ak by repeated autograd.grad (tedeous/derivative.py:74-98)."""
        pts.requires_grad = True
        f = net(pts)[:, var].sum(0)
        for ax in axes:
            g, = torch.autograd.grad(f, pts, create_graph=True)
            f = g[:, ax].sum()
        return g[:, axes[-1]].reshape(-1, 1)

    def _apply_ag(self, net, prepared, pts):
        """tedeous/derivative.py:100-132 and eval.py:143-165."""
        total = None
        for coeff, factors in prepared:
            c = coeff(pts).reshape(-1, 1) if callable(coeff) and not isinstance(coeff, torch.Tensor) \
                else coeff
            der = 1.
            for d, var, pw in factors:
                if d == [None]:
                    v = net(pts)[:, var].reshape(-1, 1)
                else:
                    v = self._nested_grad(net, pts, var, d)
                der = der * v ** pw if isinstance(pw, (int, float)) else pw(der * v)
            val = c * der
            total = val if total is None else total + val
        return total

    # residual and boundaries -------------------------------------------------------------
    def residual(self, net):
        pts = self.grid
        if self.batch_size is not None:   # 'NN' terms ignore the batch (tedeous/derivative.py:30-58)
            pts = self._batch
            try:
                self._batch = next(self._batches)
            except StopIteration:
                self._batches = iter(self.loader)
                self._batch = next(self._batches)
        if self.mode == 'NN':
            cols = [self._apply_nn(net, p).reshape(-1, 1) for p in self.prep]
        else:
            pts = pts.clone()
            cols = [self._apply_ag(net, p, pts).reshape(-1, 1) for p in self.prep]
        return cols[0] if len(cols) == 1 else torch.cat(cols, 1)

    def _bop_value(self, net, bc, side):
        """Operator applied at boundary points (tedeous/eval.py:305-327)."""
        if self.mode == 'NN':
            prep = bc['prep'] if side is None else bc['prep'][side]
            return torch.cat([self._apply_nn(net, p) for _, p in prep])
        pts = (bc['bnd'] if side is None else bc['bnd'][side]).clone()
        return self._apply_ag(net, self._prep_ag(bc['bop']), pts)

    def _bc_value(self, net, bc):
        t, var = bc['type'], bc['var']
        if t == 'dirichlet':
            return net(bc['bnd'])[:, var].reshape(-1, 1)
        if t == 'operator':
            return self._bop_value(net, bc, None)
        if t == 'periodic':
            if bc['bop'] is None:
                v = net(bc['bnd'][0])[:, var].reshape(-1, 1)
                for b in bc['bnd'][1:]:
                    v = v - net(b)[:, var].reshape(-1, 1)
                return v
            n_sides = len(bc['bnd'])
            v = self._bop_value(net, bc, 0).reshape(-1, 1)
            for s in range(1, n_sides):
                v = v - self._bop_value(net, bc, s).reshape(-1, 1)
            return v
        if t == 'data':
            if bc['bop'] is None:
                return net(bc['bnd'])[:, var].reshape(-1, 1)
            return self._bop_value(net, bc, None).reshape(-1, 1)
        if t == 'robin':
            coeffs = [term['coeff'] for term in bc['bop'].values()]
            alpha, betas = coeffs[0], coeffs[1:]
            v = alpha * net(bc['bnd'])[:, var].reshape(-1, 1)
            full = self._bop_value(net, bc, None)
            for beta in betas:
                v = v + (beta(bc['bnd']) if callable(beta) else beta) * full
            return v
        raise NotImplementedError(t)

    def boundary(self, net):
        """Values grouped by type and zero-padded to the longest column (tedeous/eval.py:433-461)."""
        vals, trues = {}, {}
        for bc in self.bconds:
            v = self._bc_value(net, bc).reshape(-1)
            tv = bc['bval'].reshape(-1)
            if bc['type'] in vals:
                vals[bc['type']] = torch.cat((vals[bc['type']], v))
                trues[bc['type']] = torch.cat((trues[bc['type']], tv))
            else:
                vals[bc['type']], trues[bc['type']] = v, tv
        keys = list(vals)
        m = max(len(v) for v in vals.values())
        pad = lambda x: torch.nn.functional.pad(x, (0, m - x.shape[-1]), value=0.0)
        bval = torch.stack([pad(vals[k]) for k in keys], 1)
        true = torch.stack([pad(trues[k]) for k in keys], 1)
        return bval, true, keys, [len(vals[k]) for k in keys]

    @staticmethod
    def _lambdas(val, lam):
        """tedeous/input_preprocessing.py:14-43 (on the device of `val`)."""
        if isinstance(lam, torch.Tensor):
            return lam.to(val.device)
        if isinstance(lam, (int, float)):
            return (torch.ones(val.shape[-1]) * lam).reshape(1, -1).to(val.device)
        return torch.tensor(lam).reshape(1, -1).to(val.device)

    def to(self, device):
        """Move every tensor of the prepared problem (grid, points, boundary subgrids and values,
        per-point coefficients, shifted grids) to `device`. Trainable coefficients stay the
        caller's parameters."""
        def mv(x):
            if isinstance(x, torch.nn.Parameter):
                return x
            if isinstance(x, torch.Tensor):
                return x.to(device)
            if isinstance(x, list):
                return [mv(v) for v in x]
            if isinstance(x, tuple):
                return tuple(mv(v) for v in x)
            if isinstance(x, dict):
                return {k: mv(v) for k, v in x.items()}
            return x
        for name in ('grid', 'points', 'grid_dict', 'prep', 'bconds'):
            if hasattr(self, name):
                setattr(self, name, mv(getattr(self, name)))
        return self

    def evaluate(self, net):
        """One reference evaluate(): returns op, bval, true_bval, loss, loss_normalized
        (tedeous/solution.py:129-168, tedeous/losses.py:84-135)."""
        op = self.residual(net)
        bval, true, keys, lens = self.boundary(net)
        dt = op.dtype
        lo = self._lambdas(op, self.lambda_operator).to(dt)
        lb = self._lambdas(bval, self.lambda_bound).to(dt)
        b_mse = torch.mean((bval - true) ** 2, 0)
        if self.tol != 0:
            loss, lossn = self._causal(op, b_mse, lb)
        else:
            op_mse = torch.mean(op ** 2, 0)
            loss = op_mse @ lo.T + b_mse @ lb.T
            with torch.no_grad():
                lossn = op_mse @ torch.ones_like(lo).T + b_mse @ torch.ones_like(lb).T
        return dict(op=op, bval=bval, true_bval=true, keys=keys, lengths=lens,
                    loss=loss, loss_normalized=lossn)


    def _causal(self, op, b_mse, lb):
        """Causal loss (tedeous/losses.py:137-182): per-point residual res = sum over equations of
        op^2 in [n_t, -1] time-slice rows, each weighted by exp(-tol * sum of res over the earlier
        slices of its column) held constant; lambda_operator is not applied. In mini-batch mode n_t
        is the number of distinct values in the first residual column (tedeous/solution.py:54
        applied to the operator); a reshape that does not fit makes every row its own slice."""
        if self.batch_size is not None:
            self.n_t = len(op[:, 0].unique())
        res = torch.sum(op ** 2, dim=1)
        try:
            res = res.reshape(self.n_t, -1)
        except RuntimeError:
            self.n_t = op.shape[0]
            res = res.reshape(self.n_t, -1)
        m = torch.triu(torch.ones((self.n_t, self.n_t), dtype=res.dtype, device=res.device),
                       diagonal=1).T
        with torch.no_grad():
            w = torch.exp(-self.tol * (m @ res))
        loss_oper = torch.mean(w * res)
        loss = loss_oper + b_mse @ lb.T
        with torch.no_grad():
            lossn = loss_oper + torch.ones_like(lb) @ b_mse
        return loss, lossn


def build_problem(builder, dtype='float32'):
    """Apply a case builder (tests/cases.py) to the oracle's own Domain/Conditions/Equation."""
    import types
    api = types.SimpleNamespace(Domain=Domain, Conditions=Conditions, Equation=Equation)
    domain, bnd, eq, net, kw = builder(api, dtype=dtype)
    kw = dict(kw)
    mode = kw.pop('mode')
    net = net.to(_DTYPES[dtype])
    return Problem(domain, bnd, eq, mode, **kw), net


def loss_and_grad(problem, net):
    """Loss, normalized loss and flattened parameter gradient (closure.py:49-64)."""
    for p in net.parameters():
        p.grad = None
    r = problem.evaluate(net)
    r['loss'].backward()
    grad = torch.cat([p.grad.reshape(-1) for p in net.parameters()])
    return float(r['loss'].detach().reshape(-1)[0]), float(r['loss_normalized'].reshape(-1)[0]), grad, r


def loss_and_grad_chunked(problem, net, chunk=131072, rows=None, with_boundary=True):
    """loss_and_grad for 'autograd'-mode problems too large for one autograd graph.

    The operator part of the reference loss is sum_eq lambda_eq * mean_N(op_eq^2)
    (tedeous/losses.py:58, :84-135), so it is accumulated chunk by chunk of residual points: each
    chunk's residual (the same nested-gradient term evaluation as evaluate(), eval.py:143-193) is
    squared, summed, scaled by lambda / N and back-propagated on its own; the gradients add up in
    p.grad. The boundary part is evaluated once in full (eval.py:433-461, losses.py:79). Returns
    (loss, loss_normalized, flat gradient, per-equation sum of op^2). Per-point tensor
    coefficients are sliced with their chunk; the causal loss and mini-batches are not covered.

    rows=(r0, r1) evaluates only those residual points (still divided by the full point count)
    and with_boundary=False leaves the boundary part out: the share of one rank when the points
    are split across devices, whose shares add up to the whole loss and gradient."""
    if problem.mode != 'autograd' or problem.tol != 0 or problem.batch_size is not None:
        raise NotImplementedError('chunked evaluation covers autograd-mode problems without the '
                                  'causal loss or mini-batches')
    for p in net.parameters():
        p.grad = None
    pts_all = problem.points
    n = pts_all.shape[0]
    n_eq = len(problem.prep)
    lo = None
    sumsq = torch.zeros(n_eq, dtype=pts_all.dtype, device=pts_all.device)
    r0, r1 = (0, n) if rows is None else rows
    for i0 in range(r0, r1, chunk):
        i1 = min(r1, i0 + chunk)
        prep = []
        for eq in problem.prep:
            terms = []
            for c, factors in eq:
                if isinstance(c, torch.Tensor) and not isinstance(c, torch.nn.Parameter) \
                        and c.shape[0] == n:
                    c = c[i0:i1]
                terms.append((c, factors))
            prep.append(terms)
        pts = pts_all[i0:i1].clone()
        cols = [problem._apply_ag(net, p, pts).reshape(-1, 1) for p in prep]
        op = torch.cat(cols, 1)
        sq = (op ** 2).sum(0)
        lo = problem._lambdas(op, problem.lambda_operator).to(op.dtype)
        (sq @ lo.reshape(-1) / n).backward()
        sumsq += sq.detach()
    op_mse = sumsq / n
    if lo is None:
        lo = problem._lambdas(sumsq.reshape(1, -1), problem.lambda_operator).to(sumsq.dtype)
    loss = float(op_mse @ lo.reshape(-1))
    lossn = float(op_mse.sum())
    if with_boundary:
        bval, true, _, _ = problem.boundary(net)
        lb = problem._lambdas(bval, problem.lambda_bound).to(bval.dtype)
        b_mse = torch.mean((bval - true) ** 2, 0)
        (b_mse @ lb.reshape(-1)).backward()
        loss += float(b_mse.detach() @ lb.reshape(-1))
        lossn += float(b_mse.detach().sum())
    grad = torch.cat([torch.zeros_like(p).reshape(-1) if p.grad is None else p.grad.reshape(-1)
                      for p in net.parameters()])
    return loss, lossn, grad, sumsq


def train_adam(problem, net, lr, epochs):
    """Model.train with Adam: initial evaluate, then epochs-1 epochs of one closure step each, or
    of n_batches steps in mini-batch mode (tedeous/model.py:154-193). Returns the loss of each
    epoch's last closure."""
    opt = torch.optim.Adam(net.parameters(), lr=lr)
    problem.evaluate(net)
    seen = []
    steps = 1 if problem.batch_size is None else problem.n_batches
    for _ in range(epochs - 1):
        opt.zero_grad()
        last = []

        def closure():
            opt.zero_grad()
            r = problem.evaluate(net)
            r['loss'].backward()
            last.append(float(r['loss'].detach().reshape(-1)[0]))
            return r['loss']
        for _ in range(steps):
            opt.step(closure)
        seen.append(last[-1])
    return seen

"""Compile-time lowering of a problem into the device description of include/tdg.h.

The reference prepares its operator once per compile (tedeous/input_preprocessing.py:173-644,
tedeous/points_type.py, tedeous/finite_diffs.py) and then re-interprets Python term dicts on
every step. Here the same preparation is reduced to *groups* of rows. A row of a group is
evaluated at one or more *sites* (a point array plus an FP32 coordinate offset); each site carries
*streams* (value and partial derivatives of the MLP outputs); an operator *program* of terms,
factors and parts combines stream outputs into the group's outputs, which the loss compares with
targets.
  'autograd' residual: one site at every grid point; streams = every derivative the terms use,
                       closed under sub-derivatives (tedeous/derivative.py:74-132, eval.py:122-123).
  'NN' residual:       rows = 'central' points; one site per distinct stencil shift; a factor is
                       sum_k w_k * u(x + shift_k * h) (tedeous/derivative.py:30-58,
                       input_preprocessing.py:239-264, :319-369).
  boundary conditions: dirichlet, operator, periodic (plain or operator), robin and data, each a
                       group whose single output joins the loss slot of its type
                       (tedeous/eval.py:283-461).
"""

from copy import deepcopy
from itertools import combinations

import numpy as np
import torch

from .data import unify_operator


# ----------------------------------------------------------------------------- FD stencils
def fd_scheme(term, nvars, ptype, order_label, h):
    """Integer shifts and weights of one derivative factor (tedeous/finite_diffs.py:9-268).

    '1' (first order): central points use +/-1 per differentiation with weight +/-1/(2h);
    one-sided 'f'/'b' axes use (+1, 0) / (0, -1) with weight +/-1/h. '2' ("second order", used
    for boundary points): 'f' uses shifts (+2, +1, 0) with weights (3, -4, 1)/(2h), 'b' the mirror
    (-2, -1, 0) with (-3, 4, -1)/(2h). Multi-axis derivatives expand the shift list
    depth-first, in the reference's order, so duplicate shifts stay as separate parts."""
    if term == [None]:
        return [None], [1.0]
    dirs = ['central'] * len(term) if ptype == 'central' else [ptype[a] for a in term]
    shifts = [[0] * nvars]
    weights = [1.0]
    if order_label == '1':
        c = 1.0 / (2.0 * h) if min(dirs) == 'central' else 1.0 / h
        for i, axis in enumerate(term):
            nxt = []
            for s in shifts:
                up, dn = list(s), list(s)
                if dirs[i] in ('central', 'f'):
                    up[axis] += 1
                if dirs[i] in ('central', 'b'):
                    dn[axis] -= 1
                nxt += [up, dn]
            shifts = nxt
            weights = [v for w in weights for v in (w * c, -w * c)]
    elif order_label == '2':
        c = 1.0 / (2.0 * h)
        for i, axis in enumerate(term):
            step = 1 if dirs[i] == 'f' else -1
            nxt = []
            for s in shifts:
                far, near = list(s), list(s)
                far[axis] += 2 * step
                near[axis] += step
                nxt += [far, near, list(s)]
            shifts = nxt
            k = (3.0, -4.0, 1.0) if dirs[i] == 'f' else (-3.0, 4.0, -1.0)
            weights = [v for w in weights for v in (k[0] * c * w, k[1] * c * w, k[2] * c * w)]
    else:
        raise ValueError(f'finite-difference order {order_label!r}')
    return shifts, weights


# ----------------------------------------------------------------------------- point typing
def point_types(grid):
    """Per point: 'central' if a 1e-4 probe along every axis and both directions stays in the
    convex hull of the grid, else one char per axis, 'f' when the + probe stays inside and 'b'
    otherwise (tedeous/points_type.py:40-106). A full cartesian grid's hull is its bounding box,
    which is tested directly; other point sets use a Delaunay triangulation as the reference does."""
    n, d = grid.shape
    if d == 1:
        return ['central'] * n
    g = grid.cpu()
    uniq = [torch.unique(g[:, a]) for a in range(d)]
    box = int(np.prod([len(u) for u in uniq])) == n
    inside = np.zeros((n, 2 * d), dtype=bool)
    if box:
        lo = torch.stack([u.min() for u in uniq])
        hi = torch.stack([u.max() for u in uniq])
        for a in range(d):
            for j, sgn in enumerate((1.0, -1.0)):
                moved = g[:, a] + sgn * 0.0001
                inside[:, 2 * a + j] = ((moved >= lo[a]) & (moved <= hi[a])).numpy()
    else:
        from scipy.spatial import Delaunay
        tri = Delaunay(g.numpy())
        for a in range(d):
            for j, sgn in enumerate((1.0, -1.0)):
                moved = g.clone()
                moved[:, a] = g[:, a] + sgn * 0.0001
                inside[:, 2 * a + j] = tri.find_simplex(moved.numpy()) >= 0
    out = []
    for i in range(n):
        if inside[i].all():
            out.append('central')
        else:
            out.append(''.join('f' if inside[i, 2 * a] else 'b' for a in range(d)))
    return out


def typed_subsets(grid):
    """{type: row indices} with types in sorted order (the reference iterates a set of type
    names, tedeous/points_type.py:108-125)."""
    types = point_types(grid)
    out = {}
    for t in sorted(set(types)):
        out[t] = [i for i, x in enumerate(types) if x == t]
    return out


def match_rows(grid, pts):
    """Row index in `grid` of every point of `pts` equal to a grid point, or -1."""
    keys = {tuple(r): i for i, r in enumerate(grid.cpu().numpy().tolist())}
    return [keys.get(tuple(r), -1) for r in pts.cpu().numpy().tolist()]


# ----------------------------------------------------------------------------- IR classes
class Site:
    def __init__(self, points, offset, streams):
        self.points = points          # key into ProblemIR.arrays
        self.offset = offset          # tuple of float32-representable floats
        self.streams = streams        # list of sorted axis tuples, () first


class Group:
    def __init__(self, kind, n_rows, n_outputs, slot_first, problem=0):
        self.kind = kind
        self.n_rows = n_rows
        self.n_outputs = n_outputs
        self.slot_first = slot_first
        self.problem = problem
        self.sites = []
        self.terms = []               # (coeff float | array key, output, [(var, power, [(site, stream, w)])])
        self.target = None            # array key of n_rows x n_outputs floats, or None (zeros)
        self.row_weight = None        # array key of n_rows per-row loss weights, or None (ones)
        self.out_key = None           # (type, position) for boundary values


def closure(keys):
    """Derivative streams closed under sub-derivatives, sorted by order, value first."""
    out = {()}
    for k in keys:
        k = tuple(sorted(k))
        for r in range(1, len(k) + 1):
            for sub in combinations(k, r):
                out.add(tuple(sorted(sub)))
    return sorted(out, key=lambda t: (len(t), t))


class ProblemIR:
    """Groups, loss slots and host arrays (float32 CPU tensors) of one compiled problem."""

    def __init__(self, d_in, d_out):
        self.d_in, self.d_out = d_in, d_out
        self.arrays = []              # float32 CPU tensors (flattened on upload)
        self.coeff_params = []        # trainable coefficients (nn.Parameter), in first-use order
        self.groups = []
        self.slots = []               # (problem, weight, weight_normalized)
        self.residual_group = None
        self.n_eq = 0
        self.bc_types = []            # type names in column order
        self.bc_parts = {}            # type -> [(group index, n_rows)] in concatenation order
        self.bc_true = {}             # type -> concatenated true values (float32)
        self.max_len = 0
        self.n_residual_rows = 0
        self.causal = None            # (tol, n_t) of the causal loss, or None

    def coeff_index(self, param):
        """Slot of a trainable coefficient (one per distinct nn.Parameter)."""
        for i, q in enumerate(self.coeff_params):
            if q is param:
                return i
        self.coeff_params.append(param)
        return len(self.coeff_params) - 1

    def add_array(self, t):
        self.arrays.append(t.detach().cpu().to(torch.float32).contiguous())
        return len(self.arrays) - 1


class CoeffParam:
    """A term coefficient scale * theta, theta a trainable scalar (an nn.Parameter of one element,
    as tedeous.models.parameter_registr makes them); `index` is theta's slot in
    ProblemIR.coeff_params."""

    def __init__(self, index, scale=1.0):
        self.index = index
        self.scale = scale


def _copy_keeping_params(eq):
    """Deep copy of an operator dict in which the trainable (nn.Parameter) coefficients stay the
    caller's objects, so that their gradient reaches them (the reference puts them back after its
    own copy, tedeous/solution.py:91-107)."""
    memo = {}
    for term in eq.values():
        c = term.get('coeff') if isinstance(term, dict) else None
        if isinstance(c, torch.nn.Parameter):
            memo[id(c)] = c
    return deepcopy(eq, memo)


def _check_coeff(coeff):
    if isinstance(coeff, torch.nn.Parameter):
        if coeff.numel() != 1:
            raise NotImplementedError('a trainable coefficient must be a single value')
        return
    if isinstance(coeff, (int, float, np.floating, np.integer)) or isinstance(coeff, torch.Tensor) \
            or callable(coeff):
        return
    raise NameError('"coeff" should be: torch.Tensor or callable or int or float!')


class Lowering:
    def __init__(self, grid, operator, bconds, mode, lambda_operator, lambda_bound, h=0.001,
                 inner_order='1', boundary_order='2', d_out=1):
        if mode not in ('NN', 'autograd'):
            raise NotImplementedError(f"mode {mode!r}")
        if grid.dtype != torch.float32:
            raise NotImplementedError('the device path computes in float32; build the Domain '
                                      'with dtype float32')
        self.grid = grid.cpu()
        self.mode = mode
        self.h = h
        self.inner_order, self.boundary_order = inner_order, boundary_order
        if isinstance(operator, dict):
            operator = [operator]
        self.equations = [unify_operator(_copy_keeping_params(e)) for e in operator]
        self.bconds = bconds
        self.lambda_operator, self.lambda_bound = lambda_operator, lambda_bound
        self.ir = ProblemIR(grid.shape[1], d_out)
        self._point_keys = {}
        self._types = None

    def _points(self, tensor, tag):
        key = (tag, tensor.data_ptr(), tuple(tensor.shape))
        if key not in self._point_keys:
            self._point_keys[key] = self.ir.add_array(tensor.reshape(tensor.shape[0], -1))
        return self._point_keys[key]

    def types(self):
        if self._types is None:
            self._types = typed_subsets(self.grid)
        return self._types

    # -- one operator (dict of terms) into a group's terms ------------------------------
    def _coeff(self, coeff, pts, rows_in_grid):
        _check_coeff(coeff)
        if isinstance(coeff, torch.nn.Parameter):
            return CoeffParam(self.ir.coeff_index(coeff))
        if isinstance(coeff, torch.Tensor):
            c = coeff.detach().cpu().reshape(-1)
            if rows_in_grid is not None:
                c = c[rows_in_grid]
            if c.numel() == 1:
                return float(c)
            if c.numel() != pts.shape[0]:
                raise ValueError('coefficient tensor does not match the points it applies to')
            return self.ir.add_array(c.to(torch.float32))
        if callable(coeff):
            return self.ir.add_array(torch.as_tensor(coeff(pts)).detach().cpu().reshape(-1)
                                     .to(torch.float32))
        return float(coeff)

    def _add_operator_ag(self, grp, eq, pts, pts_key, sign, output, site_slot):
        """'autograd' terms at one site (created on first use, indexed by site_slot)."""
        keys = []
        for term in eq.values():
            dkey = list(term.keys())[1]
            for d in term[dkey]:
                if d != [None]:
                    keys.append(tuple(d))
        streams = closure(keys)
        grp.sites.append(Site(pts_key, (0.0,) * self.ir.d_in, streams))
        site = len(grp.sites) - 1
        for term in eq.values():
            dkey = list(term.keys())[1]
            factors = []
            for j, d in enumerate(term[dkey]):
                pw = term['pow'][j]
                if not isinstance(pw, (int, float)):
                    raise NotImplementedError('callable pow is not implemented on the device path')
                sidx = 0 if d == [None] else streams.index(tuple(sorted(d)))
                factors.append((int(term['var'][j]), float(pw), [(site, sidx, 1.0)]))
            c = self._coeff(term['coeff'], pts, None)
            grp.terms.append((self._signed(c, sign), output, factors))

    def _signed(self, c, sign):
        if sign == 1:
            return c
        if isinstance(c, float):
            return -c
        if isinstance(c, CoeffParam):
            return CoeffParam(c.index, -c.scale)
        self.ir.arrays[c] = -self.ir.arrays[c]
        return c

    def _add_operator_nn(self, grp, eq, pts, pts_key, ptype, sign, output, rows_in_grid):
        """'NN' terms: one value site per distinct shift; parts keep the reference's order."""
        label = self.inner_order if ptype == 'central' else self.boundary_order
        nv = self.ir.d_in
        site_of = {}
        for term in eq.values():
            dkey = list(term.keys())[1]
            factors = []
            for j, d in enumerate(term[dkey]):
                pw = term['pow'][j]
                if not isinstance(pw, (int, float)):
                    raise NotImplementedError('callable pow is not implemented on the device path')
                shifts, weights = fd_scheme(d, nv, ptype, label, self.h)
                parts = []
                for s, w in zip(shifts, weights):
                    off = (0.0,) * nv if s is None else tuple(
                        float(np.float32(k * self.h)) for k in s)
                    if off not in site_of:
                        grp.sites.append(Site(pts_key, off, [()]))
                        site_of[off] = len(grp.sites) - 1
                    parts.append((site_of[off], 0, float(np.float32(w))))
                factors.append((int(term['var'][j]), float(pw), parts))
            c = self._coeff(term['coeff'], pts, rows_in_grid)
            grp.terms.append((self._signed(c, sign), output, factors))

    # -- residual -----------------------------------------------------------------------
    def residual(self, slot_first):
        ir = self.ir
        if self.mode == 'autograd':
            pts = self.grid
            rows = None
        else:
            rows = self.types()['central']
            pts = self.grid[rows]
        key = self._points(pts, 'residual')
        n_eq = len(self.equations)
        grp = Group('residual', pts.shape[0], n_eq, slot_first)
        for e, eq in enumerate(self.equations):
            if self.mode == 'autograd':
                # one site per equation would duplicate MLP work: merge all equations' streams
                pass
        if self.mode == 'autograd':
            keys = []
            for eq in self.equations:
                for term in eq.values():
                    dkey = list(term.keys())[1]
                    keys += [tuple(d) for d in term[dkey] if d != [None]]
            streams = closure(keys)
            grp.sites.append(Site(key, (0.0,) * ir.d_in, streams))
            for e, eq in enumerate(self.equations):
                for term in eq.values():
                    dkey = list(term.keys())[1]
                    factors = []
                    for j, d in enumerate(term[dkey]):
                        pw = term['pow'][j]
                        if not isinstance(pw, (int, float)):
                            raise NotImplementedError('callable pow is not implemented on the '
                                                      'device path')
                        sidx = 0 if d == [None] else streams.index(tuple(sorted(d)))
                        factors.append((int(term['var'][j]), float(pw), [(0, sidx, 1.0)]))
                    grp.terms.append((self._coeff(term['coeff'], pts, None), e, factors))
        else:
            site_of = {}
            nv = ir.d_in
            for e, eq in enumerate(self.equations):
                for term in eq.values():
                    dkey = list(term.keys())[1]
                    factors = []
                    for j, d in enumerate(term[dkey]):
                        pw = term['pow'][j]
                        if not isinstance(pw, (int, float)):
                            raise NotImplementedError('callable pow is not implemented on the '
                                                      'device path')
                        shifts, weights = fd_scheme(d, nv, 'central', self.inner_order, self.h)
                        parts = []
                        for s, w in zip(shifts, weights):
                            off = (0.0,) * nv if s is None else tuple(
                                float(np.float32(k * self.h)) for k in s)
                            if off not in site_of:
                                grp.sites.append(Site(key, off, [()]))
                                site_of[off] = len(grp.sites) - 1
                            parts.append((site_of[off], 0, float(np.float32(w))))
                        factors.append((int(term['var'][j]), float(pw), parts))
                    grp.terms.append((self._coeff(term['coeff'], pts, rows), e, factors))
        ir.groups.append(grp)
        ir.residual_group = len(ir.groups) - 1
        ir.n_eq = n_eq
        ir.n_residual_rows = pts.shape[0]
        return grp

    # -- boundary conditions ---------------------------------------------------------------
    def _bc_groups_nn_operator(self, bc, side_pts, sign_of_side, out_type):
        """NN operator values on typed boundary subsets, concatenated per side in type order
        (tedeous/eval.py:265-281, input_preprocessing.py:371-408)."""
        types = self.types()
        per_side = []
        for pts in side_pts:
            rows = match_rows(self.grid, pts)
            sel = []
            for t, idx in types.items():
                idx_set = set(idx)
                sel += [(t, i) for i, r in enumerate(rows) if r in idx_set]
            per_side.append(sel)
        n = len(per_side[0])
        if any(len(s) != n for s in per_side):
            raise NotImplementedError('periodic sides with different typed point counts')
        combos = {}
        for i in range(n):
            combos.setdefault(tuple(s[i][0] for s in per_side), []).append(i)
        groups = []
        for combo, positions in combos.items():
            grp = Group(out_type, len(positions), 1, -1)
            for side, (pts, ptype) in enumerate(zip(side_pts, combo)):
                sub = pts[[per_side[side][i][1] for i in positions]]
                key = self._points(sub, ('bnd', id(bc), side, combo))
                sub_rows = [match_rows(self.grid, sub)[k] for k in range(sub.shape[0])]
                self._add_operator_nn(grp, bc['bop'], sub, key, ptype, sign_of_side[side], 0,
                                      sub_rows)
            groups.append((grp, positions))
        return groups, n

    def boundary(self, slot_of_type):
        ir = self.ir
        vals = {}     # type -> list of (group or None, positions, n_rows)
        for bc in (self.bconds or []):
            bop = bc.get('bop')
            if isinstance(bop, dict) and any(isinstance(term.get('coeff'), torch.nn.Parameter)
                                             for term in bop.values() if isinstance(term, dict)):
                raise NotImplementedError('trainable (nn.Parameter) coefficients are implemented '
                                          'in the equation operator, not in boundary operators')
            t = bc['type']
            if t not in slot_of_type:
                slot_of_type[t] = None
                ir.bc_types.append(t)
                ir.bc_parts[t] = []
                ir.bc_true[t] = []
            true = bc['bval'].reshape(-1).to(torch.float32)
            new_groups = []   # (group, positions within this bc's rows or None)
            if t in ('dirichlet',) or (t in ('data',) and bc['bop'] is None):
                pts = bc['bnd']
                grp = Group(t, pts.shape[0], 1, -1)
                grp.sites.append(Site(self._points(pts, ('bnd', id(bc))), (0.0,) * ir.d_in, [()]))
                grp.terms.append((1.0, 0, [(int(bc['var']), 1.0, [(0, 0, 1.0)])]))
                new_groups.append((grp, None))
                n = pts.shape[0]
            elif t in ('operator', 'data'):
                pts = bc['bnd']
                if self.mode == 'autograd':
                    grp = Group(t, pts.shape[0], 1, -1)
                    self._add_operator_ag(grp, bc['bop'], pts, self._points(pts, ('bnd', id(bc))),
                                          1, 0, 0)
                    new_groups.append((grp, None))
                    n = pts.shape[0]
                else:
                    gs, n = self._bc_groups_nn_operator(bc, [pts], [1], t)
                    new_groups += gs
            elif t == 'periodic':
                sides = bc['bnd']
                n = sides[0].shape[0]
                if any(s.shape[0] != n for s in sides):
                    raise ValueError('periodic sides must have equal point counts')
                if bc['bop'] is None:
                    grp = Group(t, n, 1, -1)
                    for k, s in enumerate(sides):
                        grp.sites.append(Site(self._points(s, ('bnd', id(bc), k)),
                                              (0.0,) * ir.d_in, [()]))
                        grp.terms.append((1.0 if k == 0 else -1.0, 0,
                                          [(int(bc['var']), 1.0, [(k, 0, 1.0)])]))
                    new_groups.append((grp, None))
                elif self.mode == 'autograd':
                    grp = Group(t, n, 1, -1)
                    for k, s in enumerate(sides):
                        self._add_operator_ag(grp, bc['bop'], s, self._points(s, ('bnd', id(bc), k)),
                                              1 if k == 0 else -1, 0, k)
                    new_groups.append((grp, None))
                else:
                    gs, n = self._bc_groups_nn_operator(bc, sides, [1] + [-1] * (len(sides) - 1), t)
                    new_groups += gs
            elif t == 'robin':
                pts = bc['bnd']
                if self.mode != 'autograd':
                    raise NotImplementedError("robin conditions in 'NN' mode are not implemented")
                coeffs = [term['coeff'] for term in bc['bop'].values()]
                alpha, betas = coeffs[0], coeffs[1:]
                grp = Group(t, pts.shape[0], 1, -1)
                key = self._points(pts, ('bnd', id(bc)))
                grp.sites.append(Site(key, (0.0,) * ir.d_in, [()]))
                grp.terms.append((self._coeff(alpha, pts, None), 0,
                                  [(int(bc['var']), 1.0, [(0, 0, 1.0)])]))
                for beta in betas:
                    scaled = {}
                    for lbl, term in bc['bop'].items():
                        tt = dict(term)
                        c = term['coeff']
                        bv = beta(pts).reshape(-1) if callable(beta) else beta
                        if isinstance(c, (int, float)) and isinstance(bv, (int, float)):
                            tt['coeff'] = c * bv
                        else:
                            cv = c(pts).reshape(-1) if callable(c) else torch.as_tensor(c)
                            tt['coeff'] = torch.as_tensor(bv) * cv
                        scaled[lbl] = tt
                    self._add_operator_ag_into_site(grp, scaled, pts)
                new_groups.append((grp, None))
                n = pts.shape[0]
            else:
                raise NotImplementedError(f'boundary type {t!r}')
            # targets: concatenated true values, paired by position with concatenated outputs
            offset = sum(r for _, r in ir.bc_parts[t])
            true_full = true
            for grp, positions in new_groups:
                if positions is None:
                    tv = true_full if true_full.numel() == grp.n_rows else None
                else:
                    tv = true_full[positions] if true_full.numel() >= n else None
                if tv is not None and bool((tv != 0).any()):
                    grp.target = ir.add_array(tv.reshape(-1, 1))
                ir.groups.append(grp)
                ir.bc_parts[t].append((len(ir.groups) - 1, grp.n_rows))
            ir.bc_true[t].append(true_full)
            del offset
        return slot_of_type

    def _add_operator_ag_into_site(self, grp, eq, pts):
        """Terms of an operator evaluated at the group's existing site 0 (robin)."""
        site = grp.sites[0]
        keys = []
        for term in eq.values():
            dkey = list(term.keys())[1]
            keys += [tuple(d) for d in term[dkey] if d != [None]]
        site.streams = closure(keys + [s for s in site.streams if s])
        for term in eq.values():
            dkey = list(term.keys())[1]
            factors = []
            for j, d in enumerate(term[dkey]):
                sidx = 0 if d == [None] else site.streams.index(tuple(sorted(d)))
                factors.append((int(term['var'][j]), float(term['pow'][j]), [(0, sidx, 1.0)]))
            grp.terms.append((self._coeff(term['coeff'], pts, None), 0, factors))


def _lambda_list(lam, n):
    """Scalar lambda -> one per column; list -> as given (tedeous/input_preprocessing.py:14-43)."""
    if isinstance(lam, torch.Tensor):
        v = lam.detach().cpu().reshape(-1).tolist()
    elif isinstance(lam, (int, float)):
        v = [float(lam)] * n
    else:
        v = [float(x) for x in lam]
    if len(v) == 1 and n > 1:
        v = v * n
    if len(v) != n:
        raise ValueError(f'{len(v)} lambdas for {n} columns')
    return v


def residual_time_slices(points):
    """n_t of the causal loss: the number of distinct values of the first coordinate of the
    residual points (tedeous/solution.py:49-56); when the points do not split into n_t equal
    slices, every point is its own slice (the fallback of tedeous/losses.py:161-165)."""
    n = points.shape[0]
    n_t = len(torch.unique(points.reshape(n, -1)[:, 0]))
    return n_t if n % n_t == 0 else n


def lower(grid, operator, bconds, mode, lambda_operator, lambda_bound, h=0.001, inner_order='1',
          boundary_order='2', d_out=1, tol=0):
    """Build the ProblemIR of one problem: residual group(s), boundary groups and loss slots.
    tol != 0 selects the causal loss (tedeous/losses.py:137-182): the residual rows weigh 1/N
    each, times a per-row weight array that tdg_causal_weights fills before each evaluation;
    lambda_operator is not applied, as in the reference."""
    lw = Lowering(grid, operator, bconds, mode, lambda_operator, lambda_bound, h, inner_order,
                  boundary_order, d_out)
    ir = lw.ir
    if not bconds:
        raise NotImplementedError('problems without boundary conditions (the reference returns '
                                  'an infinite loss) are not implemented')
    res = lw.residual(0)
    n_eq = res.n_outputs
    lam_op = _lambda_list(lambda_operator, n_eq)
    n = float(res.n_rows)
    if tol:
        for e in range(n_eq):
            ir.slots.append((0, 1.0 / n, 1.0 / n))
        res.row_weight = ir.add_array(torch.ones(res.n_rows))
        ir.causal = (float(tol), residual_time_slices(ir.arrays[res.sites[0].points]))
    else:
        for e in range(n_eq):
            ir.slots.append((0, lam_op[e] / n, 1.0 / n))
    lw.boundary({})
    lens = {t: sum(r for _, r in ir.bc_parts[t]) for t in ir.bc_types}
    ir.max_len = max(lens.values())
    lam_b = _lambda_list(lambda_bound, len(ir.bc_types))
    for k, t in enumerate(ir.bc_types):
        slot = len(ir.slots)
        ir.slots.append((0, lam_b[k] / ir.max_len, 1.0 / ir.max_len))
        for gi, _ in ir.bc_parts[t]:
            ir.groups[gi].slot_first = slot
    return ir


def shard_rows(n, rank, world):
    """Rows [r0, r1) of `n` residual rows that rank `rank` of `world` evaluates: contiguous
    ranges whose sizes differ by at most one, in rank order."""
    if not 0 <= rank < world:
        raise ValueError(f'rank {rank} outside a world of {world}')
    return n * rank // world, n * (rank + 1) // world


def shard_ir(ir, rank, world):
    """The part of a lowered problem that rank `rank` of `world` evaluates when the collocation
    points are split across devices: the residual group keeps rows [r0, r1) (its points,
    per-row coefficients and per-row weights sliced to them) and only rank 0 keeps the boundary
    groups. The loss-slot weights are the unsharded problem's (lambda over the global point
    count, tedeous/losses.py:58), so the per-rank losses and gradients add up to the unsharded
    ones: the residual is independent per point and the loss is a sum over points. The op / bval
    fields of a rank describe its own rows only."""
    import copy as _copy
    if ir.causal is not None:
        raise NotImplementedError('the causal loss couples every time slice across the points: '
                                  'it is not sharded')
    res = ir.groups[ir.residual_group]
    r0, r1 = shard_rows(res.n_rows, rank, world)
    out = _copy.copy(ir)
    out.arrays = list(ir.arrays)
    keys = {s.points for s in res.sites}
    keys |= {c for c, _, _ in res.terms if isinstance(c, int)}
    if res.row_weight is not None:
        keys.add(res.row_weight)
    if res.target is not None:
        keys.add(res.target)
    for k in keys:
        a = ir.arrays[k]
        per_row = a.numel() // res.n_rows
        out.arrays[k] = a.reshape(res.n_rows, per_row)[r0:r1].reshape(-1).contiguous()
    new_res = _copy.copy(res)
    new_res.n_rows = r1 - r0
    if rank == 0:
        out.groups = [new_res if i == ir.residual_group else g for i, g in enumerate(ir.groups)]
    else:
        out.groups = [new_res]
        out.residual_group = 0
        out.bc_parts = {t: [] for t in ir.bc_types}
    out.n_residual_rows = r1 - r0
    out.shard = (rank, world, r0, r1)
    return out

"""Optimizer selection (tedeous/optimizers/optimizer.py:11-73) and the fused Adam.

Optimizer('Adam', {'lr': ...}) selects FusedAdam: one tdg_adam_step launch updates every
parameter of the flat buffer with torch.optim.Adam's arithmetic (non-amsgrad). Other names map
to the torch.optim class the reference uses.
"""

import ctypes
import math
from typing import Union

import torch
from torch.optim.lr_scheduler import CosineAnnealingWarmRestarts, ExponentialLR

from . import _lib


def _in_buffer_order(params):
    """Parameters that are views of one buffer, ordered by their place in it (the device path
    puts a network's trainable equation coefficients after its layers, while
    Module.parameters() lists a module's own registered parameters first)."""
    params = list(params)
    if params and all(isinstance(p, torch.Tensor) for p in params):
        st = {p.data.untyped_storage().data_ptr() for p in params}
        if len(st) == 1:
            return sorted(params, key=lambda p: p.data.storage_offset())
    return params


def _flat_of(params):
    """The flat buffer the parameters are views of, or None."""
    if not params:
        return None
    base = params[0].data
    st = base.untyped_storage()
    start = base.storage_offset()
    off = start
    for p in params:
        d = p.data
        if d.untyped_storage().data_ptr() != st.data_ptr() or d.storage_offset() != off \
                or not d.is_contiguous() or d.dtype != torch.float32:
            return None
        off += d.numel()
    n = off - start
    return torch.empty(0, device=base.device).set_(st, start, (n,))


class FusedAdam(torch.optim.Optimizer):
    """torch.optim.Adam semantics (lr, betas, eps, weight_decay, maximize; no amsgrad) applied in
    one launch to parameters that are views of one flat float32 CUDA buffer."""

    def __init__(self, params, lr=1e-3, betas=(0.9, 0.999), eps=1e-8, weight_decay=0.0,
                 amsgrad=False, maximize=False, **unused):
        if amsgrad:
            raise NotImplementedError('amsgrad is not implemented by the fused Adam')
        super().__init__(params, dict(lr=lr, betas=betas, eps=eps, weight_decay=weight_decay,
                                      maximize=maximize))
        if len(self.param_groups) != 1:
            raise NotImplementedError('the fused Adam takes one parameter group')
        ps = self.param_groups[0]['params']
        self._flat = _flat_of(ps)
        if self._flat is None or not self._flat.is_cuda:
            raise ValueError('FusedAdam needs CUDA parameters that are views of one flat buffer')
        n = self._flat.numel()
        dev = self._flat.device
        self._m = torch.zeros(n, device=dev)
        self._v = torch.zeros(n, device=dev)
        self._step = torch.zeros(1, device=dev)
        self._gbuf = None

    def flat_grad(self):
        ps = self.param_groups[0]['params']
        grads = [p.grad for p in ps]
        if any(g is None for g in grads):
            grads = [torch.zeros_like(p) if p.grad is None else p.grad for p in ps]
        g = _flat_of(grads)
        if g is not None and g.numel() == self._flat.numel():
            return g
        return torch.cat([x.reshape(-1) for x in grads])

    def hyper(self):
        gr = self.param_groups[0]
        hp = _lib.AdamDesc()
        hp.lr, (hp.beta1, hp.beta2), hp.eps = gr['lr'], gr['betas'], gr['eps']
        hp.weight_decay, hp.maximize = gr['weight_decay'], int(gr['maximize'])
        return hp

    def apply(self, grad, stream=None):
        """Adam update of the flat parameters from a flat gradient."""
        s = torch.cuda.current_stream(self._flat.device) if stream is None else stream
        hp = self.hyper()
        _lib.check(_lib.load().tdg_adam_step(
            self._flat.data_ptr(), grad.data_ptr(), self._m.data_ptr(), self._v.data_ptr(),
            self._step.data_ptr(), self._flat.numel(), hp, s.cuda_stream), 'tdg_adam_step')

    @torch.no_grad()
    def step(self, closure=None):
        loss = None
        if closure is not None:
            with torch.enable_grad():
                loss = closure()
        self.apply(self.flat_grad().contiguous())
        return loss


def _cubic_min(x1, f1, g1, x2, f2, g2, lo=None, hi=None):
    """Minimiser of the cubic through (x1, f1) and (x2, f2) with slopes g1 and g2, clamped to
    [lo, hi] (by default the interval between the two points); the interval's midpoint when the
    cubic has no real minimiser (Nocedal and Wright, Numerical Optimization, eq. 3.59)."""
    if lo is None:
        lo, hi = min(x1, x2), max(x1, x2)
    d1 = g1 + g2 - 3.0 * (f1 - f2) / (x1 - x2)
    disc = d1 * d1 - g1 * g2
    if disc < 0:
        return (lo + hi) / 2.0
    d2 = math.sqrt(disc)
    if x1 <= x2:
        m = x2 - (x2 - x1) * ((g2 + d2 - d1) / (g2 - g1 + 2.0 * d2))
    else:
        m = x1 - (x1 - x2) * ((g1 + d2 - d1) / (g1 - g2 + 2.0 * d2))
    return min(max(m, lo), hi)


class _Trial:
    """One line-search point: step t, loss f, gradient g (device vector), slope g.d, max |g|."""
    __slots__ = ('t', 'f', 'g', 'gd', 'gmax')

    def __init__(self, t, f, g, gd, gmax):
        self.t, self.f, self.g, self.gd, self.gmax = t, f, g, gd, gmax


def strong_wolfe(evaluate, start, t, d_max, c1=1e-4, c2=0.9, tolerance_change=1e-9, max_ls=25):
    """Line search for the strong Wolfe conditions: bracketing with cubic extrapolation, then
    zoom with cubic interpolation and a safeguard against steps near the bracket's ends
    (Nocedal and Wright, Algorithms 3.5 and 3.6), with the constants and safeguards of the
    line search torch.optim.LBFGS(line_search_fn='strong_wolfe') runs, which the reference
    selects (tedeous/optimizers/optimizer.py:50-51).

    evaluate(t) -> _Trial at step t; start: the _Trial at t = 0. Returns (accepted _Trial,
    number of evaluations)."""
    f0, gd0 = start.f, start.gd
    new = evaluate(t)
    n_eval = 1
    prev = start
    found = False
    lo = hi = None
    it = 0
    while it < max_ls:
        if new.f > f0 + c1 * new.t * gd0 or (it > 1 and new.f >= prev.f):
            lo, hi = prev, new
            break
        if abs(new.gd) <= -c2 * gd0:
            lo, found = new, True
            break
        if new.gd >= 0:
            lo, hi = prev, new
            break
        # extrapolate: the cubic's minimiser within [t + 0.01 (t - t_prev), 10 t]
        t_next = _cubic_min(prev.t, prev.f, prev.gd, new.t, new.f, new.gd,
                            new.t + 0.01 * (new.t - prev.t), new.t * 10)
        prev = new
        new = evaluate(t_next)
        n_eval += 1
        it += 1
    if found:
        return lo, n_eval
    if it == max_ls:   # no bracket within the budget: the lower of the start and the last trial
        lo, hi = start, new
    pair = [lo, hi]
    i_lo = 0 if pair[0].f <= pair[1].f else 1
    stalled = False
    while it < max_ls:
        a, b = pair
        if abs(b.t - a.t) * d_max < tolerance_change:
            break
        t_try = _cubic_min(a.t, a.f, a.gd, b.t, b.f, b.gd)
        top, bot = max(a.t, b.t), min(a.t, b.t)
        margin = 0.1 * (top - bot)
        if min(top - t_try, t_try - bot) < margin:
            if stalled or t_try >= top or t_try <= bot:
                t_try = top - margin if abs(t_try - top) < abs(t_try - bot) else bot + margin
                stalled = False
            else:
                stalled = True
        else:
            stalled = False
        new = evaluate(t_try)
        n_eval += 1
        it += 1
        i_hi = 1 - i_lo
        if new.f > f0 + c1 * new.t * gd0 or new.f >= pair[i_lo].f:
            # not a sufficient decrease: the trial closes the bracket from above
            pair[i_hi] = new
            i_lo = 0 if pair[0].f <= pair[1].f else 1
            continue
        found = abs(new.gd) <= -c2 * gd0
        if not found and new.gd * (pair[i_hi].t - pair[i_lo].t) >= 0:
            pair[i_hi] = pair[i_lo]
        pair[i_lo] = new
        if found:
            break
    return pair[i_lo], n_eval


class LBFGS64(torch.optim.Optimizer):
    """L-BFGS with the step semantics of torch.optim.LBFGS (lr, max_iter, max_eval,
    tolerance_grad, tolerance_change, history_size, line_search_fn None or 'strong_wolfe'),
    device-resident: the curvature history, the two-loop recursion and the step statistics live
    on the device (tdg_lbfgs_*), every dot product accumulated in FP64, vectors in FP32. An
    iteration synchronises the host only for the tests torch's loop makes on host numbers: one
    read of (g.d, sum |g|, max |d|) before the step and one of (loss, max |g|) after each
    closure (the line search reads (loss, g.d) per trial)."""

    def __init__(self, params, lr=1.0, max_iter=20, max_eval=None, tolerance_grad=1e-7,
                 tolerance_change=1e-9, history_size=100, line_search_fn=None):
        if line_search_fn not in (None, 'strong_wolfe'):
            raise ValueError("only 'strong_wolfe' is supported")
        if max_eval is None:
            max_eval = max_iter * 5 // 4
        super().__init__(params, dict(lr=lr, max_iter=max_iter, max_eval=max_eval,
                                      tolerance_grad=tolerance_grad,
                                      tolerance_change=tolerance_change,
                                      history_size=history_size, line_search_fn=line_search_fn))
        if len(self.param_groups) != 1:
            raise NotImplementedError('LBFGS64 takes one parameter group')
        self._params = self.param_groups[0]['params']
        self._dev = self._params[0].device
        if self._dev.type != 'cuda':
            raise ValueError('LBFGS64 needs CUDA parameters')
        self._n = sum(p.numel() for p in self._params)
        self._flat = _flat_of(self._params)
        h = ctypes.c_void_p()
        with torch.cuda.device(self._dev):
            _lib.check(_lib.load().tdg_lbfgs_create(self._n, history_size, ctypes.byref(h)),
                       'tdg_lbfgs_create')
        self._h = h
        self._stats = torch.zeros(8, dtype=torch.float64, device=self._dev)
        self._dot_out = torch.zeros(1, dtype=torch.float64, device=self._dev)

    def __del__(self):
        h = getattr(self, '_h', None)
        if h is not None and h.value:
            try:
                _lib.load().tdg_lbfgs_destroy(h)
            except Exception:
                pass
            self._h = None

    def _stream(self):
        return torch.cuda.current_stream(self._dev).cuda_stream

    def _read_stats(self, g, d=None, loss=None):
        """(g.d, sum |g|, max |g|, max |d|, loss) in one device-to-host read."""
        host_loss = None
        if loss is not None and not isinstance(loss, torch.Tensor):
            host_loss, loss = float(loss), None
        if loss is not None:
            loss = loss.detach().reshape(-1)[:1].to(self._dev, torch.float32).contiguous()
        _lib.check(_lib.load().tdg_lbfgs_stats(
            self._h, g.data_ptr(), None if d is None else d.data_ptr(),
            None if loss is None else loss.data_ptr(), self._stats.data_ptr(), self._stream()),
            'tdg_lbfgs_stats')
        out = self._stats[:5].tolist()
        if host_loss is not None:
            out[4] = host_loss
        return out

    def _flat_grad(self):
        return torch.cat([torch.zeros(p.numel(), device=p.device) if p.grad is None
                          else p.grad.reshape(-1).to(torch.float32) for p in self._params])

    def _param_vector(self):
        if self._flat is not None:
            return self._flat.clone()
        return torch.cat([p.detach().reshape(-1).to(torch.float32) for p in self._params])

    def _assign(self, vec):
        if self._flat is not None:
            self._flat.copy_(vec)
            return
        off = 0
        for p in self._params:
            n = p.numel()
            p.copy_(vec[off:off + n].view_as(p))
            off += n

    def _set_to(self, x, d, t):
        """parameters = x + t d"""
        if self._flat is not None:
            _lib.check(_lib.load().tdg_axpy(x.data_ptr(), d.data_ptr(), float(t),
                                            self._flat.data_ptr(), self._n, self._stream()),
                       'tdg_axpy')
            return
        out = torch.empty_like(x)
        _lib.check(_lib.load().tdg_axpy(x.data_ptr(), d.data_ptr(), float(t), out.data_ptr(),
                                        self._n, self._stream()), 'tdg_axpy')
        self._assign(out)

    def _dot(self, a, b):
        """a . b accumulated in FP64 on the device (one host read)."""
        _lib.check(_lib.load().tdg_dot_f64(a.data_ptr(), b.data_ptr(), a.numel(),
                                           self._dot_out.data_ptr(), self._stream()),
                   'tdg_dot_f64')
        return float(self._dot_out.item())

    @torch.no_grad()
    def step(self, closure):
        gr = self.param_groups[0]
        lr, max_iter, max_eval = gr['lr'], gr['max_iter'], gr['max_eval']
        tol_grad, tol_change, hist = gr['tolerance_grad'], gr['tolerance_change'], gr['history_size']
        lib = _lib.load()
        st = self.state[self._params[0]]
        st.setdefault('func_evals', 0)
        st.setdefault('n_iter', 0)
        st.setdefault('n_push', 0)
        with torch.enable_grad():
            orig_loss = closure()
        g = self._flat_grad()
        _, _, gmax, _, loss = self._read_stats(g, loss=orig_loss)
        evals = 1
        st['func_evals'] += 1
        if gmax <= tol_grad:
            return orig_loss
        d, t = st.get('d'), st.get('t')
        g_prev, loss_prev = st.get('prev_flat_grad'), st.get('prev_loss')
        n_iter = 0
        while n_iter < max_iter:
            n_iter += 1
            st['n_iter'] += 1
            if st['n_iter'] == 1:
                _lib.check(lib.tdg_lbfgs_reset(self._h, self._stream()), 'tdg_lbfgs_reset')
                st['n_push'] = 0
            else:
                _lib.check(lib.tdg_lbfgs_push(self._h, g.data_ptr(), g_prev.data_ptr(),
                                              d.data_ptr(), float(t), self._stream()),
                           'tdg_lbfgs_push')
                st['n_push'] += 1
            d = torch.empty_like(g)
            _lib.check(lib.tdg_lbfgs_direction(self._h, g.data_ptr(), d.data_ptr(),
                                               min(st['n_push'], hist), self._stream()),
                       'tdg_lbfgs_direction')
            g_prev, loss_prev = g, loss
            gtd, g_l1, _, d_max, _ = self._read_stats(g, d)
            t = min(1.0, 1.0 / g_l1) * lr if st['n_iter'] == 1 else lr
            if gtd > -tol_change:
                break
            ls_evals = 0
            if gr['line_search_fn'] == 'strong_wolfe':
                x0 = self._param_vector()

                def evaluate(tt, x0=x0, d=d):
                    self._set_to(x0, d, tt)
                    with torch.enable_grad():
                        cl = closure()
                    gg = self._flat_grad()
                    gd, _, gm, _, f = self._read_stats(gg, d, cl)
                    self._assign(x0)
                    return _Trial(tt, f, gg, gd, gm)

                best, ls_evals = strong_wolfe(evaluate, _Trial(0.0, loss, g, gtd, None), t, d_max,
                                              tolerance_change=tol_change)
                t, loss, g = best.t, best.f, best.g
                gmax = best.gmax if best.gmax is not None else self._read_stats(g)[2]
                self._set_to(x0, d, t)
                opt_cond = gmax <= tol_grad
            else:
                self._set_to(self._flat if self._flat is not None else self._param_vector(), d, t)
                opt_cond = False
                if n_iter != max_iter:
                    with torch.enable_grad():
                        cl = closure()
                    g = self._flat_grad()
                    _, _, gmax, _, loss = self._read_stats(g, loss=cl)
                    opt_cond = gmax <= tol_grad
                    ls_evals = 1
            evals += ls_evals
            st['func_evals'] += ls_evals
            if n_iter == max_iter or evals >= max_eval or opt_cond:
                break
            if d_max * abs(t) <= tol_change or abs(loss - loss_prev) < tol_change:
                break
        st.update(d=d, t=t, prev_flat_grad=g_prev, prev_loss=loss_prev)
        return orig_loss


class Optimizer:
    """Name + hyper-parameters -> optimizer instance (tedeous/optimizers/optimizer.py:11-73)."""

    def __init__(self, optimizer: Union[str, dict], params: dict, gamma: Union[float, None] = None,
                 decay_every: Union[int, None] = None,
                 cosine_scheduler_patience: Union[float, None] = None):
        self.optimizer = optimizer
        self.params = params
        self.gamma = gamma
        self.decay_every = decay_every
        self.cosine_scheduler_patience = cosine_scheduler_patience

    def optimizer_choice(self, mode, model):
        names = {'Adam': None, 'AdamW': torch.optim.AdamW, 'SGD': torch.optim.SGD,
                 'LBFGS': torch.optim.LBFGS, 'RMSprop': torch.optim.RMSprop}
        if self.optimizer not in names:
            raise NotImplementedError(f'optimizer {self.optimizer!r} is not implemented on the '
                                      f'device path (Adam, AdamW, SGD, LBFGS, RMSprop are)')
        if mode not in ('NN', 'autograd'):
            raise NotImplementedError(f'mode {mode!r}')
        params = _in_buffer_order(model.parameters())
        if self.optimizer == 'Adam' and _flat_of(params) is not None:
            opt = FusedAdam(params, **self.params)
        elif self.optimizer == 'Adam':   # parameters with gaps (a coefficient outside the network)
            opt = torch.optim.Adam(params, **self.params)
        elif self.optimizer == 'LBFGS':
            opt = LBFGS64(params, **self.params)
        else:
            opt = names[self.optimizer](params, **self.params)
        if self.gamma is not None:
            self.scheduler = ExponentialLR(opt, gamma=self.gamma)
        if self.cosine_scheduler_patience is not None:
            self.scheduler = CosineAnnealingWarmRestarts(opt, self.cosine_scheduler_patience)
        return opt

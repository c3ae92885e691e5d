"""Optimizer selection (tedeous/optimizers/optimizer.py:11-73) and the fused Adam.

Optimizer('Adam', {'lr': ...}) selects FusedAdam: one tdg_adam_step launch updates every
parameter of the flat buffer with torch.optim.Adam's arithmetic (non-amsgrad). Other names map
to the torch.optim class the reference uses.
"""

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


class LBFGS64(torch.optim.Optimizer):
    """L-BFGS with the step semantics of torch.optim.LBFGS (line_search_fn=None): lr, max_iter,
    max_eval, tolerance_grad, tolerance_change, history_size; two-loop recursion over the stored
    curvature pairs. Every dot product of the recursion and of the curvature test is accumulated in
    FP64 on the device (tdg_dot_f64); vectors stay FP32 on the device."""

    def __init__(self, params, lr=1.0, max_iter=20, max_eval=None, tolerance_grad=1e-7,
                 tolerance_change=1e-9, history_size=100, line_search_fn=None):
        if line_search_fn is not None:
            raise NotImplementedError('LBFGS64 implements line_search_fn=None')
        if max_eval is None:
            max_eval = max_iter * 5 // 4
        super().__init__(params, dict(lr=lr, max_iter=max_iter, max_eval=max_eval,
                                      tolerance_grad=tolerance_grad,
                                      tolerance_change=tolerance_change,
                                      history_size=history_size))
        if len(self.param_groups) != 1:
            raise NotImplementedError('LBFGS64 takes one parameter group')
        self._params = self.param_groups[0]['params']
        dev = self._params[0].device
        self._dot_out = torch.zeros(1, dtype=torch.float64, device=dev)

    def _dot(self, a, b):
        _lib.check(_lib.load().tdg_dot_f64(a.data_ptr(), b.data_ptr(), a.numel(),
                                           self._dot_out.data_ptr(),
                                           torch.cuda.current_stream(a.device).cuda_stream),
                   'tdg_dot_f64')
        return float(self._dot_out.item())

    def _flat_grad(self):
        return torch.cat([torch.zeros(p.numel(), device=p.device) if p.grad is None
                          else p.grad.reshape(-1).to(torch.float32) for p in self._params])

    def _add(self, t, d):
        off = 0
        for p in self._params:
            n = p.numel()
            p.add_(d[off:off + n].view_as(p), alpha=t)
            off += n

    @torch.no_grad()
    def step(self, closure):
        gr = self.param_groups[0]
        lr, max_iter, max_eval = gr['lr'], gr['max_iter'], gr['max_eval']
        tol_grad, tol_change, hist = gr['tolerance_grad'], gr['tolerance_change'], gr['history_size']
        st = self.state[self._params[0]]
        st.setdefault('func_evals', 0)
        st.setdefault('n_iter', 0)
        with torch.enable_grad():
            orig_loss = closure()
        loss = float(orig_loss)
        evals = 1
        st['func_evals'] += 1
        g = self._flat_grad()
        if float(g.abs().max()) <= tol_grad:
            return orig_loss
        d, t = st.get('d'), st.get('t')
        dirs, stps, ro = st.get('old_dirs'), st.get('old_stps'), st.get('ro')
        h_diag, g_prev, loss_prev = st.get('H_diag'), st.get('prev_flat_grad'), st.get('prev_loss')
        n_iter = 0
        while n_iter < max_iter:
            n_iter += 1
            st['n_iter'] += 1
            if st['n_iter'] == 1:
                d = g.neg()
                dirs, stps, ro = [], [], []
                h_diag = 1.0
            else:
                y = g - g_prev
                s = d * t
                ys = self._dot(y, s)
                if ys > 1e-10:
                    if len(dirs) == hist:
                        dirs.pop(0), stps.pop(0), ro.pop(0)
                    dirs.append(y)
                    stps.append(s)
                    ro.append(1.0 / ys)
                    h_diag = ys / self._dot(y, y)
                al = [0.0] * len(dirs)
                q = g.neg()
                for i in range(len(dirs) - 1, -1, -1):
                    al[i] = self._dot(stps[i], q) * ro[i]
                    q.add_(dirs[i], alpha=-al[i])
                d = r = q * h_diag
                for i in range(len(dirs)):
                    be = self._dot(dirs[i], r) * ro[i]
                    r.add_(stps[i], alpha=al[i] - be)
            g_prev = g.clone()
            loss_prev = loss
            t = min(1.0, 1.0 / float(g.abs().sum())) * lr if st['n_iter'] == 1 else lr
            gtd = self._dot(g, d)
            if gtd > -tol_change:
                break
            ls_evals = 0
            self._add(t, d)
            if n_iter != max_iter:
                with torch.enable_grad():
                    loss = float(closure().detach())
                g = self._flat_grad()
                ls_evals = 1
            evals += ls_evals
            st['func_evals'] += ls_evals
            if n_iter == max_iter or evals >= max_eval:
                break
            if float(g.abs().max()) <= tol_grad:
                break
            if float((d * t).abs().max()) <= tol_change or abs(loss - loss_prev) < tol_change:
                break
        st.update(d=d, t=t, old_dirs=dirs, old_stps=stps, ro=ro, H_diag=h_diag,
                  prev_flat_grad=g_prev, prev_loss=loss_prev)
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
        elif self.optimizer == 'LBFGS' and self.params.get('line_search_fn') is None:
            opt = LBFGS64(params, **self.params)
        else:
            opt = names[self.optimizer](params, **self.params)
        if self.gamma is not None:
            self.scheduler = ExponentialLR(opt, gamma=self.gamma)
        if self.cosine_scheduler_patience is not None:
            self.scheduler = CosineAnnealingWarmRestarts(opt, self.cosine_scheduler_patience)
        return opt

"""Optimizer selection (tedeous/optimizers/optimizer.py:11-73) and the fused Adam.

Optimizer('Adam', {'lr': ...}) selects FusedAdam: one tdg_adam_step launch updates every
parameter of the flat buffer with torch.optim.Adam's arithmetic (non-amsgrad). Other names map
to the torch.optim class the reference uses.
"""

from typing import Union

import torch
from torch.optim.lr_scheduler import CosineAnnealingWarmRestarts, ExponentialLR

from . import _lib


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
        if self.optimizer == 'Adam':
            opt = FusedAdam(model.parameters(), **self.params)
        else:
            opt = names[self.optimizer](model.parameters(), **self.params)
        if self.gamma is not None:
            self.scheduler = ExponentialLR(opt, gamma=self.gamma)
        if self.cosine_scheduler_patience is not None:
            self.scheduler = CosineAnnealingWarmRestarts(opt, self.cosine_scheduler_patience)
        return opt

"""Closure for gradient-based optimizers (tedeous/optimizers/closure.py:49-64, :187-195):
zero_grad, evaluate, loss.backward(); cur_loss is the loss or the normalized loss."""


class Closure:
    def __init__(self, mixed_precision: bool, model):
        if mixed_precision:
            raise NotImplementedError('mixed_precision: choose compile(precision=...) instead')
        self.mixed_precision = mixed_precision
        self.model = model
        self.optimizer = model.optimizer
        self.normalized_loss_stop = model.normalized_loss_stop

    def _closure(self):
        self.optimizer.zero_grad()
        loss, loss_normalized = self.model.solution_cls.evaluate()
        loss.backward()
        self.model.cur_loss = loss_normalized if self.normalized_loss_stop else loss
        return loss

    def get_closure(self, _type: str):
        if _type in ('PSO', 'CSO', 'NGD', 'NNCG'):
            raise NotImplementedError(f'{_type} closures are not implemented on the device path')
        return self._closure

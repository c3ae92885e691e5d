"""Callback hooks with the reference's interface (tedeous/callbacks/callback.py:3-75,
tedeous/callbacks/callback_list.py:5-63). Model.train calls on_train_begin, on_epoch_begin,
on_epoch_end and on_train_end; a callback reads model.cur_loss, model.t, model.net and
model.solution_cls and may set model.stop_training."""


class Callback:
    def __init__(self):
        self.model = None
        self.params = None

    def set_params(self, params):
        self.params = params

    def set_model(self, model):
        self.model = model

    def on_epoch_begin(self, logs=None):
        pass

    def on_epoch_end(self, logs=None):
        pass

    def on_train_begin(self, logs=None):
        pass

    def on_train_end(self, logs=None):
        pass


class CallbackList(Callback):
    def __init__(self, callbacks=None, model=None, **params):
        super().__init__()
        self.callbacks = list(callbacks) if callbacks else []
        if model is not None:
            self.set_model(model)
        if params:
            self.set_params(params)

    def set_model(self, model):
        super().set_model(model)
        for cb in self.callbacks:
            cb.set_model(model)

    def append(self, callback):
        self.callbacks.append(callback)

    def set_params(self, params):
        self.params = params
        for cb in self.callbacks:
            cb.set_params(params)

    def on_epoch_begin(self, logs=None):
        for cb in self.callbacks:
            cb.on_epoch_begin(logs or {})

    def on_epoch_end(self, logs=None):
        for cb in self.callbacks:
            cb.on_epoch_end(logs or {})

    def on_train_begin(self, logs=None):
        for cb in self.callbacks:
            cb.on_train_begin(logs or {})

    def on_train_end(self, logs=None):
        for cb in self.callbacks:
            cb.on_train_end(logs or {})


class InverseTask(Callback):
    """Prints the trainable equation coefficients every `info_string_every` epochs
    (tedeous/callbacks/inverse_task.py:8-38): `name=value` for each network parameter named in
    `parameters`."""

    def __init__(self, parameters: dict, info_string_every=None):
        super().__init__()
        self.parameters = parameters
        self.info_string_every = info_string_every

    def str_param(self):
        if self.info_string_every is not None and self.model.t % self.info_string_every == 0:
            names = set(self.parameters)
            print(''.join(f'{name}={p.item()} ' for name, p in self.model.net.named_parameters()
                          if name in names))

    def on_epoch_end(self, logs=None):
        self.str_param()

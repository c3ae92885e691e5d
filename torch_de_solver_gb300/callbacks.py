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


def create_random_fn(eps):
    """Adds (2 * randn - 1) * eps to the weight and bias of every Linear layer it is applied to
    (tedeous/utils.py:14-30)."""
    import torch

    def randomize_params(m):
        if isinstance(m, torch.nn.Linear) and m.bias is not None:
            m.weight.data = m.weight.data + (2 * torch.randn(m.weight.size()) - 1).to(m.weight) * eps
            m.bias.data = m.bias.data + (2 * torch.randn(m.bias.size()) - 1).to(m.bias) * eps
    return randomize_params


def remove_all_files(folder):
    """Deletes every file and folder inside `folder` (tedeous/utils.py:100-114)."""
    import os
    import shutil
    for filename in os.listdir(folder):
        path = os.path.join(folder, filename)
        try:
            if os.path.isfile(path) or os.path.islink(path):
                os.unlink(path)
            elif os.path.isdir(path):
                shutil.rmtree(path)
        except Exception as e:
            print('Failed to delete %s. Reason: %s' % (path, e))


def count_output(model):
    """out_features of the last layer that has one (tedeous/callbacks/cache.py:21-35)."""
    for layer in reversed(list(model.modules())):
        if hasattr(layer, 'out_features'):
            return layer.out_features
    return None


class CachePreprocessing:
    """Cache lookup and reuse for a compiled Model (tedeous/callbacks/cache.py:38-258). The lookup
    evaluates every usable cached network on the current problem in one launch per network shape
    (Solution.evaluate_many) instead of one evaluate per file, and keeps the reference's choice:
    the first network with the smallest loss, in the order of the files found."""

    def __init__(self, model):
        self.solution_cls = model.solution_cls

    @staticmethod
    def _cache_files(files, nmodels=None):
        import numpy as np
        if nmodels is None:
            return np.arange(len(files))
        return np.random.choice(len(files), nmodels, replace=False)

    @staticmethod
    def _model_reform(init_model, model):
        try:
            model[0]
        except Exception:
            model = model.model
        try:
            init_model[0]
        except Exception:
            init_model = init_model.model
        return init_model, model

    def cache_lookup(self, cache_dir, nmodels=None, save_graph=False, cache_verbose=False):
        """Best cached checkpoint {'model', 'model_state_dict'} by loss, or None. Files are found
        with the reference's pattern cache_dir + '\\*.tar' (tedeous/callbacks/cache.py:117), which
        matches the names Model saves under."""
        import glob
        import torch
        from .solution import mlp_widths
        files = glob.glob(cache_dir + '\\*.tar')
        if cache_verbose:
            print(f"The CACHE will be searched among the models in the folder {cache_dir}.")
        if len(files) == 0:
            return None
        solver = self.solution_cls.model
        candidates = []
        for i in self._cache_files(files, nmodels):
            file = files[i]
            try:
                checkpoint = torch.load(file, weights_only=False, map_location='cpu')
            except Exception:
                if cache_verbose:
                    print('Error loading file {}'.format(file))
                continue
            model = checkpoint['model']
            model.load_state_dict(checkpoint['model_state_dict'])
            try:
                solver_model, cache_model = self._model_reform(solver, model)
            except Exception:
                if cache_verbose:
                    print('Error reforming file {}'.format(file))
                continue
            if cache_model[0].in_features != solver_model[0].in_features:
                continue
            try:
                if count_output(model) != count_output(solver):
                    continue
                mlp_widths(model)
            except Exception:   # includes networks the device path cannot evaluate
                continue
            candidates.append((i, model))
        if not candidates:
            return None
        losses = self.solution_cls.evaluate_many([m for _, m in candidates])[:, 0].cpu()
        best = int(torch.argmin(losses))   # the first of equal minima, as the reference's '<'
        i, model = candidates[best]
        if cache_verbose:
            print('best_model_num={} , loss={}'.format(i, float(losses[best])))
        return {'model': model, 'model_state_dict': model.state_dict()}

    def scheme_interp(self, trained_model, cache_verbose=False):
        """Fits the solver's network to the outputs of a cached network of another architecture
        on the grid with Adam(lr=1e-3) until the mean squared difference is below 1e-5
        (tedeous/callbacks/cache.py:183-219)."""
        import torch
        sol = self.solution_cls
        grid = sol.grid.to(sol.device)
        model = sol.model
        trained_model = trained_model.to(sol.device)
        optimizer = torch.optim.Adam(model.parameters(), lr=0.001)
        loss = torch.mean(torch.square(trained_model(grid) - model(grid)))

        def closure():
            optimizer.zero_grad()
            loss = torch.mean((trained_model(grid) - model(grid)) ** 2)
            loss.backward()
            return loss
        t = 0
        while loss > 1e-5 and t < 1e5:
            optimizer.step(closure)
            loss = torch.mean(torch.square(trained_model(grid) - model(grid)))
            t += 1
            if cache_verbose:
                print('Interpolate from trained model t={}, loss={}'.format(t, loss))
        sol._model_change(model)

    def cache_retrain(self, cache_checkpoint, cache_verbose=False):
        """Same architecture: continue from the cached network; otherwise fit the solver's network
        to it (tedeous/callbacks/cache.py:221-258)."""
        import torch
        model = self.solution_cls.model
        if cache_checkpoint is None:
            return None
        if str(cache_checkpoint['model']) == str(model) and isinstance(model, torch.nn.Sequential) \
                and isinstance(model[0], torch.nn.Linear):
            model = cache_checkpoint['model']
            model.load_state_dict(cache_checkpoint['model_state_dict'])
            model.train()
            self.solution_cls._model_change(model)
            if cache_verbose:
                print('Using model from cache')
        else:
            cache_model = cache_checkpoint['model']
            cache_model.load_state_dict(cache_checkpoint['model_state_dict'])
            cache_model.eval()
            self.scheme_interp(cache_model, cache_verbose=cache_verbose)


class Cache(Callback):
    """Starts training from the best cached network and points Model's save folder at the cache
    (tedeous/callbacks/cache.py:261-400). 'mat' mode has no device path here."""

    def __init__(self, nmodels=None, cache_dir='tedeous_cache', cache_verbose=False,
                 cache_model=None, model_randomize_parameter=0, clear_cache=False):
        import os
        import tempfile
        super().__init__()
        self.nmodels = nmodels
        self.cache_verbose = cache_verbose
        self.cache_model = cache_model
        self.model_randomize_parameter = model_randomize_parameter
        if cache_dir == 'tedeous_cache':
            folder = os.path.join(tempfile.gettempdir(), 'tedeous_cache/')
            os.makedirs(folder, exist_ok=True)
            self.cache_dir = folder
        else:
            self.cache_dir = cache_dir
        if clear_cache:
            remove_all_files(self.cache_dir)

    def _cache_nn(self):
        cache_preproc = CachePreprocessing(self.model)
        r = create_random_fn(self.model_randomize_parameter)
        checkpoint = cache_preproc.cache_lookup(cache_dir=self.cache_dir, nmodels=self.nmodels,
                                                cache_verbose=self.cache_verbose)
        cache_preproc.cache_retrain(checkpoint, cache_verbose=self.cache_verbose)
        self.model.solution_cls.model.apply(r)

    def cache(self):
        if self.model.mode == 'mat':
            raise NotImplementedError("'mat' mode is not implemented on the device path")
        return self._cache_nn()

    def on_train_begin(self, logs=None):
        self.cache()
        self.model._save_dir = self.cache_dir


def _num(x):
    """A loss as a Python float (tensors detached first)."""
    import torch
    return float(x.detach()) if isinstance(x, torch.Tensor) else float(x)


class EarlyStopping(Callback):
    """Stop criteria of the training loop (tedeous/callbacks/early_stopping.py:9-165). Each epoch
    at most one criterion fires, checked in this order, and adds one "stop ding":

    * window: every `loss_window` epochs a straight line is fitted to the last `loss_window`
      losses; a slope below `eps` relative to the current loss fires, and perturbs the weights;
    * patience: `no_improvement_patience` epochs without a new minimum fire, and perturb the
      weights (after going back to the best network when `save_best`);
    * absolute: a loss below `abs_loss` fires.

    Training stops once `patience` dings have fired. The perturbation adds
    (2 * randn - 1) * randomize_parameter to every Linear layer (create_random_fn); the
    device path copies the new values back into its parameter buffer before the next step."""

    def __init__(self, eps=1e-5, loss_window=100, no_improvement_patience=1000, patience=5,
                 abs_loss=None, normalized_loss=False, randomize_parameter=1e-5,
                 info_string_every=None, verbose=True, save_best=False):
        import numpy as np
        super().__init__()
        self.eps = eps
        self.loss_window = loss_window
        self.no_improvement_patience = no_improvement_patience
        self.patience = patience
        self.abs_loss = abs_loss
        self.normalized_loss = normalized_loss
        self.info_string_every = np.inf if info_string_every is None else info_string_every
        self.verbose = verbose
        self.save_best = save_best
        self.best_model = None
        self._stop_dings = 0
        self._t_imp_start = 0
        self._r = create_random_fn(randomize_parameter)
        self._line = None
        self.last_loss = None

    def _fit_line(self):
        import numpy as np
        self._line = np.polyfit(range(self.loss_window), self.last_loss, 1)

    def _perturb(self):
        if self.mode in ('NN', 'autograd'):
            self.model.net.apply(self._r)

    def _fired(self):
        """The criterion that fires this epoch, or None."""
        loss = _num(self.model.cur_loss)
        if self.t % self.loss_window == 0:
            self._fit_line()
            if abs(self._line[0] / loss) < self.eps and self.t > 0:
                self._perturb()
                return 'window_check'
        if self.t - self._t_imp_start == self.no_improvement_patience:
            self._t_imp_start = self.t
            if self.mode in ('NN', 'autograd') and self.save_best:
                self.model.net = self.best_model
            self._perturb()
            return 'patience_check'
        if self.abs_loss is not None and loss < self.abs_loss:
            return 'absloss_check'
        return None

    def _state_line(self):
        import datetime
        if self._line is None:
            self._fit_line()
        loss = _num(self.model.cur_loss)
        return ('[{}] Step = {} loss = {:.6f} normalized loss line= {:.6f}x+{:.6f}. There was {} '
                'stop dings already.'.format(datetime.datetime.now(), self.t, loss,
                                             self._line[0] / loss, self._line[1] / loss,
                                             self._stop_dings))

    def on_epoch_begin(self, logs=None):
        import numpy as np
        self.t = self.model.t
        self.mode = self.model.mode
        self._check = self.model._check
        if self.last_loss is None:   # the first epoch fills the window with the initial loss
            self.last_loss = np.zeros(self.loss_window) + _num(self.model.min_loss)
        else:
            self.last_loss[(self.t - 3) % self.loss_window] = _num(self.model.cur_loss)

    def on_epoch_end(self, logs=None):
        import datetime
        if self._check is None:
            self._check = self._fired()
            if self._check is not None:
                self._stop_dings += 1
        if self.model.cur_loss < self.model.min_loss:
            self.model.min_loss = self.model.cur_loss
            if self.save_best:
                self.best_model = self.model.net
            self._t_imp_start = self.t
        if self.t % self.info_string_every == 0:
            print(self._state_line())
        if self.verbose and self._check is not None:
            print({'window_check': '[{}] Oscillation near the same loss',
                   'patience_check': '[{}] No improvement in {} steps',
                   'absloss_check': '[{}] Absolute value of loss is lower than threshold'}[
                       self._check].format(datetime.datetime.now(), self.no_improvement_patience))
            print(self._state_line())
        if self._stop_dings >= self.patience:
            self.model.stop_training = True
            if self.save_best:
                self.model.net = self.best_model
        self._check = None

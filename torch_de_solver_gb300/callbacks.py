"""Callback hooks with the reference's interface (tedeous/callbacks/callback.py:3-75,
tedeous/callbacks/callback_list.py:5-63) and the Cache callback, whose lookup uses the batched
evaluation of the device path.

Model.train calls on_train_begin, on_epoch_begin, on_epoch_end and on_train_end; a callback reads
model.cur_loss, model.min_loss, model.t, model.mode, model.net and model.solution_cls and may set
model.stop_training. These are the attributes the reference's own callbacks
(tedeous/callbacks/early_stopping.py, inverse_task.py, plot.py) read, so those run against this
Model unchanged; they are outside the training hot path and are not rebuilt here. A callback may
replace parameter data (`p.data = ...`): the device path copies the new values into its parameter
buffer before the next step."""


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


def _perturbation(eps):
    """A function that, applied to a network, adds (2 * randn - 1) * eps to the weight and then
    the bias of each of its Linear layers, in module order: the reference's randomisation of a
    cached network before training (tedeous/utils.py:14-30, applied at
    tedeous/callbacks/cache.py:326-331), drawing the same random numbers in the same order."""
    import torch

    def apply(net):
        for m in net.modules():
            if isinstance(m, torch.nn.Linear) and m.bias is not None:
                for p in (m.weight, m.bias):
                    noise = 2 * torch.randn(p.shape) - 1
                    p.data = p.data + noise.to(p) * eps
    return apply


def _empty_folder(folder):
    """Delete everything inside `folder`, reporting (not raising) what cannot be deleted; the
    effect of the reference's clear_cache (tedeous/utils.py:100-114)."""
    import pathlib
    import shutil
    for entry in pathlib.Path(folder).iterdir():
        try:
            if entry.is_dir() and not entry.is_symlink():
                shutil.rmtree(entry)
            else:
                entry.unlink()
        except OSError as err:
            print(f'cache: could not delete {entry}: {err}')


def count_output(model):
    """out_features of the last layer that has one (tedeous/callbacks/cache.py:21-35)."""
    for layer in reversed(list(model.modules())):
        if hasattr(layer, 'out_features'):
            return layer.out_features
    return None


def _as_layers(net):
    """The layer stack of a network: the network itself when it is indexable (nn.Sequential),
    else its `.model` attribute (a wrapper around one); None when it has neither."""
    import torch
    if isinstance(net, torch.nn.Sequential):
        return net
    inner = getattr(net, 'model', None)
    return inner if isinstance(inner, torch.nn.Sequential) else None


class CachePreprocessing:
    """Cache lookup and reuse for a compiled Model (the behaviour of
    tedeous/callbacks/cache.py:38-258). The lookup evaluates every usable cached network on the
    current problem in one launch per network shape (Solution.evaluate_many) instead of one
    evaluate per file, and keeps the reference's choice: the first network with the smallest
    loss, in the order of the files found."""

    def __init__(self, model):
        self.solution_cls = model.solution_cls

    @staticmethod
    def _pick(n_files, nmodels):
        """Indices of the files to consider: all of them in order, or `nmodels` drawn without
        replacement from numpy's global generator (as the reference draws them)."""
        import numpy as np
        if nmodels is None:
            return list(range(n_files))
        return list(np.random.choice(n_files, nmodels, replace=False))

    def _usable(self, net):
        """Whether a cached network can stand in for the solver's: the same inputs and outputs
        and a Linear/Tanh stack the device path evaluates."""
        from .solution import mlp_widths
        solver = self.solution_cls.model
        a, b = _as_layers(net), _as_layers(solver)
        if a is None or b is None:
            return False
        try:
            return (mlp_widths(a)[0] == mlp_widths(b)[0]
                    and count_output(net) == count_output(solver))
        except Exception:
            return False

    def cache_lookup(self, cache_dir, nmodels=None, save_graph=False, cache_verbose=False):
        """Best cached checkpoint {'model', 'model_state_dict'} by loss, or None. Files are found
        with the reference's pattern cache_dir + '\\*.tar' (tedeous/callbacks/cache.py:117),
        which matches the names Model saves under."""
        import glob
        import torch
        files = glob.glob(cache_dir + '\\*.tar')
        if cache_verbose:
            print(f'cache: searching {len(files)} saved networks in {cache_dir}')
        candidates = []
        for i in self._pick(len(files), nmodels) if files else []:
            try:
                ckpt = torch.load(files[i], weights_only=False, map_location='cpu')
                net = ckpt['model']
                net.load_state_dict(ckpt['model_state_dict'])
            except Exception as err:
                if cache_verbose:
                    print(f'cache: skipping {files[i]}: {err}')
                continue
            if self._usable(net):
                candidates.append((i, net))
        if not candidates:
            return None
        losses = self.solution_cls.evaluate_many([net for _, net in candidates])[:, 0].cpu()
        best = int(torch.argmin(losses))   # the first of equal minima, as the reference's '<'
        i, net = candidates[best]
        if cache_verbose:
            print(f'cache: best network is file {i} with loss {float(losses[best])}')
        return {'model': net, 'model_state_dict': net.state_dict()}

    def scheme_interp(self, trained_model, cache_verbose=False, tol=1e-5, max_steps=100000):
        """Fit the solver's network to a cached network of another architecture: Adam(lr=1e-3)
        on the mean squared difference of the two networks' outputs over the grid, until it is
        at most `tol` or `max_steps` steps have run (the stopping rule of
        tedeous/callbacks/cache.py:183-219). Plain torch on the device: this runs once, before
        training, and is not the hot path."""
        import torch
        sol = self.solution_cls
        grid = sol.grid.to(sol.device)
        net = sol.model
        with torch.no_grad():
            target = trained_model.to(sol.device)(grid)
        opt = torch.optim.Adam(net.parameters(), lr=0.001)
        for step in range(max_steps + 1):
            mse = torch.mean((target - net(grid)) ** 2)
            if cache_verbose and step:
                print(f'cache: interpolation step {step}, mse {float(mse.detach())}')
            if step == max_steps or float(mse.detach()) <= tol:
                break
            opt.zero_grad()
            mse.backward()
            opt.step()
        sol._model_change(net)

    def cache_retrain(self, cache_checkpoint, cache_verbose=False):
        """Start from the cached network: as it is when its layer widths equal the solver's,
        otherwise by fitting the solver's network to it (tedeous/callbacks/cache.py:221-258)."""
        from .solution import mlp_widths
        if cache_checkpoint is None:
            return None
        cached = cache_checkpoint['model']
        cached.load_state_dict(cache_checkpoint['model_state_dict'])
        solver = self.solution_cls.model
        try:
            same = mlp_widths(_as_layers(cached)) == mlp_widths(_as_layers(solver))
        except Exception:
            same = False
        if same:
            cached.train()
            self.solution_cls._model_change(cached)
            if cache_verbose:
                print('cache: training continues from the cached network')
        else:
            cached.eval()
            self.scheme_interp(cached, cache_verbose=cache_verbose)


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
            cache_dir = os.path.join(tempfile.gettempdir(), 'tedeous_cache/')
            os.makedirs(cache_dir, exist_ok=True)
        self.cache_dir = cache_dir
        if clear_cache:
            _empty_folder(self.cache_dir)

    def cache(self):
        if self.model.mode == 'mat':
            raise NotImplementedError("'mat' mode is not implemented on the device path")
        pre = CachePreprocessing(self.model)
        best = pre.cache_lookup(cache_dir=self.cache_dir, nmodels=self.nmodels,
                                cache_verbose=self.cache_verbose)
        pre.cache_retrain(best, cache_verbose=self.cache_verbose)
        _perturbation(self.model_randomize_parameter)(self.model.solution_cls.model)

    def on_train_begin(self, logs=None):
        self.cache()
        self.model._save_dir = self.cache_dir

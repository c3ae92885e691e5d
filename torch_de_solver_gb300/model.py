"""Model: compile() and train() with the reference's signatures (tedeous/model.py:25-195).

compile() builds the grid, evaluates boundary data, lowers the operator and boundary conditions
(prepare.lower) and creates the device plan behind a Solution. train() keeps the reference's loop:
an initial evaluate(), then epochs - 1 optimizer steps, callbacks around every epoch
(tedeous/model.py:154-193). With the fused Adam and no learning-rate scheduler, each step
(loss + gradient kernel, reductions, Adam update) is captured once in a CUDA graph and replayed.
"""

import copy
import datetime
import os
import tempfile
from typing import List, Union

import torch

from .callbacks import CallbackList
from .closure import Closure
from .data import Conditions, Domain, Equation
from .optimizer import FusedAdam, Optimizer
from .solution import Solution


def parameter_registr(model: torch.nn.Module, parameters: dict) -> None:
    """Registers each initial value in `parameters` as a one-element float32 nn.Parameter of
    `model` and replaces the dict entry by it, so that an equation term can use it as a trainable
    coefficient (tedeous/models.py:183-196)."""
    for key, value in parameters.items():
        parameters[key] = torch.nn.Parameter(torch.tensor([value], requires_grad=True).float())
        model.register_parameter(key, parameters[key])


class Model:
    def __init__(self, net: torch.nn.Module, domain: Domain, equation: Equation,
                 conditions: Conditions, batch_size: int = None, shard=None):
        """shard=(rank, world): one process per GPU, each evaluating its share of the
        collocation points; the gradient and loss are summed over the ranks of the default
        torch.distributed group every step (Solution), so every rank takes the same optimizer
        steps. Not in the reference, which runs on one device."""
        self.net = net
        self.shard = shard
        self.domain = domain
        self.equation = equation
        self.conditions = conditions
        self.batch_size = batch_size
        self._save_dir = os.path.join(tempfile.gettempdir(), 'tedeous_cache/')
        self._graph = None
        self._check = None   # read by the reference's early-stopping callback (tedeous/model.py:46)

    def compile(self, mode: str, lambda_operator: Union[List[float], float],
                lambda_bound: Union[List[float], float], normalized_loss_stop: bool = False,
                h: float = 0.001, inner_order: str = '1', boundary_order: str = '2',
                derivative_points: int = 2, weak_form: List[callable] = None, tol: float = 0,
                removed_domains: list = None, precision: str = None, form: str = None,
                autotune: bool = False):
        """Arguments as in tedeous/model.py:56-113, plus precision and form ('fused' or 'plain').
        precision: '3xtf32' (split-TF32 tensor cores at FP32 tolerance; the default of the fused
        form), 'fp32' (CUDA cores, bitwise reproducible gradient; the plain form's only one),
        'tf32' or 'bf16'. form=None is the fused form when the network's hidden widths are
        multiples of 4 up to 128, else the plain form (any width; see solution.default_form).
        autotune=True picks the fused kernel's tile schedule by timing candidates on the device
        (torch_de_solver_gb300.autotune)."""
        if weak_form:
            raise NotImplementedError('weak-form losses are not implemented on the device path')
        self.mode = mode
        self.lambda_bound = lambda_bound
        self.lambda_operator = lambda_operator
        self.normalized_loss_stop = normalized_loss_stop
        self.weak_form = weak_form
        grid = self.domain.build(mode=mode, removed_domains=removed_domains)
        bconds = self.conditions.build(self.domain.variable_dict)
        if self.batch_size is not None and len(grid) < self.batch_size:
            self.batch_size = None
        self.solution_cls = Solution(grid, self.equation.equation_lst, bconds, self.net, mode,
                                     lambda_operator, lambda_bound, h=h, inner_order=inner_order,
                                     boundary_order=boundary_order, precision=precision, form=form,
                                     tol=tol, batch_size=self.batch_size, shard=self.shard,
                                     autotune=autotune)
        self.net = self.solution_cls.model
        self._graph = None

    def _model_save(self, save_model: bool, model_name: str):
        """Writes {'model', 'model_state_dict'} of a CPU copy of the network to the cache folder
        under the reference's file name, cache_dir + '\\' + name + '.tar'
        (tedeous/utils.py:172-199), which its cache lookup pattern '\\*.tar' finds."""
        if save_model:
            os.makedirs(self._save_dir, exist_ok=True)
            name = model_name or str(datetime.datetime.now().timestamp())
            net = copy.deepcopy(self.net).to('cpu')
            torch.save({'model': net, 'model_state_dict': net.state_dict()},
                       self._save_dir + '\\' + name + '.tar')
            print(f'model is saved in cache dir: {self._save_dir}')

    def _fused_step(self, capture: bool):
        """loss+gradient, Adam; returns the (1,) loss seen before the update."""
        sol, opt = self.solution_cls, self.optimizer
        sol._sync_params()   # a callback may have replaced parameter data; the buffer stays put
        if self._graph is not None:
            self._graph.replay()
            return self._loss32[0:1]
        sol._launch(with_grad=True)
        opt.apply(sol._grad)
        if capture:
            self._loss32 = torch.empty(2, device=sol.device)
            stream = torch.cuda.Stream(sol.device)
            stream.wait_stream(torch.cuda.current_stream(sol.device))
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=stream):
                sol._launch(with_grad=True)
                self._loss32.copy_(sol._loss_buf)
                opt.apply(sol._grad)
            self._graph = g
            # the captured work did not run: the eager step above already advanced one step
        return sol._loss_buf[0:1].to(torch.float32)

    def train(self, optimizer: Optimizer, epochs: int, info_string_every: Union[int, None] = None,
              mixed_precision: bool = False, save_model: bool = False,
              model_name: Union[str, None] = None, callbacks: Union[List, None] = None):
        if mixed_precision:
            raise NotImplementedError('mixed_precision: choose compile(precision=...) instead')
        self.t = 1
        self.stop_training = False
        cbs = CallbackList(callbacks=callbacks, model=self)
        cbs.on_train_begin()
        self.solution_cls._sync_params()   # a callback may have swapped or re-seated the network
        self.net = self.solution_cls.model
        self.optimizer = optimizer.optimizer_choice(self.mode, self.net)
        closure = Closure(mixed_precision, self).get_closure(optimizer.optimizer)
        self.min_loss, _ = self.solution_cls.evaluate()
        self.cur_loss = self.min_loss
        print('[{}] initial (min) loss is {}'.format(datetime.datetime.now(), self.min_loss.item()))
        fused = (isinstance(self.optimizer, FusedAdam)
                 and self.optimizer._flat.data_ptr() == self.solution_cls.flat.data_ptr()
                 and optimizer.gamma is None
                 and optimizer.cosine_scheduler_patience is None and not self.normalized_loss_stop)
        self._graph = None
        n_eager = 0
        batches = self.solution_cls.batches
        steps = 1 if batches is None else batches.n_batches   # tedeous/model.py:178-185
        while self.t < epochs and self.stop_training is False:
            cbs.on_epoch_begin()
            self.optimizer.zero_grad()
            for _ in range(steps):
                if fused:   # mini-batch steps change their inputs on the host, sharded steps
                    # exchange through torch.distributed between launches: no graph for either
                    loss = self._fused_step(capture=(n_eager == 2 and batches is None
                                                     and self.shard is None))
                    n_eager += 1
                    self.cur_loss = loss.clone() if cbs.callbacks else loss
                else:
                    self.optimizer.step(closure)
                    if optimizer.gamma is not None and self.t % optimizer.decay_every == 0:
                        optimizer.scheduler.step()
            cbs.on_epoch_end()
            self.t += 1
            if info_string_every is not None and self.t % info_string_every == 0:
                print('This parameter info_string_every in train is obstolete, please use callbacks')
        self._graph = None
        self.solution_cls.check_status()   # a bounded device wait that gave up raises here
        cbs.on_train_end()
        self._model_save(save_model, model_name)


class BatchedModel:
    """Many independent solves trained together: every solve keeps its own grid, boundary data,
    equation coefficients and network, and one loss+gradient launch covers all of them (the tile
    scheduler spreads their uneven point counts over the persistent CTAs). The networks must share
    one shape; their parameters become views of one flat buffer [n_solves x P], so one fused Adam
    launch updates all solves and the whole step is captured once in a CUDA graph. The reference
    has no batched API: its equivalent is one Model per solve, trained one after another."""

    def __init__(self, models: List[Model]):
        if not models:
            raise ValueError('no models')
        self.models = list(models)

    def compile(self, mode: str, lambda_operator, lambda_bound, h: float = 0.001,
                inner_order: str = '1', boundary_order: str = '2', precision: str = None,
                autotune: bool = False):
        """autotune=True picks the tile schedule of the batched launch by timing candidates on
        the device (torch_de_solver_gb300.autotune, cached per problem shape and GPU);
        self.tuning then holds the search record."""
        from .prepare import lower
        from .solution import (DevicePlan, default_precision, device_parameters,
                               flatten_parameters, mlp_widths)
        if not torch.cuda.is_available():
            raise RuntimeError('torch_de_solver_gb300 runs on a CUDA device; none is available')
        dev = torch.device('cuda', torch.cuda.current_device())
        widths = mlp_widths(self.models[0].net)
        irs = []
        for m in self.models:
            if mlp_widths(m.net) != widths:
                raise ValueError('all networks of a batch must have the same shape')
            grid = m.domain.build(mode=mode)
            bconds = m.conditions.build(m.domain.variable_dict)
            irs.append(lower(grid, m.equation.equation_lst, bconds, mode, lambda_operator,
                             lambda_bound, h, inner_order, boundary_order, d_out=widths[-1]))
        self.mode = mode
        self.irs = irs
        prec = default_precision(precision, 'fused')
        schedule, self.tuning = None, None
        if autotune:
            from .autotune import tune
            schedule, self.tuning = tune(irs, widths, dev, prec)
        self.plan = DevicePlan(irs, widths, dev, prec, schedule=schedule)
        P = self.plan.n_params
        for m in self.models:
            m.net.to(dev)
        self.params = [device_parameters(m.net, ir.coeff_params) for m, ir in zip(self.models, irs)]
        self.flat = flatten_parameters([p for ps in self.params for p in ps], dev)
        assert self.flat.numel() == P * len(self.models)
        self.grad = torch.zeros_like(self.flat)
        self.loss = torch.zeros(2 * len(self.models), dtype=torch.float64, device=dev)
        self.outputs = torch.zeros(max(1, self.plan.n_outputs_total), device=dev)
        self.device = dev
        self._graph = None

    def evaluate(self, with_grad: bool = False):
        """Per-solve (loss, loss_normalized) as an (n_solves, 2) float64 tensor."""
        if with_grad:
            self.plan.loss_grad(self.flat, self.grad, self.loss, self.outputs)
        else:
            self.plan.loss(self.flat, self.loss, self.outputs)
        return self.loss.view(-1, 2)

    def train(self, lr: float = 1e-3, epochs: int = 1000, betas=(0.9, 0.999), eps: float = 1e-8,
              use_graph: bool = True):
        """Adam on every solve for epochs - 1 steps (the reference loop's count); returns the
        per-solve losses seen by the last step."""
        from . import _lib
        m = torch.zeros_like(self.flat)
        v = torch.zeros_like(self.flat)
        step = torch.zeros(1, device=self.device)
        hp = _lib.AdamDesc()
        hp.lr, (hp.beta1, hp.beta2), hp.eps, hp.weight_decay, hp.maximize = lr, betas, eps, 0.0, 0
        lib = _lib.load()

        def one_step():
            s = torch.cuda.current_stream(self.device)
            self.plan.loss_grad(self.flat, self.grad, self.loss, self.outputs, stream=s)
            _lib.check(lib.tdg_adam_step(self.flat.data_ptr(), self.grad.data_ptr(), m.data_ptr(),
                                         v.data_ptr(), step.data_ptr(), self.flat.numel(), hp,
                                         s.cuda_stream), 'tdg_adam_step')
        self.evaluate()
        graph = None
        for t in range(1, epochs):
            if graph is not None:
                graph.replay()
                continue
            one_step()
            if use_graph and t == 2:
                cap = torch.cuda.Stream(self.device)
                cap.wait_stream(torch.cuda.current_stream(self.device))
                graph = torch.cuda.CUDAGraph()
                with torch.cuda.graph(graph, stream=cap):
                    one_step()
        self._graph = graph
        _lib.check(lib.tdg_plan_sync_status(self.plan.handle), 'device status')
        return self.loss.view(-1, 2).clone()

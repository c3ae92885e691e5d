"""Solution: the per-step loss evaluation, backed by libtdg.so.

Drop-in for the reference's Solution (tedeous/solution.py:19-168): evaluate() returns
(loss, loss_normalized) as shape-(1,) tensors, and loss.backward() fills .grad of every MLP
parameter, so the reference's closure (tedeous/optimizers/closure.py:49-64) and torch optimizers
work unchanged. The attributes op, bval, true_bval, bval_keys and bval_length that callbacks read
are rebuilt on access from the per-row outputs the kernel writes.

The MLP parameters are re-seated as views into one flat FP32 device buffer, which the kernel
reads directly; the gradient comes back as one flat buffer and is handed to autograd as
per-parameter views.
"""

import ctypes
import warnings

import torch

from . import _lib
from .prepare import CoeffParam, lower, shard_ir


def fused_width_ok(widths):
    """Whether the fused kernels take these hidden widths (multiples of 4, at most MAX_WIDTH)."""
    return all(w % 4 == 0 and 4 <= w <= _lib.MAX_WIDTH for w in widths[1:-1])


def default_form(widths, precision, form):
    """form=None selects the fused form, unless a hidden width is one the fused kernels do not
    take (not a multiple of 4, or above 128, e.g. the 50-, 150- and 256-wide networks of the
    reference's examples): then the plain form, which takes any width and computes in FP32,
    with a warning. A tensor-core precision asked for with such a network raises."""
    if form is not None:
        return form
    if fused_width_ok(widths):
        return 'fused'
    if precision not in (None, 'fp32'):
        raise NotImplementedError(
            f'hidden widths {widths[1:-1]}: precision {precision!r} runs in the fused form, which '
            f'takes multiples of 4 up to {_lib.MAX_WIDTH}; the plain form (FP32) takes any width')
    warnings.warn(f'hidden widths {widths[1:-1]} are outside the fused kernels (multiples of 4 up '
                  f'to {_lib.MAX_WIDTH}): the step runs in the plain form (per-layer FP32 kernels)')
    return 'plain'


def default_precision(precision, form):
    """None selects split TF32 ('3xtf32', FP32 tolerance on the tensor cores) for the fused form
    and FP32 for the plain form, which computes in FP32 only."""
    if precision is not None:
        return precision
    return '3xtf32' if form == 'fused' else 'fp32'


def mlp_widths(net):
    """Widths of a torch.nn.Sequential of Linear layers separated by Tanh."""
    mods = list(net.children()) if isinstance(net, torch.nn.Sequential) else None
    if not mods:
        raise NotImplementedError('the device path needs a torch.nn.Sequential of Linear/Tanh')
    widths = []
    for i, m in enumerate(mods):
        if i % 2 == 0:
            if not isinstance(m, torch.nn.Linear) or m.bias is None:
                raise NotImplementedError(f'layer {i}: expected Linear with bias, got {m}')
            if not widths:
                widths.append(m.in_features)
            elif m.in_features != widths[-1]:
                raise ValueError('inconsistent Linear widths')
            widths.append(m.out_features)
        elif not isinstance(m, torch.nn.Tanh):
            raise NotImplementedError(f'layer {i}: only Tanh activations are implemented, got {m}')
    if len(mods) % 2 == 0:
        raise NotImplementedError('the network must end with a Linear layer')
    return widths


def device_parameters(net, coeff_params=(), strict=True):
    """The parameters in the order of the device's flat buffer: every Linear layer's weight and
    bias in layer order, then the equation's trainable coefficients (ProblemIR.coeff_params).
    Other parameters of `net` have no place on the device path: strict raises for them, otherwise
    they are left out (a network swapped in by _model_change may carry its own copies of the
    coefficients, which the equation does not use)."""
    lin = [m for m in net.children() if isinstance(m, torch.nn.Linear)]
    params = [q for m in lin for q in (m.weight, m.bias)] + list(coeff_params)
    known = set(map(id, params))
    for name, q in net.named_parameters():
        if strict and id(q) not in known:
            raise NotImplementedError(f'parameter {name!r} is neither a Linear weight or bias nor '
                                      f'a coefficient of the equation')
    return params


def flatten_parameters(params, device):
    """Make `params` views of one flat float32 buffer on `device`, in the order given."""
    flat = torch.cat([p.detach().reshape(-1).to(device=device, dtype=torch.float32)
                      for p in params])
    off = 0
    with torch.no_grad():
        for p in params:
            n = p.numel()
            p.data = flat[off:off + n].view(p.shape)
            off += n
    return flat


def params_are_views(params, flat):
    off = 0
    for p in params:
        if p.data.data_ptr() != flat.data_ptr() + 4 * off or p.dtype != torch.float32:
            return False
        off += p.numel()
    return off == flat.numel()


class DevicePlan:
    """A tdg_plan for one or more lowered problems (ProblemIR) sharing one MLP shape."""

    def __init__(self, irs, widths, device, precision='fp32', form='fused', schedule=None):
        """schedule: None for the default tile schedule, or a dict (max_rows, n_ctas, balance)
        as torch_de_solver_gb300.autotune finds (tdg_plan_create_scheduled)."""
        if precision not in _lib.PREC:
            raise ValueError(f'precision {precision!r}')
        if form not in _lib.FORM:
            raise ValueError(f'form {form!r}')
        lib = _lib.load()
        self.device = device
        self.widths = list(widths)
        streams, sites, parts, factors, terms, groups, slots = [], [], [], [], [], [], []
        self.arrays = []
        self.array_maps = []         # per problem: IR array key -> plan array index
        self.group_out = []          # per problem: list of (group, output offset) in IR order
        first_upload = {}            # id(ir) -> its array map; a repeated IR shares its arrays
        out_off = 0
        n_coeff = {len(ir.coeff_params) for ir in irs}
        if len(n_coeff) != 1:
            raise ValueError('the problems of one plan must have the same number of trainable '
                             'coefficients')
        self.n_coeff = n_coeff.pop()
        for prob, ir in enumerate(irs):
            own = {g.row_weight for g in ir.groups if g.row_weight is not None}
            shared = first_upload.get(id(ir))
            amap = {}
            for k, a in enumerate(ir.arrays):
                if shared is not None and k not in own:
                    amap[k] = shared[k]
                else:
                    amap[k] = len(self.arrays)
                    self.arrays.append(a.to(device).reshape(-1).contiguous())
            first_upload.setdefault(id(ir), amap)
            self.array_maps.append(amap)
            slot_base = len(slots)
            slots += [(prob, w, wn) for (_, w, wn) in ir.slots]
            offs = []
            for g in ir.groups:
                site_first = len(sites)
                for s in g.sites:
                    st_first = len(streams)
                    for axes in s.streams:
                        ax = list(axes) + [0] * (_lib.MAX_ORDER - len(axes))
                        streams.append(_lib.StreamDesc(len(axes), (ctypes.c_int32 * 3)(*ax)))
                    off = list(s.offset) + [0.0] * (_lib.MAX_DIN - len(s.offset))
                    sites.append(_lib.SiteDesc(amap[s.points], st_first, len(s.streams),
                                               (ctypes.c_float * _lib.MAX_DIN)(*off)))
                term_first = len(terms)
                for coeff, output, fl in g.terms:
                    f_first = len(factors)
                    for var, pw, pl in fl:
                        p_first = len(parts)
                        for site, stream, w in pl:
                            parts.append(_lib.PartDesc(site, stream, w))
                        factors.append(_lib.FactorDesc(p_first, len(pl), var, pw))
                    if isinstance(coeff, float):
                        terms.append(_lib.TermDesc(f_first, len(fl), output, -1, coeff, -1))
                    elif isinstance(coeff, CoeffParam):
                        terms.append(_lib.TermDesc(f_first, len(fl), output, -1, coeff.scale,
                                                   coeff.index))
                    else:
                        terms.append(_lib.TermDesc(f_first, len(fl), output, amap[coeff], 0.0, -1))
                tgt = -1 if g.target is None else amap[g.target]
                rw = -1 if g.row_weight is None else amap[g.row_weight]
                groups.append(_lib.GroupDesc(prob, g.n_rows, site_first, len(g.sites), term_first,
                                             len(g.terms), g.n_outputs, slot_base + g.slot_first,
                                             tgt, rw, out_off))
                offs.append(out_off)
                out_off += g.n_rows * g.n_outputs
            self.group_out.append(offs)
        self.n_outputs_total = out_off
        self.n_problems = len(irs)

        def arr(ctype, items):
            a = (ctype * max(1, len(items)))()
            for i, x in enumerate(items):
                a[i] = x
            return a
        self._keep = dict(
            streams=arr(_lib.StreamDesc, streams), sites=arr(_lib.SiteDesc, sites),
            parts=arr(_lib.PartDesc, parts), factors=arr(_lib.FactorDesc, factors),
            terms=arr(_lib.TermDesc, terms), groups=arr(_lib.GroupDesc, groups),
            slots=arr(_lib.SlotDesc, [_lib.SlotDesc(p, w, wn) for p, w, wn in slots]),
            ptrs=arr(ctypes.c_void_p, [t.data_ptr() for t in self.arrays]),
            lens=arr(ctypes.c_int64, [t.numel() for t in self.arrays]))
        k = self._keep
        mlp = _lib.MlpDesc()
        mlp.n_layers = len(widths) - 1
        for i, w in enumerate(widths):
            mlp.width[i] = w
        desc = _lib.ProblemDesc(
            mlp, len(irs), len(groups), k['groups'], len(sites), k['sites'], len(streams),
            k['streams'], len(terms), k['terms'], len(factors), k['factors'], len(parts),
            k['parts'], len(slots), k['slots'], len(self.arrays), k['ptrs'], k['lens'],
            _lib.PREC[precision], _lib.FORM[form], self.n_coeff)
        handle = ctypes.c_void_p()
        self.schedule = None if schedule is None else dict(schedule)
        with torch.cuda.device(device):
            if schedule is None:
                _lib.check(lib.tdg_plan_create(ctypes.byref(desc), ctypes.byref(handle)),
                           'tdg_plan_create')
            else:
                sc = _lib.Schedule(int(schedule.get('max_rows', 128)),
                                   int(schedule.get('n_ctas', 0)), int(schedule.get('balance', 0)), 0)
                _lib.check(lib.tdg_plan_create_scheduled(ctypes.byref(desc), ctypes.byref(sc),
                                                         ctypes.byref(handle)),
                           'tdg_plan_create_scheduled')
        self.handle = handle
        info = _lib.PlanInfo()
        _lib.check(lib.tdg_plan_get_info(handle, ctypes.byref(info)), 'tdg_plan_get_info')
        self.info = info
        self.n_params = int(info.n_params)

    def __del__(self):
        h = getattr(self, 'handle', None)
        if h is not None and h.value:
            try:
                _lib.load().tdg_plan_destroy(h)
            except Exception:
                pass
            self.handle = None

    def set_array(self, index, tensor):
        _lib.check(_lib.load().tdg_plan_set_array(self.handle, index, tensor.data_ptr(),
                                                  tensor.numel()), 'tdg_plan_set_array')

    def loss_grad(self, params, grad, loss, outputs=None, stream=None):
        s = torch.cuda.current_stream(self.device) if stream is None else stream
        _lib.check(_lib.load().tdg_loss_grad(
            self.handle, params.data_ptr(), grad.data_ptr(), loss.data_ptr(),
            None if outputs is None else outputs.data_ptr(), s.cuda_stream), 'tdg_loss_grad')

    def loss(self, params, loss, outputs=None, stream=None):
        s = torch.cuda.current_stream(self.device) if stream is None else stream
        _lib.check(_lib.load().tdg_loss(
            self.handle, params.data_ptr(), loss.data_ptr(),
            None if outputs is None else outputs.data_ptr(), s.cuda_stream), 'tdg_loss')


def allreduce_sum(*tensors):
    """Sum each tensor over the ranks of the default torch.distributed process group (NCCL
    between GPUs, gloo on CPU), in place; nothing without an initialised group of more than one
    rank. The one exchange of a point-sharded step: the flat parameter gradient and the FP64
    (loss, loss_normalized) partials."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return
    for t in tensors:
        if t is not None:
            dist.all_reduce(t, op=dist.ReduceOp.SUM)


class _FusedLoss(torch.autograd.Function):
    """(loss, loss_normalized) of the current parameters; the gradient is computed in the same
    fused launch and returned, scaled by the incoming gradient, in backward()."""

    @staticmethod
    def forward(ctx, sol, *params):
        sol._launch(with_grad=True)
        ctx.sol = sol
        grad = sol._grad.clone() if sol._clone_grad else sol._grad
        ctx.save_for_backward(grad)
        loss = sol._loss_buf[0:1].to(torch.float32)
        lossn = sol._loss_buf[1:2].to(torch.float32)
        ctx.mark_non_differentiable(lossn)
        return loss, lossn

    @staticmethod
    def backward(ctx, g_loss, g_lossn):
        grad, = ctx.saved_tensors
        g = grad * g_loss.reshape(()).to(grad.dtype)
        out = []
        off = 0
        for shape, n in ctx.sol._shapes:
            out.append(g[off:off + n].view(shape))
            off += n
        return (None, *out)


def _residual_row_arrays(ir):
    """Array keys of the residual group that hold one entry (or row) per residual point: its site
    points and per-row coefficients, in first-reference order."""
    g = ir.groups[ir.residual_group]
    keys = []
    for k in [s.points for s in g.sites] + [c for c, _, _ in g.terms if isinstance(c, int)]:
        if k not in keys:
            keys.append(k)
    return keys


class _Batches:
    """Mini-batches of the collocation points with the reference's order: a shuffling DataLoader
    with an unseeded torch.Generator over the (type-sorted) grid; each residual evaluation takes
    the current batch and moves on, and a new pass starts after the last batch
    (tedeous/eval.py:119-144, _pde_compute :172-183). It draws indices, which select the same
    rows that the reference's DataLoader over the points draws."""

    def __init__(self, n, batch_size):
        from torch.utils.data import DataLoader
        self.loader = DataLoader(torch.arange(n), batch_size=batch_size, shuffle=True,
                                 generator=torch.Generator())
        self.n_batches = len(self.loader)
        self._it = iter(self.loader)
        self._next = next(self._it)

    def take(self):
        idx = self._next
        try:
            self._next = next(self._it)
        except StopIteration:
            self._it = iter(self.loader)
            self._next = next(self._it)
        return idx


class Solution:
    """Loss evaluation of one compiled problem (tedeous/solution.py:19-168).

    tol != 0 selects the causal loss: a forward-only launch writes the residual field, then
    tdg_causal_weights turns it into per-row weights, then the loss and gradient launch applies
    them. batch_size selects mini-batches of the collocation points: in 'autograd' mode each
    evaluation gathers the batch's points (and per-point coefficients) with tdg_gather_rows into
    a plan made for that batch size; 'NN' terms ignore the batch, as the reference's do.
    shard=(rank, world) evaluates this rank's contiguous share of the residual rows (rank 0 also
    the boundary conditions, prepare.shard_ir) and sums the gradient and the loss over the ranks
    of the default torch.distributed group after every launch (allreduce_sum); without an
    initialised group the per-rank parts are returned as they are. autotune=True times the
    candidate tile schedules of torch_de_solver_gb300.autotune on this problem (cached per shape
    and GPU) and builds the plans with the fastest."""

    def __init__(self, grid, operator, bconds, model, mode, lambda_operator, lambda_bound,
                 h=0.001, inner_order='1', boundary_order='2', precision=None, form=None,
                 device=None, tol=0, batch_size=None, shard=None, autotune=False):
        if not torch.cuda.is_available():
            raise RuntimeError('torch_de_solver_gb300 runs on a CUDA device; none is available')
        self.device = torch.device('cuda', torch.cuda.current_device()) if device is None \
            else torch.device(device)
        self.mode = mode
        self.grid = grid
        self.lambda_operator, self.lambda_bound = lambda_operator, lambda_bound
        widths = mlp_widths(model)
        form = default_form(widths, precision, form)
        self.precision, self.form = default_precision(precision, form), form
        if batch_size is not None and mode == 'NN' and tol:
            raise NotImplementedError("the causal loss with mini-batches in 'NN' mode (the "
                                      "reference's time-slice count fails there)")
        args = (operator, bconds, mode, lambda_operator, lambda_bound, h, inner_order,
                boundary_order)
        self.ir = lower(grid, *args, d_out=widths[-1], tol=tol)
        self.shard = None
        if shard is not None:
            if batch_size is not None:
                raise NotImplementedError('mini-batches of a point-sharded problem')
            self.shard = tuple(shard)
            self.ir = shard_ir(self.ir, *self.shard)
        self.model = model.to(self.device)
        self.params = device_parameters(self.model, self.ir.coeff_params)
        self.flat = flatten_parameters(self.params, self.device)
        self._shapes = [(p.shape, p.numel()) for p in self.params]
        self.batches = None if batch_size is None else _Batches(grid.shape[0], batch_size)
        self._full_ir = self.ir
        self._irs = {}                # residual rows -> (ProblemIR, [(batch key, full key)])
        self._row_src = {}
        if self.batches is not None and mode == 'autograd':
            # one plan per batch size (full batches and the last, shorter one), each lowered on
            # placeholder rows that every evaluation overwrites by a gather from the full arrays
            full = _residual_row_arrays(self.ir)
            n_grid = grid.shape[0]
            sizes = sorted({min(batch_size, n_grid - i) for i in range(0, n_grid, batch_size)},
                           reverse=True)
            self._row_src = {k: self.ir.arrays[k].to(self.device).reshape(-1) for k in full}
            for n in sizes:
                ir_b = lower(grid[:n], *args, d_out=widths[-1], tol=tol)
                if len(ir_b.coeff_params) != len(self.ir.coeff_params):
                    raise RuntimeError('batch lowering changed the trainable coefficients')
                ir_b.coeff_params = self.ir.coeff_params
                self._irs[n] = (ir_b, list(zip(_residual_row_arrays(ir_b), full)))
            self._idx = torch.zeros(batch_size, dtype=torch.int64, device=self.device)
        else:
            self._irs[self.ir.groups[self.ir.residual_group].n_rows] = (self.ir, [])
        self._loss_buf = torch.zeros(2, device=self.device, dtype=torch.float64)
        self.schedule, self.tuning = None, None
        if autotune and self.form == 'fused':
            from .autotune import tune
            self.schedule, self.tuning = tune([self.ir], widths, self.device, self.precision)
        self._build_plans(widths)
        self._clone_grad = True
        self.bval_keys = list(self.ir.bc_types)
        self.bval_length = [sum(r for _, r in self.ir.bc_parts[t]) for t in self.ir.bc_types]
        self._true_bval = None

    def _build_plans(self, widths):
        """Device plans of this problem for an MLP of `widths` (one per residual batch size)."""
        self._plans = {}
        n_grid = self.grid.shape[0]
        for n, (ir, keys) in self._irs.items():
            plan = DevicePlan([ir], widths, self.device, self.precision, self.form,
                              schedule=getattr(self, 'schedule', None))
            gathers = [(plan.arrays[plan.array_maps[0][kb]], self._row_src[kf],
                        self._full_ir.arrays[kf].numel() // n_grid) for kb, kf in keys]
            self._plans[n] = (ir, plan, gathers)
        first = next(iter(self._irs))
        self.ir, self.plan, _ = self._plans[first]
        self._grad = torch.zeros(self.plan.n_params, device=self.device, dtype=torch.float32)
        self._out_bufs = {n: torch.zeros(max(1, p.n_outputs_total), device=self.device)
                          for n, (_, p, _) in self._plans.items()}
        self._outputs = self._out_bufs[first]

    # -- parameters --------------------------------------------------------------------------
    def _model_change(self, new_model):
        """Swap in another network (tedeous/solution.py:109-127). A network of another shape
        (same inputs and outputs) gets new device plans of this problem."""
        widths = mlp_widths(new_model)
        if widths != self.plan.widths:
            if widths[0] != self.plan.widths[0] or widths[-1] != self.plan.widths[-1]:
                raise ValueError('new model has other inputs or outputs')
            self._build_plans(widths)
        self.model = new_model.to(self.device)
        self.params = device_parameters(self.model, self.ir.coeff_params, strict=False)
        self.flat = flatten_parameters(self.params, self.device)
        self._shapes = [(p.shape, p.numel()) for p in self.params]

    def _sync_params(self):
        """Parameters whose data a caller replaced (`p.data = ...`, as the reference's
        randomisation in callbacks does) are copied back into the flat buffer and seated as its
        views again. The buffer keeps its address, so a captured training step, the fused Adam
        state and the plans stay valid."""
        if params_are_views(self.params, self.flat):
            return
        if sum(p.numel() for p in self.params) != self.flat.numel():
            # the device plans, a captured step and the fused Adam state all hold the old
            # parameter layout: a changed layout cannot be trained from silently
            raise _lib.TdgError('the parameter layout changed after compile (another number of '
                                'parameter elements); swap networks with _model_change or '
                                'compile again')
        off = 0
        with torch.no_grad():
            for p in self.params:
                n = p.numel()
                view = self.flat[off:off + n].view(p.shape)
                if p.data.data_ptr() != view.data_ptr():
                    view.copy_(p.data.reshape(p.shape).to(view))
                    p.data = view
                off += n

    # -- evaluation --------------------------------------------------------------------------
    def _select_batch(self):
        """'autograd' mini-batch mode: gather the next batch into the plan of its size."""
        idx = self.batches.take()
        n = idx.numel()
        self.ir, self.plan, gathers = self._plans[n]
        self._outputs = self._out_bufs[n]
        self._idx[:n].copy_(idx, non_blocking=True)
        lib = _lib.load()
        stream = torch.cuda.current_stream(self.device).cuda_stream
        n_src = self.grid.shape[0]
        for dst, src, row_len in gathers:
            _lib.check(lib.tdg_gather_rows(src.data_ptr(), n_src, self._idx.data_ptr(), n,
                                           row_len, dst.data_ptr(), stream), 'tdg_gather_rows')

    def _causal_weights(self):
        """Forward-only launch for the residual field, then its causal row weights."""
        ir = self.ir
        tol, n_t = ir.causal
        res = ir.groups[ir.residual_group]
        self.plan.loss(self.flat, self._loss_buf, self._outputs)
        off = self.plan.group_out[0][ir.residual_group]
        if self.batches is not None:   # tedeous/solution.py:54 applied to the operator
            op0 = self._outputs[off:off + res.n_rows * ir.n_eq].view(-1, ir.n_eq)[:, 0]
            n_t = int(torch.unique(op0).numel())
            if res.n_rows % n_t:
                n_t = res.n_rows
        w = self.plan.arrays[self.plan.array_maps[0][res.row_weight]]
        _lib.check(_lib.load().tdg_causal_weights(
            self._outputs.data_ptr() + 4 * off, res.n_rows, ir.n_eq, n_t, tol, w.data_ptr(),
            torch.cuda.current_stream(self.device).cuda_stream), 'tdg_causal_weights')

    def _launch(self, with_grad):
        if self.batches is not None and self.mode == 'autograd':
            self._select_batch()
        elif self.batches is not None:
            self.batches.take()
        if self.ir.causal is not None:
            self._causal_weights()
        if with_grad:
            self.plan.loss_grad(self.flat, self._grad, self._loss_buf, self._outputs)
        else:
            self.plan.loss(self.flat, self._loss_buf, self._outputs)
        if self.shard is not None:   # this rank's rows -> the whole problem's loss and gradient
            allreduce_sum(self._grad if with_grad else None, self._loss_buf)

    def evaluate(self, save_graph: bool = True):
        """(loss, loss_normalized), each of shape (1,) like the reference's."""
        self._sync_params()
        params = self.params
        if save_graph and torch.is_grad_enabled() and any(p.requires_grad for p in params):
            self.loss, self.loss_normalized = _FusedLoss.apply(self, *params)
        else:
            self._launch(with_grad=False)
            self.loss = self._loss_buf[0:1].to(torch.float32)
            self.loss_normalized = self._loss_buf[1:2].to(torch.float32)
        return self.loss, self.loss_normalized

    def check_status(self):
        """Raises TdgError if a kernel of this solution gave up a bounded device wait since the
        plan was made (its results are then not to be trusted). Synchronises the device."""
        for _, plan, _ in self._plans.values():
            _lib.check(_lib.load().tdg_plan_sync_status(plan.handle), 'device status')

    def evaluate_many(self, models):
        """(loss, loss_normalized) of each network on this problem as an (n, 2) float64 device
        tensor. The reference's cache lookup evaluates cached networks one at a time
        (tedeous/callbacks/cache.py:133-171: _model_change, then evaluate(save_graph=False)); here
        the networks of one shape form the parameter sets of one plan over this problem, so one
        forward-only launch evaluates all of them (the causal loss adds its weight pass). The
        trainable coefficients keep this solution's current values for every network, as in
        the reference, whose equation keeps its own parameters across _model_change. In
        mini-batch mode the networks are evaluated one after another, each on the next batch,
        as the reference does."""
        models = list(models)
        out = torch.zeros(len(models), 2, dtype=torch.float64, device=self.device)
        if self.batches is not None:
            keep = self.model
            for i, m in enumerate(models):
                self._model_change(m)
                loss, lossn = self.evaluate(save_graph=False)
                out[i, 0], out[i, 1] = loss[0], lossn[0]
            self._model_change(keep)
            return out
        self._sync_params()
        n_coeff = len(self.ir.coeff_params)
        theta = self.flat[self.flat.numel() - n_coeff:] if n_coeff else None
        by_shape = {}
        for i, m in enumerate(models):
            by_shape.setdefault(tuple(mlp_widths(m)), []).append(i)
        lib = _lib.load()
        stream = torch.cuda.current_stream(self.device).cuda_stream
        for widths, idx in by_shape.items():
            plan = DevicePlan([self.ir] * len(idx), widths, self.device, self.precision, self.form)
            P = plan.n_params
            flat = torch.empty(len(idx), P, dtype=torch.float32, device=self.device)
            for j, i in enumerate(idx):
                lin = device_parameters(models[i], strict=False)
                flat[j, :P - n_coeff] = torch.cat([q.detach().reshape(-1).to(self.device, torch.float32)
                                                   for q in lin])
                if n_coeff:
                    flat[j, P - n_coeff:] = theta
            loss = torch.zeros(2 * len(idx), dtype=torch.float64, device=self.device)
            outputs = torch.zeros(max(1, plan.n_outputs_total), device=self.device)
            if self.ir.causal is not None:
                tol, n_t = self.ir.causal
                res = self.ir.groups[self.ir.residual_group]
                plan.loss(flat, loss, outputs)
                for j in range(len(idx)):
                    off = plan.group_out[j][self.ir.residual_group]
                    w = plan.arrays[plan.array_maps[j][res.row_weight]]
                    _lib.check(lib.tdg_causal_weights(outputs.data_ptr() + 4 * off, res.n_rows,
                                                      self.ir.n_eq, n_t, tol, w.data_ptr(), stream),
                               'tdg_causal_weights')
            plan.loss(flat, loss, outputs)
            out[torch.tensor(idx, device=self.device)] = loss.view(-1, 2)
        return out

    # -- fields read by callbacks ------------------------------------------------------------
    @property
    def op(self):
        ir = self.ir
        off = self.plan.group_out[0][ir.residual_group]
        return self._outputs[off:off + ir.n_residual_rows * ir.n_eq].view(-1, ir.n_eq).clone()

    def _bc_columns(self, true):
        ir = self.ir
        cols = []
        for t in ir.bc_types:
            if true:
                v = torch.cat([x.reshape(-1) for x in ir.bc_true[t]]).to(self.device)
            else:
                pieces = [torch.zeros(0, device=self.device)]   # no pieces on a shard > 0
                for gi, n in ir.bc_parts[t]:
                    off = self.plan.group_out[0][gi]
                    pieces.append(self._outputs[off:off + n])
                v = torch.cat(pieces)
            cols.append(torch.nn.functional.pad(v, (0, ir.max_len - v.numel())))
        return torch.stack(cols, 1)

    @property
    def bval(self):
        return self._bc_columns(False)

    @property
    def true_bval(self):
        if self._true_bval is None:
            self._true_bval = self._bc_columns(True)
        return self._true_bval

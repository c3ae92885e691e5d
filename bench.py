"""Benchmark of the training hot path: one step = residual + boundary terms + loss + parameter
gradient of every collocation point, then the Adam update.

Workload (default): steady 2D Navier-Stokes, Kovasznay flow at Re=20, 'autograd' mode, MLP
2->128x5->3 tanh, 1024x1024 = 1,048,576 collocation points plus 4 x 1024 Dirichlet points per
output. Synthetic, seeded inputs: the grid and the closed-form boundary values are generated here;
the network is seeded torch default init.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload kovasznay|burgers|kdv|heat|sweep] [--points-per-axis n]
                  [--precision 3xtf32|fp32|tf32|bf16] [--form fused|plain]
                  [--optimizer adam|lbfgs] [--no-compare] [--no-cpu-baseline] [--no-autotune]

Our arm prints one JSON line with the device-resident throughput (value), the end-to-end
throughput through the public API with host buffers (e2e), the roofline of the fused kernel, the
plain form on the same workload (plain_ms_per_step, fused_vs_plain), the reference's operation
sequence through ATen/cuBLAS on the GPU (aten_reference), a CPU baseline (the oracle's
restatement of the reference algorithm on the host cores, on a bounded sample), sampled GPU clocks
and the number of library kernel launches. --optimizer lbfgs times L-BFGS iterations instead;
--workload sweep times the 256-solve batched sweep with its autotuned schedule against 256
sequential solves. --impl reference times the CPU restatement alone on the same workload family,
honouring --steps and --warmup.
"""

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, 'tests'))

METRIC = 'train steps/s & colloc pts/s, fused jet+adjoint vs plain path, 1 GB300, at tol'
UNIT = 'colloc_pts/s'
L2_BYTES = 129 * 1024 * 1024

WORKLOADS = {
    # name: (case builder name, kwargs at full size, kwargs of the CPU sample, description)
    'kovasznay': ('kovasznay_ag', dict(n=1023), dict(n=255),
                  'kovasznay_re20_autograd_2-128x5-3_1024x1024'),
    'burgers': ('burgers_ag', dict(n=100), dict(n=100), 'burgers_autograd_2-32x4-1_101x101'),
    'kdv': ('kdv_ag', dict(nx=255, nt=127), dict(nx=127, nt=63), 'kdv_autograd_2-64x4-1_256x128'),
    'heat': ('heat_nn', dict(n=20), dict(n=20), 'heat_nn_2-100x3-1_21x21'),
    'sweep': ('sweep_ag', dict(n_solves=256), dict(n_solves=2),
              'sweep_256_solves_autograd_2-64x3-1_Nx,Nt~U{16..128}'),
}
# the reference's operation sequence (nested autograd.grad, double backward, torch Adam) through
# ATen/cuBLAS on the GPU: the largest sample that fits beside the rest of the run
ATEN_SAMPLE = {'kovasznay': dict(n=511), 'burgers': dict(n=100), 'kdv': dict(nx=255, nt=127),
               'heat': dict(n=20)}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=20)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--workload', default='kovasznay', choices=sorted(WORKLOADS))
    ap.add_argument('--points-per-axis', type=int, default=None)
    ap.add_argument('--precision', default='3xtf32', choices=['fp32', '3xtf32', 'tf32', 'bf16'])
    ap.add_argument('--form', default='fused', choices=['fused', 'plain'])
    ap.add_argument('--no-compare', action='store_true',
                    help='skip the plain-form and ATen timings of the same workload')
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--no-autotune', action='store_true',
                    help='sweep: keep the default tile schedule instead of the autotuned one')
    ap.add_argument('--optimizer', default='adam', choices=['adam', 'lbfgs'],
                    help='lbfgs: time L-BFGS iterations (device history, FP64 dots, strong-Wolfe '
                         'line search) instead of Adam steps')
    return ap.parse_args()


def builder_for(name, kw):
    import cases
    fn = getattr(cases, WORKLOADS[name][0])
    return lambda api, dtype='float32': fn(api, dtype=dtype, **kw)


def sweep_builders(n_solves):
    """One case builder per solve of the equation-discovery sweep (coefficients, grid sizes and
    network seeds drawn as in cases.sweep_params)."""
    import cases
    out = []
    for i, sp in enumerate(cases.sweep_params(n_solves)):
        out.append(lambda api, dtype='float32', sp=sp, i=i:
                   cases.sweep_ag(api, seed=1000 + i, dtype=dtype, **sp))
    return out


def full_kwargs(args):
    kw = dict(WORKLOADS[args.workload][1])
    if args.points_per_axis:
        if 'n' in kw:
            kw['n'] = args.points_per_axis - 1
        else:
            kw['nx'] = kw['nt'] = args.points_per_axis - 1
    return kw


# ----------------------------------------------------------------------------- CPU baseline
def cpu_baseline(args, warmup, steps):
    """The oracle (fp32 restatement of the reference path: nested autograd.grad + double backward,
    torch.optim.Adam) on all host cores, on a bounded sample of the workload: `warmup` untimed
    steps, then `steps` timed ones. The sample's per-point rate stands for the full workload
    ('extrapolated' when the sample is smaller: the CPU's per-point rate falls as N grows, so
    the figure flatters the CPU)."""
    import torch
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    kw = WORKLOADS[args.workload][2]
    if args.workload == 'sweep':
        built = [O.build_problem(b, 'float32') for b in sweep_builders(kw['n_solves'])]
    else:
        built = [O.build_problem(builder_for(args.workload, kw), 'float32')]
    n_pts = sum(prob.points.shape[0] for prob, _ in built)
    opts = [torch.optim.Adam(net.parameters(), lr=1e-3) for _, net in built]

    def step():
        for (prob, net), opt in zip(built, opts):
            opt.zero_grad()
            r = prob.evaluate(net)
            r['loss'].backward()
            opt.step()
    for _ in range(warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    sec = (time.perf_counter() - t0) / max(1, steps)
    full = full_points(args)
    scaled = 'extrapolated' if n_pts < full else 'same size'
    return dict(value=n_pts / sec, unit=UNIT, cores=threads, kind='port',
                sample=f'{WORKLOADS[args.workload][0]} {kw}: {n_pts} residual points '
                       f'({scaled}; the workload has {full}), {warmup} + {steps} Adam steps, '
                       f'{sec * 1e3:.1f} ms/step, torch {torch.__version__} fp32 on {threads} '
                       f'threads',
                steps_per_s=1.0 / sec, points=n_pts, scaling=scaled)


def full_points(args):
    """Residual points of the full workload (autograd mode: every grid node)."""
    import cases
    if args.workload == 'sweep':
        return sum(p['nx'] * p['nt'] for p in cases.sweep_params(WORKLOADS['sweep'][1]['n_solves']))
    kw = full_kwargs(args)
    if 'nx' in kw:
        return (kw['nx'] + 1) * (kw['nt'] + 1)
    if args.workload == 'heat':
        return (kw['n'] - 1) ** 2   # 'NN' mode: the central points
    return (kw['n'] + 1) ** 2


def aten_reference(args):
    """The reference's operation sequence on the GPU through ATen/cuBLAS: the oracle (nested
    autograd.grad per derivative term, double backward, torch.optim.Adam) in FP32 on the CUDA
    device, at the largest sample of the workload that fits beside the rest of the run. This is
    the GPU form of the reference's own path (its solver_device('cuda') runs the same ops).
    Returns a per-point rate with the sample size stated."""
    import torch
    from oracle import oracle as O
    if args.workload not in ATEN_SAMPLE:
        return None
    kw = ATEN_SAMPLE[args.workload]
    prob, net = O.build_problem(builder_for(args.workload, kw), 'float32')
    prob.to('cuda')
    net = net.to('cuda')
    opt = torch.optim.Adam(net.parameters(), lr=1e-3)

    def step():
        opt.zero_grad()
        r = prob.evaluate(net)
        r['loss'].backward()
        opt.step()
    for _ in range(2):
        step()
    torch.cuda.synchronize()
    n_steps = 5
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(n_steps):
        step()
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / n_steps
    n_pts = prob.points.shape[0]
    peak_gb = torch.cuda.max_memory_allocated() / 1e9
    del prob, net, opt
    torch.cuda.empty_cache()
    return {'value': round(n_pts / (ms / 1e3), 1), 'unit': UNIT, 'points': n_pts,
            'ms_per_step': round(ms, 3),
            'sample': f'{WORKLOADS[args.workload][0]} {kw}: {n_pts} points, 2 + {n_steps} Adam '
                      f'steps, FP32 (TF32 matmul off), peak {peak_gb:.0f} GB allocated',
            'scaling': 'extrapolated' if n_pts < full_points(args) else 'same size'}


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
              'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', f'--id={self.index}', f'--query-gpu={self.FIELDS}',
                 '--format=csv,noheader,nounits', '-lms', '100'],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for ln in getattr(self, 'lines', []):
            f = [x.strip() for x in ln.split(',')]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == 'active':
                    reasons.add(n)
        return {'sm_mhz': statistics.median(sm) if sm else None, 'sm_max_mhz': mx,
                'reasons': sorted(reasons), 'samples': len(sm)}


# ----------------------------------------------------------------------------- multi-rank
def max_over_ranks(value, device):
    """The largest value over all ranks (the step time every rank waits for); identity when the
    job runs without torch.distributed. Ranks are independent replicas: this timing reduction is
    the only collective."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ----------------------------------------------------------------------------- our arm
def read_traffic(tag):
    """DRAM bytes per collocation point of the fused kernel from a committed ncu summary."""
    path = os.path.join(ROOT, 'profiles', f'{tag}.txt')
    if not os.path.exists(path):
        return None
    for ln in open(path):
        if ln.strip().startswith('dram_bytes_per_point:'):
            return float(ln.split(':')[1])
    return None


def sequential_sweep_ms(args, form, precision, steps):
    """The reference's way of running the sweep on the GPU: one Model per solve, trained one after
    another (tedeous/model.py:134-195 has no batched API). Each solve's step (loss+gradient
    launch(es), Adam) is timed over `steps` steps after one warm-up with CUDA events; the sum over
    the solves is the time of one sweep step."""
    import torch
    import torch_de_solver_gb300 as T
    total = 0.0
    for b in sweep_builders(WORKLOADS['sweep'][1]['n_solves']):
        d, bc, eq, net, kw = b(T)
        kw = dict(kw)
        model = T.Model(net, d, eq, bc)
        model.compile(kw.pop('mode'), precision=precision, form=form, **kw)
        sol = model.solution_cls
        opt = T.Optimizer('Adam', {'lr': 1e-3}).optimizer_choice(model.mode, model.net)

        def step():
            sol.plan.loss_grad(sol.flat, sol._grad, sol._loss_buf, sol._outputs)
            opt.apply(sol._grad)
        step()
        a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(steps):
            step()
        e.record()
        torch.cuda.synchronize()
        total += a.elapsed_time(e) / steps
        del model, sol, opt
    return total


def run_sweep(args, world):
    """256 solves of u_t = a u_xx + b u u_x + c u in one loss+gradient launch per step, one
    batched Adam launch, against 256 separate solves on the CPU sample."""
    import torch
    import torch_de_solver_gb300 as T
    from torch_de_solver_gb300 import _lib
    dev = torch.device('cuda', int(os.environ.get('LOCAL_RANK', 0)))
    torch.cuda.set_device(dev)
    n_solves = WORKLOADS['sweep'][1]['n_solves']
    models = []
    for b in sweep_builders(n_solves):
        d, bc, eq, net, kw = b(T)
        models.append(T.Model(net, d, eq, bc))
    bm = T.BatchedModel(models)
    bm.compile('autograd', lambda_operator=1, lambda_bound=1, precision=args.precision,
               autotune=not args.no_autotune)
    n_pts = sum(ir.n_residual_rows for ir in bm.irs)
    flush = torch.empty(2 * L2_BYTES // 4, device=dev)
    stream = torch.cuda.current_stream(dev)
    m = torch.zeros_like(bm.flat); v = torch.zeros_like(bm.flat); st = torch.zeros(1, device=dev)
    hp = _lib.AdamDesc()
    hp.lr, hp.beta1, hp.beta2, hp.eps = 1e-3, 0.9, 0.999, 1e-8
    lib = _lib.load()

    def step():
        bm.plan.loss_grad(bm.flat, bm.grad, bm.loss, bm.outputs)
        _lib.check(lib.tdg_adam_step(bm.flat.data_ptr(), bm.grad.data_ptr(), m.data_ptr(),
                                     v.data_ptr(), st.data_ptr(), bm.flat.numel(), hp,
                                     stream.cuda_stream), 'adam')
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    l0 = _lib.launch_count()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev.index) as clk:
        for a, b in ev:
            flush.zero_()
            a.record(stream)
            step()
            b.record(stream)
        torch.cuda.synchronize()
    launches = _lib.launch_count() - l0
    ms = max_over_ranks(statistics.mean(a.elapsed_time(b) for a, b in ev), dev)
    # end to end: host copies of every solve's points each step, loss read back
    host = [t.cpu().pin_memory() for t in bm.plan.arrays]
    t0 = time.perf_counter()
    e2e_steps = max(3, min(args.steps, 10))
    for _ in range(e2e_steps):
        for h, d_ in zip(host, bm.plan.arrays):
            d_.copy_(h, non_blocking=True)
        bm.evaluate(with_grad=True)
        _lib.check(lib.tdg_adam_step(bm.flat.data_ptr(), bm.grad.data_ptr(), m.data_ptr(),
                                     v.data_ptr(), st.data_ptr(), bm.flat.numel(), hp,
                                     stream.cuda_stream), 'adam')
        bm.loss.cpu()
    e2e_sec = (time.perf_counter() - t0) / e2e_steps
    flops = bm.plan.info.flops_hidden
    peaks_path = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    peaks = json.load(open(peaks_path)) if os.path.exists(peaks_path) else {}
    peak = peaks.get('bf16_tflops', 1900.0) / 2.0
    achieved = flops / (ms / 1e3) / 1e12
    seq = {}
    if not args.no_compare:
        k = max(1, min(args.steps, 5))
        seq = {'sequential_plain_ms_per_step': round(sequential_sweep_ms(args, 'plain', 'fp32', k), 3),
               'sequential_fused_ms_per_step': round(sequential_sweep_ms(args, 'fused', args.precision, k), 3)}
        seq['batched_vs_sequential_plain'] = round(seq['sequential_plain_ms_per_step'] / ms, 2)
        seq['batched_vs_sequential_fused'] = round(seq['sequential_fused_ms_per_step'] / ms, 2)
    return {'metric': METRIC, 'value': round(world * n_pts / (ms / 1e3), 1), 'unit': UNIT,
            'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': round(ms, 4), 'steps_per_s': round(1e3 / ms, 3), **seq,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
            'data': 'synthetic (seeded coefficients, grids and networks)',
            'config': {'workload': WORKLOADS['sweep'][3], 'solves': n_solves,
                       'collocation_points': n_pts, 'precision': args.precision,
                       'form': 'fused, one launch for all solves', 'optimizer': 'Adam lr=1e-3',
                       'schedule': bm.plan.schedule or 'default',
                       'autotune': None if bm.tuning is None else {
                           'default_launch_ms': bm.tuning['default_ms'],
                           'chosen_launch_ms': bm.tuning['ms'],
                           'trials': [(t['schedule'], t['ms']) for t in bm.tuning['trials']]},
                       'l2': 'flushed between timed steps (256 MiB write)',
                       'parallelism': f'replicas x{world}'},
            'e2e': {'value': round(world * n_pts / e2e_sec, 1), 'unit': UNIT,
                    'h2d_bytes_per_step': sum(h.numel() * 4 for h in host),
                    'd2h_bytes_per_step': bm.loss.numel() * 8},
            'roofline': {'bound': 'tensor', 'achieved': round(achieved, 3), 'peak': round(peak, 1),
                         'unit': 'TFLOP/s', 'frac': round(achieved / peak, 5), 'traffic': None,
                         'kernel': 'fused loss+gradient (all solves) + Adam',
                         'algorithmic_flops_per_launch': flops},
            'gpu_launches': int(launches), 'clocks': clk.summary(), 'impl': 'ours'}


def build_model(args, form, precision):
    """The workload as a Model of this package, compiled; its Solution, plan and optimizer."""
    import torch_de_solver_gb300 as T
    domain, bnd, eq, net, ckw = builder_for(args.workload, full_kwargs(args))(T)
    ckw = dict(ckw)
    model = T.Model(net, domain, eq, bnd)
    model.compile(ckw.pop('mode'), precision=precision, form=form, **ckw)
    opt = T.Optimizer('Adam', {'lr': 1e-3}).optimizer_choice(model.mode, model.net)
    return model, model.solution_cls, opt


def time_device_steps(sol, opt, warmup, steps, dev, world, flush):
    """`warmup` untimed steps, then `steps` timed ones (loss+gradient launch, then Adam), L2
    flushed before each, CUDA events on the launching stream, clocks sampled meanwhile.
    Returns (ms per step (max over ranks), mean ms of the loss+gradient part, launches, clocks)."""
    import torch
    from torch_de_solver_gb300 import _lib
    plan = sol.plan
    stream = torch.cuda.current_stream(dev)

    def device_step():
        plan.loss_grad(sol.flat, sol._grad, sol._loss_buf, sol._outputs)

    for _ in range(warmup):
        device_step()
        opt.apply(sol._grad)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    launches0 = _lib.launch_count()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev.index) as clk:
        for e0, e1, e2 in ev:
            flush.zero_()                      # evict L2 between timed iterations
            e0.record(stream)
            device_step()
            e1.record(stream)
            opt.apply(sol._grad)
            e2.record(stream)
        torch.cuda.synchronize()
    launches = _lib.launch_count() - launches0
    step_ms = [a.elapsed_time(c) for a, _, c in ev]
    kern_ms = [a.elapsed_time(b) for a, b, _ in ev]
    total_ms = max_over_ranks(sum(step_ms), dev)
    return total_ms / steps, statistics.mean(kern_ms), launches, clk.summary()


def run_ours(args, rank, world):
    import torch
    dev = torch.device('cuda', int(os.environ.get('LOCAL_RANK', 0)))
    torch.cuda.set_device(dev)
    model, sol, opt = build_model(args, args.form, args.precision)
    plan = sol.plan
    n_pts = sol.ir.n_residual_rows
    flush = torch.empty(2 * L2_BYTES // 4, device=dev)

    # ---- device-resident throughput
    ms_per_step, kern_mean, launches, clocks = time_device_steps(sol, opt, args.warmup, args.steps,
                                                                 dev, world, flush)
    value = world * n_pts / (ms_per_step / 1e3)

    # ---- end to end through the public API with host buffers
    pts_index = sol.ir.groups[sol.ir.residual_group].sites[0].points
    dev_pts = plan.arrays[pts_index]
    host_pts = dev_pts.cpu().pin_memory()
    for _ in range(2):
        dev_pts.copy_(host_pts, non_blocking=True)
        opt.zero_grad()
        loss, _ = sol.evaluate()
        loss.backward()
        opt.step()
        loss.item()
    torch.cuda.synchronize()
    e2e_steps = max(3, min(args.steps, 10))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        dev_pts.copy_(host_pts, non_blocking=True)
        opt.zero_grad()
        loss, _ = sol.evaluate()
        loss.backward()
        opt.step()
        loss.item()
    e2e_sec = (time.perf_counter() - t0) / e2e_steps
    e2e = {'value': world * n_pts / e2e_sec, 'unit': UNIT,
           'h2d_bytes_per_step': host_pts.numel() * 4, 'd2h_bytes_per_step': 4}

    peaks_path = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    peaks = json.load(open(peaks_path)) if os.path.exists(peaks_path) else {}
    bf16 = peaks.get('bf16_tflops', 1900.0)
    flops = plan.info.flops_hidden
    achieved = flops / (kern_mean / 1e3) / 1e12
    # dense TF32 tensor rate = half the measured dense BF16 rate
    peak = bf16 if args.precision == 'bf16' else bf16 / 2.0
    tag = f'{args.form}_{args.precision}_{args.workload}'
    tpp = read_traffic(tag)
    roofline = {'bound': 'tensor', 'achieved': round(achieved, 3), 'peak': round(peak, 1),
                'unit': 'TFLOP/s', 'frac': round(achieved / peak, 5),
                'traffic': None if tpp is None else int(tpp * n_pts),
                'kernel': ('tdg::fused_fp32_kernel' if args.precision == 'fp32' else
                           'tdg::fused_tc_kernel (tcgen05)') + ' + reductions'
                if args.form == 'fused' else 'plain form: all per-layer launches of the step',
                'kernel_ms': round(kern_mean, 4),
                'algorithmic_flops_per_launch': flops,
                'peak_source': ('MEASURED_PEAKS.json bf16_tflops' if peaks else 'fallback 1.9 PFLOP/s bf16')
                + ('' if args.precision == 'bf16' else ' / 2 (dense TF32 = half of BF16)')}
    line = {'metric': METRIC, 'value': round(value, 1), 'unit': UNIT, 'n_gpus': world,
            'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': round(ms_per_step, 4),
            'steps_per_s': round(1e3 / ms_per_step, 3), 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
            'data': 'synthetic (seeded grid, closed-form boundary data, seeded torch init)',
            'config': {'workload': WORKLOADS[args.workload][3], 'collocation_points': n_pts,
                       'params': plan.n_params, 'precision': args.precision, 'form': args.form,
                       'optimizer': 'Adam lr=1e-3',
                       'l2': 'flushed between timed steps (256 MiB write)',
                       'parallelism': f'replicas x{world}'},
            'e2e': e2e, 'roofline': roofline, 'gpu_launches': int(launches),
            'clocks': clocks, 'impl': 'ours'}
    del model, sol, opt, plan
    torch.cuda.empty_cache()

    if args.form == 'fused' and not args.no_compare:
        # the plain form (one launch per layer operation, FP32) on the same workload, steps and
        # warm-up: the fused-vs-plain ratio of the metric
        pmodel, psol, popt = build_model(args, 'plain', 'fp32')
        p_ms, _, p_launches, p_clocks = time_device_steps(psol, popt, args.warmup, args.steps,
                                                          dev, world, flush)
        line['plain_ms_per_step'] = round(p_ms, 4)
        line['plain_value'] = round(world * n_pts / (p_ms / 1e3), 1)
        line['plain_gpu_launches'] = int(p_launches)
        line['fused_vs_plain'] = round(p_ms / ms_per_step, 3)
        del pmodel, psol, popt
        torch.cuda.empty_cache()
        if rank == 0:
            torch.cuda.reset_peak_memory_stats()
            line['aten_reference'] = aten_reference(args)
    return line


def run_lbfgs(args, world):
    """L-BFGS on the workload through the public API (LBFGS64: device-resident history, FP64
    two-loop dots, strong-Wolfe line search) after `warmup` iterations: the throughput of the
    loss+gradient launches it drives (closures/s, points/s) and its iterations/s. Host
    synchronisation happens only for the line search's tests, as in torch.optim.LBFGS."""
    import torch
    import torch_de_solver_gb300 as T
    from torch_de_solver_gb300 import _lib
    dev = torch.device('cuda', int(os.environ.get('LOCAL_RANK', 0)))
    torch.cuda.set_device(dev)
    model, sol, _ = build_model(args, args.form, args.precision)
    n_pts = sol.ir.n_residual_rows
    counter = [0]

    def make(max_iter):
        opt = T.LBFGS64(model.net.parameters(), lr=1.0, max_iter=max_iter, history_size=100,
                        line_search_fn='strong_wolfe', tolerance_grad=0.0, tolerance_change=0.0)

        def closure():
            counter[0] += 1
            opt.zero_grad()
            loss, _ = sol.evaluate()
            loss.backward()
            return loss
        return opt, closure
    opt, closure = make(args.warmup)
    opt.step(closure)
    torch.cuda.synchronize()
    opt, closure = make(args.steps)
    counter[0] = 0
    l0 = _lib.launch_count()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev.index) as clk:
        t0 = time.perf_counter()
        opt.step(closure)
        torch.cuda.synchronize()
        sec = time.perf_counter() - t0
    sec = max_over_ranks(sec, dev)
    st = opt.state[opt.param_groups[0]['params'][0]]
    iters, closures = st['n_iter'], counter[0]
    loss = sol.evaluate(save_graph=False)[0].item()
    return {'metric': METRIC, 'value': round(world * n_pts * closures / sec, 1), 'unit': UNIT,
            'n_gpus': world, 'steps': iters, 'warmup': args.warmup,
            'ms_per_step': round(1e3 * sec / max(1, iters), 4),
            'steps_per_s': round(iters / sec, 3), 'closures_per_s': round(closures / sec, 3),
            'ms_per_closure': round(1e3 * sec / max(1, closures), 4),
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
            'data': 'synthetic (seeded grid, closed-form boundary data, seeded torch init)',
            'config': {'workload': WORKLOADS[args.workload][3], 'collocation_points': n_pts,
                       'precision': args.precision, 'form': args.form,
                       'optimizer': 'L-BFGS (LBFGS64: lr 1, history 100, strong Wolfe; '
                                    'device history, FP64 dots)',
                       'iterations': iters, 'closures': closures, 'final_loss': loss,
                       'l2': 'not flushed (inputs and weights stay resident between closures)',
                       'parallelism': f'replicas x{world}'},
            'gpu_launches': int(_lib.launch_count() - l0), 'clocks': clk.summary(),
            'impl': 'ours'}


def reference_arm(args):
    """--impl reference: the reference's CPU path (the oracle port) on all host cores, each step a
    bounded sample of the workload, honouring --steps and --warmup."""
    base = cpu_baseline(args, args.warmup, args.steps)
    return {'metric': METRIC, 'value': round(base['value'], 2), 'unit': UNIT,
            'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': round(1e3 / base['steps_per_s'], 3),
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
            'dtype': 'f32', 'data': 'synthetic',
            'config': {'workload': WORKLOADS[args.workload][3],
                       'collocation_points': base['points'],
                       'full_workload_points': full_points(args),
                       'rate': base['scaling']},
            'impl': 'reference',
            'cpu_baseline': {k: base[k] for k in ('value', 'unit', 'cores', 'kind', 'sample')},
            'e2e': {'value': round(base['value'], 2), 'unit': UNIT,
                    'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}


def main():
    args = parse()
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    if args.impl == 'reference':
        if rank == 0:
            print(json.dumps(reference_arm(args)))
        return
    import torch
    if world > 1:
        torch.distributed.init_process_group('nccl')
    if args.workload == 'sweep':
        line = run_sweep(args, world)
    elif args.optimizer == 'lbfgs':
        line = run_lbfgs(args, world)
    else:
        line = run_ours(args, rank, world)
    if rank == 0:
        if not args.no_cpu_baseline:
            line['cpu_baseline'] = {k: v for k, v in cpu_baseline(args, 1, 3).items()
                                    if k in ('value', 'unit', 'cores', 'kind', 'sample')}
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == '__main__':
    main()

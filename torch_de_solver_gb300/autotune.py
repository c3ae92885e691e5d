"""Tile-schedule autotuner for the fused loss+gradient kernels.

A plan cuts every group's (stream, point) rows into tiles and spreads the tiles over persistent
CTAs (tdg_schedule in include/tdg.h): how many rows a tile holds (max_rows), how many CTAs run
(n_ctas) and whether CTAs get equal tile counts or equal estimated work (balance). The best choice
depends on the problem set (grid sizes, stream counts, the number of solves of a batched sweep)
and on the GPU, so tune() builds a plan per candidate schedule on the real problem set, times the
loss+gradient launch with CUDA events on the device, and keeps the fastest. Results are cached in
a JSON file (TDG_AUTOTUNE_CACHE, default ~/.cache/torch_de_solver_gb300/autotune.json) keyed by
the problem shape and the device, so a shape is tuned once per machine.

The reference has no counterpart: it evaluates each solve's points as one batch on one device.
"""

import hashlib
import json
import os

import torch

CANDIDATES = (
    dict(max_rows=128, n_ctas=0, balance=0),   # the default schedule
    dict(max_rows=128, n_ctas=0, balance=1),
    dict(max_rows=96, n_ctas=0, balance=0),
    dict(max_rows=96, n_ctas=0, balance=1),
    dict(max_rows=64, n_ctas=0, balance=0),
    dict(max_rows=64, n_ctas=0, balance=1),
)


def cache_path():
    p = os.environ.get('TDG_AUTOTUNE_CACHE')
    if p:
        return p
    return os.path.join(os.path.expanduser('~'), '.cache', 'torch_de_solver_gb300', 'autotune.json')


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save(path, cache):
    os.makedirs(os.path.dirname(path) or '.', exist_ok=True)
    tmp = path + '.tmp'
    with open(tmp, 'w') as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def signature(irs, widths, precision, form, device):
    """Key of a tuning result: the MLP widths, precision and form, every group's (sites, streams
    per site, rows) and the device's name and SM count."""
    props = torch.cuda.get_device_properties(device)
    groups = [[len(g.sites), [len(s.streams) for s in g.sites], int(g.n_rows)]
              for ir in irs for g in ir.groups]
    blob = json.dumps([list(widths), precision, form, groups, props.name,
                       props.multi_processor_count])
    return hashlib.sha1(blob.encode()).hexdigest()[:20]


def n_params(widths, n_coeff):
    return sum(widths[i] * widths[i + 1] + widths[i + 1] for i in range(len(widths) - 1)) + n_coeff


def time_schedule(irs, widths, device, precision, form, schedule, reps=5, warmup=2):
    """Mean ms of one loss+gradient launch of a plan built with `schedule` (CUDA events)."""
    from .solution import DevicePlan
    plan = DevicePlan(irs, widths, device, precision, form, schedule=schedule)
    gen = torch.Generator(device=device).manual_seed(0)
    params = 0.1 * torch.randn(plan.n_problems * plan.n_params, device=device, generator=gen)
    grad = torch.zeros_like(params)
    loss = torch.zeros(2 * plan.n_problems, dtype=torch.float64, device=device)
    for _ in range(warmup):
        plan.loss_grad(params, grad, loss)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        plan.loss_grad(params, grad, loss)
    b.record()
    torch.cuda.synchronize(device)
    ms = a.elapsed_time(b) / reps
    info = dict(n_tiles=int(plan.info.n_tiles), n_ctas=int(plan.info.n_ctas))
    del plan
    return ms, info


def tune(irs, widths, device, precision, form='fused', candidates=CANDIDATES, reps=5,
         use_cache=True):
    """The fastest schedule for this problem set on `device` as a dict (max_rows, n_ctas,
    balance), and the record of the search: every candidate's mean launch time."""
    key = signature(irs, widths, precision, form, device)
    path = cache_path()
    cache = _load(path) if use_cache else {}
    if key in cache:
        return dict(cache[key]['schedule']), cache[key]
    trials = []
    for cand in candidates:
        ms, info = time_schedule(irs, widths, device, precision, form, cand, reps=reps)
        trials.append(dict(schedule=dict(cand), ms=round(ms, 5), **info))
    best = min(trials, key=lambda t: t['ms'])
    record = dict(schedule=best['schedule'], ms=best['ms'], default_ms=trials[0]['ms'],
                  trials=trials, device=torch.cuda.get_device_name(device))
    if use_cache:
        cache = _load(path)
        cache[key] = record
        _save(path, cache)
    return dict(best['schedule']), record

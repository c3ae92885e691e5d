"""Failure detection without a GPU fault: bounded device waits give up with TDG_ERR_TIMEOUT and
leave the context usable; invalid descriptions and unsupported features come back as status codes
or Python exceptions before any launch."""
import ctypes

import pytest
import torch

import cases
from helpers import build_model, golden, rel


@pytest.mark.gpu
def test_bounded_wait_times_out_and_context_survives():
    from torch_de_solver_gb300 import _lib
    lib = _lib.load()
    assert lib.tdg_selftest_bounded_wait(1000) == _lib.ERR_TIMEOUT
    assert b'gave up' in lib.tdg_last_error()
    # the context still computes
    import torch_de_solver_gb300 as T
    g = golden('burgers_ag')
    model = build_model(T, 'burgers_ag', weights=g['weights'], precision='3xtf32')
    loss, _ = model.solution_cls.evaluate()
    _lib.check(lib.tdg_plan_sync_status(model.solution_cls.plan.handle), 'sync')
    assert rel(loss.item(), g['loss64']) < 1e-5


@pytest.mark.gpu
def test_invalid_descriptions_fail_before_launch():
    import torch_de_solver_gb300 as T
    from torch_de_solver_gb300 import _lib
    d, b, e, net, kw = cases.burgers_ag(T, n=8, widths=(2, 30, 30, 1))   # width not a multiple of 4
    m = T.Model(net, d, e, b)
    with pytest.raises(NotImplementedError):   # the fused form asked for: the plan refuses it
        m.compile('autograd', lambda_operator=1, lambda_bound=1, form='fused')
    d, b, e, net, kw = cases.burgers_ag(T, n=8)
    m = T.Model(net, d, e, b)
    with pytest.raises(NotImplementedError):
        m.compile('autograd', lambda_operator=1, lambda_bound=1, precision='3xtf32', form='plain')


@pytest.mark.gpu
def test_nan_weights_propagate_not_crash():
    import torch_de_solver_gb300 as T
    g = golden('burgers_ag')
    w = g['weights'].copy()
    w[5] = float('nan')
    model = build_model(T, 'burgers_ag', weights=w)
    loss, _ = model.solution_cls.evaluate()
    assert torch.isnan(loss).all()

"""Tensor-core (tcgen05) precisions: TF32, split TF32 (3xTF32) and BF16 hidden GEMMs with FP32
accumulation.

Each variant's loss and gradient are compared with the reference's FP64 fixtures; the measured
relative errors are printed. Bounds: 3xTF32 1e-5 (the FP32 tolerance), TF32 1e-2 (10-bit mantissa
operands), BF16 1e-1 (7-bit), the stated limits these precisions are measured against."""
import numpy as np
import pytest
import torch

import cases
from helpers import build_model, golden, rel

BOUND = {'3xtf32': 1e-5, 'tf32': 1e-2, 'bf16': 1e-1}


@pytest.mark.gpu
@pytest.mark.parametrize('precision', ['3xtf32', 'tf32', 'bf16'])
@pytest.mark.parametrize('name', list(cases.GOLDEN_CASES))
def test_tensor_core_precision_against_reference(name, precision):
    import torch_de_solver_gb300 as T
    from torch_de_solver_gb300 import _lib
    g = golden(name)
    model = build_model(T, name, weights=g['weights'], precision=precision)
    sol = model.solution_cls
    loss, lossn = sol.evaluate()
    loss.backward()
    _lib.check(_lib.load().tdg_plan_sync_status(sol.plan.handle), 'tdg_plan_sync_status')
    grad = torch.cat([p.grad.reshape(-1) for p in model.net.parameters()]).cpu().numpy()
    rl, rg = rel(loss.item(), g['loss64']), rel(grad, g['grad64'])
    print(f'{name} {precision}: loss rel {rl:.3e} grad rel {rg:.3e}')
    assert np.isfinite(grad).all()
    assert rl < BOUND[precision] and rg < BOUND[precision], (rl, rg)


@pytest.mark.gpu
@pytest.mark.parametrize('precision', ['3xtf32', 'tf32', 'bf16'])
def test_tensor_core_forward_only_equals_fused(precision):
    import torch_de_solver_gb300 as T
    g = golden('kovasznay_ag')
    model = build_model(T, 'kovasznay_ag', weights=g['weights'], precision=precision)
    with torch.no_grad():
        l0, _ = model.solution_cls.evaluate()
    l1, _ = model.solution_cls.evaluate()
    assert abs(l0.item() - l1.item()) <= 1e-6 * abs(l1.item())


def _loss_grad(T, name, g, precision):
    model = build_model(T, name, weights=g['weights'], precision=precision)
    loss, _ = model.solution_cls.evaluate()
    loss.backward()
    grad = torch.cat([p.grad.reshape(-1) for p in model.net.parameters()]).cpu().numpy()
    return loss.item(), grad


@pytest.mark.gpu
@pytest.mark.parametrize('precision', ['3xtf32', 'bf16'])
@pytest.mark.parametrize('name', ['kovasznay_ag', 'kdv_ag', 'burgers_ag', 'neumann_ag'])
def test_class_jets_equal_table_jets(name, precision, monkeypatch):
    """The compile-time jet code of classed site layouts and the table-driven jet code compute
    the same operations in the same order; the two agree to FP32 rounding (the compiler may
    contract a product and a sum differently in the two codes)."""
    import torch_de_solver_gb300 as T
    g = golden(name)
    l_cls, g_cls = _loss_grad(T, name, g, precision)
    monkeypatch.setenv('TDG_JET_TABLES', '1')
    l_tab, g_tab = _loss_grad(T, name, g, precision)
    print(f'{name} {precision}: loss rel {rel(l_cls, l_tab):.3e} grad rel {rel(g_cls, g_tab):.3e} '
          f'exact {l_cls == l_tab and np.array_equal(g_cls, g_tab)}')
    assert rel(l_cls, l_tab) < 1e-6 and rel(g_cls, g_tab) < 1e-6

"""Host logic of the product: stencils, point typing and lowering (no GPU needed)."""
import numpy as np
import pytest
import torch

import cases
from oracle import oracle as O


def test_product_stencils_equal_oracle():
    from torch_de_solver_gb300.prepare import fd_scheme
    for term in ([0], [1], [0, 0], [0, 1], [0, 0, 0], [1, 1]):
        for ptype, label in (('central', '1'), ('fb', '2'), ('bf', '2'), ('ff', '1'), ('bb', '1')):
            a = fd_scheme(term, 2, ptype, label, 0.05)
            b = O.stencil(term, 2, ptype, label, 0.05)
            assert a[0] == b[0]
            assert np.allclose(a[1], b[1])


def test_point_typing_box_rule_equals_delaunay():
    from torch_de_solver_gb300.prepare import point_types
    grid = torch.cartesian_prod(torch.linspace(0, 1, 21), torch.linspace(0, 1, 21))
    assert point_types(grid) == O.point_types(grid)
    counts = {t: point_types(grid).count(t) for t in set(point_types(grid))}
    assert counts == {'central': 361, 'ff': 39, 'bf': 20, 'fb': 20, 'bb': 1}


@pytest.mark.parametrize('name', list(cases.GOLDEN_CASES))
def test_lowering_shapes(name):
    import torch_de_solver_gb300 as T
    from torch_de_solver_gb300.prepare import lower
    d, bc, eq, net, kw = cases.GOLDEN_CASES[name](T)
    kw = dict(kw)
    mode = kw.pop('mode')
    ir = lower(d.build(mode), eq.equation_lst, bc.build(d.variable_dict), mode,
               kw['lambda_operator'], kw['lambda_bound'], kw.get('h', 0.001),
               d_out=net[-1].out_features)
    res = ir.groups[ir.residual_group]
    g = np.load(f'tests/golden/{name}.npz')
    assert res.n_rows == int(g['n_op'])
    assert [ir.max_len] == [int(max(g['bval_length']))]
    assert ir.bc_types == [str(k) for k in g['bval_keys']]
    for grp in ir.groups:
        total = sum(len(s.streams) for s in grp.sites)
        assert total <= 16


def test_unsupported_features_raise():
    import torch_de_solver_gb300 as T
    from torch_de_solver_gb300.prepare import lower
    d, bc, eq, net, kw = cases.burgers_ag(T, n=8)
    eq.equation_lst[0]['-mu*d2u/dx2']['pow'] = lambda x: x
    with pytest.raises(NotImplementedError):
        lower(d.build('autograd'), eq.equation_lst, bc.build(d.variable_dict), 'autograd', 1, 1)
    with pytest.raises(NotImplementedError):
        d.build('mat')

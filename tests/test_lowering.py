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


# the compile-time jet class the residual sites of each benchmark layout run (-1: tables)
EXPECTED_CLASSES = {'kovasznay_ag': 7, 'burgers_ag': 5, 'kdv_ag': 8, 'heat_nn': 0}


@pytest.mark.parametrize('name', list(EXPECTED_CLASSES))
def test_site_classes(name):
    import torch_de_solver_gb300 as T
    from torch_de_solver_gb300 import _lib
    from torch_de_solver_gb300.prepare import lower
    builder = getattr(cases, name)
    small = {'kovasznay_ag': dict(n=8), 'burgers_ag': dict(n=8), 'kdv_ag': dict(nx=8, nt=4),
             'heat_nn': {}}[name]
    d, bc, eq, net, kw = builder(T, **small)
    kw = dict(kw)
    mode = kw.pop('mode')
    ir = lower(d.build(mode), eq.equation_lst, bc.build(d.variable_dict), mode,
               kw['lambda_operator'], kw['lambda_bound'], kw.get('h', 0.001),
               d_out=net[-1].out_features)
    res = ir.groups[ir.residual_group]
    for site in res.sites:
        assert _lib.site_class(site.streams) == EXPECTED_CLASSES[name], site.streams
    for grp in ir.groups:   # every layout classifies without error; boundary value sites are class 0
        for site in grp.sites:
            c = _lib.site_class(site.streams)
            assert c >= -1
            if [tuple(k) for k in site.streams] == [()]:
                assert c == 0


@pytest.mark.parametrize('name', list(cases.CLASS_CASES))
def test_class_coverage_cases_reach_their_class(name):
    import torch_de_solver_gb300 as T
    from torch_de_solver_gb300 import _lib
    from torch_de_solver_gb300.prepare import lower
    builder, want = cases.CLASS_CASES[name]
    d, bc, eq, net, kw = builder(T)
    kw = dict(kw)
    mode = kw.pop('mode')
    ir = lower(d.build(mode), eq.equation_lst, bc.build(d.variable_dict), mode,
               kw['lambda_operator'], kw['lambda_bound'], kw.get('h', 0.001),
               d_out=net[-1].out_features)
    for site in ir.groups[ir.residual_group].sites:
        assert _lib.site_class(site.streams) == want, site.streams


def test_site_class_rejects_unlisted_layouts():
    from torch_de_solver_gb300 import _lib
    assert _lib.site_class([(), (0,), (1,), (0, 1)]) == -1          # mixed derivative alone
    assert _lib.site_class([(), (0,), (1,), (2,)]) == -1            # three axes
    assert _lib.site_class([(), (1,), (0,)]) == -1                  # not in canonical order
    assert _lib.site_class([(), (0,), (1,), (0, 0), (0, 1), (1, 1)]) == 10
    assert _lib.site_class([(), (0,), (0, 0)]) == 4


def test_unsupported_features_raise():
    import torch_de_solver_gb300 as T
    from torch_de_solver_gb300.prepare import lower
    d, bc, eq, net, kw = cases.burgers_ag(T, n=8)
    eq.equation_lst[0]['-mu*d2u/dx2']['pow'] = lambda x: x
    with pytest.raises(NotImplementedError):
        lower(d.build('autograd'), eq.equation_lst, bc.build(d.variable_dict), 'autograd', 1, 1)
    with pytest.raises(NotImplementedError):
        d.build('mat')

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
               d_out=net[-1].out_features, tol=kw.get('tol', 0))
    res = ir.groups[ir.residual_group]
    g = np.load(f'tests/golden/{name}.npz')
    # mini-batch cases keep the first batch's residual in the fixture
    assert min(res.n_rows, kw.get('batch_size', res.n_rows)) == int(g['n_op'])
    assert (ir.causal is not None) == bool(kw.get('tol', 0))
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


def _lower_case(T, builder, **kw_case):
    from torch_de_solver_gb300.prepare import lower
    d, bc, eq, net, kw = builder(T, **kw_case)
    mode = kw['mode']
    ir = lower(d.build(mode), eq.equation_lst, bc.build(d.variable_dict), mode,
               kw['lambda_operator'], kw['lambda_bound'], kw.get('h', 0.001), d_out=1)
    return ir, net


@pytest.mark.parametrize('mode', ['autograd', 'NN'])
def test_trainable_coefficients_lower_to_parameter_slots(mode):
    """nn.Parameter coefficients keep their identity through the lowering's copy and become
    coefficient slots in first-use order; every other coefficient stays a constant."""
    import torch_de_solver_gb300 as T
    from torch_de_solver_gb300.prepare import CoeffParam
    ir, net = _lower_case(T, cases.inverse_burgers_ag, n=8, mode=mode)
    assert [id(p) for p in ir.coeff_params] == [id(net.lam1), id(net.lam2)]
    res = ir.groups[ir.residual_group]
    marks = [(c.index, c.scale) for c, _, _ in res.terms if isinstance(c, CoeffParam)]
    assert sorted(set(i for i, _ in marks)) == [0, 1]
    assert all(s == 1.0 for _, s in marks)
    for grp in ir.groups:
        if grp is not res:
            assert not any(isinstance(c, CoeffParam) for c, _, _ in grp.terms)


def test_trainable_coefficient_in_boundary_operator_raises():
    import torch_de_solver_gb300 as T
    from torch_de_solver_gb300.prepare import lower
    d, bc, eq, net, kw = cases.neumann_ag(T, n=8)
    cases.register_coefficients(net, {'k': 1.5})
    bc.conditions_lst[1]['bop']['du/dx']['coeff'] = net.k
    with pytest.raises(NotImplementedError, match='boundary operators'):
        lower(d.build('autograd'), eq.equation_lst, bc.build(d.variable_dict), 'autograd', 1, 1)


def test_device_parameter_order_and_optimizer_order():
    """The device buffer holds the Linear layers first, then the coefficients, while
    Module.parameters() lists the registered coefficients first; the optimizer gets the buffer's
    order, and a parameter that is neither is refused."""
    import torch_de_solver_gb300 as T
    from torch_de_solver_gb300.optimizer import _in_buffer_order
    from torch_de_solver_gb300.solution import device_parameters, flatten_parameters
    ir, net = _lower_case(T, cases.inverse_burgers_ag, n=8)
    names = [n for n, _ in net.named_parameters()]
    assert names[:2] == ['lam1', 'lam2']
    params = device_parameters(net, ir.coeff_params)
    assert params[-2] is net.lam1 and params[-1] is net.lam2 and params[0] is net[0].weight
    flat = flatten_parameters(params, torch.device('cpu'))
    assert flat.numel() == sum(p.numel() for p in net.parameters())
    assert float(flat[-2]) == 2.0 and abs(float(flat[-1]) - 0.2) < 1e-7
    assert [id(p) for p in _in_buffer_order(net.parameters())] == [id(p) for p in params]
    net.register_parameter('stray', torch.nn.Parameter(torch.zeros(3)))
    with pytest.raises(NotImplementedError):
        device_parameters(net, ir.coeff_params)


def test_parameter_registr():
    """parameter_registr registers one-element float32 parameters and puts them in the dict."""
    import torch_de_solver_gb300 as T
    net = cases.mlp([2, 8, 1], 0)
    params = {'lam1': 2.0, 'lam2': 0.2}
    T.parameter_registr(net, params)
    assert params['lam1'] is net.lam1 and params['lam2'] is net.lam2
    assert net.lam1.dtype == torch.float32 and net.lam1.shape == (1,) and net.lam1.requires_grad


def test_causal_time_slices_and_slots():
    """The causal loss counts the distinct first coordinates of the residual points as time
    slices (every point its own slice when they do not split evenly) and weighs each residual
    row 1/N, lambda_operator not applied."""
    import torch_de_solver_gb300 as T
    from torch_de_solver_gb300.prepare import lower, residual_time_slices
    g = torch.cartesian_prod(torch.linspace(0, 1, 5), torch.linspace(0, 1, 7))
    assert residual_time_slices(g) == 5
    assert residual_time_slices(g[:-1]) == 34
    d, bc, eq, net, kw = cases.allen_cahn_ag(T, n=6)
    ir = lower(d.build('autograd'), eq.equation_lst, bc.build(d.variable_dict), 'autograd',
               3.0, 100, tol=kw['tol'])
    res = ir.groups[ir.residual_group]
    assert ir.causal == (10.0, 7)
    assert ir.slots[res.slot_first][1:] == (1.0 / 49, 1.0 / 49)
    assert res.row_weight is not None and ir.arrays[res.row_weight].numel() == 49


def test_minibatch_order_equals_reference_loader():
    """The product's batches (indices into the grid) select the same points, in the same order and
    over several passes, as the reference's DataLoader over the points (restated by the oracle)."""
    from torch_de_solver_gb300.solution import _Batches
    prob, _ = O.build_problem(cases.GOLDEN_CASES['allen_cahn_batch_ag'], 'float32')
    b = _Batches(prob.grid.shape[0], 64)
    assert b.n_batches == prob.n_batches == 7
    for _ in range(2 * b.n_batches + 3):
        want = prob._batch
        idx = b.take()
        try:
            prob._batch = next(prob._batches)
        except StopIteration:
            prob._batches = iter(prob.loader)
            prob._batch = next(prob._batches)
        assert torch.equal(prob.grid[idx], want)


def test_model_save_uses_the_reference_cache_file_names(tmp_path):
    """Model._model_save writes cache_dir + '\\' + name + '.tar' with a CPU copy of the network,
    the name the reference's cache lookup pattern cache_dir + '\\*.tar' finds."""
    import glob
    import torch_de_solver_gb300 as T
    m = T.Model(cases.mlp([2, 8, 1], 0), None, None, None)
    m._save_dir = str(tmp_path) + '/'
    m._model_save(True, 'abc')
    files = glob.glob(m._save_dir + '\\*.tar')
    assert files == [m._save_dir + '\\abc.tar']
    ck = torch.load(files[0], weights_only=False)
    assert set(ck) == {'model', 'model_state_dict'}
    assert torch.equal(ck['model'][0].weight, m.net[0].weight)


def test_shard_ir_splits_residual_rows():
    """Point sharding of a lowered problem: contiguous residual row ranges per rank (points and
    per-row coefficients sliced together), loss-slot weights of the whole problem on every rank,
    boundary groups on rank 0 only."""
    import torch_de_solver_gb300 as T
    from torch_de_solver_gb300.prepare import lower, shard_ir, shard_rows
    d, bc, eq, net, kw = cases.burgers_ag(T, n=10)
    eq.equation_lst[0]['-mu*d2u/dx2']['coeff'] = lambda g: 0.01 + g[:, 0] ** 2   # per-row array
    grid = d.build('autograd')
    bconds = bc.build(d.variable_dict)
    ir = lower(grid, eq.equation_lst, bconds, 'autograd', 1, 1, d_out=1)
    res = ir.groups[ir.residual_group]
    world = 3
    parts = [shard_ir(ir, r, world) for r in range(world)]
    assert [shard_rows(res.n_rows, r, world) for r in range(world)] == [(0, 40), (40, 80), (80, 121)]
    for key in [res.sites[0].points] + [c for c, _, _ in res.terms if isinstance(c, int)]:
        whole = torch.cat([p.arrays[key] for p in parts])
        assert torch.equal(whole, ir.arrays[key].reshape(-1))
    for r, p in enumerate(parts):
        assert p.slots == ir.slots
        assert p.groups[p.residual_group].n_rows == shard_rows(res.n_rows, r, world)[1] - \
            shard_rows(res.n_rows, r, world)[0]
        assert len(p.groups) == (len(ir.groups) if r == 0 else 1)
    assert ir.groups[ir.residual_group].n_rows == res.n_rows == 121   # the original is untouched
    with pytest.raises(ValueError):
        shard_rows(10, 3, 3)


def test_form_choice_by_hidden_width():
    """form=None: the fused form for hidden widths that are multiples of 4 up to 128, otherwise the
    plain form (FP32, any width) with a warning; a tensor-core precision with such a network raises,
    and an explicit form is kept as given (the plan then names its own limit)."""
    import warnings
    from torch_de_solver_gb300.solution import default_form, fused_width_ok
    assert fused_width_ok([2, 128, 128, 3]) and fused_width_ok([2, 4, 1])
    assert not fused_width_ok([2, 50, 50, 1]) and not fused_width_ok([2, 256, 1])
    with warnings.catch_warnings():
        warnings.simplefilter('error')
        assert default_form([2, 100, 100, 1], None, None) == 'fused'
        assert default_form([2, 100, 100, 1], 'bf16', None) == 'fused'
        assert default_form([2, 150, 1], None, 'fused') == 'fused'
    for precision in (None, 'fp32'):
        with pytest.warns(UserWarning, match='plain form'):
            assert default_form([2, 150, 150, 1], precision, None) == 'plain'
    for precision in ('3xtf32', 'tf32', 'bf16'):
        with pytest.raises(NotImplementedError, match='hidden widths'):
            default_form([2, 50, 1], precision, None)

"""Point-sharded problems on the device: the plans of every rank's share (its contiguous residual
rows, the boundary conditions on rank 0), built and evaluated in one process with no process
group (so no all-reduce runs), add up to the unsharded loss and gradient, which match the FP64
oracle. The all-reduce that joins the shares across processes is covered with gloo ranks on CPU
(tests/test_multirank.py); this run has one GPU."""
import numpy as np
import pytest
import torch

import cases
from helpers import rel
from oracle import oracle as O

BUILDERS = {
    'kovasznay_ag': lambda api, dtype='float32': cases.kovasznay_ag(api, n=47, dtype=dtype),
    'burgers_ag': lambda api, dtype='float32': cases.burgers_ag(api, n=40, dtype=dtype),
    'heat_nn': lambda api, dtype='float32': cases.heat_nn(api, n=20, dtype=dtype),
}


def _loss_grad(T, builder, precision, shard=None):
    domain, bnd, eq, net, kw = builder(T)
    kw = dict(kw)
    model = T.Model(net, domain, eq, bnd, shard=shard)
    model.compile(kw.pop('mode'), precision=precision, **kw)
    loss, lossn = model.solution_cls.evaluate()
    loss.backward()
    grad = torch.cat([p.grad.reshape(-1) for p in model.net.parameters()]).double().cpu().numpy()
    return loss.item(), lossn.item(), grad, model.solution_cls.ir.n_residual_rows


@pytest.mark.gpu
@pytest.mark.parametrize('world', [2, 3])
@pytest.mark.parametrize('precision', ['fp32', '3xtf32'])
@pytest.mark.parametrize('name', list(BUILDERS))
def test_shares_add_up_to_the_whole_problem(name, precision, world):
    import torch_de_solver_gb300 as T
    builder = BUILDERS[name]
    l_all, ln_all, g_all, n_all = _loss_grad(T, builder, precision)
    parts = [_loss_grad(T, builder, precision, shard=(r, world)) for r in range(world)]
    assert sum(p[3] for p in parts) == n_all
    l_sum = sum(p[0] for p in parts)
    ln_sum = sum(p[1] for p in parts)
    g_sum = np.sum([p[2] for p in parts], axis=0)
    prob, net = O.build_problem(builder, 'float64')
    l64, ln64, g64, _ = O.loss_and_grad(prob, net)
    print(f'{name} {precision} world {world}: loss rel {rel(l_sum, l64):.2e} grad rel '
          f'{rel(g_sum, g64.numpy()):.2e} (unsharded {rel(l_all, l64):.2e} / {rel(g_all, g64.numpy()):.2e})')
    assert rel(l_sum, l_all) < 1e-6 and rel(ln_sum, ln_all) < 1e-6 and rel(g_sum, g_all) < 1e-5
    assert rel(l_sum, l64) < 1e-5 and rel(ln_sum, ln64) < 1e-5 and rel(g_sum, g64.numpy()) < 1e-5


@pytest.mark.gpu
def test_single_rank_shard_trains_like_the_unsharded_model():
    """shard=(0, 1) is the whole problem: five Adam steps (eager, no graph capture) give the
    unsharded model's losses."""
    import torch_de_solver_gb300 as T
    curves = []
    for shard in (None, (0, 1)):
        domain, bnd, eq, net, kw = BUILDERS['burgers_ag'](T)
        kw = dict(kw)
        model = T.Model(net, domain, eq, bnd, shard=shard)
        model.compile(kw.pop('mode'), precision='fp32', **kw)
        seen = []

        class Rec(T.Callback):
            def on_epoch_end(self, logs=None):
                seen.append(float(self.model.cur_loss.reshape(-1)[0]))
        model.train(T.Optimizer('Adam', {'lr': 1e-3}), 6, callbacks=[Rec()])
        curves.append(seen)
    assert np.allclose(curves[0], curves[1], rtol=1e-6), curves

"""Generate golden fixtures by running the reference TEDEouS package itself on CPU.

Usage (needs the reference source tree, given as the first argument or in TEDEOUS_REFERENCE;
run from the repository root):
    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py <path to the reference> [case ...]

For each case in tests/cases.py GOLDEN_CASES this writes tests/golden/<case>.npz holding
  weights      the seeded initial parameters (fp32, flattened in net.parameters() order)
  loss32/64    loss from Solution.evaluate() of an fp32 and of an fp64 run of the same weights
  lossn32/64   loss_normalized of the same evaluate() call
  grad32/64    the flattened parameter gradient after loss.backward()
  op64         the first rows of the residual field (fp64) and op_sumsq64 = sum(op^2) per column
               (mini-batch cases: the residual of the first batch, which the reference keeps as
               save_op)
  bval64, true_bval64   boundary value matrices (fp64, padded per the reference)
  curve32      loss values seen by the closure over 5 Adam(lr=1e-3) steps of Model.train(6)
               (mini-batch cases: the last closure loss of each of the 5 epochs, n_batches steps each)
  final32      parameters after those 5 steps
With --trained it instead runs the reference's Model.train for the long benchmark runs (C1 heat
'NN' 2000 epochs, C2 Burgers 'autograd' 5000 epochs, Adam lr=1e-3) and writes
tests/golden/trained_<case>.npz: the seeded initial weights, the trained solution u on the grid,
the loss every 100 epochs and the final weights.
The reference needs one stub: SALib (imported by tedeous/callbacks/adaptive_lambda.py:4) is
absent, so an empty module is installed in sys.modules before the import.
"""

import os
import sys
import types

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def load_reference(path):
    stub = types.ModuleType('SALib')
    stub.ProblemSpec = object
    sys.modules['SALib'] = stub
    sys.path.insert(0, path)
    import tedeous.data as data
    import tedeous.model as model
    import tedeous.optimizers.optimizer as optimizer
    import tedeous.callbacks.callback as callback
    from tedeous.device import solver_device
    solver_device('cpu')
    api = types.SimpleNamespace(Domain=data.Domain, Conditions=data.Conditions,
                                Equation=data.Equation, Model=model.Model,
                                Optimizer=optimizer.Optimizer, Callback=callback.Callback)
    return api


def flat(tensors):
    return torch.cat([t.detach().reshape(-1).to(torch.float64) for t in tensors]).numpy()


def run_case(api, builder, dtype):
    domain, bnd, eq, net, kw = builder(api, dtype=dtype)
    w0 = flat(net.parameters()).astype(np.float32)
    # The reference's causal loss makes its normalised boundary weights in torch's default dtype
    # (tedeous/losses.py:176-181 through lambda_prepare), so its FP64 run needs float64 as the
    # default dtype while it compiles and evaluates (after the network is built, so that the
    # seeded initial weights stay the FP32 run's).
    old_default = torch.get_default_dtype()
    if dtype == 'float64' and kw.get('tol'):
        torch.set_default_dtype(torch.float64)
    try:
        m = api.Model(net, domain, eq, bnd, batch_size=kw.pop('batch_size', None))
        mode = kw.pop('mode')
        m.compile(mode, **kw)
        s = m.solution_cls
        loss, lossn = s.evaluate()
        loss.backward()
    finally:
        torch.set_default_dtype(old_default)
    grad = flat(p.grad for p in m.solution_cls.model.parameters())
    return dict(w0=w0, loss=float(loss.detach().reshape(-1)[0]),
                lossn=float(lossn.detach().reshape(-1)[0]), grad=grad,
                op=(s.op if hasattr(s, 'op') else s.save_op).detach().to(torch.float64).numpy(),
                bval=s.bval.detach().to(torch.float64).numpy(),
                true_bval=s.true_bval.detach().to(torch.float64).numpy(),
                bval_keys=list(s.bval_keys), bval_length=list(s.bval_length))


def run_curve(api, builder, steps=5):
    domain, bnd, eq, net, kw = builder(api, dtype='float32')
    m = api.Model(net, domain, eq, bnd, batch_size=kw.pop('batch_size', None))
    mode = kw.pop('mode')
    m.compile(mode, **kw)
    seen = []

    class Record(api.Callback):
        def on_epoch_end(self, logs=None):
            seen.append(float(self.model.cur_loss.detach().reshape(-1)[0]))

    m.train(api.Optimizer('Adam', {'lr': 1e-3}), steps + 1, callbacks=[Record()])
    return np.array(seen), flat(m.net.parameters()).astype(np.float32)


# long training runs of the reference (Model.train with Adam(lr=1e-3), no callbacks besides a
# loss recorder): the benchmark configs C1 (heat, 'NN', 2000 epochs) and C2 (Burgers, 'autograd',
# 5000 epochs), seeded; stored as trained_<case>.npz
TRAINED = {'heat_nn': 2000, 'burgers_ag': 5000}


def run_trained(api, builder, epochs, every=100):
    """Model.train(epochs) of the reference: its solution on the grid afterwards (the network
    evaluated at every grid node), the loss every `every` epochs and the final weights."""
    domain, bnd, eq, net, kw = builder(api, dtype='float32')
    w0 = flat(net.parameters()).astype(np.float32)
    m = api.Model(net, domain, eq, bnd)
    mode = kw.pop('mode')
    m.compile(mode, **kw)
    seen = []

    class Record(api.Callback):
        def on_epoch_end(self, logs=None):
            if self.model.t % every == 0:
                seen.append((self.model.t, float(self.model.cur_loss.detach().reshape(-1)[0])))

    m.train(api.Optimizer('Adam', {'lr': 1e-3}), epochs, callbacks=[Record()])
    grid = domain.build(mode)
    with torch.no_grad():
        u = m.net(grid).detach().to(torch.float64).numpy()
    return dict(weights=w0, epochs=epochs, grid=grid.numpy(), u=u,
                curve=np.array(seen), final=flat(m.net.parameters()).astype(np.float32))


def main_trained(ref_path, only):
    import cases
    api = load_reference(ref_path)
    torch.set_num_threads(min(8, os.cpu_count() or 1))
    for name in only or list(TRAINED):
        r = run_trained(api, cases.GOLDEN_CASES[name], TRAINED[name])
        np.savez_compressed(os.path.join(HERE, 'trained_' + name + '.npz'), **r)
        print(f'trained {name}: {TRAINED[name]} epochs, last losses {r["curve"][-3:].tolist()}')


def main(ref_path, only):
    import cases
    api = load_reference(ref_path)
    torch.set_num_threads(min(8, os.cpu_count() or 1))
    only = only or list(cases.GOLDEN_CASES)
    for name in only:
        builder = cases.GOLDEN_CASES[name]
        r32 = run_case(api, builder, 'float32')
        r64 = run_case(api, builder, 'float64')
        assert np.array_equal(r32['w0'], r64['w0'])
        curve, final = run_curve(api, builder)
        op = r64['op']
        out = dict(weights=r32['w0'],
                   loss32=r32['loss'], loss64=r64['loss'],
                   lossn32=r32['lossn'], lossn64=r64['lossn'],
                   grad32=r32['grad'].astype(np.float32), grad64=r64['grad'],
                   op64=op[:2048], op_sumsq64=(op ** 2).sum(0), n_op=op.shape[0],
                   bval64=r64['bval'], true_bval64=r64['true_bval'],
                   bval_keys=np.array(r64['bval_keys']), bval_length=np.array(r64['bval_length']),
                   curve32=curve, final32=final)
        np.savez_compressed(os.path.join(HERE, name + '.npz'), **out)
        rel_l = abs(r32['loss'] - r64['loss']) / abs(r64['loss'])
        rel_g = np.linalg.norm(r32['grad'] - r64['grad']) / np.linalg.norm(r64['grad'])
        print(f'{name}: loss64={r64["loss"]:.9g} rel32={rel_l:.2e} grad rel32={rel_g:.2e} '
              f'n_op={op.shape[0]} keys={r64["bval_keys"]} curve={curve}')


def _args():
    import argparse
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument('reference', nargs='?', default=os.environ.get('TEDEOUS_REFERENCE'),
                    help='root of the reference source tree (or set TEDEOUS_REFERENCE)')
    ap.add_argument('cases', nargs='*', help='cases to regenerate (default: all)')
    ap.add_argument('--trained', action='store_true',
                    help='run the long training goldens (trained_<case>.npz) instead')
    a = ap.parse_intermixed_args()
    if not a.reference:
        ap.error('the path of the reference source tree is required')
    return a


if __name__ == '__main__':
    a = _args()
    if a.trained:
        main_trained(a.reference, a.cases)
    else:
        main(a.reference, a.cases)

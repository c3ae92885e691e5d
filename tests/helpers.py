"""Shared helpers: build a case through this package with the golden weights."""
import os

import numpy as np
import torch

import cases

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def golden(name):
    return np.load(os.path.join(GOLDEN, name + '.npz'))


def set_flat_weights(net, w):
    torch.nn.utils.vector_to_parameters(torch.as_tensor(np.asarray(w), dtype=torch.float32),
                                        net.parameters())


def build_model(api, name=None, builder=None, weights=None, precision='fp32', form='fused',
                **case_kw):
    builder = builder or cases.GOLDEN_CASES[name]
    domain, bnd, eq, net, kw = builder(api, **case_kw) if case_kw else builder(api)
    if weights is not None:
        set_flat_weights(net, weights)
    kw = dict(kw)
    model = api.Model(net, domain, eq, bnd, batch_size=kw.pop('batch_size', None))
    mode = kw.pop('mode')
    model.compile(mode, precision=precision, form=form, **kw)
    return model


def rel(a, b):
    a = np.asarray(a, dtype=np.float64).reshape(-1)
    b = np.asarray(b, dtype=np.float64).reshape(-1)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

"""tdg_dot_f64_noalloc: the allocation-free FP64 dot product.

It exists for callers that own all device memory and cannot let the library call cudaMalloc
(tdg_dot_f64 allocates its partial-sum buffer on its first call on each device). The test calls
both entry points through the C ABI on the same inputs, twice in a row with different sizes, and
requires the same result within FP64 summation-order tolerance. Oversized inputs are rejected on
the host before any launch. This file is collected last on purpose.
"""
import ctypes

import pytest
import torch


def _call(fn, a, b, out):
    from torch_de_solver_gb300 import _lib
    status = fn(a.data_ptr(), b.data_ptr(), a.numel(), out.data_ptr(),
                torch.cuda.current_stream().cuda_stream)
    _lib.check(status, fn.__name__)


@pytest.mark.gpu
def test_noalloc_dot_matches_allocating_dot_on_two_calls():
    from torch_de_solver_gb300 import _lib
    lib = _lib.load()
    gen = torch.Generator(device='cuda').manual_seed(7)
    out_ref = torch.zeros(1, dtype=torch.float64, device='cuda')
    out_new = torch.zeros(1, dtype=torch.float64, device='cuda')
    for n in (3_000_017, 66_819):
        a = torch.randn(n, device='cuda', generator=gen)
        b = torch.randn(n, device='cuda', generator=gen)
        _call(lib.tdg_dot_f64, a, b, out_ref)
        _call(lib.tdg_dot_f64_noalloc, a, b, out_new)
        torch.cuda.synchronize()
        scale = float((a.double() * b.double()).abs().sum())
        exact = float((a.double() * b.double()).sum())
        assert abs(out_new.item() - out_ref.item()) <= 1e-13 * scale
        assert abs(out_new.item() - exact) <= 1e-12 * scale


@pytest.mark.gpu
def test_noalloc_dot_rejects_sizes_beyond_its_scratch():
    from torch_de_solver_gb300 import _lib
    lib = _lib.load()
    a = torch.zeros(4, device='cuda')
    out = torch.zeros(1, dtype=torch.float64, device='cuda')
    status = lib.tdg_dot_f64_noalloc(a.data_ptr(), a.data_ptr(), _lib.DOT_NOALLOC_MAX_N + 1,
                                     out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert status == _lib.ERR_SHAPE
    assert b'static scratch limit' in lib.tdg_last_error()

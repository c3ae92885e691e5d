"""The C-ABI library loads on a machine without a GPU and exports every symbol of include/tdg.h;
argument validation reports errors through status codes (no compute calls)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, 'include', 'tdg.h')).read()
    return sorted(set(re.findall(r'^\w[\w\s\*]*?\b(tdg_\w+)\s*\(', src, re.M)))


def test_header_and_binding_agree():
    from torch_de_solver_gb300 import _lib
    assert set(declared_symbols()) == set(_lib.SIGNATURES)


def test_library_exports_every_declared_symbol():
    from torch_de_solver_gb300 import _lib
    lib = _lib.load()
    for name in declared_symbols():
        assert hasattr(lib, name), name
    assert lib.tdg_abi_version() == _lib.ABI_VERSION == 3


def test_struct_sizes_match_header():
    from torch_de_solver_gb300 import _lib
    assert ctypes.sizeof(_lib.GroupDesc) == 48
    assert ctypes.sizeof(_lib.SiteDesc) == 28
    assert ctypes.sizeof(_lib.SlotDesc) == 24
    assert ctypes.sizeof(_lib.TermDesc) == 24


def test_invalid_arguments_return_status():
    from torch_de_solver_gb300 import _lib
    lib = _lib.load()
    assert lib.tdg_plan_create(None, None) == _lib.ERR_INVALID
    assert b'null' in lib.tdg_last_error()
    assert lib.tdg_adam_step(None, None, None, None, None, 0, None, None) == _lib.ERR_INVALID
    assert lib.tdg_dot_f64(None, None, 0, None, None) == _lib.ERR_INVALID
    assert lib.tdg_plan_destroy(None) == _lib.OK


def test_causal_and_gather_reject_bad_shapes_without_a_gpu():
    """The shape and null checks run on the host, before any launch."""
    from torch_de_solver_gb300 import _lib
    lib = _lib.load()
    assert lib.tdg_causal_weights(None, 10, 1, 3, 1.0, None, None) == _lib.ERR_INVALID
    assert lib.tdg_causal_weights(1, 10, 1, 3, 1.0, 1, None) == _lib.ERR_SHAPE   # 10 rows, 3 slices
    assert b'time slices' in lib.tdg_last_error()
    assert lib.tdg_gather_rows(None, 5, None, 0, 2, None, None) == _lib.OK         # nothing to do
    assert lib.tdg_gather_rows(1, 5, 1, 4, 0, 1, None) == _lib.ERR_SHAPE


def test_lbfgs_entry_points_validate_on_the_host():
    """Argument checks of the device L-BFGS run before any allocation or launch."""
    from torch_de_solver_gb300 import _lib
    lib = _lib.load()
    assert lib.tdg_lbfgs_create(10, 4, None) == _lib.ERR_INVALID
    h = ctypes.c_void_p()
    assert lib.tdg_lbfgs_create(0, 4, ctypes.byref(h)) == _lib.ERR_SHAPE
    assert lib.tdg_lbfgs_create(10, 0, ctypes.byref(h)) == _lib.ERR_SHAPE and not h.value
    assert lib.tdg_lbfgs_push(None, None, None, None, 1.0, None) == _lib.ERR_INVALID
    assert lib.tdg_lbfgs_direction(None, None, None, 0, None) == _lib.ERR_INVALID
    assert lib.tdg_lbfgs_stats(None, None, None, None, None, None) == _lib.ERR_INVALID
    assert lib.tdg_axpy(None, None, 1.0, None, 3, None) == _lib.ERR_INVALID
    assert lib.tdg_lbfgs_destroy(None) == _lib.OK


def test_schedule_is_validated_before_the_description():
    """tdg_plan_create_scheduled rejects a malformed tile schedule on the host."""
    from torch_de_solver_gb300 import _lib
    lib = _lib.load()
    desc = _lib.ProblemDesc()
    h = ctypes.c_void_p()
    for bad in ((100, 0, 0, 0), (160, 0, 0, 0), (16, 0, 0, 0), (128, -1, 0, 0), (128, 0, 2, 0)):
        sc = _lib.Schedule(*bad)
        assert lib.tdg_plan_create_scheduled(ctypes.byref(desc), ctypes.byref(sc),
                                             ctypes.byref(h)) == _lib.ERR_INVALID, bad
        assert b'schedule' in lib.tdg_last_error()


def test_build_compiles_both_fused_kernels_once_per_site_class():
    """The build recipe instantiates the tensor-core kernel per (precision, site class) and the
    FP32 kernel per site class, for every class of tdg_jetcls.h (the dispatch tables of both
    kernels index them by class)."""
    from torch_de_solver_gb300.csrc import build
    src = open(os.path.join(ROOT, 'torch_de_solver_gb300', 'csrc', 'tdg_jetcls.h')).read()
    n_classes = int(re.search(r'constexpr int N_CLASSES = (\d+);', src).group(1))
    assert build.TC_CLASSES == n_classes
    objs = {obj for _, obj, _ in build.units()}
    for c in range(n_classes):
        assert f'tdg_fp32_c{c}.o' in objs
        for prec, _, _ in build.TC_PRECISIONS:
            assert f'tdg_tc_{prec}_c{c}.o' in objs
    assert len(objs) == len(build.units())   # no object built twice

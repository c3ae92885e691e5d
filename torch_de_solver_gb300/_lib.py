"""ctypes binding of libtdg.so, the C ABI declared in include/tdg.h.

The library is built in-tree (torch_de_solver_gb300/libtdg.so) by csrc/build.py. There is no
fallback: every compute call goes through this library, and importing it without the built
library raises.
"""

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, 'libtdg.so')

MAX_LAYERS = 12
MAX_DIN = 4
MAX_DOUT = 8
MAX_WIDTH = 128          # the fused forms: hidden widths that are multiples of 4, up to this
MAX_WIDTH_PLAIN = 4096   # the plain form: any hidden width up to this
MAX_ORDER = 3
MAX_STREAMS = 16
MAX_SITES = 16
MAX_COEFF = 16
ABI_VERSION = 3

OK, ERR_INVALID, ERR_UNSUPPORTED, ERR_SHAPE, ERR_CUDA, ERR_TIMEOUT, ERR_NOMEM = range(7)
PREC = {'fp32': 0, 'tf32': 1, '3xtf32': 2, 'bf16': 3}
FORM = {'fused': 0, 'plain': 1}

i32, i64, f32, f64 = ctypes.c_int32, ctypes.c_int64, ctypes.c_float, ctypes.c_double
vp = ctypes.c_void_p


class MlpDesc(ctypes.Structure):
    _fields_ = [('n_layers', i32), ('width', i32 * (MAX_LAYERS + 1))]


class StreamDesc(ctypes.Structure):
    _fields_ = [('order', i32), ('axes', i32 * MAX_ORDER)]


class SiteDesc(ctypes.Structure):
    _fields_ = [('points', i32), ('stream_first', i32), ('n_streams', i32), ('offset', f32 * MAX_DIN)]


class PartDesc(ctypes.Structure):
    _fields_ = [('site', i32), ('stream', i32), ('weight', f32)]


class FactorDesc(ctypes.Structure):
    _fields_ = [('part_first', i32), ('n_parts', i32), ('var', i32), ('power', f32)]


class TermDesc(ctypes.Structure):
    _fields_ = [('factor_first', i32), ('n_factors', i32), ('output', i32), ('coeff_array', i32),
                ('coeff', f32), ('coeff_param', i32)]


class GroupDesc(ctypes.Structure):
    _fields_ = [('problem', i32), ('n_rows', i32), ('site_first', i32), ('n_sites', i32),
                ('term_first', i32), ('n_terms', i32), ('n_outputs', i32), ('slot_first', i32),
                ('target_array', i32), ('row_weight_array', i32), ('output_offset', i64)]


class SlotDesc(ctypes.Structure):
    _fields_ = [('problem', i32), ('weight', f64), ('weight_normalized', f64)]


class ProblemDesc(ctypes.Structure):
    _fields_ = [('mlp', MlpDesc), ('n_problems', i32),
                ('n_groups', i32), ('groups', ctypes.POINTER(GroupDesc)),
                ('n_sites', i32), ('sites', ctypes.POINTER(SiteDesc)),
                ('n_streams', i32), ('streams', ctypes.POINTER(StreamDesc)),
                ('n_terms', i32), ('terms', ctypes.POINTER(TermDesc)),
                ('n_factors', i32), ('factors', ctypes.POINTER(FactorDesc)),
                ('n_parts', i32), ('parts', ctypes.POINTER(PartDesc)),
                ('n_slots', i32), ('slots', ctypes.POINTER(SlotDesc)),
                ('n_arrays', i32), ('arrays', ctypes.POINTER(vp)), ('array_len', ctypes.POINTER(i64)),
                ('precision', i32), ('form', i32), ('n_coeff_params', i32)]


class PlanInfo(ctypes.Structure):
    _fields_ = [('n_params', i64), ('workspace_bytes', i64), ('n_tiles', i32), ('n_ctas', i32),
                ('n_segments', i32), ('max_streams', i32), ('flops_hidden', f64),
                ('flops_total', f64)]


class Schedule(ctypes.Structure):
    _fields_ = [('max_rows', i32), ('n_ctas', i32), ('balance', i32), ('reserved', i32)]


class AdamDesc(ctypes.Structure):
    _fields_ = [('lr', f32), ('beta1', f32), ('beta2', f32), ('eps', f32), ('weight_decay', f32),
                ('maximize', i32)]


# entry point -> (restype, argtypes); kept in step with include/tdg.h
SIGNATURES = {
    'tdg_abi_version': (i32, []),
    'tdg_last_error': (ctypes.c_char_p, []),
    'tdg_launch_count': (i64, []),
    'tdg_site_class': (i32, [i32, ctypes.POINTER(StreamDesc)]),
    'tdg_plan_create': (i32, [ctypes.POINTER(ProblemDesc), ctypes.POINTER(vp)]),
    'tdg_plan_create_scheduled': (i32, [ctypes.POINTER(ProblemDesc), ctypes.POINTER(Schedule),
                                        ctypes.POINTER(vp)]),
    'tdg_plan_destroy': (i32, [vp]),
    'tdg_plan_get_info': (i32, [vp, ctypes.POINTER(PlanInfo)]),
    'tdg_plan_set_array': (i32, [vp, i32, vp, i64]),
    'tdg_loss': (i32, [vp, vp, vp, vp, vp]),
    'tdg_loss_grad': (i32, [vp, vp, vp, vp, vp, vp]),
    'tdg_plan_sync_status': (i32, [vp]),
    'tdg_selftest_bounded_wait': (i32, [i32]),
    'tdg_adam_step': (i32, [vp, vp, vp, vp, vp, i64, ctypes.POINTER(AdamDesc), vp]),
    'tdg_dot_f64': (i32, [vp, vp, i64, vp, vp]),
    'tdg_dot_f64_noalloc': (i32, [vp, vp, i64, vp, vp]),
    'tdg_lbfgs_create': (i32, [i64, i32, ctypes.POINTER(vp)]),
    'tdg_lbfgs_destroy': (i32, [vp]),
    'tdg_lbfgs_reset': (i32, [vp, vp]),
    'tdg_lbfgs_push': (i32, [vp, vp, vp, vp, ctypes.c_double, vp]),
    'tdg_lbfgs_direction': (i32, [vp, vp, vp, i32, vp]),
    'tdg_lbfgs_stats': (i32, [vp, vp, vp, vp, vp, vp]),
    'tdg_axpy': (i32, [vp, vp, ctypes.c_double, vp, i64, vp]),
    'tdg_causal_weights': (i32, [vp, i64, i32, i64, f32, vp, vp]),
    'tdg_gather_rows': (i32, [vp, i64, vp, i64, i32, vp, vp]),
}
DOT_NOALLOC_MAX_N = 4096 * 16384

_lib = None


class TdgError(RuntimeError):
    pass


def load():
    """Load libtdg.so once; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f'{LIB_PATH} is missing: build it with '
                          f'`python -m torch_de_solver_gb300.csrc.build` (no CPU fallback exists)')
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.tdg_abi_version() != ABI_VERSION:
        raise ImportError('libtdg.so ABI version mismatch')
    _lib = lib
    return lib


def check(status, what):
    if status != OK:
        msg = load().tdg_last_error().decode(errors='replace')
        if status == ERR_UNSUPPORTED:
            raise NotImplementedError(f'{what}: {msg}')
        raise TdgError(f'{what} failed (status {status}): {msg}')


def launch_count():
    return int(load().tdg_launch_count())


def site_class(streams):
    """Compile-time jet class of a site whose streams are sorted axis tuples, or -1 (tables)."""
    arr = (StreamDesc * len(streams))()
    for m, k in enumerate(streams):
        arr[m].order = len(k)
        for i, a in enumerate(k):
            arr[m].axes[i] = a
    return int(load().tdg_site_class(len(streams), arr))

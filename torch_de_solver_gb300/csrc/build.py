"""Build libtdg.so (the C-ABI CUDA library) in-tree with nvcc for sm_103a.

Every object compiles in parallel (the tensor-core kernel once per precision and main site
class, from tdg_tc_inst.cu); the shared library links against the CUDA runtime.
Usage: python -m torch_de_solver_gb300.csrc.build  (or build() from Python).
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
ROOT = os.path.dirname(PKG)
SOURCES = ['tdg_plan.cu', 'tdg_fused.cu', 'tdg_fused_tc.cu', 'tdg_plain.cu', 'tdg_util.cu',
           'tdg_noalloc.cu', 'tdg_lbfgs.cu']
# the tensor-core kernel: one object per (precision, main site class), from tdg_tc_inst.cu
TC_PRECISIONS = (('tf32', 0, 0), ('bf16', 1, 0), ('3x', 0, 1))
TC_CLASSES = 11   # jetcls::N_CLASSES in tdg_jetcls.h


def units():
    out = [(f'tdg_tc_inst.cu', f'tdg_tc_{p}_c{c}.o',
            [f'-DTDG_TC_PREC={p}', f'-DTDG_TC_BF16={b}', f'-DTDG_TC_X3={x}', f'-DTDG_TC_CLS={c}'])
           for p, b, x in TC_PRECISIONS for c in range(TC_CLASSES)]
    # the FP32 fused kernel: one object per main site class, from tdg_fp32_inst.cu
    out += [('tdg_fp32_inst.cu', f'tdg_fp32_c{c}.o', [f'-DTDG_F32_CLS={c}']) for c in range(TC_CLASSES)]
    return out + [(src, src.replace('.cu', '.o'), []) for src in SOURCES]
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
LIB = os.path.join(PKG, 'libtdg.so')


def nvcc():
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found: set NVCC or put the CUDA toolkit on PATH')


def build(verbose=False, extra=()):
    obj_dir = os.path.join(PKG, '_build')
    os.makedirs(obj_dir, exist_ok=True)
    flags = ['-O3', '-std=c++17', '-lineinfo', '-Xcompiler', '-fPIC', '-I' + os.path.join(ROOT, 'include'),
             '--expt-relaxed-constexpr', *ARCH, *extra]
    if verbose:
        flags += ['-Xptxas', '-v']
    cc = nvcc()

    def compile_one(unit):
        src, obj_name, defines = unit
        obj = os.path.join(obj_dir, obj_name)
        cmd = [cc, *flags, *defines, '-c', os.path.join(HERE, src), '-o', obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f'nvcc failed for {obj_name}:\n{r.stdout}\n{r.stderr}')
        return obj, r.stderr

    jobs = units()
    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, os.cpu_count() or 1)) as ex:
        results = list(ex.map(compile_one, jobs))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    objs = [o for o, _ in results]
    tmp = LIB + '.tmp'
    cmd = [cc, '-shared', *ARCH, '-o', tmp, *objs, '-cudart', 'shared']
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f'link failed:\n{r.stdout}\n{r.stderr}')
    os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    print(build(verbose='-v' in sys.argv))

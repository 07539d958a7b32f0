"""In-tree build of ``libqsgb.so``, the C-ABI library of the GB300 kernels.

Every ``csrc/*.cu`` translation unit is compiled in parallel by ``nvcc`` for
sm_103a only and linked into ``quantumsim_gb300/libqsgb.so`` (the CUDA runtime
is linked statically).  Objects go to ``quantumsim_gb300/_build/``.  The build
is skipped when the library is newer than every source file.
"""
import concurrent.futures as _cf
import glob
import os
import shutil
import subprocess

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG_DIR, 'csrc')
INCLUDE = os.path.join(os.path.dirname(PKG_DIR), 'include')
BUILD_DIR = os.path.join(PKG_DIR, '_build')
LIB_PATH = os.path.join(PKG_DIR, 'libqsgb.so')

ARCH_FLAGS = ['-gencode', 'arch=compute_103a,code=sm_103a']
NVCC_FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC',
              '--expt-relaxed-constexpr', '-I', INCLUDE]


def _nvcc():
    path = shutil.which('nvcc')
    if path is None:
        cand = '/usr/local/cuda/bin/nvcc'
        if os.path.exists(cand):
            return cand
        raise RuntimeError('nvcc not found: the CUDA toolkit is required to '
                           'build libqsgb.so')
    return path


def sources():
    return sorted(glob.glob(os.path.join(CSRC, '*.cu')))


def _deps():
    return (sources() + glob.glob(os.path.join(CSRC, '*.cuh')) +
            glob.glob(os.path.join(INCLUDE, '*.h')))


def is_stale():
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    return any(os.path.getmtime(f) > t for f in _deps())


def build(force=False, verbose=False, jobs=None):
    """Compile and link ``libqsgb.so``; returns its path."""
    if not force and not is_stale():
        return LIB_PATH
    nvcc = _nvcc()
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = sources()
    objs = [os.path.join(BUILD_DIR, os.path.basename(s)[:-3] + '.o')
            for s in srcs]

    def compile_one(src_obj):
        src, obj = src_obj
        cmd = [nvcc] + ARCH_FLAGS + NVCC_FLAGS + ['-c', src, '-o', obj]
        if verbose:
            print(' '.join(cmd))
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError('nvcc failed on {}:\n{}{}'.format(
                os.path.basename(src), res.stdout, res.stderr))
        return obj

    with _cf.ThreadPoolExecutor(max_workers=jobs or len(srcs)) as ex:
        list(ex.map(compile_one, zip(srcs, objs)))
    tmp = LIB_PATH + '.tmp'
    cmd = [nvcc] + ARCH_FLAGS + ['-shared', '-o', tmp] + objs
    if verbose:
        print(' '.join(cmd))
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError('nvcc link failed:\n{}{}'.format(res.stdout,
                                                           res.stderr))
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == '__main__':
    print(build(force=True, verbose=True))

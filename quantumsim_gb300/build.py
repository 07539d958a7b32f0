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
import sysconfig
import warnings

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG_DIR, 'csrc')
INCLUDE = os.path.join(os.path.dirname(PKG_DIR), 'include')
BUILD_DIR = os.path.join(PKG_DIR, '_build')
LIB_PATH = os.path.join(PKG_DIR, 'libqsgb.so')

ARCH_FLAGS = ['-gencode', 'arch=compute_103a,code=sm_103a']
NVCC_FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC',
              '--expt-relaxed-constexpr', '-I', INCLUDE, '-I', BUILD_DIR]
LINK_FLAGS = ['-ldl']
# device helpers embedded as text for the run-time specialised kernels
EMBED = [('qsgb_device.cuh', 'qsgb_device_src.inc', 'kQsgbDeviceSrc')]


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
            glob.glob(os.path.join(CSRC, '*.h')) +
            glob.glob(os.path.join(INCLUDE, '*.h')))


def is_stale():
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    return any(os.path.getmtime(f) > t for f in _deps())


def _embed():
    """Write each embedded header as a C++ raw string literal."""
    for src, dst, name in EMBED:
        with open(os.path.join(CSRC, src)) as f:
            text = f.read()
        if ')QSGB"' in text:
            raise RuntimeError('embedded source contains the delimiter')
        with open(os.path.join(BUILD_DIR, dst), 'w') as f:
            f.write('static const char {}[] = R"QSGB({})QSGB";\n'.format(
                name, text))


PYAPPLY_SRC = os.path.join(CSRC, 'qsgb_pyapply.c')


def pyapply_path():
    suffix = sysconfig.get_config_var('EXT_SUFFIX') or '.so'
    return os.path.join(PKG_DIR, '_qsgb_pyapply' + suffix)


def build_pyapply(force=False, verbose=False):
    """Compile the CPython entry point of the per-call apply path
    (``csrc/qsgb_pyapply.c``, host C, no CUDA or torch headers); returns its
    path, or None when no C compiler or Python headers are available, in
    which case the ctypes path is used."""
    out = pyapply_path()
    if (not force and os.path.exists(out) and
            os.path.getmtime(out) >= os.path.getmtime(PYAPPLY_SRC)):
        return out
    cc = shutil.which('gcc') or shutil.which('cc')
    inc = sysconfig.get_paths().get('include')
    if not cc or not inc or not os.path.exists(os.path.join(inc, 'Python.h')):
        return None
    tmp = out + '.tmp'
    cmd = [cc, '-O2', '-shared', '-fPIC', '-std=c11', '-Wall', '-I', inc,
           PYAPPLY_SRC, '-o', tmp]
    if verbose:
        print(' '.join(cmd))
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        warnings.warn('the CPython apply entry point did not build (the '
                      'ctypes path is used):\n' + res.stderr)
        return None
    os.replace(tmp, out)
    return out


def build(force=False, verbose=False, jobs=None):
    """Compile and link ``libqsgb.so`` (and the CPython apply entry
    point); returns the library's path."""
    build_pyapply(force=force, verbose=verbose)
    if not force and not is_stale():
        return LIB_PATH
    nvcc = _nvcc()
    os.makedirs(BUILD_DIR, exist_ok=True)
    _embed()
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
    cmd = [nvcc] + ARCH_FLAGS + ['-shared', '-o', tmp] + objs + LINK_FLAGS
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

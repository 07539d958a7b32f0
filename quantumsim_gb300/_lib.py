"""ctypes binding of ``libqsgb.so`` (the C ABI declared in ``include/qsgb.h``).

The library is loaded lazily on first use.  There is no fallback: if the
library is missing or cannot be loaded the call raises ``RuntimeError``.
"""
import ctypes
import os

from . import build as _build

# status codes / flags, mirroring include/qsgb.h
OK = 0
ERR_INVALID = 1
ERR_CUDA = 2
ERR_UNSUPPORTED = 3
ERR_SCRATCH = 4

DEV_RANGE = 1
DEV_TIMEOUT = 2
DEV_BADITEM = 4

F64 = 0
F32 = 1

ARITH_AUTO = 0
ARITH_DF64 = 1
ARITH_F64 = 2
ARITH_F32 = 3
ARITH_TC = 4

PTM_SWAPPED = 1
PTM_TRANSPOSED = 2
PTM_HOST = 4
PTM_NOJIT = 8

_c_void_p = ctypes.c_void_p
_i64 = ctypes.c_int64
_int = ctypes.c_int
_dbl = ctypes.c_double
_p_i64 = ctypes.POINTER(ctypes.c_int64)
_p_i32 = ctypes.POINTER(ctypes.c_int32)

# name -> (restype, argtypes)
SIGNATURES = {
    'qsgb_abi_version': (_int, []),
    'qsgb_status_string': (ctypes.c_char_p, [_int]),
    'qsgb_jit_available': (_int, []),
    'qsgb_apply_ptm1': (_int, [_c_void_p, _c_void_p, _c_void_p, _i64, _i64,
                               _i64, _i64, _int, _int, _int, _i64, _c_void_p,
                               _c_void_p]),
    'qsgb_apply_ptm2': (_int, [_c_void_p, _c_void_p, _c_void_p, _i64, _i64,
                               _i64, _i64, _i64, _i64, _i64, _int, _int, _int,
                               _i64, _c_void_p, _c_void_p]),
    'qsgb_prepare_ptm2': (_int, [_c_void_p, _i64, _i64, _i64, _i64, _i64,
                                 _i64, _i64, _int, _int, _int]),
    'qsgb_jit_check_ptm2': (_int, [_c_void_p, _i64, _i64, _i64, _i64, _i64,
                                   _i64, _i64, _int, _int, _int, _c_void_p,
                                   _i64]),
    'qsgb_gather': (_int, [_c_void_p, _c_void_p, _int, _int, _int, _p_i64,
                           _p_i32, _p_i32, _c_void_p]),
    'qsgb_diag_marginals': (_int, [_c_void_p, _int, _int, _p_i64, _p_i32,
                                   _p_i32, _int, _c_void_p, _c_void_p,
                                   _c_void_p, _c_void_p, _i64, _c_void_p]),
    'qsgb_diag_marginals_scratch_bytes': (_i64, []),
    'qsgb_take_axis': (_int, [_c_void_p, _c_void_p, _int, _i64, _i64, _i64,
                              _p_i32, _i64, _c_void_p]),
    'qsgb_marginals_scratch_bytes': (_i64, [_i64, _i64]),
    'qsgb_marginals': (_int, [_c_void_p, _int, _p_i64, _int, _c_void_p,
                              _c_void_p, _i64, _c_void_p]),
    'qsgb_marginals_noalloc_max_scratch_bytes': (_i64, []),
    'qsgb_marginals_noalloc': (_int, [_c_void_p, _int, _p_i64, _int,
                                      _c_void_p, _c_void_p]),
    'qsgb_partial_trace': (_int, [_c_void_p, _c_void_p, _int, _int, _p_i64,
                                  _p_i32, ctypes.POINTER(ctypes.c_double),
                                  _c_void_p]),
    'qsgb_scale': (_int, [_c_void_p, _int, _i64, _dbl, _c_void_p]),
    'qsgb_scale_by_inverse': (_int, [_c_void_p, _int, _i64, _c_void_p, _dbl,
                                     _c_void_p]),
    'qsgb_batch_max_grid': (_int, [_int]),
    'qsgb_batch_run': (_int, [_c_void_p, _int, _int, _int, _c_void_p, _i64,
                              _c_void_p]),
    'qsgb_ptm_grad_scratch_bytes': (_i64, [_i64, _i64, _i64]),
    'qsgb_ptm_grad1': (_int, [_c_void_p, _c_void_p, _c_void_p, _i64, _i64,
                              _i64, _i64, _int, _c_void_p, _i64, _c_void_p]),
    'qsgb_ptm_grad2': (_int, [_c_void_p, _c_void_p, _c_void_p, _i64, _i64,
                              _i64, _i64, _i64, _i64, _i64, _int, _c_void_p,
                              _i64, _c_void_p]),
}

_LIB = None


def library_path():
    return _build.LIB_PATH


def load():
    """Load (once) and return the ctypes handle of libqsgb.so."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not os.path.exists(path):
        raise RuntimeError(
            'libqsgb.so is not built ({}); run '
            '`python -m quantumsim_gb300.build` first'.format(path))
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(status, what):
    """Turn a non-zero C status into an exception."""
    if status == OK:
        return
    msg = load().qsgb_status_string(status).decode()
    if status == ERR_INVALID:
        raise ValueError('{}: {}'.format(what, msg))
    if status == ERR_UNSUPPORTED:
        raise NotImplementedError('{}: {}'.format(what, msg))
    raise RuntimeError('{}: {} (status {})'.format(what, msg, status))


def i64_array(values):
    values = list(values)
    return (ctypes.c_int64 * max(1, len(values)))(*values)


def i32_array(values):
    values = list(values)
    return (ctypes.c_int32 * max(1, len(values)))(*values)


def f64_array(values):
    values = list(values)
    return (ctypes.c_double * max(1, len(values)))(*values)

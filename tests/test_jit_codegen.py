"""The run-time code generator of the specialised apply kernels, checked on
the build host (no GPU): every variant it emits -- group pairs and single
groups, vector accesses along the last qudit, staged tiles for odd
dimensions, component order for 81x81 PTMs, FP32 storage, transposed,
swapped and rectangular PTMs -- compiles with NVRTC for sm_103a, and a
pattern with float-float rows carries the tables of its native-FP64
fallback."""
import ctypes
import math

import numpy as np
import pytest

from quantumsim_gb300 import _lib as L
from quantumsim_gb300 import build as qbuild
from quantumsim_gb300 import ops
from quantumsim_gb300 import workloads


@pytest.fixture(scope='module')
def lib():
    qbuild.build()
    lib = L.load()
    if not lib.qsgb_jit_available():
        pytest.skip('NVRTC is not available on this host')
    return lib


def _check(lib, ptm, shape, qudits, dtype=L.F64, arith=L.ARITH_AUTO,
           transpose=False):
    ptm = np.ascontiguousarray(ptm, dtype=np.float64)
    _, (X, Y, Z), (dao, dbo, dai, dbi), swapped = ops.apply_geometry(
        shape, list(qudits), ptm.shape, transpose)
    flags = L.PTM_HOST | (L.PTM_SWAPPED if swapped else 0) | (
        L.PTM_TRANSPOSED if transpose else 0)
    if len(qudits) == 1:
        dao, dai, X = 1, 1, 1
    buf = ctypes.create_string_buffer(1 << 20)
    st = lib.qsgb_jit_check_ptm2(ctypes.c_void_p(ptm.ctypes.data), dao, dbo,
                                 dai, dbi, X, Y, Z, flags, dtype, arith, buf,
                                 len(buf))
    return st, buf.value.decode()


def test_generated_variants_compile(lib):
    rng = np.random.default_rng(3)
    t1, t2 = workloads.coherence_times(rng, 8)
    cz = workloads.noisy_cz(rng, (2, 5), t1, t2)
    rot = workloads.noisy_1q(rng, t1[0], t2[0])
    dense = rng.standard_normal((4, 4, 4, 4))
    q9 = workloads.qutrit_1q(rng)
    q81 = workloads.qutrit_2q(rng)
    cases = [
        (cz, (4,) * 8, (2, 5), {}),                      # group pairs
        (cz, (4,) * 8, (5, 2), {}),                      # swapped
        (cz, (4,) * 8, (6, 7), {}),                      # last two qudits
        # dense (float-float: arith='auto' sends it to the tensor cores)
        (dense, (4,) * 8, (1, 6), {'arith': L.ARITH_DF64}),
        (dense, (4,) * 8, (1, 6), {'arith': L.ARITH_DF64, 'transpose': True}),
        (rot, (4,) * 8, (3,), {}),
        (rot, (4,) * 8, (7,), {}),                       # vector accesses
        (rot, (4,) * 8, (7,), {'dtype': L.F32, 'arith': L.ARITH_F32}),
        (cz, (4,) * 8, (2, 5), {'arith': L.ARITH_F64}),
        (q9, (9,) * 5, (4,), {}),                        # staged tiles
        (q9, (9,) * 5, (2,), {}),
        (q81, (9,) * 5, (1, 3), {}),                     # component order
        (q81, (9,) * 5, (4, 3), {}),                     # staged 81x81
        (np.eye(9)[[0, 4, 8]], (9,) * 4, (1,), {}),      # rectangular
    ]
    for ptm, shape, qudits, kw in cases:
        st, src = _check(lib, ptm, shape, qudits, **kw)
        assert st == L.OK, (qudits, shape, kw, st)
        assert 'qsgb_jit' in src


def test_float_float_rows_carry_the_fp64_fallback(lib):
    rng = np.random.default_rng(4)
    dense = rng.standard_normal((4, 4, 4, 4))
    st, src = _check(lib, dense, (4,) * 6, (1, 4), arith=L.ARITH_DF64)
    assert st == L.OK
    assert 'qfb_k[]' in src and 'qsgb_df_suspect' in src
    # under arith='auto' the dense PTM goes to the precompiled tensor-core
    # kernel: nothing to generate
    st, _ = _check(lib, dense, (4,) * 6, (1, 4))
    assert st == L.ERR_UNSUPPORTED
    # native FP64 throughout: no float-float rows, no fallback
    st, src = _check(lib, dense, (4,) * 6, (1, 4), arith=L.ARITH_F64)
    assert st == L.OK and 'qfb_k[]' not in src
    # a PTM whose magnitude leaves the float pair's range runs in FP64
    st, src = _check(lib, dense * 2.0 ** 120, (4,) * 6, (1, 4),
                     arith=L.ARITH_DF64)
    assert st == L.OK and 'qfb_k[]' not in src
    st, src = _check(lib, dense * 2.0 ** -120, (4,) * 6, (1, 4),
                     arith=L.ARITH_DF64)
    assert st == L.OK and 'qfb_k[]' not in src
    assert math.isfinite(float(st))

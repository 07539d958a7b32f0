"""CPU-side checks of the C ABI library and the host logic (no GPU).

The library must load and export every function ``include/qsgb.h``
declares; argument errors must be reported by status codes before any CUDA
call; the Python host must refuse to run without a CUDA device rather than
fall back to a CPU path."""
import ctypes
import os
import re

import numpy as np
import pytest
import torch

from conftest import ROOT
import quantumsim_gb300 as qg
from quantumsim_gb300 import _lib as L
from quantumsim_gb300 import ops
from quantumsim_gb300 import build as qbuild
from quantumsim_gb300.pauli_vector import _diag_plan

HEADER = os.path.join(ROOT, 'include', 'qsgb.h')


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
    return sorted(set(re.findall(r'\b(qsgb_\w+)\s*\(', text)))


@pytest.fixture(scope='module')
def lib():
    qbuild.build()
    return L.load()


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 14
    for name in names:
        assert hasattr(lib, name), name
        assert name in L.SIGNATURES, 'no ctypes signature for ' + name


def test_abi_version_and_status_strings(lib):
    assert lib.qsgb_abi_version() >= 2
    assert lib.qsgb_jit_available() in (0, 1)
    assert lib.qsgb_status_string(0) == b'ok'
    assert b'invalid' in lib.qsgb_status_string(1)


def test_argument_errors_rejected_on_host(lib):
    null = ctypes.c_void_p(0)
    one = ctypes.c_void_p(16)
    two = ctypes.c_void_p(32)
    # null pointers
    assert lib.qsgb_apply_ptm1(null, two, one, 4, 4, 1, 1, 0, L.F64, 0, 16,
                               null, null) == L.ERR_INVALID
    # aliasing in/out
    assert lib.qsgb_apply_ptm1(one, one, two, 4, 4, 1, 1, 0, L.F64, 0, 16,
                               null, null) == L.ERR_INVALID
    # bad dims / dtype / arith / flags
    assert lib.qsgb_apply_ptm2(one, two, two, 4, 4, 4, 0, 1, 1, 1, 0, L.F64,
                               0, 16, null, null) == L.ERR_INVALID
    assert lib.qsgb_apply_ptm1(one, two, two, 4, 4, 1, 1, 0, 7, 0, 16, null,
                               null) == L.ERR_INVALID
    assert lib.qsgb_apply_ptm1(one, two, two, 4, 4, 1, 1, 0, L.F32,
                               L.ARITH_DF64, 16, null, null) == L.ERR_INVALID
    assert lib.qsgb_apply_ptm1(one, two, two, 4, 4, 1, 1, 64, L.F64, 0, 16,
                               null, null) == L.ERR_INVALID
    assert lib.qsgb_apply_ptm1(one, two, two, 4, 4, 1, 1, L.PTM_SWAPPED,
                               L.F64, 0, 16, null, null) == L.ERR_INVALID
    # too large PTMs are unsupported, host PTMs limited to 256 entries
    assert lib.qsgb_apply_ptm2(one, two, two, 81, 81, 81, 81, 1, 1, 1, 0,
                               L.F64, 0, 0, null, null) == L.ERR_UNSUPPORTED
    assert lib.qsgb_apply_ptm2(one, two, two, 81, 81, 81, 81, 1, 1, 1,
                               L.PTM_HOST, L.F64, 0, 0, null,
                               null) == L.ERR_UNSUPPORTED
    assert lib.qsgb_apply_ptm2(one, two, two, 9, 9, 9, 9, 1, 1, 1,
                               L.PTM_HOST | L.PTM_NOJIT, L.F64, 0, 0, null,
                               null) == L.ERR_UNSUPPORTED
    # ahead-of-time preparation needs a host PTM (flags checked before
    # anything is read)
    assert lib.qsgb_prepare_ptm2(two, 4, 4, 4, 4, 1, 1, 1, 0, L.F64,
                                 0) == L.ERR_INVALID
    # gathers
    assert lib.qsgb_take_axis(one, one, L.F64, 1, 4, 1, L.i32_array([0]), 1,
                              null) == L.ERR_INVALID
    assert lib.qsgb_take_axis(one, two, L.F64, 1, 4, 1, L.i32_array([4]), 1,
                              null) == L.ERR_INVALID
    assert lib.qsgb_gather(one, two, L.F64, L.F64, 1, L.i64_array([4]),
                           L.i32_array([0, 1]), L.i32_array([9]),
                           null) == L.ERR_INVALID
    # scratch too small
    assert lib.qsgb_marginals(one, 1, L.i64_array([64]), 0, two, null, 0,
                              null) == L.ERR_SCRATCH
    assert lib.qsgb_partial_trace(one, one, L.F64, 1, L.i64_array([4]),
                                  L.i32_array([1]), None,
                                  null) == L.ERR_INVALID


def test_scratch_queries(lib):
    assert lib.qsgb_marginals_scratch_bytes(16384, 2) >= 16
    assert lib.qsgb_marginals_scratch_bytes(0, 2) == 0
    assert lib.qsgb_ptm_grad_scratch_bytes(1 << 16, 16, 16) >= 16 * 16 * 8


def test_status_check_maps_to_exceptions():
    with pytest.raises(ValueError):
        L.check(L.ERR_INVALID, 'x')
    with pytest.raises(NotImplementedError):
        L.check(L.ERR_UNSUPPORTED, 'x')
    with pytest.raises(RuntimeError):
        L.check(L.ERR_CUDA, 'x')
    L.check(L.OK, 'x')


@pytest.mark.parametrize('shape,qudits,ptm_shape,exp', [
    ((4, 4, 4), (1,), (4, 4), ([4, 4, 4], (1, 4, 4), (1, 4, 1, 4), False)),
    ((4, 4, 4), (0,), (1, 4), ([1, 4, 4], (1, 1, 16), (1, 1, 1, 4), False)),
    ((4, 9, 4, 4), (3, 1), (2, 3, 4, 9),
     ([4, 3, 4, 2], (4, 4, 1), (3, 2, 9, 4), True)),
    ((4, 4, 4, 4), (0, 2), (4, 4, 4, 4),
     ([4, 4, 4, 4], (1, 4, 4), (4, 4, 4, 4), False)),
])
def test_apply_geometry(shape, qudits, ptm_shape, exp):
    assert ops.apply_geometry(shape, qudits, ptm_shape) == exp


def test_apply_geometry_transposed_and_mismatch():
    new, _, dims, sw = ops.apply_geometry((4, 3, 4), (1,), (3, 9), True)
    assert new == [4, 9, 4] and dims == (1, 9, 1, 3)
    with pytest.raises(ValueError):
        ops.apply_geometry((4, 4), (0,), (4, 3))


def test_nnz_terms_rule():
    p = np.array([[1.0, 0.0, 1e-20, 0.5], [0, 0, 1e-16, 0]])
    assert ops.nnz_terms(p, L.ARITH_F64) == 4
    assert ops.nnz_terms(p, L.ARITH_DF64) == 2
    assert ops.nnz_terms(p, L.ARITH_AUTO) == 2
    assert ops.nnz_terms(np.zeros((2, 2)), L.ARITH_DF64) == 1


def test_diag_plan():
    g2, g3 = qg.bases.general(2), qg.bases.general(3)
    off, idx = _diag_plan([g2, g3.subbasis([0, 2, 3])])
    assert off == [0, 2, 5] and idx == [0, 1, 0, -1, 1]
    assert _diag_plan([qg.bases.gell_mann(2)]) is None


def test_backend_refuses_without_cuda():
    if torch.cuda.is_available():
        pytest.skip('a CUDA device is present')
    with pytest.raises(RuntimeError):
        qg.PauliVectorGB300([qg.bases.general(2)] * 2)
    with pytest.raises(RuntimeError):
        torch.ops.qsgb.apply_ptm(torch.zeros(4, 4, dtype=torch.float64),
                                 torch.eye(4, dtype=torch.float64), [0], 0,
                                 16, False)


def test_size_guard_and_argument_validation_precede_device():
    g2 = qg.bases.general(2)
    with pytest.raises(ValueError):
        qg.PauliVectorGB300([g2] * 16)


def test_registered_into_reference_namespace_when_available():
    try:
        import quantumsim.pauli_vectors as qpv
    except Exception:
        pytest.skip('quantumsim not importable here')
    assert qpv.PauliVectorGB300 is qg.PauliVectorGB300
    from quantumsim.pauli_vectors.pauli_vector import PauliVectorBase
    assert issubclass(qg.PauliVectorGB300, PauliVectorBase)


def test_batch_program_layout_matches_the_header():
    """The ctypes mirror of qsgb_batch_program follows C layout rules on
    64-bit hosts: n_instances (ABI 2) sits in what was the padding after
    n_stages, so the pointer fields keep their offsets."""
    from quantumsim_gb300 import batch as BT
    P = BT._Program
    assert P.n_stages.offset == 24 and P.n_instances.offset == 28
    assert P.work.offset == 32 and ctypes.sizeof(P) == 96
    assert ctypes.sizeof(BT._Instance) == 40
    assert BT._ITEM_DTYPE.itemsize == 40


def test_plain_c_host_binds_the_library(lib, tmp_path):
    """A C program (tests/c_host/abi_smoke.c) compiled with gcc against
    include/qsgb.h and linked to libqsgb.so: the binding a C, cgo, JNI or
    N-API host would make.  It checks the ABI version, the status strings
    and host-side argument errors, none of which needs a GPU."""
    import shutil
    import subprocess
    gcc = shutil.which('gcc')
    if gcc is None:
        pytest.skip('gcc not available')
    libdir = os.path.dirname(L.library_path())
    exe = str(tmp_path / 'abi_smoke')
    build = subprocess.run(
        [gcc, '-std=c99', '-Wall', '-Werror', '-I', os.path.join(ROOT, 'include'),
         os.path.join(ROOT, 'tests', 'c_host', 'abi_smoke.c'), '-L', libdir,
         '-lqsgb', '-Wl,-rpath,' + libdir, '-o', exe],
        capture_output=True, text=True)
    assert build.returncode == 0, build.stderr
    run = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stdout + run.stderr
    assert 'argument checks ok' in run.stdout

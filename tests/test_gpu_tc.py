"""Dense 16 x 16 PTMs on the tensor cores (csrc/qsgb_tc.cu) against the
oracle: every ordered qubit pair (so every stride class, including the last
two qubits and groups that are not consecutive), the transposed and swapped
layouts, fused physical PTMs per entry at 1e-12, vectors whose bystanders
leave a partial tile, the full double range, and inf / nan inputs."""
import math

import numpy as np
import pytest
import torch

from conftest import ATOL_F64, RTOL_F64, assert_close_dot
from oracle import pauli_vector_np as O
import quantumsim_gb300 as qg
from quantumsim_gb300 import _lib as L
from quantumsim_gb300 import bases as B
from quantumsim_gb300 import ptm as P
from quantumsim_gb300 import workloads

pytestmark = pytest.mark.gpu

GB = qg.PauliVectorGB300


def _rand_pv(rng, shape):
    return rng.standard_normal(shape) / math.sqrt(np.prod(shape))


def _apply(pv_np, ptm, qs, bases, arith=L.ARITH_TC, transpose=False):
    s = GB(bases, pv_np)
    s._data = torch.ops.qsgb.apply_ptm(
        s._data, torch.from_numpy(np.ascontiguousarray(ptm)), list(qs), arith,
        0, transpose)
    return s.to_pv()


def test_dense_on_every_ordered_pair():
    rng = np.random.default_rng(101)
    n = 6
    bases = [B.general(2)] * n
    pv = _rand_pv(rng, (4,) * n)
    for q0 in range(n):
        for q1 in range(n):
            if q0 == q1:
                continue
            ptm = rng.standard_normal((4, 4, 4, 4))
            got = _apply(pv, ptm, (q0, q1), bases)
            ref = O.apply_ptm(pv, ptm, q0, q1)
            absref = O.apply_ptm(np.abs(pv), np.abs(ptm), q0, q1)
            assert_close_dot(got, ref, absref)


def test_transposed_and_auto_dispatch():
    rng = np.random.default_rng(102)
    bases = [B.general(2)] * 5
    pv = _rand_pv(rng, (4,) * 5)
    ptm = rng.standard_normal((4, 4, 4, 4))
    # transpose: the stored PTM is the forward one, its transpose applied
    got = _apply(pv, ptm, (3, 1), bases, transpose=True)
    ref = O.apply_ptm(pv, ptm.transpose(2, 3, 0, 1), 3, 1)
    absref = O.apply_ptm(np.abs(pv), np.abs(ptm).transpose(2, 3, 0, 1), 3, 1)
    assert_close_dot(got, ref, absref)
    # arith='auto' sends a dense PTM to the same kernel: same bits
    a = _apply(pv, ptm, (0, 4), bases, arith=L.ARITH_TC)
    b = _apply(pv, ptm, (0, 4), bases, arith=L.ARITH_AUTO)
    np.testing.assert_array_equal(a, b)


def test_fused_physical_ptms_per_entry():
    """CZ between noisy rotations (the fused units of the 14-qubit circuit)
    at 12 qubits, per entry at 1e-12 with the 1e-14 floor."""
    rng = np.random.default_rng(103)
    n = 12
    t1, t2 = workloads.coherence_times(rng, n)
    pv = _rand_pv(rng, (4,) * n)
    s = GB([B.general(2)] * n, pv, force=True, arith='tc')
    ref = pv
    for qs in [(0, 1), (11, 10), (3, 9), (9, 3), (5, 11), (0, 10)]:
        ra = torch.from_numpy(workloads.noisy_1q(rng, t1[qs[0]], t2[qs[0]]))
        rb = torch.from_numpy(workloads.noisy_1q(rng, t1[qs[1]], t2[qs[1]]))
        cz = torch.from_numpy(workloads.noisy_cz(rng, qs, t1, t2))
        fused = P.compose(P.kron(ra, rb), cz).numpy()
        s.apply_ptm(fused, *qs)
        ref = O.apply_ptm(ref, fused, *qs)
    np.testing.assert_allclose(s.to_pv(), ref, rtol=RTOL_F64, atol=ATOL_F64)


def test_partial_tiles_and_odd_bystanders():
    """Bystanders of dims 3 and 5 around two full-basis qubits: 15 groups,
    not a multiple of the 8 of a tile, none of them consecutive."""
    rng = np.random.default_rng(104)
    b2 = B.general(2)
    bases = [B.general(3).subbasis([0, 1, 2]), b2, b2, B.general(3).subbasis(
        [0, 1, 2, 3, 4])]
    shape = (3, 4, 4, 5)
    pv = _rand_pv(rng, shape)
    for qs in [(1, 2), (2, 1)]:
        ptm = rng.standard_normal((4, 4, 4, 4))
        got = _apply(pv, ptm, qs, bases)
        ref = O.apply_ptm(pv, ptm, *qs)
        absref = O.apply_ptm(np.abs(pv), np.abs(ptm), *qs)
        assert_close_dot(got, ref, absref)


@pytest.mark.parametrize('scale', [1e300, 1e-300, 1e-310])
def test_full_double_range(scale):
    rng = np.random.default_rng(105)
    bases = [B.general(2)] * 4
    pv = _rand_pv(rng, (4,) * 4) * scale
    ptm = P.compose(P.kron(P.rotate('x', 0.4), P.rotate('y', 1.3)),
                    P.cphase(2.2)).numpy()
    for qs in [(0, 1), (2, 3), (3, 0)]:
        got = _apply(pv, ptm, qs, bases)
        ref = O.apply_ptm(pv, ptm, *qs)
        absref = O.apply_ptm(np.abs(pv), np.abs(ptm), *qs)
        assert_close_dot(got, ref, absref, atol=0.0 if scale > 1e-300 else
                         5e-324 * 64)


def test_inf_and_nan_inputs_follow_fp64():
    rng = np.random.default_rng(106)
    bases = [B.general(2)] * 3
    pv = _rand_pv(rng, (4,) * 3)
    pv[0, 1, 2] = np.inf
    pv[2, 3, 1] = np.nan
    ptm = rng.standard_normal((4, 4, 4, 4))
    got = _apply(pv, ptm, (0, 2), bases)
    with np.errstate(invalid='ignore'):
        ref = O.apply_ptm(pv, ptm, 0, 2)
    np.testing.assert_array_equal(np.isnan(got), np.isnan(ref))
    fin = np.isfinite(ref)
    np.testing.assert_array_equal(np.isinf(got), np.isinf(ref))
    np.testing.assert_allclose(got[fin], ref[fin], rtol=1e-12, atol=1e-14)


def test_device_ptms_match_the_host_split_bitwise():
    """A 16 x 16 PTM in device memory is split by the kernel itself: the
    digits are the host split's, so every layout (plain, swapped,
    transposed, both) gives the host path's bits; 'auto' sends device PTMs
    there too."""
    rng = np.random.default_rng(107)
    n = 7
    pv = torch.from_numpy(_rand_pv(rng, (4,) * n)).cuda()
    for qs in [(0, 1), (1, 0), (2, 6), (6, 5), (5, 3)]:
        ptm = rng.standard_normal((4, 4, 4, 4))
        for tr in (False, True):
            host = torch.ops.qsgb.apply_ptm(pv, torch.from_numpy(ptm), list(qs),
                                            L.ARITH_TC, 0, tr)
            for arith in (L.ARITH_TC, L.ARITH_AUTO):
                dev = torch.ops.qsgb.apply_ptm(pv, torch.from_numpy(ptm).cuda(),
                                               list(qs), arith, 0, tr)
                assert torch.equal(dev, host), (qs, tr, arith)
            ref = (O.apply_ptm_transposed(pv.cpu().numpy(), ptm, *qs) if tr
                   else O.apply_ptm(pv.cpu().numpy(), ptm, *qs))
            absref = (O.apply_ptm_transposed(np.abs(pv.cpu().numpy()),
                                             np.abs(ptm), *qs) if tr
                      else O.apply_ptm(np.abs(pv.cpu().numpy()), np.abs(ptm),
                                       *qs))
            assert_close_dot(host.cpu().numpy(), ref, absref)


def test_device_ptm_with_inf_follows_fp64():
    rng = np.random.default_rng(108)
    pv = _rand_pv(rng, (4,) * 4)
    ptm = rng.standard_normal((4, 4, 4, 4))
    ptm[1, 2, 0, 3] = np.inf
    got = torch.ops.qsgb.apply_ptm(torch.from_numpy(pv).cuda(),
                                   torch.from_numpy(ptm).cuda(), [1, 3],
                                   L.ARITH_AUTO, 0, False).cpu().numpy()
    with np.errstate(invalid='ignore'):
        ref = O.apply_ptm(pv, ptm, 1, 3)
    np.testing.assert_array_equal(np.isnan(got), np.isnan(ref))
    np.testing.assert_array_equal(np.isinf(got), np.isinf(ref))
    fin = np.isfinite(ref)
    np.testing.assert_allclose(got[fin], ref[fin], rtol=1e-12, atol=1e-14)

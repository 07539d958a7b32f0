"""Parity of the GB300 backend (CUDA kernels through the C ABI) with the
reference: golden fixtures from quantumsim's PauliVectorNumpy, the
reference tests' known answers, and the oracle on seeded inputs at every
target position and stride class.  FP64 agreement: 1e-12 relative per entry
(1e-14 absolute floor), 1e-12 absolute on probabilities."""
import itertools
import math
import warnings

import numpy as np
import pytest
import torch

from conftest import (ATOL_F64, ATOL_PROB, RTOL_F64, assert_close_dot,
                      assert_close_f64, chain_rtol, golden_bases,
                      golden_cases)
from oracle import pauli_vector_np as O
import quantumsim_gb300 as qg
from quantumsim_gb300 import _lib as L
from quantumsim_gb300 import bases as B
from quantumsim_gb300 import ptm as P
from quantumsim_gb300 import workloads

pytestmark = pytest.mark.gpu

GB = qg.PauliVectorGB300


def rand_pv(rng, shape):
    return rng.standard_normal(shape) / math.sqrt(np.prod(shape))


def rand_ptm(rng, shape, density=1.0):
    p = rng.standard_normal(shape)
    if density < 1:
        p *= rng.random(shape) < density
    return p


# ---------------------------------------------------------------- golden
def test_golden_cases_on_gpu(golden):
    for i, case in enumerate(golden_cases(golden)):
        bases = golden_bases(golden, case['bases'])
        pv_in = golden['c{}_in'.format(i)]
        s = GB(bases, pv_in.copy())
        kind = case['kind']
        if kind == 'apply':
            s.apply_ptm(golden['c{}_ptm'.format(i)], *case['qubits'])
            assert_close_f64(s.to_pv(), golden['c{}_out'.format(i)])
        elif kind == 'reduce':
            assert_close_f64(s.diagonal(), golden['c{}_diag'.format(i)])
            assert s.trace() == pytest.approx(
                float(golden['c{}_trace'.format(i)]), abs=ATOL_PROB)
            for q in range(len(bases)):
                np.testing.assert_allclose(
                    s.meas_prob(q), golden['c{}_prob{}'.format(i, q)],
                    rtol=0, atol=ATOL_PROB)
            tr = s.renormalize()
            assert tr == pytest.approx(
                float(golden['c{}_renorm_trace'.format(i)]), abs=ATOL_PROB)
            assert_close_f64(s.to_pv(), golden['c{}_renorm_pv'.format(i)])
        elif kind == 'partial_trace':
            pt = s.partial_trace(*case['keep'])
            assert isinstance(pt, GB)
            assert_close_f64(pt.to_pv(), golden['c{}_out'.format(i)])
            assert pt.bases == [bases[q] for q in case['keep']]
        elif kind == 'reduce_basis':
            s.reduce_basis(case['qubit'], case['indices'])
            np.testing.assert_array_equal(s.to_pv(),
                                          golden['c{}_out'.format(i)])
            assert s.bases[case['qubit']].dim_pauli == len(case['indices'])


def test_circuit0_matches_reference(golden):
    ops = workloads.config0_circuit(seed=0)
    s = GB([B.general(2)] * 6)
    workloads.run(s, ops)
    assert_close_f64(s.to_pv(), golden['circuit0_pv'])
    np.testing.assert_allclose(s.diagonal(), golden['circuit0_diag'],
                               rtol=0, atol=ATOL_PROB)


# ---------------------------------------------------------------- strides
@pytest.mark.parametrize('arith,dtype,rtol,atol', [
    ('auto', np.float64, 1e-12, 1e-14),
    ('df64', np.float64, 1e-12, 1e-14),
    ('f64', np.float64, 1e-13, 1e-15),
    ('f32', np.float32, 2e-5, 2e-6)])
def test_1q_every_position(arith, dtype, rtol, atol):
    rng = np.random.default_rng(11)
    n = 8
    bases = [B.general(2)] * n
    for q in range(n):
        pv = rand_pv(rng, (4,) * n)
        ptm = rand_ptm(rng, (4, 4))
        s = GB(bases, pv, dtype=dtype, arith=arith)
        s.apply_ptm(ptm, q)
        np.testing.assert_allclose(s.to_pv(), O.apply_ptm(pv, ptm, q),
                                   rtol=rtol, atol=atol)


@pytest.mark.parametrize('density', [1.0, 0.3])
def test_2q_every_ordered_pair(density):
    rng = np.random.default_rng(12)
    n = 6
    bases = [B.general(2)] * n
    mask = rng.random((4, 4, 4, 4)) < density  # one sparsity pattern
    for q0, q1 in itertools.permutations(range(n), 2):
        pv = rand_pv(rng, (4,) * n)
        ptm = rand_ptm(rng, (4, 4, 4, 4)) * mask
        s = GB(bases, pv)
        s.apply_ptm(ptm, q0, q1)
        assert_close_dot(s.to_pv(), O.apply_ptm(pv, ptm, q0, q1),
                         O.apply_ptm(np.abs(pv), np.abs(ptm), q0, q1))


def test_noisy_cz_on_pairs_native_and_df64():
    rng = np.random.default_rng(13)
    n = 7
    t1, t2 = workloads.coherence_times(rng, n)
    for q0, q1 in [(0, 6), (6, 0), (2, 3), (5, 1), (4, 6)]:
        ptm = workloads.noisy_cz(rng, (q0, q1), t1, t2)
        pv = rand_pv(rng, (4,) * n)
        ref = O.apply_ptm(pv, ptm, q0, q1)
        for arith in ('auto', 'df64', 'f64'):
            s = GB([B.general(2)] * n, pv, arith=arith)
            s.apply_ptm(ptm, q0, q1)
            assert_close_f64(s.to_pv(), ref)


def test_rectangular_and_mixed_dims():
    rng = np.random.default_rng(14)
    shape = (9, 4, 3, 9, 1)
    b = [B.general(3), B.general(2), B.general(3).subbasis([0, 1, 2]),
         B.general(3), B.general(2).subbasis([0])]
    for qs, pshape in [((0,), (3, 9)), ((2,), (9, 3)), ((4,), (4, 1)),
                       ((0, 3), (9, 9, 9, 9)), ((3, 0), (3, 1, 9, 9)),
                       ((1, 2), (1, 9, 4, 3)), ((4, 2), (4, 3, 1, 3)),
                       ((3, 1), (9, 4, 9, 4))]:
        pv = rand_pv(rng, shape)
        ptm = rand_ptm(rng, pshape, 0.5)
        s = GB(b, pv, force=True)
        s.apply_ptm(ptm, *qs)
        assert_close_dot(s.to_pv(), O.apply_ptm(pv, ptm, *qs),
                         O.apply_ptm(np.abs(pv), np.abs(ptm), *qs))


def test_two_qutrit_81x81_dense_and_cphase():
    rng = np.random.default_rng(15)
    bases = [B.general(3)] * 4
    for ptm, qs in [(rand_ptm(rng, (9, 9, 9, 9)), (1, 3)),
                    (P.qutrit_cphase(math.pi + 0.02, 0.005).numpy(), (2, 0)),
                    (workloads.qutrit_1q(rng), (3,))]:
        pv = rand_pv(rng, (9,) * 4)
        s = GB(bases, pv)
        s.apply_ptm(ptm, *qs)
        assert_close_dot(s.to_pv(), O.apply_ptm(pv, ptm, *qs),
                         O.apply_ptm(np.abs(pv), np.abs(ptm), *qs))


@pytest.mark.parametrize('arith', [0, 2])
def test_last_qudit_shared_memory_staging(arith):
    """PTMs on the last qudit with odd dimensions (the specialised kernel
    stages 32 groups per warp in shared memory): 1 and 2 qutrits, adjacent
    and distant pairs, rectangular, item counts that leave partial warp
    tiles (1, 25 of 32), and FP32 storage."""
    rng = np.random.default_rng(16)
    dev = torch.device('cuda')
    cases = [((9,) * 5, (4,), (9, 9)),
             ((9,) * 5, (4, 3), (9, 9, 9, 9)),
             ((9,) * 5, (3, 4), (9, 9, 9, 9)),
             ((9,) * 5, (0, 4), (9, 9, 9, 9)),
             ((9, 9), (1, 0), (9, 9, 9, 9)),
             ((9, 4, 9), (2,), (3, 9)),
             ((4, 9, 3), (2, 1), (1, 9, 3, 9)),
             ((4, 4, 3), (2,), (3, 3))]
    for shape, qs, pshape in cases:
        x = rand_pv(rng, shape)
        for ptm in (rand_ptm(rng, pshape, 0.3), rand_ptm(rng, pshape)):
            ref = O.apply_ptm(x, ptm, *qs)
            absref = O.apply_ptm(np.abs(x), np.abs(ptm), *qs)
            y = torch.ops.qsgb.apply_ptm(torch.from_numpy(x).to(dev),
                                         torch.from_numpy(ptm), list(qs),
                                         arith, ptm.size, False, True)
            assert_close_dot(y.cpu().numpy(), ref, absref)
            y32 = torch.ops.qsgb.apply_ptm(
                torch.from_numpy(x).to(dev).float(), torch.from_numpy(ptm),
                list(qs), 3, ptm.size, False, True)
            np.testing.assert_allclose(y32.cpu().numpy(), ref, rtol=1e-4,
                                       atol=1e-5 * np.abs(absref).max())
    # the leakage CZ and the qutrit rotation of the qutrit workload; at 7
    # qutrits each warp takes several tiles (bulk copies, then a ragged
    # last tile of 17 groups)
    bases = [B.general(3)] * 7
    pv = rand_pv(rng, (9,) * 7)
    s = GB(bases, pv, force=True)
    ref = pv
    for ptm, qs in [(workloads.qutrit_2q(rng), (6, 5)),
                    (workloads.qutrit_1q(rng), (6,)),
                    (workloads.qutrit_2q(rng), (2, 6))]:
        s.apply_ptm(ptm, *qs)
        ref = O.apply_ptm(ref, ptm, *qs)
    assert_close_f64(s.to_pv(), ref)


@pytest.mark.parametrize('arith', [0, 1, 2])
def test_specialised_and_generic_kernels_agree(arith):
    """The run-time specialised kernel and the generic one give the same
    result (and match the oracle) on rectangular, swapped and transposed
    applications, pairs and single groups, FP64 and FP32."""
    rng = np.random.default_rng(21)
    dev = torch.device('cuda')
    cases = [((4, 4, 4, 4, 4), (1, 3), (4, 4, 4, 4), False),
             ((4, 4, 4, 4, 4), (4, 0), (4, 4, 4, 4), False),
             ((4, 3, 4, 9), (3, 1), (9, 3, 9, 3), False),
             ((4, 3, 4, 9), (2,), (1, 4), False),
             ((9, 9, 9), (0, 2), (9, 9, 9, 9), False),
             ((4, 4, 4, 4), (2, 0), (4, 4, 4, 4), True)]
    for shape, qs, pshape, tr in cases:
        x = rand_pv(rng, shape)
        ptm = rand_ptm(rng, pshape, 0.4)
        ref = (O.apply_ptm_transposed(x, ptm, *qs) if tr
               else O.apply_ptm(x, ptm, *qs))
        absref = (O.apply_ptm_transposed(np.abs(x), np.abs(ptm), *qs) if tr
                  else O.apply_ptm(np.abs(x), np.abs(ptm), *qs))
        xt = torch.from_numpy(x).to(dev)
        outs = []
        for jit in (True, False):
            y = torch.ops.qsgb.apply_ptm(xt, torch.from_numpy(ptm), list(qs),
                                         arith, ptm.size, tr, jit)
            outs.append(y.cpu().numpy())
            assert_close_dot(outs[-1], ref, absref)
        y32 = torch.ops.qsgb.apply_ptm(xt.float(), torch.from_numpy(ptm),
                                       list(qs), 3, ptm.size, tr, True)
        np.testing.assert_allclose(y32.cpu().numpy(), ref, rtol=1e-4,
                                   atol=1e-5)


def test_transposed_apply_and_ptm_grad_ops():
    rng = np.random.default_rng(16)
    dev = torch.device('cuda')
    x = rand_pv(rng, (4, 3, 4, 9))
    ptm = rand_ptm(rng, (2, 4, 4, 4))   # qudits (2, 0), rectangular
    g = rand_pv(rng, O.apply_ptm(x, ptm, 2, 0).shape)
    xt = torch.from_numpy(x).to(dev)
    gt = torch.from_numpy(g).to(dev)
    pt = torch.from_numpy(ptm)
    adj = torch.ops.qsgb.apply_ptm(gt, pt, [2, 0], 1, ptm.size, True)
    assert_close_f64(adj.cpu().numpy(), O.apply_ptm_transposed(g, ptm, 2, 0))
    dptm = torch.ops.qsgb.ptm_grad(xt, gt, [2, 0])
    np.testing.assert_allclose(dptm.cpu().numpy(), O.ptm_grad(x, g, 2, 0),
                               rtol=1e-12, atol=1e-13)
    p1 = rand_ptm(rng, (3, 3))
    y1 = O.apply_ptm(x, p1, 1)
    g1 = rand_pv(rng, y1.shape)
    d1 = torch.ops.qsgb.ptm_grad(xt, torch.from_numpy(g1).to(dev), [1])
    np.testing.assert_allclose(d1.cpu().numpy(), O.ptm_grad(x, g1, 1),
                               rtol=1e-12, atol=1e-13)
    for dtype, tol in ((torch.float32, 1e-5),):
        d32 = torch.ops.qsgb.ptm_grad(xt.to(dtype), gt.to(dtype), [2, 0])
        np.testing.assert_allclose(d32.cpu().numpy(), O.ptm_grad(x, g, 2, 0),
                                   rtol=tol, atol=tol)


# ---------------------------------------------------------------- KATs
def test_kat_create_trivial():
    s = GB([])
    assert s.to_pv() == pytest.approx(1)
    assert s.diagonal() == pytest.approx(1)
    assert s.trace() == pytest.approx(1)


@pytest.mark.parametrize('dims', [[2] * 9, [3, 2, 2]])
def test_kat_create(dims):
    target = [d * d for d in dims]
    data = np.random.random_sample(target)
    bases = [B.general(d) for d in dims]
    for expansion in (None, data):
        s = GB(bases, expansion)
        assert s.n_qubits == len(dims)
        assert s.dim_hilbert == tuple(dims)
        assert s.dim_pauli == tuple(target)
        assert s.size == math.prod(np.array(dims) ** 2)
        if expansion is not None:
            np.testing.assert_array_equal(s.to_pv(), expansion)
    wrong = math.prod(dims)
    with pytest.raises(ValueError):
        GB(bases, data.reshape(wrong, wrong))
    for shape in (target, (wrong, wrong)):
        with pytest.raises(ValueError):
            GB(bases=bases, pv=np.zeros(shape, dtype=complex))
    with pytest.raises(ValueError):
        GB(bases=[B.general(2)] * 16)


@pytest.mark.parametrize('bases', [
    (B.general(2),) * 3,
    (B.general(2).subbasis([0, 1, 2]), B.general(2).subbasis([0, 1]),
     B.general(2))])
def test_kat_create_from_dm(bases):
    dm = np.zeros((8, 8), dtype=complex)
    dm[0, 0], dm[1, 1] = 0.25, 0.75
    dm[0, 1], dm[1, 0] = 0.5 - 0.33j, 0.5 + 0.33j
    s = GB.from_dm(dm, bases)
    pv = s.to_pv()
    assert pv[0, 0, 0] == 0.25 and pv[0, 0, 1] == 0.75
    assert pv[0, 0, 2] == pytest.approx(0.5 * 2 ** 0.5)
    assert pv[0, 0, 3] == pytest.approx(0.33 * 2 ** 0.5)
    assert s.to_dm() == pytest.approx(dm)


def _reshuffled():
    g = B.general(2)
    order = (0, 2, 1, 3)
    return B.PauliBasis(np.array([g.vectors[i] for i in order]),
                        [g.labels[i] for i in order])


@pytest.mark.parametrize('bases', [
    (B.general(2),) * 3, (_reshuffled(),) * 3,
    (B.general(2), B.general(2).subbasis([0, 1]),
     B.general(2).subbasis([0, 1, 2]))])
def test_kat_diagonal_meas_prob(bases):
    diag = np.array([0.25, 0, 0.75, 0, 0, 0, 0, 0])
    s = GB.from_dm(np.diag(diag), bases)
    assert np.allclose(s.diagonal(), diag)
    assert s.trace() == pytest.approx(1)
    assert np.allclose(s.meas_prob(0), (1, 0))
    assert np.allclose(s.meas_prob(1), (0.25, 0.75))
    diag = np.array([0.25, 0.5, 0, 0, 0, 0, 0, 0])
    s = GB.from_dm(np.diag(diag), bases)
    assert np.allclose(s.diagonal(), diag)
    assert s.trace() == pytest.approx(0.75)
    assert np.allclose(s.meas_prob(0), (0.75, 0.))
    assert np.allclose(s.meas_prob(1), (0.75, 0.))
    assert np.allclose(s.meas_prob(2), (0.25, 0.5))


@pytest.mark.parametrize('dims', [(2, 2), (2, 3), (3, 3)])
def test_kat_default_diagonal(dims):
    s = GB([B.general(d) for d in dims])
    ref = np.zeros(dims[0] * dims[1])
    ref[0] = 1
    assert s.diagonal() == pytest.approx(ref)


def test_kat_apply_random_unitary_each_qubit():
    from scipy.stats import unitary_group
    rng = np.random.RandomState(45)
    b = (B.general(2),)
    for qubit in range(3):
        u = unitary_group.rvs(2, random_state=rng)
        a = rng.standard_normal((8, 8)) + 1j * rng.standard_normal((8, 8))
        dm = a @ a.conj().T
        dm /= np.trace(dm)
        ops3 = [np.eye(2)] * 3
        ops3[qubit] = u
        full = ops3[0]
        for m in ops3[1:]:
            full = np.kron(full, m)
        s0 = GB.from_dm(dm, b * 3)
        s1 = GB.from_dm(full @ dm @ full.conj().T, b * 3)
        s0.apply_ptm(P.kraus_to_ptm(u, b).numpy(), qubit)
        assert_close_f64(s0.to_pv(), s1.to_pv(), rtol=1e-12, atol=1e-13)


# ---------------------------------------------------------------- API
def test_errors_match_reference():
    s = GB([B.general(2)] * 3)
    with pytest.raises(ValueError):
        s.apply_ptm(np.eye(4), 0, 1)          # wrong PTM ndim
    with pytest.raises(ValueError):
        s.apply_ptm(np.eye(4), 3)             # qubit out of range
    with pytest.raises(ValueError):
        s.apply_ptm(np.eye(3), 0)             # dimension mismatch
    with pytest.raises(NotImplementedError):
        s.apply_ptm(np.ones((4,) * 6), 0, 1, 2)
    with pytest.raises(ValueError):
        s.meas_prob(5)
    with pytest.raises(ValueError):
        s.partial_trace(0, 7)


def test_renormalize_zero_trace_warns_and_project():
    s = GB([B.general(2)] * 2)
    s.project(0, 1)                          # |0><0| projected on 1: trace 0
    with pytest.warns(UserWarning):
        assert s.renormalize() == pytest.approx(0)
    s = GB([B.general(2)] * 2)
    s.apply_ptm(P.rotate('x', 1.1).numpy(), 1)
    p1 = s.meas_prob(1)[1]
    s.project(1, 1)
    assert s.dim_pauli == (4, 1)
    assert s.renormalize() == pytest.approx(p1, abs=1e-12)
    assert s.trace() == pytest.approx(1, abs=1e-12)


def test_copy_is_deep():
    s = GB([B.general(2)] * 2)
    c = s.copy()
    s.apply_ptm(P.rotate('y', 0.4).numpy(), 0)
    assert c.to_pv()[0, 0] == 1 and not np.allclose(c.to_pv(), s.to_pv())


def test_qutrit_circuit_with_measurement_matches_oracle():
    ops = workloads.config2_circuit(seed=2, n_qutrits=4, n_layers=6)
    s = GB([B.general(3)] * 4)
    o = O.PauliVectorOracle([B.general(3)] * 4)
    ts = workloads.run(s, ops)
    to = workloads.run(o, ops)
    assert ts == pytest.approx(to, abs=1e-12)
    assert_close_f64(s.to_pv(), o.to_pv())
    assert [b.dim_pauli for b in s.bases] == [b.dim_pauli for b in o.bases]


def test_float32_storage_probabilities():
    ops = workloads.config0_circuit(seed=4)
    s = GB([B.general(2)] * 6, dtype=np.float32)
    o = O.PauliVectorOracle([B.general(2)] * 6)
    workloads.run(s, ops)
    workloads.run(o, ops)
    assert s.to_pv().dtype == np.float32
    np.testing.assert_allclose(s.diagonal(), o.diagonal(), rtol=0, atol=1e-6)
    assert s.trace() == pytest.approx(o.trace(), abs=1e-6)


def _range_cases(rng):
    """(bases, ptm, qudits) covering every kernel form: group pairs, single
    groups (dense), vector accesses on the last qubit, staged qutrit tiles
    (9x9 and 81x81 on the last qutrits) and component order (81x81)."""
    t1, t2 = workloads.coherence_times(rng, 6)
    q2 = [B.general(2)] * 6
    q3 = [B.general(3)] * 4
    return [
        (q2, workloads.noisy_1q(rng, t1[0], t2[0]), (0,)),
        (q2, workloads.noisy_1q(rng, t1[5], t2[5]), (5,)),
        (q2, workloads.noisy_cz(rng, (1, 4), t1, t2), (1, 4)),
        (q2, workloads.noisy_cz(rng, (5, 4), t1, t2), (5, 4)),
        (q2, P.compose(P.cphase(0.7),
                       P.kron(P.rotate('x', 0.3), P.rotate('y', 1.1))).numpy(),
         (2, 3)),
        (q3, workloads.qutrit_1q(rng), (3,)),
        (q3, workloads.qutrit_2q(rng), (2, 3)),
        (q3, workloads.qutrit_2q(rng), (0, 2)),
    ]


@pytest.mark.parametrize("scale", [1e300, 1e-300, 1e-35, 1e-40])
def test_full_double_range_matches_oracle(scale):
    """States whose entries lie far outside the float-float range (near
    1e300, 1e-300, and just below the float pair's 2^-102 floor) give the
    oracle's result under arith='auto': the kernels recompute such items in
    native FP64 instead of failing.  Checked per entry at 1e-12 relative,
    with the absolute floor scaled with the state."""
    rng = np.random.default_rng(91)
    for bases, ptm, qs in _range_cases(rng):
        shape = tuple(b.dim_pauli for b in bases)
        pv = rand_pv(rng, shape) * scale
        ref = O.apply_ptm(pv, ptm, *qs)
        for jit in (True, False):
            s = GB(bases, pv)
            s._data = torch.ops.qsgb.apply_ptm(
                s._data, torch.from_numpy(np.ascontiguousarray(ptm)),
                list(qs), L.ARITH_AUTO, 0, False, jit)
            np.testing.assert_allclose(s.to_pv(), ref, rtol=RTOL_F64,
                                       atol=ATOL_F64 * scale)


def test_mixed_magnitudes_in_one_group():
    """One group holding entries of 1e300, 1, 1e-300 and 0: the items that
    hold them run in FP64, every other item in float-float, and the whole
    result matches the oracle per entry.  The PTM's construction residue
    (entries at or below 2^-52 of the largest, which the kernels skip under
    arith='auto') is zeroed for both: next to a 1e300 input that residue
    would decide entries the test checks at 1e-12."""
    rng = np.random.default_rng(92)
    t1, t2 = workloads.coherence_times(rng, 5)
    ptm = workloads.noisy_cz(rng, (1, 3), t1, t2)
    ptm = np.where(np.abs(ptm) > np.abs(ptm).max() * 2.0 ** -52, ptm, 0.0)
    pv = rand_pv(rng, (4,) * 5)
    pv[0, 1, 0, 2, 0] = 1e300
    pv[0, 2, 0, 3, 0] = -3e-300
    pv[0, 3, 0, 1, 0] = 0.0
    pv[1, 0, 1, 1, 1] = 7e-310            # a subnormal double
    ref = O.apply_ptm(pv, ptm, 1, 3)
    s = GB([B.general(2)] * 5, pv)
    s.apply_ptm(ptm, 1, 3)
    got = s.to_pv()
    np.testing.assert_allclose(got, ref, rtol=RTOL_F64, atol=0)


@pytest.mark.parametrize('dtype', [torch.float64, torch.float32])
def test_take_axis_bit_exact_every_axis(dtype):
    """reduce_basis / project as a copy of rows: every axis of a mixed
    qutrit/qubit tensor (long rows in 16-byte units, short rows unit by
    unit), aligned and 4/8-byte-offset tensors, and -1 entries (zeros);
    bit-exact against numpy's take."""
    rng = np.random.default_rng(71)
    shape = (9, 3, 9, 4, 9, 9)
    host = rng.standard_normal(shape)
    for off in (0, 1):
        buf = torch.empty(int(np.prod(shape)) + 1, dtype=dtype,
                          device='cuda')
        x = buf[off:off + int(np.prod(shape))].view(shape)
        x.copy_(torch.from_numpy(host).to(dtype))
        ref_host = x.cpu().numpy()
        for axis, d in enumerate(shape):
            for idx in ([0, d // 2, d - 1], [d - 1], [-1, 1] if d > 1
                        else [0]):
                got = torch.ops.qsgb.take_axis(x, axis, idx).cpu().numpy()
                exp = np.take(ref_host, [max(i, 0) for i in idx], axis=axis)
                if -1 in idx:
                    sl = [slice(None)] * len(shape)
                    sl[axis] = [j for j, i in enumerate(idx) if i < 0]
                    exp[tuple(sl)] = 0
                np.testing.assert_array_equal(got, exp)


# ---------------------------------------------------------------- full size
def test_12_qubit_apply_matches_oracle():
    rng = np.random.default_rng(17)
    n = 12
    pv = rand_pv(rng, (4,) * n)
    s = GB([B.general(2)] * n, pv, force=True)
    ref = pv
    t1, t2 = workloads.coherence_times(rng, n)
    for qs in [(0,), (11,), (5,), (0, 11), (11, 0), (6, 7), (3, 9)]:
        ptm = (workloads.noisy_1q(rng, t1[qs[0]], t2[qs[0]]) if len(qs) == 1
               else workloads.noisy_cz(rng, qs, t1, t2))
        s.apply_ptm(ptm, *qs)
        ref = O.apply_ptm(ref, ptm, *qs)
    assert_close_f64(s.to_pv(), ref)


def test_14_qubit_properties():
    """At the full 14-qubit size: trace preservation of trace-preserving
    PTMs, marginals summing to the trace, partial trace keeping the trace,
    and linearity of apply_ptm."""
    rng = np.random.default_rng(18)
    n = 14
    s = GB([B.general(2)] * n, force=True)
    ops, keep = workloads.config1_circuit(seed=1, n_qubits=n, n_layers=2)
    workloads.run(s, ops)
    tr = s.trace()
    assert tr == pytest.approx(1.0, abs=1e-12)
    for q in (0, 7, 13):
        assert s.meas_prob(q).sum() == pytest.approx(tr, abs=1e-12)
    pt = s.partial_trace(*keep)
    assert pt.trace() == pytest.approx(tr, abs=1e-12)
    # linearity: P(a x) == a P(x) exactly for a power of two
    x = s.copy()
    x.apply_ptm(2.0 * np.eye(4), 3)
    ptm = workloads.noisy_cz(rng, (2, 9), *workloads.coherence_times(rng, n))
    x.apply_ptm(ptm, 2, 9)
    s.apply_ptm(ptm, 2, 9)
    a = x.data
    b = s.data
    assert torch.equal(a, 2 * b)


def test_diagonal_target_array_and_flatten():
    """The reference GPU backend's diagonal() keywords: an allocated target
    tensor receives the values, flatten=False shapes them as dim_hilbert."""
    rng = np.random.default_rng(61)
    bases = [B.general(2), B.general(3), B.general(2)]
    pv = rand_pv(rng, (4, 9, 4))
    s = GB(bases, pv)
    ref = O.diagonal(pv, bases)
    target = torch.zeros(40, dtype=torch.float64, device='cuda')
    d = s.diagonal(get_data=False, target_array=target)
    assert d.data_ptr() == target.data_ptr()
    np.testing.assert_allclose(target[:12].cpu().numpy(), ref, rtol=0,
                               atol=ATOL_PROB)
    shaped = s.diagonal(flatten=False)
    assert shaped.shape == (2, 3, 2)
    np.testing.assert_allclose(shaped.reshape(-1), ref, rtol=0,
                               atol=ATOL_PROB)
    with pytest.raises(ValueError):
        s.diagonal(target_array=torch.zeros(5, dtype=torch.float64,
                                            device='cuda'))


def test_exp_value_matches_reference_fixtures():
    """Pauli-string expectation values on the device against the
    reference's State.exp_value (full bases, reshuffled subbases, a circuit
    run from State's one-element starting bases, the starting state)."""
    from conftest import exp_value_cases
    for name, pv, bases, ops, vals in exp_value_cases():
        s = GB(bases, pv.copy())
        for op, v in zip(ops, vals):
            assert s.exp_value(op) == pytest.approx(float(v.real), abs=1e-13), \
                (name, op)


def test_exp_value_large_state_storage_types_and_errors():
    rng = np.random.default_rng(62)
    n = 10
    bases = [B.general(2)] * n
    pv = rand_pv(rng, (4,) * n)
    s = GB(bases, pv)
    s32 = GB(bases, pv.astype(np.float32), dtype=np.float32)
    for op in ['XYZIZYXIIZ', 'IIIIIIIIII', 'ZZZZZZZZZZ', 'xyzixyzixy']:
        ref = float(O.exp_value(pv, bases, op).real)
        assert s.exp_value(op) == pytest.approx(ref, rel=1e-12, abs=1e-13)
        ref32 = float(O.exp_value(pv.astype(np.float32).astype(np.float64),
                                  bases, op).real)
        assert s32.exp_value(op) == pytest.approx(ref32, rel=1e-6, abs=1e-7)
    with pytest.raises(ValueError, match='same length'):
        s.exp_value('XX')
    with pytest.raises(ValueError, match='only I, X'):
        s.exp_value('XXXXXXXXXA')
    with pytest.raises(NotImplementedError):
        s.exp_value(np.eye(2 ** n))


def test_compiled_entry_point_matches_ctypes_path():
    """apply_ptm through the CPython entry point (csrc/qsgb_pyapply.c) and
    through ctypes runs the same kernels: the same bits for one- and
    two-qudit, swapped, rectangular and qutrit PTMs in FP64 and FP32; and
    the entry point is the path in use wherever it was built."""
    from quantumsim_gb300 import ops
    if not ops._pyapply():
        pytest.skip('the CPython entry point is not built on this host')
    rng = np.random.default_rng(77)
    b2, b3 = B.general(2), B.general(3)
    cases = [([b2] * 6, rand_ptm(rng, (4, 4, 4, 4), 0.5), (1, 4)),
             ([b2] * 6, rand_ptm(rng, (4, 4, 4, 4), 0.5), (5, 2)),
             ([b2] * 6, rand_ptm(rng, (4, 4)), (5,)),
             ([b2] * 6, np.eye(4)[[0, 3]], (2,)),
             ([b3, b2, b3], rand_ptm(rng, (9, 9, 9, 9), 0.1), (2, 0))]
    for dtype in (np.float64, np.float32):
        for bases, ptm, qs in cases:
            pv = rand_pv(rng, tuple(b.dim_pauli for b in bases))
            outs = []
            for fast in (True, False):
                saved = ops._PYAPPLY
                ops._PYAPPLY = saved if fast else False
                try:
                    s = GB(bases, pv, dtype=dtype)
                    s.apply_ptm(ptm, *qs)
                    outs.append(s.to_pv())
                finally:
                    ops._PYAPPLY = saved
            np.testing.assert_array_equal(outs[0], outs[1])


@pytest.mark.parametrize('n', [6, 12, 13])
def test_fused_marginals_over_many_blocks(n):
    """trace and meas_prob through the fused kernel, which spreads diagonals
    of more than 512 entries per outcome over several blocks (the last block
    adds the partials in block order): against sums of the state's own
    diagonal on the host, on repeated calls (the block ticket is left at
    zero)."""
    rng = np.random.default_rng(n)
    s = GB([B.general(2)] * n, force=True)
    s._data.copy_(torch.rand_like(s._data))
    diag = s.diagonal().reshape((2,) * n)
    for _ in range(3):
        assert abs(s.trace() - diag.sum()) <= 1e-12 * diag.sum()
        for q in (0, n // 2, n - 1):
            ref = diag.sum(axis=tuple(a for a in range(n) if a != q))
            np.testing.assert_allclose(s.meas_prob(q), ref, rtol=1e-12,
                                       atol=0)


def test_ptm_layouts_converted_on_the_fast_path():
    """A non-contiguous or float32 numpy PTM takes the conversion path of the
    per-call entry point and gives the contiguous float64 PTM's bits."""
    rng = np.random.default_rng(78)
    bases = [B.general(2)] * 5
    pv = rand_pv(rng, (4,) * 5)
    ptm = rand_ptm(rng, (4, 4, 4, 4), 0.5)
    ref = GB(bases, pv)
    ref.apply_ptm(ptm, 3, 1)
    strided = np.asfortranarray(ptm)
    assert not strided.flags.c_contiguous
    for p in (strided, ptm.astype(np.float32).astype(np.float64)[::1],
              ptm[:, :, :, ::-1][:, :, :, ::-1]):
        s = GB(bases, pv)
        s.apply_ptm(p, 3, 1)
        np.testing.assert_array_equal(s.to_pv(), ref.to_pv()) if p is not \
            None and np.array_equal(p, ptm) else None
    p32 = ptm.astype(np.float32)
    s32 = GB(bases, pv)
    s32.apply_ptm(p32, 3, 1)
    r32 = GB(bases, pv)
    r32.apply_ptm(p32.astype(np.float64), 3, 1)
    np.testing.assert_array_equal(s32.to_pv(), r32.to_pv())


def test_device_ptms_on_fp32_vectors():
    """PTMs in device memory on FP32 vectors: the dense FP32 kernel (K <= 16,
    no term limit: max_terms 0 or the PTM's size) and the generic kernel
    (the 81 x 81 PTM),
    against the oracle at FP32 accuracy, forward and transposed, in both
    argument orders, one and two qudits, rectangular and qutrit PTMs."""
    rng = np.random.default_rng(79)
    cases = [((4,) * 6, (1, 4), (4, 4, 4, 4)),
             ((4,) * 6, (5, 2), (4, 4, 4, 4)),
             ((4,) * 6, (3,), (4, 4)),
             ((4,) * 6, (5,), (4, 4)),
             ((4, 4, 9, 4, 3), (2,), (9, 9)),
             ((9, 4, 9), (0, 2), (9, 9, 9, 9)),
             ((9, 4, 9), (1,), (2, 4))]
    for shape, qs, pshape in cases:
        x = rand_pv(rng, shape).astype(np.float32)
        ptm = rand_ptm(rng, pshape, 0.7)
        for tr in (False, True):
            if tr and pshape[:len(qs)] != pshape[len(qs):]:
                continue
            ref = (O.apply_ptm_transposed(x.astype(np.float64), ptm, *qs)
                   if tr else O.apply_ptm(x.astype(np.float64), ptm, *qs))
            scale = np.abs(ref).max()
            for max_terms in (0, ptm.size):
                y = torch.ops.qsgb.apply_ptm(
                    torch.from_numpy(x).cuda(), torch.from_numpy(ptm).cuda(),
                    list(qs), L.ARITH_F32, max_terms, tr)
                np.testing.assert_allclose(y.cpu().numpy(), ref, rtol=1e-5,
                                           atol=1e-5 * scale)


def test_small_device_ptms_fp64():
    """One-qubit PTMs in device memory on small FP64 vectors take the dense
    kernel in native FP64 (the same products and sums as numpy): per entry
    at 1e-12 against the oracle, forward and transposed, every position,
    including a qubit in a 3-element subbasis; a larger vector takes the
    generic kernel and agrees too."""
    rng = np.random.default_rng(80)
    for shape in ((4,) * 6, (4, 3, 4, 4), (4,) * 11):
        x = rand_pv(rng, shape)
        for q in range(len(shape)):
            d = shape[q]
            ptm = rand_ptm(rng, (d, d))
            for tr in (False, True):
                ref = (O.apply_ptm_transposed(x, ptm, q) if tr
                       else O.apply_ptm(x, ptm, q))
                y = torch.ops.qsgb.apply_ptm(
                    torch.from_numpy(x).cuda(), torch.from_numpy(ptm).cuda(),
                    [q], L.ARITH_AUTO, 0, tr).cpu().numpy()
                absref = (O.apply_ptm_transposed(np.abs(x), np.abs(ptm), q)
                          if tr else O.apply_ptm(np.abs(x), np.abs(ptm), q))
                assert_close_dot(y, ref, absref)


def test_state_buffers_swap_and_handed_out_tensors_stay():
    """apply_ptm writes each result into the buffer of two applications
    back (no new tensor per call, as the reference swaps two buffers):
    the chain of applications still matches the oracle bit for bit against
    fresh tensors, a tensor passed to the constructor or handed out by
    `data` is never written, and a shape change drops the spare buffer."""
    from quantumsim_gb300 import ops
    rng = np.random.default_rng(91)
    bases = [B.general(2)] * 6
    pv = rand_pv(rng, (4,) * 6)
    ptms = [(rand_ptm(rng, (4, 4, 4, 4), 0.5), (1, 4)),
            (rand_ptm(rng, (4, 4)), (5,)),
            (rand_ptm(rng, (4, 4, 4, 4), 0.5), (3, 0)),
            (rand_ptm(rng, (4, 4)), (2,)),
            (rand_ptm(rng, (4, 4, 4, 4), 0.5), (2, 5))]
    user = torch.from_numpy(pv).cuda()
    keep = user.clone()
    s = GB(bases, user)
    ref, absref = pv, np.abs(pv)
    ptrs = []
    for k, (ptm, qs) in enumerate(ptms):
        s.apply_ptm(ptm, *qs)
        ptrs.append(s._data.data_ptr())
        ref = O.apply_ptm(ref, ptm, *qs)
        absref = O.apply_ptm(absref, np.abs(ptm), *qs)
        assert_close_dot(s.to_pv(), ref, absref,
                         rtol=chain_rtol(ptms[:k + 1]))
    assert torch.equal(user, keep)
    if ops._pyapply():
        # from the third application on, the results alternate between two
        # buffers
        assert ptrs[2] == ptrs[0] and ptrs[3] == ptrs[1] and \
            ptrs[4] == ptrs[2]
    # the same chain with a fresh tensor per call gives the same bits
    fresh = GB(bases, pv)
    for ptm, qs in ptms:
        fresh.apply_ptm(ptm, *qs)
        fresh._owned = False
    np.testing.assert_array_equal(fresh.to_pv(), s.to_pv())
    # a handed-out tensor keeps its values through later applications
    out = s.data
    snap = out.clone()
    for ptm, qs in ptms:
        s.apply_ptm(ptm, *qs)
    assert torch.equal(out, snap)
    # a rectangular PTM changes the shape; the spare buffer goes
    s.apply_ptm(np.eye(4)[[0, 3]], 2)
    s.apply_ptm(rand_ptm(rng, (4, 4)), 1)
    assert s._work is None or tuple(s._work.shape) == tuple(s._data.shape)

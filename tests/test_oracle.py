"""The CPU oracle pinned against the reference (golden fixtures generated by
running quantumsim's PauliVectorNumpy) and against the known-answer values
of the reference's own backend tests (test/test_pauli_vectors.py)."""
import math

import numpy as np
import pytest

from conftest import assert_close_f64, golden_bases, golden_cases
from oracle import pauli_vector_np as O
from oracle import ref_gpu
from quantumsim_gb300 import bases as B
from quantumsim_gb300 import ptm as P
from quantumsim_gb300 import workloads


def test_oracle_matches_reference_fixtures(golden):
    n = 0
    for i, case in enumerate(golden_cases(golden)):
        bases = golden_bases(golden, case['bases'])
        pv = golden['c{}_in'.format(i)]
        kind = case['kind']
        if kind == 'apply':
            out = O.apply_ptm(pv, golden['c{}_ptm'.format(i)], *case['qubits'])
            assert_close_f64(out, golden['c{}_out'.format(i)], rtol=1e-13,
                             atol=1e-15)
        elif kind == 'reduce':
            assert_close_f64(O.diagonal(pv, bases), golden['c{}_diag'.format(i)])
            assert O.trace(pv, bases) == pytest.approx(
                float(golden['c{}_trace'.format(i)]), abs=1e-14)
            for q in range(len(bases)):
                assert_close_f64(O.meas_prob(pv, bases, q),
                                 golden['c{}_prob{}'.format(i, q)])
            pv2, tr = O.renormalize(pv, bases)
            assert tr == pytest.approx(float(golden['c{}_renorm_trace'
                                                    .format(i)]), abs=1e-14)
            assert_close_f64(pv2, golden['c{}_renorm_pv'.format(i)])
        elif kind == 'partial_trace':
            out, obases = O.partial_trace(pv, bases, *case['keep'])
            assert_close_f64(out, golden['c{}_out'.format(i)])
            assert [b.dim_pauli for b in obases] == [
                bases[q].dim_pauli for q in case['keep']]
        elif kind == 'reduce_basis':
            out = O.reduce_basis(pv, case['qubit'], case['indices'])
            np.testing.assert_array_equal(out, golden['c{}_out'.format(i)])
        else:
            raise AssertionError(kind)
        n += 1
    assert n >= 40


def test_oracle_circuit0_matches_reference(golden):
    ops = workloads.config0_circuit(seed=0)
    assert len(ops) == int(golden['circuit0_nops'])
    bases = [B.general(2)] * 6
    pv = O.initial_pv(bases)
    for _, ptm, qs in ops:
        pv = O.apply_ptm(pv, ptm, *qs)
    assert_close_f64(pv, golden['circuit0_pv'], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(O.diagonal(pv, bases), golden['circuit0_diag'],
                               rtol=0, atol=1e-12)


@pytest.mark.parametrize('name,build', [
    ('rx_0.7', lambda: P.rotate('x', 0.7)),
    ('ry_2.1', lambda: P.rotate('y', 2.1)),
    ('rz_-1.3', lambda: P.rotate('z', -1.3)),
    ('apd_0.01_0.03', lambda: P.amp_phase_damping(0.01, 0.03)),
    ('cz_3.0', lambda: P.cphase(3.0)),
    ('noisy_cz', lambda: P.compose(P.cphase(math.pi), P.kron(
        P.amp_phase_damping(0.002, 0.003), P.amp_phase_damping(0.001, 0.004)))),
    ('q3_rx_0.7', lambda: P.rotate('x', 0.7, B.general(3))),
    ('q3_ry_1.9', lambda: P.rotate('y', 1.9, B.general(3))),
    ('q3_damp', lambda: P.qutrit_amp_damping(0.01, 0.002, 0.03, 0.04)),
    ('q3_cz', lambda: P.qutrit_cphase(math.pi + 0.013, 0.004)),
])
def test_ptm_builder_matches_reference_gates(golden, name, build):
    np.testing.assert_allclose(build().numpy(), golden['gate_' + name],
                               rtol=0, atol=1e-14)


def test_bases_match_reference_fixture_bases(golden):
    seen = {tuple(np.asarray(golden['basis{}_labels'.format(i)]))
            for i in range(64) if 'basis{}_labels'.format(i) in golden}
    g2 = tuple(B.general(2).labels)
    g3 = tuple(B.general(3).labels)
    assert g2 in seen and g3 in seen
    for i in range(64):
        key = 'basis{}_vectors'.format(i)
        if key not in golden:
            break
        v = golden[key]
        for cand in (B.general(2), B.general(3), B.gell_mann(2),
                     B.gell_mann(3)):
            if cand.vectors.shape == v.shape and np.allclose(cand.vectors, v):
                assert tuple(cand.labels) == tuple(
                    golden['basis{}_labels'.format(i)]) or \
                    cand in (B.gell_mann(2), B.gell_mann(3))


# ---- known answers of the reference's backend tests -----------------------
def _oracle_from_dm(dm, bases):
    return O.PauliVectorOracle.from_dm(dm, bases)


@pytest.mark.parametrize('bases', [
    (B.general(2),) * 3,
    (B.general(2).subbasis([0, 1, 2]), B.general(2).subbasis([0, 1]),
     B.general(2))])
def test_kat_create_from_dm(bases):
    dm = np.zeros((8, 8), dtype=complex)
    dm[0, 0], dm[1, 1] = 0.25, 0.75
    dm[0, 1], dm[1, 0] = 0.5 - 0.33j, 0.5 + 0.33j
    pv = _oracle_from_dm(dm, bases).to_pv()
    assert pv.shape == tuple(b.dim_pauli for b in bases)
    assert pv[0, 0, 0] == 0.25 and pv[0, 0, 1] == 0.75
    assert pv[0, 0, 2] == pytest.approx(0.5 * 2 ** 0.5)
    assert pv[0, 0, 3] == pytest.approx(0.33 * 2 ** 0.5)


def _reshuffled():
    g = B.general(2)
    order = (0, 2, 1, 3)
    return B.PauliBasis(np.array([g.vectors[i] for i in order]),
                        [g.labels[i] for i in order])


KAT_DIAG_BASES = [
    (B.general(2),) * 3,
    (_reshuffled(),) * 3,
    (B.general(2), B.general(2).subbasis([0, 1]),
     B.general(2).subbasis([0, 1, 2]))]


@pytest.mark.parametrize('bases', KAT_DIAG_BASES)
def test_kat_diagonal_meas_prob(bases):
    diag = np.array([0.25, 0, 0.75, 0, 0, 0, 0, 0])
    s = _oracle_from_dm(np.diag(diag), bases)
    assert np.allclose(s.diagonal(), diag)
    assert s.trace() == pytest.approx(1)
    assert np.allclose(s.meas_prob(0), (1, 0))
    assert np.allclose(s.meas_prob(1), (0.25, 0.75))
    diag = np.array([0.25, 0.5, 0, 0, 0, 0, 0, 0])
    s = _oracle_from_dm(np.diag(diag), bases)
    assert np.allclose(s.diagonal(), diag)
    assert s.trace() == pytest.approx(0.75)
    assert np.allclose(s.meas_prob(0), (0.75, 0.))
    assert np.allclose(s.meas_prob(1), (0.75, 0.))
    assert np.allclose(s.meas_prob(2), (0.25, 0.5))


@pytest.mark.parametrize('dims', [(2, 2), (2, 3), (3, 3)])
def test_kat_default_diagonal(dims):
    s = O.PauliVectorOracle([B.general(d) for d in dims])
    ref = np.zeros(dims[0] * dims[1])
    ref[0] = 1
    assert np.allclose(s.diagonal(), ref)


@pytest.mark.parametrize('bases', [
    (B.general(2),) * 3, (_reshuffled(),) * 3,
    (B.general(2).subbasis([0, 1]), B.general(2).subbasis([0, 1, 2]),
     B.general(2).subbasis([0, 1]))])
def test_kat_diagonal_indicated(bases):
    dm = np.array([[min(i, j) * 10 + max(i, j) for i in range(1, 9)]
                   for j in range(1, 9)])
    s = _oracle_from_dm(dm, bases)
    assert np.allclose(s.diagonal(), np.diag(dm))


def test_oracle_adjoint_and_grad_are_consistent():
    """<g, P x> == <P^T g, x> and d<g, P x>/dP == ptm_grad(x, g)."""
    rng = np.random.default_rng(5)
    x = rng.standard_normal((4, 3, 4, 9))
    ptm = rng.standard_normal((2, 4, 4, 4))  # qudits (2, 0): out (2, 4)
    y = O.apply_ptm(x, ptm, 2, 0)
    g = rng.standard_normal(y.shape)
    lhs = np.sum(g * y)
    rhs = np.sum(O.apply_ptm_transposed(g, ptm, 2, 0) * x)
    assert lhs == pytest.approx(rhs, rel=1e-12)
    grad = O.ptm_grad(x, g, 2, 0)
    assert grad.shape == ptm.shape
    assert np.sum(grad * ptm) == pytest.approx(lhs, rel=1e-12)


def test_workloads_are_deterministic():
    a = workloads.config0_circuit(seed=3)
    b = workloads.config0_circuit(seed=3)
    assert len(a) == len(b) == 20 * (6 + 3)
    for (_, pa, qa), (_, pb, qb) in zip(a, b):
        assert qa == qb
        np.testing.assert_array_equal(pa, pb)
    ops, keep = workloads.config1_circuit(seed=1, n_qubits=8, n_layers=2)
    assert len(keep) == 4 and list(keep) == sorted(keep)
    assert len(ops) == 2 * (8 + 7)
    c2 = workloads.config2_circuit(seed=2, n_qutrits=4, n_layers=4)
    kinds = [op[0] for op in c2]
    assert kinds.count('project') == 2 and kinds.count('renormalize') == 1


def test_oracle_runs_qutrit_circuit_trace_one():
    ops = workloads.config2_circuit(seed=2, n_qutrits=4, n_layers=6)
    pv = O.PauliVectorOracle([B.general(3)] * 4)
    traces = workloads.run(pv, ops)
    assert len(traces) == 1 and 0 < traces[0] <= 1
    assert pv.trace() == pytest.approx(1.0, abs=1e-12)


def test_reference_geometry_has_no_partial_blocks_for_qubits():
    """Host-side check of the launch rule: for qubit states every block of
    the reference's launch lies inside the output (no early-returning
    threads before its barrier)."""
    for n in range(2, 15):
        shape = (4,) * n
        for qs in [(0,), (n - 1,), (0, n - 1), (n - 1, 0)] + \
                ([(1, 2)] if n > 2 else []):
            pshape = (4, 4) if len(qs) == 1 else (4, 4, 4, 4)
            _, dims, grid, block, _, _ = ref_gpu.geometry(shape, pshape, qs)
            assert dims[-1] % (block[0] * block[1] * block[2]) == 0
            assert grid * block[0] * block[1] * block[2] == dims[-1]


def test_fused_model_layers_equal_unfused_on_host():
    """The differentiable model with each CZ absorbing its qubits' rotations
    gives the same probabilities and parameter gradients as unit by unit
    (float64 torch.einsum backend on the host)."""
    import torch
    from quantumsim_gb300 import fitting
    m = fitting.NoisyCircuitModel(n_qubits=5, n_layers=6, n_groups=3, seed=4)
    target = m.probabilities(m.perturbed(), backend='einsum').detach()
    res = {}
    for fuse in (False, True):
        p = m.params()
        loss = m.loss(p, target, backend='einsum', fuse=fuse)
        loss.backward()
        res[fuse] = (float(loss.detach()), torch.cat([p[k].grad.reshape(-1)
                                             for k in m.init]))
    assert res[True][0] == pytest.approx(res[False][0], rel=1e-12)
    np.testing.assert_allclose(res[True][1], res[False][1], rtol=1e-9,
                               atol=1e-14)


def test_oracle_exp_value_matches_reference_fixtures():
    """The oracle's Pauli-string expectation values against
    State.exp_value of the reference (quantumsim/states/state.py:43-83)."""
    from conftest import exp_value_cases
    for name, pv, bases, ops, vals in exp_value_cases():
        for op, v in zip(ops, vals):
            np.testing.assert_allclose(O.exp_value(pv, bases, op), v,
                                       rtol=0, atol=1e-14, err_msg=name)

"""Oracle parity at the sizes the benchmark runs the workloads at.

The seeded workload generators (quantumsim_gb300.workloads) are run on the
GPU backend and on the CPU oracle (the numpy restatement of
PauliVectorNumpy, quantumsim/pauli_vectors/numpy.py:50-117) at full size:

* the qutrit leakage circuit in full: 8 qutrits (9^8 entries), 30 layers of
  9x9 and 81x81 PTMs, with the mid-circuit reduce_basis 9 -> 3, project
  and renormalize of two qutrits;
* the scaled qubit circuit at 14 qubits (4^14 entries, 2.15 GB) for two
  full layers (14 noisy rotations and 7 noisy CZs on random ordered pairs
  each), then the partial trace keeping the 4 seeded qubits;
* the same circuit's full 50 layers (1050 PTMs) at 12 qubits.

Each runs unit by unit (PauliVectorGB300.apply_ptm) and through the fused
executor.  Required agreement: 1e-12 relative per Pauli-vector entry with a
1e-14 absolute floor, and 1e-12 absolute on diagonals, marginals and traces
(for the qutrit circuit under arith='auto', the per-entry bar scaled by the
conditioning of its projection, as its test explains).
"""
import numpy as np
import pytest

from conftest import ATOL_F64, ATOL_PROB, RTOL_F64
from oracle import pauli_vector_np as O
import quantumsim_gb300 as qg
from quantumsim_gb300 import bases as B
from quantumsim_gb300 import circuit as C
from quantumsim_gb300 import workloads

pytestmark = pytest.mark.gpu


def _close(gpu, ref):
    np.testing.assert_allclose(gpu, ref, rtol=RTOL_F64, atol=ATOL_F64)


def _run_fused(pv, ops):
    """Apply `ops` with the PTM runs between non-PTM operations fused."""
    traces, run = [], []

    def flush():
        if run:
            C.FusedCircuit(run)(pv)
            run.clear()

    for op in ops:
        if op[0] == 'ptm':
            run.append((op[1], op[2]))
            continue
        flush()
        traces += workloads.run(pv, [op])
    flush()
    return traces


def _measurements_agree(gpu, ref, qudits):
    np.testing.assert_allclose(gpu.diagonal(), ref.diagonal(), rtol=0,
                               atol=ATOL_PROB)
    assert abs(gpu.trace() - ref.trace()) <= ATOL_PROB
    for q in qudits:
        np.testing.assert_allclose(gpu.meas_prob(q), ref.meas_prob(q),
                                   rtol=0, atol=ATOL_PROB)


@pytest.fixture(scope='module')
def qutrit_oracle():
    ops = workloads.config2_circuit(seed=2, n_qutrits=8, n_layers=30)
    ref = O.PauliVectorOracle([B.general(3)] * 8)
    traces = workloads.run(ref, ops)
    return ops, ref, traces


@pytest.mark.parametrize('arith,fused', [('f64', False), ('f64', True),
                                         ('auto', False), ('auto', True)])
def test_qutrit_8q_30_layers_with_measurement(qutrit_oracle, arith, fused):
    """Native FP64 meets the flat bar.  The float-float rows of
    arith='auto' carry 2^-48 per application where FP64 carries 2^-53, and
    this circuit multiplies every error made before its mid-circuit
    projection by 1/p on the surviving entries: the projected outcome has
    probability p = 0.0092 (the renormalisation trace), so 'auto' is held to
    the same bar scaled by 1/p."""
    ops, ref, ref_traces = qutrit_oracle
    s = qg.PauliVectorGB300([B.general(3)] * 8, force=True, arith=arith)
    traces = (_run_fused if fused else workloads.run)(s, ops)
    assert len(traces) == len(ref_traces) == 1
    assert abs(traces[0] - ref_traces[0]) <= ATOL_PROB
    assert [b.dim_pauli for b in s.bases] == [b.dim_pauli for b in ref.bases]
    amp = 1.0 if arith == 'f64' else 1.0 / ref_traces[0]
    np.testing.assert_allclose(s.to_pv(), ref.to_pv(), rtol=RTOL_F64 * amp,
                               atol=ATOL_F64 * amp)
    _measurements_agree(s, ref, (0, 3, 7))


@pytest.fixture(scope='module')
def qubit14_oracle():
    ops, keep = workloads.config1_circuit(seed=1, n_qubits=14, n_layers=2)
    ref = O.PauliVectorOracle([B.general(2)] * 14)
    workloads.run(ref, ops)
    return ops, keep, ref, ref.partial_trace(*keep)


@pytest.mark.parametrize('fused', [False, True])
def test_qubit_14q_two_layers_and_partial_trace(qubit14_oracle, fused):
    ops, keep, ref, ref_pt = qubit14_oracle
    assert len(ops) == 2 * (14 + 7)
    s = qg.PauliVectorGB300([B.general(2)] * 14, force=True)
    (_run_fused if fused else workloads.run)(s, ops)
    _close(s.to_pv(), ref.to_pv())
    pt = s.partial_trace(*keep)
    _close(pt.to_pv(), ref_pt.to_pv())
    np.testing.assert_allclose(pt.diagonal(), ref_pt.diagonal(), rtol=0,
                               atol=ATOL_PROB)
    _measurements_agree(s, ref, (0, keep[0], 13))


@pytest.fixture(scope='module')
def qubit12_oracle():
    ops, keep = workloads.config1_circuit(seed=1, n_qubits=12, n_layers=50)
    ref = O.PauliVectorOracle([B.general(2)] * 12)
    workloads.run(ref, ops)
    return ops, keep, ref, ref.partial_trace(*keep)


@pytest.mark.parametrize('fused', [False, True])
def test_qubit_12q_50_layers_and_partial_trace(qubit12_oracle, fused):
    ops, keep, ref, ref_pt = qubit12_oracle
    assert len(ops) == 50 * (12 + 7)
    s = qg.PauliVectorGB300([B.general(2)] * 12, force=True)
    (_run_fused if fused else workloads.run)(s, ops)
    _close(s.to_pv(), ref.to_pv())
    _close(s.partial_trace(*keep).to_pv(), ref_pt.to_pv())
    _measurements_agree(s, ref, (0, 6, 11))

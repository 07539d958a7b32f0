"""Fused circuits on the GPU: the fused PTMs applied by PauliVectorGB300 match
the oracle's unit-by-unit application (FP64, dot-product forward-error
bound), and the CUDA-graph replay gives the same bits as the eager fused
run on any input of the captured shape."""
import math

import numpy as np
import pytest
import torch

from conftest import ATOL_F64, assert_close_dot, chain_rtol
from oracle import pauli_vector_np as O
import quantumsim_gb300 as qg
from quantumsim_gb300 import bases as B
from quantumsim_gb300 import circuit as C
from quantumsim_gb300 import workloads

pytestmark = pytest.mark.gpu


def _seq(pv, units, absval=False):
    for ptm, qs in units:
        pv = O.apply_ptm(pv, np.abs(ptm) if absval else ptm, *qs)
    return pv


def test_fused_qubit_circuit_matches_oracle():
    rng = np.random.default_rng(11)
    units = [(p, qs) for _, p, qs in workloads.config1_circuit(
        seed=7, n_qubits=8, n_layers=5, n_2q=4)[0]]
    circ = C.FusedCircuit(units)
    assert circ.n_passes < circ.n_units
    pv0 = rng.standard_normal((4,) * 8) / 256
    s = qg.PauliVectorGB300([B.general(2)] * 8, pv0)
    circ(s)
    assert_close_dot(s.to_pv(), _seq(pv0, units),
                     _seq(np.abs(pv0), units, True), rtol=chain_rtol(units))


def test_fused_qutrit_circuit_matches_oracle():
    rng = np.random.default_rng(12)
    units = [(op[1], op[2]) for op in workloads.config2_circuit(
        seed=5, n_qutrits=4, n_layers=4) if op[0] == 'ptm']
    circ = C.FusedCircuit(units)
    pv0 = rng.standard_normal((9,) * 4) / 81
    s = qg.PauliVectorGB300([B.general(3)] * 4, pv0)
    circ(s)
    assert_close_dot(s.to_pv(), _seq(pv0, units),
                     _seq(np.abs(pv0), units, True), rtol=chain_rtol(units))


@pytest.mark.parametrize('dtype', [np.float64, np.float32])
def test_graph_replay_equals_eager(dtype):
    rng = np.random.default_rng(13)
    units = [(p, qs) for _, p, qs in workloads.config1_circuit(
        seed=8, n_qubits=6, n_layers=20, n_2q=3)[0]]
    circ = C.FusedCircuit(units)
    bases = [B.general(2)] * 6
    proto = qg.PauliVectorGB300(bases, dtype=dtype)
    graph = circ.capture(proto)
    for k in range(2):
        pv0 = rng.standard_normal((4,) * 6) / 64
        eager = qg.PauliVectorGB300(bases, pv0, dtype=dtype)
        circ(eager)
        replay = qg.PauliVectorGB300(bases, pv0, dtype=dtype)
        graph.run(replay)
        torch.cuda.synchronize()
        assert torch.equal(replay._data, eager._data)
        if dtype == np.float64:
            assert_close_dot(replay.to_pv(), _seq(pv0, units),
                             _seq(np.abs(pv0), units, True),
                             rtol=chain_rtol(units))
    with pytest.raises(ValueError):
        graph.run(qg.PauliVectorGB300([B.general(2)] * 5, dtype=dtype))


def test_reference_operations_fused_on_gpu():
    """Units extracted from quantumsim operations (golden fixtures: an
    uncompiled chain, the chain on permuted qubits, compiled, compiled into
    reduced bases, and a FinalizedCircuit applied to a State with `@`, whose
    qubits start in one-element subbases) run fused on the GPU and reproduce
    the reference's output."""
    import json
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), 'golden',
                             'circuit_golden.npz'))
    meta = json.loads(str(d['meta']))
    for i, m in enumerate(meta):
        units = [(d['c{}_u{}'.format(i, j)], tuple(qs))
                 for j, qs in enumerate(m['unit_qudits'])]
        x_in, x_out = d['c{}_in'.format(i)], d['c{}_out'.format(i)]
        bases = [B.general(2) if d == 4 else B.general(2).subbasis([0])
                 for d in m['dims_in']]
        for fuse in (False, True):
            s = qg.PauliVectorGB300(bases, x_in)
            C.FusedCircuit(units, fuse=fuse)(s)
            assert list(s._data.shape) == m['dims_out']
            # absolute floor as in the golden checks: the kernels drop PTM
            # entries below 2^-52 of the largest (the ~1e-17 residue of the
            # complex arithmetic that built them), which leaves entries made
            # only of such residue at 0 instead of ~1e-17
            assert_close_dot(s.to_pv(), x_out,
                             _seq(np.abs(x_in), units, True),
                             rtol=chain_rtol(units), atol=ATOL_F64)


def test_parallel_preparation_then_apply():
    """Kernels compiled ahead of time on several host threads
    (FusedCircuit.prepare -> qsgb_prepare_ptm2) serve the applications:
    results equal the unfused oracle, for FP64 and FP32 vectors."""
    rng = np.random.default_rng(14)
    units = [(p, qs) for _, p, qs in workloads.config1_circuit(
        seed=21, n_qubits=7, n_layers=4, n_2q=3)[0]]
    circ = C.FusedCircuit(units)
    for dtype in (torch.float64, torch.float32):
        circ.prepare((4,) * 7, dtype, 0, threads=8)
        pv0 = rng.standard_normal((4,) * 7) / 128
        s = qg.PauliVectorGB300([B.general(2)] * 7, pv0,
                                dtype=np.float64 if dtype == torch.float64
                                else np.float32)
        circ(s)
        ref = _seq(pv0, units)
        if dtype == torch.float64:
            assert_close_dot(s.to_pv(), ref, _seq(np.abs(pv0), units, True),
                             rtol=chain_rtol(units))
        else:
            np.testing.assert_allclose(s.to_pv(), ref, rtol=0,
                                       atol=1e-5 * np.abs(ref).max())

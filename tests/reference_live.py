"""The reference's own call path driving PauliVectorGB300, compared with the
reference's PauliVectorNumpy on the same calls.

Run by tests/test_gpu_reference_live.py in a child process whose path puts
the reference package (and the stand-ins for its optional imports) ahead of
this repository, as a quantumsim user would have it: quantumsim_gb300 then
subclasses the reference's own PauliVectorBase and registers itself into
quantumsim.pauli_vectors.  Each scenario runs once per backend through
reference objects only:

* ``FinalizedCircuit @ State(..., pauli_vector_class=...)``
  (quantumsim/circuits/circuit.py:456-471, quantumsim/states/state.py:20-35):
  qubits start in the one-element subbasis of |0><0|, so the first units
  expand bases; then State.trace, State.partial_trace, State.exp_value and
  the backend's diagonal and meas_prob;
* the same for qutrits (``State(..., dim=3)``) with the reference's qutrit
  gates, a leakage CZ and an amplitude-damping channel;
* ``Operation.from_kraus(U)`` applied with ``op(pv, *qubits)``
  (PTMOperation.__call__, quantumsim/operations/operation.py:529-551) on
  mixed-dimension vectors at every qudit and every ordered pair, and the
  known-answer state of the reference's backend tests
  (test/test_pauli_vectors.py: full, reshuffled and mixed subbases);
* a chain compiled by the reference's compiler into reduced bases
  (quantumsim/operations/compiler.py) and applied to both backends.

Prints one line per scenario and 'all scenarios agree' at the end; any
disagreement raises (non-zero exit).
"""
import sys
import warnings

import numpy as np

warnings.simplefilter('ignore')

import quantumsim  # noqa: E402
import quantumsim.bases as qb  # noqa: E402
from quantumsim.circuits import Gate  # noqa: E402
from quantumsim.operations import Operation  # noqa: E402
from quantumsim.operations import qubits as lib2  # noqa: E402
from quantumsim.operations import qutrits as lib3  # noqa: E402
from quantumsim.pauli_vectors.numpy import PauliVectorNumpy  # noqa: E402
from quantumsim.pauli_vectors.pauli_vector import PauliVectorBase  # noqa: E402
from quantumsim.states import State  # noqa: E402
from scipy.stats import unitary_group  # noqa: E402

import quantumsim_gb300 as qg  # noqa: E402

GB = qg.PauliVectorGB300
RTOL, ATOL, ATOL_PROB = 1e-12, 1e-14, 1e-12


def close(a, b, what, atol=ATOL, rtol=RTOL):
    a, b = np.asarray(a), np.asarray(b)
    if a.shape != b.shape:
        raise AssertionError('{}: shape {} != {}'.format(what, a.shape,
                                                         b.shape))
    np.testing.assert_allclose(a, b, rtol=rtol, atol=atol, err_msg=what)


def same_states(gpu, ref, what):
    close(gpu.to_pv(), ref.to_pv(), what + ' pv')
    assert [b.dim_pauli for b in gpu.bases] == \
        [b.dim_pauli for b in ref.bases], what + ' bases'
    close(gpu.diagonal(), ref.diagonal(), what + ' diagonal', atol=ATOL_PROB,
          rtol=0)
    close(gpu.trace(), ref.trace(), what + ' trace', atol=ATOL_PROB, rtol=0)
    for q in range(ref.n_qubits):
        close(gpu.meas_prob(q), ref.meas_prob(q), what + ' meas_prob',
              atol=ATOL_PROB, rtol=0)


def circuit_at_state():
    circ = (Gate('Q0', 2, lib2.rotate_x(0.7))
            + Gate('Q1', 2, lib2.rotate_y(1.3))
            + Gate(('Q0', 'Q1'), 2, lib2.cphase(np.pi))
            + Gate('Q2', 2, lib2.hadamard())
            + Gate(('Q1', 'Q2'), 2, lib2.cphase(2.1))
            + Gate(('Q3', 'Q0'), 2, lib2.cnot())
            + Gate('Q3', 2, lib2.rotate_z(0.4))
            + Gate('Q0', 2, lib2.amp_phase_damping(0.02, 0.01))
            + Gate('Q2', 2, lib2.depolarization(0.03)))
    fc = circ.finalize()
    states = {}
    for cls in (PauliVectorNumpy, GB):
        st = State(['Q2', 'Q0', 'Q3', 'Q1'], pauli_vector_class=cls)
        fc @ st
        states[cls] = st
    ref, gpu = states[PauliVectorNumpy], states[GB]
    assert isinstance(gpu.pauli_vector, GB)
    same_states(gpu.pauli_vector, ref.pauli_vector, 'circuit @ State')
    close(gpu.trace(), ref.trace(), 'State.trace', atol=ATOL_PROB, rtol=0)
    pg, pr = gpu.partial_trace('Q1', 'Q3'), ref.partial_trace('Q1', 'Q3')
    assert isinstance(pg.pauli_vector, GB)
    same_states(pg.pauli_vector, pr.pauli_vector, 'State.partial_trace')
    for op in ('ZZII', 'XIYZ', 'IIIZ'):
        close(gpu.exp_value(op), ref.exp_value(op), 'exp_value ' + op,
              atol=ATOL_PROB, rtol=0)
    print('FinalizedCircuit @ State: 4 qubits, {} units'.format(
        len(list(fc.operation.units()))))


def qutrit_circuit_at_state():
    circ = (Gate('A', 3, lib3.rotate_x(0.9))
            + Gate('B', 3, lib3.rotate_y(2.2))
            + Gate(('A', 'B'), 3, lib3.cphase(np.pi, leakage_rate=0.05))
            + Gate('C', 3, lib3.hadamard())
            + Gate(('B', 'C'), 3, lib3.cphase(1.7, model='NetZero',
                                              leakage_rate=0.01))
            + Gate('A', 3, lib3.amp_damping(0.0, 0.01, 0.02, 0.04)))
    fc = circ.finalize()
    states = {}
    for cls in (PauliVectorNumpy, GB):
        st = State(['C', 'A', 'B'], dim=3, pauli_vector_class=cls)
        fc @ st
        states[cls] = st
    same_states(states[GB].pauli_vector, states[PauliVectorNumpy].pauli_vector,
                'qutrit circuit @ State')
    print('FinalizedCircuit @ State: 3 qutrits')


def random_density_matrix(dim, rng):
    vs = rng.standard_normal((dim, dim)) + 1j * rng.standard_normal((dim, dim))
    w = rng.random(dim)
    dm = sum(wk * np.outer(v, v.conj()) / np.vdot(v, v)
             for wk, v in zip(w / w.sum(), vs))
    return dm


def kraus_operations_everywhere():
    """One-qudit units on every qudit and two-qudit units on every ordered
    pair of equal dimension (the reference builds two-qudit PTMs for one
    dimension), on vectors of mixed qutrit / qubit dimensions."""
    rng = np.random.default_rng(5)
    b2, b3 = qb.general(2), qb.general(3)
    n_cases = 0
    for dims in ([3, 2, 2], [3, 3, 2]):
        bases = [b3 if d == 3 else b2 for d in dims]
        # the reference's dm_to_pv takes one dimension for all qudits:
        # seeded Pauli coefficients stand in for a density matrix
        shape = tuple(d * d for d in dims)
        pv0 = rng.standard_normal(shape) / np.sqrt(np.prod(shape))
        targets = [(q,) for q in range(3)] + [
            (q0, q1) for q0 in range(3) for q1 in range(3)
            if q0 != q1 and dims[q0] == dims[q1]]
        for qs in targets:
            d = int(np.prod([dims[q] for q in qs]))
            u = unitary_group.rvs(d, random_state=int(rng.integers(1 << 30)))
            decay = np.diag(np.linspace(1.0, 0.8, d))  # non-unitary
            op = Operation.from_kraus(decay @ u, [bases[q] for q in qs])
            pvs = {cls: cls(list(bases), pv0.copy())
                   for cls in (PauliVectorNumpy, GB)}
            for pv in pvs.values():
                op(pv, *qs)
            same_states(pvs[GB], pvs[PauliVectorNumpy],
                        'kraus on {} of {}'.format(qs, dims))
            n_cases += 1
    # the known-answer bases of the reference backend tests: full,
    # reshuffled and mixed subbases of general(2)
    for bs in ([b2, b2], [b2.subbasis([0, 1]), b2.subbasis([3, 0])],
               [b2.subbasis([1, 0, 3]), b2]):
        dm2 = random_density_matrix(4, rng)
        pvs = {cls: cls.from_dm(dm2, bs) for cls in (PauliVectorNumpy, GB)}
        same_states(pvs[GB], pvs[PauliVectorNumpy], 'subbases')
        n_cases += 1
    print('Operation.from_kraus applied with op(pv, *qubits): {} cases'
          .format(n_cases))


def compiled_into_reduced_bases():
    b = qb.general(2)
    chain = Operation.from_sequence(
        lib2.rotate_x(0.3).at(0), lib2.cphase(np.pi).at(0, 1),
        lib2.rotate_y(1.1).at(1), lib2.cnot().at(1, 2),
        lib2.amp_damping(0.05).at(2))
    bases_in = (b, b, b)
    bases_out = (b.computational_subbasis(),) * 3
    compiled = chain.compile(bases_in=bases_in, bases_out=bases_out)
    rng = np.random.default_rng(8)
    dm = random_density_matrix(8, rng)
    pvs = {cls: cls.from_dm(dm, list(bases_in))
           for cls in (PauliVectorNumpy, GB)}
    for pv in pvs.values():
        compiled(pv, 0, 1, 2)
    same_states(pvs[GB], pvs[PauliVectorNumpy], 'compiled chain')
    print('compiled chain into reduced bases: dims {}'.format(
        [bb.dim_pauli for bb in pvs[GB].bases]))
    # the same reduction done by this backend's planner on the uncompiled
    # chain (quantumsim_gb300.circuit.reduce_bases), fused, on the GPU
    from quantumsim_gb300.circuit import FusedCircuit
    fc = FusedCircuit.from_operation(chain, list(bases_in), 0, 1, 2,
                                     bases_out=list(bases_out))
    gpv = GB.from_dm(dm, list(bases_in))
    fc(gpv)
    same_states(gpv, pvs[PauliVectorNumpy], 'planner-reduced chain')
    print('planner-reduced fused chain: {} units in {} passes, dims {}'.format(
        fc.n_units, fc.n_passes, [bb.dim_pauli for bb in gpv.bases]))


def main():
    assert issubclass(GB, PauliVectorBase), 'not a reference subclass'
    assert quantumsim.pauli_vectors.PauliVectorGB300 is GB
    circuit_at_state()
    qutrit_circuit_at_state()
    kraus_operations_everywhere()
    compiled_into_reduced_bases()
    print('all scenarios agree')


if __name__ == '__main__':
    sys.exit(main())

"""Generate the golden fixtures of whole-operation runs (tests/golden/
circuit_golden.npz).

Builds operations with quantumsim's own gate library and ``Operation``
machinery (an uncompiled ``_Chain``, the same chain compiled for full
bases, one compiled into reduced bases, and a ``FinalizedCircuit`` of
``Gate``s applied to a ``State`` with ``@``), runs them on seeded Pauli
vectors with the reference's ``PauliVectorNumpy`` (``op(pv, *qubits)``:
quantumsim/operations/operation.py:529-551, 600-604), and stores, per case,
the input, the reference output, the bases' dimensions before and after,
and the (ptm, qudits) units that ``quantumsim_gb300.circuit.units_of``
extracts.
It needs the reference source tree (``$QUANTUMSIM_REF``, or
``../reference`` beside the checkout) and the stand-ins in ``tests/golden/_stubs``; the file
it writes is self-contained.

Usage:  python tests/golden/make_circuit_golden.py
"""
import json
import os
import sys
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle.refsrc import reference_tree  # noqa: E402
REF = reference_tree()
if REF is None:
    sys.exit('reference source tree not found: set $QUANTUMSIM_REF')
sys.path[:0] = [os.path.join(HERE, '_stubs'), REF]
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
warnings.simplefilter('ignore')

import quantumsim.bases as qb  # noqa: E402
from quantumsim.operations import qubits as lib  # noqa: E402
from quantumsim.operations.operation import Operation  # noqa: E402
from quantumsim.pauli_vectors.numpy import PauliVectorNumpy  # noqa: E402
from quantumsim.circuits import Gate  # noqa: E402
from quantumsim.states import State  # noqa: E402

from quantumsim_gb300.circuit import units_of  # noqa: E402

OUT = os.path.join(HERE, 'circuit_golden.npz')


def chain():
    return Operation.from_sequence(
        lib.rotate_x(0.3).at(0), lib.rotate_y(1.1).at(1),
        lib.cphase(np.pi).at(0, 1), lib.amp_phase_damping(0.01, 0.02).at(1),
        lib.rotate_z(0.7).at(2), lib.cphase(np.pi).at(1, 2),
        lib.rotate_x(0.5).at(2), lib.cphase(2.0).at(2, 0),
        lib.amp_phase_damping(0.03, 0.01).at(0))


def main():
    rng = np.random.default_rng(2024)
    g2 = qb.general(2)
    full = [g2] * 3
    cases = [
        ('chain', chain(), full, (0, 1, 2)),
        ('chain_on_2_0_1', chain(), full, (2, 0, 1)),
        ('compiled', chain().compile(bases_in=full), full, (0, 1, 2)),
        ('compiled_reduced', chain().compile(
            bases_in=full, bases_out=[g2.computational_subbasis()] * 3),
         full, (0, 1, 2)),
    ]
    arrays, meta = {}, []

    def record(name, op, pv, qubits, apply):
        i = len(meta)
        x_in = pv.to_pv().copy()
        dims_in = [b.dim_pauli for b in pv.bases]
        units, after = units_of(op, pv.bases, *qubits)
        apply()
        arrays['c{}_in'.format(i)] = x_in
        arrays['c{}_out'.format(i)] = pv.to_pv()
        for j, (ptm, qs) in enumerate(units):
            arrays['c{}_u{}'.format(i, j)] = ptm
        meta.append({'name': name, 'qubits': list(qubits),
                     'unit_qudits': [list(qs) for _, qs in units],
                     'dims_in': dims_in,
                     'dims_out': [b.dim_pauli for b in pv.bases],
                     'dims_after': [b.dim_pauli for b in after]})

    for name, op, bases, qubits in cases:
        # a random valid state: a mixture of random pure states, as a dm
        d = 2 ** 3
        vs = rng.standard_normal((3, d)) + 1j * rng.standard_normal((3, d))
        w = rng.random(3)
        dm = sum(wk * np.outer(v, v.conj()) / np.vdot(v, v)
                 for wk, v in zip(w / w.sum(), vs))
        pv = PauliVectorNumpy.from_dm(dm, bases)
        record(name, op, pv, qubits, lambda: op(pv, *qubits))

    # FinalizedCircuit @ State (quantumsim/circuits/circuit.py:456-471): the
    # state starts in the one-element subbasis of |0><0| on every qubit
    # (quantumsim/states/state.py:20-35), so the first units expand bases
    circ = (Gate('Q0', 2, lib.rotate_x(0.7)) + Gate('Q1', 2, lib.rotate_y(1.3))
            + Gate(('Q0', 'Q1'), 2, lib.cphase(np.pi))
            + Gate('Q2', 2, lib.hadamard())
            + Gate(('Q1', 'Q2'), 2, lib.cphase(2.1))
            + Gate('Q0', 2, lib.amp_phase_damping(0.02, 0.01)))
    fc = circ.finalize()
    state = State(['Q2', 'Q0', 'Q1'])
    indices = [state.qubits.index(q) for q in fc.qubits]
    record('finalized_circuit_at_state', fc.operation, state.pauli_vector,
           tuple(indices), lambda: fc @ state)
    arrays['meta'] = np.array(json.dumps(meta))
    np.savez_compressed(OUT, **arrays)
    print('wrote', OUT, len(meta), 'cases')


if __name__ == '__main__':
    main()

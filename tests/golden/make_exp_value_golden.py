"""Generate the golden fixtures of Pauli-string expectation values
(tests/golden/exp_value_golden.npz).

Runs the reference's ``State.exp_value`` (quantumsim/states/state.py:43-83)
on seeded states held in ``PauliVectorNumpy``: random mixed states in the
full qubit basis, a state in reshuffled subbases, and states a
``FinalizedCircuit`` produced from ``State``'s one-element starting bases.
Stores each state's Pauli vector, its bases (vectors and labels), the
operator strings and the reference's values.  It needs the
reference source tree (``$QUANTUMSIM_REF``, or ``../reference`` beside the checkout)
and the stand-ins in ``tests/golden/_stubs``; the file it writes is
self-contained.

Usage:  python tests/golden/make_exp_value_golden.py
"""
import contextlib
import io
import itertools
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
warnings.simplefilter('ignore')

import quantumsim.bases as qb  # noqa: E402
from quantumsim.circuits import Gate  # noqa: E402
from quantumsim.operations import qubits as lib  # noqa: E402
from quantumsim.pauli_vectors.numpy import PauliVectorNumpy  # noqa: E402
from quantumsim.states import State  # noqa: E402

OUT = os.path.join(HERE, 'exp_value_golden.npz')


def random_dm(rng, n):
    d = 2 ** n
    vs = rng.standard_normal((3, d)) + 1j * rng.standard_normal((3, d))
    w = rng.random(3)
    return sum(wk * np.outer(v, v.conj()) / np.vdot(v, v)
               for wk, v in zip(w / w.sum(), vs))


def exp_value(state, op):
    # State.exp_value prints its einsum arguments; keep them off the console
    with contextlib.redirect_stdout(io.StringIO()):
        return complex(state.exp_value(op))


def main():
    rng = np.random.default_rng(77)
    g2 = qb.general(2)
    cases = []
    # full bases, 3 and 4 qubits
    for n in (3, 4):
        pv = PauliVectorNumpy.from_dm(random_dm(rng, n), [g2] * n)
        cases.append(('full_%dq' % n, State(['Q%d' % i for i in range(n)],
                                              pauli_vector=pv)))
    # subbases in a shuffled order (the reference test's reshuffled basis)
    bases = [g2.subbasis([1, 0, 3, 2]), g2.subbasis([0, 1]),
             g2.subbasis([2, 3, 0, 1])]
    pv = PauliVectorNumpy.from_dm(random_dm(rng, 3), bases)
    cases.append(('subbases', State(['A', 'B', 'C'], pauli_vector=pv)))
    # a circuit applied to State's |0..0> in one-element subbases
    circ = (Gate('Q0', 2, lib.rotate_x(0.7)) + Gate('Q1', 2, lib.rotate_y(1.3))
            + Gate(('Q0', 'Q1'), 2, lib.cphase(np.pi))
            + Gate('Q2', 2, lib.hadamard())
            + Gate(('Q1', 'Q2'), 2, lib.cphase(2.1))
            + Gate('Q0', 2, lib.amp_phase_damping(0.02, 0.01)))
    state = State(['Q2', 'Q0', 'Q1'])
    circ.finalize() @ state
    cases.append(('circuit_state', state))
    # the untouched starting state: only |0><0| present on every qubit
    cases.append(('initial_state', State(['Q0', 'Q1'])))

    arrays, meta = {}, []
    for i, (name, st) in enumerate(cases):
        pvec = st.pauli_vector
        n = len(pvec.bases)
        ops = [''.join(p) for p in itertools.product('IXYZ', repeat=n)]
        if len(ops) > 40:
            ops = [ops[j] for j in rng.choice(len(ops), 40, replace=False)]
        ops += [ops[0].lower()]
        vals = np.array([exp_value(st, op) for op in ops])
        arrays['c%d_pv' % i] = pvec.to_pv()
        arrays['c%d_val' % i] = vals
        for q, b in enumerate(pvec.bases):
            arrays['c%d_b%d_vectors' % (i, q)] = b.vectors
        meta.append({'name': name, 'ops': ops,
                     'labels': [list(b.labels) for b in pvec.bases]})
    arrays['meta'] = np.array(json.dumps(meta))
    np.savez_compressed(OUT, **arrays)
    print('wrote', OUT, len(meta), 'cases')


if __name__ == '__main__':
    main()

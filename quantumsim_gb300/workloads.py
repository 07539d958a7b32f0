"""Seeded synthetic circuits: the benchmark and parity workloads.

A circuit is a list of operations applied in order to a Pauli vector:

* ``('ptm', ptm, qubits)``      -- ``pv.apply_ptm(ptm, *qubits)``
* ``('reduce_basis', q, idx)``  -- keep basis elements ``idx`` of qudit q
* ``('project', q, state)``     -- project qudit q on a computational state
* ``('renormalize',)``

All randomness comes from ``numpy.random.default_rng(seed)``; the same seed
gives the same PTMs (float64 numpy arrays) on every machine.

Noise model (per qubit, drawn once per circuit): T1 ~ U[20, 60] us,
T2 ~ U[10, T1] us; one-qubit gates last 20 ns, two-qubit gates 40 ns; see
:mod:`quantumsim_gb300.ptm` for the T1/T2 -> rate mapping.
"""
import math

import numpy as np

from . import bases as _bases
from . import ptm as P

T_1Q = 20e-9
T_2Q = 40e-9
AXES = ('x', 'y', 'z')


def coherence_times(rng, n):
    t1 = rng.uniform(20e-6, 60e-6, n)
    t2 = rng.uniform(10e-6, t1)
    return t1, t2


def noisy_1q(rng, t1, t2):
    axis = AXES[rng.integers(3)]
    angle = rng.uniform(0, 2 * math.pi)
    return P.noisy_rotation(axis, angle, t1, t2, T_1Q).numpy()


def line_matching(rng, n):
    """Pairs (i, i+1) of a perfect (n even) or maximal matching of a line,
    offset 0 or 1 at random, each pair in random orientation."""
    off = int(rng.integers(2)) if n % 2 else 0
    pairs = []
    for i in range(off, n - 1, 2):
        pairs.append((i, i + 1) if rng.integers(2) else (i + 1, i))
    return pairs


def config0_circuit(seed=0, n_qubits=6, n_layers=20):
    """Plain method, CPU-runnable: per layer a noisy rotation on every qubit,
    then ideal CZ (16x16) on a matching of line neighbours."""
    rng = np.random.default_rng(seed)
    t1, t2 = coherence_times(rng, n_qubits)
    cz = P.cphase(math.pi).numpy()
    ops = []
    for _ in range(n_layers):
        for q in range(n_qubits):
            ops.append(('ptm', noisy_1q(rng, t1[q], t2[q]), (q,)))
        for pair in line_matching(rng, n_qubits):
            ops.append(('ptm', cz, pair))
    return ops


def random_pair(rng, n):
    a, b = rng.choice(n, size=2, replace=False)
    return int(a), int(b)


def noisy_cz(rng, pair, t1, t2):
    a, b = pair
    return P.noisy_cphase(math.pi, t1[a], t2[a], t1[b], t2[b], T_2Q).numpy()


def config1_layer(rng, n_qubits, t1, t2, n_2q):
    ops = []
    for q in range(n_qubits):
        ops.append(('ptm', noisy_1q(rng, t1[q], t2[q]), (q,)))
    for _ in range(n_2q):
        pair = random_pair(rng, n_qubits)
        ops.append(('ptm', noisy_cz(rng, pair, t1, t2), pair))
    return ops


def config1_circuit(seed=1, n_qubits=14, n_layers=50, n_2q=7):
    """Plain method, scaled: per layer a noisy rotation on every qubit and
    `n_2q` noisy CZs on uniformly random ordered pairs; the partial trace
    keeps 4 random qubits at the end (returned separately, sorted)."""
    rng = np.random.default_rng(seed)
    t1, t2 = coherence_times(rng, n_qubits)
    ops = []
    for _ in range(n_layers):
        ops += config1_layer(rng, n_qubits, t1, t2, n_2q)
    keep = tuple(sorted(int(q) for q in rng.choice(n_qubits, 4,
                                                    replace=False)))
    return ops, keep


def config1_2q_batch(seed, n_qubits=14, n_apps=7):
    """One step of the scaled benchmark: `n_apps` noisy CZ PTMs on uniformly
    random ordered qubit pairs (every stride class occurs over steps)."""
    rng = np.random.default_rng(seed)
    t1, t2 = coherence_times(rng, n_qubits)
    return [('ptm', noisy_cz(rng, p, t1, t2), p)
            for p in (random_pair(rng, n_qubits) for _ in range(n_apps))]


def qutrit_1q(rng):
    b3 = _bases.general(3)
    axis = AXES[rng.integers(2)]  # rotation in the 0-1 subspace (x or y)
    angle = rng.uniform(0, 2 * math.pi)
    leak = rng.uniform(1e-4, 1e-2)
    damp = rng.uniform(2e-4, 1e-3)
    rot = P.rotate(axis, angle, b3)
    noise = P.qutrit_amp_damping(0.0, leak, damp, 2 * damp, b3)
    return P.compose(rot, noise).numpy()


def qutrit_2q(rng):
    angle = math.pi + rng.normal(0, 0.02)
    leak = rng.uniform(1e-4, 1e-2)
    return P.qutrit_cphase(angle, leak).numpy()


def config2_circuit(seed=2, n_qutrits=8, n_layers=30):
    """Qutrit leakage model: per layer a 9x9 PTM on every qutrit and 81x81
    CZ-with-leakage PTMs on a line matching; after layer n_layers // 2 two
    qutrits are reduced to their computational subbasis (9 -> 3), projected
    onto a seeded outcome and the state renormalised."""
    rng = np.random.default_rng(seed)
    ops = []
    mid = n_layers // 2
    measured = sorted(int(q) for q in rng.choice(n_qutrits, 2, replace=False))
    outcomes = [int(rng.integers(2)) for _ in measured]
    b3 = _bases.general(3)
    comp = [b3.computational_basis_indices[i] for i in range(3)]
    for layer in range(n_layers):
        for q in range(n_qutrits):
            if layer > mid and q in measured:
                continue
            ops.append(('ptm', qutrit_1q(rng), (q,)))
        for pair in line_matching(rng, n_qutrits):
            if layer >= mid and (pair[0] in measured or pair[1] in measured):
                continue
            ops.append(('ptm', qutrit_2q(rng), pair))
        if layer == mid:
            for q, k in zip(measured, outcomes):
                ops.append(('reduce_basis', q, comp))
                ops.append(('project', q, k))
            ops.append(('renormalize',))
    return ops


def run(pv, ops):
    """Apply a circuit to a Pauli-vector object (any backend with the
    interface); returns the list of renormalisation traces."""
    traces = []
    for op in ops:
        kind = op[0]
        if kind == 'ptm':
            pv.apply_ptm(op[1], *op[2])
        elif kind == 'reduce_basis':
            pv.reduce_basis(op[1], op[2])
        elif kind == 'project':
            pv.project(op[1], op[2])
        elif kind == 'renormalize':
            traces.append(pv.renormalize())
        else:
            raise ValueError('unknown operation {!r}'.format(kind))
    return traces

"""CPU oracle of the density-matrix hot path -- TEST INFRASTRUCTURE ONLY.

A plain-numpy restatement of the reference backend ``PauliVectorNumpy``
(quantumsim/pauli_vectors/numpy.py), the oracle of the GB300
kernels: only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` may import it.  The product (``quantumsim_gb300``) never
calls it.

Parity is pinned: ``tests/golden/make_golden.py`` ran the reference
``PauliVectorNumpy`` itself on seeded cases and stored its outputs in
``tests/golden/*.npz``; ``tests/test_oracle.py`` checks every function here
against those fixtures and against the known-answer values of the
reference's own tests (test/test_pauli_vectors.py).

Each function names the reference lines it follows.  Arrays are C-order
tensors of shape ``dim_pauli`` (qudit 0 most significant); ``bases`` are
objects with ``vectors`` (d_pauli, d, d) and ``computational_basis_vectors``.
"""
import math
import warnings

import numpy as np


def initial_pv(bases):
    """|0...0>: coefficient 1 at index (0, ..., 0) (numpy.py:39-41)."""
    pv = np.zeros(tuple(b.dim_pauli for b in bases))
    pv[(0,) * len(bases)] = 1
    return pv


def apply_ptm(pv, ptm, *qubits):
    """out = einsum over the PTM's input axes (numpy.py:50-64)."""
    if ptm.ndim != 2 * len(qubits):
        raise ValueError('{}-qubit PTM must have {} dimensions, got {}'
                         .format(len(qubits), 2 * len(qubits), ptm.ndim))
    n = pv.ndim
    dm_in = list(range(n))
    ptm_in = list(qubits)
    ptm_out = list(range(n, n + len(qubits)))
    dm_out = list(dm_in)
    for i_in, i_out in zip(ptm_in, ptm_out):
        dm_out[i_in] = i_out
    return np.einsum(pv, dm_in, ptm, ptm_out + ptm_in, dm_out, optimize=True)


def diagonal(pv, bases):
    """DM diagonal, length prod(d_hilbert): contraction with each qudit's
    computational_basis_vectors (numpy.py:66-80)."""
    n = len(bases)
    args = [pv, list(range(n))]
    for i, b in enumerate(bases):
        args += [b.computational_basis_vectors, [i + n, i]]
    out = np.einsum(*args, list(range(n, 2 * n)), optimize=True).real
    return out.reshape(math.prod(b.dim_hilbert for b in bases))


def trace(pv, bases):
    """sum(diagonal) (numpy.py:82-84)."""
    return np.sum(diagonal(pv, bases))


def partial_trace(pv, bases, *qubits):
    """Keep `qubits`, trace the rest with weights tr(P_x) (numpy.py:86-95).
    Returns (data with kept axes in ascending order, bases in argument
    order) -- the reference's own convention."""
    n = len(bases)
    args = [pv, list(range(n))]
    for i, b in enumerate(bases):
        if i not in qubits:
            args += [b.vectors, [i, n + i, n + i]]
    out = np.einsum(*args, optimize=True).real
    return out, [bases[q] for q in qubits]


def meas_prob(pv, bases, qubit):
    """Marginal probabilities of `qubit` (numpy.py:97-107)."""
    n = len(bases)
    args = [pv, list(range(n))]
    for i, b in enumerate(bases):
        args += [b.vectors, [i, n + i, n + i]]
    args.append([n + qubit])
    return np.einsum(*args, optimize=True).real


def renormalize(pv, bases):
    """Scale to unit trace if trace > 1e-8, else warn; returns (pv, trace
    before scaling) (numpy.py:109-117)."""
    tr = trace(pv, bases)
    if tr > 1e-8:
        pv = pv * trace(pv, bases) ** -1
    else:
        warnings.warn('Density matrix trace is 0; likely your further '
                      'computation will fail. Have you projected DM on a '
                      'state with zero weight?')
    return pv, tr


PAULI = {
    'I': np.array([[1, 0], [0, 1]], dtype=complex),
    'X': np.array([[0, 1], [1, 0]], dtype=complex),
    'Y': np.array([[0, -1j], [1j, 0]], dtype=complex),
    'Z': np.array([[1, 0], [0, -1]], dtype=complex),
}


def exp_value(pv, bases, operator):
    """Expectation value of a Pauli string, one letter per qubit
    (quantumsim/states/state.py:43-83): the contraction of sigma_q[a, b],
    the Pauli vector and each basis' vectors[k, b, a].  Complex, as numpy's
    einsum of complex arrays returns it."""
    n = len(bases)
    args = []
    for i, ch in enumerate(operator):
        args += [PAULI[ch.upper()], [i, n + i]]
    args += [pv, [2 * n + i for i in range(n)]]
    for i, b in enumerate(bases):
        args += [b.vectors, [2 * n + i, n + i, i]]
    return np.einsum(*args, optimize=True)


def reduce_basis(pv, qubit, indices):
    """Basis reduction as the selection PTM eye(d)[indices] applied to
    `qubit` (quantumsim/operations/operation.py:549-551 with a rectangular
    PTM)."""
    sel = np.eye(pv.shape[qubit])[list(indices)]
    return apply_ptm(pv, sel, qubit)


def apply_ptm_transposed(g, ptm, *qubits):
    """Adjoint of apply_ptm w.r.t. the state: apply PTM^T (in <-> out)."""
    k = len(qubits)
    perm = list(range(k, 2 * k)) + list(range(k))
    return apply_ptm(g, np.transpose(ptm, perm), *qubits)


def ptm_grad(x_in, g_out, *qubits):
    """dL/dPTM[out..., in...] = sum over bystanders of g_out * x_in."""
    n = x_in.ndim
    k = len(qubits)
    x_idx = list(range(n))
    g_idx = list(range(n))
    out_axes = list(range(n, n + k))
    for q, o in zip(qubits, out_axes):
        g_idx[q] = o
    return np.einsum(g_out, g_idx, x_in, x_idx, out_axes + list(qubits),
                     optimize=True)


def dm_to_pv(dm, bases):
    """quantumsim/algebra/algebra.py:44-52."""
    n = len(bases)
    d = bases[0].dim_hilbert
    args = [np.asarray(dm).reshape((d,) * (2 * n)), list(range(2 * n))]
    for i, b in enumerate(bases):
        args += [b.vectors, [2 * n + i, n + i, i]]
    return np.einsum(*args, optimize=True).real


class PauliVectorOracle:
    """Object form of the functions above, with the backend interface, so
    that tests can run one body against the oracle and the GPU backend."""

    def __init__(self, bases, pv=None, **_):
        self.bases = list(bases)
        self._data = initial_pv(self.bases) if pv is None else \
            np.array(pv, dtype=np.float64)

    @classmethod
    def from_dm(cls, dm, bases):
        return cls(bases, dm_to_pv(dm, bases))

    @property
    def n_qubits(self):
        return len(self.bases)

    @property
    def dim_pauli(self):
        return tuple(b.dim_pauli for b in self.bases)

    @property
    def dim_hilbert(self):
        return tuple(b.dim_hilbert for b in self.bases)

    def to_pv(self):
        return self._data

    def apply_ptm(self, ptm, *qubits):
        self._data = apply_ptm(self._data, np.asarray(ptm), *qubits)

    def diagonal(self):
        return diagonal(self._data, self.bases)

    def trace(self):
        return trace(self._data, self.bases)

    def meas_prob(self, qubit):
        return meas_prob(self._data, self.bases, qubit)

    def partial_trace(self, *qubits):
        data, bases = partial_trace(self._data, self.bases, *qubits)
        return PauliVectorOracle(bases, data)

    def renormalize(self):
        self._data, tr = renormalize(self._data, self.bases)
        return tr

    def reduce_basis(self, qubit, indices):
        self._data = reduce_basis(self._data, qubit, indices)
        self.bases[qubit] = self.bases[qubit].subbasis(list(indices))

    def project(self, qubit, state):
        idx = self.bases[qubit].computational_basis_indices[state]
        self.reduce_basis(qubit, [idx])

    def copy(self):
        return PauliVectorOracle(self.bases, self._data.copy())

"""Pauli bases: the per-qudit metadata the backend reads.

A self-contained equivalent of ``quantumsim.bases`` (quantumsim/bases/
pauli_basis.py:9-120 and quantumsim/bases/library.py:11-105) so that the
backend, its tests and the benchmark run where the quantumsim package is not
installed.  The backend only reads ``vectors``, ``dim_hilbert``,
``dim_pauli`` and the hints below, so objects of the reference class work
interchangeably with these.

Conventions kept from the reference (they define the data layout):

* ``vectors[x]`` is the x-th basis element, a Hermitian d x d matrix; the
  basis is orthonormal under tr(A B^dagger).
* ``general(d)``: first the d projectors |i><i|, then for every i > j the pair
  (|i><j| + |j><i|)/sqrt(2) ("Xij") and i(|i><j| - |j><i|)/sqrt(2) ("Yij").
* ``computational_basis_vectors[i, x] = vectors[x, i, i]``;
  ``computational_basis_indices[i]`` is the x for which that row is a unit
  vector, else ``None``.
"""
import functools

import numpy as np

_SQRT_HALF = np.sqrt(0.5)


def _unit_index(row):
    """Index of the single non-zero of a row that sums to 1, else None."""
    if not np.allclose(np.sum(row), 1):
        return None
    nz = np.flatnonzero(np.round(row, 8))
    return int(nz[0]) if len(nz) == 1 else None


class PauliBasis:
    """An orthonormal basis of Hermitian d x d matrices."""

    def __init__(self, vectors, labels, superbasis=None):
        vectors = np.asarray(vectors)
        if vectors.ndim != 3 or vectors.shape[1] != vectors.shape[2]:
            raise ValueError('Pauli basis vectors must be square matrices, '
                             'got shape {}'.format(vectors.shape))
        self.vectors = vectors
        self.labels = labels
        self._superbasis = superbasis
        self.computational_basis_vectors = np.einsum('xii->ix', vectors)
        self.computational_basis_indices = {
            i: _unit_index(row)
            for i, row in enumerate(self.computational_basis_vectors)}
        traces = np.einsum('xii->x', vectors) / np.sqrt(self.dim_hilbert)
        self.trace_index = _unit_index(traces)

    @property
    def dim_hilbert(self):
        return self.vectors.shape[1]

    @property
    def dim_pauli(self):
        return self.vectors.shape[0]

    @property
    def superbasis(self):
        return self._superbasis or self

    def subbasis(self, indices):
        indices = list(indices)
        return PauliBasis(self.vectors[indices],
                          [self.labels[i] for i in indices], self)

    def computational_subbasis(self):
        return self.subbasis([x for x in self.computational_basis_indices
                              .values() if x is not None])

    def hilbert_to_pauli_vector(self, rho):
        return np.einsum('xab,ba->x', self.vectors, rho)

    def __eq__(self, other):
        return (hasattr(other, 'vectors') and
                self.vectors.shape == other.vectors.shape and
                np.allclose(self.vectors, other.vectors))

    def __hash__(self):
        return hash(np.ascontiguousarray(self.vectors).tobytes())

    def __repr__(self):
        return '<PauliBasis d_hilbert={}, d_pauli={}, {}>'.format(
            self.dim_hilbert, self.dim_pauli, ' '.join(map(str, self.labels)))


@functools.lru_cache(maxsize=64)
def general(dim_hilbert):
    """Projectors first, then X-like / Y-like pairs for every i > j."""
    d = dim_hilbert
    vecs = np.zeros((d * d, d, d), dtype=complex)
    labels = []
    for i in range(d):
        vecs[len(labels), i, i] = 1
        labels.append(str(i))
    for i in range(d):
        for j in range(i):
            n = len(labels)
            vecs[n, i, j] = vecs[n, j, i] = _SQRT_HALF
            labels.append('X{}{}'.format(i, j))
            vecs[n + 1, i, j] = 1j * _SQRT_HALF
            vecs[n + 1, j, i] = -1j * _SQRT_HALF
            labels.append('Y{}{}'.format(i, j))
    return PauliBasis(vecs, labels)


@functools.lru_cache(maxsize=64)
def gell_mann(dim_hilbert):
    """Generalised Gell-Mann matrices: identity/sqrt(d) and traceless ones."""
    d = dim_hilbert
    vecs = np.zeros((d * d, d, d), dtype=complex)
    labels = []
    for i in range(d):
        for j in range(d):
            m = vecs[len(labels)]
            if i == j:
                if i == 0:
                    diag = np.full(d, 1 / np.sqrt(d))
                else:
                    diag = np.zeros(d)
                    diag[:i] = 1
                    diag[i] = -i
                    diag /= np.sqrt(i * (i + 1))
                m[np.arange(d), np.arange(d)] = diag
            elif i < j:
                m[i, j] = m[j, i] = _SQRT_HALF
            else:
                m[i, j] = 1j * _SQRT_HALF
                m[j, i] = -1j * _SQRT_HALF
            labels.append('g{}{}'.format(i, j))
    return PauliBasis(vecs, labels)

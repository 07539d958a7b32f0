"""Stand-in for ``quantumsim.pauli_vectors.PauliVectorBase``.

The GB300 backend subclasses the reference's abstract base class
(quantumsim/pauli_vectors/pauli_vector.py:6-116) whenever the ``quantumsim``
package is importable.  Where it is not (e.g. a bare GPU host), this module
supplies an abstract class with the same constructor contract, size guard,
conversions, properties and validation helpers, so the backend keeps the same
surface and error behaviour.
"""
import abc
import math

import numpy as np


def dm_to_pv(dm, bases):
    """Expand a density matrix in the tensor-product Pauli basis (real part).

    Same contraction as quantumsim/algebra/algebra.py:44-52:
    pv[x_0..x_n-1] = Re tr(rho (P_x0 (x) ... (x) P_xn-1))."""
    n = len(bases)
    d = bases[0].dim_hilbert
    args = [np.asarray(dm).reshape((d,) * (2 * n)), list(range(2 * n))]
    for i, b in enumerate(bases):
        args += [b.vectors, [2 * n + i, n + i, i]]
    return np.einsum(*args, optimize=True).real


def pv_to_dm(pv, bases):
    """Inverse of :func:`dm_to_pv` (quantumsim/algebra/algebra.py:55-62)."""
    n = len(bases)
    d = bases[0].dim_hilbert
    args = [pv, list(range(2 * n, 3 * n))]
    for i, b in enumerate(bases):
        args += [b.vectors, [2 * n + i, i, n + i]]
    return np.einsum(*args, optimize=True).reshape((d ** n,) * 2)


class PauliVectorBase(metaclass=abc.ABCMeta):
    """Abstract density-matrix backend: same interface as the reference."""

    _size_max = 2 ** 22

    @abc.abstractmethod
    def __init__(self, bases, pv=None, *, force=False):
        self.bases = list(bases)
        if self.size > self._size_max and not force:
            raise ValueError(
                'Density matrix of the system is going to have {} items. It '
                'is probably too much. If you know what you are doing, pass '
                '`force=True` argument to the constructor.'.format(self.size))

    @classmethod
    def from_pv(cls, pv, bases, *, force=False):
        return cls(bases, pv, force=force)

    @classmethod
    def from_dm(cls, dm, bases, *, force=False):
        if not hasattr(bases, '__iter__'):
            n = len(dm) // bases.dim_hilbert
            bases = [bases] * n
        return cls(bases, dm_to_pv(dm, bases), force=force)

    @abc.abstractmethod
    def to_pv(self):
        pass

    def to_dm(self):
        return pv_to_dm(self.to_pv(), self.bases)

    @property
    def n_qubits(self):
        return len(self.bases)

    @property
    def dim_hilbert(self):
        return tuple(b.dim_hilbert for b in self.bases)

    @property
    def size(self):
        return math.prod(self.dim_hilbert) ** 2

    @property
    def dim_pauli(self):
        return tuple(b.dim_pauli for b in self.bases)

    @abc.abstractmethod
    def apply_ptm(self, operation, *qubits):
        pass

    @abc.abstractmethod
    def diagonal(self, *, get_data=True):
        pass

    @abc.abstractmethod
    def trace(self):
        pass

    @abc.abstractmethod
    def partial_trace(self, *qubits):
        pass

    @abc.abstractmethod
    def meas_prob(self, qubit):
        pass

    @abc.abstractmethod
    def renormalize(self):
        pass

    @abc.abstractmethod
    def copy(self):
        pass

    def _validate_qubit(self, number, name):
        if number < 0 or number >= self.n_qubits:
            raise ValueError(
                '`{}` number {} does not exist in the system, it contains {} '
                'qubits in total.'.format(name, number, self.n_qubits))

    def _validate_ptm_shape(self, ptm, target_shape, name):
        if ptm.shape != target_shape:
            raise ValueError('`{}` shape must be {}, got {}'.format(
                name, target_shape, ptm.shape))

"""GB300-native density-matrix backend for quantumsim.

``PauliVectorGB300`` is a drop-in ``PauliVectorBase`` backend whose hot path
(PTM application, diagonal / marginals / trace, partial trace, basis
reduction, renormalisation) runs in hand-written sm_103a CUDA kernels behind
the C ABI of ``include/qsgb.h`` (``libqsgb.so``), called through the
``torch.ops.qsgb`` operators.
"""
from . import bases
from . import ptm
from ._lib import load as load_library
from .pauli_vector import PauliVectorGB300, register
from .autograd import ApplyPTM, apply_ptm_diff, diagonal_diff, checkpointed
from .batch import BatchedSimulator
from .circuit import FusedCircuit, units_of

__all__ = ['PauliVectorGB300', 'register', 'bases', 'ptm', 'load_library',
           'ApplyPTM', 'apply_ptm_diff', 'diagonal_diff', 'checkpointed',
           'BatchedSimulator', 'FusedCircuit', 'units_of']

register()

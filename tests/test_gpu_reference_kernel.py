"""The reference's own GPU kernel (quantumsim/pauli_vectors/primitives.cu,
compiled unchanged for sm_103a into oracle/_ref) as a second oracle: on the
same inputs it agrees with the GB300 kernels and with the oracle, for
one-qubit PTMs at every position and two-qubit PTMs on every ordered pair
(the reference's transposition for qubit0 > qubit1 included)."""
import itertools
import math

import numpy as np
import pytest
import torch

from conftest import assert_close_dot
from oracle import pauli_vector_np as O
from oracle import ref_gpu
import quantumsim_gb300  # noqa: F401  (registers the torch.ops.qsgb operators)

pytestmark = pytest.mark.gpu


def _need_cubin():
    if not ref_gpu.available():
        pytest.skip('oracle/_ref/primitives_sm103a.cubin not built (the '
                    'reference source tree was absent when building)')


def test_reference_kernel_one_qubit_every_position():
    _need_cubin()
    rng = np.random.default_rng(41)
    n = 6
    x = rng.standard_normal((4,) * n) / 64
    xt = torch.from_numpy(x).cuda()
    for q in range(n):
        ptm = rng.standard_normal((4, 4))
        ref = ref_gpu.apply(xt, ptm, (q,))
        ours = torch.ops.qsgb.apply_ptm(xt, torch.from_numpy(ptm), [q], 0, 0,
                                        False)
        torch.cuda.synchronize()
        absref = O.apply_ptm(np.abs(x), np.abs(ptm), q)
        assert_close_dot(ref.cpu().numpy(), O.apply_ptm(x, ptm, q), absref)
        assert_close_dot(ours.cpu().numpy(), ref.cpu().numpy(), absref)


def test_reference_kernel_two_qubits_every_ordered_pair():
    _need_cubin()
    rng = np.random.default_rng(42)
    n = 5
    x = rng.standard_normal((4,) * n) / 32
    xt = torch.from_numpy(x).cuda()
    for q0, q1 in itertools.permutations(range(n), 2):
        ptm = rng.standard_normal((4, 4, 4, 4)) * \
            (rng.random((4, 4, 4, 4)) < 0.5)
        ref = ref_gpu.apply(xt, ptm, (q0, q1))
        ours = torch.ops.qsgb.apply_ptm(xt, torch.from_numpy(ptm), [q0, q1],
                                        0, 0, False)
        torch.cuda.synchronize()
        absref = O.apply_ptm(np.abs(x), np.abs(ptm), q0, q1)
        assert_close_dot(ref.cpu().numpy(), O.apply_ptm(x, ptm, q0, q1),
                         absref)
        assert_close_dot(ours.cpu().numpy(), ref.cpu().numpy(), absref)

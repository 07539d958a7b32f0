"""The largest states: 16 qubits in FP64, 4^16 = 4.29e9 entries (34 GB), past
2^32 entries.  The oracle cannot run at this size, so parity is checked on
properties that do not depend on it: every output group sampled at random
against the PTM product of its own input group (host FP64), the diagonal
against the state's own entries, and a partial trace against a torch
reduction of the same tensor."""
import math

import numpy as np
import pytest
import torch

import quantumsim_gb300 as qg
from quantumsim_gb300 import bases as B
from quantumsim_gb300 import workloads

pytestmark = pytest.mark.gpu

N = 16
BYTES = 8 * 4 ** N


def _free_bytes():
    free, _ = torch.cuda.mem_get_info()
    return free


@pytest.fixture(scope='module')
def state():
    if _free_bytes() < 4 * BYTES:
        pytest.skip('needs {:.0f} GB of free device memory'.format(
            4 * BYTES / 1e9))
    g = torch.Generator(device='cuda').manual_seed(5)
    x = torch.randn((4,) * N, dtype=torch.float64, device='cuda',
                    generator=g) / math.sqrt(4.0 ** N)
    yield x
    del x
    torch.cuda.empty_cache()


def _sample_groups(rng, qs, count=256):
    """Random bystander indices (full index tuples with the targets' axes
    set to slice(None))."""
    out = []
    for _ in range(count):
        idx = [int(v) for v in rng.integers(4, size=N)]
        for q in qs:
            idx[q] = slice(None)
        out.append(tuple(idx))
    return out


@pytest.mark.parametrize('qs', [(0,), (7,), (15,), (0, 15), (15, 0), (7, 8),
                                (14, 15)])
def test_apply_ptm_past_2_32_entries(state, qs):
    rng = np.random.default_rng(sum(qs) + 10 * len(qs))
    t1, t2 = workloads.coherence_times(rng, N)
    if len(qs) == 1:
        ptm = workloads.noisy_1q(rng, t1[qs[0]], t2[qs[0]])
    else:
        ptm = workloads.noisy_cz(rng, qs, t1, t2)
    pv = qg.PauliVectorGB300([B.general(2)] * N, state, force=True)
    pv.apply_ptm(ptm, *qs)
    out = pv._data
    assert out.data_ptr() != state.data_ptr()
    for idx in _sample_groups(rng, qs):
        x_in = state[idx].cpu().numpy()
        y = out[idx].cpu().numpy()
        if len(qs) == 1:
            ref = ptm @ x_in
            absref = np.abs(ptm) @ np.abs(x_in)
        else:
            # x_in axes follow ascending qubit order; the PTM is in argument
            # order (q0, q1)
            xi = x_in if qs[0] < qs[1] else x_in.T
            ref = np.einsum('abcd,cd->ab', ptm, xi)
            absref = np.einsum('abcd,cd->ab', np.abs(ptm), np.abs(xi))
            if qs[0] > qs[1]:
                ref, absref = ref.T, absref.T
        assert np.all(np.abs(y - ref) <= 1e-12 * absref + 1e-300)
    del pv, out
    torch.cuda.empty_cache()


def test_diagonal_and_partial_trace_past_2_32_entries(state):
    pv = qg.PauliVectorGB300([B.general(2)] * N, state, force=True)
    diag = pv.diagonal(get_data=False)
    assert diag.numel() == 2 ** N
    rng = np.random.default_rng(3)
    b = B.general(2)
    comp = [b.computational_basis_indices[i] for i in range(2)]
    d = diag.cpu().numpy()
    for _ in range(512):
        bits = [int(v) for v in rng.integers(2, size=N)]
        flat = int(''.join(str(v) for v in bits), 2)
        entry = state[tuple(comp[v] for v in bits)].item()
        assert d[flat] == entry
    # partial trace keeping qubits 3 and 12, against a torch reduction
    w = torch.tensor(np.real(np.einsum('xkk->x', b.vectors)),
                     dtype=torch.float64, device='cuda')
    keep = (3, 12)
    ref = state
    for q in reversed(range(N)):
        if q not in keep:
            ref = torch.tensordot(ref, w, dims=([q], [0]))
    pt = pv.partial_trace(*keep).to_pv()
    ref = ref.cpu().numpy()
    np.testing.assert_allclose(pt, ref, rtol=1e-10,
                               atol=1e-12 * np.abs(ref).max())
    del pv, diag
    torch.cuda.empty_cache()

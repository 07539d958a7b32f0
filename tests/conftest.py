"""Shared pytest configuration: the `gpu` marker, golden fixtures, helpers."""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, 'tests', 'golden', 'pauli_vector_golden.npz')

# Agreement with float64 numpy required of the FP64 path (relative per
# entry, with an absolute floor for entries that cancel to ~0) and on
# probabilities (absolute).
RTOL_F64 = 1e-12
ATOL_F64 = 1e-14
ATOL_PROB = 1e-12


def pytest_configure(config):
    config.addinivalue_line(
        'markers', 'gpu: needs a CUDA device (GB300) and libqsgb.so')


def has_cuda():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope='session')
def golden():
    data = np.load(GOLDEN, allow_pickle=False)
    return data


EXP_GOLDEN = os.path.join(ROOT, 'tests', 'golden', 'exp_value_golden.npz')


def exp_value_cases():
    """(name, Pauli vector, bases, operator strings, reference values) of
    the State.exp_value fixtures."""
    from quantumsim_gb300.bases import PauliBasis
    data = np.load(EXP_GOLDEN, allow_pickle=False)
    out = []
    for i, c in enumerate(json.loads(str(data['meta']))):
        bases = [PauliBasis(data['c{}_b{}_vectors'.format(i, q)], labels)
                 for q, labels in enumerate(c['labels'])]
        out.append((c['name'], data['c{}_pv'.format(i)], bases, c['ops'],
                    data['c{}_val'.format(i)]))
    return out


def golden_cases(data):
    return json.loads(str(data['manifest']))


def golden_bases(data, ids):
    from quantumsim_gb300.bases import PauliBasis
    return [PauliBasis(data['basis{}_vectors'.format(i)],
                       list(data['basis{}_labels'.format(i)])) for i in ids]


def assert_close_dot(actual, expected, absref, rtol=RTOL_F64, atol=0.0):
    """Per-entry forward-error check of a contraction: |a - e| <= rtol *
    (sum_k |P_rk| |x_k|) + atol, the natural scale of a dot product whose
    terms may cancel (`absref` = the same contraction applied to |P| and
    |x|)."""
    actual, expected = np.asarray(actual), np.asarray(expected)
    bound = rtol * np.asarray(absref) + atol + 1e-300
    err = np.abs(actual - expected)
    worst = np.max(err / bound) if err.size else 0.0
    assert worst <= 1.0, 'max error / bound = {:.3g}'.format(worst)


def chain_rtol(units):
    """Relative forward-error bound, against the |P| chain applied to |x|,
    of applying `units` ((ptm, qudits) pairs) one after another, as the GPU
    does and as the oracle does.

    One application's row is a dot product of K = (PTM input size) terms.
    On the GPU each term is formed in float-float: the input truncated to 47
    significant bits, the PTM entry rounded to 48, the product error kept to
    48 bits, one two-sum per term, and the row rounded once to double, so
    the row's error is at most (K + 4) 2^-47 of sum_k |P_rk| |x_k|.  The
    oracle's FP64 dot product adds K 2^-53 of the same sum, and a fused PTM
    formed on the host in FP64 adds K 2^-53 of its |P| product.  An error
    made at one unit reaches the output through the later PTMs, where it is
    bounded by the |P| chain.  Summing over the units: sum_u (K_u + 4)
    2^-46 bounds the whole chain."""
    total = 0.0
    for ptm, qudits in units:
        k = int(np.prod(np.shape(ptm)[len(qudits):]))
        total += (k + 4) * 2.0 ** -46
    return total


def assert_close_f64(actual, expected, rtol=RTOL_F64, atol=ATOL_F64):
    np.testing.assert_allclose(np.asarray(actual), np.asarray(expected),
                               rtol=rtol, atol=atol)

"""Basis reduction of a unit list (quantumsim_gb300.circuit.reduce_bases),
the planner's counterpart of the reference compiler's optimal_bases
(quantumsim/operations/compiler.py:303-362), on the CPU oracle:

* random circuits of qubits and qutrits with sparse PTMs, some qudits read
  afterwards only in a subbasis: the reduced units give the kept entries of
  the unreduced result (to rounding) on smaller vectors;
* a state that starts in one-element bases (as a reference State does):
  only entries that stay exactly zero are dropped;
* the reference's own chain compiled into the computational subbasis
  (golden fixture made by running the reference's compiler): reducing the
  uncompiled chain's units for that output basis reproduces the
  reference's output."""
import json
import os

import numpy as np
import pytest

from oracle import pauli_vector_np as O
from quantumsim_gb300 import bases as B
from quantumsim_gb300 import circuit as C

HERE = os.path.dirname(os.path.abspath(__file__))


def _random_units(rng, dims, n_units, density):
    n = len(dims)
    units = []
    for _ in range(n_units):
        if rng.random() < 0.4 or n < 2:
            q = int(rng.integers(n))
            d = dims[q]
            p = rng.standard_normal((d, d)) * (rng.random((d, d)) < density)
            units.append((p, (q,)))
        else:
            a, b = (int(v) for v in rng.choice(n, 2, replace=False))
            da, db = dims[a], dims[b]
            p = rng.standard_normal((da, db, da, db))
            p *= rng.random(p.shape) < density / 2
            units.append((p, (a, b)))
    return units


def _run(x, units):
    for p, qs in units:
        x = O.apply_ptm(x, p, *qs)
    return x


@pytest.mark.parametrize('seed', range(6))
def test_kept_entries_match_the_unreduced_run(seed):
    rng = np.random.default_rng(seed)
    dims = [4, 9, 4, 4] if seed % 2 else [4, 4, 4, 4, 4]
    units = _random_units(rng, dims, 14, 0.5)
    x = rng.standard_normal(dims)
    ref = _run(x, units)
    keep_out = [None] * len(dims)
    for q in rng.choice(len(dims), 2, replace=False):
        keep_out[int(q)] = sorted(rng.choice(dims[q], 2, replace=False))
    red, kept = C.reduce_bases(units, dims, keep_out)
    y = _run(x, red)
    assert np.prod(y.shape) <= np.prod(ref.shape)
    idx = [k if k is not None else np.arange(d) for k, d in zip(kept, dims)]
    req = [np.asarray(k) if k is not None else np.arange(d)
           for k, d in zip(keep_out, dims)]
    # requested entries the reduction kept: the same values; requested
    # entries it dropped: identically zero in the unreduced run
    both = [np.intersect1d(i, r) for i, r in zip(idx, req)]
    pos = [np.searchsorted(i, b) for i, b in zip(idx, both)]
    np.testing.assert_allclose(y[np.ix_(*pos)], ref[np.ix_(*both)],
                               rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    sub = ref[np.ix_(*req)]
    mask = np.ones(sub.shape, dtype=bool)
    mask[np.ix_(*[np.searchsorted(r, b) for r, b in zip(req, both)])] = False
    assert np.all(sub[mask] == 0)


def test_one_element_start_drops_only_zeros():
    """Qubits start in the |0><0| element (dims 1, as a reference State):
    CZs and damping keep most entries at zero, so the vector stays small,
    and every dropped entry of the unreduced run is exactly zero."""
    rng = np.random.default_rng(9)
    g = B.general(2)
    zero = g.computational_basis_indices[0]
    # units_of-style PTMs: the first unit on each qubit takes its input in
    # the one-element basis (a column of the full PTM)
    cz = np.diag([1.0, 1.0, 1.0, 1.0] * 4).reshape(4, 4, 4, 4)
    units = [(cz[:, :, zero:zero + 1, zero:zero + 1], (0, 1)),
             (cz[:, :, :, zero:zero + 1], (1, 2))]
    x = np.ones((1, 1, 1))
    ref = _run(x, units)
    red, kept = C.reduce_bases(units, [1, 1, 1])
    y = _run(x, red)
    assert np.prod(y.shape) < np.prod(ref.shape)
    idx = [k if k is not None else np.arange(d)
           for k, d in zip(kept, ref.shape)]
    np.testing.assert_array_equal(y, ref[np.ix_(*idx)])
    mask = np.ones(ref.shape, dtype=bool)
    mask[np.ix_(*idx)] = False
    assert np.all(ref[mask] == 0)
    del rng


def test_reference_compiled_chain_into_the_computational_subbasis():
    d = np.load(os.path.join(HERE, 'golden', 'circuit_golden.npz'))
    meta = json.loads(str(d['meta']))
    names = [m['name'] for m in meta]
    i_chain = names.index('chain')
    i_red = names.index('compiled_reduced')
    m = meta[i_chain]
    units = [(d['c{}_u{}'.format(i_chain, j)], tuple(qs))
             for j, qs in enumerate(m['unit_qudits'])]
    g = B.general(2)
    comp = sorted(int(g.computational_basis_indices[i]) for i in range(2))
    red, kept = C.reduce_bases(units, m['dims_in'], [comp] * 3)
    x = d['c{}_in'.format(i_red)]
    y = _run(x, red)
    ref = d['c{}_out'.format(i_red)]
    assert meta[i_red]['dims_out'] == [2, 2, 2]
    assert [list(k) for k in kept] == [comp] * 3
    np.testing.assert_allclose(y, ref, rtol=1e-12, atol=1e-14)

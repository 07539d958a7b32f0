"""Fusion planning of circuits (host side, checked with the oracle): the fused
unit list applied by the oracle equals the unit-by-unit application, merges
happen where the rules allow them and never across a unit on the same
qudit or across a rectangular unit."""
import math

import numpy as np

from conftest import assert_close_dot, chain_rtol
from oracle import pauli_vector_np as O
from quantumsim_gb300 import circuit as C
from quantumsim_gb300 import workloads


def _apply_all(pv, units):
    for ptm, qs in units:
        pv = O.apply_ptm(pv, ptm, *qs)
    return pv


def _abs_all(pv, units):
    for ptm, qs in units:
        pv = O.apply_ptm(pv, np.abs(ptm), *qs)
    return pv


def _rand_pv(rng, shape):
    return rng.standard_normal(shape) / math.sqrt(np.prod(shape))


def test_fused_noisy_circuit_equals_unit_by_unit():
    rng = np.random.default_rng(1)
    units = [(p, qs) for _, p, qs in workloads.config1_circuit(
        seed=4, n_qubits=6, n_layers=6, n_2q=3)[0]]
    fused = C.plan(units)
    assert len(fused) < len(units)
    pv = _rand_pv(rng, (4,) * 6)
    # the fused products are formed in FP64: equal up to the rounding of a
    # chain of dot products
    assert_close_dot(_apply_all(pv, fused), _apply_all(pv, units),
                     _abs_all(np.abs(pv), units), rtol=chain_rtol(units))


def test_merge_rules():
    rng = np.random.default_rng(2)
    t1, t2 = workloads.coherence_times(rng, 4)
    r = [workloads.noisy_1q(rng, t1[q], t2[q]) for q in range(4)]
    cz01 = workloads.noisy_cz(rng, (0, 1), t1, t2)
    cz10 = workloads.noisy_cz(rng, (1, 0), t1, t2)
    cz12 = workloads.noisy_cz(rng, (1, 2), t1, t2)
    # 1q on 0 and 1 move into the CZ on (0, 1); the 1q on 3 stays
    f = C.plan([(r[0], (0,)), (r[1], (1,)), (r[3], (3,)), (cz01, (0, 1))])
    assert [qs for _, qs in f] == [(3,), (0, 1)]
    # a unit on qudit 1 in between blocks the 1q on 1 from reaching (0, 1)
    # from behind, but it merges into the CZ on (1, 2) it meets first
    f = C.plan([(r[1], (1,)), (cz12, (1, 2)), (cz01, (0, 1))])
    assert [qs for _, qs in f] == [(1, 2), (0, 1)]
    # two CZs on one pair (either order) become one two-qudit unit
    f = C.plan([(cz01, (0, 1)), (cz10, (1, 0))])
    assert [qs for _, qs in f] == [(1, 0)]
    # a later 1q unit joins the previous CZ on its qudit
    f = C.plan([(cz01, (0, 1)), (r[0], (0,))])
    assert [qs for _, qs in f] == [(0, 1)]
    # rectangular units are barriers: the projection on qudit 1 is kept and
    # nothing on qudit 1 merges across it
    proj = np.eye(4)[[0]]
    units = [(r[1], (1,)), (proj, (1,)), (r[0], (0,))]
    f = C.plan(units)
    assert [p.shape for p, _ in f] == [(4, 4), (1, 4), (4, 4)]
    pv = _rand_pv(rng, (4, 4, 4))
    assert_close_dot(_apply_all(pv, f), _apply_all(pv, units),
                     _abs_all(np.abs(pv), units) * 4)


def test_dense_units_are_not_merged_when_the_model_says_no():
    rng = np.random.default_rng(3)
    d1 = rng.standard_normal((16, 16)).reshape(4, 4, 4, 4)
    d2 = rng.standard_normal((16, 16)).reshape(4, 4, 4, 4)
    # two dense 16x16 passes cost as much as their (dense) product: kept
    # apart only if the product is not cheaper; the model compares
    # 16 + 16 terms per row against 16
    f = C.plan([(d1, (0, 1)), (d2, (0, 1))])
    assert len(f) == 1
    # a dense 1q unit into a sparse CZ: merged only while cheaper
    t1, t2 = workloads.coherence_times(rng, 2)
    cz = workloads.noisy_cz(rng, (0, 1), t1, t2)
    dense1 = rng.standard_normal((4, 4))
    f = C.plan([(dense1, (0,)), (dense1, (1,)), (cz, (0, 1))])
    costs = [C.pass_cost(p.reshape(int(math.isqrt(p.size)), -1))
             for p, _ in f]
    assert sum(costs) <= 3 * max(C.pass_cost(dense1), C.pass_cost(
        cz.reshape(16, 16))) + 1e-30


def test_qutrit_units_fuse():
    rng = np.random.default_rng(5)
    units = [(p, qs) for kind, p, qs in
             (op for op in workloads.config2_circuit(seed=3, n_qutrits=3,
                                                      n_layers=4)
              if op[0] == 'ptm')]
    fused = C.plan(units)
    assert len(fused) < len(units)
    pv = _rand_pv(rng, (9, 9, 9))
    assert_close_dot(_apply_all(pv, fused), _apply_all(pv, units),
                     _abs_all(np.abs(pv), units), rtol=chain_rtol(units))


# ------------------------------------------------ reference operation runs
def _golden_circuits():
    import json
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), 'golden',
                             'circuit_golden.npz'))
    meta = json.loads(str(d['meta']))
    out = []
    for i, m in enumerate(meta):
        units = [(d['c{}_u{}'.format(i, j)], tuple(qs))
                 for j, qs in enumerate(m['unit_qudits'])]
        out.append((m, d['c{}_in'.format(i)], d['c{}_out'.format(i)], units))
    return out


def test_reference_operation_runs_reproduced_by_units_and_fusion():
    """The units extracted from quantumsim operations (uncompiled chain, on
    permuted qubits, compiled, compiled into reduced bases), applied by the
    oracle one by one and fused, give the reference's own output."""
    for m, x_in, x_out, units in _golden_circuits():
        assert m['dims_after'] == m['dims_out']
        seq = _apply_all(x_in, units)
        np.testing.assert_allclose(seq, x_out, rtol=1e-12, atol=1e-14)
        fused = C.plan(units)
        assert len(fused) <= len(units)
        assert_close_dot(_apply_all(x_in, fused), x_out,
                         _abs_all(np.abs(x_in), units),
                         rtol=chain_rtol(units))


def test_units_of_matches_reference_when_available():
    """Re-extract the units from the reference's operations (only where the
    reference source tree is present) and compare with the fixture."""
    import os
    import sys
    import warnings
    from oracle.refsrc import reference_tree
    ref = reference_tree()
    if ref is None:
        import pytest
        pytest.skip('reference source tree not present')
    here = os.path.join(os.path.dirname(__file__), 'golden')
    sys.path[:0] = [os.path.join(here, '_stubs'), ref, here]
    warnings.simplefilter('ignore')
    try:
        import make_circuit_golden as G
        import quantumsim.bases as qb
        g2 = qb.general(2)
        full = [g2] * 3
        ops = {'chain': (G.chain(), (0, 1, 2)),
               'chain_on_2_0_1': (G.chain(), (2, 0, 1)),
               'compiled': (G.chain().compile(bases_in=full), (0, 1, 2))}
        for m, _, _, units in _golden_circuits():
            if m['name'] not in ops:
                continue
            op, qubits = ops[m['name']]
            got, after = C.units_of(op, full, *qubits)
            assert [qs for _, qs in got] == [qs for _, qs in units]
            for (a, _), (b, _) in zip(got, units):
                np.testing.assert_allclose(a, b, rtol=1e-13, atol=1e-15)
    finally:
        for p in (os.path.join(here, '_stubs'), ref, here):
            sys.path.remove(p)


def _random_units(rng):
    """A random unit list over 2-4 qudits of dims 4 (qubit, full basis) or 9
    (qutrit): sparse physical PTMs on single qudits and on ordered pairs,
    and now and then a rectangular basis reduction (a barrier that changes
    the qudit's dimension)."""
    n = int(rng.integers(2, 5))
    dims = [int(rng.choice([4, 4, 9])) for _ in range(n)]
    t1, t2 = workloads.coherence_times(rng, n)
    units = []
    for _ in range(int(rng.integers(3, 15))):
        u = rng.random()
        if u < 0.45:
            q = int(rng.integers(n))
            if dims[q] == 4:
                units.append((workloads.noisy_1q(rng, t1[q], t2[q]), (q,)))
            elif dims[q] == 9:
                units.append((workloads.qutrit_1q(rng), (q,)))
            else:
                units.append((rng.standard_normal((dims[q], dims[q])), (q,)))
        elif u < 0.9:
            a, b = (int(v) for v in rng.choice(n, 2, replace=False))
            if dims[a] == dims[b] == 4:
                ptm = workloads.noisy_cz(rng, (a, b), t1, t2)
            elif dims[a] == dims[b] == 9:
                ptm = workloads.qutrit_2q(rng)
            else:
                ptm = rng.standard_normal((dims[a], dims[b], dims[a], dims[b]))
                ptm *= rng.random(ptm.shape) < 0.15
            units.append((ptm, (a, b)))
        else:
            q = int(rng.integers(n))
            keep = sorted(int(v) for v in rng.choice(
                dims[q], int(rng.integers(1, dims[q])), replace=False))
            units.append((np.eye(dims[q])[keep], (q,)))
            dims[q] = len(keep)
    return units, n


def test_plan_random_unit_sequences():
    """Random unit lists: the fused plan applied by the oracle equals the
    units applied one by one (rectangular units act as barriers)."""
    for seed in range(24):
        rng = np.random.default_rng(300 + seed)
        units, n = _random_units(rng)
        shape = []
        for q in range(n):
            first = [u for u in units if q in u[1]]
            d = 4
            if first:
                ptm, qs = first[0]
                d = ptm.shape[len(qs) + qs.index(q)]
            shape.append(d)
        pv = _rand_pv(rng, tuple(shape))
        fused = C.plan(units)
        assert len(fused) <= len(units)
        assert_close_dot(_apply_all(pv, fused), _apply_all(pv, units),
                         _abs_all(np.abs(pv), units) * 16 + 1e-300)


def test_both_planners_on_random_sequences():
    """The greedy planner and the assignment search each give a correct
    plan on their own (plan() returns whichever the model prefers)."""
    for seed in range(12):
        rng = np.random.default_rng(500 + seed)
        units, n = _random_units(rng)
        shape = []
        for q in range(n):
            first = [u for u in units if q in u[1]]
            d = 4
            if first:
                ptm, qs = first[0]
                d = ptm.shape[len(qs) + qs.index(q)]
            shape.append(d)
        pv = _rand_pv(rng, tuple(shape))
        ref = _apply_all(pv, units)
        bound = _abs_all(np.abs(pv), units) * 16 + 1e-300
        for planner in (C._plan_greedy, C._plan_assigned):
            fused = planner(units)
            assert len(fused) <= len(units)
            assert_close_dot(_apply_all(pv, fused), ref, bound)


def test_assignment_search_on_the_noisy_circuit():
    """Noisy rotations and CZs on random pairs (the 14-qubit circuit's
    structure at 6 qubits): the assignment plan is correct, and on the
    14-qubit circuit itself its modelled time is below the greedy plan's
    with no more passes."""
    rng = np.random.default_rng(7)
    units = [(p, qs) for _, p, qs in workloads.config1_circuit(
        seed=5, n_qubits=6, n_layers=8, n_2q=3)[0]]
    fused = C._plan_assigned(units)
    assert len(fused) < len(units)
    pv = _rand_pv(rng, (4,) * 6)
    assert_close_dot(_apply_all(pv, fused), _apply_all(pv, units),
                     _abs_all(np.abs(pv), units), rtol=chain_rtol(units))
    big = [(p, qs) for _, p, qs in workloads.config1_circuit(seed=1)[0]]
    g, a = C._plan_greedy(big), C._plan_assigned(big)
    assert len(a) <= len(g)
    assert C.plan_cost(a) < 0.95 * C.plan_cost(g)
    assert C.plan_cost(C.plan(big)) == C.plan_cost(a)


def test_runs_join_the_cheaper_neighbour():
    """A rotation between two CZs on its qubit joins one of them (not
    both, not neither), and a second run on the qudit (one whose product
    with the first the model rejects) is left for the unit after it."""
    rng = np.random.default_rng(8)
    t1, t2 = workloads.coherence_times(rng, 2)
    cz = workloads.noisy_cz(rng, (0, 1), t1, t2)
    r = workloads.noisy_1q(rng, t1[0], t2[0])
    f = C._plan_assigned([(cz, (0, 1)), (r, (0,)), (cz, (0, 1))])
    assert [qs for _, qs in f] in ([(0, 1)], [(0, 1), (0, 1)])
    assert all(len(qs) == 2 for _, qs in f)


def test_assignment_search_respects_barriers():
    """A rectangular unit on a qudit is a barrier for the assignment search
    too: the rotation before the projection stays on its side of it, and
    the fused list applied by the oracle equals the units one by one."""
    rng = np.random.default_rng(12)
    t1, t2 = workloads.coherence_times(rng, 3)
    r1 = workloads.noisy_1q(rng, t1[1], t2[1])
    r0 = workloads.noisy_1q(rng, t1[0], t2[0])
    cz = workloads.noisy_cz(rng, (0, 1), t1, t2)
    proj = np.eye(4)[[0, 3]]
    units = [(cz, (0, 1)), (r1, (1,)), (proj, (1,)), (r0, (0,)),
             (workloads.noisy_cz(rng, (0, 2), t1, t2), (0, 2))]
    fused = C._plan_assigned(units)
    shapes = [(p.shape, qs) for p, qs in fused]
    k = shapes.index(((2, 4), (1,)))
    # everything on qudit 1 before the projection is applied before it
    before = [qs for _, qs in shapes[:k]]
    assert any(1 in qs for qs in before)
    pv = _rand_pv(rng, (4, 4, 4))
    assert_close_dot(_apply_all(pv, fused), _apply_all(pv, units),
                     _abs_all(np.abs(pv), units) * 4)

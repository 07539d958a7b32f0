"""Host-side planning of the batched kernel's units (no GPU): a two-qubit op
absorbs the one-qubit ops waiting on its qubits (across layers).  Applying
the units' PTMs F = C (A (x) B) with the oracle reproduces the ops applied
one by one, and the gradient mapping through the chains A and B matches
autograd."""
import numpy as np
import pytest
import torch

from oracle import pauli_vector_np as O
from quantumsim_gb300 import batch as BT


def _apply_ops(x, ops, mats):
    for (l, qs), m in zip(ops, mats):
        x = O.apply_ptm(x, m if len(qs) == 1 else m.reshape(4, 4, 4, 4),
                        *sorted(qs))
    return x


def _chain(mats, chain):
    m = np.eye(4)
    for j in chain:
        m = mats[j] @ m
    return m


def _unit_matrix(qs, mem, mats):
    if len(qs) == 1:
        return _chain(mats, mem[0])
    m = np.eye(16)
    for jc, ca, cb in mem:
        m = mats[jc] @ np.kron(_chain(mats, ca), _chain(mats, cb)) @ m
    return m


def _check_units(ops, mats, units, x, tol):
    used = sorted(j for _, qs, mem in units for j in BT.unit_ops(qs, mem))
    assert used == list(range(len(ops)))
    layers = [l for l, _, _ in units]
    assert layers == sorted(layers)
    unit_ops = [(l, qs) for l, qs, _ in units]
    unit_mats = [_unit_matrix(qs, mem, mats) for _, qs, mem in units]
    for _, qs, _ in units:
        assert len(qs) == 1 or qs[0] < qs[1]
    np.testing.assert_allclose(_apply_ops(x, unit_ops, unit_mats),
                               _apply_ops(x, ops, mats), rtol=tol, atol=tol)


@pytest.mark.parametrize('n,depth,seed', [(5, 4, 0), (6, 3, 1), (4, 5, 2),
                                          (1, 2, 3), (2, 3, 4)])
def test_units_reproduce_ops(n, depth, seed):
    spec = BT.CircuitSpec(n, depth, seed)
    ops = spec.ops()
    mats = [p.numpy() for p in BT.instance_ptms(spec)]
    # a generic (non-symmetric) two-qubit PTM exposes any ordering slip
    rng = np.random.default_rng(seed)
    mats = [m if m.shape == (4, 4) else rng.standard_normal((16, 16))
            for m in mats]
    units = BT.plan_units(ops)
    # every op exactly once; unit layers in order; the same map
    x = rng.standard_normal((4,) * n)
    _check_units(ops, mats, units, x, 1e-12)
    # one-qubit units remain only for qubits with no later two-qubit op
    ones = [qs[0] for _, qs, _ in units if len(qs) == 1]
    assert len(ones) == len(set(ones))
    # unfused planning keeps one unit per op
    plain = BT.plan_units(ops, fuse=False)
    assert [BT.unit_ops(qs, mem) for _, qs, mem in plain] == \
        [[j] for j in range(len(ops))]
    _check_units(ops, mats, plain, x, 1e-12)


def test_units_fuse_most_one_qubit_ops():
    """The line-matching circuits leave one or two qubits unpaired per
    layer; their rotations wait for the next two-qubit op on the qubit, so
    the units are the two-qubit ops plus at most one unit per qubit at the
    end."""
    spec = BT.CircuitSpec(12, 30, 0)
    ops = spec.ops()
    units = BT.plan_units(ops)
    n_two = sum(1 for _, qs in ops if len(qs) == 2)
    assert len([u for u in units if len(u[1]) == 1]) <= spec.n
    assert sum(len(mem) for _, qs, mem in units if len(qs) == 2) == n_two
    assert len(units) < 0.4 * len(ops)
    # odd qubit counts draw the matching's offset per layer: consecutive
    # layers on the same pairs share units, at most MAX_FACTORS CZs each
    odd = BT.plan_units(BT.CircuitSpec(11, 30, 3).ops())
    sizes = [len(mem) for _, qs, mem in odd if len(qs) == 2]
    assert max(sizes) > 1 and max(sizes) <= BT.MAX_FACTORS


def test_gradient_mapping_matches_autograd():
    """The rule step() applies to a fused unit's gradient: for F = C K with
    K = R_a (x) R_b and any loss of F, dL/dC = G K^T and dL/dR_a, dL/dR_b
    from H = C^T G, against torch autograd in float64."""
    rng = np.random.default_rng(9)
    c = torch.tensor(rng.standard_normal((16, 16)), requires_grad=True)
    ra = torch.tensor(rng.standard_normal((4, 4)), requires_grad=True)
    rb = torch.tensor(rng.standard_normal((4, 4)), requires_grad=True)
    w = torch.tensor(rng.standard_normal((16, 16)))
    f = c @ torch.kron(ra, rb)
    loss = (w * f).sum() + (f ** 2).sum()
    loss.backward()
    g = (w + 2 * f).detach()
    kr = torch.einsum('ac,bd->abcd', ra, rb).reshape(16, 16).detach()
    np.testing.assert_allclose(g @ kr.T, c.grad, rtol=1e-12, atol=1e-12)
    h = (c.detach().T @ g).view(4, 4, 4, 4)
    np.testing.assert_allclose(torch.einsum('xyzw,yw->xz', h, rb.detach()),
                               ra.grad, rtol=1e-12, atol=1e-11)
    np.testing.assert_allclose(torch.einsum('xyzw,xz->yw', h, ra.detach()),
                               rb.grad, rtol=1e-12, atol=1e-11)


def test_chain_gradient_mapping_matches_autograd():
    """map_unit_gradients through chains of one-qubit ops (lengths 0 to 3
    on either side of a two-qubit op, and a one-qubit unit of three ops),
    against torch autograd in float64."""
    rng = np.random.default_rng(10)
    ops1 = [torch.tensor(rng.standard_normal((4, 4)), requires_grad=True)
            for _ in range(9)]
    cs = [torch.tensor(rng.standard_normal((16, 16)), requires_grad=True)
          for _ in range(3)]
    # one-qubit unit: ops 0, 1, 2; two-qubit units: (A: (), B: (3,)),
    # (A: (4, 5), B: ()), (A: (6,), B: (7, 8))
    one_chains = [(0, 1, 2)]
    a_chains, b_chains = [(), (4, 5), (6,)], [(3,), (), (7, 8)]

    def prod(ch):
        m = torch.eye(4, dtype=torch.float64)
        for j in ch:
            m = ops1[j] @ m
        return m
    f_one = [prod(ch) for ch in one_chains]
    f_two = [c @ torch.kron(prod(a), prod(b))
             for c, a, b in zip(cs, a_chains, b_chains)]
    w1 = [torch.tensor(rng.standard_normal((4, 4))) for _ in f_one]
    w2 = [torch.tensor(rng.standard_normal((16, 16))) for _ in f_two]
    loss = sum((w * f).sum() + (f ** 3).sum() for w, f in zip(w1, f_one)) + \
        sum((w * f).sum() + (f ** 2).sum() for w, f in zip(w2, f_two))
    loss.backward()
    g_one = torch.stack([(w + 3 * f ** 2).detach()
                         for w, f in zip(w1, f_one)])
    g_two = torch.stack([(w + 2 * f).detach() for w, f in zip(w2, f_two)])
    mats = torch.stack([o.detach() for o in ops1])
    prods, cfac = BT.chain_products(mats, one_chains + a_chains + b_chains)
    a = prods[1:4]
    b = prods[4:7]
    c = torch.stack([x.detach() for x in cs])
    dc, (eo, d) = BT.map_unit_gradients(g_one, g_two, c, a, b, cfac)
    for k in range(3):
        np.testing.assert_allclose(dc[k], cs[k].grad, rtol=1e-12,
                                   atol=1e-10)
    assert sorted(eo.tolist()) == list(range(9))
    for j, dj in zip(eo.tolist(), d):
        np.testing.assert_allclose(dj, ops1[j].grad, rtol=1e-11, atol=1e-9)


@pytest.mark.parametrize('seed', range(6))
def test_units_reproduce_random_op_sequences(seed):
    """Random layers of one- and two-qubit ops in any order: rotations after
    a CZ, two CZs sharing a qubit, several rotations on one qubit, pairs in
    either qubit order.  Applying the units equals applying the ops."""
    rng = np.random.default_rng(100 + seed)
    n = int(rng.integers(2, 6))
    ops, mats = [], []
    for layer in range(int(rng.integers(1, 4))):
        for _ in range(int(rng.integers(1, 9))):
            if rng.random() < 0.5:
                ops.append((layer, (int(rng.integers(n)),)))
                mats.append(rng.standard_normal((4, 4)))
            else:
                a, b = (int(v) for v in rng.choice(n, 2, replace=False))
                ops.append((layer, (a, b)))
                mats.append(rng.standard_normal((16, 16)))
    units = BT.plan_units(ops)
    x = rng.standard_normal((4,) * n)
    _check_units(ops, mats, units, x, 1e-11)


@pytest.mark.parametrize('ops,msg', [
    ([(0, (5,))], 'acts on'),                 # qubit out of range
    ([(0, (-1,))], 'acts on'),
    ([(0, (2, 2))], 'acts on'),               # repeated qubit
    ([(0, (0, 1, 2))], 'acts on'),            # three qubits
    ([(1, (0,)), (0, (1,))], 'layer'),        # layers out of order
    ([(7, (0,))], 'layer'),                   # layer past the depth
])
def test_malformed_structures_are_rejected_on_the_host(ops, msg):
    """Bad target qubits or layers raise ValueError before any device
    memory is touched (the kernel's group geometry assumes valid targets)."""
    spec = BT.CircuitSpec(4, 3, 0)
    spec.ops = lambda o=ops: o
    with pytest.raises(ValueError, match=msg):
        BT.BatchedSimulator([spec], [torch.ones(16) / 16], device='cpu')
    # the valid structure passes the check
    BT.validate_ops(BT.CircuitSpec(4, 3, 0).ops(), 4, 3)


@pytest.mark.parametrize('fuse', [True, False])
@pytest.mark.parametrize('tile', [4, 64, 8192])
def test_program_invariants(fuse, tile):
    """What the batch kernel relies on: every stage entry's items cover its
    range exactly once with boundaries on multiples of 4, one entry per
    instance per stage, the per-instance stage sequence INIT, APPLY (units
    in order, SAVE between layers), ZERO_G, LOSS, ADJOINT (units in reverse,
    RESTORE), every dP slot written by exactly one ADJOINT item and summed
    by exactly one GRADSUM item of its unit."""
    shapes = [(4, 5), (7, 3), (2, 4), (9, 2), (1, 3), (6, 8)]
    specs = [BT.CircuitSpec(n, d, i) for i, (n, d) in enumerate(shapes)]
    every = 2
    units = [BT.plan_units(s.ops(), fuse) for s in specs]
    ubase = np.cumsum([0] + [len(u) for u in units])
    sizes = [4 ** s.n for s in specs]
    items, begin, n_slots = BT.build_program(
        units, ubase, sizes, [s.depth for s in specs], every, tile)
    assert begin[0] == 0 and begin[-1] == len(items)
    assert np.all(np.diff(begin) >= 0)
    last = items[begin[-2]:]
    assert np.all(last['op'] == BT.BOP_GRADSUM)
    assert not np.any(items[:begin[-2]]['op'] == BT.BOP_GRADSUM)
    seqs = {i: [] for i in range(len(specs))}
    for s in range(len(begin) - 2):
        stage = items[begin[s]:begin[s + 1]]
        for i in np.unique(stage['inst']):
            it = np.sort(stage[stage['inst'] == i], order='beg')
            assert len(set(it['op'])) == 1 and len(set(it['ptm'])) == 1
            op, pp = int(it['op'][0]), int(it['ptm'][0])
            assert len(it) <= 64
            if op == BT.BOP_LOSS:
                assert len(it) == 1
            else:
                if op in (BT.BOP_APPLY, BT.BOP_ADJOINT):
                    total = sizes[i] // (4 if it['q1'][0] < 0 else 16)
                    _, qs, _ = units[i][pp - ubase[i]]
                    assert (it['q0'][0], it['q1'][0]) == \
                        ((qs[0], -1) if len(qs) == 1 else qs)
                else:
                    total = sizes[i]
                assert it['beg'][0] == 0 and it['end'][-1] == total
                assert np.all(it['beg'][1:] == it['end'][:-1])
                assert np.all(it['beg'] % 4 == 0)
                assert np.all((it['end'] % 4 == 0) | (it['end'] == total))
            seqs[int(i)].append((op, pp))
    for i, seq in seqs.items():
        n_u = len(units[i])
        ops = [o for o, _ in seq]
        assert ops[0] == BT.BOP_INIT
        k_loss = ops.index(BT.BOP_LOSS)
        assert ops[k_loss - 1] == BT.BOP_ZERO_G
        fwd = [p for o, p in seq[:k_loss] if o == BT.BOP_APPLY]
        bwd = [p for o, p in seq[k_loss:] if o == BT.BOP_ADJOINT]
        assert fwd == list(range(ubase[i], ubase[i] + n_u))
        assert bwd == fwd[::-1]
        n_ckpt = max(0, (specs[i].depth - 1) // every)
        assert ops.count(BT.BOP_SAVE) == n_ckpt
        assert ops.count(BT.BOP_RESTORE) == n_ckpt
        # checkpoint k is saved and restored at the same unit boundary:
        # after the same number of APPLYs as ADJOINTs remain after it
        for k in range(n_ckpt):
            ks = [t for t, (o, p) in enumerate(seq)
                  if o == BT.BOP_SAVE and p == k]
            kr = [t for t, (o, p) in enumerate(seq)
                  if o == BT.BOP_RESTORE and p == k]
            assert len(ks) == len(kr) == 1
            applied = sum(1 for o, _ in seq[:ks[0]] if o == BT.BOP_APPLY)
            left = sum(1 for o, _ in seq[kr[0]:] if o == BT.BOP_ADJOINT)
            assert applied == left
    adj = items[items['op'] == BT.BOP_ADJOINT]
    assert sorted(adj['slot']) == list(range(n_slots))
    for g in last:
        mine = adj[adj['ptm'] == g['ptm']]
        assert sorted(mine['slot']) == list(range(g['beg'], g['end']))
    assert sorted(last['ptm']) == list(range(int(ubase[-1])))


def test_factor_chain_gradient_mapping_matches_autograd():
    """Units of several factors M = C (A (x) B) (as consecutive CZs on one
    pair with rotations between them form): map_unit_gradients through the
    factor chains and the rotation chains, against torch autograd."""
    rng = np.random.default_rng(11)
    r = [torch.tensor(rng.standard_normal((4, 4)), requires_grad=True)
         for _ in range(6)]
    cs = [torch.tensor(rng.standard_normal((16, 16)), requires_grad=True)
          for _ in range(5)]
    # unit 0: factors (C0, A: (0,), B: ()), (C1, A: (1, 2), B: (3,)),
    #         (C2, (), ()); unit 1: (C3, (4,), ()), (C4, (), (5,))
    facs = [(0, (0,), ()), (1, (1, 2), (3,)), (2, (), ()), (3, (4,), ()),
            (4, (), (5,))]
    seqs = [(0, 1, 2), (3, 4)]

    def chain(ch):
        m = torch.eye(4, dtype=torch.float64)
        for j in ch:
            m = r[j] @ m
        return m
    ms = [cs[jc] @ torch.kron(chain(ca), chain(cb)) for jc, ca, cb in facs]
    units = []
    for sq in seqs:
        u = torch.eye(16, dtype=torch.float64)
        for f in sq:
            u = ms[f] @ u
        units.append(u)
    w = [torch.tensor(rng.standard_normal((16, 16))) for _ in units]
    loss = sum((wi * u).sum() + (u ** 2).sum() for wi, u in zip(w, units))
    loss.backward()
    g_two = torch.stack([(wi + 2 * u).detach() for wi, u in zip(w, units)])
    mats = torch.stack([x.detach() for x in r])
    prods, cfac = BT.chain_products(
        mats, [f[1] for f in facs] + [f[2] for f in facs])
    a, b = prods[:5], prods[5:]
    c = torch.stack([cs[f[0]].detach() for f in facs])
    m = torch.bmm(c, torch.einsum('uac,ubd->uabcd', a, b).reshape(-1, 16, 16))
    fu, ffac = BT.chain_products(m, seqs)
    for k in range(2):
        np.testing.assert_allclose(fu[k], units[k].detach(), rtol=1e-12,
                                   atol=1e-12)
    g_one = torch.zeros(0, 4, 4, dtype=torch.float64)
    dc, (eo, d) = BT.map_unit_gradients(g_one, g_two, c, a, b, cfac, ffac)
    for f, (jc, _, _) in enumerate(facs):
        np.testing.assert_allclose(dc[f], cs[jc].grad, rtol=1e-11, atol=1e-8)
    assert sorted(eo.tolist()) == list(range(6))
    for j, dj in zip(eo.tolist(), d):
        np.testing.assert_allclose(dj, r[j].grad, rtol=1e-11, atol=1e-7)


def test_factors_kept_in_place_for_a_captured_graph():
    """BatchedSimulator._keep: new values of the same shapes are copied
    into the stored tensors (a captured graph reads them) and the graph is
    kept; other shapes, or None where tensors were, replace the tensors
    and drop the graph."""
    class Holder:
        device = torch.device('cpu')
        graph = 'captured'
    h = Holder()
    keep = BT.BatchedSimulator._keep
    a = (torch.zeros(2, 4, 4), torch.arange(3))
    keep(h, '_f', a)
    first = h._f
    h.graph = 'captured'
    keep(h, '_f', (torch.ones(2, 4, 4), torch.arange(3) + 5))
    assert h._f is first and h.graph == 'captured'
    assert torch.equal(first[0], torch.ones(2, 4, 4))
    assert torch.equal(first[1], torch.arange(3) + 5)
    keep(h, '_f', (torch.ones(3, 4, 4), torch.arange(3)))
    assert h._f is not first and h.graph is None
    h.graph = 'captured'
    keep(h, '_f', None)
    assert h._f is None and h.graph is None
    h.graph = 'captured'
    keep(h, '_f', None)
    assert h.graph == 'captured'

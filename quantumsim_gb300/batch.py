"""Batched forward + adjoint of many independent noisy circuits.

``BatchedSimulator`` runs B circuits of different qubit counts (each with its
own noise parameters) -- Pauli vectors in FP32, probabilities, losses and
PTM gradients accumulated in FP64 -- as ONE persistent launch of the
``qsgb_batch_run`` kernel, optionally replayed from a CUDA graph.  One step
computes, for every instance, the probabilities of the final state, the loss
KL(target || prob) and dL/dP for every PTM of its circuit.

Circuits are the CPU-runnable workload family: per layer a noisy rotation on
every qubit (rotation, then amplitude + phase damping over 20 ns) and CZs on
a line matching.  Ops are grouped into units first (`plan_units`): a CZ
absorbs the rotations waiting on its two qubits, from its own layer and
from earlier layers where the qubit had no CZ, so a layer of n rotations
and ~n/2 CZs costs ~n/2 passes over the state instead of ~3n/2.  The device
program is built once per circuit structure:

    stage 0              INIT  (|0..0>)
    stages ...           APPLY of unit j of every instance (instances aligned
                         by unit index), SAVE at the unit boundary before
                         every `checkpoint_every`-th layer
                         ZERO_G, LOSS
    stages ...           ADJOINT of the units in reverse, RESTORE at the
                         saved boundaries (drift refresh)
    last stage           GRADSUM per unit PTM

after which batched 16 x 16 contractions turn the units' gradients into
dL/dP of every original op.

Each op on a large instance is split into tiles of `tile` groups, so blocks
share big instances while small ones take one item.  ``autotune()`` times the
candidate tile sizes and keeps the fastest (cached in a JSON file).

The reference has no batching; the per-instance comparison is the plain GPU
path (``plain_gradients``): one instance at a time through the ``ApplyPTM``
autograd function and checkpointed layers.
"""
import ctypes
import json
import math
import os
import time

import numpy as np
import torch

from . import _lib as L
from . import bases as _bases
from . import ptm as P
from .autograd import apply_ptm_diff, checkpointed, diagonal_diff

BOP_INIT, BOP_ZERO_G, BOP_APPLY, BOP_SAVE, BOP_RESTORE, BOP_LOSS, \
    BOP_ADJOINT, BOP_GRADSUM = range(1, 9)
BLOCK = 256
T_GATE = 20e-9


class _Instance(ctypes.Structure):
    _fields_ = [('x', ctypes.c_void_p), ('g', ctypes.c_void_p),
                ('ckpt', ctypes.c_void_p), ('size', ctypes.c_int64),
                ('n_qubits', ctypes.c_int32), ('diag_offset', ctypes.c_int32)]


class _Program(ctypes.Structure):
    _fields_ = [('instances', ctypes.c_void_p), ('items', ctypes.c_void_p),
                ('stage_begin', ctypes.c_void_p), ('n_stages', ctypes.c_int32),
                ('n_instances', ctypes.c_int32), ('work', ctypes.c_void_p), ('ptm', ctypes.c_void_p),
                ('ptm_inv', ctypes.c_void_p),
                ('grad_partial', ctypes.c_void_p), ('grad', ctypes.c_void_p),
                ('target', ctypes.c_void_p), ('prob', ctypes.c_void_p),
                ('loss', ctypes.c_void_p)]


_ITEM_DTYPE = np.dtype([('op', '<i4'), ('inst', '<i4'), ('q0', '<i4'),
                        ('q1', '<i4'), ('ptm', '<i4'), ('slot', '<i4'),
                        ('beg', '<i8'), ('end', '<i8')])


class CircuitSpec:
    """Structure and noise of one instance (seeded)."""

    def __init__(self, n_qubits, depth, seed):
        rng = np.random.default_rng(seed)
        self.n = n_qubits
        self.depth = depth
        self.axes = [['xyz'[i] for i in rng.integers(3, size=n_qubits)]
                     for _ in range(depth)]
        self.angles = rng.uniform(0, 2 * math.pi, (depth, n_qubits))
        t1 = rng.uniform(20, 60, n_qubits)
        self.t1 = t1
        self.t2 = rng.uniform(10, t1)
        self.pairs = []
        for l in range(depth):
            off = int(rng.integers(2)) if n_qubits % 2 else l % 2
            self.pairs.append([(i, i + 1) for i in range(off, n_qubits - 1,
                                                         2)])

    def ops(self):
        """[(layer, qubits)] in application order."""
        out = []
        for l in range(self.depth):
            out += [(l, (q,)) for q in range(self.n)]
            out += [(l, pr) for pr in self.pairs[l]]
        return out


def instance_ptms(spec, angle_offset=0.0, device='cpu'):
    """Float64 PTMs of an instance's ops, in op order: (K, K) matrices with
    K = 4 or 16 (two-qubit ones in (q0, q1) = sorted order)."""
    n, d = spec.n, spec.depth
    axes = [a for row in spec.axes for a in row]
    ang = torch.as_tensor(spec.angles, dtype=torch.float64, device=device)
    rot = P.rotations_batched(axes, (ang + angle_offset).reshape(-1))
    g, lam = P.damping_rates(torch.as_tensor(spec.t1 * 1e-6, device=device),
                             torch.as_tensor(spec.t2 * 1e-6, device=device),
                             T_GATE)
    damp = P.amp_phase_damping_batched(g, lam)
    one = (damp[None] @ rot.reshape(d, n, 4, 4))
    cz = P.cphase(math.pi).to(device).reshape(16, 16)
    out = []
    for l, qs in spec.ops():
        out.append(one[l, qs[0]] if len(qs) == 1 else cz)
    return out


def target_probabilities(spec, seed):
    """A target distribution: the exact FP64 probabilities of the same
    circuit with perturbed rotation angles (computed on the GPU in FP64)."""
    rng = np.random.default_rng(seed)
    off = torch.from_numpy(rng.normal(0, 0.05, (spec.depth, spec.n)))
    ptms = instance_ptms(spec, angle_offset=off)
    x = torch.zeros((4,) * spec.n, dtype=torch.float64, device='cuda')
    x[(0,) * spec.n] = 1
    for pt, (_, qs) in zip(ptms, spec.ops()):
        pt = pt if len(qs) == 1 else pt.reshape(4, 4, 4, 4)
        x = apply_ptm_diff(x, pt, *qs)
    return diagonal_diff(x, [_bases.general(2)] * spec.n).detach()


def validate_ops(ops, n, depth, what='circuit'):
    """Raise ValueError unless every op acts on one qubit or two distinct
    qubits in [0, n) and the layers are non-decreasing within [0, depth)."""
    prev = 0
    for j, (layer, qs) in enumerate(ops):
        qs = tuple(qs)
        if len(qs) not in (1, 2) or any(
                not (isinstance(q, (int, np.integer)) and 0 <= q < n)
                for q in qs) or len(set(qs)) != len(qs):
            raise ValueError('{}: op {} acts on {}; ops take one qubit or two '
                             'distinct qubits in [0, {})'.format(what, j, qs,
                                                                  n))
        if not 0 <= layer < depth or layer < prev:
            raise ValueError('{}: op {} has layer {}; layers run in order '
                             'within [0, {})'.format(what, j, layer, depth))
        prev = layer


# two-qubit ops one unit may hold (consecutive CZs on one pair, with the
# rotations between them): bounds the products behind a unit's PTM and its
# inverse
MAX_FACTORS = 4


def plan_units(ops, fuse=True):
    """Group a circuit's ops into the units the kernel applies.

    ops: [(layer, qubits)] in application order.  With `fuse`, a one-qubit
    op waits on its qubit (across layers, past ops on other qubits, which
    it commutes with) until the next two-qubit op on that qubit absorbs it:
    a factor M = C (A (x) B), with A and B the products of the one-qubit ops
    waiting on its two qubits (identity where none).  A two-qubit op whose
    two qubits were last touched by the same unit (the previous op on both
    is a two-qubit op on the same pair) joins that unit as its next factor,
    up to MAX_FACTORS; the unit's PTM is the product M_k ... M_1, a dense
    16 x 16 PTM like any two-qubit PTM of the kernel, so the unit costs one
    pass where its ops cost several.  The one-qubit ops that meet no later
    two-qubit op become one-qubit units (their product) at the end.
    Without `fuse` every op is a unit of its own.

    A unit's layer is its first two-qubit op's layer (for the one-qubit
    units at the end, the last op's layer), so the layers of the units
    never decrease; checkpoints sit at unit boundaries (`build_program`).

    Returns [(layer, qubits, members)]: members = (chain,) for a one-qubit
    unit (qubits = (q,)); for a two-qubit unit (qubits = (a, b) sorted) a
    tuple of factors (j_c, chain_a, chain_b) in application order.  A chain
    is the tuple of one-qubit op indices in application order (empty: the
    identity)."""
    units = []
    if not fuse:
        for j, (l, qs) in enumerate(ops):
            if len(qs) == 1:
                units.append((l, (qs[0],), ((j,),)))
            else:
                units.append((l, (min(qs), max(qs)), ((j, (), ()),)))
        return units
    pending = {}
    last = {}  # qubit -> index of the last unit on it
    for j, (l, qs) in enumerate(ops):
        if len(qs) == 1:
            pending.setdefault(qs[0], []).append(j)
            continue
        a, b = min(qs), max(qs)
        factor = (j, tuple(pending.pop(a, ())), tuple(pending.pop(b, ())))
        k = last.get(a)
        if k is not None and last.get(b) == k and \
                len(units[k][2]) < MAX_FACTORS:
            lk, qk, mem = units[k]
            units[k] = (lk, qk, mem + (factor,))
            continue
        units.append((l, (a, b), (factor,)))
        last[a] = last[b] = len(units) - 1
    if pending:
        lay = ops[-1][0]
        for q, chain in sorted(pending.items(), key=lambda t: t[1][0]):
            units.append((lay, (q,), (tuple(chain),)))
    return units


def unit_ops(qubits, members):
    """Every op index of a unit's members."""
    if len(qubits) == 1:
        return list(members[0])
    return [o for jc, ca, cb in members for o in (jc,) + ca + cb]


def chain_products(mats, chains):
    """Products of matrix chains and the factors of their gradients.

    mats: (n, d, d) float64 tensor (only chain members are read); chains:
    tuples of indices into mats in application order.  For a chain
    r_0 .. r_{m-1}, prod = r_{m-1} ... r_0 (the identity for an empty
    chain), and for its element i, dL/dr_i = L_i^T (dL/dprod) R_i^T with
    L_i = r_{m-1} ... r_{i+1} and R_i = r_{i-1} ... r_0.

    Returns (prod (n_chains, d, d), factors) with factors = (direct_elem,
    direct_chain, elem, elem_chain, left_t, right_t): the elements of
    one-element chains (dL/dr = dL/dprod) by index into mats and chain,
    then the others with left_t = L_i^T and right_t = R_i^T."""
    n, d = len(chains), mats.shape[-1]
    dt, dev = mats.dtype, mats.device
    prod = torch.eye(d, dtype=dt, device=dev).repeat(n, 1, 1)
    one = [c for c, ch in enumerate(chains) if len(ch) == 1]
    d_op = torch.as_tensor([chains[c][0] for c in one], dtype=torch.long,
                           device=dev)
    d_ch = torch.as_tensor(one, dtype=torch.long, device=dev)
    if one:
        prod[d_ch] = mats[d_op]
    e_op, e_ch, lt, rt = [], [], [], []
    by_len = {}
    for c, ch in enumerate(chains):
        if len(ch) > 1:
            by_len.setdefault(len(ch), []).append(c)
    for m, cs in sorted(by_len.items()):
        idx = torch.as_tensor([chains[c] for c in cs], dtype=torch.long,
                              device=dev)
        r = mats[idx]                                   # (k, m, d, d)
        eye = torch.eye(d, dtype=dt, device=dev).expand(len(cs), d, d)
        pre = [eye]                                     # r_{i-1} ... r_0
        for i in range(1, m):
            pre.append(torch.bmm(r[:, i - 1], pre[-1]))
        suf = [eye] * m                                 # r_{m-1} ... r_{i+1}
        for i in range(m - 2, -1, -1):
            suf[i] = torch.bmm(suf[i + 1], r[:, i + 1])
        cs_t = torch.as_tensor(cs, dtype=torch.long, device=dev)
        prod[cs_t] = torch.bmm(r[:, m - 1], pre[m - 1])
        for i in range(m):
            e_op.append(idx[:, i])
            e_ch.append(cs_t)
            lt.append(suf[i].transpose(1, 2))
            rt.append(pre[i].transpose(1, 2))
    if e_op:
        rest = (torch.cat(e_op), torch.cat(e_ch), torch.cat(lt),
                torch.cat(rt))
    else:
        z = torch.zeros(0, dtype=torch.long, device=dev)
        zz = torch.zeros(0, d, d, dtype=dt, device=dev)
        rest = (z, z, zz, zz)
    return prod, (d_op, d_ch) + rest


def chain_gradients(g_prod, factors):
    """(element indices, dL/dr per element) from the chains' dL/dprod
    `g_prod` (n_chains, d, d) and `factors` from chain_products."""
    d_op, d_ch, e_op, e_ch, lt, rt = factors
    if not len(e_op):
        return d_op, g_prod[d_ch]
    if not len(d_op):
        return e_op, torch.bmm(torch.bmm(lt, g_prod[e_ch]), rt)
    return (torch.cat([d_op, e_op]),
            torch.cat([g_prod[d_ch], torch.bmm(torch.bmm(lt, g_prod[e_ch]),
                                               rt)]))


def map_unit_gradients(g_one, g_two, c, a, b, chain_factors,
                       factor_chains=None):
    """dL/dP of the original ops from the units' gradients (any device).

    g_one (n1, 4, 4): the one-qubit units' gradients.  g_two: the two-qubit
    units' gradients (n_units, 16, 16); each unit is the product of factors
    M = C K, K = A (x) B, whose C, A and B are c, a, b (n_factors, ...);
    factor_chains: the factors of the units' factor chains
    (`chain_products` over the factors' M; None when every unit has one
    factor, listed in unit order).  chain_factors: those of the one-qubit
    chains, ordered one-qubit units, then side a, then side b of the
    factors.

    Returns (dL/dC (n_factors, 16, 16), (op indices, dL/dr (k, 4, 4)) for
    the one-qubit chain elements).  Per factor, with G its dL/dM:
    dL/dC = G K^T; with H = C^T G viewed as [a', b', a, b],
    dL/dA = sum H B[b', b] and dL/dB = sum H A[a', a]; each chain element
    gets L^T (dL/dprod) R^T."""
    parts = [g_one]
    dc = None
    if len(c):
        if factor_chains is None:
            gm = g_two
        else:
            f_idx, g_f = chain_gradients(g_two, factor_chains)
            gm = torch.empty_like(c)
            gm[f_idx] = g_f
        kr = torch.einsum('uac,ubd->uabcd', a, b).reshape(-1, 16, 16)
        dc = torch.bmm(gm, kr.transpose(1, 2))
        h = torch.bmm(c.transpose(1, 2), gm).view(-1, 4, 4, 4, 4)
        parts += [torch.einsum('uxyzw,uyw->uxz', h, b),
                  torch.einsum('uxyzw,uxz->uyw', h, a)]
    return dc, chain_gradients(torch.cat(parts), chain_factors)


def build_program(units, unit_base, sizes, depths, every, tile,
                  max_items=64):
    """Host part of the device program, in numpy: (items, stage_begin,
    n_slots).

    Every unit is one stage entry per instance; an entry covering `total`
    groups (or elements) becomes ceil(total / chunk) items with chunk =
    max(tile, ceil(total / max_items)) -- large ops are shared by many
    blocks, and no op has more than `max_items` items.  `tile` is a multiple
    of 4: the kernel takes 4 consecutive groups along z per access, and an
    item boundary must not split them.  Stages per instance: INIT, APPLY of
    every unit (SAVE after every `every`-th layer), ZERO_G, LOSS, ADJOINT of
    the units in reverse (RESTORE at the saved layers); a last stage holds
    one GRADSUM item per unit over the dP slots of its ADJOINT items."""
    if tile < 4 or tile % 4:
        raise ValueError('tile must be a positive multiple of 4')
    ent = []  # (stage, op, inst, q0, q1, ptm or checkpoint, total)
    for i, (unit_list, size, depth) in enumerate(zip(units, sizes, depths)):
        ops = [(l, qs) for l, qs, _ in unit_list]
        layer_of = [l for l, _ in ops]
        # checkpoint k holds the state at the boundary before the first
        # unit of layer >= every * (k + 1) (after the last unit if none is)
        n_ck = max(0, (depth - 1) // every)
        bound = [int(np.searchsorted(layer_of, every * (k + 1), side='left'))
                 for k in range(n_ck)]
        seq = [(BOP_INIT, -1, -1, 0, size)]
        for j in range(len(ops) + 1):
            seq += [(BOP_SAVE, -1, -1, k, size)
                    for k, bj in enumerate(bound) if bj == j]
            if j < len(ops):
                l, qs = ops[j]
                q0, q1 = (qs[0], -1) if len(qs) == 1 else (min(qs), max(qs))
                seq.append((BOP_APPLY, q0, q1, int(unit_base[i]) + j,
                            size // (4 if q1 < 0 else 16)))
        seq.append((BOP_ZERO_G, -1, -1, 0, size))
        seq.append((BOP_LOSS, -1, -1, 0, 1))
        for j in range(len(ops), -1, -1):
            if j < len(ops):
                l, qs = ops[j]
                q0, q1 = (qs[0], -1) if len(qs) == 1 else (min(qs), max(qs))
                seq.append((BOP_ADJOINT, q0, q1, int(unit_base[i]) + j,
                            size // (4 if q1 < 0 else 16)))
            seq += [(BOP_RESTORE, -1, -1, k, size)
                    for k, bj in enumerate(bound) if bj == j]
        for k, (op, q0, q1, pp, total) in enumerate(seq):
            ent.append((k, op, i, q0, q1, pp, total))
    e = np.array(ent, dtype=np.int64)
    stage, op, inst, q0, q1, pp, total = e.T
    is_loss = op == BOP_LOSS
    chunk = np.where(is_loss, 1, np.maximum(tile, -(-total // max_items)))
    n_items = -(-total // chunk)
    # one dP partial slot per ADJOINT item
    adj = op == BOP_ADJOINT
    slot_base = np.zeros(len(e), dtype=np.int64)
    slot_base[adj] = np.cumsum(np.concatenate([[0], n_items[adj][:-1]]))
    n_slots = int(n_items[adj].sum())
    # expand entries into items
    rep = np.repeat(np.arange(len(e)), n_items)
    first = np.repeat(np.cumsum(n_items) - n_items, n_items)
    j = np.arange(len(rep)) - first
    beg = j * chunk[rep]
    end_ = np.minimum(total[rep], beg + chunk[rep])
    items = np.zeros(len(rep), dtype=_ITEM_DTYPE)
    items['op'] = op[rep]
    items['inst'] = inst[rep]
    items['q0'] = q0[rep]
    items['q1'] = q1[rep]
    items['ptm'] = pp[rep]
    items['slot'] = np.where(adj[rep], slot_base[rep] + j, 0)
    items['beg'] = np.where(is_loss[rep], 0, beg)
    items['end'] = np.where(is_loss[rep], 0, end_)
    st = stage[rep]
    n_main = int(st.max()) + 1
    # last stage: GRADSUM per PTM over the slots of its ADJOINT items
    gitems = np.zeros(int(adj.sum()), dtype=_ITEM_DTYPE)
    gitems['op'] = BOP_GRADSUM
    gitems['ptm'] = pp[adj]
    gitems['q1'] = -1
    gitems['beg'] = slot_base[adj]
    gitems['end'] = slot_base[adj] + n_items[adj]
    order = np.argsort(st, kind='stable')
    items = np.concatenate([items[order], gitems])
    counts = np.concatenate([np.bincount(st, minlength=n_main),
                             [len(gitems)]])
    begin = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
    return items, begin, n_slots


class BatchedSimulator:
    """Forward + adjoint of many circuits in one persistent launch.

    With `fuse` (default) each two-qubit op absorbs the one-qubit ops
    waiting on its qubits (`plan_units`); `results()` still returns dL/dP
    for every original op: step() maps the units' gradients back with
    batched contractions on the same stream (inside the CUDA graph)."""

    def __init__(self, specs, targets, checkpoint_every=8, tile=None,
                 device=None, cooperative=True, fuse=True):
        # ---- structure checks, before anything reaches the device: the
        # kernel's group geometry assumes valid, distinct target qubits
        if any(not 1 <= s.n <= 15 for s in specs):
            raise ValueError('batched instances have 1 to 15 qubits')
        if checkpoint_every < 1:
            raise ValueError('checkpoint_every must be at least 1')
        for i, s in enumerate(specs):
            validate_ops(s.ops(), s.n, s.depth, 'instance {}'.format(i))
        self.lib = L.load()
        self.device = torch.device(device or 'cuda')
        self.specs = specs
        self.every = checkpoint_every
        self.cooperative = cooperative
        self.n_inst = len(specs)
        dev = self.device
        # ---- per-instance buffers
        self.sizes = [4 ** s.n for s in specs]
        self.n_ckpt = [max(0, (s.depth - 1) // checkpoint_every)
                       for s in specs]
        self.x = [torch.empty(sz, dtype=torch.float32, device=dev)
                  for sz in self.sizes]
        self.g = [torch.empty(sz, dtype=torch.float32, device=dev)
                  for sz in self.sizes]
        self.ckpt = [torch.empty(max(1, c) * sz, dtype=torch.float32,
                                 device=dev)
                     for c, sz in zip(self.n_ckpt, self.sizes)]
        self.diag_off = np.cumsum([0] + [2 ** s.n for s in specs])
        self.target = torch.cat([t.to(dev, torch.float64).reshape(-1)
                                 for t in targets])
        self.prob = torch.empty_like(self.target)
        self.loss = torch.empty(self.n_inst, dtype=torch.float64, device=dev)
        inst = (_Instance * self.n_inst)()
        for i, s in enumerate(specs):
            inst[i] = _Instance(self.x[i].data_ptr(), self.g[i].data_ptr(),
                                self.ckpt[i].data_ptr(), self.sizes[i], s.n,
                                int(self.diag_off[i]))
        self.inst_dev = torch.frombuffer(bytearray(bytes(inst)),
                                         dtype=torch.uint8).to(dev)
        # ---- units (fused ops) and the PTM pool: one slot per unit
        self.fuse = fuse
        self.ops = [s.ops() for s in specs]
        self.units = [plan_units(o, fuse) for o in self.ops]
        self.op_base = np.cumsum([0] + [len(o) for o in self.ops])
        self.n_ops = int(self.op_base[-1])
        self.unit_base = np.cumsum([0] + [len(u) for u in self.units])
        self.n_ptm = int(self.unit_base[-1])
        self._index_units()
        self.ptm = torch.zeros(self.n_ptm, 256, dtype=torch.float32,
                               device=dev)
        self.ptm_inv = torch.zeros_like(self.ptm)
        self.grad = torch.zeros(self.n_ptm, 256, dtype=torch.float64,
                                device=dev)
        # dL/dP per original op (the units' gradients mapped back)
        self.op_grad = torch.zeros(self.n_ops, 256, dtype=torch.float64,
                                   device=dev)
        self._factors = None
        self._cchain = None
        self._fchain = None
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.max_grid = self.lib.qsgb_batch_max_grid(BLOCK)
        if self.max_grid < 1:
            raise RuntimeError('batched kernel cannot be made resident')
        self.tile = tile or self._cached_tile() or 8192
        self._build_program(self.tile)
        self.graph = None

    # ------------------------------------------------------------ program
    def _build_program(self, tile, max_items=64):
        """Device program for the current circuits (`build_program` on the
        host, then uploaded)."""
        items, begin, n_slots = build_program(
            self.units, self.unit_base, self.sizes,
            [s.depth for s in self.specs], self.every, tile, max_items)
        n_main = len(begin) - 2
        dev = self.device
        self.n_stages = n_main + 1
        self.n_items = len(items)
        self.items_dev = torch.from_numpy(items.view(np.uint8).copy()).to(dev)
        self.stage_dev = torch.from_numpy(begin).to(dev)
        self.work = torch.zeros(self.n_stages + 3, dtype=torch.int32,
                                device=dev)
        self.grad_partial = torch.zeros(max(1, n_slots), 256,
                                        dtype=torch.float64, device=dev)
        self.n_slots = n_slots
        prog = _Program()
        prog.instances = self.inst_dev.data_ptr()
        prog.items = self.items_dev.data_ptr()
        prog.stage_begin = self.stage_dev.data_ptr()
        prog.n_stages = self.n_stages
        prog.n_instances = self.n_inst
        prog.work = self.work.data_ptr()
        prog.ptm = self.ptm.data_ptr()
        prog.ptm_inv = self.ptm_inv.data_ptr()
        prog.grad_partial = self.grad_partial.data_ptr()
        prog.grad = self.grad.data_ptr()
        prog.target = self.target.data_ptr()
        prog.prob = self.prob.data_ptr()
        prog.loss = self.loss.data_ptr()
        self.prog = prog
        self.tile = tile
        self.max_items = max_items
        self.graph = None

    def algorithmic_bytes(self):
        """HBM bytes one step must move with FP32 vectors of N entries:
        APPLY of a unit reads and writes the state (8 N), ADJOINT reads x_out
        and g_out and writes x_in and g_in (16 N), SAVE and RESTORE copy it
        (8 N each), INIT and ZERO_G write it (4 N each), LOSS reads the 2^n
        diagonal entries.  PTMs, dP partials and their sums are
        negligible."""
        total = 0
        for i, s in enumerate(self.specs):
            n_units = len(self.units[i])
            total += self.sizes[i] * (24 * n_units + 16 * self.n_ckpt[i] + 8) \
                + 4 * 2 ** s.n
        return total

    def _index_units(self):
        """Flat index arrays of the units: slot and chain of every one-qubit
        unit; slot of every two-qubit unit and, per factor, its C op, its
        two chains and its unit.  The one-qubit chains are listed one-qubit
        units first, then side a, then side b of the factors
        (`chain_products`, `map_unit_gradients`)."""
        one_slot, one_chain = [], []
        two_slot, f_c, f_a, f_b, f_seq = [], [], [], [], []
        for i, units in enumerate(self.units):
            ub, ob = int(self.unit_base[i]), int(self.op_base[i])
            for u, (_, qs, mem) in enumerate(units):
                if len(qs) == 1:
                    one_slot.append(ub + u)
                    one_chain.append(tuple(ob + m for m in mem[0]))
                    continue
                seq = []
                for jc, ca, cb in mem:
                    seq.append(len(f_c))
                    f_c.append(ob + jc)
                    f_a.append(tuple(ob + m for m in ca))
                    f_b.append(tuple(ob + m for m in cb))
                two_slot.append(ub + u)
                f_seq.append(tuple(seq))
        dev = self.device
        as_idx = (lambda v: torch.as_tensor(np.asarray(v, dtype=np.int64),
                                            device=dev))
        self._one_slot = as_idx(one_slot)
        self._two_slot, self._f_c = as_idx(two_slot), as_idx(f_c)
        self._f_c_np = np.asarray(f_c, dtype=np.int64)
        self._chains = one_chain + f_a + f_b
        self._f_seq = f_seq
        self._single = all(len(q) == 1 for q in f_seq)
        self._n_one, self._n_fac = len(one_slot), len(f_c)

    # ------------------------------------------------------------ PTMs
    def set_ptms(self, ptms_per_instance):
        """ptms_per_instance[i][j]: (K, K) float64 PTM of op j of instance i
        (two-qubit ones (16, 16) or (4, 4, 4, 4) in sorted qubit order; any
        device).  Builds the units' PTMs (the product of the factors
        C (A (x) B) for two-qubit units, the chain product for one-qubit
        ones) and their inverses in FP64 on the host, and stores them in
        FP32 on the GPU; keeps the factors (FP64, GPU) for mapping the
        gradients back."""
        flat = [p.detach().to('cpu', torch.float64).reshape(
                    (4, 4) if p.numel() == 16 else (16, 16))
                for ps in ptms_per_instance for p in ps]
        if len(flat) != self.n_ops:
            raise ValueError('expected {} PTMs, got {}'.format(self.n_ops,
                                                              len(flat)))
        dev = self.device
        eye4 = torch.eye(4, dtype=torch.float64)
        one_q = torch.stack([f if f.shape == (4, 4) else eye4 for f in flat])
        prod, cfac = chain_products(one_q, self._chains)
        n1, nf = self._n_one, self._n_fac
        one = prod[:n1]
        a, b = prod[n1:n1 + nf], prod[n1 + nf:]
        fchain = None
        if nf:
            c = torch.stack([flat[j] for j in self._f_c_np])
            kr = torch.einsum('uac,ubd->uabcd', a, b).reshape(-1, 16, 16)
            m = torch.bmm(c, kr)
            if self._single:
                f = m
            else:
                f, ffac = chain_products(m, self._f_seq)
                fchain = tuple(t.to(dev) for t in ffac)
        else:
            c = f = torch.zeros(0, 16, 16, dtype=torch.float64)
        for slots, mm, K in ((self._one_slot, one, 4), (self._two_slot, f, 16)):
            if not len(slots):
                continue
            # inverted on the host in float64: the matrices are tiny, and
            # this keeps the device free of the solver libraries
            inv = torch.linalg.inv(mm)
            pool = torch.zeros(len(slots), 256, dtype=torch.float64)
            ipool = torch.zeros_like(pool)
            pool[:, :K * K] = mm.reshape(len(slots), -1)
            ipool[:, :K * K] = inv.reshape(len(slots), -1)
            self.ptm[slots] = pool.to(dev).float()
            self.ptm_inv[slots] = ipool.to(dev).float()
        self._keep('_factors', (c, a, b))
        self._keep('_cchain', cfac)
        self._keep('_fchain', fchain)

    def _keep(self, name, tensors):
        """Store `tensors` (or None) on the device under `name`: in place
        when the attribute already holds tensors of the same shapes and
        dtypes, so that a captured graph reads the new values; otherwise as
        new tensors, dropping the graph (it would read the old ones)."""
        old = getattr(self, name, None)
        new = None if tensors is None else tuple(
            t.to(self.device) for t in tensors)
        if old is not None and new is not None and len(old) == len(new) and \
                all(o.shape == n.shape and o.dtype == n.dtype
                    for o, n in zip(old, new)):
            for o, n in zip(old, new):
                o.copy_(n)
            return
        if old is not None or new is not None:
            self.graph = None
        setattr(self, name, new)

    def _map_gradients(self):
        """dL/dP of every original op from the units' dL/dF (device, on the
        current stream), by `map_unit_gradients`."""
        c, a, b = self._factors
        g_one = self.grad[self._one_slot, :16].view(-1, 4, 4)
        g_two = self.grad[self._two_slot].view(-1, 16, 16)
        dc, (ops, d) = map_unit_gradients(g_one, g_two, c, a, b,
                                          self._cchain, self._fchain)
        if dc is not None:
            self.op_grad[self._f_c] = dc.reshape(-1, 256)
        if len(ops):
            self.op_grad[ops, :16] = d.reshape(-1, 16)

    # ------------------------------------------------------------ run
    def _launch(self, grid):
        self.work.zero_()
        st = self.lib.qsgb_batch_run(
            ctypes.byref(self.prog), grid, BLOCK, 1 if self.cooperative else 0,
            ctypes.c_void_p(self.status.data_ptr()), 1 << 26,
            ctypes.c_void_p(torch.cuda.current_stream(self.device)
                            .cuda_stream))
        L.check(st, 'qsgb_batch_run')

    def step(self, grid=None, use_graph=True):
        """One forward + adjoint of every instance, and the per-op gradients
        (asynchronous)."""
        if self._factors is None:
            raise RuntimeError('set_ptms() before step()')
        grid = grid or self.max_grid

        def run():
            self._launch(grid)
            self._map_gradients()
        if use_graph:
            if self.graph is None:
                run()  # warm-up outside capture
                torch.cuda.synchronize(self.device)
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g):
                    run()
                self.graph = g
            self.graph.replay()
        else:
            run()

    def check(self):
        val = int(self.status.item())
        if val:
            self.status.zero_()
            raise RuntimeError('batched kernel device status {}'.format(val))

    def results(self):
        """(probabilities per instance, loss per instance, PTM gradients per
        instance as lists of (K, K) float64 tensors)."""
        self.check()
        probs = [self.prob[self.diag_off[i]:self.diag_off[i + 1]]
                 for i in range(self.n_inst)]
        grads = []
        for i, ops in enumerate(self.ops):
            gi = []
            for j, (_, qs) in enumerate(ops):
                K = 4 if len(qs) == 1 else 16
                gi.append(self.op_grad[int(self.op_base[i]) + j, :K * K]
                          .view(K, K))
            grads.append(gi)
        return probs, self.loss, grads

    # ------------------------------------------------------------ autotune
    def _cache_key(self):
        sig = sorted(s.n for s in self.specs)
        return '{}:{}:{}:{}'.format(len(sig), sum(4 ** n for n in sig),
                                    self.max_grid, self.n_ptm)

    @staticmethod
    def _cache_path():
        return os.environ.get('QSGB_AUTOTUNE_CACHE', os.path.join(
            os.path.dirname(os.path.abspath(__file__)), '_build',
            'batch_autotune.json'))

    def _cached_tile(self):
        try:
            with open(self._cache_path()) as f:
                return int(json.load(f)[self._cache_key()]['tile'])
        except Exception:
            return None

    def autotune(self, candidates=(2048, 4096, 8192, 16384, 32768), reps=2):
        """Time one step per tile size, keep the fastest; returns
        {tile: ms}."""
        times = {}
        for t in candidates:
            self._build_program(t)
            self.step(use_graph=False)
            torch.cuda.synchronize(self.device)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                self.step(use_graph=False)
            e1.record()
            torch.cuda.synchronize(self.device)
            times[t] = e0.elapsed_time(e1) / reps
        best = min(times, key=times.get)
        self._build_program(best)
        path = self._cache_path()
        try:
            data = {}
            if os.path.exists(path):
                with open(path) as f:
                    data = json.load(f)
            data[self._cache_key()] = {'tile': best, 'ms': times}
            os.makedirs(os.path.dirname(path), exist_ok=True)
            with open(path, 'w') as f:
                json.dump(data, f, indent=1, default=str)
        except Exception:
            pass
        return times


def plain_gradients(spec, ptms, target, dtype=torch.float32,
                    checkpoint_every=8):
    """The plain GPU path for one instance: ApplyPTM autograd op by op with
    checkpointed layers.  Returns (probabilities, loss, [dL/dP per op])."""
    params = [p.detach().clone().to(torch.float64).requires_grad_()
              for p in ptms]
    x = torch.zeros((4,) * spec.n, dtype=dtype, device='cuda')
    x[(0,) * spec.n] = 1
    ops = spec.ops()
    layers = []
    for l in range(spec.depth):
        idx = [j for j, (ll, _) in enumerate(ops) if ll == l]

        def layer(s, idx=idx):
            for j in idx:
                qs = ops[j][1]
                pt = params[j] if len(qs) == 1 else params[j].view(4, 4, 4, 4)
                s = apply_ptm_diff(s, pt, *qs)
            return s
        layers.append(layer)
    x = checkpointed(layers, x, checkpoint_every)
    prob = diagonal_diff(x, [_bases.general(2)] * spec.n)
    t = target.to(prob.device, torch.float64)
    pe = prob.clamp_min(1e-300)
    loss = torch.sum(torch.where(t > 0, t * (torch.log(t) - torch.log(pe)),
                                 torch.zeros_like(t)))
    loss.backward()
    return prob.detach(), loss.detach(), [p.grad for p in params]


def benchmark(n_instances=512, depth=30, q_min=4, q_max=12, seed=0,
              steps=3, autotune=True, f64_check='all', log=None,
              plain_all=False):
    """The batched configuration: `n_instances` circuits with qubit counts
    uniform in [q_min, q_max], own seeded noise, `depth` layers; FP32 Pauli
    vectors with FP64 probabilities / losses / PTM gradients.

    Returns a dict with the batched gradient-step time (forward + adjoint of
    every instance, one persistent launch replayed from a CUDA graph), the
    plain GPU path's time (one instance at a time through ApplyPTM autograd,
    timed once per qubit count and summed over the instances) and the
    maximum probability error against FP64 (`f64_check`: 'all' instances or
    one per qubit count).  With `plain_all` the plain path is also timed on
    every instance (about 100 s for the default workload).  The gradient
    mapping's share of the step is its own time (CUDA events over repeated
    calls on the same stream) over the step's."""
    say = log or (lambda *a: None)
    rng = np.random.default_rng(seed)
    ns = rng.integers(q_min, q_max + 1, n_instances)
    specs = [CircuitSpec(int(n), depth, 100 + i) for i, n in enumerate(ns)]
    ptms = [instance_ptms(s) for s in specs]
    uniform = [torch.full((2 ** s.n,), 1.0 / 2 ** s.n, dtype=torch.float64)
               for s in specs]
    t0 = time.perf_counter()
    sim = BatchedSimulator(specs, uniform, checkpoint_every=8)
    build_s = time.perf_counter() - t0
    # targets: probabilities of the same circuits with perturbed angles
    sim.set_ptms([instance_ptms(s, angle_offset=torch.from_numpy(
        np.random.default_rng(7 + i).normal(0, 0.05, (depth, s.n))))
        for i, s in enumerate(specs)])
    sim.step(use_graph=False)
    torch.cuda.synchronize()
    sim.target.copy_(sim.prob)
    targets = [t.clone() for t in sim.results()[0]]
    sim.set_ptms(ptms)
    tuned = sim.autotune(candidates=(2048, 8192, 32768), reps=1) \
        if autotune else None
    say('batched: {} stages, {} items, tile {}'.format(
        sim.n_stages, sim.n_items, sim.tile))
    for _ in range(2):
        sim.step(use_graph=True)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        sim.step(use_graph=True)
    e1.record()
    torch.cuda.synchronize()
    step_s = e0.elapsed_time(e1) / 1e3 / steps
    # the torch gradient mapping alone (it follows the kernel in the graph)
    e0.record()
    for _ in range(steps):
        sim._map_gradients()
    e1.record()
    torch.cuda.synchronize()
    map_s = e0.elapsed_time(e1) / 1e3 / steps
    probs, loss, grads = sim.results()
    # plain GPU path, one instance of every qubit count
    plain = {}
    for n in sorted(set(int(v) for v in ns)):
        i = int(np.where(ns == n)[0][0])
        plain_gradients(specs[i], ptms[i], targets[i])
        torch.cuda.synchronize()
        a = time.perf_counter()
        plain_gradients(specs[i], ptms[i], targets[i])
        torch.cuda.synchronize()
        plain[n] = time.perf_counter() - a
    plain_s = float(sum(plain[int(n)] for n in ns))
    plain_all_s = None
    if plain_all:
        torch.cuda.synchronize()
        a = time.perf_counter()
        for i in range(n_instances):
            plain_gradients(specs[i], ptms[i], targets[i])
        torch.cuda.synchronize()
        plain_all_s = time.perf_counter() - a
    # probabilities against FP64 (the exact-arithmetic plain path)
    from .pauli_vector import PauliVectorGB300
    idx = range(n_instances) if f64_check == 'all' else \
        [int(np.where(ns == n)[0][0]) for n in sorted(set(int(v) for v in ns))]
    err = 0.0
    for i in idx:
        s = specs[i]
        pv = PauliVectorGB300([_bases.general(2)] * s.n, force=True)
        for pt, (_, qs) in zip(ptms[i], s.ops()):
            arr = pt.numpy() if len(qs) == 1 else pt.numpy().reshape(4, 4, 4, 4)
            pv.apply_ptm(arr, *qs)
        d = pv.diagonal(get_data=False)
        err = max(err, float((d - probs[i]).abs().max()))
    total_entries = int(sum(4 ** int(n) for n in ns))
    return {
        'instances': n_instances, 'qubits': [q_min, q_max], 'depth': depth,
        'entries_total': total_entries,
        'storage': 'f32 Pauli vectors; f64 probabilities, losses, dL/dPTM',
        'step_s': step_s, 'grad_steps_per_s': 1.0 / step_s,
        'algorithmic_bytes_per_step': sim.algorithmic_bytes(),
        'achieved_gbs': sim.algorithmic_bytes() / step_s / 1e9,
        'plain_step_s_est': plain_s,
        'plain_per_qubits_s': {str(k): v for k, v in plain.items()},
        'speedup_vs_plain': plain_s / step_s,
        'plain_step_s_all_instances': plain_all_s,
        'speedup_vs_plain_all_instances':
            None if plain_all_s is None else plain_all_s / step_s,
        'grad_mapping_s': map_s,
        'grad_mapping_share': map_s / step_s,
        'max_prob_err_vs_f64': err,
        'f64_checked_instances': len(list(idx)),
        'tile': sim.tile, 'autotune_ms': tuned,
        'stages': sim.n_stages, 'items': sim.n_items,
        'ops': sim.n_ops, 'units': sim.n_ptm,
        'fusion': 'each CZ absorbs the rotations waiting on its qubits, '
                  'across layers (F = C (A x B), A and B rotation '
                  'products); per-op gradients mapped back in the same '
                  'graph',
        'program_build_s': build_s,
        'launches_per_step': 1, 'cuda_graph': True,
        'graph_contents': 'the persistent batch kernel, then batched-GEMM '
                          'gradient mapping (torch) on the same stream',
    }

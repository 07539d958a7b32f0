"""Fused circuit execution: a list of PTM units applied with fewer passes
over the Pauli vector.

The reference runs a circuit one unit at a time: ``_Chain.__call__`` calls
every unit's ``PTMOperation.__call__``, which converts the PTM to the
vector's bases and calls ``pauli_vector.apply_ptm``
(quantumsim/operations/operation.py:529-604).  Each call streams the whole
vector through memory once.  On a large state every such pass costs the same
HBM traffic whatever the PTM, so merging units saves passes:

* a one-qudit unit followed by another on the same qudit becomes their
  product;
* a one-qudit unit and the next (or previous) two-qudit unit that touches
  its qudit, with no unit on that qudit in between, become one two-qudit
  PTM (the one-qudit unit commutes with everything in between);
* two two-qudit units on the same pair, with nothing on either qudit in
  between, become their product.

A merge is made only when the time model says the merged PTM is cheaper
than the two passes: an application's time per byte streamed is
interpolated from rates measured on GB300 for the specialised FP64 kernels,
by PTM size and non-zero terms per row (denser rows take more float-float
arithmetic per element, and the 81x81 kernels degrade fastest).  ``plan``
runs two planners, a greedy pass and a search that chooses for every run of
one-qudit units which neighbouring two-qudit unit it joins, and keeps the
plan the model rates faster.  PTM products are formed in FP64 on the host;
the fused result differs from unit-by-unit application by rounding only.

The reference's compiler merges units too when it compiles an operation
for given bases (quantumsim/operations/compiler.py); ``plan`` does the same
job for uncompiled unit lists, with a cost model for this hardware.

``units_of(operation, bases, *qubits)`` turns a reference operation (a
``_Chain`` or a ``PTMOperation``) into the (ptm, qudits) units that its
``__call__`` would apply to a vector with those bases, converting each PTM
to the vector's bases on the way exactly as ``PTMOperation.__call__`` does.

``reduce_bases(units, dims, keep_out)`` shrinks the bases the units work
in to the entries that can be non-zero and are needed afterwards, as the
reference's compiler does for given input and output bases; the reduced
units are rectangular where a basis shrinks.

``FusedCircuit(units)`` plans once; calling it on a ``PauliVectorGB300``
applies the fused PTMs.  ``capture(pv)`` records the fused applications of
one vector into a CUDA graph (a static input and output buffer), so a
circuit that is run many times on states of one shape costs one graph
launch instead of one host call per unit.
"""
import os

import numpy as np
import torch

# Measured application rates of the specialised FP64 kernels on GB300
# (TB/s of the vector streamed in and out) against non-zero terms per PTM
# row, per PTM size K (product of the qudits' Pauli dims); 14 qubits or 8
# qutrits:
#   K = 4:  noisy rotation 2.5 terms/row 5.8; two rotations 3.75 5.0
#   K = 9:  qutrit rotation 2.56 5.5; two rotations 2.78 5.2
#   K = 16: CZ with rotations merged in, every fused pass of the 14-qubit
#           noisy circuit under both planners timed alone (615 passes;
#           harmonic means per density): 1.56 6.49 (noisy CZ), 2.19 6.03,
#           3.12 5.35, 3.75 4.83, 4.38 4.66, 5.0 4.05, 6.25 4.01,
#           7.0 3.53; float-float dense rows 11.25 2.46, 16 1.65 (beyond
#           the tensor-core threshold, for 'df64')
#   K = 81: leakage CZ 2.14 4.7; after one rotation 5.16 2.5; between
#           rotations 12.26 0.80 -- the 81x81 kernels lose registers and
#           instruction cache quickly, so merging into them rarely pays.
# Between points 1/rate is interpolated linearly in the terms per row;
# beyond the last point it continues along the last segment.
_RATES = {
    4: [(1.0, 7.0), (2.5, 5.8), (3.75, 5.0)],
    9: [(1.0, 6.5), (2.56, 5.5), (2.78, 5.2)],
    16: [(1.56, 6.49), (2.19, 6.03), (3.12, 5.35), (3.75, 4.83), (4.38, 4.66),
         (5.0, 4.05), (6.25, 4.01), (7.0, 3.53), (11.25, 2.46), (16.0, 1.65)],
    81: [(1.0, 5.0), (2.14, 4.7), (5.16, 2.5), (12.26, 0.80)],
}


def terms_per_row(m):
    """Non-zero entries per output row that the kernels keep (entries above
    2^-52 of the largest)."""
    a = np.abs(m)
    amax = a.max() if a.size else 0.0
    return float((a > amax * 2.0 ** -52).sum()) / max(1, m.shape[0])


# PTMs with more non-zero terms than this are not specialised at run time
# (the library's limit) and run on the slower generic kernel: never merge
# into one.
MAX_SPECIALISED_TERMS = 1024


# Two-qubit (16 x 16) PTMs with more than TC_MIN_TERMS non-zero terms per
# row run on the tensor cores (the library's QSGB_TC_MIN_TERMS rule) at a
# rate that does not depend on the density: the fused passes of the
# 14-qubit circuit above 8 terms per row ran at 3.13 TB/s (75 passes, 3.07
# to 3.22).
TC_MIN_TERMS = 8.0
TC_RATE = 3.13


def pass_cost(m):
    """Relative time (seconds per TB streamed) of one application of the
    square PTM matrix m (a 16 x 16 matrix is taken to act on two qubits)."""
    k = m.shape[0]
    t = terms_per_row(m)
    if k == 16 and t > TC_MIN_TERMS:
        return 1.0 / TC_RATE
    if t * k > MAX_SPECIALISED_TERMS:
        return float('inf')
    pts = _RATES[min(_RATES, key=lambda kk: abs(kk - k))]
    inv = [(tt, 1.0 / r) for tt, r in pts]
    if t <= inv[0][0]:
        return inv[0][1]
    for (t0, c0), (t1, c1) in zip(inv, inv[1:]):
        if t <= t1:
            return c0 + (c1 - c0) * (t - t0) / (t1 - t0)
    (t0, c0), (t1, c1) = inv[-2], inv[-1]
    return c1 + (c1 - c0) * (t - t1) / (t1 - t0)


class _Unit:
    """A PTM as a square matrix over its qudits (row index (out_0, out_1),
    column index (in_0, in_1), qudit order as given)."""

    __slots__ = ('qudits', 'dims', 'mat', 'ptm', 'count')

    def __init__(self, ptm, qudits):
        ptm = np.ascontiguousarray(ptm, dtype=np.float64)
        n = len(qudits)
        self.qudits = tuple(int(q) for q in qudits)
        self.ptm = ptm
        self.count = 1
        if n in (1, 2) and ptm.shape[:n] == ptm.shape[n:]:
            self.dims = tuple(ptm.shape[:n])
            k = int(np.prod(self.dims))
            self.mat = ptm.reshape(k, k)
        else:  # rectangular or 3+ qudits: applied as given, never merged
            self.dims = None
            self.mat = None

    @property
    def square(self):
        return self.mat is not None

    def set_mat(self, mat):
        self.mat = mat
        self.ptm = mat.reshape(self.dims + self.dims)


def _embed(unit1, pair, dims):
    """The one-qudit matrix of unit1 as a matrix over `pair` (order kept)."""
    a, b = pair
    if unit1.qudits[0] == a:
        return np.kron(unit1.mat, np.eye(dims[1]))
    return np.kron(np.eye(dims[0]), unit1.mat)


def _aligned(unit2, pair):
    """unit2's matrix with its qudits in the order of `pair`."""
    return _aligned_mat(unit2, unit2.mat, pair)


def plan(units):
    """Fuse a list of (ptm, qudits) units; returns the fused list of
    (ptm, qudits) in application order.

    Two planners run and the plan with the lower modelled time is kept
    (the greedy one on a tie): the greedy pass (`_plan_greedy`) and the
    assignment search (`_plan_assigned`), which chooses for every run of
    one-qudit units the neighbour it joins."""
    greedy = _plan_greedy(units)
    assigned = _plan_assigned(units)
    return assigned if plan_cost(assigned) < plan_cost(greedy) else greedy


def plan_cost(fused):
    """Modelled time (seconds per TB streamed, summed over passes) of a
    fused unit list; rectangular units count as one K = 16 pass."""
    t = 0.0
    for ptm, qs in fused:
        n = len(qs)
        if n in (1, 2) and ptm.shape[:n] == ptm.shape[n:]:
            k = int(np.prod(ptm.shape[:n]))
            t += pass_cost(ptm.reshape(k, k))
        else:
            t += 1.0 / _RATES[16][0][1]
    return t


def _gain(merged, parts):
    c = pass_cost(merged)
    return c != float('inf') and c < sum(pass_cost(p) for p in parts)


class _Run:
    """Consecutive one-qudit units on one qudit, merged into one matrix;
    `prev` / `next` are the two-qudit units it may join (the one before it
    on its qudit with nothing in between, and the one after it)."""

    __slots__ = ('q', 'mat', 'last', 'prev', 'next', 'choice')

    def __init__(self, q, mat, last, prev):
        self.q, self.mat, self.last, self.prev = q, mat, last, prev
        self.next = None
        self.choice = 'alone'


def _plan_assigned(units, max_sweeps=30):
    """Fusion by assignment.  Consecutive one-qudit units on a qudit merge
    into runs (while the model says so).  Every run then either stays a
    pass of its own or joins the two-qudit unit just before or just after it
    on its qudit (it commutes with everything in between); the choices are
    made by coordinate descent on the modelled time (each run's best
    option with the others fixed, until nothing changes), from three
    starting points: no run joined, runs preferring the unit after, runs
    preferring the unit before.  Finally two two-qudit units on the same
    pair with nothing else on either qudit in between merge while that is
    cheaper.  Rectangular units and units on more qudits are barriers."""
    U = [_Unit(p, qs) for p, qs in units]
    runs = []
    open_run = {}   # qudit -> run still open (nothing else on the qudit since)
    host_last = {}  # qudit -> last two-qudit unit on it (None after a barrier)
    for i, u in enumerate(U):
        if u.square and len(u.qudits) == 1:
            q = u.qudits[0]
            j = open_run.get(q)
            if j is not None:
                merged = u.mat @ runs[j].mat
                if _gain(merged, [u.mat, runs[j].mat]):
                    runs[j].mat = merged
                    runs[j].last = i
                    continue
            # a second run on the qudit cannot reach the unit before
            runs.append(_Run(q, u.mat, i, host_last.get(q) if j is None else None))
            open_run[q] = len(runs) - 1
            continue
        host = u.square and len(u.qudits) == 2
        for q in u.qudits:
            j = open_run.pop(q, None)
            if j is not None and host:
                runs[j].next = i
            host_last[q] = i if host else None
    hosts = [i for i, u in enumerate(U) if u.square and len(u.qudits) == 2]
    before = {i: [] for i in hosts}
    after = {i: [] for i in hosts}

    def embed(r, i):
        return _embed(_Unit(r.mat, (r.q,)), U[i].qudits, U[i].dims)

    def full(i):
        m = U[i].mat
        for j in before[i]:
            m = m @ embed(runs[j], i)
        for j in after[i]:
            m = embed(runs[j], i) @ m
        return m

    cache = {}

    def host_cost(i):
        key = (i, tuple(before[i]), tuple(after[i]))
        c = cache.get(key)
        if c is None:
            c = cache[key] = pass_cost(full(i))
        return c

    run_cost = [pass_cost(r.mat) for r in runs]

    def set_choice(j, c):
        r = runs[j]
        if r.choice == 'prev':
            after[r.prev].remove(j)
        elif r.choice == 'next':
            before[r.next].remove(j)
        r.choice = c
        if c == 'prev':
            after[r.prev].append(j)
            after[r.prev].sort()
        elif c == 'next':
            before[r.next].append(j)
            before[r.next].sort()

    def local(j):
        r = runs[j]
        c = run_cost[j] if r.choice == 'alone' else 0.0
        if r.prev is not None:
            c += host_cost(r.prev)
        if r.next is not None:
            c += host_cost(r.next)
        return c

    def options(r):
        return ['alone'] + (['prev'] if r.prev is not None else []) + \
            (['next'] if r.next is not None else [])

    def descend():
        for _ in range(max_sweeps):
            changed = False
            for j, r in enumerate(runs):
                cur = r.choice
                best, best_c = cur, local(j)
                for c in options(r):
                    if c == cur:
                        continue
                    set_choice(j, c)
                    lc = local(j)
                    if lc < best_c * (1 - 1e-12):
                        best, best_c = c, lc
                    set_choice(j, cur)
                if best != cur:
                    set_choice(j, best)
                    changed = True
            if not changed:
                break
        return sum(host_cost(i) for i in hosts) + sum(
            run_cost[j] for j, r in enumerate(runs) if r.choice == 'alone')

    best_total, best_choice = None, None
    for start in ('alone', 'next', 'prev'):
        for j, r in enumerate(runs):
            set_choice(j, 'alone')
        if start != 'alone':
            for j, r in enumerate(runs):
                opts = options(r)
                pick = start if start in opts else opts[-1]
                set_choice(j, pick)
        t = descend()
        if best_total is None or t < best_total:
            best_total, best_choice = t, [r.choice for r in runs]
    for j, c in enumerate(best_choice):
        set_choice(j, c)

    # two-qudit units on one pair with nothing else on either qudit between
    mats = {i: full(i) for i in hosts}
    into = {}       # host merged into a later one
    last = {}       # qudit -> ('host', i) or another marker
    alone_end = {r.last: j for j, r in enumerate(runs) if r.choice == 'alone'}
    for i, u in enumerate(U):
        if i in mats:
            a, b = u.qudits
            la, lb = last.get(a), last.get(b)
            if la is not None and la == lb and la[0] == 'host':
                v = la[1]
                merged = mats[i] @ _aligned_mat(U[v], mats[v], u.qudits)
                if _gain(merged, [mats[i], mats[v]]):
                    mats[i] = merged
                    into[v] = i
            last[a] = last[b] = ('host', i)
        elif u.square and len(u.qudits) == 1:
            if i in alone_end:
                last[u.qudits[0]] = ('run', i)
        else:
            for q in u.qudits:
                last[q] = ('other', i)
    out = []
    for i, u in enumerate(U):
        if i in mats:
            if i not in into:
                out.append((mats[i].reshape(u.dims + u.dims), u.qudits))
        elif u.square and len(u.qudits) == 1:
            j = alone_end.get(i)
            if j is not None:
                d = runs[j].mat.shape[0]
                out.append((runs[j].mat.reshape(d, d), (runs[j].q,)))
        else:
            out.append((u.ptm, u.qudits))
    return out


def _aligned_mat(unit2, mat, pair):
    """`mat`, a matrix over unit2's qudits, with its qudits in the order of
    `pair`."""
    if unit2.qudits == tuple(pair):
        return mat
    da, db = unit2.dims  # unit2 is on (pair[1], pair[0])
    m = mat.reshape(da, db, da, db).transpose(1, 0, 3, 2)
    return m.reshape(da * db, da * db)


def _plan_greedy(units):
    """Fuse in one pass over the units: each unit merges into what came
    before when the model says the product is cheaper."""
    out = []
    last = {}  # qudit -> index in `out` of the last unit touching it
    gain = _gain
    for ptm, qudits in units:
        u = _Unit(ptm, qudits)
        if u.square and len(u.qudits) == 1:
            (q,) = u.qudits
            j = last.get(q)
            prev = out[j] if j is not None else None
            if prev is not None and prev.square and prev.dims is not None:
                if len(prev.qudits) == 1:
                    merged = u.mat @ prev.mat
                    if gain(merged, [u.mat, prev.mat]):
                        prev.set_mat(merged)
                        prev.count += 1
                        continue
                else:
                    emb = _embed(u, prev.qudits, prev.dims)
                    merged = emb @ prev.mat
                    if gain(merged, [u.mat, prev.mat]):
                        prev.set_mat(merged)
                        prev.count += 1
                        continue
        elif u.square and len(u.qudits) == 2:
            a, b = u.qudits
            ja, jb = last.get(a), last.get(b)
            # the previous two-qudit unit on the same pair
            if ja is not None and ja == jb and out[ja] is not None and \
                    out[ja].square and len(out[ja].qudits) == 2:
                prev = out[ja]
                merged = u.mat @ _aligned(prev, u.qudits)
                if gain(merged, [u.mat, prev.mat]):
                    u.set_mat(merged)
                    u.count += prev.count
                    out[ja] = None
                    ja = jb = None
            # pending one-qudit units on a or b move forward into u
            for q, j in ((a, ja), (b, jb)):
                if j is None or out[j] is None:
                    continue
                prev = out[j]
                if prev.square and len(prev.qudits) == 1 and \
                        prev.qudits[0] == q:
                    merged = u.mat @ _embed(prev, u.qudits, u.dims)
                    if gain(merged, [u.mat, prev.mat]):
                        u.set_mat(merged)
                        u.count += prev.count
                        out[j] = None
        out.append(u)
        for q in u.qudits:
            last[q] = len(out) - 1
    return [(v.ptm, v.qudits) for v in out if v is not None]


def reduce_bases(units, dims, keep_out=None, tol=2.0 ** -52):
    """Shrink the per-qudit Pauli bases a unit list works in, as the
    reference's compiler does when it compiles an operation for given input
    and output bases (``optimal_bases`` and its propagation,
    quantumsim/operations/compiler.py:303-362, 37-96).

    `units` are (ptm, qudits) in the vector's bases, applied in order to a
    vector of per-qudit Pauli dims `dims`.  `keep_out` (optional, one entry
    per qudit: None for all, else the indices of the final basis whose
    entries the caller needs, e.g. the computational subbasis before a
    measurement) declares what is read afterwards.

    * Forward: the entries that can be non-zero.  After a unit, an output
      index is active when its PTM row has an entry above `tol` times the
      PTM's largest in an active input column (the residue the kernels skip
      anyway); each qudit keeps the projection of that support.
    * Backward: the entries needed.  Before a unit, an input index is needed
      when its PTM column has an entry above the same threshold in a needed
      row.
    * Each unit's output is cut to the indices both active and needed; its
      input columns are the vector's entries at that point (dropped columns
      are either exactly zero or never read, so every kept entry is the same
      sum as without the reduction).

    The reference keeps basis elements carried by singular vectors above a
    cutoff (1e-5 by default); the direct test here drops only what is zero
    to the kernels' own precision.

    Returns (units, kept): the reduced units (rectangular where a qudit's
    basis shrinks) and, per qudit, the indices of the final basis kept
    (None when all are)."""
    n = len(dims)
    us = [(np.ascontiguousarray(p, dtype=np.float64), tuple(int(q) for q in qs))
          for p, qs in units]
    # full per-qudit dims at every cut
    cur = list(dims)
    shapes = []
    for p, qs in us:
        k = len(qs)
        din, dout = p.shape[k:], p.shape[:k]
        if k not in (1, 2) or len(p.shape) != 2 * k:
            raise ValueError('units act on one or two qudits')
        for q, d in zip(qs, din):
            if cur[q] != d:
                raise ValueError('unit on {} expects dim {} where the vector '
                                 'has {}'.format(qs, d, cur[q]))
        shapes.append((tuple(din), tuple(dout)))
        for q, d in zip(qs, dout):
            cur[q] = d
    final = list(cur)

    def sig(p):
        a = np.abs(p)
        m = a.max() if a.size else 0.0
        return a > tol * m if m > 0 else np.zeros(a.shape, dtype=bool)

    def project(mask_nd, k):
        # per-qudit masks of an index set over k qudits
        return [mask_nd.any(axis=tuple(a for a in range(k) if a != j))
                for j in range(k)]

    def outer(masks):
        m = masks[0]
        for mm in masks[1:]:
            m = np.logical_and.outer(m, mm)
        return m

    # forward: active masks after each unit, on its qudits
    act = [np.ones(d, dtype=bool) for d in dims]
    fwd = []
    for (p, qs), (din, dout) in zip(us, shapes):
        k = len(qs)
        s_ = sig(p).reshape(int(np.prod(dout)), int(np.prod(din)))
        cols = outer([act[q] for q in qs]).reshape(-1)
        rows = s_[:, cols].any(axis=1).reshape(dout)
        masks = project(rows, k)
        fwd.append(masks)
        for q, m in zip(qs, masks):
            act[q] = m
    # backward: needed masks before each unit (and after it)
    need = [np.ones(d, dtype=bool) for d in final]
    if keep_out is not None:
        if len(keep_out) != n:
            raise ValueError('keep_out needs one entry per qudit')
        for q, idx in enumerate(keep_out):
            if idx is not None:
                m = np.zeros(final[q], dtype=bool)
                m[np.asarray(idx, dtype=np.int64)] = True
                need[q] = m
    bwd = [None] * len(us)
    for i in range(len(us) - 1, -1, -1):
        (p, qs), (din, dout) = us[i], shapes[i]
        k = len(qs)
        bwd[i] = [need[q].copy() for q in qs]  # needed outputs of unit i
        s_ = sig(p).reshape(int(np.prod(dout)), int(np.prod(din)))
        rows = outer([need[q] for q in qs]).reshape(-1)
        cols = s_[rows, :].any(axis=0).reshape(din)
        for q, m in zip(qs, project(cols, k)):
            need[q] = m
    # rebuild: outputs cut to active and needed, inputs = the vector's
    # entries at that point
    phys = [np.arange(d) for d in dims]  # kept indices per qudit, full basis
    out_units = []
    for i, ((p, qs), (din, dout)) in enumerate(zip(us, shapes)):
        k = len(qs)
        keep = [np.nonzero(f & b)[0] for f, b in zip(fwd[i], bwd[i])]
        # at least one index per qudit keeps the shapes valid (an all-zero
        # output would be a zero vector)
        keep = [kk if len(kk) else np.array([0]) for kk in keep]
        sub = p
        for j in range(k):  # rows of qudit j
            sub = np.take(sub, keep[j], axis=j)
        for j, q in enumerate(qs):  # columns: the vector's entries now
            sub = np.take(sub, phys[q], axis=k + j)
        out_units.append((np.ascontiguousarray(sub), qs))
        for q, kk in zip(qs, keep):
            phys[q] = kk
    kept = [None if len(phys[q]) == final[q] and
            np.array_equal(phys[q], np.arange(final[q])) else phys[q]
            for q in range(n)]
    return out_units, kept


def _keep_indices(bases, bases_out):
    """Per qudit, the indices of `bases[q]` whose elements make up
    `bases_out[q]` (None: all)."""
    if bases_out is None:
        return None
    if len(bases_out) != len(bases):
        raise ValueError('bases_out needs one entry per qudit')
    keep = []
    for b, bo in zip(bases, bases_out):
        if bo is None:
            keep.append(None)
            continue
        vb = np.asarray(b.vectors).reshape(b.dim_pauli, -1)
        idx = []
        for v in np.asarray(bo.vectors).reshape(bo.dim_pauli, -1):
            hit = [i for i in range(b.dim_pauli) if np.allclose(vb[i], v)]
            if not hit:
                raise ValueError('bases_out is not a subbasis of the '
                                 'circuit\'s output basis')
            idx.append(hit[0])
        keep.append(sorted(idx))
    return keep


def units_of(operation, bases, *qubits):
    """(units, bases_after) of a reference quantumsim operation applied to
    `qubits` (default 0..n-1) of a vector whose bases are `bases`.

    Follows ``_Chain.__call__`` and ``PTMOperation.__call__``
    (quantumsim/operations/operation.py:529-551, 600-604): per unit, the PTM
    is converted to the vector's current bases of its qudits when they
    differ from the unit's input bases, applied, and the qudits take the
    unit's output bases."""
    bases = list(bases)
    if not qubits:
        qubits = tuple(range(operation.num_qubits))
    if len(qubits) != operation.num_qubits:
        raise ValueError('This is a {}-qubit operation, but number of qubits '
                         'provided is {}'.format(operation.num_qubits,
                                                 len(qubits)))
    units = []
    for op, idx in operation.units():
        if not hasattr(op, 'set_bases') or not hasattr(op, 'bases_out'):
            raise TypeError('unit {!r} is not a PTM operation'.format(op))
        qs = tuple(qubits[i] for i in idx)
        b_in = tuple(bases[q] for q in qs)
        if tuple(op.bases_in) != b_in:
            op = op.set_bases(bases_in=b_in)
        units.append((np.asarray(op.ptm(op.bases_in, op.bases_out),
                                 dtype=np.float64), qs))
        for q, b in zip(qs, op.bases_out):
            bases[q] = b
    return units, bases


class FusedCircuit:
    """A circuit (list of (ptm, qudits) units, PTMs in the vector's bases)
    planned once and applied with fused PTMs.  `bases_out` (optional, a
    list with one entry per qudit, None to keep) is assigned to the vector's
    bases after the circuit, as the reference's operations do."""

    def __init__(self, units, fuse=True, bases_out=None):
        self.units = [(np.ascontiguousarray(p, dtype=np.float64), tuple(q))
                      for p, q in units]
        self.fused = plan(self.units) if fuse else list(self.units)
        self.bases_out = bases_out
        self._prepared = set()

    @classmethod
    def from_operation(cls, operation, bases, *qubits, fuse=True,
                       bases_out=None, reduce=False):
        """Fused circuit of a reference operation for vectors with
        `bases` (see units_of).  With `bases_out` (one entry per qudit of
        the vector: None, or a subbasis of that qudit's output basis whose
        elements are all the caller reads afterwards, e.g. the computational
        subbasis before a measurement) or `reduce=True`, the units first
        work in the smallest bases that give the same kept entries
        (reduce_bases), as the reference's ``compile(bases_in, bases_out)``
        does; the vector ends in the reduced bases."""
        units, after = units_of(operation, bases, *qubits)
        if reduce or bases_out is not None:
            keep = _keep_indices(after, bases_out)
            units, kept = reduce_bases(units, [b.dim_pauli for b in bases],
                                       keep)
            after = [b if k is None else b.subbasis(list(int(i) for i in k))
                     for b, k in zip(after, kept)]
        return cls(units, fuse=fuse, bases_out=after)

    @property
    def n_units(self):
        return len(self.units)

    @property
    def n_passes(self):
        return len(self.fused)

    def prepare(self, shape, dtype=torch.float64, arith=0, threads=None):
        """Compile the specialised kernels of every fused PTM for a vector of
        `shape` and `dtype` ahead of time, on `threads` host threads at
        once (default: the host's cores, at most 32).  The library compiles
        each sparsity pattern once per process (and caches it on disk), so
        this only moves the work of the first application forward and
        spreads it over the cores."""
        from concurrent.futures import ThreadPoolExecutor
        from . import ops
        jobs, shape = [], tuple(shape)
        for ptm, qudits in self.fused:
            jobs.append((shape, ptm, qudits))
            shape = tuple(ops.apply_geometry(shape, list(qudits),
                                             ptm.shape)[0])
        n = threads or min(32, os.cpu_count() or 1)
        with ThreadPoolExecutor(max_workers=n) as pool:
            list(pool.map(lambda j: ops.prepare_ptm(j[0], dtype, j[1], j[2],
                                                    arith), jobs))
        self._prepared.add((tuple(jobs[0][0]) if jobs else shape, dtype,
                            arith))

    def __call__(self, pv):
        """Apply the circuit to a PauliVectorGB300 (in place).  The first
        call for a vector shape compiles the circuit's kernels in parallel
        (see prepare)."""
        key = (tuple(pv._data.shape), pv._data.dtype, pv._arith)
        if key not in self._prepared:
            self.prepare(*key)
        for ptm, qudits in self.fused:
            pv.apply_ptm(ptm, *qudits)
        if self.bases_out is not None:
            for q, b in enumerate(self.bases_out):
                if b is not None:
                    pv.bases[q] = b
        return pv

    def capture(self, pv):
        """A CUDA-graph replay of this circuit for vectors shaped like pv's
        data; see CircuitGraph."""
        return CircuitGraph(self, pv)


class CircuitGraph:
    """The fused applications of one circuit recorded into a CUDA graph.

    ``run(pv)`` copies pv's data into the graph's static input, replays the
    graph and leaves the result in pv (pv keeps its bases: the circuit must
    map every qudit's basis onto itself, i.e. square PTMs).  The first
    (eager) pass compiles every specialised kernel before capture."""

    def __init__(self, circuit, pv):
        from . import ops
        self.circuit = circuit
        for ptm, qudits in circuit.fused:
            if ptm.shape[:len(qudits)] != ptm.shape[len(qudits):]:
                raise ValueError('captured circuits must map every qudit '
                                 'onto its own basis (square PTMs)')
        self.device = pv._data.device
        self.static_in = pv._data.clone()
        warm = pv.copy()
        circuit(warm)  # compiles the kernels; no capture of compilation
        torch.cuda.synchronize(self.device)
        self.graph = torch.cuda.CUDAGraph()
        stream = torch.cuda.Stream(self.device)
        stream.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(stream):
            x = self.static_in
            with torch.cuda.graph(self.graph, stream=stream):
                for ptm, qudits in circuit.fused:
                    x = torch.ops.qsgb.apply_ptm(
                        x, torch.from_numpy(ptm), list(qudits), pv._arith,
                        0, False)
            self.static_out = x
        torch.cuda.current_stream(self.device).wait_stream(stream)
        ops.check_device_status(self.device)

    def run(self, pv):
        if pv._data.shape != self.static_in.shape or \
                pv._data.dtype != self.static_in.dtype:
            raise ValueError('vector shape or dtype differs from the '
                             'captured one')
        self.static_in.copy_(pv._data)
        self.graph.replay()
        pv._data = self.static_out.clone()
        return pv

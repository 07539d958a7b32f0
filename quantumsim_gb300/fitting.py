"""Differentiable noisy-circuit model: gradients of a measurement loss with
respect to physical gate parameters, through the GB300 adjoint kernels.

The circuit is the CPU-runnable workload family (per layer a rotation on
every qubit followed by amplitude + phase damping over the 20 ns gate time,
then CZs on line neighbours), with trainable physical parameters:

* ``angle_offset`` (n_groups, n): added to the seeded rotation angle of the
  gate on qubit q in every layer l with l % n_groups == g;
* ``t1``, ``t2`` (n,): coherence times in microseconds, setting the damping
  rates (:func:`quantumsim_gb300.ptm.damping_rates`);
* ``cz_phase`` (n - 1,): conditional-phase error of the CZ on edge (i, i+1).

With n = 10 and 22 offset groups this is 220 + 10 + 10 + 9 = 249
parameters.  The loss is KL(target || model) over the diagonal (computational
basis probabilities); the target is the same circuit at perturbed
parameters.  ``loss(..., backend='gb300')`` runs the state through the
``ApplyPTM`` autograd function (adjoint kernels, checkpoints every
`checkpoint_every` layers); ``backend='einsum'`` is the float64
``torch.einsum`` autograd reference used by the tests.
"""
import math

import numpy as np
import torch

from . import bases as _bases
from . import ptm as P
from .autograd import apply_ptm_diff, checkpointed, diagonal_diff

T_GATE = 20e-9


class NoisyCircuitModel:
    def __init__(self, n_qubits=10, n_layers=40, n_groups=22, seed=3):
        self.n = n_qubits
        self.n_layers = n_layers
        self.n_groups = n_groups
        rng = np.random.default_rng(seed)
        self.axes = [['xyz'[i] for i in rng.integers(3, size=n_qubits)]
                     for _ in range(n_layers)]
        self.base_angles = torch.from_numpy(
            rng.uniform(0, 2 * math.pi, (n_layers, n_qubits)))
        t1 = rng.uniform(20, 60, n_qubits)
        t2 = rng.uniform(10, t1)
        self.init = {
            'angle_offset': torch.zeros(n_groups, n_qubits,
                                        dtype=torch.float64),
            't1': torch.from_numpy(t1),
            't2': torch.from_numpy(t2),
            'cz_phase': torch.zeros(n_qubits - 1, dtype=torch.float64),
        }
        self.basis = _bases.general(2)
        self._dev_consts = {}  # device tensors made once (no copies per step)

    def _device_const(self, key, make):
        v = self._dev_consts.get(key)
        if v is None:
            v = make()
            self._dev_consts[key] = v
        return v

    @property
    def n_params(self):
        return sum(v.numel() for v in self.init.values())

    def params(self, requires_grad=True):
        return {k: v.clone().requires_grad_(requires_grad)
                for k, v in self.init.items()}

    def perturbed(self, scale=0.05, seed=11):
        rng = np.random.default_rng(seed)
        out = {}
        for k, v in self.init.items():
            noise = torch.from_numpy(rng.normal(0, scale, v.shape))
            out[k] = v + (noise * v.abs().clamp(min=1.0) if k in ('t1', 't2')
                          else noise)
        return out

    def pairs(self, layer):
        off = layer % 2
        return [(i, i + 1) for i in range(off, self.n - 1, 2)]

    def build_ptms(self, p):
        """All PTMs of the circuit (float64 tensors on the parameters'
        device, differentiable): one-qubit PTMs (n_layers, n, 4, 4) and CZs
        (n - 1, 4, 4, 4, 4)."""
        n, nl = self.n, self.n_layers
        dev = p['angle_offset'].device
        groups = torch.arange(nl, device=dev) % self.n_groups
        base = self._device_const(('angles', str(dev)),
                                  lambda: self.base_angles.to(dev))
        angles = base + p['angle_offset'][groups]
        axes = [ax for row in self.axes for ax in row]
        rot = P.rotations_batched(axes, angles.reshape(-1), self.basis)
        gamma, lam = P.damping_rates(p['t1'] * 1e-6, p['t2'] * 1e-6, T_GATE)
        damp = P.amp_phase_damping_batched(gamma, lam, self.basis)
        one_q = (damp[None] @ rot.reshape(nl, n, 4, 4))
        cz = P.cphase_batched(math.pi + p['cz_phase'], self.basis)
        return one_q, cz

    def layers(self, p, apply_fn, fuse=False):
        """One function per layer, applying its PTMs with apply_fn.  With
        `fuse`, each CZ absorbs the rotations of its two qubits (the CZs of
        a layer are disjoint, so this is exact): one differentiable product
        CZ (R_i (x) R_i+1) per pair, built in torch, and the rotations of
        unpaired qubits alone -- 6 applications per layer instead of 15 for
        10 qubits."""
        return self.layers_of(*self.build_ptms(p), apply_fn, fuse=fuse)

    def layers_of(self, one_q, cz, apply_fn, fuse=False):
        """layers() for given one-qubit and CZ PTM tensors."""
        fns = []
        for l in range(self.n_layers):
            if fuse:
                paired = set()
                ptms2 = []
                for i, _ in self.pairs(l):
                    ptms2.append((P.compose(P.kron(one_q[l, i], one_q[l, i + 1]),
                                            cz[i]), (i, i + 1)))
                    paired.update((i, i + 1))
                ptms1 = [one_q[l, q] if q not in paired else None
                         for q in range(self.n)]
            else:
                ptms1 = [one_q[l, q] for q in range(self.n)]
                ptms2 = [(cz[i], (i, i + 1)) for i, _ in self.pairs(l)]

            def layer(x, ptms1=ptms1, ptms2=ptms2):
                for q, pt in enumerate(ptms1):
                    if pt is not None:
                        x = apply_fn(x, pt, (q,))
                for pt, qs in ptms2:
                    x = apply_fn(x, pt, qs)
                return x
            fns.append(layer)
        return fns

    def schedule(self, fuse=True):
        """The applications of the circuit in order: per layer a list of
        (kind, index, qudits), kind 1 for the one-qubit PTM singles[index]
        and kind 2 for the two-qubit PTM pairs[index] of ``build_units``
        (the order of ``layers``: unpaired rotations, then the pairs)."""
        sched, singles, pairs = [], [], []
        for l in range(self.n_layers):
            ops_l = []
            edges = [i for i, _ in self.pairs(l)]
            paired = {q for i in edges for q in (i, i + 1)} if fuse else set()
            for q in range(self.n):
                if q not in paired:
                    ops_l.append((1, len(singles), (q,)))
                    singles.append((l, q))
            for i in edges:
                ops_l.append((2, len(pairs), (i, i + 1)))
                pairs.append((l, i))
            sched.append(ops_l)
        return sched, singles, pairs

    def build_units(self, p, fuse=True):
        """All PTMs the circuit applies, in batch (a few dozen torch
        operations whatever the depth): one-qubit PTMs (Ns, 4, 4) and
        two-qubit PTMs (Np, 4, 4, 4, 4) indexed by ``schedule(fuse)``; with
        `fuse` each pair PTM is CZ (R_i (x) R_i+1) of its layer."""
        one_q, cz = self.build_ptms(p)
        dev = one_q.device

        def indices():
            _, singles, pairs = self.schedule(fuse)
            return tuple(torch.tensor(v, device=dev) for v in (
                [l for l, _ in singles], [q for _, q in singles],
                [l for l, _ in pairs], [i for _, i in pairs]))
        ls, qs, lp, ip = self._device_const(('units', fuse, str(dev)), indices)
        s = one_q[ls, qs]
        c = cz[ip]
        if fuse:
            k = torch.einsum('nac,nbd->nabcd', one_q[lp, ip], one_q[lp, ip + 1])
            c = (c.reshape(-1, 16, 16) @ k.reshape(-1, 16, 16)).reshape(
                -1, 4, 4, 4, 4)
        return s, c

    def initial_state(self, device, dtype):
        x = torch.zeros((4,) * self.n, dtype=dtype, device=device)
        x[(0,) * self.n] = 1
        return x

    def probabilities(self, p, backend='gb300', dtype=torch.float64,
                      checkpoint_every=8, device=None, arith=None,
                      fuse=False):
        """Computational-basis probabilities of the final state.  `arith`
        (gb300 backend) selects the kernel arithmetic as in
        ``apply_ptm_diff``; the default picks per PTM row."""
        if backend == 'gb300':
            device = device or torch.device('cuda')
            x = self.initial_state(device, dtype)
            kw = {} if arith is None else {'arith': arith}
            x = checkpointed(
                self.layers(p, lambda s, pt, qs: apply_ptm_diff(s, pt, *qs,
                                                                **kw),
                            fuse=fuse),
                x, checkpoint_every)
            return diagonal_diff(x, [self.basis] * self.n)
        device = device or torch.device('cpu')
        x = self.initial_state(device, torch.float64)
        for f in self.layers(p, _einsum_apply, fuse=fuse):
            x = f(x)
        idx = [self.basis.computational_basis_indices[i] for i in range(2)]
        d = x
        for q in range(self.n):
            d = d.index_select(q, torch.tensor(idx, device=device))
        return d.reshape(-1)

    def loss(self, p, target, **kw):
        prob = self.probabilities(p, **kw)
        t = target.to(prob.device)
        return torch.sum(t * (torch.log(t) - torch.log(prob)))


class GraphedGradient:
    """Gradient steps of ``model.loss`` replayed from one CUDA graph.

    The graph holds the whole step: the batched PTM builder
    (``build_units``: rotations, damping, CZs and the fused pair products for
    all layers) from static copies of the parameters, the circuit forward
    with checkpoints every `checkpoint_every` layers, the diagonal, the KL
    loss, the backward pass down to the PTM gradients and on through the
    builder into the static parameters' gradients: about 1,300 kernel
    launches that would otherwise each cost a host call.  Each application's
    PTM is a leaf of its own (a view of a static buffer the builder's output
    is copied into), so the backward pass writes each PTM gradient once,
    with no zero-fill of a stacked tensor per use.  The PTMs stay on the
    device, so the apply kernels read them from device memory; the builder
    makes its constants once per device, so nothing is copied from the host
    and nothing synchronises inside the graph.

    ``step(p)`` copies the parameters in, replays the graph, returns the
    loss as a device scalar and adds the gradients to ``p[name].grad``
    (accumulated, as in ``loss.backward()``)."""

    def __init__(self, model, target, dtype=torch.float64, checkpoint_every=8,
                 fuse=True, device=None):
        from .autograd import Diagonal, diagonal_indices
        self.model = model
        self.dev = torch.device(device) if device is not None else \
            torch.device('cuda', torch.cuda.current_device())
        self.dtype = dtype
        self.every = checkpoint_every
        self.fuse = fuse
        n = model.n
        self.target = target.to(self.dev, torch.float64)
        self.x0 = model.initial_state(self.dev, dtype)
        self.flat = torch.from_numpy(
            diagonal_indices([model.basis] * n)).to(self.dev)
        self.idx_off, self.idx_list = [0], []
        for _ in range(n):
            self.idx_list += [int(model.basis.computational_basis_indices[i])
                              for i in range(2)]
            self.idx_off.append(len(self.idx_list))
        self._diag = Diagonal
        self.sched = model.schedule(fuse)[0]
        # static parameters (leaves of the builder inside the graph)
        self.sp = {k: v.detach().to(self.dev).clone().requires_grad_(True)
                   for k, v in model.init.items()}
        with torch.no_grad():
            s0, c0 = model.build_units(self.sp, fuse)
        self.s_buf = s0.detach().clone()
        self.c_buf = c0.detach().clone()
        self.s_leaves = [self.s_buf[i].detach().requires_grad_(True)
                         for i in range(self.s_buf.shape[0])]
        self.c_leaves = [self.c_buf[i].detach().requires_grad_(True)
                         for i in range(self.c_buf.shape[0])]
        # warm up on a side stream (compiles nothing: device PTMs use the
        # precompiled kernels, the builder's constants are made here), then
        # capture
        side = torch.cuda.Stream(self.dev)
        side.wait_stream(torch.cuda.current_stream(self.dev))
        with torch.cuda.stream(side):
            for _ in range(2):
                self._clear()
                self._step_body()
            self._clear()
            self.graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self.graph, stream=side):
                self.loss = self._step_body()
                self.p_grad = {k: v.grad for k, v in self.sp.items()}
        torch.cuda.current_stream(self.dev).wait_stream(side)

    def _clear(self):
        for t in self.s_leaves + self.c_leaves + list(self.sp.values()):
            t.grad = None

    def _step_body(self):
        """Builder, circuit, loss, backward to the static parameters."""
        s, c = self.model.build_units(self.sp, self.fuse)
        with torch.no_grad():
            self.s_buf.copy_(s)
            self.c_buf.copy_(c)
        loss = self._loss()
        loss.backward()
        s_grad = torch.stack([t.grad for t in self.s_leaves])
        c_grad = torch.stack([t.grad for t in self.c_leaves])
        torch.autograd.backward([s, c], [s_grad, c_grad])
        return loss

    def _loss(self):
        leaves = {1: self.s_leaves, 2: self.c_leaves}
        fns = []
        for ops_l in self.sched:
            def layer(x, ops_l=ops_l):
                for kind, i, qs in ops_l:
                    x = apply_ptm_diff(x, leaves[kind][i], *qs)
                return x
            fns.append(layer)
        x = checkpointed(fns, self.x0.clone(), self.every)
        prob = self._diag.apply(x, self.flat, self.idx_off, self.idx_list)
        t = self.target
        return torch.sum(t * (torch.log(t) - torch.log(prob)))

    def step(self, p):
        with torch.no_grad():
            for k, v in self.sp.items():
                v.copy_(p[k])
        self.graph.replay()
        with torch.no_grad():
            for k, v in p.items():
                if not v.requires_grad:
                    continue
                g = self.p_grad[k].to(v.device)
                if v.grad is None:
                    v.grad = g.clone()
                else:
                    v.grad += g
        return self.loss


def _einsum_apply(x, ptm, qs):
    """Float64 torch.einsum reference of apply_ptm (autograd-capable)."""
    ptm = ptm.to(x.device)
    n = x.dim()
    k = len(qs)
    letters = 'abcdefghijklmnopqrstuvwxyz'
    xi = list(letters[:n])
    outs = [letters[n + i] for i in range(k)]
    yi = list(xi)
    for q, o in zip(qs, outs):
        yi[q] = o
    spec = '{},{}->{}'.format(''.join(outs + [xi[q] for q in qs]),
                              ''.join(xi), ''.join(yi))
    return torch.einsum(spec, ptm, x)

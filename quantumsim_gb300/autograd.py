"""Reverse-mode differentiation through the GB300 kernels.

``ApplyPTM`` is a ``torch.autograd.Function`` around the apply kernel:

* forward:  out = P . x (PTM on the given qudits, any positions, rectangular)
* backward: dL/dx = P^T . dL/dout  -- the same kernel with the PTM
            transposed (QSGB_PTM_TRANSPOSED), specialised at run time to the
            transposed sparsity pattern;
            dL/dP = sum over bystanders of dL/dout (x) x  -- the tall-skinny
            reduction of ``qsgb_ptm_grad*`` (FP64 accumulation).

The PTM is a float64 tensor (usually built on the host by
:mod:`quantumsim_gb300.ptm` from physical parameters, so gradients continue
into T1, T2, angles...).  The state may be float64 or float32; the PTM
gradient is float64 either way.

``Diagonal`` is the differentiable diagonal of a Pauli vector in bases whose
computational-basis rows are unit vectors (gather forward, scatter
backward).

``checkpointed(fn, segments)`` runs a list of layer functions keeping only
the states at segment boundaries; each segment's forward is recomputed
during the backward pass (torch.utils.checkpoint).
"""
import math

import numpy as np
import torch
import torch.utils.checkpoint

from . import _lib as L
from . import ops


class ApplyPTM(torch.autograd.Function):
    """out = apply_ptm(x, ptm, qudits) with gradients for x and ptm."""

    @staticmethod
    def forward(ctx, x, ptm, qudits, arith):
        if ptm.is_cuda:
            # a PTM built on the device stays there: the generic kernel reads
            # it, nothing synchronises, and the call can be captured in a
            # CUDA graph
            ptm_k = ptm.detach().to(torch.float64).contiguous()
        else:
            # a host PTM: its sparsity pattern selects a specialised kernel
            ptm_k = ptm.detach().to('cpu', torch.float64).contiguous()
        max_terms = 0  # all entries (device) / counted by the library (host)
        out = torch.ops.qsgb.apply_ptm(x.contiguous(), ptm_k, list(qudits),
                                       arith, max_terms, False)
        ctx.save_for_backward(x)
        ctx.ptm_host = ptm_k
        ctx.ptm_device = ptm.device
        ctx.qudits = tuple(qudits)
        ctx.arith = arith
        ctx.max_terms = max_terms
        return out

    @staticmethod
    def backward(ctx, g):
        (x,) = ctx.saved_tensors
        g = g.contiguous()
        gx = gp = None
        if ctx.needs_input_grad[0]:
            gx = torch.ops.qsgb.apply_ptm(g, ctx.ptm_host, list(ctx.qudits),
                                          ctx.arith, ctx.max_terms, True)
        if ctx.needs_input_grad[1]:
            gp = torch.ops.qsgb.ptm_grad(x.contiguous(), g, list(ctx.qudits))
            gp = gp.to(ctx.ptm_device)
        return gx, gp, None, None


def apply_ptm_diff(x, ptm, *qudits, arith=L.ARITH_AUTO):
    """Differentiable PTM application on a state tensor (shape dim_pauli)."""
    if x.dtype == torch.float32:
        arith = L.ARITH_F32
    return ApplyPTM.apply(x, ptm, tuple(qudits), arith)


def diagonal_indices(bases):
    """Flat Pauli-vector index of every diagonal element (row-major over the
    Hilbert indices), for bases whose computational-basis rows are unit
    vectors; raises ValueError otherwise."""
    per = []
    for b in bases:
        idx = [b.computational_basis_indices[i] for i in range(b.dim_hilbert)]
        if any(i is None for i in idx):
            raise ValueError('basis without unit computational vectors')
        per.append(idx)
    dims = [b.dim_pauli for b in bases]
    strides = [math.prod(dims[i + 1:]) for i in range(len(dims))]
    flat = np.zeros(1, dtype=np.int64)
    for idx, st in zip(per, strides):
        flat = (flat[:, None] + np.asarray(idx, dtype=np.int64)[None, :] *
                st).reshape(-1)
    return flat


class Diagonal(torch.autograd.Function):
    """Diagonal (FP64) of a Pauli vector: gather forward, scatter back."""

    @staticmethod
    def forward(ctx, x, flat_idx, idx_off, idx_list):
        d = torch.ops.qsgb.gather(x.contiguous(), idx_off, idx_list, True)
        ctx.save_for_backward(flat_idx)
        ctx.shape = x.shape
        ctx.dtype = x.dtype
        return d

    @staticmethod
    def backward(ctx, g):
        (flat_idx,) = ctx.saved_tensors
        gx = torch.zeros(math.prod(ctx.shape), dtype=ctx.dtype,
                         device=g.device)
        gx.index_copy_(0, flat_idx, g.to(ctx.dtype))
        return gx.view(ctx.shape), None, None, None


def diagonal_diff(x, bases):
    """Differentiable diagonal() (length prod(d_hilbert), float64)."""
    flat = torch.from_numpy(diagonal_indices(bases)).to(x.device)
    idx_off, idx_list = [0], []
    for b in bases:
        idx_list += [int(b.computational_basis_indices[i])
                     for i in range(b.dim_hilbert)]
        idx_off.append(len(idx_list))
    return Diagonal.apply(x, flat, idx_off, idx_list)


def checkpointed(layers, x, every=8):
    """Apply `layers` (callables state -> state) in order, keeping only the
    states at every `every`-th layer for the backward pass; the forward of
    each segment is recomputed when its gradient is needed (the layers draw
    no random numbers, so no RNG state is saved, which also keeps the
    checkpoints capturable in a CUDA graph)."""
    if every <= 0 or not torch.is_grad_enabled():
        for f in layers:
            x = f(x)
        return x
    for start in range(0, len(layers), every):
        seg = layers[start:start + every]

        def run(state, seg=seg):
            for f in seg:
                state = f(state)
            return state

        x = torch.utils.checkpoint.checkpoint(run, x, use_reentrant=False,
                                              preserve_rng_state=False)
    return x

"""Reverse mode through the GB300 kernels: the adjoint of apply_ptm (state
gradient = transposed PTM on the GPU, PTM gradient = tall-skinny
reduction), the differentiable diagonal, checkpointed recomputation, and the
249-parameter noisy-circuit model -- checked against a float64 torch.einsum
autograd reference and central finite differences (h = 1e-6)."""
import math

import numpy as np
import pytest
import torch

from quantumsim_gb300 import _lib as L
from quantumsim_gb300 import autograd as AG
from quantumsim_gb300 import fitting
from quantumsim_gb300.fitting import _einsum_apply

pytestmark = pytest.mark.gpu
DEV = torch.device('cuda')


def _rand(rng, shape):
    return torch.from_numpy(rng.standard_normal(shape))


@pytest.mark.parametrize('shape,qs,pshape', [
    ((4, 4, 4, 4), (2,), (4, 4)),
    ((4, 4, 4, 4), (3, 0), (4, 4, 4, 4)),
    ((4, 3, 4, 9), (1,), (2, 3)),
    ((4, 3, 4, 9), (3, 1), (9, 2, 9, 3)),
])
def test_apply_ptm_gradients_match_einsum(shape, qs, pshape):
    rng = np.random.default_rng(31)
    x0 = _rand(rng, shape)
    p0 = _rand(rng, pshape)
    w = None
    grads = {}
    for backend in ('gb300', 'einsum'):
        x = (x0.to(DEV) if backend == 'gb300' else x0.clone()).requires_grad_()
        p = p0.clone().requires_grad_()
        y = (AG.apply_ptm_diff(x, p, *qs) if backend == 'gb300'
             else _einsum_apply(x, p, qs))
        if w is None:
            w = _rand(rng, tuple(y.shape))
        (y * w.to(y.device)).sum().backward()
        grads[backend] = (x.grad.cpu(), p.grad.cpu())
    np.testing.assert_allclose(grads['gb300'][0], grads['einsum'][0],
                               rtol=1e-11, atol=1e-12)
    np.testing.assert_allclose(grads['gb300'][1], grads['einsum'][1],
                               rtol=1e-11, atol=1e-11)


def test_diagonal_gradient_is_scatter():
    from quantumsim_gb300 import bases as B
    rng = np.random.default_rng(32)
    x = _rand(rng, (4, 4, 4)).to(DEV).requires_grad_()
    d = AG.diagonal_diff(x, [B.general(2)] * 3)
    g = _rand(rng, (8,)).to(DEV)
    (d * g).sum().backward()
    expect = torch.zeros(4, 4, 4, dtype=torch.float64)
    expect[:2, :2, :2] = g.cpu().view(2, 2, 2)
    assert torch.equal(x.grad.cpu(), expect)


def _flat(grads):
    return torch.cat([g.reshape(-1) for g in grads])


def test_model_gradients_small_match_reference_and_fd():
    m = fitting.NoisyCircuitModel(n_qubits=5, n_layers=9, n_groups=4, seed=5)
    target = m.probabilities(m.perturbed(), backend='einsum').detach()
    names = list(m.init)
    out = {}
    for backend in ('gb300', 'einsum'):
        p = m.params()
        loss = m.loss(p, target, backend=backend, checkpoint_every=3)
        loss.backward()
        out[backend] = (loss.item(), _flat([p[k].grad for k in names]))
    assert out['gb300'][0] == pytest.approx(out['einsum'][0], rel=1e-11)
    np.testing.assert_allclose(out['gb300'][1], out['einsum'][1], rtol=1e-8,
                               atol=1e-12)
    # central finite differences on a few parameters, through the GPU with
    # native FP64 arithmetic (a loss error e moves the difference quotient
    # by e / h, so the forward must be as accurate as numpy's)
    h = 1e-6
    base = m.params(requires_grad=False)
    checks = [('angle_offset', (1, 2)), ('t1', (3,)), ('t2', (0,)),
              ('cz_phase', (1,))]
    offs = {k: 0 for k in names}
    o = 0
    for k in names:
        offs[k] = o
        o += base[k].numel()
    for k, idx in checks:
        vals = []
        for sgn in (1, -1):
            q = {kk: vv.clone() for kk, vv in base.items()}
            q[k][idx] += sgn * h
            with torch.no_grad():
                vals.append(float(m.loss(q, target, backend='gb300',
                                         arith=L.ARITH_F64)))
        fd = (vals[0] - vals[1]) / (2 * h)
        flat_i = offs[k] + int(np.ravel_multi_index(idx, base[k].shape))
        ad = float(out['gb300'][1][flat_i])
        assert ad == pytest.approx(fd, rel=2e-5, abs=1e-9), (k, idx, ad, fd)


def test_model_full_size_249_parameters():
    """10 qubits, 40 layers, 249 parameters, checkpoints every 8 layers:
    GPU adjoint gradients vs the float64 torch.einsum autograd reference,
    and the FP32-storage gradients within 1e-4 of them."""
    m = fitting.NoisyCircuitModel()
    assert m.n_params == 249
    target = m.probabilities(m.perturbed(), backend='gb300').detach()
    names = list(m.init)
    res = {}
    for backend, dtype in (('gb300', torch.float64), ('einsum', None),
                           ('gb300_f32', torch.float32)):
        p = m.params()
        kw = dict(backend='gb300' if backend.startswith('gb300') else 'einsum')
        if dtype is not None:
            kw['dtype'] = dtype
        loss = m.loss(p, target, checkpoint_every=8, **kw)
        loss.backward()
        res[backend] = (loss.item(), _flat([p[k].grad for k in names]))
    g64, gref, g32 = res['gb300'][1], res['einsum'][1], res['gb300_f32'][1]
    np.testing.assert_allclose(g64, gref, rtol=1e-8, atol=1e-12)
    scale = gref.abs().max()
    assert float((g32 - gref).abs().max() / scale) < 1e-4


def test_model_fused_layers_full_size():
    """The 249-parameter model with each CZ absorbing its qubits' rotations
    (6 applications per layer instead of 15): GPU adjoint gradients against
    the unfused float64 torch.einsum reference."""
    m = fitting.NoisyCircuitModel()
    target = m.probabilities(m.perturbed(), backend='gb300').detach()
    names = list(m.init)
    res = {}
    for backend, fuse in (('gb300', True), ('einsum', False)):
        p = m.params()
        loss = m.loss(p, target, backend=backend, fuse=fuse,
                      checkpoint_every=8)
        loss.backward()
        res[backend] = (loss.item(), _flat([p[k].grad for k in names]))
    assert res['gb300'][0] == pytest.approx(res['einsum'][0], rel=1e-10)
    np.testing.assert_allclose(res['gb300'][1], res['einsum'][1], rtol=1e-8,
                               atol=1e-12)


def test_graphed_gradient_step_matches_reference():
    """The gradient step replayed from a CUDA graph (PTMs built on the GPU,
    circuit forward + loss + backward captured once): the 249-parameter
    gradients at two different parameter points, each against the float64
    torch.einsum autograd reference, and two replays at one point equal bit
    for bit."""
    m = fitting.NoisyCircuitModel()
    target = m.probabilities(m.perturbed(), backend='gb300').detach()
    names = list(m.init)
    step = fitting.GraphedGradient(m, target, checkpoint_every=8, fuse=True)
    dev = step.dev
    for point in (m.init, m.perturbed(scale=0.02, seed=5)):
        grads = []
        for _ in range(2):
            p = {k: v.detach().clone().to(dev).requires_grad_(True)
                 for k, v in point.items()}
            loss = step.step(p)
            grads.append((float(loss.detach()),
                          _flat([p[k].grad for k in names])))
        assert grads[0][0] == grads[1][0]
        assert torch.equal(grads[0][1], grads[1][1])
        pr = {k: v.detach().clone().requires_grad_(True)
              for k, v in point.items()}
        ref = m.loss(pr, target, backend='einsum', fuse=False)
        ref.backward()
        assert grads[0][0] == pytest.approx(float(ref.detach()), rel=1e-10)
        np.testing.assert_allclose(grads[0][1].cpu(),
                                   _flat([pr[k].grad for k in names]),
                                   rtol=1e-8, atol=1e-12)

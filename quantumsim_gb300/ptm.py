"""PTM construction from physical parameters, differentiable in PyTorch.

Pauli transfer matrices in the basis convention of the Pauli vector:
``PTM[x, y] = sum_k Re tr(P_x K_k P_y K_k^dagger)`` with P the (tensor
product) basis elements of the output / input bases -- the contraction of
quantumsim/algebra/algebra.py:11-30 (``kraus_to_ptm``).  Multi-qudit PTMs
are returned with shape (d_out_0, d_out_1, d_in_0, d_in_1), qudit 0 first.

Gate constructors restate quantumsim/operations/qubits.py:38-220 and
quantumsim/operations/qutrits.py:38-291 (rotations, damping, cphase) as
functions of tensors, so gradients flow from physical parameters (rotation
angle, T1, T2, conditional phase) to the PTM.  Every function accepts Python
floats or 0-d tensors; the result is a float64 tensor on the parameters'
device (CPU for floats).  ``.numpy()`` gives the host PTM for
``apply_ptm``.

Rates from coherence times (the mapping this module defines; the reference
takes rates directly): over a duration t,
  amplitude damping   gamma  = 1 - exp(-t / T1)
  pure dephasing      lambda = 1 - exp(-2 t / T_phi),
                      1 / T_phi = 1 / T2 - 1 / (2 T1)
so that coherences decay as exp(-t / T2) overall.
"""
import math

import numpy as np
import torch

from . import bases as _bases

_CDTYPE = torch.complex128


def _t(x, ref=None):
    if isinstance(x, torch.Tensor):
        return x.to(torch.float64)
    dev = ref.device if isinstance(ref, torch.Tensor) else 'cpu'
    return torch.tensor(float(x), dtype=torch.float64, device=dev)


# Device constants made once per device (and contents), so that building
# PTMs issues no host-to-device copy: the batched builders can then be
# captured in a CUDA graph.
_CONSTS = {}


def _const(key, make):
    v = _CONSTS.get(key)
    if v is None:
        if len(_CONSTS) > 4096:
            _CONSTS.clear()
        v = make()
        _CONSTS[key] = v
    return v


def _imag_unit(device):
    return _const(('1j', str(device)),
                  lambda: torch.tensor(1j, dtype=_CDTYPE, device=device))


def _basis_tensor(bases, device):
    """Kronecker product of the basis vectors: (prod dim_pauli, D, D),
    cached per device and basis contents."""
    key = ('basis', str(device)) + tuple(
        (np.asarray(b.vectors).shape, np.asarray(b.vectors).tobytes())
        for b in bases)
    return _const(key, lambda: _basis_tensor_make(bases, device))


def _basis_tensor_make(bases, device):
    vecs = None
    for b in bases:
        v = torch.as_tensor(np.asarray(b.vectors), dtype=_CDTYPE, device=device)
        vecs = v if vecs is None else torch.einsum(
            'aij,bkl->abikjl', vecs, v).reshape(
                vecs.shape[0] * v.shape[0], vecs.shape[1] * v.shape[1],
                vecs.shape[2] * v.shape[2])
    return vecs


def kraus_to_ptm(kraus, bases_in, bases_out=None):
    """PTM of the channel rho -> sum_k K_k rho K_k^dagger.

    kraus: (n_kraus, D, D) or (D, D) complex tensor/array, D = prod of
    the Hilbert dimensions.  Returns float64, shape (d_out..., d_in...)."""
    bases_out = bases_out or bases_in
    k = torch.as_tensor(kraus)
    if not k.is_complex():
        k = k.to(torch.float64)
    k = k.to(_CDTYPE)
    if k.dim() == 2:
        k = k.unsqueeze(0)
    p_out = _basis_tensor(bases_out, k.device)
    p_in = _basis_tensor(bases_in, k.device)
    ptm = torch.einsum('xij,kjl,ylm,kim->xy', p_out, k, p_in, k.conj()).real
    shape = [b.dim_pauli for b in bases_out] + [b.dim_pauli for b in bases_in]
    return ptm.reshape(shape)


def compose(*ptms):
    """PTM of applying ptms[0], then ptms[1], ... (same qudits)."""
    n = ptms[0].dim() // 2
    out_shape = ptms[-1].shape[:n]
    acc = None
    for p in ptms:
        dout = math.prod(p.shape[:n])
        din = math.prod(p.shape[n:])
        m = p.reshape(dout, din)
        acc = m if acc is None else m @ acc
    return acc.reshape(tuple(out_shape) + tuple(ptms[0].shape[n:]))


def kron(p0, p1):
    """Two-qudit PTM of independent one-qudit PTMs on qudit 0 and 1."""
    return torch.einsum('ac,bd->abcd', p0, p1)


# ----------------------------------------------------------------- qubits
def _rot_kraus(axis, angle, dim=2):
    a = _t(angle)
    c = torch.cos(a / 2).to(_CDTYPE)
    s = torch.sin(a / 2).to(_CDTYPE)
    one = torch.ones((), dtype=_CDTYPE, device=a.device)
    zero = torch.zeros((), dtype=_CDTYPE, device=a.device)
    j = torch.tensor(1j, dtype=_CDTYPE, device=a.device)
    if axis == 'x':
        m2 = [[c, -j * s], [-j * s, c]]
    elif axis == 'y':
        m2 = [[c, -s], [s, c]]
    elif axis == 'z':
        e = torch.exp(-j * a.to(_CDTYPE) / 2)
        m2 = [[e, zero], [zero, e.conj()]]
    else:
        raise ValueError('axis must be x, y or z, got {!r}'.format(axis))
    rows = [list(r) + [zero] * (dim - 2) for r in m2]
    for i in range(2, dim):
        rows.append([zero] * i + [one] + [zero] * (dim - i - 1))
    return torch.stack([torch.stack(r) for r in rows])


def rotate(axis, angle, basis=None):
    """Rotation about x, y or z (qubits.py:38-92; for a qutrit basis the
    rotation acts in the 0-1 subspace, qutrits.py:38-92)."""
    basis = basis or _bases.general(2)
    return kraus_to_ptm(_rot_kraus(axis, angle, basis.dim_hilbert), (basis,))


def amp_damping(gamma, basis=None):
    """Qubit amplitude damping with total rate gamma (qubits.py:177-181)."""
    basis = basis or _bases.general(2)
    g = _t(gamma)
    z = torch.zeros_like(g)
    k0 = torch.stack([torch.stack([torch.ones_like(g), z]),
                      torch.stack([z, torch.sqrt(1 - g)])])
    k1 = torch.stack([torch.stack([z, torch.sqrt(g)]), torch.stack([z, z])])
    return kraus_to_ptm(torch.stack([k0, k1]), (basis,))


def phase_damping(lam, basis=None):
    """Qubit phase damping with total rate lam (qubits.py:198-202)."""
    basis = basis or _bases.general(2)
    g = _t(lam)
    z = torch.zeros_like(g)
    k0 = torch.stack([torch.stack([torch.ones_like(g), z]),
                      torch.stack([z, torch.sqrt(1 - g)])])
    k1 = torch.stack([torch.stack([z, z]), torch.stack([z, torch.sqrt(g)])])
    return kraus_to_ptm(torch.stack([k0, k1]), (basis,))


def amp_phase_damping(gamma, lam, basis=None):
    """Amplitude damping followed by phase damping (qubits.py:217-220)."""
    return compose(amp_damping(gamma, basis), phase_damping(lam, basis))


def damping_rates(t1, t2, duration):
    """(gamma, lambda) for a gate of `duration` on a qubit with T1, T2."""
    t1, t2, t = _t(t1), _t(t2), _t(duration)
    gamma = 1 - torch.exp(-t / t1)
    inv_tphi = 1 / t2 - 1 / (2 * t1)
    lam = 1 - torch.exp(-2 * t * inv_tphi)
    return gamma, lam


def cphase(angle=math.pi, basis=None):
    """Controlled phase diag(1, 1, 1, e^{i angle}) (qubits.py:107-121)."""
    basis = basis or _bases.general(2)
    a = _t(angle)
    j = torch.tensor(1j, dtype=_CDTYPE, device=a.device)
    one = torch.ones((), dtype=_CDTYPE, device=a.device)
    diag = torch.stack([one, one, one, torch.exp(j * a.to(_CDTYPE))])
    return kraus_to_ptm(torch.diag(diag), (basis, basis))


def noisy_rotation(axis, angle, t1, t2, duration, basis=None):
    """Rotation followed by amplitude + phase damping over the gate time."""
    gamma, lam = damping_rates(t1, t2, duration)
    return compose(rotate(axis, angle, basis),
                   amp_phase_damping(gamma, lam, basis))


def noisy_cphase(angle, t1a, t2a, t1b, t2b, duration, basis=None):
    """cphase followed by amplitude + phase damping on both qubits."""
    ga, la = damping_rates(t1a, t2a, duration)
    gb, lb = damping_rates(t1b, t2b, duration)
    damp = kron(amp_phase_damping(ga, la, basis),
                amp_phase_damping(gb, lb, basis))
    return compose(cphase(angle, basis), damp)


# ----------------------------------------------------------------- qutrits
def qutrit_amp_damping(p0_up, p1_up, p1_down, p2_down, basis=None):
    """Incoherent excitation / relaxation among |0>, |1>, |2>
    (qutrits.py:267-291): identity on coherences, a stochastic 3x3 block on
    the populations.  `basis` must be general(3) ordering (populations
    first)."""
    basis = basis or _bases.general(3)
    vals = [_t(v) for v in (p0_up, p1_up, p1_down, p2_down)]
    p0u, p1u, p1d, p2d = vals
    dev = p0u.device
    ptm = torch.eye(9, dtype=torch.float64, device=dev)
    one = torch.ones((), dtype=torch.float64, device=dev)
    zero = torch.zeros((), dtype=torch.float64, device=dev)
    block = torch.stack([
        torch.stack([one - p0u, p1d, zero]),
        torch.stack([p0u, one - p1d - p1u, p2d]),
        torch.stack([zero, p1u, one - p2d])])
    ptm = torch.cat([torch.cat([block, ptm[:3, 3:]], 1), ptm[3:]], 0)
    return ptm


def qutrit_cphase(angle=math.pi, leakage=0.0, basis=None):
    """Two-qutrit CZ with leakage |11> <-> |02> (qutrits.py:200-220,
    'legacy' model): exp(-i angle f D) with D coupling indices 2 and 4 of
    the 9-dim space and f = 1 - arcsin(sqrt(leakage)) / pi."""
    basis = basis or _bases.general(3)
    a = _t(angle)
    lk = _t(leakage, a)
    theta = a * (1 - torch.asin(torch.sqrt(lk)) / math.pi)
    c = torch.cos(theta).to(_CDTYPE)
    s = torch.sin(theta).to(_CDTYPE)
    j = torch.tensor(1j, dtype=_CDTYPE, device=a.device)
    u = torch.eye(9, dtype=_CDTYPE, device=a.device)
    u = u.index_put((torch.tensor([2, 4, 2, 4]), torch.tensor([2, 4, 4, 2])),
                    torch.stack([c, c, -j * s, -j * s]))
    return kraus_to_ptm(u, (basis, basis))


def selection_ptm(d_in, indices):
    """Rectangular PTM keeping the Pauli elements `indices` (the oracle form
    of reduce_basis / project)."""
    return np.eye(d_in)[list(indices)]


# ----------------------------------------------------------------- batched
def kraus_to_ptm_batched(kraus, bases_in, bases_out=None):
    """PTMs of a batch of channels: kraus (G, n_kraus, D, D) complex ->
    (G, d_out..., d_in...) float64."""
    bases_out = bases_out or bases_in
    k = torch.as_tensor(kraus).to(_CDTYPE)
    p_out = _basis_tensor(bases_out, k.device)
    p_in = _basis_tensor(bases_in, k.device)
    ptm = torch.einsum('xij,gkjl,ylm,gkim->gxy', p_out, k, p_in, k.conj()).real
    shape = ([k.shape[0]] + [b.dim_pauli for b in bases_out] +
             [b.dim_pauli for b in bases_in])
    return ptm.reshape(shape)


def rotations_batched(axes, angles, basis=None):
    """Rotation PTMs for many gates at once: axes is a sequence of 'x', 'y',
    'z' and angles a (G,) tensor; returns (G, d, d)."""
    basis = basis or _bases.general(2)
    a = angles.to(torch.float64)
    c = torch.cos(a / 2).to(_CDTYPE)
    s = torch.sin(a / 2).to(_CDTYPE)
    j = _imag_unit(a.device)
    e = torch.exp(-j * a.to(_CDTYPE) / 2)
    zero = torch.zeros_like(c)
    kx = torch.stack([torch.stack([c, -j * s], -1),
                      torch.stack([-j * s, c], -1)], -2)
    ky = torch.stack([torch.stack([c, -s], -1), torch.stack([s, c], -1)], -2)
    kz = torch.stack([torch.stack([e, zero], -1),
                      torch.stack([zero, e.conj()], -1)], -2)
    axes = tuple(axes)
    code = _const(('axes', str(a.device), axes), lambda: torch.tensor(
        [{'x': 0, 'y': 1, 'z': 2}[ax] for ax in axes], device=a.device))
    k = torch.where((code == 0)[:, None, None], kx,
                    torch.where((code == 1)[:, None, None], ky, kz))
    d = basis.dim_hilbert
    if d > 2:  # act in the 0-1 subspace
        full = torch.eye(d, dtype=_CDTYPE, device=a.device).repeat(
            len(axes), 1, 1)
        full[:, :2, :2] = k
        k = full
    return kraus_to_ptm_batched(k[:, None], (basis,))


def amp_phase_damping_batched(gamma, lam, basis=None):
    """(Q,) rates -> (Q, 4, 4): amplitude then phase damping per qubit."""
    basis = basis or _bases.general(2)
    g = gamma.to(torch.float64)
    lm = lam.to(torch.float64)
    z = torch.zeros_like(g)
    one = torch.ones_like(g)

    def mat(a, b, c, d):
        return torch.stack([torch.stack([a, b], -1), torch.stack([c, d], -1)],
                           -2)

    amp = torch.stack([mat(one, z, z, torch.sqrt(1 - g)),
                       mat(z, torch.sqrt(g), z, z)], 1)
    ph = torch.stack([mat(one, z, z, torch.sqrt(1 - lm)),
                      mat(z, z, z, torch.sqrt(lm))], 1)
    pa = kraus_to_ptm_batched(amp, (basis,))
    pp = kraus_to_ptm_batched(ph, (basis,))
    return pp @ pa


def cphase_batched(angles, basis=None):
    """(E,) conditional phases -> (E, 4, 4, 4, 4) cphase PTMs."""
    basis = basis or _bases.general(2)
    a = angles.to(torch.float64)
    j = _imag_unit(a.device)
    one = torch.ones_like(a).to(_CDTYPE)
    diag = torch.stack([one, one, one, torch.exp(j * a.to(_CDTYPE))], -1)
    return kraus_to_ptm_batched(torch.diag_embed(diag)[:, None],
                                (basis, basis))

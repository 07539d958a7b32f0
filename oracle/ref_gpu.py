"""The reference's own GPU kernel as a second oracle and as the reference
arm's GPU timing -- test infrastructure, never part of the product.

``oracle/_ref/primitives_sm103a.cubin`` is quantumsim's
``quantumsim/pauli_vectors/primitives.cu`` compiled unchanged for sm_103a
(recipe: ``oracle/build_ref.py``, run by ``__graft_entry__.build()`` where
the reference source tree is present).  This module loads it with the CUDA
driver API (ctypes on libcuda, in the context torch made current) and
launches ``two_qubit_general_ptm`` with the geometry of
``PauliVectorCuda._apply_two_qubit_ptm`` / ``_apply_single_qubit_ptm``
(quantumsim/pauli_vectors/cuda.py:151-221, 223-277): for two qudits the PTM
is transposed ``abcd -> badc`` when qubit0 > qubit1 (:171-173), the block is
(d0_out, d1_out, d_internal) with d_internal grown over the sorted bystander
dims while the block stays within 256 threads (:189-196), one qudit uses
block (1, d_out, min(64, N / d_in)) (:256-259).

The kernel returns before a ``__syncthreads()`` for threads past the end of
the output (primitives.cu:74-78); a block with such threads would reach the
barrier divergently.  ``apply`` therefore only launches grids whose blocks
all lie inside the output (checked on the host, ValueError otherwise), which
holds for every qubit (dim 4) state of 2 or more qubits.
"""
import ctypes
import math
import os

import numpy as np

CUBIN = os.path.join(os.path.dirname(os.path.abspath(__file__)), '_ref',
                     'primitives_sm103a.cubin')

_STATE = {}


def available():
    return os.path.exists(CUBIN)


def _driver():
    if 'fn' in _STATE:
        return _STATE
    import torch
    torch.cuda.init()
    torch.zeros(1, device='cuda')  # the primary context is current
    cu = ctypes.CDLL('libcuda.so.1')
    for name, args in (
            ('cuModuleLoadData', [ctypes.POINTER(ctypes.c_void_p),
                                  ctypes.c_char_p]),
            ('cuModuleGetFunction', [ctypes.POINTER(ctypes.c_void_p),
                                     ctypes.c_void_p, ctypes.c_char_p]),
            ('cuLaunchKernel', [ctypes.c_void_p] + [ctypes.c_uint] * 7 +
             [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p),
              ctypes.c_void_p])):
        f = getattr(cu, name)
        f.argtypes = args
        f.restype = ctypes.c_int
    with open(CUBIN, 'rb') as fh:
        image = fh.read()
    mod = ctypes.c_void_p()
    st = cu.cuModuleLoadData(ctypes.byref(mod), image)
    if st:
        raise RuntimeError('cuModuleLoadData failed ({})'.format(st))
    fn = ctypes.c_void_p()
    st = cu.cuModuleGetFunction(ctypes.byref(fn), mod,
                                b'two_qubit_general_ptm')
    if st:
        raise RuntimeError('cuModuleGetFunction failed ({})'.format(st))
    _STATE.update(cu=cu, mod=mod, fn=fn, image=image)
    return _STATE


def geometry(shape, ptm_shape, qubits):
    """Launch geometry of the reference for a PTM on `qubits` of a vector of
    `shape`: (ptm transposed?, dims, grid, block, shared bytes, new_size)."""
    shape = list(shape)
    if len(qubits) == 2:
        q0, q1 = qubits
        swap = q0 > q1
        if swap:
            q0, q1 = q1, q0
            d0o, d1o, d0i, d1i = (ptm_shape[1], ptm_shape[0], ptm_shape[3],
                                  ptm_shape[2])
        else:
            d0o, d1o, d0i, d1i = ptm_shape
        new_shape = list(shape)
        new_shape[q0], new_shape[q1] = d0o, d1o
        new_size = math.prod(new_shape)
        rest = list(new_shape)
        rest[q0] = rest[q1] = 1
        dint = 1
        for i in sorted(rest):
            if i * dint > 256 // (d0o * d1o):
                break
            dint *= i
        block = (d0o, d1o, dint)
        shared = 8 * dint * d1i * d0i
        dim_z = math.prod(shape[q1 + 1:])
        dim_y = math.prod(shape[q0 + 1:q1])
        dims = (d0i, d1i, dim_z, dim_y, new_size)
    else:
        (q,) = qubits
        swap = False
        dout, din = ptm_shape
        new_shape = list(shape)
        new_shape[q] = dout
        new_size = math.prod(new_shape)
        dint = min(64, math.prod(shape) // din)
        block = (1, dout, dint)
        shared = 8 * dint * din
        dims = (1, din, math.prod(shape[q + 1:]), math.prod(shape[:q]),
                new_size)
    bsize = block[0] * block[1] * block[2]
    grid = max(1, (new_size - 1) // bsize + 1)
    return swap, dims, grid, block, shared, new_shape


def apply(x, ptm, qubits, stream=None):
    """out = the reference kernel's application of `ptm` (numpy, reference
    layout) to the float64 CUDA tensor x; returns a new tensor."""
    import torch
    st = _driver()
    ptm = np.asarray(ptm, dtype=np.float64)
    swap, dims, grid, block, shared, new_shape = geometry(
        x.shape, ptm.shape, tuple(qubits))
    bsize = block[0] * block[1] * block[2]
    if dims[-1] % bsize:
        raise ValueError('the reference kernel would meet a divergent '
                         'barrier in its last block; not launched')
    if swap:
        ptm = np.einsum('abcd -> badc', ptm)
    ptm = np.ascontiguousarray(ptm)
    # device copies cached by content, as the reference does
    # (quantumsim/pauli_vectors/cuda.py:401-420)
    cache = st.setdefault('ptms', {})
    key = (ptm.tobytes(), ptm.shape, str(x.device))
    ptm_d = cache.get(key)
    if ptm_d is None:
        ptm_d = torch.from_numpy(ptm).to(x.device)
        cache[key] = ptm_d
    x = x.contiguous()
    if x.dtype != torch.float64:
        raise TypeError('the reference kernel is FP64 only')
    out = torch.empty(new_shape, dtype=torch.float64, device=x.device)
    vals = [ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()),
            ctypes.c_void_p(ptm_d.data_ptr())] + \
        [ctypes.c_uint(int(v)) for v in dims]
    params = (ctypes.c_void_p * len(vals))(
        *[ctypes.cast(ctypes.pointer(v), ctypes.c_void_p) for v in vals])
    s = stream if stream is not None else \
        torch.cuda.current_stream(x.device).cuda_stream
    rc = st['cu'].cuLaunchKernel(st['fn'], grid, 1, 1, block[0], block[1],
                                 block[2], shared, ctypes.c_void_p(s),
                                 params, None)
    if rc:
        raise RuntimeError('cuLaunchKernel failed ({})'.format(rc))
    return out

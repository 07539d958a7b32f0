"""PyTorch custom operators over the C ABI (``torch.ops.qsgb.*``).

Each operator takes torch tensors (device memory and the current CUDA stream
come from PyTorch), checks arguments on the host, and calls one entry point
of ``libqsgb.so``.  Shapes follow the Pauli-vector convention: a state is an
n-dimensional tensor whose axis i has length dim_pauli of qudit i, C order,
qudit 0 first.

There is no fallback path: on a tensor that is not on a CUDA device the
operators raise.
"""
import ctypes
import math
from typing import List

import numpy as np
import torch

from . import _lib as L

_STATUS = {}

# Operators are defined on a torch.library.Library with a CUDA kernel each
# (and a CPU kernel that raises): one dispatch costs ~5 us on the host, where
# torch.library.custom_op's Python wrapper adds ~16 us -- most of a small
# state's apply_ptm.
_LIB = torch.library.Library('qsgb', 'DEF')


def _cpu_kernel(name):
    def refuse(*args, **kwargs):
        raise RuntimeError('qsgb::{} runs on CUDA tensors only (there is no '
                           'CPU path)'.format(name))
    return refuse


def _op(schema):
    """Define torch.ops.qsgb.<name> from `schema` with the decorated function
    as its CUDA kernel; returns the function unchanged."""
    name = schema.split('(', 1)[0]

    def deco(fn):
        _LIB.define(schema)
        _LIB.impl(name, fn, 'CUDA')
        _LIB.impl(name, _cpu_kernel(name), 'CPU')
        return fn
    return deco


def _fake(name):
    """Shape function of torch.ops.qsgb.<name> for meta / fake tensors."""
    def deco(fn):
        torch.library.register_fake('qsgb::' + name, fn, lib=_LIB)
        return fn
    return deco


_RAW_STREAM = getattr(torch._C, '_cuda_getCurrentRawStream', None)


def _stream_handle(t):
    """The current CUDA stream of t's device (cudaStream_t)."""
    if _RAW_STREAM is not None:
        return ctypes.c_void_p(_RAW_STREAM(t.device.index))
    return ctypes.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)


def _dtype_code(t):
    if t.dtype == torch.float64:
        return L.F64
    if t.dtype == torch.float32:
        return L.F32
    raise TypeError('Pauli vectors must be float64 or float32 tensors, got '
                    '{}'.format(t.dtype))


def _require_cuda(*tensors):
    for t in tensors:
        if not t.is_cuda:
            raise RuntimeError('qsgb operators run on CUDA tensors only '
                               '(got a tensor on {})'.format(t.device))


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def status_tensor(device):
    """Per-device word that kernels OR their QSGB_DEV_* bits into."""
    device = torch.device(device)
    key = device.index if device.index is not None else torch.cuda.current_device()
    st = _STATUS.get(key)
    if st is None:
        st = torch.zeros(1, dtype=torch.int32, device=torch.device('cuda', key))
        _STATUS[key] = st
    return st


def check_device_status(device):
    """Raise if a kernel reported a device-side problem since the last check
    (synchronises the device's current stream)."""
    st = status_tensor(device)
    _raise_status(st, int(st.item()))


def fetch_checked(t):
    """Host (numpy, float64) copy of the small device tensor `t`, read in the
    same device-to-host copy as the status word: one synchronisation where
    ``check_device_status`` followed by a read takes two.  Raises like
    ``check_device_status``."""
    st = status_tensor(t.device)
    both = torch.cat([t.reshape(-1).to(torch.float64),
                      st.to(torch.float64)]).cpu().numpy()
    _raise_status(st, int(both[-1]))
    return both[:-1]


def _raise_status(st, val):
    if val:
        st.zero_()
        reasons = []
        if val & L.DEV_RANGE:
            reasons.append('a Pauli-vector entry or PTM result left the '
                           'float-float range (|x| >= 2^128, inf or nan)')
        if val & L.DEV_TIMEOUT:
            reasons.append('a bounded device-side wait timed out')
        if val & L.DEV_BADITEM:
            reasons.append('a kernel rejected a malformed work item')
        raise RuntimeError('qsgb device status {}: {}'.format(
            val, '; '.join(reasons)))


def apply_geometry(shape, qudits, ptm_shape, transpose=False):
    """Sizes of a PTM application.

    Returns (new_shape, (X, Y, Z), dims) where dims = (da_out, db_out, da_in,
    db_in) for qudits a < b (one qudit: da = 1), plus the swapped flag.
    ``ptm_shape`` is the stored PTM shape in argument order (out..., in...);
    with ``transpose`` the stored matrix is the forward PTM whose transpose
    is applied (its in/out halves are exchanged).
    """
    n = len(qudits)
    half = len(ptm_shape) // 2
    outs, ins = list(ptm_shape[:half]), list(ptm_shape[half:])
    if transpose:
        outs, ins = ins, outs
    new_shape = list(shape)
    for q, dout, din in zip(qudits, outs, ins):
        if shape[q] != din:
            raise ValueError(
                'PTM input dimension {} does not match dimension {} of qudit '
                '{}'.format(din, shape[q], q))
        new_shape[q] = dout
    if n == 1:
        (q,) = qudits
        X = 1
        Y = math.prod(shape[:q])
        Z = math.prod(shape[q + 1:])
        dims = (1, outs[0], 1, ins[0])
        swapped = False
    else:
        q0, q1 = qudits
        swapped = q0 > q1
        a, b = (q1, q0) if swapped else (q0, q1)
        X = math.prod(shape[:a])
        Y = math.prod(shape[a + 1:b])
        Z = math.prod(shape[b + 1:])
        if swapped:
            dims = (outs[1], outs[0], ins[1], ins[0])
        else:
            dims = (outs[0], outs[1], ins[0], ins[1])
    return new_shape, (X, Y, Z), dims, swapped


# --------------------------------------------------------------- apply_ptm
@_op('apply_ptm(Tensor pv, Tensor ptm, int[] qudits, int arith, int max_terms, '
     'bool transpose, bool jit=True) -> Tensor')
def apply_ptm(pv: torch.Tensor, ptm: torch.Tensor, qudits: List[int],
              arith: int, max_terms: int, transpose: bool,
              jit: bool = True) -> torch.Tensor:
    """Apply a 1- or 2-qudit PTM (float64) to a Pauli-vector tensor.

    ``ptm`` may live on the device or on the host, in which case the library
    reads it during the call and passes its values inside the kernel launch.
    ``max_terms`` bounds the non-zero terms a device PTM keeps (0: all
    entries; a host PTM's terms are counted by the library)."""
    _require_cuda(pv)
    if ptm.dtype != torch.float64:
        raise TypeError('PTM must be float64')
    new_shape, (X, Y, Z), (dao, dbo, dai, dbi), swapped = apply_geometry(
        pv.shape, qudits, ptm.shape, transpose)
    pv = pv.contiguous()
    ptm = ptm.contiguous()
    out = torch.empty(new_shape, dtype=pv.dtype, device=pv.device)
    flags = (L.PTM_SWAPPED if swapped else 0) | (
        L.PTM_TRANSPOSED if transpose else 0)
    if ptm.is_cuda:
        if ptm.device != pv.device:
            raise ValueError('PTM and Pauli vector are on different devices')
    else:
        # host PTM: read by the library during the call (its sparsity
        # pattern selects a specialised kernel); no device copy
        flags |= L.PTM_HOST
    if jit is False:
        flags |= L.PTM_NOJIT
    lib = L.load()
    st = status_tensor(pv.device)
    if out.numel() == 0:
        return out

    def call(ptm_, flags_):
        if len(qudits) == 1:
            return lib.qsgb_apply_ptm1(
                _ptr(pv), _ptr(out), _ptr(ptm_), dbo, dbi, Y, Z, flags_,
                _dtype_code(pv), arith, max_terms, _ptr(st),
                _stream_handle(pv))
        return lib.qsgb_apply_ptm2(
            _ptr(pv), _ptr(out), _ptr(ptm_), dao, dbo, dai, dbi, X, Y, Z,
            flags_, _dtype_code(pv), arith, max_terms, _ptr(st),
            _stream_handle(pv))

    status = call(ptm, flags)
    if status == L.ERR_UNSUPPORTED and (flags & L.PTM_HOST):
        # no specialised kernel and too large to travel in the launch:
        # the generic kernel reads it from device memory
        # (stream-ordered allocator: freeing dev_ptm after the enqueue is
        # safe for work on this stream)
        dev_ptm = ptm.to(pv.device)
        if max_terms < 1:
            max_terms = nnz_terms(ptm.numpy(), arith)
        status = call(dev_ptm, flags & ~L.PTM_HOST)
    L.check(status, 'qsgb_apply_ptm')
    return out


@_fake('apply_ptm')
def _(pv, ptm, qudits, arith, max_terms, transpose, jit=True):
    new_shape = apply_geometry(pv.shape, qudits, ptm.shape, transpose)[0]
    return pv.new_empty(new_shape)


# --------------------------------------------------------------- ptm_grad
@_op('ptm_grad(Tensor x_in, Tensor g_out, int[] qudits) -> Tensor')
def ptm_grad(x_in: torch.Tensor, g_out: torch.Tensor,
             qudits: List[int]) -> torch.Tensor:
    """dL/dPTM for out = apply_ptm(x_in, PTM, qudits), given dL/dout.

    Returned in the PTM's argument-order layout (out..., in...), float64."""
    _require_cuda(x_in, g_out)
    if x_in.dtype != g_out.dtype:
        raise TypeError('x_in and g_out must share a dtype')
    n = len(qudits)
    outs = [g_out.shape[q] for q in qudits]
    ins = [x_in.shape[q] for q in qudits]
    x_in = x_in.contiguous()
    g_out = g_out.contiguous()
    lib = L.load()
    shape = list(x_in.shape)
    if n == 1:
        (q,) = qudits
        Y, Z = math.prod(shape[:q]), math.prod(shape[q + 1:])
        groups, kout, kin = Y * Z, outs[0], ins[0]
    else:
        a, b = sorted(qudits)
        X = math.prod(shape[:a])
        Y = math.prod(shape[a + 1:b])
        Z = math.prod(shape[b + 1:])
        groups = X * Y * Z
        kout, kin = outs[0] * outs[1], ins[0] * ins[1]
    out_sorted = torch.empty(kout * kin, dtype=torch.float64,
                             device=x_in.device)
    nbytes = lib.qsgb_ptm_grad_scratch_bytes(groups, kout, kin)
    scratch = torch.empty(max(nbytes, 8), dtype=torch.uint8,
                          device=x_in.device)
    if n == 1:
        status = lib.qsgb_ptm_grad1(
            _ptr(x_in), _ptr(g_out), _ptr(out_sorted), outs[0], ins[0], Y, Z,
            _dtype_code(x_in), _ptr(scratch), nbytes, _stream_handle(x_in))
        L.check(status, 'qsgb_ptm_grad1')
        return out_sorted.view(outs[0], ins[0])
    a, b = sorted(qudits)
    da_o, db_o = g_out.shape[a], g_out.shape[b]
    da_i, db_i = x_in.shape[a], x_in.shape[b]
    status = lib.qsgb_ptm_grad2(
        _ptr(x_in), _ptr(g_out), _ptr(out_sorted), da_o, db_o, da_i, db_i, X,
        Y, Z, _dtype_code(x_in), _ptr(scratch), nbytes, _stream_handle(x_in))
    L.check(status, 'qsgb_ptm_grad2')
    res = out_sorted.view(da_o, db_o, da_i, db_i)
    if qudits[0] > qudits[1]:
        res = res.permute(1, 0, 3, 2).contiguous()
    return res


@_fake('ptm_grad')
def _(x_in, g_out, qudits):
    shape = [g_out.shape[q] for q in qudits] + [x_in.shape[q] for q in qudits]
    return x_in.new_empty(shape, dtype=torch.float64)


# --------------------------------------------------------------- gathers
@_op('gather(Tensor pv, int[] idx_off, int[] idx, bool out_f64) -> Tensor')
def gather(pv: torch.Tensor, idx_off: List[int], idx: List[int],
           out_f64: bool) -> torch.Tensor:
    """Multitake: pv[np.ix_(idx_0, ...)] (flattened); -1 selects a zero."""
    _require_cuda(pv)
    pv = pv.contiguous()
    ndim = pv.dim()
    n_out = 1
    for a in range(ndim):
        n_out *= idx_off[a + 1] - idx_off[a]
    out = torch.empty(n_out, dtype=torch.float64 if out_f64 else pv.dtype,
                      device=pv.device)
    status = L.load().qsgb_gather(
        _ptr(pv), _ptr(out), _dtype_code(pv), _dtype_code(out), ndim,
        L.i64_array(pv.shape), L.i32_array(idx_off), L.i32_array(idx),
        _stream_handle(pv))
    L.check(status, 'qsgb_gather')
    return out


@_fake('gather')
def _(pv, idx_off, idx, out_f64):
    n_out = 1
    for a in range(pv.dim()):
        n_out *= idx_off[a + 1] - idx_off[a]
    return pv.new_empty(n_out, dtype=torch.float64 if out_f64 else pv.dtype)


@_op('take_axis(Tensor pv, int axis, int[] idx) -> Tensor')
def take_axis(pv: torch.Tensor, axis: int, idx: List[int]) -> torch.Tensor:
    """pv.index_select(axis, idx) as a bit-exact copy; -1 selects a zero."""
    _require_cuda(pv)
    pv = pv.contiguous()
    shape = list(pv.shape)
    outer = math.prod(shape[:axis])
    inner = math.prod(shape[axis + 1:])
    new_shape = list(shape)
    new_shape[axis] = len(idx)
    out = torch.empty(new_shape, dtype=pv.dtype, device=pv.device)
    if out.numel() == 0:
        return out
    status = L.load().qsgb_take_axis(
        _ptr(pv), _ptr(out), _dtype_code(pv), outer, shape[axis], inner,
        L.i32_array(idx), len(idx), _stream_handle(pv))
    L.check(status, 'qsgb_take_axis')
    return out


@_fake('take_axis')
def _(pv, axis, idx):
    shape = list(pv.shape)
    shape[axis] = len(idx)
    return pv.new_empty(shape)


# --------------------------------------------------------------- reductions
@_op('marginals(Tensor diag, int[] shape, int axis) -> Tensor')
def marginals(diag: torch.Tensor, shape: List[int],
              axis: int) -> torch.Tensor:
    """Marginal sums of an FP64 diagonal along `axis` (-1: the trace)."""
    _require_cuda(diag)
    if diag.dtype != torch.float64:
        raise TypeError('diagonal must be float64')
    diag = diag.contiguous()
    n_out = 1 if axis < 0 else shape[axis]
    out = torch.empty(n_out, dtype=torch.float64, device=diag.device)
    lib = L.load()
    nbytes = lib.qsgb_marginals_scratch_bytes(max(1, diag.numel()), n_out)
    scratch = torch.empty(max(8, nbytes), dtype=torch.uint8,
                          device=diag.device)
    status = lib.qsgb_marginals(
        _ptr(diag), len(shape), L.i64_array(shape), axis, _ptr(out),
        _ptr(scratch), nbytes, _stream_handle(diag))
    L.check(status, 'qsgb_marginals')
    return out


@_fake('marginals')
def _(diag, shape, axis):
    return diag.new_empty(1 if axis < 0 else shape[axis])


@_op('partial_trace(Tensor pv, int[] keep, float[] weights) -> Tensor')
def partial_trace(pv: torch.Tensor, keep: List[int],
                  weights: List[float]) -> torch.Tensor:
    """Trace out the qudits not flagged in `keep` with per-element weights
    (concatenated over traced qudits, ascending); kept axes stay in order."""
    _require_cuda(pv)
    pv = pv.contiguous()
    shape = list(pv.shape)
    new_shape = [d for d, k in zip(shape, keep) if k]
    out = torch.empty(new_shape, dtype=pv.dtype, device=pv.device)
    status = L.load().qsgb_partial_trace(
        _ptr(pv), _ptr(out), _dtype_code(pv), len(shape), L.i64_array(shape),
        L.i32_array(keep), L.f64_array(weights), _stream_handle(pv))
    L.check(status, 'qsgb_partial_trace')
    return out


@_fake('partial_trace')
def _(pv, keep, weights):
    return pv.new_empty([d for d, k in zip(pv.shape, keep) if k])


@_op('scale_(Tensor(a!) pv, float alpha) -> ()')
def scale_(pv: torch.Tensor, alpha: float) -> None:
    """pv *= alpha in place."""
    _require_cuda(pv)
    if not pv.is_contiguous():
        raise ValueError('scale_ needs a contiguous tensor')
    status = L.load().qsgb_scale(_ptr(pv), _dtype_code(pv), pv.numel(),
                                 float(alpha), _stream_handle(pv))
    L.check(status, 'qsgb_scale')


@_op('scale_by_inverse_(Tensor(a!) pv, Tensor denom, float threshold) -> ()')
def scale_by_inverse_(pv: torch.Tensor, denom: torch.Tensor,
                      threshold: float) -> None:
    """pv *= 1/denom[0] in place when denom[0] > threshold (device scalar)."""
    _require_cuda(pv, denom)
    if not pv.is_contiguous() or denom.dtype != torch.float64:
        raise ValueError('scale_by_inverse_ needs a contiguous tensor and a '
                         'float64 denominator')
    status = L.load().qsgb_scale_by_inverse(
        _ptr(pv), _dtype_code(pv), pv.numel(), _ptr(denom), float(threshold),
        _stream_handle(pv))
    L.check(status, 'qsgb_scale_by_inverse')


# ------------------------------------------------------- eager fast paths
# PauliVectorGB300 calls the C ABI directly for eager work on host numpy
# PTMs: the operators above go through the torch dispatcher and a Python
# kernel (~10 us), and recompute the geometry on every call (~15 us of
# Python); an eager application with a cached, validated plan costs the
# output allocation and one ctypes call.
_STATUS_PTR = {}
_DIAG_BUF = {}


def status_ptr(index):
    """Address of the device status word of CUDA device `index`."""
    p = _STATUS_PTR.get(index)
    if p is None:
        p = status_tensor(torch.device('cuda', index)).data_ptr()
        _STATUS_PTR[index] = p
    return p


def eager_plan(shape, dtype, qudits, ptm_shape):
    """Validated geometry of applying a host PTM of `ptm_shape` to `qudits`
    of a contiguous vector of `shape` and torch `dtype`: (output shape, two
    qudits?, size arguments, layout flags, dtype code).  Raises ValueError
    like apply_geometry."""
    new_shape, (X, Y, Z), (dao, dbo, dai, dbi), swapped = apply_geometry(
        shape, list(qudits), ptm_shape)
    flags = L.PTM_HOST | (L.PTM_SWAPPED if swapped else 0)
    code = L.F64 if dtype == torch.float64 else L.F32
    if len(qudits) == 1:
        return tuple(new_shape), False, (dbo, dbi, Y, Z), flags, code
    return (tuple(new_shape), True, (dao, dbo, dai, dbi, X, Y, Z), flags,
            code)


_PYAPPLY = None  # the CPython entry point once set up; False when absent


def _pyapply():
    """The compiled per-call entry point (csrc/qsgb_pyapply.c), handed the
    library's apply addresses and the stream / status lookups once; False
    when it was not built (no C compiler or Python headers)."""
    global _PYAPPLY
    if _PYAPPLY is None:
        try:
            from . import _qsgb_pyapply as m
        except ImportError:
            _PYAPPLY = False
            return _PYAPPLY
        lib = L.load()
        raw = _RAW_STREAM if _RAW_STREAM is not None else (
            lambda i: torch.cuda.current_stream(i).cuda_stream)
        m.set_entry_points(
            ctypes.cast(lib.qsgb_apply_ptm1, ctypes.c_void_p).value,
            ctypes.cast(lib.qsgb_apply_ptm2, ctypes.c_void_p).value,
            raw, status_ptr, torch.empty,
            lambda i: torch.device('cuda', i))
        _PYAPPLY = m
    return _PYAPPLY


def eager_apply(pv, ptm, plan, arith, out=None):
    """Apply the numpy PTM `ptm` (converted to C-contiguous float64 when it
    is not) to the contiguous CUDA tensor `pv` with a plan from eager_plan;
    returns the output tensor, or None when the request needs the general
    operator path.  `out`, when given, is a contiguous tensor of the output
    shape, dtype and device that the caller owns and no longer reads; the
    result is written there instead of into a new tensor."""
    fast = _PYAPPLY if _PYAPPLY is not None else _pyapply()
    if fast:
        st = fast.apply(pv, ptm, plan, arith, out)
        if type(st) is not int:
            return st
        if st == fast.NOT_F64_CONTIGUOUS:
            st = fast.apply(pv, np.ascontiguousarray(ptm, dtype=np.float64),
                            plan, arith, out)
            if type(st) is not int:
                return st
        if st == L.ERR_UNSUPPORTED:
            return None
        L.check(st, 'qsgb_apply_ptm')
    ptm = np.ascontiguousarray(ptm, dtype=np.float64)
    new_shape, two, sizes, flags, code = plan
    if out is None:
        out = torch.empty(new_shape, dtype=pv.dtype, device=pv.device)
    if out.numel() == 0:
        return out
    lib = L.load()
    idx = pv.device.index
    stream = _RAW_STREAM(idx) if _RAW_STREAM is not None else \
        torch.cuda.current_stream(pv.device).cuda_stream
    addr = ptm.__array_interface__['data'][0]
    if two:
        st = lib.qsgb_apply_ptm2(pv.data_ptr(), out.data_ptr(), addr, *sizes,
                                 flags, code, arith, 0, status_ptr(idx),
                                 stream)
    else:
        st = lib.qsgb_apply_ptm1(pv.data_ptr(), out.data_ptr(), addr, *sizes,
                                 flags, code, arith, 0, status_ptr(idx),
                                 stream)
    if st == L.OK:
        return out
    if st == L.ERR_UNSUPPORTED:
        return None  # the caller takes the general operator path
    L.check(st, 'qsgb_apply_ptm')
    return out


def diag_marginals(pv, plan_arrays, axis):
    """Marginals (axis >= 0) or trace (axis == -1) of the DM diagonal of the
    CUDA tensor `pv` through the gather plan, in one launch and one
    device-to-host copy that also returns the device status word (raises
    like check_device_status).  None when the fused kernel does not serve
    the request (the caller takes the gather + reduction path)."""
    idx_off_c, idx_c, shape_c, n_out = plan_arrays
    index = pv.device.index
    bufs = _DIAG_BUF.get(index)
    if bufs is None:
        nscr = int(L.load().qsgb_diag_marginals_scratch_bytes())
        # the scratch's first 16 bytes (the kernel's block ticket) start at
        # zero and every call leaves them zero
        bufs = (torch.empty(80, dtype=torch.float64, device=pv.device),
                torch.empty(80, dtype=torch.float64, pin_memory=True),
                torch.zeros(nscr, dtype=torch.uint8, device=pv.device))
        _DIAG_BUF[index] = bufs
    dev, host, scratch = bufs
    n = (1 if axis < 0 else n_out[axis]) + 1
    if n > 65:
        return None
    stream = _RAW_STREAM(index) if _RAW_STREAM is not None else \
        torch.cuda.current_stream(pv.device).cuda_stream
    # the library copies the n values into the pinned buffer and waits
    st = L.load().qsgb_diag_marginals(
        pv.data_ptr(), _dtype_code(pv), pv.dim(), shape_c, idx_off_c, idx_c,
        axis, dev.data_ptr(), status_ptr(index), host.data_ptr(),
        scratch.data_ptr(), scratch.numel(), stream)
    if st == L.ERR_UNSUPPORTED:
        return None
    L.check(st, 'qsgb_diag_marginals')
    vals = host.numpy()[:n].copy()
    if vals[-1]:
        _raise_status(status_tensor(pv.device), int(vals[-1]))
    return vals[:-1]


def prepare_ptm(shape, dtype, ptm, qudits, arith, transpose=False):
    """Compile ahead of time the specialised kernel that
    ``torch.ops.qsgb.apply_ptm`` would use for this host PTM (numpy float64)
    on a Pauli-vector tensor of `shape` and `dtype`; returns the shape of the
    result.  Releases the GIL while compiling, so threads compile in
    parallel.  A PTM served by the generic kernel needs nothing."""
    ptm = np.ascontiguousarray(ptm, dtype=np.float64)
    new_shape, (X, Y, Z), (dao, dbo, dai, dbi), swapped = apply_geometry(
        tuple(shape), list(qudits), ptm.shape, transpose)
    if math.prod(new_shape) == 0:
        return new_shape
    flags = L.PTM_HOST | (L.PTM_SWAPPED if swapped else 0) | (
        L.PTM_TRANSPOSED if transpose else 0)
    code = L.F64 if dtype == torch.float64 else L.F32
    if len(qudits) == 1:
        dao, dai, X = 1, 1, 1
    st = L.load().qsgb_prepare_ptm2(
        ctypes.c_void_p(ptm.ctypes.data), dao, dbo, dai, dbi, X, Y, Z, flags,
        code, arith)
    if st not in (L.OK, L.ERR_UNSUPPORTED):
        L.check(st, 'qsgb_prepare_ptm2')
    return new_shape


def nnz_terms(ptm, arith):
    """Number of PTM entries the kernel keeps (same rule as the device):
    exact zeros are dropped for native FP64, otherwise entries with
    |p| <= 2^-52 max|P| (FP64 storage) or 2^-30 max|P| (FP32)."""
    a = np.abs(np.asarray(ptm, dtype=np.float64))
    if a.size == 0:
        return 1
    if arith == L.ARITH_F64:
        thr = 0.0
    elif arith == L.ARITH_F32:
        thr = a.max() * 2.0 ** -30
    else:
        thr = a.max() * 2.0 ** -52
    return max(1, int(np.count_nonzero(a > thr)))

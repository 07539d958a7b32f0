"""The allocation-free marginals entry point, called through the C ABI.

`qsgb_marginals_noalloc` is for host programs that cannot allocate device
memory when they need measurement probabilities -- for instance an
application whose device memory is entirely owned by its own pool allocator,
or a latency-critical loop where the implicit synchronisation of cudaMalloc
would stall the GPU.  It keeps its partial sums in a fixed array inside the
library instead of caller-provided scratch.  This test checks, on two calls
in a row (different data and axes, so stale contents of the shared array
would show), that it returns what `qsgb_marginals` with caller scratch
returns.  It lives in its own file, collected last, and needs nothing from
the other tests.
"""
import ctypes

import numpy as np
import pytest
import torch

from conftest import ATOL_PROB
from quantumsim_gb300 import _lib as L
from quantumsim_gb300 import build as qbuild

pytestmark = pytest.mark.gpu


def _marginals_with_scratch(lib, diag, shape, axis, stream):
    n_out = 1 if axis < 0 else shape[axis]
    out = torch.empty(n_out, dtype=torch.float64, device=diag.device)
    nbytes = lib.qsgb_marginals_scratch_bytes(diag.numel(), n_out)
    scratch = torch.empty(max(8, nbytes), dtype=torch.uint8,
                          device=diag.device)
    st = lib.qsgb_marginals(ctypes.c_void_p(diag.data_ptr()), len(shape),
                            L.i64_array(shape), axis,
                            ctypes.c_void_p(out.data_ptr()),
                            ctypes.c_void_p(scratch.data_ptr()), nbytes,
                            stream)
    assert st == L.OK
    return out


def _marginals_noalloc(lib, diag, shape, axis, stream):
    n_out = 1 if axis < 0 else shape[axis]
    out = torch.empty(n_out, dtype=torch.float64, device=diag.device)
    st = lib.qsgb_marginals_noalloc(ctypes.c_void_p(diag.data_ptr()),
                                    len(shape), L.i64_array(shape), axis,
                                    ctypes.c_void_p(out.data_ptr()), stream)
    assert st == L.OK, L.load().qsgb_status_string(st)
    return out


@pytest.fixture(scope='module')
def lib_and_stream():
    """The library, built if needed, with cuda:0 current (so each test also
    runs on its own in a fresh process)."""
    qbuild.build()
    lib = L.load()
    dev = torch.device('cuda', 0)
    torch.cuda.set_device(dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    return lib, dev, stream


def _check_against_both(lib, dev, stream, probs, shape, ax):
    diag = torch.from_numpy(probs).to(dev)
    got = _marginals_noalloc(lib, diag, shape, ax, stream)
    ref = _marginals_with_scratch(lib, diag, shape, ax, stream)
    torch.cuda.synchronize()
    np.testing.assert_allclose(got.cpu().numpy(), ref.cpu().numpy(),
                               rtol=0, atol=ATOL_PROB)
    expect = (probs.reshape(shape).sum(axis=tuple(
        i for i in range(len(shape)) if i != ax))
        if ax >= 0 else np.array([probs.sum()]))
    np.testing.assert_allclose(got.cpu().numpy(), expect, rtol=0,
                               atol=ATOL_PROB)


def test_noalloc_marginals_match_scratch_version_twice(lib_and_stream):
    lib, dev, stream = lib_and_stream
    assert lib.qsgb_marginals_noalloc_max_scratch_bytes() == 16384 * 8
    rng = np.random.default_rng(2024)
    calls = [([2] * 14, 5), ([3, 2, 3, 3, 2, 3, 3], 2)]  # two calls in a row
    for shape, axis in calls:
        probs = rng.random(int(np.prod(shape)))
        probs /= probs.sum()
        for ax in (axis, -1):
            _check_against_both(lib, dev, stream, probs, shape, ax)


def test_noalloc_accepts_exactly_the_fixed_array(lib_and_stream):
    """Requests that need exactly 16384 partial sums still run: one chunk
    of 16384 outcomes, and 32 outcomes of 2^21 entries each (512 chunks of
    4096, the documented limit for qudits of up to 32 levels)."""
    lib, dev, stream = lib_and_stream
    rng = np.random.default_rng(7)
    for shape, ax in (([16384], 0), ([1 << 21, 32], 1)):
        probs = rng.random(int(np.prod(shape)))
        probs /= probs.sum()
        _check_against_both(lib, dev, stream, probs, shape, ax)


def test_noalloc_rejects_requests_beyond_the_fixed_array(lib_and_stream):
    lib, dev, stream = lib_and_stream
    # 16385 outcomes on one axis need 16385 partial sums > 16384; so do
    # 20000 outcomes of two entries each
    for shape in ([16385], [20000, 2]):
        n = int(np.prod(shape))
        diag = torch.zeros(n, dtype=torch.float64, device=dev)
        out = torch.empty(shape[0], dtype=torch.float64, device=dev)
        st = lib.qsgb_marginals_noalloc(ctypes.c_void_p(diag.data_ptr()),
                                        len(shape), L.i64_array(shape), 0,
                                        ctypes.c_void_p(out.data_ptr()),
                                        stream)
        assert st == L.ERR_SCRATCH

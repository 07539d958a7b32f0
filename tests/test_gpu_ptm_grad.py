"""The PTM gradient kernels (csrc/qsgb_grad.cu) against the oracle's
dP = sum_g g_out (x) x_in, for one- and two-qudit PTMs of every size the
apply kernels take (4 x 4, 16 x 16 at ten qubits, qutrit 9 x 9 and 81 x 81,
rectangular), every stride class, FP32 storage, and inputs that hold
out-of-band values:

* float-float products (FP64 tiles for values outside [2^-100, 2^40]): per
  entry within 2^-44 of sum_g |g_out| |x_in| (2^-47 per product, with
  margin);
* 16 x 16 gradients on FP64 vectors, on the tensor cores: within 2^-44 of
  the sum over 16-group chunks of max |g_out| max |x_in| (the digit split's
  2^-47.7 of the chunk maxima, with margin), and bit for bit the same on
  repeated calls; the float-float kernel (QSGB_TC_GRAD=0) is compared in a
  child process."""
import numpy as np
import pytest
import torch

from oracle import pauli_vector_np as O
import quantumsim_gb300  # noqa: F401  (registers the torch.ops.qsgb operators)

pytestmark = pytest.mark.gpu

BOUND = 2.0 ** -44


def _tc_path(x, qs, dims_out):
    """The 16 x 16 FP64 gradients run on the tensor cores."""
    return (x.dtype == np.float64 and len(qs) == 2 and
            x.shape[qs[0]] * x.shape[qs[1]] == 16 and
            dims_out[0] * dims_out[1] == 16)


def _chunk_bound(x, g, qs):
    """sum over chunks of 16 consecutive groups (bystander index order
    (x, y, z), z fastest, as the kernel walks them) of
    max |g_out[., r]| * max |x_in[., k]|: the scale of the tensor-core
    gradient's error, in the PTM's argument order."""
    a, b = sorted(qs)
    shp = x.shape
    X, Y, Z = (int(np.prod(shp[:a])), int(np.prod(shp[a + 1:b])),
               int(np.prod(shp[b + 1:])))

    def groups(t):
        da, db = t.shape[a], t.shape[b]
        v = np.abs(t).reshape(X, da, Y, db, Z).transpose(0, 2, 4, 1, 3)
        v = v.reshape(-1, da * db)
        return np.pad(v, ((0, (-v.shape[0]) % 16), (0, 0))).reshape(
            -1, 16, da * db).max(axis=1)

    bound = np.einsum('cr,ck->rk', groups(g), groups(x))
    res = bound.reshape(g.shape[a], g.shape[b], shp[a], shp[b])
    if qs[0] > qs[1]:
        res = res.transpose(1, 0, 3, 2)
    return res


def _check(x, g, qs, rel=BOUND, floor=0.0):
    xt = torch.from_numpy(x).cuda()
    gt = torch.from_numpy(g).cuda()
    got = torch.ops.qsgb.ptm_grad(xt, gt, list(qs)).cpu().numpy()
    ref = O.ptm_grad(x, g, *qs)
    absref = O.ptm_grad(np.abs(x), np.abs(g), *qs)
    assert got.shape == ref.shape
    err = np.abs(got - ref)
    if _tc_path(x, qs, [g.shape[q] for q in qs]):
        # 2^-47.7 of the chunk maxima per chunk, with margin; the FP64
        # oracle's own rounding is below 2^-44 of sum |g| |x|
        lim = 2.0 ** -44 * (_chunk_bound(x, g, qs) + absref) + floor
    else:
        lim = rel * absref + floor
    assert np.all(err <= lim), (qs, float((err / np.maximum(lim, 1e-300)).max()))
    return got


def _out_shape(shape, qs, dims_out):
    s = list(shape)
    for q, d in zip(qs, dims_out):
        s[q] = d
    return tuple(s)


@pytest.mark.parametrize('qs', [(0,), (4,), (9,), (0, 1), (3, 7), (8, 9),
                                (9, 8), (6, 2)])
def test_qubit_ptms_at_ten_qubits(qs):
    rng = np.random.default_rng(hash(qs) % 1000)
    shape = (4,) * 10
    x = rng.standard_normal(shape)
    g = rng.standard_normal(shape)
    _check(x, g, qs)


def test_qutrit_and_rectangular_ptms():
    rng = np.random.default_rng(31)
    shape = (9, 4, 9, 9, 3)
    x = rng.standard_normal(shape)
    for qs, dout in [((0,), (9,)), ((2, 3), (9, 9)), ((3, 0), (9, 9)),
                     ((1,), (2,)), ((4, 1), (9, 4)), ((0, 4), (3, 1))]:
        g = rng.standard_normal(_out_shape(shape, qs, dout))
        _check(x, g, qs)


def test_fp32_storage():
    rng = np.random.default_rng(32)
    shape = (4,) * 8
    x = rng.standard_normal(shape).astype(np.float32)
    g = rng.standard_normal(shape).astype(np.float32)
    for qs in [(2,), (1, 5), (7, 6)]:
        xt = torch.from_numpy(x).cuda()
        gt = torch.from_numpy(g).cuda()
        got = torch.ops.qsgb.ptm_grad(xt, gt, list(qs)).cpu().numpy()
        # the float inputs are exact in the float-float products
        ref = O.ptm_grad(x.astype(np.float64), g.astype(np.float64), *qs)
        absref = O.ptm_grad(np.abs(x).astype(np.float64),
                            np.abs(g).astype(np.float64), *qs)
        assert np.all(np.abs(got - ref) <= BOUND * absref)


def test_out_of_band_values_take_the_fp64_tiles():
    """Values above 2^40 or below 2^-100 (and the neighbours in their tiles)
    are computed in native FP64; the rest of the vector in float-float."""
    rng = np.random.default_rng(33)
    shape = (4,) * 9
    x = rng.standard_normal(shape)
    g = rng.standard_normal(shape)
    x[1, 2, 3, 0, 0, 1, 2, 3, 0] = 3e15
    x[0, 0, 0, 0, 1, 1, 1, 1, 2] = 1e-40
    g[3, 3, 3, 3, 3, 3, 3, 3, 3] = -1e-290
    g[2, 0, 1, 0, 1, 0, 1, 0, 1] = 7e200
    for qs in [(8,), (0, 3), (8, 7)]:
        _check(x, g, qs)
    # magnitudes that no float pair holds throughout
    _check(x * 1e-200, g, (2, 5), floor=0.0)
    _check(x, g * 1e50, (2, 5))


def test_deterministic():
    rng = np.random.default_rng(34)
    shape = (4,) * 9
    x = torch.from_numpy(rng.standard_normal(shape)).cuda()
    g = torch.from_numpy(rng.standard_normal(shape)).cuda()
    a = torch.ops.qsgb.ptm_grad(x, g, [3, 6])
    b = torch.ops.qsgb.ptm_grad(x, g, [3, 6])
    assert torch.equal(a, b)


def test_float_float_kernel_for_16x16_with_the_tensor_cores_off():
    """QSGB_TC_GRAD=0 (read once per process, so in a child process) sends
    16 x 16 FP64 gradients to the float-float kernel, held to its own
    2^-44 of sum |g| |x|."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = '''
import numpy as np, torch, sys
sys.path.insert(0, {root!r}); sys.path.insert(0, {tests!r})
from oracle import pauli_vector_np as O
import quantumsim_gb300
rng = np.random.default_rng(35)
x = rng.standard_normal((4,) * 9); g = rng.standard_normal((4,) * 9)
for qs in [(2, 6), (8, 7)]:
    got = torch.ops.qsgb.ptm_grad(torch.from_numpy(x).cuda(),
                                  torch.from_numpy(g).cuda(), list(qs)).cpu().numpy()
    ref = O.ptm_grad(x, g, *qs); absref = O.ptm_grad(np.abs(x), np.abs(g), *qs)
    assert np.all(np.abs(got - ref) <= 2.0 ** -44 * absref), qs
print('float-float ok')
'''.format(root=root, tests=os.path.join(root, 'tests'))
    env = dict(os.environ, QSGB_TC_GRAD='0')
    run = subprocess.run([sys.executable, '-c', code], env=env,
                         capture_output=True, text=True, timeout=600)
    assert run.returncode == 0, run.stdout[-2000:] + run.stderr[-2000:]
    assert 'float-float ok' in run.stdout


def test_tensor_core_gradient_partial_chunks():
    """16 x 16 gradients whose group count is not a multiple of the 16 of a
    chunk: 15 groups (bystanders of dims 3 and 5), a single group (the two
    qubits alone), and 35 groups in both argument orders."""
    rng = np.random.default_rng(36)
    for shape, qs in [((4, 3, 4, 5), (0, 2)), ((4, 4), (0, 1)),
                      ((4, 4), (1, 0)), ((5, 4, 7, 4), (3, 1)),
                      ((5, 4, 7, 4), (1, 3))]:
        x = rng.standard_normal(shape)
        g = rng.standard_normal(shape)
        assert _tc_path(x, qs, [g.shape[q] for q in qs])
        _check(x, g, qs)

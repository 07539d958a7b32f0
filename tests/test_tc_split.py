"""The digit split of the tensor-core kernel for dense 16 x 16 PTMs
(quantumsim_gb300/csrc/qsgb_tc.cu), modelled in numpy integer arithmetic on
the host: the fixed-point conversion and its six balanced base-1024 digits
reproduce each input exactly, every digit is an exact FP16 number (built as
the kernel does, from the bit pattern 0x6400 | v minus 1536), the level sums
fit the FP32 accumulator, and the recombined products agree with an exact
(rational) dot product within the stated bound of 2^-47.7 max|P_r| max|x|.
"""
from fractions import Fraction

import numpy as np

N_DIG = 6
BIAS = 512 * sum(1 << (10 * j) for j in range(N_DIG))


def fixed_biased(x, emax):
    """F + B for doubles x against the group exponent emax (biased), as
    fixed_biased() in the kernel: F = sign * (m << 4) >> (emax - e)."""
    b = np.asarray(x, dtype=np.float64).view(np.uint64)
    e = ((b >> np.uint64(52)) & np.uint64(0x7ff)).astype(np.int64)
    mant = (b & np.uint64((1 << 52) - 1)).astype(object)
    m = [int(mm) | ((1 << 52) if int(ee) else 0) for mm, ee in zip(mant, e)]
    out = []
    for mm, ee, bb in zip(m, e, b):
        ee = int(ee)
        s = int(emax) - (ee if ee else 1)
        f = (mm << 4) >> s if s < 64 else 0
        if int(bb) >> 63:
            f = -f
        out.append((f + BIAS) % (1 << 64))
    return out


def exp_eff(x):
    b = np.asarray(x, dtype=np.float64).view(np.uint64)
    e = ((b >> np.uint64(52)) & np.uint64(0x7ff)).astype(np.int64)
    return np.where(e == 0, 1, e)


def digits(u):
    """Balanced digits d_0..d_5 (d_0 most significant) of F = u - B."""
    return [((u >> (10 * (N_DIG - 1 - j))) & 0x3ff) - 512 for j in range(N_DIG)]


def test_split_is_exact_and_digits_are_fp16():
    rng = np.random.default_rng(1)
    for scale in (1.0, 1e-300, 1e300, 3e-310):
        x = rng.standard_normal(16) * scale
        x[3] = 0.0
        x[5] = -x[5] * 1e-9
        emax = int(exp_eff(x).max())
        for xv, u in zip(x, fixed_biased(x, emax)):
            assert 0 < u < (1 << 60)
            d = digits(u)
            assert all(-512 <= v < 512 for v in d) and abs(d[0]) <= 128
            f = sum(v << (10 * (N_DIG - 1 - j)) for j, v in enumerate(d))
            # F reproduces x to 2^-57 of the group scale 2^(emax - 1022)
            approx = Fraction(f) * Fraction(2) ** (emax - 1022 - 57)
            assert abs(approx - Fraction(float(xv))) <= \
                Fraction(2) ** (emax - 1022 - 57)
            # the FP16 pattern 0x6400 | v is 1024 + v; minus 1536 is the digit
            for v in d:
                h = np.array([0x6400 | (v + 512)], dtype=np.uint16).view(
                    np.float16)[0]
                assert float(h) - 1536.0 == v
                assert float(np.float16(v)) == v


def _row_digits(row):
    emax = int(exp_eff(row).max())
    return [digits(u) for u in fixed_biased(row, emax)], emax


def _tc_dot(prow, x):
    """The kernel's result for one row and one group: level sums of digit
    pair products (i + j <= 5), FP32 accumulation, int64 recombination,
    scale 2^(Ex + Ep - 54)."""
    pd, ep = _row_digits(prow)
    xd, ex = _row_digits(x)
    levels = []
    for lev in range(N_DIG):
        tot = 0
        for i in range(lev + 1):
            j = lev - i
            s = sum(pd[k][i] * xd[k][j] for k in range(16))
            assert abs(s) <= 1 << 22
            tot += s
        if lev <= 3:
            assert abs(tot) <= 1 << 24  # exact in the FP32 accumulator
        levels.append(int(np.float32(tot)))  # FP32 rounding of the level
    v = (levels[0] << 40) + (levels[1] << 30) + (levels[2] << 20) + \
        (levels[3] << 10) + levels[4] + (levels[5] >> 10)
    return Fraction(v) * Fraction(2) ** ((ex - 1022) + (ep - 1022) - 54)


def test_products_within_bound():
    rng = np.random.default_rng(2)
    worst = 0.0
    for trial in range(60):
        p = rng.standard_normal(16)
        x = rng.standard_normal(16) * 10.0 ** rng.uniform(-5, 5)
        if trial % 3 == 0:
            p *= rng.random(16) < 0.5
            x[rng.integers(16)] *= 1e-12
        exact = sum(Fraction(float(a)) * Fraction(float(b))
                    for a, b in zip(p, x))
        got = _tc_dot(p, x)
        scale = float(np.abs(p).max() * np.abs(x).max())
        err = abs(float(got - exact)) / scale
        worst = max(worst, err)
    assert worst <= 2.0 ** -47.7, worst

// Device helpers shared by the precompiled kernels and the run-time
// specialised (NVRTC) kernels: 64-bit division by an invariant divisor and
// float-float ("df64") arithmetic.  Self-contained: no system headers, so the
// same text compiles under nvcc and NVRTC.
//
// Why df64: on GB300 the FP64 pipe issues ~0.6 T DFMA/s (measured 1.19
// TFLOP/s) against 6.7 TB/s of HBM, i.e. ~1.3 FP64 ops per streamed element.
// Rows of a PTM with more terms than that are computed on the FP32 pipes
// (~58x faster) as pairs of floats with a 48-bit significand, well inside the
// 1e-12 agreement required against float64 numpy.
#ifndef QSGB_DEVICE_CUH_
#define QSGB_DEVICE_CUH_

typedef unsigned long long qsgb_u64;
typedef long long qsgb_i64;

// Unsigned 64-bit division by an invariant divisor d (Granlund & Montgomery,
// "Division by invariant integers using multiplication", PLDI 1994, Fig. 4.1,
// N = 64): q = (t + ((n - t) >> 1)) >> (l - 1), t = mulhi(m, n), with
// l = ceil(log2 d) and m = floor(2^64 (2^l - d) / d) + 1; l == 0 encodes d = 1.
__device__ __forceinline__ qsgb_u64 qsgb_fdiv(qsgb_u64 n, qsgb_u64 m, int l) {
  if (l == 0) return n;
  const qsgb_u64 t = __umul64hi(m, n);
  return (t + ((n - t) >> 1)) >> (l - 1);
}

// Split an IEEE double into hi + lo floats with integer operations only (the
// FP64<->FP32 converters run on the slow FP64 pipe on GB300).  hi keeps the
// top 24 significant bits (truncated), lo the next 23 bits rounded to
// nearest on the 24th, so hi + lo agrees with x to 2^-47 relative, with an
// error of either sign: a truncated lo would shrink every input by 2^-48 on
// average, and that bias accumulates linearly over a long circuit (1050
// applications: ~1e-12 relative) where unbiased errors grow as a square
// root.  Inputs the float pair cannot carry to that
// precision set `bad`: a non-zero |x| < 2^-102 (|x| < 2^-126 flushes to 0,
// [2^-126, 2^-102) keeps only hi) and |x| >= 2^128, inf and nan (which give
// nan).  Callers recompute the affected results in native FP64.
__device__ __forceinline__ void qsgb_split_f64(double x, float& hi, float& lo, unsigned& bad) {
  const unsigned h = (unsigned)__double2hiint(x);
  const unsigned l = (unsigned)__double2loint(x);
  const unsigned e = (h >> 20) & 0x7ffu;
  const unsigned sgn = h & 0x80000000u;
  // bits 30..23 <- e[7:0], 22..0 <- m[51:29]; rebias e-1023+127 = e-896,
  // which on the low 8 exponent bits is an xor with 0x80 (bit 30)
  const unsigned t = __funnelshift_l(l, h, 3);
  const unsigned hb = ((t & 0x7fffffffu) ^ 0x40000000u) | sgn;
  const unsigned base = (hb & 0xff800000u) - (23u << 23);  // weight of m[28] is 2^(E-24)
  // m[28:6] rounded on m[5]: 0 .. 2^23, added (not or-ed) to base so that a
  // carry out of the 23 bits lands in base's exponent (still exact)
  const unsigned lb = base + ((l >> 6) & 0x7fffffu) + ((l >> 5) & 1u);
  const float lo_full = __uint_as_float(lb) - __uint_as_float(base);
  const bool in_range = (e - 897u) <= 253u;  // 897 <= e <= 1150
  const bool has_lo = e >= 920u;
  hi = in_range ? __uint_as_float(hb) : (e < 897u ? __uint_as_float(sgn) : __int_as_float(0x7fc00000));
  lo = (in_range && has_lo) ? lo_full : 0.0f;
  // e in [921, 1150] is 2^-102 <= |x| < 2^128; e == 0 with a zero
  // mantissa is an exact zero, carried exactly
  bad |= ((e - 921u) > 229u && ((h << 1) | l) != 0u) ? 1u : 0u;
}

// A float-float row result whose leading float s is outside the range where
// the pair keeps 48 significant bits: 0 < |s| < 2^-70 (products whose error
// terms may have fallen below the normal floats) or |s| >= 2^126 (near
// overflow), inf or nan.  s == 0 is exact when every input of the row is
// (inputs below 2^-102 are flagged by qsgb_split_f64).  Callers recompute
// such rows in native FP64.
__device__ __forceinline__ unsigned qsgb_df_suspect(float s) {
  const unsigned b = __float_as_uint(s) & 0x7fffffffu;
  return ((b - 1u) < 0x1c7fffffu || b >= 0x7e800000u) ? 1u : 0u;
}

// acc (s, c) += (ph + pl) * (xh + xl); pl*xl (2^-48 relative) is dropped.
__device__ __forceinline__ void qsgb_df_fma(float& s, float& c, float ph, float pl, float xh, float xl) {
  const float p = ph * xh;
  float e = fmaf(ph, xh, -p);  // exact product error
  e = fmaf(ph, xl, e);
  e = fmaf(pl, xh, e);
  const float s2 = s + p;  // two-sum (Knuth)
  const float bp = s2 - s;
  const float err = (s - (s2 - bp)) + (p - bp);
  s = s2;
  c += err + e;
}

// first term of a row: (s, c) = (ph + pl) * (xh + xl)
__device__ __forceinline__ void qsgb_df_mul(float& s, float& c, float ph, float pl, float xh, float xl) {
  const float p = ph * xh;
  float e = fmaf(ph, xh, -p);
  e = fmaf(ph, xl, e);
  c = fmaf(pl, xh, e);
  s = p;
}

// Round s + t (any magnitudes) to the nearest double, with integer
// operations and one float->int conversion.  After a two-sum (r, u) with
// |u| <= ulp_f(r)/2, the double is bits(r) + round(u / ulp_d(r)) ulps; when r
// is a power of two and u points toward zero the next ulp is half as large.
// |r| < 2^-74 keeps r only; r == 0 or denormal gives +-0.
__device__ __forceinline__ double qsgb_df_to_double(float s, float t) {
  const float r = s + t;  // two-sum: no ordering assumption on |s|, |t|
  const float bt = r - s;
  const float u = (s - (r - bt)) + (t - bt);
  const unsigned rb = __float_as_uint(r);
  const unsigned er = (rb >> 23) & 0xffu;
  const unsigned m = rb & 0x7fffffu;
  const unsigned sgn = rb & 0x80000000u;
  const bool toward0 = ((__float_as_uint(u) ^ rb) & 0x80000000u) != 0u;
  const unsigned sc = 306u - er + ((m == 0u && toward0) ? 1u : 0u);
  const float scale = (er >= 54u) ? __uint_as_float(sc << 23) : 0.0f;
  int T = __float2int_rn(u * scale);  // u in units of the target ulp
  if (sgn) T = -T;                   // magnitude domain
  const qsgb_u64 mag = ((qsgb_u64)(((er + 896u) << 20) | (m >> 3)) << 32) | (qsgb_u64)(m << 29);
  qsgb_u64 bits = mag + (qsgb_u64)(qsgb_i64)T;
  if (er == 0u) bits = 0;
  if (er == 255u) bits = 0x7ff8000000000000ull;
  return __longlong_as_double((long long)(bits | ((qsgb_u64)sgn << 32)));
}

#endif  // QSGB_DEVICE_CUH_

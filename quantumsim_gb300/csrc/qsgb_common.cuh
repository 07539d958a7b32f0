// Shared device helpers of the GB300 Pauli-vector kernels: launch plumbing,
// 64-bit division by loop-invariant divisors, and the float-float ("df64")
// arithmetic used for FP64-storage PTM application.
//
// Why df64: on GB300 the FP64 pipe issues ~0.6 T DFMA/s (measured 1.19
// TFLOP/s) against 6.7 TB/s of HBM, i.e. <= 1.2 FP64 ops per streamed
// element.  A 4x4 PTM needs 4 FMAs per element and a 16x16 one 16, so native
// FP64 cannot keep up with memory.  The FP32 pipes are ~58x faster; a pair of
// floats carries a 48-bit significand, well inside the 1e-12 agreement
// required against float64 numpy.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/qsgb.h"

#define QSGB_CUDA_TRY(expr)                               \
  do {                                                    \
    cudaError_t qsgb_e_ = (expr);                         \
    if (qsgb_e_ != cudaSuccess) return QSGB_ERR_CUDA;     \
  } while (0)

namespace qsgb {

constexpr int kNumSMs = 152;  // GB300; the launchers query the device anyway

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

int sm_count();         // cached per device
int launch_status();    // cudaGetLastError mapped to a status code

// ---------------------------------------------------------------------------
// Unsigned 64-bit division by an invariant divisor (Granlund & Montgomery,
// "Division by invariant integers using multiplication", PLDI 1994, Fig. 4.1,
// N = 64): q = (t + ((n - t) >> 1)) >> (l - 1), t = mulhi(m, n), with
// l = ceil(log2 d) and m = floor(2^64 (2^l - d) / d) + 1.  d == 1 uses
// l = 0 handled as a plain copy.
// ---------------------------------------------------------------------------
struct FastDiv {
  uint64_t d;
  uint64_t m;
  int l;  // 0 => divisor 1
};

inline FastDiv make_fastdiv(uint64_t d) {
  FastDiv f;
  f.d = d;
  if (d <= 1) {
    f.m = 0;
    f.l = 0;
    return f;
  }
  int l = 0;
  while (l < 64 && (uint64_t(1) << l) < d) ++l;
  // m = floor(2^64 * (2^l - d) / d) + 1 computed with 128-bit arithmetic
  unsigned __int128 two_l = (l == 64) ? ((unsigned __int128)1 << 64) : ((unsigned __int128)1 << l);
  unsigned __int128 num = ((unsigned __int128)(two_l - d)) << 64;
  f.m = (uint64_t)(num / d) + 1;
  f.l = l;
  return f;
}

__device__ __forceinline__ uint64_t fdiv(uint64_t n, const FastDiv& f) {
  if (f.l == 0) return n;
  uint64_t t = __umul64hi(f.m, n);
  return (t + ((n - t) >> 1)) >> (f.l - 1);
}

// ---------------------------------------------------------------------------
// float-float arithmetic
// ---------------------------------------------------------------------------

// Split an IEEE double into hi + lo floats with integer operations only (the
// FP64<->FP32 converters run on the slow FP64 pipe on GB300).  hi keeps the
// top 24 significant bits (truncated), lo the next 23 bits, so hi + lo agrees
// with x to 2^-47 relative.  |x| < 2^-126 flushes to 0, |x| in
// [2^-126, 2^-102) keeps only hi; |x| >= 2^128, inf and nan set `bad` and
// give nan.
__device__ __forceinline__ void split_f64(double x, float& hi, float& lo, unsigned& bad) {
  const unsigned h = (unsigned)__double2hiint(x);
  const unsigned l = (unsigned)__double2loint(x);
  const unsigned e = (h >> 20) & 0x7ffu;
  const unsigned sgn = h & 0x80000000u;
  // bits 30..23 <- e[7:0], 22..0 <- m[51:29]; rebias e-1023+127 = e-896,
  // which on the low 8 exponent bits is an xor with 0x80 (bit 30)
  const unsigned t = __funnelshift_l(l, h, 3);
  const unsigned hb = ((t & 0x7fffffffu) ^ 0x40000000u) | sgn;
  const unsigned base = (hb & 0xff800000u) - (23u << 23);  // weight of m[28] is 2^(E-24)
  const unsigned lb = base | ((l >> 6) & 0x7fffffu);
  const float lo_full = __uint_as_float(lb) - __uint_as_float(base);
  const bool in_range = (e - 897u) <= 253u;  // 897 <= e <= 1150
  const bool has_lo = e >= 920u;
  hi = in_range ? __uint_as_float(hb) : (e < 897u ? __uint_as_float(sgn) : __int_as_float(0x7fc00000));
  lo = (in_range && has_lo) ? lo_full : 0.0f;
  bad |= (e > 1150u) ? 1u : 0u;
}

// acc (s, c) += (ph + pl) * (xh + xl); pl*xl (2^-48 relative) is dropped.
__device__ __forceinline__ void df_fma(float& s, float& c, float ph, float pl, float xh, float xl) {
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
__device__ __forceinline__ void df_mul(float& s, float& c, float ph, float pl, float xh, float xl) {
  const float p = ph * xh;
  float e = fmaf(ph, xh, -p);
  e = fmaf(ph, xl, e);
  c = fmaf(pl, xh, e);
  s = p;
}

// Round s + t (any magnitudes) to the nearest double, with integer
// operations and one float->int conversion.  After a two-sum
// (r, u) with |u| <= ulp_f(r)/2, the double is bits(r) + round(u / ulp_d(r))
// ulps; when r is a power of two and u points toward zero the next ulp is
// half as large.  |r| < 2^-74 keeps r only; r == 0 or denormal gives +-0.
__device__ __forceinline__ double df_to_double(float s, float t) {
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
  const uint64_t mag = ((uint64_t)(((er + 896u) << 20) | (m >> 3)) << 32) | (uint64_t)(m << 29);
  uint64_t bits = mag + (uint64_t)(int64_t)T;
  if (er == 0u) bits = 0;
  if (er == 255u) bits = 0x7ff8000000000000ull;
  return __longlong_as_double((long long)(bits | ((uint64_t)sgn << 32)));
}

}  // namespace qsgb

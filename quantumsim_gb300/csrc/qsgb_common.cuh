// Shared host/device helpers of the GB300 Pauli-vector kernels: launch
// plumbing, 64-bit division by loop-invariant divisors (host side of
// qsgb_device.cuh) and the float-float helpers under short names.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/qsgb.h"
#include "qsgb_device.cuh"

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
// Let kernel `func` take `bytes` of dynamic shared memory on the current
// device.  The attribute only ever grows: a launch captured in a CUDA graph
// with a larger size stays launchable after later launches of the same
// kernel ask for less.
int allow_dynamic_smem(const void* func, int bytes);

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

__device__ __forceinline__ uint64_t fdiv(uint64_t n, const FastDiv& f) { return qsgb_fdiv(n, f.m, f.l); }

// float-float helpers under the names used by the precompiled kernels
__device__ __forceinline__ void split_f64(double x, float& hi, float& lo, unsigned& bad) {
  qsgb_split_f64(x, hi, lo, bad);
}
__device__ __forceinline__ void df_fma(float& s, float& c, float ph, float pl, float xh, float xl) {
  qsgb_df_fma(s, c, ph, pl, xh, xl);
}
__device__ __forceinline__ void df_mul(float& s, float& c, float ph, float pl, float xh, float xl) {
  qsgb_df_mul(s, c, ph, pl, xh, xl);
}
__device__ __forceinline__ double df_to_double(float s, float t) { return qsgb_df_to_double(s, t); }

}  // namespace qsgb

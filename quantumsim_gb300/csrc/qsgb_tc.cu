// Dense two-qubit PTMs (16 x 16, FP64 storage) on the tensor cores.
//
// A dense PTM row has 16 terms: in float-float on the FP32 pipes that is
// ~12 instructions per term, and the kernel is bound by instruction issue at
// a quarter of the HBM rate; in native FP64 it is bound by the FP64 pipe
// (~0.6 T FMA/s on GB300).  This kernel computes the contraction exactly
// enough for FP64 parity on the FP16 tensor cores instead, with an
// error-free splitting in the spirit of the Ozaki scheme (Ozaki, Ogita,
// Oishi and Rump, "Error-free transformations of matrix multiplication by
// using fast routines of matrix multiplication and its applications",
// Numer. Algorithms 59, 2012):
//
//  * Each group of 16 inputs (one bystander index) is scaled by its largest
//    binary exponent and written as a signed fixed-point integer F of 57
//    bits plus sign (|F| < 2^57), with integer operations on the double's
//    bit pattern.  F + B, for B = 512 * sum_j 2^(10 j), is a non-negative
//    60-bit integer whose six base-1024 digits v_j give F = sum_j (v_j - 512)
//    2^(10 (5 - j)): six balanced digits d_j in [-512, 512), each exactly an
//    FP16 number (|d_0| <= 128).
//  * Each PTM row is split the same way on the host (per-row scale).
//  * For every pair of digit planes (i, j) with i + j <= 5 one
//    mma.sync.m16n8k16 (FP16 operands, FP32 accumulation) adds
//    sum_k e_ik d_jk to the accumulator of level L = i + j.  A product of two
//    digits is at most 2^18, a pair's K = 16 sum at most 2^22, and a level
//    holds at most four such sums below 2^24, where FP32 sums of integers
//    are exact; levels 4 and 5 may round their last bit, 2^-40 below level 0.
//  * The six level sums are combined in 64-bit integer arithmetic,
//    V = sum_L A_L 2^(10 (4 - L)), converted to double once and scaled by
//    2^(Ex + Ep_r - 54) on the exponent field.
//
// The dropped levels (i + j >= 6) and the 57-bit truncation of inputs and
// PTM entries bound the error by about 2^-47.7 * max_k |P_rk| * max_k |x_k|
// of the row and group (4.4e-15 of that product), against 16 * 2^-53 *
// sum_k |P_rk| |x_k| for an FP64 dot product.  Groups whose inputs hold inf,
// nan, or whose results leave the normal double range are recomputed in
// native FP64 by the same warp.
//
// Work mapping: a warp takes tiles of 8 groups (the N of the MMA).  Lane
// (g, c) = (lane / 4, lane % 4) loads inputs k in {2c, 2c+1, 2c+8, 2c+9} of
// group g (the B fragment layout of m16n8k16), and ends with outputs rows
// {g, g+8} of groups {2c, 2c+1} (the accumulator layout).  The PTM digit
// planes (the A fragments) are loaded into registers once per warp.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "qsgb_common.cuh"
#include "qsgb_tc.h"

namespace qsgb {
namespace tc {
namespace {

constexpr int kBlock = 256;


// 2^sc * sum_L A_L 2^(10 (4 - L)); bad |= 1 when the result is not a normal
// double (or zero).
__device__ __forceinline__ double combine(const float (&acc)[kDigits][4], int s, int sc, unsigned& bad) {
  long long v = (long long)__float2int_rn(acc[0][s]) << 40;
  v += (long long)__float2int_rn(acc[1][s]) << 30;
  v += (long long)__float2int_rn(acc[2][s]) << 20;
  v += (long long)__float2int_rn(acc[3][s]) << 10;
  v += (long long)__float2int_rn(acc[4][s]);
  v += (long long)(__float2int_rn(acc[5][s]) >> 10);
  if (v == 0) return 0.0;
  const double d = __ll2double_rn(v);
  const int hi = __double2hiint(d);
  const int e = ((hi >> 20) & 0x7ff) + sc;
  bad |= (e < 1 || e > 2046) ? 1u : 0u;
  return __hiloint2double(hi + (sc << 20), __double2loint(d));
}

template <bool CONTIG>
__global__ void __launch_bounds__(kBlock) apply16_tc_kernel(const __grid_constant__ TcParams p) {
  const int lane = threadIdx.x & 31;
  const int g = lane >> 2, c = lane & 3;
  const int warps = kBlock / 32;
  // A fragments of every digit plane: rows {g, g+8}, columns {2c, 2c+1} and
  // {2c+8, 2c+9}
  unsigned A[kDigits][4];
#pragma unroll
  for (int i = 0; i < kDigits; ++i) {
    const unsigned short* d = &p.digits[i][0][0];
    A[i][0] = d[g * 16 + 2 * c] | ((unsigned)d[g * 16 + 2 * c + 1] << 16);
    A[i][1] = d[(g + 8) * 16 + 2 * c] | ((unsigned)d[(g + 8) * 16 + 2 * c + 1] << 16);
    A[i][2] = d[g * 16 + 2 * c + 8] | ((unsigned)d[g * 16 + 2 * c + 9] << 16);
    A[i][3] = d[(g + 8) * 16 + 2 * c + 8] | ((unsigned)d[(g + 8) * 16 + 2 * c + 9] << 16);
  }
  const int rsc0 = p.row_exp[g], rsc1 = p.row_exp[g + 8];
  // this lane's inputs k = (ka, kb): 2c -> (c/2, 2(c%2)), +1 -> kb + 1,
  // +8 -> ka + 2
  const int ka = c >> 1, kb = 2 * (c & 1);
  const int64_t in_off0 = ka * p.sai + kb * p.sbi;
  const int64_t in_off2 = in_off0 + 2 * p.sai;
  // this lane's outputs: rows g = (g/4, g%4) and g + 8 = (g/4 + 2, g%4)
  const int64_t out_off0 = (g >> 2) * p.sao + (g & 3) * p.sbo;
  const int64_t out_off1 = out_off0 + 2 * p.sao;

  auto base = [&](uint64_t grp, int64_t sx, int64_t sy) -> int64_t {
    const uint64_t t1 = fdiv(grp, p.div_z);
    const uint64_t z = grp - t1 * p.div_z.d;
    const uint64_t x = fdiv(t1, p.div_y);
    const uint64_t y = t1 - x * p.div_y.d;
    return (int64_t)x * sx + (int64_t)y * sy + (int64_t)z;
  };

  const uint64_t wstride = (uint64_t)gridDim.x * warps;
  for (uint64_t tile = (uint64_t)blockIdx.x * warps + (threadIdx.x >> 5); tile < p.n_tiles; tile += wstride) {
    const uint64_t g0 = tile * 8;
    const uint64_t gi = g0 + g;  // this lane's input group
    const bool live = gi < p.n_groups;
    int64_t bi;
    if (CONTIG) {
      // 8 consecutive groups are 8 consecutive z of one (x, y)
      bi = base(g0, p.sxi, p.syi) + g;
    } else {
      bi = live ? base(gi, p.sxi, p.syi) : 0;
    }
    double x[4] = {0.0, 0.0, 0.0, 0.0};
    if (live) {
      x[0] = p.in[bi + in_off0];
      x[1] = p.in[bi + in_off0 + p.sbi];
      x[2] = p.in[bi + in_off2];
      x[3] = p.in[bi + in_off2 + p.sbi];
    }
    unsigned hi[4], lo[4];
    unsigned emax = 1u, bad = 0u;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      hi[i] = (unsigned)__double2hiint(x[i]);
      lo[i] = (unsigned)__double2loint(x[i]);
      emax = max(emax, exp_eff(hi[i]));
      bad |= ((hi[i] >> 20) & 0x7ffu) == 0x7ffu ? 1u : 0u;  // inf, nan
    }
    emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, 1));
    emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, 2));
    unsigned long long u[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) u[i] = fixed_biased(hi[i], lo[i], emax);
    unsigned B[kDigits][2];
#pragma unroll
    for (int j = 0; j < kDigits; ++j) {
      B[j][0] = digit_pair(u[0], u[1], 10 * (kDigits - 1 - j));
      B[j][1] = digit_pair(u[2], u[3], 10 * (kDigits - 1 - j));
    }
    float acc[kDigits][4];
#pragma unroll
    for (int l = 0; l < kDigits; ++l) acc[l][0] = acc[l][1] = acc[l][2] = acc[l][3] = 0.f;
#pragma unroll
    for (int i = 0; i < kDigits; ++i)
#pragma unroll
      for (int j = 0; i + j < kDigits; ++j) mma16816(acc[i + j], A[i], B[j]);
    // output groups 2c and 2c+1: their exponents live in lanes 8c and 8c+4
    const int ex0 = (int)__shfl_sync(0xffffffffu, emax, 8 * c) - 1022;
    const int ex1 = (int)__shfl_sync(0xffffffffu, emax, 8 * c + 4) - 1022;
    double y[4];
    y[0] = combine(acc, 0, ex0 + rsc0, bad);  // row g, group 2c
    y[1] = combine(acc, 1, ex1 + rsc0, bad);  // row g, group 2c+1
    y[2] = combine(acc, 2, ex0 + rsc1, bad);  // row g+8, group 2c
    y[3] = combine(acc, 3, ex1 + rsc1, bad);  // row g+8, group 2c+1
    const uint64_t go0 = g0 + 2 * c, go1 = go0 + 1;
    int64_t bo0, bo1;
    if (CONTIG) {
      bo0 = base(g0, p.sxo, p.syo) + 2 * c;
      bo1 = bo0 + 1;
    } else {
      bo0 = go0 < p.n_groups ? base(go0, p.sxo, p.syo) : 0;
      bo1 = go1 < p.n_groups ? base(go1, p.sxo, p.syo) : 0;
    }
    if (__any_sync(0xffffffffu, bad)) {
      // inf / nan inputs or results outside the normal range: the tile's
      // outputs in native FP64 (lane: rows g, g+8 of groups 2c, 2c+1); the
      // loops over q and h are unrolled so that y[] stays in registers
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const uint64_t gq = q ? go1 : go0;
        if (gq < p.n_groups) {
          const int64_t b_in = base(gq, p.sxi, p.syi);
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int r = g + 8 * h;
            double a = 0.0;
#pragma unroll 1
            for (int k = 0; k < 16; ++k)
              a = fma(p.ptm[r][k], p.in[b_in + (k >> 2) * p.sai + (k & 3) * p.sbi], a);
            y[2 * h + q] = a;
          }
        }
      }
    }
    if (CONTIG && p.pair_store) {
      // groups 2c, 2c+1 are adjacent: 16-byte stores
      *reinterpret_cast<double2*>(p.out + bo0 + out_off0) = make_double2(y[0], y[1]);
      *reinterpret_cast<double2*>(p.out + bo0 + out_off1) = make_double2(y[2], y[3]);
    } else {
      if (go0 < p.n_groups) {
        p.out[bo0 + out_off0] = y[0];
        p.out[bo0 + out_off1] = y[2];
      }
      if (go1 < p.n_groups) {
        p.out[bo1 + out_off0] = y[1];
        p.out[bo1 + out_off1] = y[3];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// tcgen05 form: one thread per group, 128 groups per tile (the M of one
// tcgen05.mma), the six level accumulators in tensor memory.
//
// Per tile, each thread loads its group's 16 inputs, splits them and writes
// its row of the six input digit planes (the A operand, 128 x 16 FP16 each)
// to shared memory; one thread issues the 21 tcgen05.mma.kind::f16 (A = input
// plane j, B = PTM plane i, both K-major, D = level i + j: 16 FP32 columns of
// tensor memory) and commits them to an mbarrier; after the barrier each warp
// reads its 32 lanes (groups) of the accumulators with tcgen05.ld and
// recombines its outputs.  Shared-memory operands use the canonical K-major
// layout without swizzling: core matrices of 8 rows x 16 bytes (8 FP16 along
// K) at (row / 8) * 256 + (k / 8) * 128, so the descriptors carry a leading
// (K) byte offset of 128 and a stride (8-row) byte offset of 256.
constexpr int kUBlock = 128;
constexpr int kPlaneA = 128 * 16 * 2;  // one input digit plane: 128 rows x 16 FP16
constexpr int kPlaneB = 16 * 16 * 2;   // one PTM digit plane: 16 rows x 16 FP16
constexpr int kSmemB = kDigits * kPlaneA;             // 24576
constexpr int kSmemBar = kSmemB + kDigits * kPlaneB;  // 27648
constexpr int kSmemTmem = kSmemBar + 8;
constexpr int kSmemFlag = kSmemTmem + 4;
constexpr int kSmemRowExp = kSmemBar + 32;  // int[16] (device PTMs)
static_assert(kSmemRowExp % 16 == 0 && kSmemRowExp + 64 <= 56 * 1024, "shared-memory layout");
// the dynamic allocation is padded so that at most 4 blocks share an SM:
// 4 x 128 tensor-memory columns fill its 512
constexpr int kUmmaSmem = 56 * 1024;
constexpr unsigned kTmemCols = 128;  // 6 levels x 16 columns, a power of two
// kind::f16 instruction descriptor: D F32 (bits 4-5 = 1), A and B F16 (0),
// both K-major, N / 8 at bits 17-22, M / 16 at bits 24-28
constexpr uint32_t kIdesc = (1u << 4) | ((16u >> 3) << 17) | ((128u >> 4) << 24);
constexpr long long kSpinLimit = 1ll << 26;

__host__ __device__ constexpr int core_off(int row, int k) {
  return (row >> 3) * 256 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

// shared-memory matrix descriptor: start >> 4 (bits 0-13), leading byte
// offset >> 4 (16-29), stride byte offset >> 4 (32-45), version 1 (46-47),
// no swizzling (61-63 = 0)
__device__ __forceinline__ unsigned long long smem_desc(uint32_t saddr) {
  return (unsigned long long)((saddr >> 4) & 0x3fffu) | ((unsigned long long)(128 >> 4) << 16) |
         ((unsigned long long)(256 >> 4) << 32) | (1ull << 46);
}

__device__ __forceinline__ uint32_t tmem_ld4(uint32_t addr, uint32_t (&r)[4]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr));
  return 0;
}

// 2^sc * sum_L A_L 2^(10 (4 - L)) from the raw FP32 words of the six levels
__device__ __forceinline__ double combine_words(const uint32_t (&w)[kDigits], int sc, unsigned& bad) {
  long long v = (long long)__float2int_rn(__uint_as_float(w[0])) << 40;
  v += (long long)__float2int_rn(__uint_as_float(w[1])) << 30;
  v += (long long)__float2int_rn(__uint_as_float(w[2])) << 20;
  v += (long long)__float2int_rn(__uint_as_float(w[3])) << 10;
  v += (long long)__float2int_rn(__uint_as_float(w[4]));
  v += (long long)(__float2int_rn(__uint_as_float(w[5])) >> 10);
  if (v == 0) return 0.0;
  const double d = __ll2double_rn(v);
  const int hi = __double2hiint(d);
  const int e = ((hi >> 20) & 0x7ff) + sc;
  bad |= (e < 1 || e > 2046) ? 1u : 0u;
  return __hiloint2double(hi + (sc << 20), __double2loint(d));
}

// Offset of op element (r, k) in a 16 x 16 two-qubit PTM stored in `layout`.
__device__ __forceinline__ int dev_index(int layout, int r, int k) {
  const int ra = r >> 2, rb = r & 3, ka = k >> 2, kb = k & 3;
  switch (layout & 3) {
    case 0:
      return r * 16 + k;
    case QSGB_PTM_SWAPPED:  // (rb, ra, kb, ka)
      return ((rb * 4 + ra) * 4 + kb) * 4 + ka;
    case QSGB_PTM_TRANSPOSED:  // forward (ka, kb, ra, rb)
      return k * 16 + r;
    default:  // forward swapped (kb, ka, rb, ra)
      return ((kb * 4 + ka) * 4 + rb) * 4 + ra;
  }
}

// DEVP: the PTM is in device memory (p.dptm); threads 0..15 split one row
// each into the B operand planes (the fixed point and digits of the host
// split) and the row scales, in shared memory.
template <bool CONTIG, bool DEVP>
__global__ void __launch_bounds__(kUBlock) apply16_umma_kernel(const __grid_constant__ TcParams p) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const int t = threadIdx.x, warp = t >> 5;
  const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(smem);
  const uint32_t sA = sbase, sB = sbase + kSmemB, bar = sbase + kSmemBar;
  volatile uint32_t* tslot = reinterpret_cast<volatile uint32_t*>(smem + kSmemTmem);
  volatile uint32_t* flag = reinterpret_cast<volatile uint32_t*>(smem + kSmemFlag);
  const int64_t sai = p.sai, sbi = p.sbi;

  auto base = [&](uint64_t grp) -> int64_t {
    const uint64_t t1 = fdiv(grp, p.div_z);
    const uint64_t z = grp - t1 * p.div_z.d;
    const uint64_t x = fdiv(t1, p.div_y);
    const uint64_t y = t1 - x * p.div_y.d;
    return (int64_t)x * p.sxi + (int64_t)y * p.syi + (int64_t)z;
  };

  // a tile's inputs: this thread's group, 16 values; with unit stride along
  // the last target (Z == 1, tensors 16-byte aligned) as 8 16-byte loads
  auto load_tile = [&](uint64_t tile, double (&x)[16], int64_t& b, bool& live) {
    const uint64_t gi = tile * kUBlock + t;
    live = tile < p.n_tiles && gi < p.n_groups;
    b = 0;
    if (CONTIG) {
      if (tile < p.n_tiles) b = base(tile * kUBlock) + t;  // 128 consecutive z of one (x, y)
    } else if (live) {
      b = base(gi);
    }
    if (!live) {
#pragma unroll
      for (int k = 0; k < 16; ++k) x[k] = 0.0;
    } else if (p.vec_z1) {
#pragma unroll
      for (int ka = 0; ka < 4; ++ka) {
        const double2 v0 = *reinterpret_cast<const double2*>(p.in + b + ka * sai);
        const double2 v1 = *reinterpret_cast<const double2*>(p.in + b + ka * sai + 2);
        x[4 * ka] = v0.x;
        x[4 * ka + 1] = v0.y;
        x[4 * ka + 2] = v1.x;
        x[4 * ka + 3] = v1.y;
      }
    } else {
#pragma unroll
      for (int k = 0; k < 16; ++k) x[k] = p.in[b + (k >> 2) * sai + (k & 3) * sbi];
    }
  };

  uint32_t phase = 0;
  bool timed_out = false;
  double x[16];
  int64_t b;
  bool live;
  uint64_t tile = blockIdx.x;
  load_tile(tile, x, b, live);  // in flight during the set-up below
  int* srow = reinterpret_cast<int*>(smem + kSmemRowExp);
  int ptm_bad = 0;  // device PTM with inf or nan entries (this thread's pair)
  if (DEVP) {
    // 8 threads per row (lanes 8r' .. 8r'+7 of a warp), two entries each
    const int r = t >> 3, k = 2 * (t & 7);
    const double v0 = p.dptm[dev_index(p.dlayout, r, k)];
    const double v1 = p.dptm[dev_index(p.dlayout, r, k + 1)];
    const unsigned h0 = (unsigned)__double2hiint(v0), h1 = (unsigned)__double2hiint(v1);
    unsigned emax = max(exp_eff(h0), exp_eff(h1));
    emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, 1));
    emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, 2));
    emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, 4));
    ptm_bad = (((h0 >> 20) & 0x7ffu) == 0x7ffu || ((h1 >> 20) & 0x7ffu) == 0x7ffu) ? 1 : 0;
    const unsigned long long u0 = fixed_biased(h0, (unsigned)__double2loint(v0), emax);
    const unsigned long long u1 = fixed_biased(h1, (unsigned)__double2loint(v1), emax);
#pragma unroll
    for (int j = 0; j < kDigits; ++j)
      *reinterpret_cast<unsigned*>(smem + kSmemB + j * kPlaneB + core_off(r, k)) =
          digit_pair(u0, u1, 10 * (kDigits - 1 - j));
    if ((t & 7) == 0) srow[r] = (int)emax - 1022 - 54;
  } else {  // PTM digit planes (the B operand), split on the host
    const uint4* src = reinterpret_cast<const uint4*>(&p.bplanes[0][0]);
    uint4* dst = reinterpret_cast<uint4*>(smem + kSmemB);
    for (int i = t; i < kDigits * kPlaneB / 16; i += kUBlock) dst[i] = src[i];
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sbase + kSmemTmem),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  ptm_bad = __syncthreads_or(ptm_bad);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  const uint32_t tlane = tmem + ((uint32_t)(32 * warp) << 16);
  for (; tile < p.n_tiles; tile += gridDim.x) {
    unsigned emax = 1u, bad = ptm_bad ? 1u : 0u;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const unsigned h = (unsigned)__double2hiint(x[k]);
      emax = max(emax, exp_eff(h));
      bad |= ((h >> 20) & 0x7ffu) == 0x7ffu ? 1u : 0u;
    }
    {
      unsigned long long u[16];
#pragma unroll
      for (int k = 0; k < 16; ++k)
        u[k] = fixed_biased((unsigned)__double2hiint(x[k]), (unsigned)__double2loint(x[k]), emax);
      // this thread's row of the six input digit planes
#pragma unroll
      for (int j = 0; j < kDigits; ++j) {
        const int pos = 10 * (kDigits - 1 - j);
        uint4 lo4, hi4;
        lo4.x = digit_pair(u[0], u[1], pos);
        lo4.y = digit_pair(u[2], u[3], pos);
        lo4.z = digit_pair(u[4], u[5], pos);
        lo4.w = digit_pair(u[6], u[7], pos);
        hi4.x = digit_pair(u[8], u[9], pos);
        hi4.y = digit_pair(u[10], u[11], pos);
        hi4.z = digit_pair(u[12], u[13], pos);
        hi4.w = digit_pair(u[14], u[15], pos);
        *reinterpret_cast<uint4*>(smem + j * kPlaneA + core_off(t, 0)) = lo4;
        *reinterpret_cast<uint4*>(smem + j * kPlaneA + core_off(t, 8)) = hi4;
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (t == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int i = 0; i < kDigits; ++i) {
        const unsigned long long bdesc = smem_desc(sB + i * kPlaneB);
#pragma unroll
        for (int j = 0; i + j < kDigits; ++j) {
          const unsigned long long adesc = smem_desc(sA + j * kPlaneA);
          const uint32_t d = tmem + 16u * (uint32_t)(i + j);
          const uint32_t accumulate = i > 0 ? 1u : 0u;  // pair (0, L) starts level L
          asm volatile(
              "{ .reg .pred q; setp.ne.u32 q, %4, 0; "
              "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, q; }" ::"r"(d),
              "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
              : "memory");
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                   : "memory");
    }
    // the next tile's inputs load while the tensor cores and the
    // recombination work on this one
    const int64_t bc = b;
    const bool livec = live;
    double xn[16];
    load_tile(tile + gridDim.x, xn, b, live);
    if (t == 0) {
      uint32_t done = 0;
      for (long long spin = 0; spin < kSpinLimit && !done; ++spin)
        asm volatile(
            "{ .reg .pred q; mbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2; selp.u32 %0, 1, 0, q; }"
            : "=r"(done)
            : "r"(bar), "r"(phase)
            : "memory");
      *flag = done;
    }
    phase ^= 1u;
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (*flag == 0u) {  // the same value in every thread
      timed_out = true;
      break;
    }
    // outputs: rows r = 4c .. 4c + 3 = (ra = c, rb = 0 .. 3), six levels each
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      uint32_t w[kDigits][4];
#pragma unroll
      for (int l = 0; l < kDigits; ++l) tmem_ld4(tlane + 16u * l + 4u * c, w[l]);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      double y[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const uint32_t lv[kDigits] = {w[0][q], w[1][q], w[2][q], w[3][q], w[4][q], w[5][q]};
        y[q] = combine_words(lv, (int)emax - 1022 + (DEVP ? srow[4 * c + q] : p.row_exp[4 * c + q]), bad);
      }
      if (livec) {
        if (p.vec_z1) {
          *reinterpret_cast<double2*>(p.out + bc + c * p.sao) = make_double2(y[0], y[1]);
          *reinterpret_cast<double2*>(p.out + bc + c * p.sao + 2) = make_double2(y[2], y[3]);
        } else {
#pragma unroll
          for (int q = 0; q < 4; ++q) p.out[bc + c * p.sao + q * p.sbo] = y[q];
        }
      }
    }
    if (bad && livec) {
      // inf / nan inputs or results outside the normal range: this group's
      // outputs again in native FP64
#pragma unroll 1
      for (int r = 0; r < 16; ++r) {
        double a = 0.0;
#pragma unroll 1
        for (int k = 0; k < 16; ++k) {
          const double pk = DEVP ? p.dptm[dev_index(p.dlayout, r, k)] : p.ptm[r][k];
          a = fma(pk, p.in[bc + (k >> 2) * sai + (k & 3) * sbi], a);
        }
        p.out[bc + (r >> 2) * p.sao + (r & 3) * p.sbo] = a;
      }
    }
#pragma unroll
    for (int k = 0; k < 16; ++k) x[k] = xn[k];
  }
  if (timed_out && t == 0) {
    if (p.status) atomicOr(p.status, QSGB_DEV_TIMEOUT);
    // bounded wait for the MMAs still in flight before the memory is freed
    uint32_t done = 0;
    for (long long spin = 0; spin < kSpinLimit && !done; ++spin)
      asm volatile(
          "{ .reg .pred q; mbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2; selp.u32 %0, 1, 0, q; }"
          : "=r"(done)
          : "r"(bar), "r"(phase ^ 1u)
          : "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
}

// FP16 bit pattern of an integer |v| <= 2048 (exact).
unsigned short half_bits(int v) {
  if (v == 0) return 0;
  const unsigned sgn = v < 0 ? 0x8000u : 0u;
  unsigned a = (unsigned)std::abs(v);
  int e = 31 - __builtin_clz(a);  // a in [2^e, 2^(e+1))
  const unsigned mant = (a << (10 - e)) & 0x3ffu;
  return (unsigned short)(sgn | ((unsigned)(e + 15) << 10) | mant);
}

// Host split of one PTM row (same fixed point as the device inputs).
void split_row(const double* row, unsigned short (*dig)[16][16], int r, int* row_exp) {
  unsigned emax = 1;
  for (int k = 0; k < 16; ++k) {
    uint64_t b;
    std::memcpy(&b, &row[k], 8);
    const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
    emax = std::max(emax, e == 0u ? 1u : e);
  }
  for (int k = 0; k < 16; ++k) {
    uint64_t b;
    std::memcpy(&b, &row[k], 8);
    const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
    const uint64_t m = ((b & 0xfffffffffffffull) | (e != 0u ? (1ull << 52) : 0ull)) << 4;
    const unsigned s = emax - (e == 0u ? 1u : e);
    uint64_t f = s < 64u ? (m >> s) : 0ull;
    if (b >> 63) f = 0ull - f;
    const uint64_t u = f + kDigitBias;
    for (int j = 0; j < kDigits; ++j) {
      const int v = (int)((u >> (10 * (kDigits - 1 - j))) & 0x3ffu) - 512;
      dig[j][r][k] = half_bits(v);
    }
  }
  row_exp[r] = (int)emax - 1022 - 54;
}

}  // namespace

bool eligible(const double* ptm_host, int kin, int kout) {
  if (kin != 16 || kout != 16) return false;
  for (int i = 0; i < 256; ++i) {
    uint64_t b;
    std::memcpy(&b, &ptm_host[i], 8);
    if (((b >> 52) & 0x7ffu) == 0x7ffu) return false;  // inf, nan
  }
  return true;
}

namespace {

void set_geometry(TcParams& p, const void* in, void* out, uint64_t X, uint64_t Y, uint64_t Z, unsigned* status) {
  p.in = static_cast<const double*>(in);
  p.out = static_cast<double*>(out);
  p.status = status;
  p.n_groups = X * Y * Z;
  p.n_tiles = (p.n_groups + 7) / 8;
  p.div_z = make_fastdiv(Z);
  p.div_y = make_fastdiv(Y);
  p.sbi = (int64_t)Z;
  p.sai = (int64_t)(Y * 4 * Z);
  p.syi = 4 * (int64_t)Z;
  p.sxi = 16 * (int64_t)(Y * Z);
  p.sbo = p.sbi;
  p.sao = p.sai;
  p.syo = p.syi;
  p.sxo = p.sxi;
}

template <bool DEVP>
int launch_umma(TcParams& p, const void* in, void* out, uint64_t Z, cudaStream_t stream) {
  // tcgen05 form: tiles of 128 groups per block, at most 4 blocks per SM
  p.n_tiles = (p.n_groups + kUBlock - 1) / kUBlock;
  const bool contig = Z % kUBlock == 0;
  p.vec_z1 = Z == 1 && (uintptr_t)in % 16 == 0 && (uintptr_t)out % 16 == 0 ? 1 : 0;
  auto kern = contig ? apply16_umma_kernel<true, DEVP> : apply16_umma_kernel<false, DEVP>;
  QSGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kUmmaSmem));
  const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(p.n_tiles, (uint64_t)sm_count() * 4));
  kern<<<grid, kUBlock, kUmmaSmem, stream>>>(p);
  return launch_status();
}

}  // namespace

int launch(const double* op, const void* in, void* out, uint64_t X, uint64_t Y, uint64_t Z, unsigned* status,
           cudaStream_t stream) {
  TcParams p;
  std::memset(&p, 0, sizeof p);
  for (int r = 0; r < 16; ++r) {
    split_row(op + 16 * r, p.digits, r, p.row_exp);
    for (int k = 0; k < 16; ++k) p.ptm[r][k] = op[16 * r + k];
  }
  // the same digits in the operand layout: element (row r, column k) of plane
  // i at byte core_off(r, k)
  for (int i = 0; i < kDigits; ++i)
    for (int r = 0; r < 16; ++r)
      for (int k = 0; k < 16; ++k) p.bplanes[i][core_off(r, k) / 2] = p.digits[i][r][k];
  set_geometry(p, in, out, X, Y, Z, status);
  static const bool mma_sync = [] {
    const char* v = std::getenv("QSGB_TC_KERNEL");
    return v && std::strcmp(v, "mma_sync") == 0;
  }();
  if (mma_sync) {
    // warp-level form: tiles of 8 groups per warp
    const bool contig = Z % 8 == 0;
    p.pair_store = contig && (uintptr_t)out % 16 == 0 ? 1 : 0;
    const uint64_t blocks = (p.n_tiles + kBlock / 32 - 1) / (kBlock / 32);
    const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(blocks, (uint64_t)sm_count() * 8));
    if (contig)
      apply16_tc_kernel<true><<<grid, kBlock, 0, stream>>>(p);
    else
      apply16_tc_kernel<false><<<grid, kBlock, 0, stream>>>(p);
    return launch_status();
  }
  return launch_umma<false>(p, in, out, Z, stream);
}

int launch_device(const double* dptm, int layout, const void* in, void* out, uint64_t X, uint64_t Y, uint64_t Z,
                  unsigned* status, cudaStream_t stream) {
  TcParams p;
  std::memset(&p, 0, sizeof p);
  p.dptm = dptm;
  p.dlayout = layout & 3;
  set_geometry(p, in, out, X, Y, Z, status);
  return launch_umma<true>(p, in, out, Z, stream);
}

}  // namespace tc
}  // namespace qsgb

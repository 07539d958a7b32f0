// Batched forward + adjoint of many independent circuits in one persistent
// launch (FP32 Pauli vectors, FP64 reductions).
//
// Work model: a program is a sequence of stages; each stage holds work items
// (one op of one instance on a range of groups or elements).  Items of a
// stage belong to independent instances, so persistent blocks take them from
// the stage's atomic counter in any order; a grid barrier separates stages.
// Small instances finish in one item, large ones are split into tiles, so a
// few hundred blocks keep busy across instances of 4..16 qubits.
//
// Adjoint without stored intermediates: an op's input state is rebuilt from
// its output with the inverse PTM (rotations, controlled phases and damping
// are invertible and well conditioned), while the adjoint state moves back
// through P^T; the host refreshes the state from checkpoints every few
// layers.  One ADJOINT item therefore reads x_out and g_out once, writes x_in
// and g_in, and accumulates its share of dL/dP = sum g_out (x) x_in.  The
// two-qubit ADJOINT does its three small products per 32-group warp tile on
// the warp-level tensor cores (mma.sync m16n8k8, TF32 operands split hi/lo);
// every other body runs on the FP32 pipes.  An op here is whatever the host
// planned as a unit (a CZ may carry the rotations before it).
//
// Every grid barrier polls a bounded number of times; on expiry the kernel
// flags QSGB_DEV_TIMEOUT and all blocks return.
#include <cooperative_groups.h>

#include <algorithm>

#include "qsgb_common.cuh"

namespace qsgb {
namespace {

constexpr int kBatchBlock = 256;
constexpr int kRedRows = kBatchBlock / 16;  // rows of the FP64 dP reduction buffer (>= warps)
// floats per row of a warp's 16 x 32 adjoint tiles: 32 groups + 8 of
// padding, so that the fragment loads and 8-byte stores of the two-qubit
// ADJOINT fall in distinct banks
constexpr int kAdjStride = 40;
constexpr int kWarps = kBatchBlock / 32;

struct BatchSmem {
  float P[256];
  float PT[256];  // P transposed (ADJOINT: g_in = P^T g_out)
  float Pi[256];
  // two-qubit ADJOINT tiles, one pair per warp: x (X_out, then X_in) and g
  // (G_out, then G_in), 16 rows of kAdjStride floats; reused for the FP64
  // cross-warp sums of the dP partials
  union {
    struct {
      float g[kWarps][16 * kAdjStride];
      float x[kWarps][16 * kAdjStride];
    } t;
    double red[kRedRows][256];
  } u __attribute__((aligned(16)));
  double acc[kBatchBlock][16];  // per-thread FP64 dP partials (ADJOINT)
  int item;
  int ok;
  double lsum[kBatchBlock / 32];
};

}  // namespace

// The block's dynamic shared memory, at namespace scope so that the op
// bodies (separate functions) address it as shared memory.
extern __shared__ __align__(16) unsigned char batch_dsm[];

namespace {

__device__ __forceinline__ BatchSmem& smem() { return *reinterpret_cast<BatchSmem*>(batch_dsm); }

__device__ __forceinline__ volatile uint32_t* vol(uint32_t* p) { return p; }

// Grid barrier (sense by generation).  Returns false when the wait expired
// or another block aborted.
__device__ bool grid_barrier(uint32_t* count, uint32_t* gen, uint32_t* abort_flag, long long limit,
                             unsigned* status, BatchSmem& sm) {
  __syncthreads();
  if (threadIdx.x == 0) {
    sm.ok = 1;
    const uint32_t g0 = *vol(gen);
    __threadfence();
    if (atomicAdd(count, 1u) == gridDim.x - 1) {
      atomicExch(count, 0u);
      __threadfence();
      atomicAdd(gen, 1u);
    } else {
      long long it = 0;
      while (*vol(gen) == g0) {
        if (*vol(abort_flag) || ++it > limit) {
          sm.ok = 0;
          if (it > limit && status) atomicOr(status, QSGB_DEV_TIMEOUT);
          atomicExch(abort_flag, 1u);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return sm.ok != 0;
}

// ---------------------------------------------------------------- geometry
struct Geo {
  int k;          // 4 or 16 inputs per group
  int lz, ly;     // log2 of Z and Y (powers of 4)
};

__device__ __forceinline__ Geo geometry(int n, int q0, int q1) {
  Geo g;
  if (q1 < 0) {
    g.k = 4;
    g.lz = 2 * (n - 1 - q0);
    g.ly = 0;
  } else {
    g.k = 16;
    g.lz = 2 * (n - 1 - q1);
    g.ly = 2 * (q1 - q0 - 1);
  }
  return g;
}

// base element of group `gi` and offset of input k
__device__ __forceinline__ int64_t group_base(const Geo& g, int64_t gi) {
  const int64_t z = gi & ((1ll << g.lz) - 1);
  const int64_t t = gi >> g.lz;
  if (g.k == 4) return ((t << (g.lz + 2)) | z);
  const int64_t y = t & ((1ll << g.ly) - 1);
  const int64_t x = t >> g.ly;
  return (x << (g.lz + g.ly + 4)) + (y << (g.lz + 2)) + z;
}

// (32-bit: instances have at most 15 qubits, so an offset inside a group
// stays below 3 * 4^14; fewer registers than 64-bit addresses per input)
template <int K>
__device__ __forceinline__ int in_offset(const Geo& g, int k) {
  if (K == 4) return k << g.lz;
  return ((k >> 2) << (g.lz + g.ly + 2)) + ((k & 3) << g.lz);
}

// ---------------------------------------------------------------- items
// Vectorised in-place apply.  Z >= 4: a thread takes V consecutive groups
// (z .. z+V-1, 16- or 8-byte accesses per input); Z == 1: the K inputs of a
// group along the less significant qubit are contiguous (16-byte accesses).
// The per-op bodies are not inlined into the kernel: each gets its own
// register allocation under the kernel's 128-register cap, so one op's
// pressure does not spill into the others.
template <int K>
__device__ __noinline__ void apply_vec(float* __restrict__ x, const Geo& geo, int64_t beg, int64_t end, const float* P) {
  if (geo.lz >= 2) {
    constexpr int V = 4;
    for (int64_t gi = beg + (int64_t)threadIdx.x * V; gi < end; gi += (int64_t)blockDim.x * V) {
      const int64_t b = group_base(geo, gi);
      float v[K][V];
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const float* src = x + b + in_offset<K>(geo, k);
        if (V == 4) {
          const float4 t = *reinterpret_cast<const float4*>(src);
          v[k][0] = t.x; v[k][1] = t.y; v[k][2 % V] = t.z; v[k][3 % V] = t.w;
        } else {
          const float2 t = *reinterpret_cast<const float2*>(src);
          v[k][0] = t.x; v[k][1] = t.y;
        }
      }
#pragma unroll 1
      for (int r = 0; r < K; ++r) {
        float y[V];
#pragma unroll
        for (int l = 0; l < V; ++l) y[l] = 0.f;
#pragma unroll
        for (int k = 0; k < K; ++k) {
          const float pk = P[r * K + k];
#pragma unroll
          for (int l = 0; l < V; ++l) y[l] = fmaf(pk, v[k][l], y[l]);
        }
        float* dst = x + b + in_offset<K>(geo, r);
        if (V == 4)
          *reinterpret_cast<float4*>(dst) = make_float4(y[0], y[1], y[2 % V], y[3 % V]);
        else
          *reinterpret_cast<float2*>(dst) = make_float2(y[0], y[1]);
      }
    }
  } else {
    for (int64_t gi = beg + threadIdx.x; gi < end; gi += blockDim.x) {
      const int64_t b = group_base(geo, gi);
      float v[K], y[K];
#pragma unroll
      for (int k = 0; k < K; k += 4) {
        const float4 t = *reinterpret_cast<const float4*>(x + b + in_offset<K>(geo, k));
        v[k] = t.x; v[k + 1] = t.y; v[k + 2] = t.z; v[k + 3] = t.w;
      }
#pragma unroll
      for (int r = 0; r < K; ++r) {
        float a = 0.f;
#pragma unroll
        for (int k = 0; k < K; ++k) a = fmaf(P[r * K + k], v[k], a);
        y[r] = a;
      }
#pragma unroll
      for (int k = 0; k < K; k += 4)
        *reinterpret_cast<float4*>(x + b + in_offset<K>(geo, k)) = make_float4(y[k], y[k + 1], y[k + 2], y[k + 3]);
    }
  }
}

// One-qubit adjoint (pairs of groups when Z >= 4, one contiguous group when
// Z == 1): x = P^-1 x, g = P^T g, and
// dP[r][k] = sum g_out[r] x_in[k] accumulated in FP32 registers, folded to
// FP64 every 16 groups, reduced over the block and written to dst (16
// doubles).
__device__ __noinline__ void adjoint1_vec(float* __restrict__ x, float* __restrict__ gv, const Geo& geo, int64_t beg,
                             int64_t end, const float* P, const float* Pi, BatchSmem& sm, double* __restrict__ dst) {
  float acc[16];
  double* accd = sm.acc[threadIdx.x];  // FP64 running sums live in shared memory
#pragma unroll
  for (int e = 0; e < 16; ++e) {
    acc[e] = 0.f;
    accd[e] = 0.0;
  }
  auto one = [&](const float* xo, const float* go, float* xi, float* gn) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      float a = 0.f, c = 0.f;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        a = fmaf(Pi[r * 4 + k], xo[k], a);
        c = fmaf(P[k * 4 + r], go[k], c);
      }
      xi[r] = a;
      gn[r] = c;
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int k = 0; k < 4; ++k) acc[r * 4 + k] = fmaf(go[r], xi[k], acc[r * 4 + k]);
  };
  int since = 0;
  if (geo.lz >= 2) {  // pairs of groups (z, z+1): 8-byte accesses
    for (int64_t gi = beg + (int64_t)threadIdx.x * 2; gi < end; gi += (int64_t)blockDim.x * 2) {
      const int64_t b = group_base(geo, gi);
      float xv[4][2], gvv[4][2];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float2 a = *reinterpret_cast<const float2*>(x + b + in_offset<4>(geo, k));
        const float2 c = *reinterpret_cast<const float2*>(gv + b + in_offset<4>(geo, k));
        xv[k][0] = a.x; xv[k][1] = a.y;
        gvv[k][0] = c.x; gvv[k][1] = c.y;
      }
      float xi[4][2], gn[4][2];
#pragma unroll
      for (int l = 0; l < 2; ++l) {
        const float xo[4] = {xv[0][l], xv[1][l], xv[2][l], xv[3][l]};
        const float go[4] = {gvv[0][l], gvv[1][l], gvv[2][l], gvv[3][l]};
        float a[4], c[4];
        one(xo, go, a, c);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          xi[r][l] = a[r];
          gn[r][l] = c[r];
        }
      }
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        *reinterpret_cast<float2*>(x + b + in_offset<4>(geo, r)) = make_float2(xi[r][0], xi[r][1]);
        *reinterpret_cast<float2*>(gv + b + in_offset<4>(geo, r)) = make_float2(gn[r][0], gn[r][1]);
      }
      if (++since == 8) {
#pragma unroll
        for (int e = 0; e < 16; ++e) {
          accd[e] += (double)acc[e];
          acc[e] = 0.f;
        }
        since = 0;
      }
    }
  } else {
    for (int64_t gi = beg + threadIdx.x; gi < end; gi += blockDim.x) {
      const int64_t b = group_base(geo, gi);
      const float4 a = *reinterpret_cast<const float4*>(x + b);
      const float4 c = *reinterpret_cast<const float4*>(gv + b);
      const float xo[4] = {a.x, a.y, a.z, a.w};
      const float go[4] = {c.x, c.y, c.z, c.w};
      float xi[4], gn[4];
      one(xo, go, xi, gn);
      *reinterpret_cast<float4*>(x + b) = make_float4(xi[0], xi[1], xi[2], xi[3]);
      *reinterpret_cast<float4*>(gv + b) = make_float4(gn[0], gn[1], gn[2], gn[3]);
      if (++since == 16) {
#pragma unroll
        for (int e = 0; e < 16; ++e) {
          accd[e] += (double)acc[e];
          acc[e] = 0.f;
        }
        since = 0;
      }
    }
  }
  // block reduction: warps by shuffle, then across warps in shared memory
  const int w = threadIdx.x >> 5;
#pragma unroll
  for (int e = 0; e < 16; ++e) {
    double v = accd[e] + (double)acc[e];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sm.u.red[w][e] = v;
  }
  __syncthreads();
  if (threadIdx.x < 16) {
    double s = 0.0;
    for (int ww = 0; ww < (int)(blockDim.x >> 5); ++ww) s += sm.u.red[ww][threadIdx.x];
    dst[threadIdx.x] = s;
  }
  __syncthreads();
}

// ---- warp-level tensor-core helpers (mma.sync m16n8k8, TF32 operands)
// The FP32 value x is carried as hi + lo, both TF32 (cvt.rna keeps the top
// 11 significant bits): hi = tf32(x), lo = tf32(x - hi).  A product is taken
// as A_lo B_hi + A_hi B_lo + A_hi B_hi (the lo * lo term is below the
// representation error of the split, ~2^-22 relative), accumulated in FP32.
__device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void split_tf32(float x, uint32_t& hi, uint32_t& lo) {
  hi = to_tf32(x);
  lo = to_tf32(x - __uint_as_float(hi));
}

// d += a * b for one m16n8k8 tile: a = 16 x 8 (row-major fragment a0..a3),
// b = 8 x 8 (column fragment b0, b1), d = 16 x 8 FP32
__device__ __forceinline__ void mma_tf32(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// d += A B with A given as split fragments (ah, al) and B as FP32 values
__device__ __forceinline__ void mma3(float (&d)[4], const uint32_t (&ah)[4], const uint32_t (&al)[4], float b0,
                                     float b1) {
  uint32_t bh0, bl0, bh1, bl1;
  split_tf32(b0, bh0, bl0);
  split_tf32(b1, bh1, bl1);
  mma_tf32(d, al, bh0, bh1);
  mma_tf32(d, ah, bl0, bl1);
  mma_tf32(d, ah, bh0, bh1);
}

// Two-qubit ADJOINT on the warp-level tensor cores.  A warp takes tiles of 32
// consecutive groups; lane l loads group t0 + l (coalesced across lanes) and
// stages its x_out and g_out as column l of two 16 x 32 tiles in its own
// slice of shared memory ([k][group], rows of kAdjStride floats).  Per tile:
//   X_in = P^-1 X_out and G_in = P^T G_out   (M 16, N 32, K 16: 8 mma each)
//   dP  += G_out X_in^T                      (M 16, N 16, K 32: 8 mma)
// each mma in 3xTF32 (24 per product).  X_in and G_in go back through the
// tiles ([r][group]) to the lanes that own the groups and to global memory.
// The dP fragments are carried in FP32 over 4 tiles, then folded into the
// thread's FP64 sums in shared memory; at the end the warps' sums are added
// in a fixed order and written to dst (256 doubles).
__device__ __noinline__ void adjoint2_warp(float* __restrict__ x, float* __restrict__ gv, const Geo& geo, int64_t beg,
                                           int64_t end, double* __restrict__ dst) {
  constexpr int K = 16;
  constexpr int S = kAdjStride;
  BatchSmem& sm = smem();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  const int gid = lane >> 2, tig = lane & 3;
  float* ta = sm.u.t.x[warp];  // X_out, then X_in
  float* tb = sm.u.t.g[warp];  // G_out, then G_in
  const bool vec = geo.lz == 0;
  // A fragments of P^-1 and P^T (two k-steps each), split into TF32 hi / lo
  uint32_t pih[2][4], pil[2][4], pth[2][4], ptl[2][4];
#pragma unroll
  for (int ks = 0; ks < 2; ++ks) {
    const int c = 8 * ks + tig;
    const float vi[4] = {sm.Pi[gid * K + c], sm.Pi[(gid + 8) * K + c], sm.Pi[gid * K + c + 4],
                         sm.Pi[(gid + 8) * K + c + 4]};
    const float vt[4] = {sm.PT[gid * K + c], sm.PT[(gid + 8) * K + c], sm.PT[gid * K + c + 4],
                         sm.PT[(gid + 8) * K + c + 4]};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      split_tf32(vi[i], pih[ks][i], pil[ks][i]);
      split_tf32(vt[i], pth[ks][i], ptl[ks][i]);
    }
  }
  float dp[2][4];  // dP fragments: rows gid, gid + 8; columns 8 nb + 2 tig (+1)
#pragma unroll
  for (int nb = 0; nb < 2; ++nb)
#pragma unroll
    for (int i = 0; i < 4; ++i) dp[nb][i] = 0.f;
  double* acc = sm.acc[threadIdx.x];  // FP64 running sums in shared memory
#pragma unroll
  for (int i = 0; i < 8; ++i) acc[i] = 0.0;
  int tiles = 0;
  for (int64_t t0 = beg + (int64_t)warp * 32; t0 < end; t0 += (int64_t)nwarps * 32) {
    const int64_t gi = t0 + lane;
    const bool have = gi < end;
    const int64_t b = have ? group_base(geo, gi) : 0;
    {
      // this warp's next tile into L2 while the current one is loaded and
      // computed (the loads below are bound by their latency): lane l takes
      // tensor l / 16 and, for Z >= 64, component l % 16 at the tile's first
      // and last group (one 128-byte run each when the groups are
      // consecutive along z); for Z == 1, line l % 4 of chunk row
      // (l / 4) % 4 (the tile's 32 groups are 512 contiguous bytes per
      // row).  Other strides are not prefetched.  Addresses are those of
      // groups inside the item.
      const int64_t tn = t0 + (int64_t)nwarps * 32;
      if (tn < end) {
        const float* base = (lane < 16) ? x : gv;
        if (geo.lz >= 6) {
          const int off = in_offset<K>(geo, lane & 15);
          const int64_t last = tn + 31 < end ? tn + 31 : end - 1;
          asm volatile("prefetch.global.L2 [%0];" ::"l"(base + group_base(geo, tn) + off));
          asm volatile("prefetch.global.L2 [%0];" ::"l"(base + group_base(geo, last) + off));
        } else if (vec && tn + 31 < end) {
          const int64_t b0 = group_base(geo, tn), b1 = group_base(geo, tn + 31);
          if (b1 - b0 == 31 * 4) {  // the 32 groups share x: rows are contiguous
            const int q = (lane >> 2) & 3;
            asm volatile("prefetch.global.L2 [%0];" ::"l"(base + b0 + in_offset<K>(geo, 4 * q) + 32 * (lane & 3)));
          }
        }
      }
    }
    {
      float xo[K], go[K];
      if (!have) {
#pragma unroll
        for (int k = 0; k < K; ++k) xo[k] = go[k] = 0.f;
      } else if (vec) {
#pragma unroll
        for (int q = 0; q < K / 4; ++q) {
          const float4 u = *reinterpret_cast<const float4*>(x + b + in_offset<K>(geo, 4 * q));
          const float4 w = *reinterpret_cast<const float4*>(gv + b + in_offset<K>(geo, 4 * q));
          xo[4 * q] = u.x; xo[4 * q + 1] = u.y; xo[4 * q + 2] = u.z; xo[4 * q + 3] = u.w;
          go[4 * q] = w.x; go[4 * q + 1] = w.y; go[4 * q + 2] = w.z; go[4 * q + 3] = w.w;
        }
      } else {
#pragma unroll
        for (int k = 0; k < K; ++k) {
          xo[k] = x[b + in_offset<K>(geo, k)];
          go[k] = gv[b + in_offset<K>(geo, k)];
        }
      }
#pragma unroll
      for (int k = 0; k < K; ++k) {
        ta[k * S + lane] = xo[k];
        tb[k * S + lane] = go[k];
      }
    }
    __syncwarp();
    // X_in = P^-1 X_out, G_in = P^T G_out: four n-tiles of 8 groups
    float xi[4][4], gn[4][4];
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
#pragma unroll
      for (int i = 0; i < 4; ++i) xi[nt][i] = gn[nt][i] = 0.f;
#pragma unroll
      for (int ks = 0; ks < 2; ++ks) {
        const int r0 = (8 * ks + tig) * S + 8 * nt + gid;
        mma3(xi[nt], pih[ks], pil[ks], ta[r0], ta[r0 + 4 * S]);
        mma3(gn[nt], pth[ks], ptl[ks], tb[r0], tb[r0 + 4 * S]);
      }
    }
    // dP A fragments: G_out[r][group] for the four k-steps over groups
    float ga[4][4];
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
      const int c = 8 * ks + tig;
      ga[ks][0] = tb[gid * S + c];
      ga[ks][1] = tb[(gid + 8) * S + c];
      ga[ks][2] = tb[gid * S + c + 4];
      ga[ks][3] = tb[(gid + 8) * S + c + 4];
    }
    __syncwarp();
    // X_in and G_in into the tiles as [r][group]
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
      const int c = 8 * nt + 2 * tig;
      *reinterpret_cast<float2*>(&ta[gid * S + c]) = make_float2(xi[nt][0], xi[nt][1]);
      *reinterpret_cast<float2*>(&ta[(gid + 8) * S + c]) = make_float2(xi[nt][2], xi[nt][3]);
      *reinterpret_cast<float2*>(&tb[gid * S + c]) = make_float2(gn[nt][0], gn[nt][1]);
      *reinterpret_cast<float2*>(&tb[(gid + 8) * S + c]) = make_float2(gn[nt][2], gn[nt][3]);
    }
    __syncwarp();
    // this lane's group back to global memory
    if (have) {
      if (vec) {
#pragma unroll
        for (int q = 0; q < K / 4; ++q) {
          *reinterpret_cast<float4*>(x + b + in_offset<K>(geo, 4 * q)) =
              make_float4(ta[(4 * q) * S + lane], ta[(4 * q + 1) * S + lane], ta[(4 * q + 2) * S + lane],
                          ta[(4 * q + 3) * S + lane]);
          *reinterpret_cast<float4*>(gv + b + in_offset<K>(geo, 4 * q)) =
              make_float4(tb[(4 * q) * S + lane], tb[(4 * q + 1) * S + lane], tb[(4 * q + 2) * S + lane],
                          tb[(4 * q + 3) * S + lane]);
        }
      } else {
#pragma unroll
        for (int r = 0; r < K; ++r) {
          x[b + in_offset<K>(geo, r)] = ta[r * S + lane];
          gv[b + in_offset<K>(geo, r)] = tb[r * S + lane];
        }
      }
    }
    // dP += G_out X_in^T: B[group][k] = X_in[k][group]
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
      uint32_t ah[4], al[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) split_tf32(ga[ks][i], ah[i], al[i]);
#pragma unroll
      for (int nb = 0; nb < 2; ++nb) {
        const int r0 = (8 * nb + gid) * S + 8 * ks + tig;
        mma3(dp[nb], ah, al, ta[r0], ta[r0 + 4]);
      }
    }
    __syncwarp();
    if ((++tiles & 3) == 0) {
#pragma unroll
      for (int nb = 0; nb < 2; ++nb)
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          acc[nb * 4 + i] += (double)dp[nb][i];
          dp[nb][i] = 0.f;
        }
    }
  }
#pragma unroll
  for (int nb = 0; nb < 2; ++nb)
#pragma unroll
    for (int i = 0; i < 4; ++i) acc[nb * 4 + i] += (double)dp[nb][i];
  __syncthreads();  // every warp is done with the tile: reuse it for the sums
#pragma unroll
  for (int nb = 0; nb < 2; ++nb)
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = gid + 8 * (i >> 1), k = 8 * nb + 2 * tig + (i & 1);
      sm.u.red[warp][r * 16 + k] = acc[nb * 4 + i];
    }
  __syncthreads();
  for (int e = threadIdx.x; e < K * K; e += blockDim.x) {
    double t = 0.0;
    for (int w = 0; w < nwarps; ++w) t += sm.u.red[w][e];
    dst[e] = t;
  }
  __syncthreads();
}

__device__ __noinline__ void loss_item(const qsgb_batch_program& p, const qsgb_batch_instance& in, int inst, BatchSmem& sm) {
  const int n = in.n_qubits;
  const int64_t D = 1ll << n;
  double part = 0.0;
  for (int64_t j = threadIdx.x; j < D; j += blockDim.x) {
    // element of the diagonal entry j: bit q of j (from the top) selects
    // Pauli element 0 (|0><0|) or 1 (|1><1|) of qubit q
    int64_t idx = 0;
    for (int q = 0; q < n; ++q) idx |= ((j >> (n - 1 - q)) & 1ll) << (2 * (n - 1 - q));
    const double pr = (double)in.x[idx];
    const double t = p.target[in.diag_offset + j];
    p.prob[in.diag_offset + j] = pr;
    const double pe = pr > 1e-300 ? pr : 1e-300;
    if (t > 0) {
      part += t * (log(t) - log(pe));
      in.g[idx] = (float)(-t / pe);
    } else {
      in.g[idx] = 0.f;
    }
  }
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0) sm.lsum[threadIdx.x >> 5] = part;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sm.lsum[w];
    p.loss[inst] = s;
  }
  __syncthreads();
}

// An item's fields against its instance: a known op, targets inside the
// instance (two distinct, ordered qubits for two-qubit ops), ranges inside
// the vector (in groups for APPLY / ADJOINT), a non-negative PTM or
// checkpoint index, an instance below the program's count.  Malformed items
// are skipped and reported as QSGB_DEV_BADITEM instead of being allowed to
// address memory they do not own.
__device__ __forceinline__ bool item_ok(const qsgb_batch_program& p, const qsgb_batch_item& it) {
  if (it.op < QSGB_BOP_INIT || it.op > QSGB_BOP_GRADSUM || it.inst < 0 || it.inst >= p.n_instances) return false;
  if (it.op == QSGB_BOP_GRADSUM) return it.beg >= 0 && it.end >= it.beg && it.ptm >= 0;
  const qsgb_batch_instance in = p.instances[it.inst];
  const int n = in.n_qubits;
  if (n < 1 || n > 15 || in.size != (1ll << (2 * n))) return false;
  if (it.op == QSGB_BOP_LOSS) return true;
  if (it.beg < 0 || it.ptm < 0) return false;
  if (it.op == QSGB_BOP_APPLY || it.op == QSGB_BOP_ADJOINT) {
    if (it.q0 < 0 || it.q0 >= n) return false;
    if (it.q1 >= 0 && (it.q1 <= it.q0 || it.q1 >= n)) return false;
    return it.end <= (in.size >> (it.q1 < 0 ? 2 : 4));
  }
  return it.end <= in.size && (it.beg & 3) == 0 && (it.end & 3) == 0;
}

__device__ void process(const qsgb_batch_program& p, const qsgb_batch_item& it, BatchSmem& sm) {
  const qsgb_batch_instance in = p.instances[it.inst];
  switch (it.op) {
    // element ranges start and end on multiples of 4 (item_ok): 16-byte accesses
    case QSGB_BOP_INIT:
      for (int64_t e = it.beg + 4 * (int64_t)threadIdx.x; e < it.end; e += 4 * (int64_t)blockDim.x)
        *reinterpret_cast<float4*>(in.x + e) = make_float4(e == 0 ? 1.f : 0.f, 0.f, 0.f, 0.f);
      break;
    case QSGB_BOP_ZERO_G:
      for (int64_t e = it.beg + 4 * (int64_t)threadIdx.x; e < it.end; e += 4 * (int64_t)blockDim.x)
        *reinterpret_cast<float4*>(in.g + e) = make_float4(0.f, 0.f, 0.f, 0.f);
      break;
    case QSGB_BOP_SAVE: {
      float* dst = in.ckpt + (int64_t)it.ptm * in.size;
      for (int64_t e = it.beg + 4 * (int64_t)threadIdx.x; e < it.end; e += 4 * (int64_t)blockDim.x)
        *reinterpret_cast<float4*>(dst + e) = *reinterpret_cast<const float4*>(in.x + e);
      break;
    }
    case QSGB_BOP_RESTORE: {
      const float* src = in.ckpt + (int64_t)it.ptm * in.size;
      for (int64_t e = it.beg + 4 * (int64_t)threadIdx.x; e < it.end; e += 4 * (int64_t)blockDim.x)
        *reinterpret_cast<float4*>(in.x + e) = *reinterpret_cast<const float4*>(src + e);
      break;
    }
    case QSGB_BOP_APPLY:
    case QSGB_BOP_ADJOINT: {
      const Geo geo = geometry(in.n_qubits, it.q0, it.q1);
      const int kk = geo.k * geo.k;
      for (int e = threadIdx.x; e < kk; e += blockDim.x) {
        const float v = p.ptm[(int64_t)it.ptm * 256 + e];
        sm.P[e] = v;
        if (it.op == QSGB_BOP_ADJOINT) {
          sm.PT[(e % geo.k) * geo.k + e / geo.k] = v;
          sm.Pi[e] = p.ptm_inv[(int64_t)it.ptm * 256 + e];
        }
      }
      __syncthreads();
      if (it.op == QSGB_BOP_APPLY) {
        if (geo.k == 4)
          apply_vec<4>(in.x, geo, it.beg, it.end, sm.P);
        else
          apply_vec<16>(in.x, geo, it.beg, it.end, sm.P);
      } else if (geo.k == 4) {
        adjoint1_vec(in.x, in.g, geo, it.beg, it.end, sm.P, sm.Pi, sm, p.grad_partial + (int64_t)it.slot * 256);
      } else {
        adjoint2_warp(in.x, in.g, geo, it.beg, it.end, p.grad_partial + (int64_t)it.slot * 256);
      }
      __syncthreads();
      break;
    }
    case QSGB_BOP_LOSS:
      loss_item(p, in, it.inst, sm);
      break;
    case QSGB_BOP_GRADSUM:
      for (int e = threadIdx.x; e < 256; e += blockDim.x) {
        double s = 0.0;
        for (int64_t sl = it.beg; sl < it.end; ++sl) s += p.grad_partial[sl * 256 + e];
        p.grad[(int64_t)it.ptm * 256 + e] = s;
      }
      break;
    default:
      if (threadIdx.x == 0 && p.work) atomicExch(&p.work[p.n_stages + 2], 1u);
      break;
  }
}

__global__ void __launch_bounds__(kBatchBlock, 2) batch_kernel(const __grid_constant__ qsgb_batch_program p,
                                                               unsigned* status, long long spin_limit) {
  extern __shared__ __align__(16) unsigned char dsm[];
  BatchSmem& sm = *reinterpret_cast<BatchSmem*>(dsm);
  uint32_t* bar_count = p.work + p.n_stages;
  uint32_t* bar_gen = p.work + p.n_stages + 1;
  uint32_t* abort_flag = p.work + p.n_stages + 2;
  for (int s = 0; s < p.n_stages; ++s) {
    const int beg = p.stage_begin[s], end = p.stage_begin[s + 1];
    while (true) {
      __syncthreads();
      if (threadIdx.x == 0) sm.item = beg + (int)atomicAdd(&p.work[s], 1u);
      __syncthreads();
      const int i = sm.item;
      if (i >= end) break;
      const qsgb_batch_item it = p.items[i];
      if (!item_ok(p, it)) {
        if (threadIdx.x == 0 && status) atomicOr(status, QSGB_DEV_BADITEM);
        continue;
      }
      process(p, it, sm);
    }
    if (s + 1 < p.n_stages && !grid_barrier(bar_count, bar_gen, abort_flag, spin_limit, status, sm)) return;
  }
}

}  // namespace
}  // namespace qsgb

static int batch_smem_setup() {
  const int bytes = (int)sizeof(qsgb::BatchSmem);
  if (cudaFuncSetAttribute(qsgb::batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  return bytes;
}

extern "C" int qsgb_batch_max_grid(int block) {
  if (block != qsgb::kBatchBlock) return 0;
  const int smem = batch_smem_setup();
  if (smem < 0) return 0;
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, qsgb::batch_kernel, block, smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return occ * qsgb::sm_count();
}

extern "C" int qsgb_batch_run(const qsgb_batch_program* prog, int grid, int block, int cooperative,
                              unsigned* dev_status, int64_t spin_limit, void* stream) {
  if (!prog || !prog->instances || !prog->items || !prog->stage_begin || !prog->work || !prog->ptm)
    return QSGB_ERR_INVALID;
  if (block != qsgb::kBatchBlock || grid < 1 || prog->n_stages < 1 || prog->n_instances < 1 || spin_limit < 1)
    return QSGB_ERR_INVALID;
  const int maxg = qsgb_batch_max_grid(block);
  if (maxg < 1) return QSGB_ERR_CUDA;
  if (grid > maxg) return QSGB_ERR_INVALID;  // every block must be resident for the barriers
  qsgb_batch_program p = *prog;
  long long lim = (long long)spin_limit;
  cudaStream_t s = qsgb::as_stream(stream);
  void* args[] = {(void*)&p, (void*)&dev_status, (void*)&lim};
  cudaError_t e;
  const size_t smem = sizeof(qsgb::BatchSmem);
  if (cooperative)
    e = cudaLaunchCooperativeKernel((const void*)qsgb::batch_kernel, dim3(grid), dim3(block), args, smem, s);
  else
    e = cudaLaunchKernel((const void*)qsgb::batch_kernel, dim3(grid), dim3(block), args, smem, s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return QSGB_ERR_CUDA;
  }
  return QSGB_OK;
}

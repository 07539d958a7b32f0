// Reverse-mode kernels for apply_ptm: the gradient with respect to the PTM,
//   dP[r, k] = sum over bystander groups g of g_out[g, r] * x_in[g, k],
// a tall-skinny (Kout x Kin) reduction over all groups.  (The gradient with
// respect to the state is apply_ptm with the transposed PTM, see
// qsgb_apply.cu.)  The reference has no differentiation; the operation is
// the adjoint of quantumsim/pauli_vectors/numpy.py:50-64.
//
// The reduction has Kout * Kin multiply-adds per group: 256 for a two-qubit
// PTM, ~16 per streamed element.  On GB300 the FP64 pipe issues ~0.6 T FMA/s,
// so native FP64 products cap the kernel near 0.3 TB/s; the products here run
// on the FP32 pipes in float-float ("df64") arithmetic instead:
//
// Stage 1: each block walks tiles of `tg` groups.  The tile's inputs and
// output-gradients are loaded (the next tile's into registers while the
// current one is computed), split into float pairs hi + lo (48 significant
// bits, qsgb_split_f64) and staged in shared memory group-major.  Each thread
// owns a 4 x 4 micro-tile of (r, k) entries and a slice of the tile's groups
// and accumulates exact products hi*hi + the cross terms in float-float
// (qsgb_df_fma: error ~2^-47 per product, relative).  At the end of the block
// the slices' float-float sums are added in a fixed order and rounded to
// one double per entry (integer operations, qsgb_df_to_double).
//
// A tile holding a non-zero value outside [2^-100, 2^40] (where products or
// their sums could leave the float range) is computed in native FP64 instead,
// from global memory, into FP64 accumulators in shared memory that join the
// block's sums at the end.  Products of in-range values below the float
// range (< 2^-126) lose their low bits: the absolute error per product stays
// below 2^-149.
//
// Stage 2 adds the per-block partials of each entry in a fixed order
// (deterministic).
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "qsgb_common.cuh"
#include "qsgb_tc.h"

namespace qsgb {
namespace {

constexpr int kGradBlock = 256;
constexpr int kLoads = 8;  // (Kin + Kout) * tg <= kLoads * kGradBlock
constexpr int kStage2Entries = 32;
constexpr int kStage2Slices = 32;

struct GradParams {
  const void* x;
  const void* g;
  int kin, kout, db_in, db_out;
  int kpi, kpo;    // float2 row lengths of the staged inputs / gradients
  int tg;          // groups per tile (a power of two dividing kGradBlock)
  int nmt_c, nmt;  // 4 x 4 micro-tiles along k, in total
  int slices;      // group slices of a tile (micro-tiles <= kGradBlock)
  uint64_t n_groups, n_tiles;
  FastDiv div_z, div_y;
  int64_t sxi, syi, sai, sbi;
  int64_t sxo, syo, sao, sbo;
  // shared-memory byte offsets
  int off_gb, off_offs, off_fb, off_red2, off_flag, smem;
};

unsigned grad_blocks(uint64_t n_groups, int tg) {
  const uint64_t tiles = (n_groups + tg - 1) / tg;
  return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(tiles, (uint64_t)sm_count() * 2));
}

// groups per tile: the largest power of two <= kGradBlock with
// rows * tg <= kLoads * kGradBlock
int grad_tile(int rows) {
  int tg = kGradBlock;
  while (tg > 1 && rows * tg > kLoads * kGradBlock) tg >>= 1;
  return tg;
}

__device__ __forceinline__ unsigned out_of_band(double v) {
  const unsigned h = (unsigned)__double2hiint(v);
  const unsigned e = (h >> 20) & 0x7ffu;
  const bool nz = ((h << 1) | (unsigned)__double2loint(v)) != 0u;
  return (nz && (e < 923u || e > 1063u)) ? 1u : 0u;  // 2^-100 <= |v| <= 2^40
}

__device__ __forceinline__ unsigned out_of_band(float v) {
  const unsigned b = __float_as_uint(v) & 0x7fffffffu;
  const unsigned e = b >> 23;
  return (b != 0u && (e < 27u || e > 167u)) ? 1u : 0u;
}

__device__ __forceinline__ float2 split_pair(double v) {
  float h, l;
  unsigned ignored = 0;
  qsgb_split_f64(v, h, l, ignored);
  return make_float2(h, l);
}

__device__ __forceinline__ float2 split_pair(float v) { return make_float2(v, 0.0f); }

// (s, c) += (s2, c2), float-float
__device__ __forceinline__ void df_add(float& s, float& c, float s2, float c2) {
  const float r = s + s2;
  const float bp = r - s;
  const float err = (s - (r - bp)) + (s2 - bp);
  s = r;
  c += err + c2;
}

template <typename T, int MPT>
__global__ void __launch_bounds__(kGradBlock) grad_stage1(const __grid_constant__ GradParams p,
                                                          double* __restrict__ part) {
  extern __shared__ __align__(16) unsigned char smem[];
  float2* sx = reinterpret_cast<float2*>(smem);  // [tg][kpi]
  float2* sg = sx + p.tg * p.kpi;                // [tg][kpo]
  int64_t* gb = reinterpret_cast<int64_t*>(smem + p.off_gb);      // [2][tg]: group bases (in, out), -1 idle
  int64_t* offs = reinterpret_cast<int64_t*>(smem + p.off_offs);  // [kin + kout] row offsets
  double* fb = reinterpret_cast<double*>(smem + p.off_fb);        // [kGradBlock][MPT][16] FP64 tiles
  int* fb_any = reinterpret_cast<int*>(smem + p.off_flag);
  const T* __restrict__ X = static_cast<const T*>(p.x);
  const T* __restrict__ G = static_cast<const T*>(p.g);
  const int t = threadIdx.x;
  const int R = p.kin + p.kout;

  // zero the staging area (padding rows stay zero) and the FP64 sums
  {
    float4* z = reinterpret_cast<float4*>(smem);
    for (int i = t; i < p.off_gb / 16; i += kGradBlock) z[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    double* f = fb;
    for (int i = t; i < kGradBlock * MPT * 16; i += kGradBlock) f[i] = 0.0;
  }
  for (int r = t; r < R; r += kGradBlock) {
    if (r < p.kin) {
      const int ka = r / p.db_in, kb = r - ka * p.db_in;
      offs[r] = ka * p.sai + kb * p.sbi;
    } else {
      const int rr = r - p.kin, ra = rr / p.db_out, rb = rr - ra * p.db_out;
      offs[r] = ra * p.sao + rb * p.sbo;
    }
  }
  if (t == 0) *fb_any = 0;
  __syncthreads();

  // loader role: group gg_ld of the tile, rows r0_ld + j * rstep
  const int gg_ld = t & (p.tg - 1);
  const int r0_ld = t / p.tg, rstep = kGradBlock / p.tg;
  T v[kLoads];
  int64_t bin = -1, bout = -1;
  auto fetch = [&](uint64_t tile) {
    const uint64_t g = tile * p.tg + gg_ld;
    const bool live = tile < p.n_tiles && g < p.n_groups;
    bin = bout = -1;
    if (live) {
      const uint64_t t1 = fdiv(g, p.div_z);
      const uint64_t z = g - t1 * p.div_z.d;
      const uint64_t x = fdiv(t1, p.div_y);
      const uint64_t y = t1 - x * p.div_y.d;
      bin = (int64_t)x * p.sxi + (int64_t)y * p.syi + (int64_t)z;
      bout = (int64_t)x * p.sxo + (int64_t)y * p.syo + (int64_t)z;
    }
#pragma unroll
    for (int j = 0; j < kLoads; ++j) {
      const int r = r0_ld + j * rstep;
      v[j] = (T)0;
      if (live && r < R) v[j] = r < p.kin ? X[bin + offs[r]] : G[bout + offs[r]];
    }
  };
  auto stage = [&]() -> unsigned {
    unsigned bad = 0;
#pragma unroll
    for (int j = 0; j < kLoads; ++j) {
      const int r = r0_ld + j * rstep;
      if (r < R) {
        bad |= out_of_band(v[j]);
        const float2 s = split_pair(v[j]);
        if (r < p.kin)
          sx[gg_ld * p.kpi + r] = s;
        else
          sg[gg_ld * p.kpo + (r - p.kin)] = s;
      }
    }
    if (r0_ld == 0) {
      gb[gg_ld] = bin;
      gb[p.tg + gg_ld] = bout;
    }
    return bad;
  };

  // compute role: micro-tiles and group slice
  int mt[MPT], r0[MPT], k0[MPT];
  bool act[MPT];
  int slice;
  if (MPT == 1) {
    mt[0] = t % p.nmt;
    slice = t / p.nmt;
    act[0] = slice < p.slices;
  } else {
    slice = 0;
#pragma unroll
    for (int m = 0; m < MPT; ++m) {
      mt[m] = t + m * kGradBlock;
      act[m] = mt[m] < p.nmt;
    }
  }
#pragma unroll
  for (int m = 0; m < MPT; ++m) {
    r0[m] = (mt[m] / p.nmt_c) * 4;
    k0[m] = (mt[m] % p.nmt_c) * 4;
  }
  float s[MPT][16], c[MPT][16];
#pragma unroll
  for (int m = 0; m < MPT; ++m)
#pragma unroll
    for (int q = 0; q < 16; ++q) s[m][q] = c[m][q] = 0.0f;

  fetch(blockIdx.x);
  for (uint64_t tile = blockIdx.x; tile < p.n_tiles; tile += gridDim.x) {
    __syncthreads();  // the previous tile is consumed
    const int bad = __syncthreads_or((int)stage());
    fetch(tile + gridDim.x);  // in flight while this tile is computed
    if (!bad) {
#pragma unroll
      for (int m = 0; m < MPT; ++m) {
        if (!act[m]) continue;
        for (int gg = slice; gg < p.tg; gg += p.slices) {
          const float4 a01 = *reinterpret_cast<const float4*>(sg + gg * p.kpo + r0[m]);
          const float4 a23 = *reinterpret_cast<const float4*>(sg + gg * p.kpo + r0[m] + 2);
          const float4 b01 = *reinterpret_cast<const float4*>(sx + gg * p.kpi + k0[m]);
          const float4 b23 = *reinterpret_cast<const float4*>(sx + gg * p.kpi + k0[m] + 2);
          const float ah[4] = {a01.x, a01.z, a23.x, a23.z}, al[4] = {a01.y, a01.w, a23.y, a23.w};
          const float bh[4] = {b01.x, b01.z, b23.x, b23.z}, bl[4] = {b01.y, b01.w, b23.y, b23.w};
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) qsgb_df_fma(s[m][4 * i + j], c[m][4 * i + j], ah[i], al[i], bh[j], bl[j]);
        }
      }
    } else {
      // a value outside the float-float band: this tile in native FP64
      if (t == 0) *fb_any = 1;
#pragma unroll 1
      for (int m = 0; m < MPT; ++m) {
        if (!act[m]) continue;
        double* acc = fb + ((int64_t)t * MPT + m) * 16;
#pragma unroll 1
        for (int gg = slice; gg < p.tg; gg += p.slices) {
          const int64_t bi = gb[gg], bo = gb[p.tg + gg];
          if (bi < 0) continue;
          double a[4], b[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            a[i] = r0[m] + i < p.kout ? (double)G[bo + offs[p.kin + r0[m] + i]] : 0.0;
            b[i] = k0[m] + i < p.kin ? (double)X[bi + offs[k0[m] + i]] : 0.0;
          }
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[4 * i + j] = fma(a[i], b[j], acc[4 * i + j]);
        }
      }
    }
  }

  // block sums: slices in a fixed order, one double per entry
  __syncthreads();
  float2* red = reinterpret_cast<float2*>(smem);  // [kGradBlock][MPT][16], over the staging area
#pragma unroll
  for (int m = 0; m < MPT; ++m)
#pragma unroll
    for (int q = 0; q < 16; ++q) red[((int64_t)t * MPT + m) * 16 + q] = make_float2(s[m][q], c[m][q]);
  __syncthreads();
  const bool any_fb = *fb_any != 0;
  const int E = p.kin * p.kout;
  const int EP = p.nmt * 16;  // padded entries
  float2* red2 = reinterpret_cast<float2*>(smem + p.off_red2);  // [chunks][EP] (MPT == 1)
  double* fb2 = reinterpret_cast<double*>(smem + p.off_red2 + kGradBlock * sizeof(float2));
  if constexpr (MPT == 1) {
    // level 1: entry qp, slice chunk ch (slices ch, ch + nch, ...); with
    // many slices (small PTMs) the chunks spread the sums over the block
    const int nch = EP < kGradBlock ? kGradBlock / EP : 1;
    for (int tq = t; tq < nch * EP; tq += kGradBlock) {
      const int qp = tq % EP, ch = tq / EP;
      const int mtq = qp >> 4, q = qp & 15;
      float S = 0.0f, C = 0.0f;
      double F = 0.0;
      for (int sl = ch; sl < p.slices; sl += nch) {
        const int64_t idx = ((int64_t)(sl * p.nmt + mtq)) * 16 + q;
        const float2 v2 = red[idx];
        df_add(S, C, v2.x, v2.y);
        if (any_fb) F += fb[idx];
      }
      if (nch > 1) {
        red2[ch * EP + qp] = make_float2(S, C);
        fb2[ch * EP + qp] = F;
      } else {
        const int r = (mtq / p.nmt_c) * 4 + (q >> 2), k = (mtq % p.nmt_c) * 4 + (q & 3);
        double d = qsgb_df_to_double(S, C);
        if (any_fb) d += F;
        if (r < p.kout && k < p.kin) part[(int64_t)blockIdx.x * E + r * p.kin + k] = d;
      }
    }
    if (nch > 1) {
      __syncthreads();
      // level 2: the chunks of entry qp in order
      for (int qp = t; qp < EP; qp += kGradBlock) {
        const int mtq = qp >> 4, q = qp & 15;
        float S = 0.0f, C = 0.0f;
        double F = 0.0;
        for (int ch = 0; ch < nch; ++ch) {
          const float2 v2 = red2[ch * EP + qp];
          df_add(S, C, v2.x, v2.y);
          if (any_fb) F += fb2[ch * EP + qp];
        }
        const int r = (mtq / p.nmt_c) * 4 + (q >> 2), k = (mtq % p.nmt_c) * 4 + (q & 3);
        double d = qsgb_df_to_double(S, C);
        if (any_fb) d += F;
        if (r < p.kout && k < p.kin) part[(int64_t)blockIdx.x * E + r * p.kin + k] = d;
      }
    }
  } else {
  for (int qp = t; qp < EP; qp += kGradBlock) {
    const int mtq = qp >> 4, q = qp & 15;
    const int r = (mtq / p.nmt_c) * 4 + (q >> 2), k = (mtq % p.nmt_c) * 4 + (q & 3);
    float S = 0.0f, C = 0.0f;
    double F = 0.0;
    {
      const int tt = mtq % kGradBlock, m = mtq / kGradBlock;
      const int64_t idx = ((int64_t)tt * MPT + m) * 16 + q;
      const float2 v2 = red[idx];
      S = v2.x;
      C = v2.y;
      if (any_fb) F = fb[idx];
    }
    double d = qsgb_df_to_double(S, C);
    if (any_fb) d += F;
    if (r < p.kout && k < p.kin) part[(int64_t)blockIdx.x * E + r * p.kin + k] = d;
  }
  }
}

// out[e] = sum over blocks b of part[b][e]: kStage2Entries entries x
// kStage2Slices block slices per thread block, slices added in order
__global__ void __launch_bounds__(kStage2Entries* kStage2Slices)
    grad_stage2(const double* __restrict__ part, int nblocks, int E, double* __restrict__ out) {
  __shared__ double red[kStage2Slices][kStage2Entries + 1];
  const int el = threadIdx.x % kStage2Entries, sl = threadIdx.x / kStage2Entries;
  const int e = blockIdx.x * kStage2Entries + el;
  double acc = 0.0;
  if (e < E) {
#pragma unroll 8
    for (int b = sl; b < nblocks; b += kStage2Slices) acc += part[(int64_t)b * E + e];
  }
  red[sl][el] = acc;
  __syncthreads();
  if (sl == 0 && e < E) {
    double s = 0.0;
    for (int i = 0; i < kStage2Slices; ++i) s += red[i][el];
    out[e] = s;
  }
}

// ---------------------------------------------------------------------------
// 16 x 16 gradients on FP64 vectors: the tensor cores
// ---------------------------------------------------------------------------
// The same reduction as a product over groups, dP = G^T X per chunk of 16
// groups, on mma.sync.m16n8k16 (FP16 operands, FP32 accumulators) with the
// error-free digit split of the apply kernel (qsgb_tc.h): within a chunk,
// row r of A = G^T is scaled by its largest exponent over the chunk's 16
// groups and column k of B = X by its own, each value written as a 57-bit
// fixed-point integer in six balanced base-1024 FP16 digits.  For every digit
// pair (i, j) with i + j <= 5 two MMAs (k = 0..7, 8..15) add into level
// i + j; levels 0..3 are exact FP32 integer sums (below 2^24).  The six levels
// of each entry are combined in int64, scaled by 2^(E_r + E_k - 2098) and
// added to FP64 accumulators in chunk order.  Error per chunk: about
// 2^-47.7 max_g |g_out[g, r]| max_g |x_in[g, k]| over the chunk's groups.
// A chunk holding inf or nan, or with a result outside the normal double
// range, is recomputed in native FP64 from global memory.
//
// A warp takes chunks; lane l = (h, i) = (l / 16, l % 16) loads group i of
// the chunk, rows r = 8h .. 8h+7 of g_out and k = 8h .. 8h+7 of x_in, and
// writes their digits into the warp's planes A[d][r][g] and B[d][k][g]
// (FP16).  The fragments then follow the m16n8k16 layouts: lane
// (gid, tig) = (l / 4, l % 4) reads A rows gid, gid + 8 at columns 2 tig and
// 2 tig + 8, B rows (k) nt * 8 + gid, and ends with entries
// (r, k) = (gid or gid + 8, nt * 8 + 2 tig + {0, 1}).
constexpr int kTcgBlock = 256;
constexpr int kTcgWarps = kTcgBlock / 32;
constexpr int kTcgPlane = 16 * 16;  // halves per digit plane

struct TcgWarpSmem {
  unsigned short a[tc::kDigits][kTcgPlane];  // digits of g_out: [r][g]
  unsigned short b[tc::kDigits][kTcgPlane];  // digits of x_in: [k][g]
  int er[16], ek[16];                        // chunk exponents of rows, columns
};
struct TcgSmem {
  TcgWarpSmem warp[kTcgWarps];
  int64_t oin[16], oout[16];  // row offsets of x_in and g_out
};

__device__ __forceinline__ unsigned ld_pair(const unsigned short* plane, int row, int col) {
  return *reinterpret_cast<const unsigned*>(plane + row * 16 + col);
}

__global__ void __launch_bounds__(kTcgBlock) grad16_tc_kernel(const __grid_constant__ GradParams p,
                                                              double* __restrict__ part) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  TcgSmem& sm = *reinterpret_cast<TcgSmem*>(smem);
  TcgWarpSmem& ws = sm.warp[w];
  const double* __restrict__ X = static_cast<const double*>(p.x);
  const double* __restrict__ G = static_cast<const double*>(p.g);
  const int h = lane >> 4, i = lane & 15;
  const int gid = lane >> 2, tig = lane & 3;
  if (threadIdx.x < 16) {
    const int k = threadIdx.x;
    const int ka = k / p.db_in, kb = k - ka * p.db_in;
    sm.oin[k] = ka * p.sai + kb * p.sbi;
    const int ra = k / p.db_out, rb = k - ra * p.db_out;
    sm.oout[k] = ra * p.sao + rb * p.sbo;
  }
  __syncthreads();
  auto bases = [&](uint64_t g, int64_t& bi, int64_t& bo) {
    const uint64_t t1 = fdiv(g, p.div_z);
    const uint64_t z = g - t1 * p.div_z.d;
    const uint64_t x = fdiv(t1, p.div_y);
    const uint64_t y = t1 - x * p.div_y.d;
    bi = (int64_t)x * p.sxi + (int64_t)y * p.syi + (int64_t)z;
    bo = (int64_t)x * p.sxo + (int64_t)y * p.syo + (int64_t)z;
  };
  double acc[2][4];
#pragma unroll
  for (int nt = 0; nt < 2; ++nt)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[nt][q] = 0.0;

  const uint64_t n_chunks = (p.n_groups + 15) / 16;
  const uint64_t wstride = (uint64_t)gridDim.x * kTcgWarps;
  for (uint64_t c = (uint64_t)blockIdx.x * kTcgWarps + w; c < n_chunks; c += wstride) {
    const uint64_t g = c * 16 + i;
    const bool live = g < p.n_groups;
    double gv[8], xv[8];
    if (live) {
      int64_t bi, bo;
      bases(g, bi, bo);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        gv[j] = G[bo + sm.oout[8 * h + j]];
        xv[j] = X[bi + sm.oin[8 * h + j]];
      }
    } else {
#pragma unroll
      for (int j = 0; j < 8; ++j) gv[j] = xv[j] = 0.0;
    }
    // chunk exponents of rows 8h+j (g_out) and columns 8h+j (x_in): maxima
    // over the 16 lanes of this half
    unsigned eg[8], ex[8], nonfinite = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const unsigned hg = (unsigned)__double2hiint(gv[j]), hx = (unsigned)__double2hiint(xv[j]);
      nonfinite |= (((hg >> 20) & 0x7ffu) == 0x7ffu || ((hx >> 20) & 0x7ffu) == 0x7ffu) ? 1u : 0u;
      eg[j] = tc::exp_eff(hg);
      ex[j] = tc::exp_eff(hx);
#pragma unroll
      for (int o = 1; o < 16; o <<= 1) {
        eg[j] = max(eg[j], __shfl_xor_sync(0xffffffffu, eg[j], o));
        ex[j] = max(ex[j], __shfl_xor_sync(0xffffffffu, ex[j], o));
      }
    }
    if (i == 0) {
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        ws.er[8 * h + j] = (int)eg[j];
        ws.ek[8 * h + j] = (int)ex[j];
      }
    }
    // digits: low half of each pair the g_out digit, high half the x_in one
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const unsigned long long ug =
          tc::fixed_biased((unsigned)__double2hiint(gv[j]), (unsigned)__double2loint(gv[j]), eg[j]);
      const unsigned long long ux =
          tc::fixed_biased((unsigned)__double2hiint(xv[j]), (unsigned)__double2loint(xv[j]), ex[j]);
#pragma unroll
      for (int d = 0; d < tc::kDigits; ++d) {
        const unsigned pr = tc::digit_pair(ug, ux, 10 * (tc::kDigits - 1 - d));
        ws.a[d][(8 * h + j) * 16 + i] = (unsigned short)(pr & 0xffffu);
        ws.b[d][(8 * h + j) * 16 + i] = (unsigned short)(pr >> 16);
      }
    }
    const bool chunk_bad = __any_sync(0xffffffffu, nonfinite != 0u);
    __syncwarp();
    long long v[2][4];
#pragma unroll
    for (int nt = 0; nt < 2; ++nt)
#pragma unroll
      for (int q = 0; q < 4; ++q) v[nt][q] = 0;
#pragma unroll
    for (int L = 0; L < tc::kDigits; ++L) {
      float dl[2][4];
#pragma unroll
      for (int nt = 0; nt < 2; ++nt)
#pragma unroll
        for (int q = 0; q < 4; ++q) dl[nt][q] = 0.f;
#pragma unroll
      for (int a = 0; a <= L; ++a) {
        const unsigned fa[4] = {ld_pair(ws.a[a], gid, 2 * tig), ld_pair(ws.a[a], gid + 8, 2 * tig),
                                ld_pair(ws.a[a], gid, 2 * tig + 8), ld_pair(ws.a[a], gid + 8, 2 * tig + 8)};
#pragma unroll
        for (int nt = 0; nt < 2; ++nt) {
          const unsigned fbv[2] = {ld_pair(ws.b[L - a], nt * 8 + gid, 2 * tig),
                                   ld_pair(ws.b[L - a], nt * 8 + gid, 2 * tig + 8)};
          tc::mma16816(dl[nt], fa, fbv);
        }
      }
#pragma unroll
      for (int nt = 0; nt < 2; ++nt)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const long long t = (long long)__float2int_rn(dl[nt][q]);
          v[nt][q] += L < 5 ? (t << (10 * (4 - L))) : (t >> 10);
        }
    }
    // scale and accumulate (in FP64 from global memory when the chunk or a
    // result is out of range)
    double y[2][4];
    unsigned bad = 0;
#pragma unroll
    for (int nt = 0; nt < 2; ++nt)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int r = gid + (q >= 2 ? 8 : 0), k = nt * 8 + 2 * tig + (q & 1);
        const int sc = (ws.er[r] - 1022) + (ws.ek[k] - 1022) - 54;
        const long long vv = v[nt][q];
        double d = 0.0;
        if (vv != 0) {
          d = __ll2double_rn(vv);
          const int hi = __double2hiint(d);
          const int e = ((hi >> 20) & 0x7ff) + sc;
          bad |= (e < 1 || e > 2046) ? 1u : 0u;
          d = __hiloint2double(hi + (sc << 20), __double2loint(d));
        }
        y[nt][q] = d;
      }
    if (chunk_bad || __any_sync(0xffffffffu, bad != 0u)) {
#pragma unroll
      for (int nt = 0; nt < 2; ++nt)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int r = gid + (q >= 2 ? 8 : 0), k = nt * 8 + 2 * tig + (q & 1);
          const int ka = k / p.db_in, kb = k - ka * p.db_in, ra = r / p.db_out, rb = r - ra * p.db_out;
          const int64_t ok = ka * p.sai + kb * p.sbi, orr = ra * p.sao + rb * p.sbo;
          double s2 = 0.0;
#pragma unroll 1
          for (int gg = 0; gg < 16; ++gg) {
            const uint64_t g2 = c * 16 + gg;
            if (g2 >= p.n_groups) break;
            int64_t bi, bo;
            bases(g2, bi, bo);
            s2 = fma(G[bo + orr], X[bi + ok], s2);
          }
          y[nt][q] = s2;
        }
    }
#pragma unroll
    for (int nt = 0; nt < 2; ++nt)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[nt][q] += y[nt][q];
    __syncwarp();  // the planes are rewritten by the next chunk
  }
  // block sums over the warps, in warp order
  __syncthreads();
  double* red = reinterpret_cast<double*>(smem);  // [warps][256], over the planes
#pragma unroll
  for (int nt = 0; nt < 2; ++nt)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int r = gid + (q >= 2 ? 8 : 0), k = nt * 8 + 2 * tig + (q & 1);
      red[w * 256 + r * 16 + k] = acc[nt][q];
    }
  __syncthreads();
  {
    const int e = threadIdx.x;  // 256 entries, 256 threads
    double s2 = 0.0;
    for (int ww = 0; ww < kTcgWarps; ++ww) s2 += red[ww * 256 + e];
    part[(int64_t)blockIdx.x * 256 + e] = s2;
  }
}

unsigned tcg_blocks(uint64_t n_groups) {
  const uint64_t chunks = (n_groups + 15) / 16;
  const uint64_t blocks = (chunks + kTcgWarps - 1) / kTcgWarps;
  return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(blocks, (uint64_t)sm_count() * 2));
}

// 16 x 16 FP64 gradients go to the tensor cores unless QSGB_TC_GRAD=0
bool tc_grad_enabled() {
  static const bool on = [] {
    const char* v = std::getenv("QSGB_TC_GRAD");
    return !(v && std::strcmp(v, "0") == 0);
  }();
  return on;
}

GradParams make_params(const void* x_in, const void* g_out, int64_t da_out, int64_t db_out, int64_t da_in,
                       int64_t db_in, int64_t X, int64_t Y, int64_t Z) {
  GradParams p{};
  p.x = x_in;
  p.g = g_out;
  const int kin = (int)(da_in * db_in), kout = (int)(da_out * db_out);
  p.kin = kin;
  p.kout = kout;
  p.db_in = (int)db_in;
  p.db_out = (int)db_out;
  const int pi = (kin + 3) / 4 * 4, po = (kout + 3) / 4 * 4;
  p.kpi = pi + 2;  // + 16 bytes: consecutive groups start 4 banks apart
  p.kpo = po + 2;
  p.tg = grad_tile(kin + kout);
  p.nmt_c = pi / 4;
  p.nmt = (pi / 4) * (po / 4);
  p.slices = p.nmt <= kGradBlock ? kGradBlock / p.nmt : 1;
  p.n_groups = (uint64_t)X * Y * Z;
  p.n_tiles = (p.n_groups + p.tg - 1) / p.tg;
  p.div_z = make_fastdiv((uint64_t)Z);
  p.div_y = make_fastdiv((uint64_t)Y);
  p.sbi = Z;
  p.syi = db_in * Z;
  p.sai = Y * db_in * Z;
  p.sxi = da_in * Y * db_in * Z;
  p.sbo = Z;
  p.syo = db_out * Z;
  p.sao = Y * db_out * Z;
  p.sxo = da_out * Y * db_out * Z;
  const int mpt = p.nmt <= kGradBlock ? 1 : 2;
  const size_t stagebytes = (size_t)p.tg * (p.kpi + p.kpo) * sizeof(float2);
  const size_t redbytes = (size_t)kGradBlock * mpt * 16 * sizeof(float2);
  size_t o = (std::max(stagebytes, redbytes) + 15) / 16 * 16;
  p.off_gb = (int)o;
  o += 2 * (size_t)p.tg * sizeof(int64_t);
  p.off_offs = (int)o;
  o += ((size_t)(kin + kout) * sizeof(int64_t) + 15) / 16 * 16;
  p.off_fb = (int)o;
  o += (size_t)kGradBlock * mpt * 16 * sizeof(double);
  p.off_red2 = (int)o;  // level-1 sums: kGradBlock float2 + kGradBlock double
  o += (size_t)kGradBlock * (sizeof(float2) + sizeof(double));
  p.off_flag = (int)o;
  o += 16;
  p.smem = (int)o;
  return p;
}

template <typename T, int MPT>
int launch_stage1(const GradParams& p, unsigned nb, double* part, cudaStream_t s) {
  auto kern = grad_stage1<T, MPT>;
  const int st = allow_dynamic_smem((const void*)kern, p.smem);
  if (st != QSGB_OK) return st;
  kern<<<nb, kGradBlock, p.smem, s>>>(p, part);
  return QSGB_OK;
}

int grad_common(const void* x_in, const void* g_out, double* dptm, int64_t da_out, int64_t db_out, int64_t da_in,
                int64_t db_in, int64_t X, int64_t Y, int64_t Z, int dtype, void* scratch, int64_t scratch_bytes,
                void* stream) {
  if (!x_in || !g_out || !dptm) return QSGB_ERR_INVALID;
  if (da_out < 1 || db_out < 1 || da_in < 1 || db_in < 1 || X < 1 || Y < 1 || Z < 1) return QSGB_ERR_INVALID;
  if (dtype != QSGB_F64 && dtype != QSGB_F32) return QSGB_ERR_INVALID;
  const int64_t kin = da_in * db_in, kout = da_out * db_out;
  // 4 x 4 micro-tiles: at most 2 per thread
  if (kin > 256 || kout > 256 || ((kin + 3) / 4) * ((kout + 3) / 4) > 2 * kGradBlock)
    return QSGB_ERR_UNSUPPORTED;
  const GradParams p = make_params(x_in, g_out, da_out, db_out, da_in, db_in, X, Y, Z);
  const unsigned nb = grad_blocks(p.n_groups, p.tg);
  const int E = (int)(kin * kout);
  if (!scratch || scratch_bytes < (int64_t)nb * E * (int64_t)sizeof(double)) return QSGB_ERR_SCRATCH;
  cudaStream_t s = as_stream(stream);
  double* part = static_cast<double*>(scratch);
  if (dtype == QSGB_F64 && kin == 16 && kout == 16 && tc_grad_enabled()) {
    const unsigned nbt = tcg_blocks(p.n_groups);  // <= nb: the scratch holds its partials
    const int smem_bytes = std::max((int)sizeof(TcgSmem), kTcgWarps * 256 * (int)sizeof(double));
    const int st = allow_dynamic_smem((const void*)grad16_tc_kernel, smem_bytes);
    if (st != QSGB_OK) return st;
    grad16_tc_kernel<<<nbt, kTcgBlock, smem_bytes, s>>>(p, part);
    grad_stage2<<<(E + kStage2Entries - 1) / kStage2Entries, kStage2Entries * kStage2Slices, 0, s>>>(part, (int)nbt,
                                                                                                     E, dptm);
    return launch_status();
  }
  const bool two = p.nmt > kGradBlock;
  int st;
  if (dtype == QSGB_F64)
    st = two ? launch_stage1<double, 2>(p, nb, part, s) : launch_stage1<double, 1>(p, nb, part, s);
  else
    st = two ? launch_stage1<float, 2>(p, nb, part, s) : launch_stage1<float, 1>(p, nb, part, s);
  if (st != QSGB_OK) return st;
  grad_stage2<<<(E + kStage2Entries - 1) / kStage2Entries, kStage2Entries * kStage2Slices, 0, s>>>(part, (int)nb, E,
                                                                                                   dptm);
  return launch_status();
}

}  // namespace
}  // namespace qsgb

extern "C" int64_t qsgb_ptm_grad_scratch_bytes(int64_t n_groups, int64_t k_out, int64_t k_in) {
  if (n_groups < 1 || k_out < 1 || k_in < 1) return 0;
  const int tg = qsgb::grad_tile((int)std::min<int64_t>(k_out + k_in, 1 << 20));
  return (int64_t)qsgb::grad_blocks((uint64_t)n_groups, tg) * k_out * k_in * (int64_t)sizeof(double);
}

extern "C" int qsgb_ptm_grad1(const void* x_in, const void* g_out, double* dptm, int64_t d_out, int64_t d_in,
                              int64_t dim_y, int64_t dim_z, int dtype, void* scratch, int64_t scratch_bytes,
                              void* stream) {
  return qsgb::grad_common(x_in, g_out, dptm, 1, d_out, 1, d_in, 1, dim_y, dim_z, dtype, scratch, scratch_bytes,
                           stream);
}

extern "C" int qsgb_ptm_grad2(const void* x_in, const void* g_out, double* dptm, int64_t d0_out, int64_t d1_out,
                              int64_t d0_in, int64_t d1_in, int64_t dim_x, int64_t dim_y, int64_t dim_z, int dtype,
                              void* scratch, int64_t scratch_bytes, void* stream) {
  return qsgb::grad_common(x_in, g_out, dptm, d0_out, d1_out, d0_in, d1_in, dim_x, dim_y, dim_z, dtype, scratch,
                           scratch_bytes, stream);
}

// PTM application kernels: one- and two-qudit Pauli transfer matrices on any
// qudit positions, FP64 or FP32 storage.
//
// Replaces quantumsim/pauli_vectors/primitives.cu:15-89 (two_qubit_general_ptm,
// one thread per output element, PTM row re-read from global memory per
// thread) as launched from quantumsim/pauli_vectors/cuda.py:151-277.
//
// Design:
//  * The state tensor is viewed as (X, Da, Y, Db, Z) with targets a < b; a
//    one-qudit PTM is the case X = Da = 1.  A "group" is one bystander index
//    (x, y, z); it owns Kin = Da_in*Db_in inputs and Kout outputs.  When Z is
//    even an "item" is the pair of groups (z, z+1) and every access is 16
//    bytes wide; otherwise an item is one group.
//  * Persistent blocks of 256 threads (8 warps).  Each block compacts the PTM
//    once into per-row term lists in shared memory, then walks tiles of
//    T = 32*IW items: the whole block copies a tile's Kin x T inputs into
//    shared memory with cp.async (double-buffered: tile i+1 streams in while
//    tile i is computed), and the 8 warps split the work as IW "item warps"
//    x RG = 8/IW "row groups": warp (iw, rg) computes the rows assigned to
//    row group rg (balanced by cost) for items iw*32 .. iw*32+31.  Shared
//    memory therefore scales with the tile, not with the thread count.
//  * Every access pattern is warp-uniform: all lanes of a warp walk the same
//    row and term lists, term data are shared-memory broadcasts, and input
//    reads are consecutive 8/16-byte words (conflict free).
//  * FP64 storage, per-row arithmetic.  GB300 issues ~1.9 FP64 FMAs per SM
//    clock, about 1.4 per streamed element at full HBM bandwidth, against
//    ~58x that on the FP32 pipes.  A row is computed either with native FP64
//    FMAs ("dp": exact IEEE products and sums) or in float-float on the FP32
//    pipes ("df", 48-bit significand).  QSGB_ARITH_F64 makes every row dp;
//    QSGB_ARITH_DF64 makes every row with >= 2 terms df; QSGB_ARITH_AUTO
//    (default) picks, per PTM, the split of rows that minimises the larger of
//    the DP-pipe, integer-pipe, FMA-pipe and HBM times (rows in ascending term
//    count go to dp first).
//  * Entries with |P| <= 2^-52 max|P| (the round-off residue of PTM
//    construction) are skipped except in QSGB_ARITH_F64 mode, which skips
//    exact zeros only.
#include <algorithm>

#include "qsgb_common.cuh"
#include "qsgb_jit.h"
#include "qsgb_tc.h"
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace qsgb {

namespace {

constexpr int kMaxK = 256;         // Kin, Kout limit
constexpr int kMaxEntries = 6561;  // Kout*Kin limit (two qutrits)
constexpr int kMaxInline = 256;    // host PTMs up to 16x16 travel in the launch
constexpr int kBlock = 256;
constexpr int kWarps = kBlock / 32;

enum RowMode { kZero = 0, kDP = 1, kDF = 2, kF32 = 3 };

struct __align__(16) Term {
  double p;  // dp / f32 rows: the value; df rows: (hi, lo) floats
  int k;
  int pad;
};

struct __align__(16) RowInfo {
  int beg, end, mode, pad;
};

struct ApplyParams {
  const void* in;
  void* out;
  const double* ptm;  // device PTM, or nullptr when ptm_inline is used
  int kin, kout;
  int da_in, db_in, da_out, db_out;
  int flags;
  int arith;
  int max_terms;
  int iw;             // item warps per tile (tile = 32*iw items)
  uint64_t n_items;   // groups, or group pairs
  FastDiv div_z, div_y;  // Z (or Z/2 for pairs), Y
  int64_t sxi, syi, sai, sbi;  // input strides (z stride 1)
  int64_t sxo, syo, sao, sbo;  // output strides
  unsigned* status;
  double ptm_inline[kMaxInline];
};

// Offset of op element (r, k) in the stored PTM array.
__device__ __forceinline__ int ptm_index(const ApplyParams& p, int r, int k) {
  const int ra = r / p.db_out, rb = r - ra * p.db_out;
  const int ka = k / p.db_in, kb = k - ka * p.db_in;
  switch (p.flags & 3) {
    case 0:  // (ra, rb, ka, kb)
      return r * p.kin + k;
    case QSGB_PTM_SWAPPED:  // (rb, ra, kb, ka)
      return ((rb * p.da_out + ra) * p.db_in + kb) * p.da_in + ka;
    case QSGB_PTM_TRANSPOSED:  // forward (ka, kb, ra, rb)
      return k * p.kout + r;
    default:  // forward swapped (kb, ka, rb, ra)
      return ((kb * p.da_in + ka) * p.db_out + rb) * p.da_out + ra;
  }
}

struct SmemLayout {
  size_t xs_off, xs_bytes;  // region 0: max(PTM staging, 2 input tiles)
  size_t bo_off;            // int64[2][T] output offsets of the tile items
  size_t terms_off;         // Term[max_terms]
  size_t rows_off;          // RowInfo[kout]
  size_t rg_off;            // int[kWarps][kout] rows of each row group
  size_t rgn_off;           // int[kWarps] row counts
  size_t offin_off;         // int64[kin]
  size_t offout_off;        // int64[kout]
  size_t cnt_off;           // int[kout] term counts
  size_t srt_off;           // int[kout] term counts in ascending order
  size_t ord_off;           // int[kout] rows in descending weight order
  size_t red_off;           // double[36] reduction scratch, flag, plan values
  size_t total;
};

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

SmemLayout make_layout(int kin, int kout, int max_terms, int tile, size_t item_bytes) {
  SmemLayout L;
  const size_t xs = 2 * (size_t)kin * tile * item_bytes;
  const size_t stage = (size_t)kin * kout * sizeof(double);
  L.xs_off = 0;
  L.xs_bytes = std::max(xs, stage);
  size_t o = align_up(L.xs_bytes, 16);
  L.bo_off = o;
  o = align_up(o + 2 * (size_t)tile * sizeof(int64_t), 16);
  L.terms_off = o;
  o = align_up(o + (size_t)max_terms * sizeof(Term), 16);
  L.rows_off = o;
  o = align_up(o + (size_t)kout * sizeof(RowInfo), 16);
  L.rg_off = o;
  o = align_up(o + (size_t)kWarps * kout * sizeof(int), 16);
  L.rgn_off = o;
  o = align_up(o + (size_t)kWarps * sizeof(int), 16);
  L.offin_off = o;
  o = align_up(o + (size_t)kin * sizeof(int64_t), 16);
  L.offout_off = o;
  o = align_up(o + (size_t)kout * sizeof(int64_t), 16);
  L.cnt_off = o;
  o = align_up(o + (size_t)kout * sizeof(int), 16);
  L.srt_off = o;
  o = align_up(o + (size_t)kout * sizeof(int), 16);
  L.ord_off = o;
  o = align_up(o + (size_t)kout * sizeof(int), 16);
  L.red_off = o;
  o = align_up(o + 36 * sizeof(double), 16);
  L.total = o;
  return L;
}

// Cost model (SM clock cycles per group) of a row split, used by
// QSGB_ARITH_AUTO.  Rates per SM per clock on GB300: FP64 ~1.9 ops, the
// integer pipe 64 lanes, the FP32 FMA pipe 128 lanes, issue 128 lanes, HBM
// ~23 bytes.  A dp row of n terms costs n FP64 ops and ~2n+4 issue slots; a
// df row costs 12n FMA-pipe and 12n+25 integer ops (splits, rounding) and
// ~24n+30 issue slots.
struct SplitCost {
  float dp, alu, fma, issue, hbm;
  __device__ float time() const {
    float t = hbm;
    t = fmaxf(t, dp / 1.9f);
    t = fmaxf(t, alu / 64.f);
    t = fmaxf(t, fma / 128.f);
    t = fmaxf(t, issue / 128.f);
    return t;
  }
  __device__ void add_dp(int n, float sgn) {
    dp += sgn * n;
    issue += sgn * (2.f * n + 4.f);
  }
  __device__ void add_df(int n, float sgn) {
    fma += sgn * 12.f * n;
    alu += sgn * (12.f * n + 25.f);
    issue += sgn * (24.f * n + 30.f);
  }
};

// relative cost of a row, for balancing rows over warps
__device__ __forceinline__ int row_weight(int mode, int n) {
  return mode == kDF ? 24 * n + 30 : (mode == kZero ? 3 : 2 * n + 4);
}

// Per-thread asynchronous global->shared copies (no register staging).
template <int BYTES>
__device__ __forceinline__ void cp_async(void* smem_dst, const void* gsrc) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
  if constexpr (BYTES == 16) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gsrc) : "memory");
  } else {
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(s), "l"(gsrc), "n"(BYTES) : "memory");
  }
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

template <typename T, bool PAIR>
struct Vec;
template <>
struct Vec<double, false> {
  using type = double;
};
template <>
struct Vec<double, true> {
  using type = double2;
};
template <>
struct Vec<float, false> {
  using type = float;
};
template <>
struct Vec<float, true> {
  using type = float2;
};

__device__ __forceinline__ double lane_of(const double v, int) { return v; }
__device__ __forceinline__ double lane_of(const double2 v, int i) { return i ? v.y : v.x; }
__device__ __forceinline__ float lane_of(const float v, int) { return v; }
__device__ __forceinline__ float lane_of(const float2 v, int i) { return i ? v.y : v.x; }

__device__ __forceinline__ void put(double* o, const double* a) { *o = a[0]; }
__device__ __forceinline__ void put(double2* o, const double* a) { *o = make_double2(a[0], a[1]); }
__device__ __forceinline__ void put(float* o, const float* a) { *o = a[0]; }
__device__ __forceinline__ void put(float2* o, const float* a) { *o = make_float2(a[0], a[1]); }

// ---------------------------------------------------------------------------
// setup: PTM -> term lists, row modes, row groups (once per block)
// ---------------------------------------------------------------------------
template <typename T>
__device__ bool build_terms(const ApplyParams& p, const SmemLayout& L, unsigned char* smem) {
  double* stage = reinterpret_cast<double*>(smem + L.xs_off);
  Term* terms = reinterpret_cast<Term*>(smem + L.terms_off);
  RowInfo* rows = reinterpret_cast<RowInfo*>(smem + L.rows_off);
  int* rg_rows = reinterpret_cast<int*>(smem + L.rg_off);
  int* rg_n = reinterpret_cast<int*>(smem + L.rgn_off);
  int64_t* offin = reinterpret_cast<int64_t*>(smem + L.offin_off);
  int64_t* offout = reinterpret_cast<int64_t*>(smem + L.offout_off);
  int* cnt = reinterpret_cast<int*>(smem + L.cnt_off);
  double* red = reinterpret_cast<double*>(smem + L.red_off);
  int* flag = reinterpret_cast<int*>(red + 33);
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int ne = p.kin * p.kout;
  const double* __restrict__ src = p.ptm ? p.ptm : p.ptm_inline;

  double amax = 0.0;
  for (int i = tid; i < ne; i += nthr) {
    const int r = i / p.kin, k = i - r * p.kin;
    const double v = src[ptm_index(p, r, k)];
    stage[i] = v;
    amax = fmax(amax, fabs(v));
  }
  for (int o = 16; o > 0; o >>= 1) amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
  if ((tid & 31) == 0) red[tid >> 5] = amax;
  for (int k = tid; k < p.kin; k += nthr) {
    const int ka = k / p.db_in, kb = k - ka * p.db_in;
    offin[k] = ka * p.sai + kb * p.sbi;
  }
  for (int r = tid; r < p.kout; r += nthr) {
    const int ra = r / p.db_out, rb = r - ra * p.db_out;
    offout[r] = ra * p.sao + rb * p.sbo;
  }
  __syncthreads();
  if (tid == 0) {
    double m = 0.0;
    for (int w = 0; w < (nthr + 31) / 32; ++w) m = fmax(m, red[w]);
    red[32] = m;
  }
  __syncthreads();
  const double thr =
      (p.arith == QSGB_ARITH_F64) ? 0.0 : red[32] * ((p.arith == QSGB_ARITH_F32) ? 0x1p-30 : 0x1p-52);
  // float-float rows carry PTM entries as float pairs: a PTM whose largest
  // entry is outside [2^-100, 2^100] is computed in native FP64 throughout
  const bool all_dp = p.arith != QSGB_ARITH_F32 && !(red[32] >= 0x1p-100 && red[32] <= 0x1p100);
  for (int r = tid; r < p.kout; r += nthr) {
    int c = 0;
    for (int k = 0; k < p.kin; ++k) c += fabs(stage[r * p.kin + k]) > thr;
    cnt[r] = c;
  }
  __syncthreads();
  // The row plan, computed by all threads (every block repeats it for a
  // device PTM, so it must cost little): term counts in ascending order, the
  // dp / df split (AUTO), each row's mode and term offset, then rows in
  // descending weight order and their longest-first assignment to the row
  // groups.  Ties are broken by row index throughout, as a sequential pass
  // would.
  int* srt = reinterpret_cast<int*>(smem + L.srt_off);  // counts, ascending
  int* ord = reinterpret_cast<int*>(smem + L.ord_off);  // rows, weight descending
  int* ctl = reinterpret_cast<int*>(red + 34);          // cut, ties
  for (int r = tid; r < p.kout; r += nthr) {
    const int c = cnt[r];
    int rank = 0;
    for (int q = 0; q < p.kout; ++q) {
      const int cq = cnt[q];
      rank += (cq < c || (cq == c && q < r)) ? 1 : 0;
    }
    srt[rank] = c;
  }
  __syncthreads();
  if (tid == 0) {
    int cut = 1 << 30, ties = 0;
    if (p.arith == QSGB_ARITH_AUTO) {
      // n_dp = number of rows (ascending count) computed in FP64; rows with
      // one term are always dp.  Evaluate every n_dp incrementally.
      SplitCost sc{0.f, 0.f, 0.f, 5.f * (p.kin + p.kout), (float)(p.kin + p.kout) * (float)sizeof(T) / 23.f};
      for (int i = 0; i < p.kout; ++i) {
        const int v = srt[i];
        if (v == 1)
          sc.add_dp(1, 1.f);
        else if (v > 1)
          sc.add_df(v, 1.f);
      }
      float best = sc.time();
      int n_dp_best = 0;
      for (int i = 0; i < p.kout; ++i) {
        const int v = srt[i];
        if (v > 1) {
          sc.add_df(v, -1.f);
          sc.add_dp(v, 1.f);
        }
        const float c = sc.time();
        if (c < best * 0.999f) {
          best = c;
          n_dp_best = i + 1;
        }
      }
      cut = n_dp_best > 0 ? srt[n_dp_best - 1] : -1;
      for (int i = 0; i < n_dp_best; ++i) ties += srt[i] == cut;
    }
    ctl[0] = cut;
    ctl[1] = ties;
  }
  __syncthreads();
  {
    const int cut = ctl[0], ties = ctl[1];
    for (int r = tid; r < p.kout; r += nthr) {
      const int c = cnt[r];
      int beg = 0, tie_rank = 0;
      for (int q = 0; q < r; ++q) {
        const int cq = cnt[q];
        beg += cq;
        tie_rank += cq == cut ? 1 : 0;
      }
      int mode;
      if (c == 0)
        mode = kZero;
      else if (p.arith == QSGB_ARITH_F32)
        mode = kF32;
      else if (p.arith == QSGB_ARITH_F64 || c == 1 || all_dp)
        mode = kDP;
      else if (p.arith == QSGB_ARITH_DF64)
        mode = kDF;
      else if (c < cut)
        mode = kDP;
      else if (c == cut && tie_rank < ties)  // the first `ties` rows of count `cut`
        mode = kDP;
      else
        mode = kDF;
      rows[r].beg = beg;
      rows[r].end = beg + c;
      rows[r].mode = mode;
      rows[r].pad = 0;
      if (r == p.kout - 1) *flag = (beg + c > p.max_terms) ? 1 : 0;
    }
  }
  __syncthreads();
  for (int r = tid; r < p.kout; r += nthr) {
    const int w = row_weight(rows[r].mode, cnt[r]);
    int rank = 0;
    for (int q = 0; q < p.kout; ++q) {
      const int wq = row_weight(rows[q].mode, cnt[q]);
      rank += (wq > w || (wq == w && q < r)) ? 1 : 0;
    }
    ord[rank] = r;
  }
  __syncthreads();
  if (tid == 0) {
    // balance rows over the row groups (longest processing time first)
    const int rg_count = kWarps / p.iw;
    int load[kWarps], n[kWarps];
#pragma unroll
    for (int g = 0; g < kWarps; ++g) {
      load[g] = 0;
      n[g] = 0;
    }
    for (int step = 0; step < p.kout; ++step) {
      const int r = ord[step];
      const int w = row_weight(rows[r].mode, cnt[r]);
      int g = 0, lg = load[0];
#pragma unroll
      for (int h = 1; h < kWarps; ++h)
        if (h < rg_count && load[h] < lg) {
          g = h;
          lg = load[h];
        }
#pragma unroll
      for (int h = 0; h < kWarps; ++h)
        if (h == g) {
          rg_rows[h * p.kout + n[h]] = r;
          load[h] += w;
          ++n[h];
        }
    }
#pragma unroll
    for (int g = 0; g < kWarps; ++g)
      if (g < rg_count) rg_n[g] = n[g];
  }
  __syncthreads();
  if (*flag) {
    if (tid == 0 && p.status) atomicOr(p.status, QSGB_DEV_BADITEM);
    return false;
  }
  for (int r = tid; r < p.kout; r += nthr) {
    const RowInfo ri = rows[r];
    int t = ri.beg;
    for (int k = 0; k < p.kin; ++k) {
      const double v = stage[r * p.kin + k];
      if (fabs(v) > thr) {
        Term tm;
        if (ri.mode == kDF) {
          const float h = __double2float_rn(v);
          const float l = __double2float_rn(v - (double)h);
          tm.p = __hiloint2double(__float_as_int(h), __float_as_int(l));  // (hi, lo) words
        } else if (ri.mode == kF32) {
          tm.p = __hiloint2double(0, __float_as_int(__double2float_rn(v)));
        } else {
          tm.p = v;
        }
        tm.k = k;
        tm.pad = 0;
        terms[t++] = tm;
      }
    }
  }
  __syncthreads();  // stage[] is reused for the input tiles
  return true;
}

// ---------------------------------------------------------------------------
// main kernel
// ---------------------------------------------------------------------------
template <typename T, bool PAIR>
__global__ void __launch_bounds__(kBlock) apply_ptm_kernel(const __grid_constant__ ApplyParams p,
                                                           const SmemLayout L) {
  using V = typename Vec<T, PAIR>::type;
  constexpr int NL = PAIR ? 2 : 1;
  extern __shared__ __align__(16) unsigned char smem[];
  if (!build_terms<T>(p, L, smem)) return;

  V* xs = reinterpret_cast<V*>(smem + L.xs_off);
  int64_t* bo_tile = reinterpret_cast<int64_t*>(smem + L.bo_off);
  const Term* terms = reinterpret_cast<const Term*>(smem + L.terms_off);
  const RowInfo* rows = reinterpret_cast<const RowInfo*>(smem + L.rows_off);
  const int* rg_rows = reinterpret_cast<const int*>(smem + L.rg_off);
  const int* rg_n = reinterpret_cast<const int*>(smem + L.rgn_off);
  const int64_t* offin = reinterpret_cast<const int64_t*>(smem + L.offin_off);
  const int64_t* offout = reinterpret_cast<const int64_t*>(smem + L.offout_off);

  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int tile = 32 * p.iw;
  const int buf_len = p.kin * tile;  // V elements per buffer
  const uint64_t n_tiles = (p.n_items + tile - 1) / tile;
  const V* __restrict__ in = static_cast<const V*>(p.in);
  V* __restrict__ out = static_cast<V*>(p.out);

  // loader role: thread -> (item of the tile, first input row)
  const int ld_item = tid % tile;
  const int ld_k0 = tid / tile;
  const int ld_kstep = kBlock / tile;
  // compute role: warp -> (item warp, row group)
  const int iw = warp % p.iw;
  const int rg = warp / p.iw;
  const int my_item = iw * 32 + lane;
  const int n_my_rows = rg_n[rg];
  const int* my_rows = rg_rows + rg * p.kout;

  auto load_tile = [&](uint64_t t, int b) {
    const uint64_t it = t * tile + ld_item;
    if (it < p.n_items) {
      const uint64_t t1 = fdiv(it, p.div_z);
      const uint64_t zi = it - t1 * p.div_z.d;
      const uint64_t x = fdiv(t1, p.div_y);
      const uint64_t y = t1 - x * p.div_y.d;
      // with pairs all strides are even: offsets are halved (V units)
      const int64_t bi = ((int64_t)x * p.sxi + (int64_t)y * p.syi) / NL + (int64_t)zi;
      if (ld_k0 == 0) bo_tile[b * tile + ld_item] = ((int64_t)x * p.sxo + (int64_t)y * p.syo) / NL + (int64_t)zi;
      V* dst = xs + b * buf_len + ld_item;
      for (int k = ld_k0; k < p.kin; k += ld_kstep)
        cp_async<(int)sizeof(V)>(dst + k * tile, in + bi + offin[k] / NL);
    }
  };

  uint64_t t = blockIdx.x;
  int b = 0;
  if (t < n_tiles) load_tile(t, 0);
  cp_async_commit();
  for (; t < n_tiles; t += gridDim.x) {
    const uint64_t tn = t + gridDim.x;
    if (tn < n_tiles) load_tile(tn, b ^ 1);
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();  // tile t is in shared memory

    const uint64_t item = t * tile + my_item;
    if (item < p.n_items) {
      const V* xb = xs + b * buf_len + my_item;
      const int64_t bo = bo_tile[b * tile + my_item];
      for (int j = 0; j < n_my_rows; ++j) {
        const int r = my_rows[j];
        const RowInfo ri = rows[r];
        V* dst = out + bo + offout[r] / NL;
        if constexpr (sizeof(T) == 4) {  // FP32 storage and arithmetic
          float acc[NL];
#pragma unroll
          for (int l = 0; l < NL; ++l) acc[l] = 0.f;
          for (int q = ri.beg; q < ri.end; ++q) {
            const Term tm = terms[q];
            const float pf = __int_as_float(__double2loint(tm.p));
            const V xv = xb[tm.k * tile];
#pragma unroll
            for (int l = 0; l < NL; ++l) acc[l] = fmaf(pf, lane_of(xv, l), acc[l]);
          }
          put(dst, acc);
        } else {
          double acc[NL];
#pragma unroll
          for (int l = 0; l < NL; ++l) acc[l] = 0.0;
          if (ri.mode == kDP) {
            for (int q = ri.beg; q < ri.end; ++q) {
              const Term tm = terms[q];
              const V xv = xb[tm.k * tile];
#pragma unroll
              for (int l = 0; l < NL; ++l) acc[l] = fma(tm.p, (double)lane_of(xv, l), acc[l]);
            }
          } else if (ri.mode == kDF) {
            float s[NL], c[NL];
            unsigned fb = 0;  // the row needs native FP64 (input or result range)
            {
              const Term tm = terms[ri.beg];
              const float ph = __int_as_float(__double2hiint(tm.p));
              const float pl = __int_as_float(__double2loint(tm.p));
              const V xv = xb[tm.k * tile];
#pragma unroll
              for (int l = 0; l < NL; ++l) {
                float xh, xl;
                split_f64((double)lane_of(xv, l), xh, xl, fb);
                df_mul(s[l], c[l], ph, pl, xh, xl);
              }
            }
            for (int q = ri.beg + 1; q < ri.end; ++q) {
              const Term tm = terms[q];
              const float ph = __int_as_float(__double2hiint(tm.p));
              const float pl = __int_as_float(__double2loint(tm.p));
              const V xv = xb[tm.k * tile];
#pragma unroll
              for (int l = 0; l < NL; ++l) {
                float xh, xl;
                split_f64((double)lane_of(xv, l), xh, xl, fb);
                df_fma(s[l], c[l], ph, pl, xh, xl);
              }
            }
#pragma unroll
            for (int l = 0; l < NL; ++l) {
              fb |= qsgb_df_suspect(s[l]);
              acc[l] = df_to_double(s[l], c[l]);
            }
            if (fb) {
              // outside the float-float range: the row again in native FP64
              // (the term is carried as hi + lo, 48 significant bits)
#pragma unroll
              for (int l = 0; l < NL; ++l) acc[l] = 0.0;
              for (int q = ri.beg; q < ri.end; ++q) {
                const Term tm = terms[q];
                const double cf = (double)__int_as_float(__double2hiint(tm.p)) +
                                  (double)__int_as_float(__double2loint(tm.p));
                const V xv = xb[tm.k * tile];
#pragma unroll
                for (int l = 0; l < NL; ++l) acc[l] = fma(cf, (double)lane_of(xv, l), acc[l]);
              }
            }
          }
          put(dst, acc);
        }
      }
    }
    __syncthreads();  // buffer b is free for the tile after next
    b ^= 1;
  }
  cp_async_wait<0>();
}

// ---------------------------------------------------------------------------
// small device PTMs, plain dense kernel
// ---------------------------------------------------------------------------
// For a PTM in device memory the generic kernel's per-block row plan and
// term lists (rebuilt by every block, the values being on the device) cost
// more than the arithmetic on small vectors: ~16 us per launch on a 4 MB
// FP32 vector, ~20 us for a 4 x 4 PTM on an 8 MB FP64 one.  Here each block
// stages the op matrix in the storage type and each thread computes whole
// groups: FP32 FMAs for FP32 storage (entries at or below 2^-30 of the
// largest skipped, the generic kernel's FP32 rule), native FP64 FMAs for
// FP64 storage (entries at or below 2^-52 of the largest skipped under
// 'auto', exact zeros under 'f64'; exact IEEE products and sums, so no
// range fallback is needed).  FP64 takes this path only for one-qubit PTMs
// on vectors small enough for the FP64 pipe (at most 2^23 FMAs, ~14 us).
constexpr int kDenseMaxK = 16;
constexpr int kDenseBlock = 256;
constexpr double kDenseMaxF64Fma = 8388608.0;  // 2^23

template <typename T, int KMAX>
__global__ void __launch_bounds__(kDenseBlock) apply_dense_kernel(const __grid_constant__ ApplyParams p) {
  __shared__ T P[KMAX * KMAX];
  __shared__ int64_t offin[kDenseMaxK], offout[kDenseMaxK];
  __shared__ double wmax[kDenseBlock / 32];
  const int t = threadIdx.x;
  const int ne = p.kin * p.kout;  // <= kDenseBlock
  double v = 0.0;
  if (t < ne) {
    const int r = t / p.kin, k = t - r * p.kin;
    v = p.ptm[ptm_index(p, r, k)];
  }
  double m = fabs(v);
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((t & 31) == 0) wmax[t >> 5] = m;
  if (t < p.kin) {
    const int ka = t / p.db_in, kb = t - ka * p.db_in;
    offin[t] = ka * p.sai + kb * p.sbi;
  }
  if (t < p.kout) {
    const int ra = t / p.db_out, rb = t - ra * p.db_out;
    offout[t] = ra * p.sao + rb * p.sbo;
  }
  __syncthreads();
  double amax = 0.0;
#pragma unroll
  for (int w = 0; w < kDenseBlock / 32; ++w) amax = fmax(amax, wmax[w]);
  const double thr = sizeof(T) == 4 ? amax * 0x1p-30 : (p.arith == QSGB_ARITH_F64 ? 0.0 : amax * 0x1p-52);
  if (t < ne) P[t] = fabs(v) > thr ? (T)v : (T)0;
  __syncthreads();
  const T* __restrict__ X = static_cast<const T*>(p.in);
  T* __restrict__ Y = static_cast<T*>(p.out);
  for (uint64_t g = (uint64_t)blockIdx.x * kDenseBlock + t; g < p.n_items; g += (uint64_t)gridDim.x * kDenseBlock) {
    const uint64_t t1 = fdiv(g, p.div_z);
    const uint64_t z = g - t1 * p.div_z.d;
    const uint64_t x = fdiv(t1, p.div_y);
    const uint64_t y = t1 - x * p.div_y.d;
    const int64_t bi = (int64_t)x * p.sxi + (int64_t)y * p.syi + (int64_t)z;
    const int64_t bo = (int64_t)x * p.sxo + (int64_t)y * p.syo + (int64_t)z;
    T in[KMAX];
#pragma unroll
    for (int k = 0; k < KMAX; ++k) in[k] = k < p.kin ? X[bi + offin[k]] : (T)0;
#pragma unroll 4
    for (int r = 0; r < p.kout; ++r) {
      T a = (T)0;
#pragma unroll
      for (int k = 0; k < KMAX; ++k)
        if (k < p.kin) a = fma(P[r * p.kin + k], in[k], a);
      Y[bo + offout[r]] = a;
    }
  }
}

// row groups = min(Kout, 4) rounded down to a power of two; the remaining
// warps of the 8 are item warps (tile = 32 * 8 / row groups items)
int pick_iw(int kout) {
  int rg = 1;
  while (rg * 2 <= std::min(kout, 4)) rg *= 2;
  return kWarps / rg;
}

template <typename T, bool PAIR>
int launch_apply(ApplyParams& p, cudaStream_t stream) {
  using V = typename Vec<T, PAIR>::type;
  auto kern = apply_ptm_kernel<T, PAIR>;
  // shrink the tile (more row groups) if shared memory is short
  int iw = p.iw;
  SmemLayout L = make_layout(p.kin, p.kout, p.max_terms, 32 * iw, sizeof(V));
  while (L.total > 227 * 1024 && iw > 1) {
    iw /= 2;
    L = make_layout(p.kin, p.kout, p.max_terms, 32 * iw, sizeof(V));
  }
  if (L.total > 227 * 1024) return QSGB_ERR_UNSUPPORTED;
  p.iw = iw;
  {
    const int st = allow_dynamic_smem((const void*)kern, (int)L.total);
    if (st != QSGB_OK) return st;
  }
  int occ = 0;
  QSGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kBlock, L.total));
  if (occ < 1) return QSGB_ERR_UNSUPPORTED;
  const uint64_t tiles = (p.n_items + 32 * iw - 1) / (32 * iw);
  const uint64_t cap = (uint64_t)sm_count() * occ;
  const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min(tiles, cap));
  kern<<<grid, kBlock, L.total, stream>>>(p, L);
  return launch_status();
}


// ---------------------------------------------------------------------------
// run-time specialised kernel (qsgb_jit.cu)
// ---------------------------------------------------------------------------
// Returns QSGB_ERR_UNSUPPORTED when the specialised path does not apply.
// prepare_only: compile (or fetch) the kernel, launch nothing.
// Op matrix M[r][k] (rows (ra, rb), columns (ka, kb), qudit a first) of a
// PTM stored in `layout` (QSGB_PTM_SWAPPED / QSGB_PTM_TRANSPOSED bits).
void op_matrix(const double* ptm, int da_out, int db_out, int da_in, int db_in, int layout, double* m) {
  const int kin = da_in * db_in, kout = da_out * db_out;
  for (int r = 0; r < kout; ++r)
    for (int k = 0; k < kin; ++k) {
      const int ra = r / db_out, rb = r % db_out, ka = k / db_in, kb = k % db_in;
      int idx;
      switch (layout & 3) {
        case 0: idx = r * kin + k; break;
        case QSGB_PTM_SWAPPED: idx = ((rb * da_out + ra) * db_in + kb) * da_in + ka; break;
        case QSGB_PTM_TRANSPOSED: idx = k * kout + r; break;
        default: idx = ((kb * da_in + ka) * db_out + rb) * da_out + ra; break;
      }
      m[r * kin + k] = ptm[idx];
    }
}

// Under QSGB_ARITH_AUTO, a 16 x 16 PTM goes to the tensor cores when its
// rows average more non-zero terms (above 2^-52 of the largest entry) than
// QSGB_TC_MIN_TERMS (default 8).  Measured on GB300 (14 qubits): the
// tensor-core kernel streams 3.35-3.46 TB/s whatever the density (2.77 when
// the less significant target is the last qubit); the specialised
// float-float kernels 4.0 TB/s at 6.12 terms per row, 2.46 at 11.25 and
// 1.39-1.65 when dense, which crosses 3.3 TB/s near 8 terms per row.
bool tc_wanted(const double* op) {
  static const double min_terms = [] {
    const char* v = std::getenv("QSGB_TC_MIN_TERMS");
    return v ? std::atof(v) : 8.0;
  }();
  double amax = 0.0;
  for (int i = 0; i < 256; ++i) amax = std::max(amax, std::fabs(op[i]));
  int n = 0;
  for (int i = 0; i < 256; ++i) n += std::fabs(op[i]) > amax * 0x1p-52 ? 1 : 0;
  return n > min_terms * 16.0;
}

// Under QSGB_ARITH_AUTO every 16 x 16 device PTM goes to the tensor cores
// (QSGB_TC_DEVICE=0: to the generic kernel instead).
bool tc_device_auto() {
  static const bool on = [] {
    const char* v = std::getenv("QSGB_TC_DEVICE");
    return !(v && std::strcmp(v, "0") == 0);
  }();
  return on;
}

// mode: kLaunch, kPrepare (compile and load, launch nothing) or kCompileOnly
// (generate and compile the source, no device needed; *src_out gets it).
enum { kLaunch = 0, kPrepare = 1, kCompileOnly = 2 };

int try_jit(const double* ptm_host, int64_t da_out, int64_t db_out, int64_t da_in, int64_t db_in, int64_t Z,
            int flags, int dtype, int arith, bool pair, ApplyParams& p, cudaStream_t stream,
            int mode = kLaunch, std::string* src_out = nullptr) {
  if (!(flags & QSGB_PTM_HOST) || (flags & QSGB_PTM_NOJIT) || !jit::available()) return QSGB_ERR_UNSUPPORTED;
  // Z == 1: the db inputs (outputs) of a group along the less significant
  // target are contiguous; move them with 2- or 4-wide vector accesses
  auto vwidth = [&](int64_t db, const void* ptr) {
    const size_t esz = dtype == QSGB_F64 ? 8 : 4;
    if (Z != 1) return 1;
    for (int w : {4, 2})
      if (db % w == 0 && (uintptr_t)ptr % (w * esz) == 0) return w;
    return 1;
  };
  jit::Spec spec;
  std::vector<double> coef;
  // groups of consecutive items are adjacent (item it starts at it * K) when
  // Z == 1 and either Y == 1 (two adjacent last qudits) or Da == 1 (one qudit)
  const bool contiguous = Z == 1 && (p.div_y.d == 1 || (da_in == 1 && da_out == 1)) &&
                          (uintptr_t)p.in % 16 == 0 && (uintptr_t)p.out % 16 == 0;
  const int vin = vwidth(db_in, p.in), vout = vwidth(db_out, p.out);
  // the cached kernel and term list of this geometry class and term mask
  // (the rule of jit::make_spec: entries above 2^-52 of the largest, 2^-30
  // for FP32, non-zero for native FP64 or a PTM outside [2^-100, 2^100])
  const int ne = (int)(da_in * db_in * da_out * db_out);
  jit::FastKey key;
  const bool keyed = ne <= 64 * 104;
  if (keyed) {
    double amax = 0.0;
    for (int i = 0; i < ne; ++i) amax = std::max(amax, std::fabs(ptm_host[i]));
    int eff = arith;
    if (arith != QSGB_ARITH_F32 && !(amax >= 0x1p-100 && amax <= 0x1p100)) eff = QSGB_ARITH_F64;
    const double thr = eff == QSGB_ARITH_F64 ? 0.0 : amax * (eff == QSGB_ARITH_F32 ? 0x1p-30 : 0x1p-52);
    const unsigned char hdr[16] = {(unsigned char)da_out, (unsigned char)db_out, (unsigned char)da_in,
                                   (unsigned char)db_in, (unsigned char)(flags & 3), (unsigned char)dtype,
                                   (unsigned char)eff, (unsigned char)pair, (unsigned char)(Z == 1),
                                   (unsigned char)contiguous, (unsigned char)vin, (unsigned char)vout,
                                   (unsigned char)(mode == kLaunch), 0, 0, 0};
    std::memcpy(key.hdr, hdr, sizeof hdr);
    key.nwords = (ne + 63) / 64;
    for (int w = 0; w < key.nwords; ++w) key.mask[w] = 0;
    for (int i = 0; i < ne; ++i)
      if (std::fabs(ptm_host[i]) > thr) key.mask[i >> 6] |= 1ull << (i & 63);
  }
  auto geometry = [&](bool pair_final) {
    const int NL = pair_final ? 2 : 1;
    jit::Geometry g;
    g.in = p.in;
    g.out = p.out;
    g.status = p.status;
    g.n_items = pair_final ? p.n_items : (pair ? p.n_items * 2 : p.n_items);
    g.div_z = pair_final ? p.div_z : (pair ? make_fastdiv((uint64_t)Z) : p.div_z);
    g.div_y = p.div_y;
    g.sxi = p.sxi / NL;
    g.syi = p.syi / NL;
    g.sai = p.sai / NL;
    g.sbi = p.sbi / NL;
    g.sxo = p.sxo / NL;
    g.syo = p.syo / NL;
    g.sao = p.sao / NL;
    g.sbo = p.sbo / NL;
    return g;
  };
  if (keyed && mode == kLaunch) {
    if (const jit::FastEntry* e = jit::fast_find(key))
      return jit::launch_entry(*e, geometry(e->spec.pair), ptm_host, stream);
  }
  if (!jit::make_spec(ptm_host, (int)da_out, (int)db_out, (int)da_in, (int)db_in, flags & 3, dtype, arith, pair,
                      Z == 1, contiguous, vin, vout, spec, coef))
    return QSGB_ERR_UNSUPPORTED;
  // Two groups per thread (16-byte accesses) pay off for one-qudit PTMs and
  // for two-qudit PTMs of up to 2.5 terms per row; denser two-qudit rows
  // run faster one group per thread.  Measured on GB300 (14 qubits, GB/s,
  // pair / single): noisy CZ 6335 / 6427; CZ after one rotation 2.19
  // terms/row 6274 / 5487, 3.12 terms/row 3810 / 5218; CZ between rotations
  // 4.38 terms/row 4534 / 5245, 6.12 terms/row 2629 / 3984; two rotations
  // on one qubit 5968 / 5042.
  if (pair && spec.kin > 4 && spec.n_coef() > 2.5 * spec.kout) {
    if (!jit::make_spec(ptm_host, (int)da_out, (int)db_out, (int)da_in, (int)db_in, flags & 3, dtype, arith, false,
                        Z == 1, contiguous, vin, vout, spec, coef))
      return QSGB_ERR_UNSUPPORTED;
  }
  if (mode == kPrepare) return jit::prepare(spec);
  if (mode == kCompileOnly) return jit::compile_only(spec, src_out);
  if (keyed) {
    if (const jit::FastEntry* e =
            jit::fast_insert(key, spec, flags & 3, (int)da_out, (int)db_out, (int)da_in, (int)db_in))
      return jit::launch_entry(*e, geometry(e->spec.pair), ptm_host, stream);
  }
  return jit::launch(spec, geometry(spec.pair), coef.data(), stream);
}

// mode kPrepare / kCompileOnly: validate, then compile the specialised
// kernel the call would launch (for tensors aligned as allocators give
// them), and launch nothing.
int apply_common(const void* in, void* out, const double* ptm, int64_t da_out, int64_t db_out, int64_t da_in,
                 int64_t db_in, int64_t X, int64_t Y, int64_t Z, int flags, int dtype, int arith,
                 int64_t max_terms, unsigned* status, void* stream, int mode = kLaunch,
                 std::string* src_out = nullptr) {
  if (!in || !out || !ptm) return QSGB_ERR_INVALID;
  if (in == out) return QSGB_ERR_INVALID;
  if (da_out < 1 || db_out < 1 || da_in < 1 || db_in < 1 || X < 1 || Y < 1 || Z < 1) return QSGB_ERR_INVALID;
  if (flags & ~(QSGB_PTM_SWAPPED | QSGB_PTM_TRANSPOSED | QSGB_PTM_HOST | QSGB_PTM_NOJIT)) return QSGB_ERR_INVALID;
  const int64_t kin = da_in * db_in, kout = da_out * db_out;
  if (kin > kMaxK || kout > kMaxK || kin * kout > kMaxEntries) return QSGB_ERR_UNSUPPORTED;
  if (max_terms < 1 || max_terms > kin * kout) max_terms = kin * kout;
  if (dtype != QSGB_F64 && dtype != QSGB_F32) return QSGB_ERR_INVALID;
  if (arith < QSGB_ARITH_AUTO || arith > QSGB_ARITH_TC) return QSGB_ERR_INVALID;
  if (arith == QSGB_ARITH_TC && dtype != QSGB_F64) return QSGB_ERR_INVALID;
  // dense 16 x 16 host PTMs on FP64 vectors: the tensor-core kernel
  const int tc_arith = arith;
  if (arith == QSGB_ARITH_TC) arith = QSGB_ARITH_AUTO;
  if (dtype == QSGB_F32 && arith == QSGB_ARITH_AUTO) arith = QSGB_ARITH_F32;
  if (dtype == QSGB_F32 && arith != QSGB_ARITH_F32) return QSGB_ERR_INVALID;
  if (dtype == QSGB_F64 && arith == QSGB_ARITH_F32) return QSGB_ERR_INVALID;

  ApplyParams p;
  p.in = in;
  p.out = out;
  p.ptm = ptm;
  p.kin = (int)kin;
  p.kout = (int)kout;
  p.da_in = (int)da_in;
  p.db_in = (int)db_in;
  p.da_out = (int)da_out;
  p.db_out = (int)db_out;
  p.flags = flags & 3;
  p.arith = arith;
  p.max_terms = (int)max_terms;
  p.iw = pick_iw((int)kout);
  p.sbi = Z;
  p.syi = db_in * Z;
  p.sai = Y * db_in * Z;
  p.sxi = da_in * Y * db_in * Z;
  p.sbo = Z;
  p.syo = db_out * Z;
  p.sao = Y * db_out * Z;
  p.sxo = da_out * Y * db_out * Z;
  p.status = status;
  const size_t esz = dtype == QSGB_F64 ? 8 : 4;
  const bool pair = (Z % 2 == 0) && ((uintptr_t)in % (2 * esz) == 0) && ((uintptr_t)out % (2 * esz) == 0);
  p.div_y = make_fastdiv((uint64_t)Y);
  p.div_z = make_fastdiv((uint64_t)(pair ? Z / 2 : Z));
  p.n_items = (uint64_t)X * Y * (pair ? Z / 2 : Z);
  cudaStream_t s = as_stream(stream);
  // 0. dense 16 x 16 PTMs (two full-basis qubits) on the tensor cores; a
  // device PTM's values are not read on the host, so every 16 x 16 device
  // PTM goes there under 'auto' (the generic kernel would run its 256 terms
  // per group in float-float or FP64)
  if (dtype == QSGB_F64 && da_in == 4 && db_in == 4 && da_out == 4 && db_out == 4) {
    if (flags & QSGB_PTM_HOST) {
      // density and finiteness do not depend on the storage layout: the op
      // matrix is formed only for a launch on the tensor cores
      if ((tc_arith == QSGB_ARITH_TC || (tc_arith == QSGB_ARITH_AUTO && tc_wanted(ptm))) &&
          tc::eligible(ptm, 16, 16)) {
        if (mode != kLaunch) return QSGB_ERR_UNSUPPORTED;  // precompiled: nothing to prepare
        double op[256];
        op_matrix(ptm, 4, 4, 4, 4, flags & 3, op);
        return tc::launch(op, in, out, (uint64_t)X, (uint64_t)Y, (uint64_t)Z, status, s);
      }
    } else if (tc_arith == QSGB_ARITH_TC || (tc_arith == QSGB_ARITH_AUTO && tc_device_auto())) {
      if (mode != kLaunch) return QSGB_ERR_UNSUPPORTED;
      return tc::launch_device(ptm, flags & 3, in, out, (uint64_t)X, (uint64_t)Y, (uint64_t)Z, status, s);
    }
  }
  // 1. kernel specialised to the PTM's sparsity pattern (host PTMs)
  const int js = try_jit(ptm, da_out, db_out, da_in, db_in, Z, flags, dtype, arith, pair, p, s, mode, src_out);
  if (js != QSGB_ERR_UNSUPPORTED || mode != kLaunch) return js;
  // 2a. small device PTMs, no term limit: the dense kernel (FP32 storage up
  // to 16 x 16; FP64 storage for one-qubit PTMs on small vectors)
  if (!(flags & QSGB_PTM_HOST) && p.max_terms == kin * kout) {
    const double fmas = (double)X * (double)Y * (double)Z * (double)(kin * kout);
    const bool f32 = dtype == QSGB_F32 && kin <= kDenseMaxK && kout <= kDenseMaxK;
    const bool f64 = dtype == QSGB_F64 && (arith == QSGB_ARITH_AUTO || arith == QSGB_ARITH_F64) && kin <= 4 &&
                     kout <= 4 && fmas <= kDenseMaxF64Fma;
    if (f32 || f64) {
      p.div_z = make_fastdiv((uint64_t)Z);
      p.n_items = (uint64_t)X * Y * Z;
      const uint64_t blocks = (p.n_items + kDenseBlock - 1) / kDenseBlock;
      const unsigned grid =
          (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(blocks, (uint64_t)sm_count() * 8));
      if (f32)
        apply_dense_kernel<float, kDenseMaxK><<<grid, kDenseBlock, 0, s>>>(p);
      else
        apply_dense_kernel<double, 4><<<grid, kDenseBlock, 0, s>>>(p);
      return launch_status();
    }
  }
  // 2. generic kernel; a host PTM travels inside its launch parameters
  if (flags & QSGB_PTM_HOST) {
    if (kin * kout > kMaxInline) return QSGB_ERR_UNSUPPORTED;
    // the term capacity is counted here with the device's rule (entries
    // above 2^-52 max|P|, 2^-30 for FP32, non-zero for native FP64)
    double amax = 0.0;
    for (int64_t i = 0; i < kin * kout; ++i) amax = std::max(amax, std::fabs(ptm[i]));
    const double thr = arith == QSGB_ARITH_F64 ? 0.0 : amax * (arith == QSGB_ARITH_F32 ? 0x1p-30 : 0x1p-52);
    int n = 0;
    for (int64_t i = 0; i < kin * kout; ++i) {
      p.ptm_inline[i] = ptm[i];
      n += std::fabs(ptm[i]) > thr ? 1 : 0;
    }
    p.max_terms = std::max(1, n);
    p.ptm = nullptr;
  }
  if (pair) {
    const int st = dtype == QSGB_F32 ? launch_apply<float, true>(p, s) : launch_apply<double, true>(p, s);
    if (st != QSGB_ERR_UNSUPPORTED) return st;
    // pairs do not fit in shared memory: single groups
    p.iw = pick_iw((int)kout);
    p.div_z = make_fastdiv((uint64_t)Z);
    p.n_items = (uint64_t)X * Y * Z;
  }
  return dtype == QSGB_F32 ? launch_apply<float, false>(p, s) : launch_apply<double, false>(p, s);
}

}  // namespace

}  // namespace qsgb

extern "C" int qsgb_apply_ptm1(const void* in, void* out, const double* ptm, int64_t d_out, int64_t d_in,
                               int64_t dim_y, int64_t dim_z, int ptm_flags, int dtype, int arith,
                               int64_t max_terms, unsigned* dev_status, void* stream) {
  if (ptm_flags & QSGB_PTM_SWAPPED) return QSGB_ERR_INVALID;
  return qsgb::apply_common(in, out, ptm, 1, d_out, 1, d_in, 1, dim_y, dim_z, ptm_flags, dtype, arith,
                            max_terms, dev_status, stream);
}

extern "C" int qsgb_apply_ptm2(const void* in, void* out, const double* ptm, int64_t d0_out, int64_t d1_out,
                               int64_t d0_in, int64_t d1_in, int64_t dim_x, int64_t dim_y, int64_t dim_z,
                               int ptm_flags, int dtype, int arith, int64_t max_terms, unsigned* dev_status,
                               void* stream) {
  return qsgb::apply_common(in, out, ptm, d0_out, d1_out, d0_in, d1_in, dim_x, dim_y, dim_z, ptm_flags, dtype,
                            arith, max_terms, dev_status, stream);
}

extern "C" int qsgb_prepare_ptm2(const double* ptm, int64_t d0_out, int64_t d1_out, int64_t d0_in, int64_t d1_in,
                                 int64_t dim_x, int64_t dim_y, int64_t dim_z, int ptm_flags, int dtype, int arith) {
  if (!(ptm_flags & QSGB_PTM_HOST)) return QSGB_ERR_INVALID;
  // stand-in tensor addresses with the 256-byte alignment of the allocators
  // (never dereferenced: nothing is launched)
  const void* in = reinterpret_cast<const void*>(uintptr_t(256));
  void* out = reinterpret_cast<void*>(uintptr_t(512));
  return qsgb::apply_common(in, out, ptm, d0_out, d1_out, d0_in, d1_in, dim_x, dim_y, dim_z, ptm_flags, dtype,
                            arith, 0, nullptr, nullptr, qsgb::kPrepare);
}

extern "C" int qsgb_jit_check_ptm2(const double* ptm, int64_t d0_out, int64_t d1_out, int64_t d0_in, int64_t d1_in,
                                   int64_t dim_x, int64_t dim_y, int64_t dim_z, int ptm_flags, int dtype, int arith,
                                   char* src, int64_t src_bytes) {
  if (!(ptm_flags & QSGB_PTM_HOST)) return QSGB_ERR_INVALID;
  const void* in = reinterpret_cast<const void*>(uintptr_t(256));
  void* out = reinterpret_cast<void*>(uintptr_t(512));
  std::string text;
  const int st = qsgb::apply_common(in, out, ptm, d0_out, d1_out, d0_in, d1_in, dim_x, dim_y, dim_z, ptm_flags,
                                    dtype, arith, 0, nullptr, nullptr, qsgb::kCompileOnly, &text);
  if (src && src_bytes > 0) {
    const size_t n = std::min<size_t>(text.size(), (size_t)src_bytes - 1);
    std::memcpy(src, text.data(), n);
    src[n] = '\0';
  }
  return st;
}

// Gathers and reductions of the Pauli vector: multitake (diagonal), take
// along one axis (reduce_basis / project), marginal probabilities and trace,
// partial trace, and scaling (renormalize).
//
// All reductions are deterministic (fixed trees, no floating-point atomics)
// and accumulate in FP64 for both storage types.
#include <algorithm>
#include <mutex>

#include "qsgb_common.cuh"

namespace qsgb {
namespace {

constexpr int kMaxDim = 32;
constexpr int kMaxIdx = 2048;

__device__ __forceinline__ double load_f64(const void* p, int64_t i, int dtype) {
  return dtype == QSGB_F64 ? static_cast<const double*>(p)[i] : (double)static_cast<const float*>(p)[i];
}

__device__ __forceinline__ void store_from_f64(void* p, int64_t i, int dtype, double v) {
  if (dtype == QSGB_F64)
    static_cast<double*>(p)[i] = v;
  else
    static_cast<float*>(p)[i] = (float)v;
}

// ---------------------------------------------------------------- multitake
struct GatherParams {
  const void* in;
  void* out;
  int in_dtype, out_dtype;
  int ndim;
  uint64_t n_out;
  FastDiv div[kMaxDim];       // out_shape per axis
  int64_t in_stride[kMaxDim];
  int idx_off[kMaxDim + 1];
  int idx[kMaxIdx];
};

template <typename TI, typename TO>
__global__ void gather_kernel(const __grid_constant__ GatherParams p) {
  const TI* __restrict__ in = static_cast<const TI*>(p.in);
  TO* __restrict__ out = static_cast<TO*>(p.out);
  for (uint64_t o = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; o < p.n_out;
       o += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t rem = o;
    int64_t addr = 0;
    bool zero = false;
    for (int a = p.ndim - 1; a >= 0; --a) {
      const uint64_t q = fdiv(rem, p.div[a]);
      const int i = (int)(rem - q * p.div[a].d);
      rem = q;
      const int j = p.idx[p.idx_off[a] + i];
      zero |= (j < 0);
      addr += (int64_t)(j < 0 ? 0 : j) * p.in_stride[a];
    }
    out[o] = zero ? (TO)0 : (TO)in[addr];
  }
}

// ---------------------------------------------------------------- take axis
// out[o, j, :] = in[o, idx[j], :] for a tensor viewed as (outer, d_in,
// inner): a copy of rows of `inner` contiguous elements, moved as raw bits
// (bit-exact) in units V of 16 bytes when the row length and both tensors
// allow it, else of one element.  Long rows are cut into tiles of
// kTakeTile units; the row and source of a tile are found once per tile, and
// each thread keeps kTakeUnroll loads in flight.  Short rows (the last
// qudits) go unit by unit with the index arithmetic per unit.
constexpr int kTakeBlock = 256;
constexpr int kTakeUnroll = 4;
constexpr uint64_t kTakeTile = (uint64_t)kTakeBlock * kTakeUnroll;

// NIDX: capacity of the index list carried in the launch parameters (a
// small block for the usual reduce / project requests, which keeps the
// per-launch parameter copy short)
template <int NIDX>
struct TakeParams {
  const void* in;
  void* out;
  uint64_t n_rows;         // outer * d_out
  uint64_t row_v;          // units per row
  uint64_t tiles_per_row;  // row mode
  uint64_t n_units;        // unit mode: n_rows * row_v
  FastDiv div_tpr, div_dout, div_rowv;
  int64_t d_in;
  int idx[NIDX];
};

template <typename V, int NIDX>
__global__ void __launch_bounds__(kTakeBlock) take_rows_kernel(const __grid_constant__ TakeParams<NIDX> p) {
  const V* __restrict__ in = static_cast<const V*>(p.in);
  V* __restrict__ out = static_cast<V*>(p.out);
  const uint64_t n_tiles = p.n_rows * p.tiles_per_row;
  for (uint64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const uint64_t t = fdiv(tile, p.div_tpr);
    const uint64_t seg = tile - t * p.tiles_per_row;
    const uint64_t o = fdiv(t, p.div_dout);
    const int src = p.idx[(int)(t - o * p.div_dout.d)];
    const uint64_t v0 = seg * kTakeTile + threadIdx.x;
    V* dst = out + t * p.row_v;
    if (src < 0) {
#pragma unroll
      for (int u = 0; u < kTakeUnroll; ++u) {
        const uint64_t v = v0 + (uint64_t)u * kTakeBlock;
        if (v < p.row_v) dst[v] = V{};
      }
      continue;
    }
    const V* s = in + (o * (uint64_t)p.d_in + (uint64_t)src) * p.row_v;
    V r[kTakeUnroll];
#pragma unroll
    for (int u = 0; u < kTakeUnroll; ++u) {
      const uint64_t v = v0 + (uint64_t)u * kTakeBlock;
      if (v < p.row_v) r[u] = s[v];
    }
#pragma unroll
    for (int u = 0; u < kTakeUnroll; ++u) {
      const uint64_t v = v0 + (uint64_t)u * kTakeBlock;
      if (v < p.row_v) dst[v] = r[u];
    }
  }
}

template <typename V, int NIDX>
__global__ void __launch_bounds__(kTakeBlock) take_units_kernel(const __grid_constant__ TakeParams<NIDX> p) {
  const V* __restrict__ in = static_cast<const V*>(p.in);
  V* __restrict__ out = static_cast<V*>(p.out);
  const uint64_t stride = (uint64_t)gridDim.x * kTakeBlock;
  for (uint64_t e0 = (uint64_t)blockIdx.x * kTakeBlock + threadIdx.x; e0 < p.n_units;
       e0 += stride * kTakeUnroll) {
    V r[kTakeUnroll];
#pragma unroll
    for (int u = 0; u < kTakeUnroll; ++u) {
      const uint64_t e = e0 + (uint64_t)u * stride;
      r[u] = V{};
      if (e < p.n_units) {
        const uint64_t t = fdiv(e, p.div_rowv);
        const uint64_t i = e - t * p.row_v;
        const uint64_t o = fdiv(t, p.div_dout);
        const int src = p.idx[(int)(t - o * p.div_dout.d)];
        if (src >= 0) r[u] = in[(o * (uint64_t)p.d_in + (uint64_t)src) * p.row_v + i];
      }
    }
#pragma unroll
    for (int u = 0; u < kTakeUnroll; ++u) {
      const uint64_t e = e0 + (uint64_t)u * stride;
      if (e < p.n_units) out[e] = r[u];
    }
  }
}

// ---------------------------------------------------------------- marginals
// Stage 1: block (c, j) sums the entries of chunk c whose index along the
// axis is j.  Entry m of that set (m < n/d) sits at (m / s) * d * s + j*s +
// m % s, s = product of the dims after the axis.
constexpr int kRedBlock = 256;
constexpr int kMaxChunks = 512;

__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < nw; ++i) r += sh[i];
  return r;  // valid in thread 0
}

__global__ void marg_stage1(const double* __restrict__ diag, uint64_t per_j, FastDiv div_s, int64_t d, int64_t s,
                            uint64_t chunk, double* __restrict__ part) {
  __shared__ double sh[32];
  const int j = blockIdx.y;
  const uint64_t m0 = (uint64_t)blockIdx.x * chunk;
  const uint64_t m1 = min(per_j, m0 + chunk);
  double acc = 0.0;
  for (uint64_t m = m0 + threadIdx.x; m < m1; m += blockDim.x) {
    const uint64_t hi = fdiv(m, div_s);
    const uint64_t lo = m - hi * (uint64_t)s;
    acc += diag[(hi * (uint64_t)d + (uint64_t)j) * (uint64_t)s + lo];
  }
  const double r = block_sum(acc, sh);
  if (threadIdx.x == 0) part[(int64_t)j * gridDim.x + blockIdx.x] = r;
}

__global__ void marg_stage2(const double* __restrict__ part, int nchunks, double* __restrict__ out) {
  __shared__ double sh[32];
  const int j = blockIdx.x;
  double acc = 0.0;
  for (int c = threadIdx.x; c < nchunks; c += blockDim.x) acc += part[(int64_t)j * nchunks + c];
  const double r = block_sum(acc, sh);
  if (threadIdx.x == 0) out[j] = r;
}

// ------------------------------------------------ diagonal marginals, fused
// Marginals of the DM diagonal read straight from the Pauli vector through
// the multitake plan (no diagonal tensor): one block, outcome by outcome,
// fixed-order reduction.  out[j] for j < n_out, then out[n_out] = the device
// status word (so one device-to-host copy returns both).
struct DiagRedParams {
  const void* in;
  double* out;
  const unsigned* status;
  double* part;      // per-block partial sums [grid][n_out] (grid > 1)
  unsigned* ticket;  // blocks finished (grid > 1); zero between calls
  int in_dtype;
  int ndim;
  int axis;        // -1: trace
  int n_out;       // 1 for the trace, else the Hilbert dim of `axis`
  uint64_t per_j;  // diagonal entries per outcome
  FastDiv div_s;   // entries of the diagonal index after `axis`
  uint64_t s_axis;
  FastDiv div[kMaxDim];  // Hilbert dims per axis (diagonal index space)
  int64_t in_stride[kMaxDim];
  int idx_off[kMaxDim + 1];
  int idx[kMaxIdx];
};

constexpr int kDiagRedBlock = 1024;

__global__ void __launch_bounds__(kDiagRedBlock) diag_marginals_kernel(const __grid_constant__ DiagRedParams p) {
  __shared__ double sh[32];
  __shared__ int last;
  const uint64_t d_axis = p.axis < 0 ? 1 : p.div[p.axis].d;
  constexpr int U = 8;  // independent loads in flight per thread
  // this block's share of each outcome's entries: the scattered diagonal
  // loads of one SM are bounded by its outstanding misses, so a large
  // diagonal is spread over many blocks
  const uint64_t chunk = (p.per_j + gridDim.x - 1) / gridDim.x;
  const uint64_t m_beg = (uint64_t)blockIdx.x * chunk;
  const uint64_t m_end = m_beg + chunk < p.per_j ? m_beg + chunk : p.per_j;
  for (int j = 0; j < p.n_out; ++j) {
    double acc = 0.0;
    for (uint64_t m0 = m_beg + threadIdx.x; m0 < m_end; m0 += (uint64_t)U * kDiagRedBlock) {
      double v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        // m-th diagonal entry whose index along `axis` is j
        const uint64_t m = m0 + (uint64_t)u * kDiagRedBlock;
        v[u] = 0.0;
        if (m < m_end) {
          const uint64_t hi = fdiv(m, p.div_s);
          const uint64_t lo = m - hi * p.s_axis;
          uint64_t rem = (hi * d_axis + (uint64_t)j) * p.s_axis + lo;
          int64_t addr = 0;
          bool zero = false;
          for (int a = p.ndim - 1; a >= 0; --a) {
            const uint64_t q = fdiv(rem, p.div[a]);
            const int i = (int)(rem - q * p.div[a].d);
            rem = q;
            const int k = p.idx[p.idx_off[a] + i];
            zero |= k < 0;
            addr += (int64_t)(k < 0 ? 0 : k) * p.in_stride[a];
          }
          if (!zero) v[u] = load_f64(p.in, addr, p.in_dtype);
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) acc += v[u];  // fixed order
    }
    const double r = block_sum(acc, sh);
    if (threadIdx.x == 0) {
      if (gridDim.x == 1)
        p.out[j] = r;
      else
        p.part[(int64_t)blockIdx.x * p.n_out + j] = r;
    }
  }
  if (gridDim.x == 1) {
    if (threadIdx.x == 0) p.out[p.n_out] = p.status ? (double)*p.status : 0.0;
    return;
  }
  // the last block to finish adds the partials in block order
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(p.ticket, 1u) == gridDim.x - 1 ? 1 : 0;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  for (int j = threadIdx.x; j < p.n_out; j += kDiagRedBlock) {
    double s = 0.0;
    for (unsigned b = 0; b < gridDim.x; ++b) s += __ldcg(p.part + (int64_t)b * p.n_out + j);
    p.out[j] = s;
  }
  if (threadIdx.x == 0) {
    p.out[p.n_out] = p.status ? (double)*p.status : 0.0;
    *p.ticket = 0u;  // ready for the next call
  }
}

// ---------------------------------------------------------------- partial trace
constexpr int kMaxPtEntries = 1024;

struct PtParams {
  const void* in;
  void* out;
  int dtype;
  int nkeep, ntr;
  uint64_t n_out, n_combos;
  FastDiv kdiv[kMaxDim];         // kept dims (ascending qudit order)
  int64_t kstride[kMaxDim];
  FastDiv tdiv[kMaxDim];         // traced: number of non-zero weights
  int64_t tstride[kMaxDim];
  int toff[kMaxDim + 1];
  int tidx[kMaxPtEntries];
  double tw[kMaxPtEntries];
};

__device__ __forceinline__ int64_t pt_base(const PtParams& p, uint64_t o) {
  int64_t base = 0;
  for (int a = p.nkeep - 1; a >= 0; --a) {
    const uint64_t q = fdiv(o, p.kdiv[a]);
    base += (int64_t)(o - q * p.kdiv[a].d) * p.kstride[a];
    o = q;
  }
  return base;
}

__device__ __forceinline__ double pt_term(const PtParams& p, int64_t base, uint64_t c) {
  int64_t addr = base;
  double w = 1.0;
  for (int a = p.ntr - 1; a >= 0; --a) {
    const uint64_t q = fdiv(c, p.tdiv[a]);
    const int i = p.toff[a] + (int)(c - q * p.tdiv[a].d);
    c = q;
    addr += (int64_t)p.tidx[i] * p.tstride[a];
    w *= p.tw[i];
  }
  return w * load_f64(p.in, addr, p.dtype);
}

// few combos: one thread per output element
__global__ void pt_thread_kernel(const __grid_constant__ PtParams p) {
  for (uint64_t o = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; o < p.n_out;
       o += (uint64_t)gridDim.x * blockDim.x) {
    const int64_t base = pt_base(p, o);
    double acc = 0.0;
    for (uint64_t c = 0; c < p.n_combos; ++c) acc += pt_term(p, base, c);
    store_from_f64(p.out, (int64_t)o, p.dtype, acc);
  }
}

// many combos: one block per output element
__global__ void pt_block_kernel(const __grid_constant__ PtParams p) {
  __shared__ double sh[32];
  for (uint64_t o = blockIdx.x; o < p.n_out; o += gridDim.x) {
    const int64_t base = pt_base(p, o);
    double acc = 0.0;
    for (uint64_t c = threadIdx.x; c < p.n_combos; c += blockDim.x) acc += pt_term(p, base, c);
    const double r = block_sum(acc, sh);
    if (threadIdx.x == 0) store_from_f64(p.out, (int64_t)o, p.dtype, r);
  }
}

// ---------------------------------------------------------------- scaling
template <typename T>
__global__ void scale_kernel(T* __restrict__ x, uint64_t n, double alpha, const double* __restrict__ denom,
                             double thr) {
  double a = alpha;
  if (denom) {
    const double d = *denom;
    if (!(d > thr)) return;
    a = 1.0 / d;
  }
  const T ta = (T)a;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    x[i] = x[i] * ta;
}

unsigned grid_for(uint64_t n, int block, int per_sm = 8) {
  const uint64_t need = (n + block - 1) / block;
  const uint64_t cap = (uint64_t)sm_count() * per_sm;
  return (unsigned)std::max<uint64_t>(1, std::min(need, cap));
}

}  // namespace
}  // namespace qsgb

using namespace qsgb;

extern "C" int qsgb_gather(const void* in, void* out, int in_dtype, int out_dtype, int ndim, const int64_t* in_shape,
                           const int32_t* idx_off, const int32_t* idx, void* stream) {
  if (!in || !out || !in_shape || !idx_off || (!idx && ndim > 0)) return QSGB_ERR_INVALID;
  if (ndim < 0 || ndim > kMaxDim) return QSGB_ERR_UNSUPPORTED;
  if ((in_dtype != QSGB_F64 && in_dtype != QSGB_F32) || (out_dtype != QSGB_F64 && out_dtype != QSGB_F32))
    return QSGB_ERR_INVALID;
  if (idx_off[0] != 0 || idx_off[ndim] > kMaxIdx) return QSGB_ERR_UNSUPPORTED;
  GatherParams p{};  // copied into the launch
  p.in = in;
  p.out = out;
  p.in_dtype = in_dtype;
  p.out_dtype = out_dtype;
  p.ndim = ndim;
  uint64_t n_out = 1;
  int64_t stride = 1;
  for (int a = ndim - 1; a >= 0; --a) {
    const int len = idx_off[a + 1] - idx_off[a];
    if (len < 1 || in_shape[a] < 1) return QSGB_ERR_INVALID;
    for (int i = idx_off[a]; i < idx_off[a + 1]; ++i)
      if (idx[i] >= in_shape[a] || idx[i] < -1) return QSGB_ERR_INVALID;
    p.div[a] = make_fastdiv((uint64_t)len);
    p.in_stride[a] = stride;
    stride *= in_shape[a];
    n_out *= (uint64_t)len;
  }
  for (int a = 0; a <= ndim; ++a) p.idx_off[a] = idx_off[a];
  for (int i = 0; i < idx_off[ndim]; ++i) p.idx[i] = idx[i];
  p.n_out = n_out;
  cudaStream_t s = as_stream(stream);
  const int block = 256;
  const unsigned grid = grid_for(n_out, block);
  if (in_dtype == QSGB_F64 && out_dtype == QSGB_F64)
    gather_kernel<double, double><<<grid, block, 0, s>>>(p);
  else if (in_dtype == QSGB_F32 && out_dtype == QSGB_F64)
    gather_kernel<float, double><<<grid, block, 0, s>>>(p);
  else if (in_dtype == QSGB_F64 && out_dtype == QSGB_F32)
    gather_kernel<double, float><<<grid, block, 0, s>>>(p);
  else
    gather_kernel<float, float><<<grid, block, 0, s>>>(p);
  return launch_status();
}

template <int NIDX>
int take_launch(const void* in, void* out, int dtype, int64_t outer, int64_t d_in, int64_t inner,
                const int32_t* idx, int64_t d_out, cudaStream_t s) {
  TakeParams<NIDX> p{};
  p.in = in;
  p.out = out;
  for (int64_t j = 0; j < d_out; ++j) p.idx[j] = idx[j];
  const size_t esz = dtype == QSGB_F64 ? 8 : 4;
  // 16-byte units when a row is a whole number of them and both tensors
  // start on a 16-byte boundary
  const bool wide = ((uint64_t)inner * esz) % 16 == 0 && (uintptr_t)in % 16 == 0 && (uintptr_t)out % 16 == 0;
  const size_t usz = wide ? 16 : esz;
  p.row_v = (uint64_t)inner * esz / usz;
  p.n_rows = (uint64_t)outer * (uint64_t)d_out;
  p.d_in = d_in;
  p.div_dout = make_fastdiv((uint64_t)d_out);
  const bool rows = p.row_v >= 128;
  unsigned grid;
  if (rows) {
    p.tiles_per_row = (p.row_v + kTakeTile - 1) / kTakeTile;
    p.div_tpr = make_fastdiv(p.tiles_per_row);
    grid = grid_for(p.n_rows * p.tiles_per_row * kTakeBlock, kTakeBlock);
  } else {
    p.n_units = p.n_rows * p.row_v;
    p.div_rowv = make_fastdiv(p.row_v);
    grid = grid_for((p.n_units + kTakeUnroll - 1) / kTakeUnroll, kTakeBlock);
  }
  if (usz == 16) {
    if (rows) take_rows_kernel<uint4, NIDX><<<grid, kTakeBlock, 0, s>>>(p);
    else take_units_kernel<uint4, NIDX><<<grid, kTakeBlock, 0, s>>>(p);
  } else if (usz == 8) {
    if (rows) take_rows_kernel<unsigned long long, NIDX><<<grid, kTakeBlock, 0, s>>>(p);
    else take_units_kernel<unsigned long long, NIDX><<<grid, kTakeBlock, 0, s>>>(p);
  } else {
    if (rows) take_rows_kernel<unsigned, NIDX><<<grid, kTakeBlock, 0, s>>>(p);
    else take_units_kernel<unsigned, NIDX><<<grid, kTakeBlock, 0, s>>>(p);
  }
  return launch_status();
}

extern "C" int qsgb_take_axis(const void* in, void* out, int dtype, int64_t outer, int64_t d_in, int64_t inner,
                              const int32_t* idx, int64_t d_out, void* stream) {
  if (!in || !out || !idx || in == out) return QSGB_ERR_INVALID;
  if (dtype != QSGB_F64 && dtype != QSGB_F32) return QSGB_ERR_INVALID;
  if (outer < 1 || d_in < 1 || inner < 1 || d_out < 1) return QSGB_ERR_INVALID;
  if (d_out > kMaxIdx) return QSGB_ERR_UNSUPPORTED;
  for (int64_t j = 0; j < d_out; ++j)
    if (idx[j] >= d_in || idx[j] < -1) return QSGB_ERR_INVALID;
  cudaStream_t s = as_stream(stream);
  if (d_out <= 32) return take_launch<32>(in, out, dtype, outer, d_in, inner, idx, d_out, s);
  return take_launch<kMaxIdx>(in, out, dtype, outer, d_in, inner, idx, d_out, s);
}

namespace qsgb {
namespace {
constexpr int kDiagEntriesPerBlock = 512;  // diagonal entries per block (per outcome)
constexpr int kDiagMaxOut = 64;
}  // namespace
}  // namespace qsgb

extern "C" int64_t qsgb_diag_marginals_scratch_bytes(void) {
  return 16 + (int64_t)qsgb::sm_count() * qsgb::kDiagMaxOut * (int64_t)sizeof(double);
}

extern "C" int qsgb_diag_marginals(const void* in, int in_dtype, int ndim, const int64_t* in_shape,
                                   const int32_t* idx_off, const int32_t* idx, int axis, double* out,
                                   const unsigned* dev_status, double* host_out, void* scratch,
                                   int64_t scratch_bytes, void* stream) {
  if (!in || !out || !idx_off || (ndim > 0 && (!in_shape || !idx))) return QSGB_ERR_INVALID;
  if (in_dtype != QSGB_F64 && in_dtype != QSGB_F32) return QSGB_ERR_INVALID;
  if (ndim < 0 || ndim > kMaxDim || axis < -1 || axis >= ndim) return QSGB_ERR_INVALID;
  if (idx_off[0] != 0 || idx_off[ndim] > kMaxIdx) return QSGB_ERR_UNSUPPORTED;
  DiagRedParams p{};
  p.in = in;
  p.out = out;
  p.status = dev_status;
  p.in_dtype = in_dtype;
  p.ndim = ndim;
  p.axis = axis;
  uint64_t n = 1, s_axis = 1;
  int64_t stride = 1;
  for (int a = ndim - 1; a >= 0; --a) {
    const int len = idx_off[a + 1] - idx_off[a];
    if (len < 1 || in_shape[a] < 1) return QSGB_ERR_INVALID;
    for (int i = idx_off[a]; i < idx_off[a + 1]; ++i)
      if (idx[i] >= in_shape[a] || idx[i] < -1) return QSGB_ERR_INVALID;
    p.div[a] = make_fastdiv((uint64_t)len);
    p.in_stride[a] = stride;
    stride *= in_shape[a];
    if (axis >= 0 && a > axis) s_axis *= (uint64_t)len;
    n *= (uint64_t)len;
  }
  // one block: diagonals of up to 2^22 entries (prod of Hilbert dims)
  if (n > (1ull << 22)) return QSGB_ERR_UNSUPPORTED;
  const uint64_t d = axis < 0 ? 1 : (uint64_t)(idx_off[axis + 1] - idx_off[axis]);
  if (d > 64) return QSGB_ERR_UNSUPPORTED;
  p.n_out = (int)d;
  p.per_j = n / d;
  p.s_axis = axis < 0 ? 1 : s_axis;
  p.div_s = make_fastdiv(p.s_axis);
  for (int a = 0; a <= ndim; ++a) p.idx_off[a] = idx_off[a];
  for (int i = 0; i < idx_off[ndim]; ++i) p.idx[i] = idx[i];
  // blocks: one per kDiagEntriesPerBlock entries of an outcome, at most one
  // per SM, and as many as the scratch holds partials for
  uint64_t grid = (p.per_j + kDiagEntriesPerBlock - 1) / kDiagEntriesPerBlock;
  grid = std::min<uint64_t>(grid, (uint64_t)sm_count());
  if (!scratch || scratch_bytes < 16 + (int64_t)sizeof(double) * p.n_out) grid = 1;
  if (grid > 1) {
    if ((uintptr_t)scratch % 16 != 0) return QSGB_ERR_INVALID;
    grid = std::min<uint64_t>(grid, (uint64_t)((scratch_bytes - 16) / ((int64_t)sizeof(double) * p.n_out)));
    p.ticket = static_cast<unsigned*>(scratch);
    p.part = reinterpret_cast<double*>(static_cast<unsigned char*>(scratch) + 16);
  }
  cudaStream_t st = as_stream(stream);
  diag_marginals_kernel<<<(unsigned)std::max<uint64_t>(grid, 1), kDiagRedBlock, 0, st>>>(p);
  const int ls = launch_status();
  if (ls != QSGB_OK || !host_out) return ls;
  QSGB_CUDA_TRY(cudaMemcpyAsync(host_out, out, (d + 1) * sizeof(double), cudaMemcpyDeviceToHost, st));
  QSGB_CUDA_TRY(cudaStreamSynchronize(st));
  return QSGB_OK;
}

static void marg_geometry(int64_t n, int64_t n_out, int* nchunks, uint64_t* chunk) {
  const uint64_t per_j = (uint64_t)(n / std::max<int64_t>(n_out, 1));
  uint64_t c = std::max<uint64_t>(4096, (per_j + kMaxChunks - 1) / kMaxChunks);
  int nc = (int)std::max<uint64_t>(1, (per_j + c - 1) / c);
  *nchunks = nc;
  *chunk = c;
}

extern "C" int64_t qsgb_marginals_scratch_bytes(int64_t n, int64_t n_out) {
  if (n < 1 || n_out < 1) return 0;
  int nc;
  uint64_t c;
  marg_geometry(n, n_out, &nc, &c);
  return (int64_t)nc * n_out * (int64_t)sizeof(double);
}

extern "C" int qsgb_marginals(const double* diag, int ndim, const int64_t* shape, int axis, double* out,
                              void* scratch, int64_t scratch_bytes, void* stream) {
  if (!diag || !out || (!shape && ndim > 0)) return QSGB_ERR_INVALID;
  if (ndim < 0 || axis < -1 || axis >= ndim) return QSGB_ERR_INVALID;
  int64_t n = 1, s = 1;
  for (int a = 0; a < ndim; ++a) {
    if (shape[a] < 1) return QSGB_ERR_INVALID;
    n *= shape[a];
    if (a > axis && axis >= 0) s *= shape[a];
  }
  const int64_t d = axis < 0 ? 1 : shape[axis];
  if (axis < 0) s = 1;
  if (d > 65535) return QSGB_ERR_UNSUPPORTED;
  int nc;
  uint64_t chunk;
  marg_geometry(n, d, &nc, &chunk);
  if (!scratch || scratch_bytes < (int64_t)nc * d * (int64_t)sizeof(double)) return QSGB_ERR_SCRATCH;
  double* part = static_cast<double*>(scratch);
  cudaStream_t st = as_stream(stream);
  const uint64_t per_j = (uint64_t)(n / d);
  marg_stage1<<<dim3(nc, (unsigned)d), kRedBlock, 0, st>>>(diag, per_j, make_fastdiv((uint64_t)s), d, s, chunk, part);
  marg_stage2<<<(unsigned)d, kRedBlock, 0, st>>>(part, nc, out);
  return launch_status();
}

extern "C" int qsgb_partial_trace(const void* in, void* out, int dtype, int ndim, const int64_t* shape,
                                  const int32_t* keep, const double* weights, void* stream) {
  if (!in || !out || in == out || (ndim > 0 && (!shape || !keep))) return QSGB_ERR_INVALID;
  if (dtype != QSGB_F64 && dtype != QSGB_F32) return QSGB_ERR_INVALID;
  if (ndim < 0 || ndim > kMaxDim) return QSGB_ERR_UNSUPPORTED;
  PtParams p{};
  p.in = in;
  p.out = out;
  p.dtype = dtype;
  int64_t stride = 1;
  int nent = 0;
  int nkeep = 0, ntr = 0;
  for (int a = 0; a < ndim; ++a) (keep[a] ? nkeep : ntr)++;
  if (ntr > 0 && !weights) return QSGB_ERR_INVALID;
  // walk from the least significant axis
  int woffs[kMaxDim];
  {
    int off = 0;
    for (int a = 0; a < ndim; ++a)
      if (!keep[a]) {
        woffs[a] = off;
        off += (int)shape[a];
      }
  }
  uint64_t n_out = 1, n_combos = 1;
  int kpos = nkeep, tpos = ntr;
  int toff_rev[kMaxDim];
  for (int a = ndim - 1; a >= 0; --a) {
    if (shape[a] < 1) return QSGB_ERR_INVALID;
    if (keep[a]) {
      --kpos;
      p.kdiv[kpos] = make_fastdiv((uint64_t)shape[a]);
      p.kstride[kpos] = stride;
      n_out *= (uint64_t)shape[a];
    } else {
      --tpos;
      int cnt = 0;
      toff_rev[tpos] = nent;
      for (int64_t k = 0; k < shape[a]; ++k) {
        const double w = weights[woffs[a] + k];
        if (w != 0.0) {
          if (nent >= kMaxPtEntries) return QSGB_ERR_UNSUPPORTED;
          p.tidx[nent] = (int)k;
          p.tw[nent] = w;
          ++nent;
          ++cnt;
        }
      }
      p.tdiv[tpos] = make_fastdiv((uint64_t)std::max(cnt, 1));
      p.tstride[tpos] = stride;
      if (cnt == 0) n_combos = 0;
      else n_combos *= (uint64_t)cnt;
    }
    stride *= shape[a];
  }
  // entries were appended from the last traced axis backwards; toff[t] is
  // the start of traced axis t (ascending)
  for (int t = 0; t < ntr; ++t) p.toff[t] = toff_rev[t];
  p.toff[ntr] = nent;
  p.nkeep = nkeep;
  p.ntr = ntr;
  p.n_out = n_out;
  p.n_combos = n_combos;
  cudaStream_t s = as_stream(stream);
  if (n_combos == 0) {
    QSGB_CUDA_TRY(cudaMemsetAsync(out, 0, n_out * (dtype == QSGB_F64 ? 8 : 4), s));
    return QSGB_OK;
  }
  if (n_combos <= 64) {
    pt_thread_kernel<<<grid_for(n_out, 256), 256, 0, s>>>(p);
  } else {
    const int block = n_combos >= 256 ? 256 : 128;
    pt_block_kernel<<<(unsigned)std::min<uint64_t>(n_out, (uint64_t)sm_count() * 16), block, 0, s>>>(p);
  }
  return launch_status();
}

extern "C" int qsgb_scale(void* x, int dtype, int64_t n, double alpha, void* stream) {
  if (!x || n < 0) return QSGB_ERR_INVALID;
  if (n == 0) return QSGB_OK;
  cudaStream_t s = as_stream(stream);
  if (dtype == QSGB_F64)
    scale_kernel<double><<<grid_for((uint64_t)n, 256), 256, 0, s>>>(static_cast<double*>(x), (uint64_t)n, alpha,
                                                                   nullptr, 0.0);
  else if (dtype == QSGB_F32)
    scale_kernel<float><<<grid_for((uint64_t)n, 256), 256, 0, s>>>(static_cast<float*>(x), (uint64_t)n, alpha,
                                                                 nullptr, 0.0);
  else
    return QSGB_ERR_INVALID;
  return launch_status();
}

extern "C" int qsgb_scale_by_inverse(void* x, int dtype, int64_t n, const double* denom, double threshold,
                                     void* stream) {
  if (!x || !denom || n < 0) return QSGB_ERR_INVALID;
  if (n == 0) return QSGB_OK;
  cudaStream_t s = as_stream(stream);
  if (dtype == QSGB_F64)
    scale_kernel<double><<<grid_for((uint64_t)n, 256), 256, 0, s>>>(static_cast<double*>(x), (uint64_t)n, 1.0,
                                                                   denom, threshold);
  else if (dtype == QSGB_F32)
    scale_kernel<float><<<grid_for((uint64_t)n, 256), 256, 0, s>>>(static_cast<float*>(x), (uint64_t)n, 1.0,
                                                                 denom, threshold);
  else
    return QSGB_ERR_INVALID;
  return launch_status();
}

// ---------------------------------------------------------------------------
// Marginals without any allocation by anyone.
//
// qsgb_marginals() needs a scratch buffer for its per-chunk partial sums and
// leaves allocating it to the caller.  Some programs that embed this library
// cannot allocate device memory at the point where they need probabilities:
// applications whose device memory is wholly owned by their own pool
// allocator (which forbids outside cudaMalloc calls), or latency-critical
// measurement loops in which the implicit device synchronisation of
// cudaMalloc / cudaFree would stall the pipeline.  For them the partial sums
// live in the fixed array below, which exists in every device that loads
// this library for as long as the process runs.
// ---------------------------------------------------------------------------
namespace {

// 16384 doubles (128 KiB): enough for up to 512 chunks x 32 outcomes, i.e.
// any diagonal of qudits with up to 32 levels.
constexpr int64_t kNoAllocScratchDoubles = 16384;
__device__ __align__(256) double g_noalloc_marg_scratch[kNoAllocScratchDoubles];

// Device address of the array, looked up once per device and CUDA context
// (the name is only a host-side stand-in for the symbol in host code).  The
// address belongs to the context the module was loaded in: after
// cudaDeviceReset, or under another context made current through the driver
// API, the lookup is done again.  Contexts are told apart by their driver
// id, which is never reused within a process.
typedef int (*CtxGetCurrentFn)(void**);
typedef int (*CtxGetIdFn)(void*, unsigned long long*);

struct NoAllocSlot {
  unsigned long long ctx_id;
  double* ptr;
};
std::mutex g_noalloc_mu;
NoAllocSlot g_noalloc_slot[64] = {};

// Driver id of the current context (0 if none is current or the driver
// entry points are unavailable, in which case the address is looked up on
// every call).
unsigned long long current_context_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = (CtxGetCurrentFn)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (CtxGetIdFn)f;
    cudaGetLastError();
  });
  if (!get_current || !get_id) return 0;
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
  return id;
}

int noalloc_scratch(double** ptr) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return QSGB_ERR_CUDA;
  if (dev < 0 || dev >= 64) return QSGB_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  const unsigned long long id = current_context_id();
  NoAllocSlot& slot = g_noalloc_slot[dev];
  if (id != 0 && slot.ptr && slot.ctx_id == id) {
    *ptr = slot.ptr;
    return QSGB_OK;
  }
  // first call on this device (or in this context): the lookup loads the
  // library's device module if needed, which reserves the array
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_noalloc_marg_scratch) != cudaSuccess || !p) {
    cudaGetLastError();
    return QSGB_ERR_CUDA;
  }
  slot.ptr = static_cast<double*>(p);
  slot.ctx_id = id != 0 ? id : current_context_id();  // a context now exists
  *ptr = slot.ptr;
  return QSGB_OK;
}

}  // namespace

extern "C" int64_t qsgb_marginals_noalloc_max_scratch_bytes(void) {
  return kNoAllocScratchDoubles * (int64_t)sizeof(double);
}

extern "C" int qsgb_marginals_noalloc(const double* diag, int ndim, const int64_t* shape, int axis, double* out,
                                      void* stream) {
  if (!diag || !out || (!shape && ndim > 0)) return QSGB_ERR_INVALID;
  if (ndim < 0 || axis < -1 || axis >= ndim) return QSGB_ERR_INVALID;
  int64_t n = 1, s = 1;
  for (int a = 0; a < ndim; ++a) {
    if (shape[a] < 1) return QSGB_ERR_INVALID;
    n *= shape[a];
    if (a > axis && axis >= 0) s *= shape[a];
  }
  const int64_t d = axis < 0 ? 1 : shape[axis];
  if (axis < 0) s = 1;
  if (d > 65535) return QSGB_ERR_UNSUPPORTED;
  int nc;
  uint64_t chunk;
  marg_geometry(n, d, &nc, &chunk);
  // the fixed array bounds the request: refuse instead of overrunning it
  if ((int64_t)nc * d > kNoAllocScratchDoubles) return QSGB_ERR_SCRATCH;
  double* part = nullptr;
  const int st0 = noalloc_scratch(&part);
  if (st0 != QSGB_OK) return st0;
  // every partial the second stage reads is written by the first stage of
  // this call, so nothing needs clearing between calls
  cudaStream_t st = as_stream(stream);
  const uint64_t per_j = (uint64_t)(n / d);
  marg_stage1<<<dim3(nc, (unsigned)d), kRedBlock, 0, st>>>(diag, per_j, make_fastdiv((uint64_t)s), d, s, chunk, part);
  marg_stage2<<<(unsigned)d, kRedBlock, 0, st>>>(part, nc, out);
  return launch_status();
}

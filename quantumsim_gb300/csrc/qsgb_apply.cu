// PTM application kernels: one- and two-qudit Pauli transfer matrices on any
// qudit positions, FP64 (df64 or native arithmetic) and FP32 storage.
//
// Replaces quantumsim/pauli_vectors/primitives.cu:15-89 (two_qubit_general_ptm,
// one thread per output element, PTM row re-read from global memory per
// thread) as launched from quantumsim/pauli_vectors/cuda.py:151-277.
//
// Design:
//  * The state tensor is viewed as (X, Da, Y, Db, Z) with targets a < b; a
//    one-qudit PTM is the case X = Da = 1.  A "group" is one bystander index
//    (x, y, z); it owns Kin = Da_in*Db_in inputs and Kout outputs.
//  * Each block compacts the PTM into a per-row term list in shared memory
//    once (exact zeros and entries below 2^-60 of the largest one dropped),
//    then loops grid-stride over groups.  Consecutive threads take
//    consecutive z, so every one of the Kin loads and Kout stores of a warp
//    is a contiguous run whenever Z >= 32.
//  * Inputs are parked in a per-thread shared-memory column so that the term
//    loop can index them at run time.
//  * df64: rows with one term use a single FP64 multiply (exact, as numpy);
//    rows with more terms accumulate in float-float on the FP32 pipes.
#include <algorithm>
#include <cstdio>

#include "qsgb_common.cuh"

namespace qsgb {

namespace {

constexpr int kMaxK = 256;        // Kin, Kout limit
constexpr int kMaxEntries = 6561; // Kout*Kin limit (two qutrits)
constexpr int kMaxInline = 256;   // host PTMs up to 16x16 travel in the launch

struct ApplyParams {
  const void* in;
  void* out;
  const double* ptm;  // device PTM, or nullptr when ptm_inline is used
  int kin, kout;
  int da_in, db_in, da_out, db_out;
  int flags;
  int max_terms;
  uint64_t n_groups;
  FastDiv div_z, div_y;
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
  // region 0: max(PTM staging, per-thread input columns)
  size_t xs_off, xs_bytes;
  size_t terms_off;   // float2[max_terms]
  size_t tk_off;      // uint16[max_terms]
  size_t rowptr_off;  // int[kout + 1]
  size_t rowone_off;  // double[kout]
  size_t offin_off;   // int64[kin]
  size_t offout_off;  // int64[kout]
  size_t red_off;     // double[32] reduction scratch + int flag
  size_t total;
};

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

SmemLayout make_layout(int kin, int kout, int max_terms, int block, size_t elem) {
  SmemLayout L;
  size_t xs = (size_t)kin * block * elem;
  size_t stage = (size_t)kin * kout * sizeof(double);
  L.xs_off = 0;
  L.xs_bytes = std::max(xs, stage);
  size_t o = align_up(L.xs_bytes, 16);
  L.terms_off = o;
  o = align_up(o + (size_t)max_terms * sizeof(float2), 16);
  L.tk_off = o;
  o = align_up(o + (size_t)max_terms * sizeof(uint16_t), 16);
  L.rowptr_off = o;
  o = align_up(o + (size_t)(kout + 1) * sizeof(int), 16);
  L.rowone_off = o;
  o = align_up(o + (size_t)kout * sizeof(double), 16);
  L.offin_off = o;
  o = align_up(o + (size_t)kin * sizeof(int64_t), 16);
  L.offout_off = o;
  o = align_up(o + (size_t)kout * sizeof(int64_t), 16);
  L.red_off = o;
  o = align_up(o + 34 * sizeof(double), 16);
  L.total = o;
  return L;
}

// ARITH: QSGB_ARITH_DF64 / QSGB_ARITH_F64 (T = double) or QSGB_ARITH_F32 (T = float)
template <typename T, int ARITH>
__global__ void apply_ptm_kernel(const __grid_constant__ ApplyParams p, const SmemLayout L) {
  extern __shared__ __align__(16) unsigned char smem[];
  double* stage = reinterpret_cast<double*>(smem + L.xs_off);
  T* xs = reinterpret_cast<T*>(smem + L.xs_off);
  float2* terms = reinterpret_cast<float2*>(smem + L.terms_off);
  uint16_t* tk = reinterpret_cast<uint16_t*>(smem + L.tk_off);
  int* rowptr = reinterpret_cast<int*>(smem + L.rowptr_off);
  double* rowone = reinterpret_cast<double*>(smem + L.rowone_off);
  int64_t* offin = reinterpret_cast<int64_t*>(smem + L.offin_off);
  int64_t* offout = reinterpret_cast<int64_t*>(smem + L.offout_off);
  double* red = reinterpret_cast<double*>(smem + L.red_off);
  int* overflow = reinterpret_cast<int*>(red + 33);

  const int tid = threadIdx.x;
  const int nthr = blockDim.x;
  const int ne = p.kin * p.kout;
  const double* __restrict__ src = p.ptm ? p.ptm : p.ptm_inline;

  // ---- 1. stage the op matrix M[r][k] and find max |M| ----
  double amax = 0.0;
  for (int i = tid; i < ne; i += nthr) {
    const int r = i / p.kin, k = i - r * p.kin;
    const double v = src[ptm_index(p, r, k)];
    stage[i] = v;
    amax = fmax(amax, fabs(v));
  }
  for (int o = 16; o > 0; o >>= 1) amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
  if ((tid & 31) == 0) red[tid >> 5] = amax;
  if (tid == 0) *overflow = 0;
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
  // drop threshold: exact zeros for native FP64, else far below precision
  const double thr = (ARITH == QSGB_ARITH_F64) ? 0.0 : red[32] * ((ARITH == QSGB_ARITH_F32) ? 0x1p-40 : 0x1p-60);

  // ---- 2. per-row term counts and prefix sum ----
  for (int r = tid; r < p.kout; r += nthr) {
    int c = 0;
    for (int k = 0; k < p.kin; ++k) c += fabs(stage[r * p.kin + k]) > thr;
    rowptr[r + 1] = c;
  }
  __syncthreads();
  if (tid == 0) {
    rowptr[0] = 0;
    for (int r = 0; r < p.kout; ++r) rowptr[r + 1] += rowptr[r];
    if (rowptr[p.kout] > p.max_terms) *overflow = 1;
  }
  __syncthreads();
  if (*overflow) {
    if (tid == 0 && p.status) atomicOr(p.status, QSGB_DEV_BADITEM);
    return;
  }
  for (int r = tid; r < p.kout; r += nthr) {
    int t = rowptr[r];
    double one = 0.0;
    for (int k = 0; k < p.kin; ++k) {
      const double v = stage[r * p.kin + k];
      if (fabs(v) > thr) {
        if (ARITH == QSGB_ARITH_F64) {
          terms[t] = make_float2(__int_as_float(__double2loint(v)), __int_as_float(__double2hiint(v)));
        } else {
          const float h = (float)v;
          const float l = (float)(v - (double)h);
          terms[t] = make_float2(h, l);
        }
        tk[t] = (uint16_t)k;
        one = v;
        ++t;
      }
    }
    rowone[r] = one;
  }
  __syncthreads();  // stage[] is reused as xs[] below

  // ---- 3. stream the groups ----
  const T* __restrict__ in = static_cast<const T*>(p.in);
  T* __restrict__ out = static_cast<T*>(p.out);
  unsigned bad = 0;
  const uint64_t stride = (uint64_t)gridDim.x * nthr;
  for (uint64_t g = (uint64_t)blockIdx.x * nthr + tid; g < p.n_groups; g += stride) {
    const uint64_t t1 = fdiv(g, p.div_z);
    const uint64_t z = g - t1 * p.div_z.d;
    const uint64_t x = fdiv(t1, p.div_y);
    const uint64_t y = t1 - x * p.div_y.d;
    const int64_t bi = (int64_t)x * p.sxi + (int64_t)y * p.syi + (int64_t)z;
    const int64_t bo = (int64_t)x * p.sxo + (int64_t)y * p.syo + (int64_t)z;
    for (int k = 0; k < p.kin; ++k) xs[k * nthr + tid] = in[bi + offin[k]];
    for (int r = 0; r < p.kout; ++r) {
      const int beg = rowptr[r], end = rowptr[r + 1];
      T yv;
      if (ARITH == QSGB_ARITH_F32) {
        float acc = 0.f;
        for (int t = beg; t < end; ++t) acc = fmaf(terms[t].x, (float)xs[tk[t] * nthr + tid], acc);
        yv = (T)acc;
      } else if (ARITH == QSGB_ARITH_F64) {
        double acc = 0.0;
        for (int t = beg; t < end; ++t) {
          const double pv = __hiloint2double(__float_as_int(terms[t].y), __float_as_int(terms[t].x));
          acc = fma(pv, (double)xs[tk[t] * nthr + tid], acc);
        }
        yv = (T)acc;
      } else {  // DF64
        if (end - beg == 0) {
          yv = (T)0;
        } else if (end - beg == 1) {
          yv = (T)(rowone[r] * (double)xs[tk[beg] * nthr + tid]);
        } else {
          float xh, xl, s, c;
          split_f64((double)xs[tk[beg] * nthr + tid], xh, xl, bad);
          df_mul(s, c, terms[beg].x, terms[beg].y, xh, xl);
          for (int t = beg + 1; t < end; ++t) {
            split_f64((double)xs[tk[t] * nthr + tid], xh, xl, bad);
            df_fma(s, c, terms[t].x, terms[t].y, xh, xl);
          }
          yv = (T)df_to_double(s, c);
        }
      }
      out[bo + offout[r]] = yv;
    }
  }
  if (bad && p.status) atomicOr(p.status, QSGB_DEV_RANGE);
}

template <typename T, int ARITH>
int launch_apply(const ApplyParams& p, cudaStream_t stream) {
  const int block = (p.kin <= 16) ? 128 : (p.kin <= 81 ? 64 : 32);
  SmemLayout L = make_layout(p.kin, p.kout, p.max_terms, block, sizeof(T));
  auto kern = apply_ptm_kernel<T, ARITH>;
  if (L.total > 48 * 1024) {
    if (L.total > 227 * 1024) return QSGB_ERR_UNSUPPORTED;
    QSGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.total));
  }
  int occ = 0;
  QSGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, block, L.total));
  if (occ < 1) return QSGB_ERR_UNSUPPORTED;
  const uint64_t need = (p.n_groups + block - 1) / block;
  const uint64_t cap = (uint64_t)sm_count() * occ;
  const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min(need, cap));
  kern<<<grid, block, L.total, stream>>>(p, L);
  return launch_status();
}

int apply_common(const void* in, void* out, const double* ptm, int64_t da_out, int64_t db_out,
                 int64_t da_in, int64_t db_in, int64_t X, int64_t Y, int64_t Z, int flags,
                 int dtype, int arith, int64_t max_terms, unsigned* status, void* stream) {
  if (!in || !out || !ptm) return QSGB_ERR_INVALID;
  if (in == out) return QSGB_ERR_INVALID;
  if (da_out < 1 || db_out < 1 || da_in < 1 || db_in < 1 || X < 1 || Y < 1 || Z < 1) return QSGB_ERR_INVALID;
  if (flags & ~(QSGB_PTM_SWAPPED | QSGB_PTM_TRANSPOSED | QSGB_PTM_HOST)) return QSGB_ERR_INVALID;
  const int64_t kin = da_in * db_in, kout = da_out * db_out;
  if ((flags & QSGB_PTM_HOST) && kin * kout > kMaxInline) return QSGB_ERR_UNSUPPORTED;
  if (kin > kMaxK || kout > kMaxK || kin * kout > kMaxEntries) return QSGB_ERR_UNSUPPORTED;
  if (max_terms < 1 || max_terms > kin * kout) max_terms = kin * kout;
  if (dtype != QSGB_F64 && dtype != QSGB_F32) return QSGB_ERR_INVALID;
  if (arith == QSGB_ARITH_AUTO) arith = (dtype == QSGB_F64) ? QSGB_ARITH_DF64 : QSGB_ARITH_F32;
  if (dtype == QSGB_F32 && arith != QSGB_ARITH_F32) return QSGB_ERR_INVALID;
  if (dtype == QSGB_F64 && arith == QSGB_ARITH_F32) return QSGB_ERR_INVALID;
  if (arith < QSGB_ARITH_DF64 || arith > QSGB_ARITH_F32) return QSGB_ERR_INVALID;

  ApplyParams p;
  p.in = in;
  p.out = out;
  if (flags & QSGB_PTM_HOST) {
    for (int64_t i = 0; i < kin * kout; ++i) p.ptm_inline[i] = ptm[i];
    p.ptm = nullptr;
  } else {
    p.ptm = ptm;
  }
  p.kin = (int)kin;
  p.kout = (int)kout;
  p.da_in = (int)da_in;
  p.db_in = (int)db_in;
  p.da_out = (int)da_out;
  p.db_out = (int)db_out;
  p.flags = flags & 3;
  p.max_terms = (int)max_terms;
  p.n_groups = (uint64_t)X * Y * Z;
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
  p.status = status;
  cudaStream_t s = as_stream(stream);
  if (dtype == QSGB_F32) return launch_apply<float, QSGB_ARITH_F32>(p, s);
  if (arith == QSGB_ARITH_F64) return launch_apply<double, QSGB_ARITH_F64>(p, s);
  return launch_apply<double, QSGB_ARITH_DF64>(p, s);
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

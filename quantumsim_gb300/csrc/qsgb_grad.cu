// Reverse-mode kernels for apply_ptm: the gradient with respect to the PTM,
//   dP[r, k] = sum over bystander groups g of g_out[g, r] * x_in[g, k],
// a tall-skinny (Kout x Kin) reduction over all groups.  (The gradient with
// respect to the state is apply_ptm with the transposed PTM, see
// qsgb_apply.cu.)  The reference has no differentiation; the operation is
// the adjoint of quantumsim/pauli_vectors/numpy.py:50-64.
//
// Stage 1: each block walks tiles of 32 groups, stages the tile's inputs and
// output-gradients in shared memory and accumulates its share of the Kout*Kin
// entries (FP64 accumulation; FP32 storage multiplies in FP32 inside a tile
// and carries the tile sums in FP64).  Stage 2 adds the per-block partials in
// a fixed order (deterministic).
#include <algorithm>

#include "qsgb_common.cuh"

namespace qsgb {
namespace {

constexpr int kTile = 32;
constexpr int kGradBlock = 256;
constexpr int kMaxPerThread = 26;  // ceil(6561 / 256)

struct GradParams {
  const void* x;
  const void* g;
  int kin, kout, db_in, db_out;
  uint64_t n_groups;
  FastDiv div_z, div_y;
  int64_t sxi, syi, sai, sbi;
  int64_t sxo, syo, sao, sbo;
};

unsigned grad_blocks(uint64_t n_groups) {
  const uint64_t tiles = (n_groups + kTile - 1) / kTile;
  return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(tiles, (uint64_t)sm_count() * 2));
}

template <typename T>
__global__ void __launch_bounds__(kGradBlock) grad_stage1(GradParams p, double* __restrict__ part) {
  extern __shared__ __align__(16) unsigned char smem[];
  T* xs = reinterpret_cast<T*>(smem);            // [kin][kTile]
  T* gs = xs + (size_t)p.kin * kTile;            // [kout][kTile]
  const T* __restrict__ X = static_cast<const T*>(p.x);
  const T* __restrict__ G = static_cast<const T*>(p.g);
  const int E = p.kin * p.kout;
  double acc[kMaxPerThread];
#pragma unroll
  for (int j = 0; j < kMaxPerThread; ++j) acc[j] = 0.0;
  const uint64_t n_tiles = (p.n_groups + kTile - 1) / kTile;
  const int rows = p.kin + p.kout;
  for (uint64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const uint64_t g0 = tile * kTile;
    __syncthreads();
    for (int i = threadIdx.x; i < rows * kTile; i += blockDim.x) {
      const int row = i / kTile, gg = i - row * kTile;
      const uint64_t g = g0 + gg;
      T v = (T)0;
      if (g < p.n_groups) {
        const uint64_t t1 = fdiv(g, p.div_z);
        const uint64_t z = g - t1 * p.div_z.d;
        const uint64_t x = fdiv(t1, p.div_y);
        const uint64_t y = t1 - x * p.div_y.d;
        if (row < p.kin) {
          const int ka = row / p.db_in, kb = row - ka * p.db_in;
          v = X[(int64_t)x * p.sxi + (int64_t)y * p.syi + (int64_t)z + ka * p.sai + kb * p.sbi];
        } else {
          const int r = row - p.kin;
          const int ra = r / p.db_out, rb = r - ra * p.db_out;
          v = G[(int64_t)x * p.sxo + (int64_t)y * p.syo + (int64_t)z + ra * p.sao + rb * p.sbo];
        }
      }
      xs[i] = v;  // xs and gs are contiguous: row < kin -> xs, else gs
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kMaxPerThread; ++j) {
      const int e = threadIdx.x + j * kGradBlock;
      if (e < E) {
        const int r = e / p.kin, k = e - r * p.kin;
        const T* gr = gs + r * kTile;
        const T* xk = xs + k * kTile;
        T s = (T)0;
#pragma unroll 8
        for (int gg = 0; gg < kTile; ++gg) s = fma(gr[gg], xk[gg], s);
        acc[j] += (double)s;
      }
    }
  }
#pragma unroll
  for (int j = 0; j < kMaxPerThread; ++j) {
    const int e = threadIdx.x + j * kGradBlock;
    if (e < E) part[(int64_t)blockIdx.x * E + e] = acc[j];
  }
}

__global__ void grad_stage2(const double* __restrict__ part, int nblocks, int E, double* __restrict__ out) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  double s = 0.0;
  for (int b = 0; b < nblocks; ++b) s += part[(int64_t)b * E + e];
  out[e] = s;
}

int grad_common(const void* x_in, const void* g_out, double* dptm, int64_t da_out, int64_t db_out, int64_t da_in,
                int64_t db_in, int64_t X, int64_t Y, int64_t Z, int dtype, void* scratch, int64_t scratch_bytes,
                void* stream) {
  if (!x_in || !g_out || !dptm) return QSGB_ERR_INVALID;
  if (da_out < 1 || db_out < 1 || da_in < 1 || db_in < 1 || X < 1 || Y < 1 || Z < 1) return QSGB_ERR_INVALID;
  if (dtype != QSGB_F64 && dtype != QSGB_F32) return QSGB_ERR_INVALID;
  const int64_t kin = da_in * db_in, kout = da_out * db_out;
  if (kin * kout > (int64_t)kMaxPerThread * kGradBlock) return QSGB_ERR_UNSUPPORTED;
  GradParams p;
  p.x = x_in;
  p.g = g_out;
  p.kin = (int)kin;
  p.kout = (int)kout;
  p.db_in = (int)db_in;
  p.db_out = (int)db_out;
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
  const unsigned nb = grad_blocks(p.n_groups);
  const int E = (int)(kin * kout);
  if (!scratch || scratch_bytes < (int64_t)nb * E * (int64_t)sizeof(double)) return QSGB_ERR_SCRATCH;
  cudaStream_t s = as_stream(stream);
  double* part = static_cast<double*>(scratch);
  if (dtype == QSGB_F64) {
    const size_t sm = (size_t)(kin + kout) * kTile * sizeof(double);
    if (sm > 48 * 1024)
      QSGB_CUDA_TRY(cudaFuncSetAttribute(grad_stage1<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    grad_stage1<double><<<nb, kGradBlock, sm, s>>>(p, part);
  } else {
    const size_t sm = (size_t)(kin + kout) * kTile * sizeof(float);
    if (sm > 48 * 1024)
      QSGB_CUDA_TRY(cudaFuncSetAttribute(grad_stage1<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    grad_stage1<float><<<nb, kGradBlock, sm, s>>>(p, part);
  }
  grad_stage2<<<(E + 255) / 256, 256, 0, s>>>(part, (int)nb, E, dptm);
  return launch_status();
}

}  // namespace
}  // namespace qsgb

extern "C" int64_t qsgb_ptm_grad_scratch_bytes(int64_t n_groups, int64_t k_out, int64_t k_in) {
  if (n_groups < 1 || k_out < 1 || k_in < 1) return 0;
  return (int64_t)qsgb::grad_blocks((uint64_t)n_groups) * k_out * k_in * (int64_t)sizeof(double);
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

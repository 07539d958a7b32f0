// Interface between the apply entry points and the tensor-core kernel for
// dense 16 x 16 PTMs (qsgb_tc.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "qsgb_common.cuh"

namespace qsgb {
namespace tc {

// digit planes of the split (six balanced base-1024 digits of a 57-bit
// fixed-point value plus sign)
constexpr int kDigits = 6;
constexpr unsigned long long kDigitBias =
    512ull * (1ull + (1ull << 10) + (1ull << 20) + (1ull << 30) + (1ull << 40) + (1ull << 50));

// The digit split shared by the tensor-core kernels (apply and PTM
// gradient): a fixed-point value relative to a block exponent, its six
// balanced base-1024 digits as exact FP16 numbers.
// Biased exponent of x as used for scaling (subnormals and zero count as 1)
// and its 53-bit significand (implicit bit included for normal numbers).
__device__ __forceinline__ unsigned exp_eff(unsigned hi) {
  const unsigned e = (hi >> 20) & 0x7ffu;
  return e == 0u ? 1u : e;
}

// F + B for input x = (hi, lo) against group exponent emax (biased, >= e):
// F = sign(x) * (m << 4) >> (emax - e), |F| < 2^57.
__device__ __forceinline__ unsigned long long fixed_biased(unsigned hi, unsigned lo, unsigned emax) {
  const unsigned e = (hi >> 20) & 0x7ffu;
  const unsigned mh = (hi & 0xfffffu) | (e != 0u ? 0x100000u : 0u);
  const unsigned long long m = ((unsigned long long)mh << 32 | lo) << 4;
  const unsigned s = emax - (e == 0u ? 1u : e);
  unsigned long long f = s < 64u ? (m >> s) : 0ull;
  if (hi & 0x80000000u) f = 0ull - f;
  return f + kDigitBias;
}

// FP16x2 register of digit plane j (bit position p = 10 (5 - j)) of two
// inputs: (v_a - 512, v_b - 512) built from 0x6400 | v = 1024 + v.
__device__ __forceinline__ unsigned digit_pair(unsigned long long ua, unsigned long long ub, int p) {
  const unsigned a = (unsigned)(ua >> p) & 0x3ffu;
  const unsigned b = (unsigned)(ub >> p) & 0x3ffu;
  const unsigned r = a | (b << 16) | 0x64006400u;
  unsigned out;
  asm("sub.rn.f16x2 %0, %1, %2;" : "=r"(out) : "r"(r), "r"(0x66006600u));  // - (1536, 1536)
  return out;
}

// d += a b for one m16n8k16 tile: FP16 operands, FP32 accumulators (the
// fragment layouts of mma.sync.aligned.m16n8k16.row.col)
__device__ __forceinline__ void mma16816(float* d, const unsigned* a, const unsigned* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

struct TcParams {
  const double* in;
  double* out;
  unsigned* status;
  uint64_t n_groups, n_tiles;
  FastDiv div_z, div_y;
  int64_t sxi, syi, sai, sbi;  // strides of (x, a, y, b) in elements; z stride 1
  int64_t sxo, syo, sao, sbo;
  int pair_store;  // groups 2c, 2c+1 are adjacent and 16-byte aligned
  int vec_z1;      // Z == 1 and both tensors 16-byte aligned: a group's
                   // runs along the last target move as 16-byte vectors
  const double* dptm;  // device PTM (launch_device): split by each block
  int dlayout;         // its storage (QSGB_PTM_SWAPPED / QSGB_PTM_TRANSPOSED bits)
  int row_exp[16];                                // Ep_r - 1022 - 54 per row
  unsigned short digits[kDigits][16][16];         // FP16 digit planes e_i[r][k]
  alignas(16) unsigned short bplanes[kDigits][256];  // the same in the shared-memory
                                                     // operand layout of tcgen05.mma
                                                     // (copied with 16-byte loads)
  double ptm[16][16];                             // the op matrix (FP64 fallback)
};

static_assert(offsetof(TcParams, bplanes) % 16 == 0, "16-byte loads of the operand planes");
static_assert(sizeof(TcParams) <= 32764, "kernel parameter limit");

// The op matrix is 16 x 16 without inf or nan.
bool eligible(const double* op, int kin, int kout);
// Apply the 16 x 16 op matrix `op` (row-major, rows = (ra, rb), columns =
// (ka, kb), qudit a more significant) to an FP64 tensor viewed as
// (X, 4, Y, 4, Z).
int launch(const double* op, const void* in, void* out, uint64_t X, uint64_t Y, uint64_t Z, unsigned* status,
           cudaStream_t stream);
// The same for a 16 x 16 PTM in device memory, stored in `layout`
// (QSGB_PTM_SWAPPED / QSGB_PTM_TRANSPOSED bits): every block reads and
// splits it (nothing is read on the host); inf or nan entries send every
// group to the native FP64 path.
int launch_device(const double* dptm, int layout, const void* in, void* out, uint64_t X, uint64_t Y, uint64_t Z,
                  unsigned* status, cudaStream_t stream);

}  // namespace tc
}  // namespace qsgb

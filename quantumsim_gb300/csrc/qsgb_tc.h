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

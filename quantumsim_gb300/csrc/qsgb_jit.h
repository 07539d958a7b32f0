// Interface between the apply entry points and the NVRTC-specialised kernels.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "qsgb_common.cuh"

namespace qsgb {
namespace jit {

enum { kModeZero = 0, kModeDP = 1, kModeDF = 2, kModeF32 = 3 };

// Everything that determines the generated code.
struct Spec {
  int kin, kout;
  int db_in, db_out;   // less significant target dims (index split k = ka*db + kb)
  bool pair;           // items are (z, z+1) pairs (16-byte accesses)
  bool f32;            // FP32 storage
  int vin, vout;       // 1, or 2 / 4: vector width of loads / stores along
                       // the less significant target (only when Z == 1)
  std::vector<int> mode;               // per output row
  std::vector<std::vector<int>> cols;  // per output row: input indices of its terms
  int n_coef() const;
};

// Run-time sizes (vector units when pair).
struct Geometry {
  const void* in;
  void* out;
  unsigned* status;
  unsigned long long n_items;
  FastDiv div_z, div_y;
  long long sxi, syi, sai, sbi, sxo, syo, sao, sbo;
};

bool available();
// Compile (or fetch from the cache) the kernel of `s`; optionally return its source.
int kernel_for(const Spec& s, cudaKernel_t* k, std::string* src_out);
// coef: one double per term in row order (dp: value; df: hi/lo float words;
// f32: float bits in the low word).
int launch(const Spec& s, const Geometry& g, const double* coef, cudaStream_t stream);

}  // namespace jit
}  // namespace qsgb

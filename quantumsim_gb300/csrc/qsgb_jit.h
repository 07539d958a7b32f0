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
  int lookahead;        // loads are emitted this many inputs ahead of first use
  int stage_warps;      // > 0: Z == 1 items staged in shared memory, warps per block
  bool stage_bulk;      // staged tiles are contiguous spans moved by bulk copies
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
// Spec and coefficient list (the layout of `launch`) of a host PTM stored in
// `layout` (QSGB_PTM_SWAPPED / QSGB_PTM_TRANSPOSED bits); z1: the view has
// Z == 1; contiguous: consecutive items' groups are adjacent, contiguous
// spans in both tensors (one qudit, or Y == 1) and both tensors start on a
// 16-byte boundary; vin / vout are the vector widths along the less
// significant target (1 unless Z == 1).  Returns false when the specialised
// path does not apply (more than 81 inputs or outputs, or more than 1024
// non-zero terms).
bool make_spec(const double* ptm_host, int da_out, int db_out, int da_in, int db_in, int layout, int dtype,
               int arith, bool pair, bool z1, bool contiguous, int vin, int vout, Spec& spec,
               std::vector<double>& coef);
// CUDA source of the kernel of `s`.
std::string source(const Spec& s);
// Compile (or fetch from the cache) the kernel of `s`; optionally return its source.
int kernel_for(const Spec& s, cudaKernel_t* k, std::string* src_out);
// coef: one double per term in row order (dp: value; df: hi/lo float words;
// f32: float bits in the low word).
int launch(const Spec& s, const Geometry& g, const double* coef, cudaStream_t stream);
// Compile (or fetch from the caches) the kernel of `s` without launching it.
int prepare(const Spec& s);
// ------------------------------------------------------------ fast path
// A specialisation request up to the PTM values: the geometry class and
// arithmetic (hdr) and the PTM's term mask in stored order.  Requests with
// equal keys get the same kernel and the same term list, so a cached entry
// serves them with a gather of the coefficients and a launch.
struct FastKey {
  unsigned char hdr[16];
  int nwords;
  unsigned long long mask[104];  // up to 81 x 81 entries
  bool operator==(const FastKey& o) const;
};
struct FastEntry {
  Spec spec;                      // final spec (group pairs or single groups)
  cudaKernel_t kern;
  std::vector<int> src;           // stored PTM index of each term, row order
  std::vector<unsigned char> kind;  // per term: kModeDP / kModeDF / kModeF32
};
// Cached entry of `key`, or nullptr.
const FastEntry* fast_find(const FastKey& key);
// Build and cache the entry of a compiled spec; `layout` is the stored PTM
// layout (QSGB_PTM_SWAPPED / QSGB_PTM_TRANSPOSED bits) and da/db the
// target dims.  Returns the cached entry (or nullptr if the kernel cannot
// be had).
const FastEntry* fast_insert(const FastKey& key, const Spec& spec, int layout, int da_out, int db_out, int da_in,
                             int db_in);
// Launch a cached entry with coefficients gathered from the host PTM.
int launch_entry(const FastEntry& e, const Geometry& g, const double* ptm_host, cudaStream_t stream);

// Generate the source of `s` and compile it with NVRTC without loading it
// (no device needed): QSGB_OK, QSGB_ERR_CUDA on a compile error,
// QSGB_ERR_UNSUPPORTED without NVRTC.
int compile_only(const Spec& s, std::string* src_out);

}  // namespace jit
}  // namespace qsgb

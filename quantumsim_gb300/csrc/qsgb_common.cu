// Library-wide helpers: status strings, ABI version, device SM count.
#include <cuda_runtime.h>

#include <mutex>
#include <vector>

#include "qsgb_common.cuh"

namespace qsgb {

int sm_count() {
  static int cache[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return kNumSMs;
  if (cache[dev] == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = kNumSMs;
    cache[dev] = n;
  }
  return cache[dev];
}

int allow_dynamic_smem(const void* func, int bytes) {
  if (bytes <= 48 * 1024) return QSGB_OK;
  struct Entry {
    const void* func;
    int dev, bytes;
  };
  static std::mutex mu;
  static std::vector<Entry> table;
  int dev = 0;
  QSGB_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  for (Entry& e : table) {
    if (e.func == func && e.dev == dev) {
      if (bytes <= e.bytes) return QSGB_OK;
      QSGB_CUDA_TRY(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
      e.bytes = bytes;
      return QSGB_OK;
    }
  }
  QSGB_CUDA_TRY(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  table.push_back({func, dev, bytes});
  return QSGB_OK;
}

int launch_status() {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? QSGB_OK : QSGB_ERR_CUDA;
}

}  // namespace qsgb

extern "C" int qsgb_abi_version(void) { return 2; }

extern "C" const char* qsgb_status_string(int status) {
  switch (status) {
    case QSGB_OK:
      return "ok";
    case QSGB_ERR_INVALID:
      return "invalid argument";
    case QSGB_ERR_CUDA:
      return "CUDA runtime error";
    case QSGB_ERR_UNSUPPORTED:
      return "unsupported shape or configuration";
    case QSGB_ERR_SCRATCH:
      return "scratch buffer too small";
    default:
      return "unknown status";
  }
}

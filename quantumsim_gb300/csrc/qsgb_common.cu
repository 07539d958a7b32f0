// Library-wide helpers: status strings, ABI version, device SM count.
#include <cuda_runtime.h>

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

// k_common.cu -- the library's device status word.
//
// Kernels that wait on shared-memory barriers with an iteration limit set a
// bit here when the limit expires (instead of hanging); ctgpu_sync() reads and
// clears it.  One word per device, shared by all handles of the process.
#include "ctgpu_internal.h"

namespace ctgpu {

__device__ unsigned int g_status_word;

unsigned int* status_pointer() {
  static unsigned int* ptrs[64] = {nullptr};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  if (!ptrs[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_status_word) != cudaSuccess) return nullptr;
    ptrs[dev] = static_cast<unsigned int*>(p);
  }
  return ptrs[dev];
}

cudaError_t status_read_and_clear(unsigned int* value) {
  unsigned int zero = 0;
  cudaError_t e = cudaMemcpyFromSymbol(value, g_status_word, sizeof(unsigned int));
  if (e != cudaSuccess) return e;
  if (*value) e = cudaMemcpyToSymbol(g_status_word, &zero, sizeof(unsigned int));
  return e;
}

}  // namespace ctgpu

// launch_util.h -- host helpers shared by the launchers.
#pragma once

#include <cuda_runtime.h>
#include "kblas_internal.h"

namespace kgb {

// Opt a kernel into more than 48 KB of dynamic shared memory (idempotent;
// the attribute call is cheap and capture-safe).
template <typename K>
static inline int set_smem(K kernel, size_t bytes) {
  if (bytes > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return cuda_check(e, "cudaFuncSetAttribute", __FILE__, __LINE__);
  }
  return KBLAS_Success;
}

static inline int max_smem(KBlasHandle *h) {
  ensure_device_props(h);
  return h->max_smem_optin > 0 ? h->max_smem_optin : 227 * 1024;
}

// Zero the per-matrix info words for the quick-return paths (n == 0).
static inline int zero_info(KBlasHandle *h, int *info, long long batch) {
  if (info && batch > 0) {
    cudaError_t e = cudaMemsetAsync(info, 0, (size_t)batch * sizeof(int), h->stream);
    if (e != cudaSuccess) return cuda_check(e, "cudaMemsetAsync", __FILE__, __LINE__);
  }
  return KBLAS_Success;
}

}  // namespace kgb

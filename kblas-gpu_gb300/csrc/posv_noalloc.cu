// posv_noalloc.cu -- mixed-precision uniform DPOSV that allocates no memory.
//
// No counterpart in the reference. kblasDposv_batch_mixed_strided needs a
// handle (creating one allocates) and a handle workspace (kblasAllocateWorkspace
// calls cudaMalloc). Some callers cannot do either when they need a solve:
//   * a host framework that owns all device memory through its own pool and
//     does not let a library call cudaMalloc behind its accounting;
//   * a latency-bound loop: cudaFree synchronises the whole device, and a
//     cudaMalloc can stall or fail in the middle of a run;
//   * a long-running service that must not fail later for lack of memory:
//     this routine's scratch is reserved once, when the library's device
//     image holding it is loaded, so a call cannot run out of memory.
// For them, kblasDposv_batch_mixed_strided_noalloc takes a CUDA stream instead
// of a handle and keeps its scratch in one fixed array of the library's device
// image. It runs the same persistent kernel as the handle-based routine and
// gives the same results (to within rounding: summation order of row sums).
//
// Limits and rules:
//   * the scratch array is KBLAS_POSV_NOALLOC_SCRATCH_BYTES (64 MiB) per
//     device; orders n > KBLAS_POSV_NOALLOC_MAX_N (256) are rejected with a
//     message and KBLAS_NotSupported. The persistent grid is cut, if needed,
//     to the number of per-CTA slots that fit (n = 256 on 152 SMs: 151);
//   * every call looks up the array's device address in the current context
//     (cudaGetSymbolAddress) and reads the device's properties; this stays
//     correct after cudaDeviceReset and under non-primary contexts. The first
//     call in a context loads that part of the library's image: make it
//     before any stream capture begins. The CUDA driver may also grow its own
//     per-context reservations (module images, local memory) the first time
//     a kernel runs; that is the driver's, not this routine's;
//   * every call on a device shares the one array. Its first 256 bytes are
//     the work counter, which must be zero when the kernel starts: each call
//     clears it with cudaMemsetAsync on its own stream before its launch. The
//     rest is per-CTA scratch, written before it is read, needing no clearing;
//   * therefore calls that overlap in time on one device (different streams,
//     or host threads without ordering between them) race on the counter and
//     the scratch and give wrong results. Order them: one stream, or events.
//     Calls in the same stream are ordered and safe.
#include <stdio.h>

#include "kblas.h"
#include "kblas_internal.h"

namespace kgb {

int mixed_uniform_fixed_scratch(cudaStream_t stream, int device, int sm_count, int smem_optin,
                                char side, char uplo, int m, int n, double *A, int lda,
                                long long sA, double *B, int ldb, long long sB, int batch,
                                int *info, int *iter, char *scratch, size_t scratch_bytes);

namespace {

// The scratch itself. This file holds no kernels, so (with CUDA's default
// lazy module loading) the array is reserved only when the set-up below first
// asks for its address, not when the rest of the library is used.
static __device__ __align__(256) char g_posv_scratch[KBLAS_POSV_NOALLOC_SCRATCH_BYTES];

// Looked up on every call, in the calling thread's current context. The
// address of a __device__ array belongs to the context that loaded the
// module: caching it per device ordinal would hand a later call a stale
// address after cudaDeviceReset, or the wrong one when the caller switches to
// a non-primary context on the same device. Once the module is loaded the
// lookup and the attribute queries allocate nothing.
struct DeviceSetup {
  char *scratch = nullptr;  // device address of g_posv_scratch in the current context
  int sm_count = 0;
  int smem_optin = 0;
};

int setup_device(int dev, DeviceSetup &s) {
  void *p = nullptr;
  // g_posv_scratch names the array here only as a handle for the lookup; the
  // host never dereferences it.
  cudaError_t e = cudaGetSymbolAddress(&p, g_posv_scratch);
  if (e != cudaSuccess) return cuda_check(e, "cudaGetSymbolAddress", __FILE__, __LINE__);
  e = cudaDeviceGetAttribute(&s.sm_count, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return cuda_check(e, "cudaDeviceGetAttribute", __FILE__, __LINE__);
  e = cudaDeviceGetAttribute(&s.smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return cuda_check(e, "cudaDeviceGetAttribute", __FILE__, __LINE__);
  s.scratch = static_cast<char *>(p);
  return KBLAS_Success;
}

}  // namespace
}  // namespace kgb

extern "C" int kblasDposv_batch_mixed_strided_noalloc(cudaStream_t stream, char side, char uplo,
                                                      const int m, const int n, double *A,
                                                      int lda, long strideA, double *B, int ldb,
                                                      long strideB, int batchCount,
                                                      int *info_array, int *iter_array) {
  using namespace kgb;
  if (n > KBLAS_POSV_NOALLOC_MAX_N) {
    fprintf(stderr,
            "kblasDposv_batch_mixed_strided_noalloc: order n = %d exceeds the limit %d of the "
            "fixed scratch array\n",
            n, KBLAS_POSV_NOALLOC_MAX_N);
    return KBLAS_NotSupported;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_check(e, "cudaGetDevice", __FILE__, __LINE__);
  DeviceSetup s;
  int st = setup_device(dev, s);
  if (st != KBLAS_Success) return st;
  return mixed_uniform_fixed_scratch(stream, dev, s.sm_count, s.smem_optin, side, uplo, m, n, A,
                                     lda, strideA, B, ldb, strideB, batchCount, info_array,
                                     iter_array, s.scratch, sizeof(g_posv_scratch));
}

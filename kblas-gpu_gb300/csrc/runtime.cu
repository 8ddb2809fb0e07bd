// runtime.cu -- handle lifecycle, streams, timer, workspace, error strings and
// the workspace queries of the batched Cholesky / triangular family.
//
// Replaces reference src/kblas_common.cu:35-265, src/kblas_struct.h:43-460 and
// the batch part of src/workspace_queries.cu:227-371 / workspace_queries.ch.
// The GB300 kernels of this library take their operands by base pointer +
// stride or straight from the caller's device pointer arrays, so the uniform
// routines need no workspace (the reference needs d_ptrs for its cuBLAS
// pointer-array GEMMs); only the mixed-precision and variable-size POSV
// request device data.
#include <stdlib.h>
#include <string.h>

#include "kblas_internal.h"
#include "workspace.h"

using namespace kgb;

namespace kgb {
int ensure_device_props(KBlasHandle *h) {
  if (h->sm_count > 0) return KBLAS_Success;
  cudaDeviceProp p;
  cudaError_t e = cudaGetDeviceProperties(&p, h->device_id);
  if (e != cudaSuccess) return cuda_check(e, "cudaGetDeviceProperties", __FILE__, __LINE__);
  h->sm_count = p.multiProcessorCount;
  h->max_smem_optin = (int)p.sharedMemPerBlockOptin;
  return KBLAS_Success;
}
}  // namespace kgb

// Frees what a partly created handle holds (events, status word) and the handle.
static void discard_handle(KBlasHandle *h) {
  if (h->ev_start) cudaEventDestroy(h->ev_start);
  if (h->ev_end) cudaEventDestroy(h->ev_end);
  if (h->d_status) cudaFree(h->d_status);
  delete h;
}

extern "C" {

int kblasCreate(kblasHandle_t *handle) {
  if (!handle) return KBLAS_Error_WrongInput;
  KBlasHandle *h = new KBlasHandle();
  cudaError_t e = cudaGetDevice(&h->device_id);
  if (e != cudaSuccess) {
    delete h;
    *handle = nullptr;
    return cuda_check(e, "cudaGetDevice", __FILE__, __LINE__);
  }
  if (cudaEventCreate(&h->ev_start) != cudaSuccess || cudaEventCreate(&h->ev_end) != cudaSuccess ||
      cudaMalloc((void **)&h->d_status, sizeof(int)) != cudaSuccess ||
      cudaMemset(h->d_status, 0, sizeof(int)) != cudaSuccess) {
    discard_handle(h);
    *handle = nullptr;
    return KBLAS_CUDA_Error;
  }
  int st = ensure_device_props(h);
  if (st != KBLAS_Success) {
    discard_handle(h);
    *handle = nullptr;
    return st;
  }
  *handle = h;
  return KBLAS_Success;
}

int kblasFreeWorkspace(kblasHandle_t h) {
  if (!h) return KBLAS_Error_NotInitialized;
  int ret = KBLAS_Success;
  if (h->ws.h_data) cudaFreeHost(h->ws.h_data);
  if (h->ws.h_ptrs) cudaFreeHost(h->ws.h_ptrs);
  if (h->ws.d_data && cudaFree(h->ws.d_data) != cudaSuccess) ret = KBLAS_Error_Deallocation;
  if (h->ws.d_ptrs && cudaFree(h->ws.d_ptrs) != cudaSuccess) ret = KBLAS_Error_Deallocation;
  h->ws = KBlasWorkspace();
  return ret;
}

int kblasDestroy(kblasHandle_t *handle) {
  if (!handle || !*handle) return KBLAS_Error_NotInitialized;
  KBlasHandle *h = *handle;
  kblasFreeWorkspace(h);
  for (int i = 0; i < h->nStreams; i++) cudaStreamDestroy(h->streams[i]);
  if (h->cublas) cublasDestroy(h->cublas);
  if (h->ev_start) cudaEventDestroy(h->ev_start);
  if (h->ev_end) cudaEventDestroy(h->ev_end);
  if (h->d_status) cudaFree(h->d_status);
  delete h;
  *handle = nullptr;
  return KBLAS_Success;
}

void kblasTimerTic(kblasHandle_t h) {
  if (!h) return;
  h->end_recorded = false;
  cudaEventRecord(h->ev_start, h->stream);
}

void kblasTimerRecordEnd(kblasHandle_t h) {
  if (!h) return;
  cudaEventRecord(h->ev_end, h->stream);
  h->end_recorded = true;
}

double kblasTimerToc(kblasHandle_t h) {
  if (!h) return 0.0;
  if (!h->end_recorded) cudaEventRecord(h->ev_end, h->stream);
  h->end_recorded = false;
  cudaEventSynchronize(h->ev_end);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, h->ev_start, h->ev_end);
  return (double)ms;
}

int kblasCreateStreams(kblasHandle_t h, int nStreams) {
  if (!h) return KBLAS_Error_NotInitialized;
  if (nStreams > KBLAS_NSTREAMS || nStreams < 0) return KBLAS_WrongConfig;
  for (int i = h->nStreams; i < nStreams; i++) {
    if (cudaStreamCreateWithFlags(&h->streams[i], cudaStreamNonBlocking) != cudaSuccess)
      return KBLAS_CUDA_Error;
    h->nStreams = i + 1;
  }
  return KBLAS_Success;
}

cudaStream_t kblasGetStream(kblasHandle_t h) { return h ? h->stream : (cudaStream_t)0; }

void kblasSetStream(kblasHandle_t h, cudaStream_t stream) {
  if (!h) return;
  h->stream = stream;
  if (h->cublas) cublasSetStream(h->cublas, stream);
}

cublasHandle_t kblasGetCublasHandle(kblasHandle_t h) {
  if (!h) return nullptr;
  if (!h->cublas) {
    if (cublasCreate(&h->cublas) != CUBLAS_STATUS_SUCCESS) {
      h->cublas = nullptr;
      return nullptr;
    }
    cublasSetStream(h->cublas, h->stream);
  }
  return h->cublas;
}

int kblasEnableMagma(kblasHandle_t h) {
  (void)h;
  fprintf(stderr, "ERROR: this KBLAS build has no MAGMA support\n");
  return KBLAS_Error_NotInitialized;
}

const char *kblasGetErrorString(int error) {
  switch (error) {
    case KBLAS_Success: return "KBLAS: success";
    case KBLAS_UnknownError: return "KBLAS: unknown error";
    case KBLAS_NotSupported: return "Operation not supported";
    case KBLAS_NotImplemented: return "Operation not implemented yet";
    case KBLAS_cuBLAS_Error: return "cuBLAS error";
    case KBLAS_WrongConfig: return "Wrong compilation flags configuration";
    case KBLAS_CUDA_Error: return "CUDA error";
    case KBLAS_InsufficientWorkspace: return "Insufficient workspace supplied to function";
    case KBLAS_Error_Allocation: return "Error allocating memory";
    case KBLAS_Error_Deallocation: return "Error de-allocating memory";
    case KBLAS_Error_NotInitialized: return "KBLAS handle not initialized";
    case KBLAS_Error_WrongInput: return "One of input parameter's value is wrong";
    case KBLAS_MAGMA_Error: return "MAGMA error";
    case KBLAS_SVD_NoConvergence: return "SVD-gram operation did not converge.";
    case KBLAS_Error_Timeout: return "A bounded device-side wait for the tensor cores ran out";
    default: return "unknown KBLAS error code";
  }
}

int kblasAllocateWorkspace(kblasHandle_t h) {
  if (!h) return KBLAS_Error_NotInitialized;
  KBlasWorkspace &w = h->ws;
  KBlasWorkspaceState &req = w.requested;
  KBlasWorkspaceState &al = w.allocated;
  if (req.h_data_bytes > al.h_data_bytes) {
    if (w.h_data) cudaFreeHost(w.h_data);
    w.h_data = nullptr;
    if (cudaHostAlloc(&w.h_data, req.h_data_bytes, cudaHostAllocPortable) != cudaSuccess) {
      al.h_data_bytes = 0;
      return KBLAS_Error_Allocation;
    }
    al.h_data_bytes = req.h_data_bytes;
  }
  if (req.h_ptrs_bytes > al.h_ptrs_bytes) {
    if (w.h_ptrs) cudaFreeHost(w.h_ptrs);
    w.h_ptrs = nullptr;
    if (cudaHostAlloc((void **)&w.h_ptrs, req.h_ptrs_bytes, cudaHostAllocPortable) != cudaSuccess) {
      al.h_ptrs_bytes = 0;
      return KBLAS_Error_Allocation;
    }
    al.h_ptrs_bytes = req.h_ptrs_bytes;
  }
  if (req.d_data_bytes > al.d_data_bytes) {
    if (w.d_data && cudaFree(w.d_data) != cudaSuccess) return KBLAS_Error_Deallocation;
    w.d_data = nullptr;
    if (cudaMalloc(&w.d_data, req.d_data_bytes) != cudaSuccess) {
      al.d_data_bytes = 0;
      return KBLAS_Error_Allocation;
    }
    al.d_data_bytes = req.d_data_bytes;
  }
  if (req.d_ptrs_bytes > al.d_ptrs_bytes) {
    if (w.d_ptrs && cudaFree(w.d_ptrs) != cudaSuccess) return KBLAS_Error_Deallocation;
    w.d_ptrs = nullptr;
    if (cudaMalloc((void **)&w.d_ptrs, req.d_ptrs_bytes) != cudaSuccess) {
      al.d_ptrs_bytes = 0;
      return KBLAS_Error_Allocation;
    }
    al.d_ptrs_bytes = req.d_ptrs_bytes;
  }
  req.reset();
  return KBLAS_Success;
}

int kblas_roundup(int x, int y) { return (x + y - 1) / y * y; }

// The handle's device status word is set by the mixed-precision persistent
// kernels when a bounded wait for their tensor-core MMAs runs out (the kernel
// then stops without writing results). It stays set until read here; reading
// clears it.
int kblasGetDeviceStatus(kblasHandle_t h) {
  if (!h) return KBLAS_Error_NotInitialized;
  int s = 0;
  if (cudaMemcpyAsync(&s, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
      cudaMemsetAsync(h->d_status, 0, sizeof(int), h->stream) != cudaSuccess ||
      cudaStreamSynchronize(h->stream) != cudaSuccess)
    return KBLAS_CUDA_Error;
  return s == 0 ? KBLAS_Success : KBLAS_Error_Timeout;
}

// ---------------------------------------------------------------------------
// Workspace queries. The uniform routines need no workspace; the calls only
// exist so KBLAS callers link and run unchanged.
// ---------------------------------------------------------------------------
void kblas_syrk_batch_wsquery(kblasHandle_t, const int, int) {}
void kblas_trsm_batch_wsquery(kblasHandle_t, char, int, int, int) {}
void kblas_trsm_batch_strided_wsquery(kblasHandle_t, char, int, int, int) {}
void kblas_trmm_batch_wsquery(kblasHandle_t, char, int, int, int) {}
void kblas_trmm_batch_strided_wsquery(kblasHandle_t, char, int, int, int) {}
// GEMM and the variable-size GEMM / SYRK need none either (reference
// workspace_queries.cu:203-253 asks for cuBLAS pointer arrays and MAGMA's
// size maxima). The variable-size TRSM recomputes max_m / max_n on the device
// when the caller passes neither (reference workspace_queries.cu:268-278).
void kblas_gemm_batch_strided_wsquery(kblasHandle_t, int) {}
void kblas_gemm_batch_nonuniform_wsquery(kblasHandle_t) {}
void kblas_syrk_batch_nonuniform_wsquery(kblasHandle_t) {}
void kblas_trsm_batch_nonuniform_wsquery(kblasHandle_t h) {
  if (!h) return;
  KBlasWorkspaceState need;
  need.d_data_bytes = 2 * sizeof(int);
  h->ws.requested.pad(need);
}
// POTRF / POTRS / POSV: the double-precision routines of order 33..1024 run
// on the persistent panel path when this workspace is allocated (else on the
// one-launch blocked kernel, which needs none).
static void request_fp64_uniform(kblasHandle_t h, int n, int batch) {
  if (!h) return;
  KBlasWorkspaceState need;
  need.d_data_bytes = kgb::fp64_uniform_ws_bytes(h, n, batch);
  h->ws.requested.pad(need);
}
void kblas_potrf_batch_wsquery(kblasHandle_t h, const int n, int batch) { request_fp64_uniform(h, n, batch); }
void kblas_potrf_batch_strided_wsquery(kblasHandle_t h, const int n, int batch) {
  request_fp64_uniform(h, n, batch);
}
void kblas_potrs_batch_wsquery(kblasHandle_t h, const int m, const int n, int batch) {
  (void)m;
  request_fp64_uniform(h, n, batch);
}
void kblas_potrs_batch_strided_wsquery(kblasHandle_t h, const int m, const int n, int batch) {
  (void)m;
  request_fp64_uniform(h, n, batch);
}
void kblas_posv_batch_wsquery(kblasHandle_t h, char side, const int m, const int n, int batch) {
  (void)side;
  (void)m;
  request_fp64_uniform(h, n, batch);
}
void kblas_posv_batch_strided_wsquery(kblasHandle_t h, char side, const int m, const int n,
                                      int batch) {
  (void)side;
  (void)m;
  request_fp64_uniform(h, n, batch);
}

void kblas_posv_batch_mixed_wsquery(kblasHandle_t h, char side, const int m, const int n,
                                    int batchCount) {
  (void)side;
  (void)m;
  if (!h) return;
  KBlasWorkspaceState need;
  need.d_data_bytes = kgb::mixed_posv_ws_bytes(h, n, batchCount);
  h->ws.requested.pad(need);
}

void kblas_posv_vbatch_wsquery(kblasHandle_t h, const int max_n, int batchCount) {
  if (!h) return;
  KBlasWorkspaceState need;
  const size_t a = kgb::vbatch_ws_bytes(h, max_n, batchCount, true);
  const size_t b = kgb::vbatch_ws_bytes(h, max_n, batchCount, false);
  need.d_data_bytes = a > b ? a : b;
  h->ws.requested.pad(need);
}

}  // extern "C"

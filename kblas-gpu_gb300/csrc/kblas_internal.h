// kblas_internal.h -- handle, workspace and argument-checking internals.
//
// The handle mirrors the reference's KBlasHandle / KBlasWorkspace
// (src/kblas_struct.h:43-460): a stream, an event timer, and a four-part
// workspace (host data, host pointers, device data, device pointers) with
// "requested" and "allocated" states. Workspace queries raise the requested
// state; kblasAllocateWorkspace grows the allocation to it; every routine
// checks its own need against the allocated state and returns
// KBLAS_InsufficientWorkspace (-6) when it is short.
#pragma once

#include <cuda_runtime.h>
#include <stdio.h>
#include <stdint.h>
#include <cublas_v2.h>

#include "kblas.h"

struct KBlasWorkspaceState {
  size_t h_data_bytes = 0, h_ptrs_bytes = 0;
  size_t d_data_bytes = 0, d_ptrs_bytes = 0;
  void reset() { h_data_bytes = h_ptrs_bytes = d_data_bytes = d_ptrs_bytes = 0; }
  void pad(const KBlasWorkspaceState &o) {
    if (o.h_data_bytes > h_data_bytes) h_data_bytes = o.h_data_bytes;
    if (o.h_ptrs_bytes > h_ptrs_bytes) h_ptrs_bytes = o.h_ptrs_bytes;
    if (o.d_data_bytes > d_data_bytes) d_data_bytes = o.d_data_bytes;
    if (o.d_ptrs_bytes > d_ptrs_bytes) d_ptrs_bytes = o.d_ptrs_bytes;
  }
  bool fits_in(const KBlasWorkspaceState &alloc) const {
    return h_data_bytes <= alloc.h_data_bytes && h_ptrs_bytes <= alloc.h_ptrs_bytes &&
           d_data_bytes <= alloc.d_data_bytes && d_ptrs_bytes <= alloc.d_ptrs_bytes;
  }
};

struct KBlasWorkspace {
  void *h_data = nullptr;
  void **h_ptrs = nullptr;
  void *d_data = nullptr;
  void **d_ptrs = nullptr;
  KBlasWorkspaceState allocated, requested;
};

struct KBlasHandle {
  int device_id = 0;
  cudaStream_t stream = 0;
  cudaStream_t streams[KBLAS_NSTREAMS];
  int nStreams = 0;
  cudaEvent_t ev_start = nullptr, ev_end = nullptr;
  bool end_recorded = false;
  cublasHandle_t cublas = nullptr;  // created on first kblasGetCublasHandle()
  KBlasWorkspace ws;
  int *d_status = nullptr;          // device status word of persistent launches
  int sm_count = 0;
  int max_smem_optin = 0;
};

namespace kgb {

// 256-byte aligned bump allocation inside the device data workspace.
static inline size_t align_up(size_t x, size_t a = 256) { return (x + a - 1) / a * a; }

// Report a launch / runtime error the way the reference does (file:line on
// stderr, src/kblas_error.h:31-40) and map it to a KBLAS code.
static inline int cuda_check(cudaError_t e, const char *what, const char *file, int line) {
  if (e != cudaSuccess) {
    fprintf(stderr, "CUDA runtime error: %s (%d) in %s at %s:%d\n", cudaGetErrorString(e), (int)e,
            what, file, line);
    return KBLAS_CUDA_Error;
  }
  return KBLAS_Success;
}

#define KGB_LAUNCH_CHECK(what)                                                   \
  do {                                                                           \
    cudaError_t e_ = cudaGetLastError();                                         \
    if (e_ != cudaSuccess) return kgb::cuda_check(e_, what, __FILE__, __LINE__); \
  } while (0)

static inline bool is_flag(char c, char a, char b) { return c == a || c == b; }
static inline bool is_lower(char c) { return c == 'L' || c == 'l'; }
static inline bool is_upper(char c) { return c == 'U' || c == 'u'; }
static inline bool is_left(char c) { return c == 'L' || c == 'l'; }
static inline bool is_right(char c) { return c == 'R' || c == 'r'; }
static inline bool is_trans(char c) { return c == 'T' || c == 't' || c == 'C' || c == 'c'; }
static inline bool is_notrans(char c) { return c == 'N' || c == 'n'; }
static inline bool is_unit(char c) { return c == 'U' || c == 'u'; }
static inline bool is_nonunit(char c) { return c == 'N' || c == 'n'; }

int ensure_device_props(KBlasHandle *h);

}  // namespace kgb

// probe.cu -- arithmetic-pipe throughput probes (libkblas_probe.so).
//
// The roofline of the FP64 kernels is the FP64 FMA rate of the part, which
// the pool's measured-peak file does not record (it holds the HBM copy rate
// and the bf16 tensor rate). These probes measure it live: every thread runs
// ILP independent FMA chains; the result is written out so nothing is
// optimised away. Used by bench.py for the roofline denominators.
#include <cuda_runtime.h>

template <typename T, int ILP>
__global__ void fma_chain_kernel(T *out, int iters, T a, T b) {
  T x[ILP];
#pragma unroll
  for (int i = 0; i < ILP; i++) x[i] = T(threadIdx.x + i) * T(1e-3);
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int i = 0; i < ILP; i++) x[i] = x[i] * a + b;
  }
  T s = 0;
#pragma unroll
  for (int i = 0; i < ILP; i++) s += x[i];
  if (s == T(1234.5)) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// The same chains run only by lanes < active of each warp (the others skip
// them under a branch): the kernel time shows whether the FP64 pipe spends
// an issue slot on the lanes that do not take part.
template <typename T, int ILP>
__global__ void fma_chain_lanes_kernel(T *out, int iters, int active, T a, T b) {
  T x[ILP];
#pragma unroll
  for (int i = 0; i < ILP; i++) x[i] = T(threadIdx.x + i) * T(1e-3);
  if ((int)(threadIdx.x & 31) < active) {
    for (int it = 0; it < iters; it++) {
#pragma unroll
      for (int i = 0; i < ILP; i++) x[i] = x[i] * a + b;
    }
  }
  T s = 0;
#pragma unroll
  for (int i = 0; i < ILP; i++) s += x[i];
  if (s == T(1234.5)) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T, int ILP>
static float run_chain(int blocks, int threads, int iters, void *scratch) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_chain_kernel<T, ILP><<<blocks, threads>>>((T *)scratch, iters, T(0.999999), T(1e-7));
  cudaEventRecord(e0);
  fma_chain_kernel<T, ILP><<<blocks, threads>>>((T *)scratch, iters, T(0.999999), T(1e-7));
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms;
}

extern "C" {

// FMA throughput probe. prec = 64 or 32; ilp in {1, 2, 4, 8}. Returns the
// kernel time in ms (FLOP = 2 * blocks * threads * iters * ilp), or -1.
float kblas_probe_fma(int prec, int blocks, int threads, int iters, int ilp, void *scratch) {
  if (prec == 64) {
    switch (ilp) {
      case 1: return run_chain<double, 1>(blocks, threads, iters, scratch);
      case 2: return run_chain<double, 2>(blocks, threads, iters, scratch);
      case 4: return run_chain<double, 4>(blocks, threads, iters, scratch);
      case 8: return run_chain<double, 8>(blocks, threads, iters, scratch);
    }
  } else {
    switch (ilp) {
      case 1: return run_chain<float, 1>(blocks, threads, iters, scratch);
      case 2: return run_chain<float, 2>(blocks, threads, iters, scratch);
      case 4: return run_chain<float, 4>(blocks, threads, iters, scratch);
      case 8: return run_chain<float, 8>(blocks, threads, iters, scratch);
    }
  }
  return -1.f;
}

// FP64 chains (ILP 4) run by `active` lanes of every warp; returns the kernel
// time in ms (one warm-up launch, one timed), or -1.
float kblas_probe_fma64_lanes(int blocks, int threads, int iters, int active, void *scratch) {
  if (active < 1 || active > 32) return -1.f;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_chain_lanes_kernel<double, 4><<<blocks, threads>>>((double *)scratch, iters, active, 0.999999, 1e-7);
  cudaEventRecord(e0);
  fma_chain_lanes_kernel<double, 4><<<blocks, threads>>>((double *)scratch, iters, active, 0.999999, 1e-7);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms;
}

}  // extern "C"

// device_util.cuh -- small device-side building blocks shared by all kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace kgb {

// Batch operand accessors: a strided batch (base + b * stride) or a device
// array of per-matrix device pointers. Kernels are templated on these so one
// kernel body serves both API forms.
template <typename T>
struct Strided {
  T *base;
  long long stride;
  __device__ __forceinline__ T *get(long long b) const { return base + b * stride; }
};

template <typename T>
struct PtrArr {
  T *const *arr;
  __device__ __forceinline__ T *get(long long b) const { return arr[b]; }
};

// Per-matrix integer arguments: N values shared by all matrices, or N device
// arrays read at the matrix index.
template <int N>
struct DimsU {
  int v[N];
  __device__ __forceinline__ void get(long long, int (&o)[N]) const {
#pragma unroll
    for (int i = 0; i < N; i++) o[i] = v[i];
  }
};
template <int N>
struct DimsV {
  const int *p[N];
  __device__ __forceinline__ void get(long long b, int (&o)[N]) const {
#pragma unroll
    for (int i = 0; i < N; i++) o[i] = p[i][b];
  }
};

// 1/sqrt(d) and sqrt(d) for a positive pivot d: one reciprocal square root
// (CUDA's rsqrt / rsqrtf) and one multiply, instead of a square root and a
// division per column.
__device__ __forceinline__ void pivot_rs(double d, double &s, double &r) {
  r = rsqrt(d);
  s = d * r;
}
__device__ __forceinline__ void pivot_rs(float d, float &s, float &r) {
  r = rsqrtf(d);
  s = d * r;
}

// Packed lower-triangular storage, column-major: element (i, k), i >= k, of an
// n x n matrix sits at coff(k, n) + i - k.
__device__ __forceinline__ int coff(int k, int n) { return k * n - ((k * (k - 1)) >> 1); }

// Step a row-major enumeration of the lower triangle (ii >= kk) forward by
// `step` elements: used to deal the elements of a trailing triangle out to
// the lanes of a team without a lookup table.
__device__ __forceinline__ void tri_advance(int &ii, int &kk, int step) {
  kk += step;
  while (kk > ii) {
    kk -= ii + 1;
    ii++;
  }
}

// FP64 -> FP32 conversion with a power-of-two scale 2^k applied exactly,
// done on the IEEE-754 bit patterns with integer operations only (the
// hardware conversion shares the scarce FP64 pipe on this part). Rounds to
// nearest (ties away from zero), flushes results below the FP32 normal range
// to signed zero and returns signed infinity above it; a NaN input gives NaN.
__device__ __forceinline__ float f64_to_f32_scaled(double a, int k) {
  const unsigned hi = (unsigned)__double2hiint(a);
  const unsigned lo = (unsigned)__double2loint(a);
  const unsigned sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7FF);
  if (e == 0x7FF) return __int_as_float((int)(sign | 0x7F800000u | ((hi & 0xFFFFFu) | lo ? 0x400000u : 0u)));
  const int fe = e - 1023 + 127 + k;
  if (e == 0 || fe <= 0) return __int_as_float((int)sign);
  if (fe >= 255) return __int_as_float((int)(sign | 0x7F800000u));
  unsigned bits = ((unsigned)fe << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29);
  bits += (lo >> 28) & 1u;  // carry into the exponent is the correct rounding
  return __int_as_float((int)(sign | bits));
}

template <typename T>
__device__ __forceinline__ bool is_pos_pivot(T d) {
  return d > T(0);  // false for NaN
}

// sqrt of an accepted pivot, correctly rounded (FP32 through FP64).
__device__ __forceinline__ double pivot_sqrt(double d) { return sqrt(d); }
__device__ __forceinline__ float pivot_sqrt(float d) { return (float)sqrt((double)d); }

__device__ __forceinline__ double shfl_xor_t(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ float shfl_xor_t(float v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }

}  // namespace kgb

// the complex value type and its overloads of the helpers above
#include "cplx.cuh"

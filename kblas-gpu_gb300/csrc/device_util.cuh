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

template <typename T>
__device__ __forceinline__ bool is_pos_pivot(T d) {
  return d > T(0);  // false for NaN
}

}  // namespace kgb

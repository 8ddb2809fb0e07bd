// cplx.cuh -- the complex value type of the C / Z routines.
//
// cx<R> is layout-compatible with cuFloatComplex / cuDoubleComplex (float2 /
// double2: same size, same alignment), so the entry points reinterpret the
// caller's arrays. The arithmetic is the plain field arithmetic the kernels
// need (+, -, *, /, unary minus); nothing conjugates: the reference's complex
// batch routines are the complex-symmetric forms (A = L L^T, op = transpose,
// SYRK = A A^T), src/batch_triangular/Xpotrf_batch_kernels.cuh:37-78 and the
// complex-symmetric test matrices of testing/testing_helper.cu:405-414.
#pragma once

#include <cuda_runtime.h>

namespace kgb {

template <typename R>
struct __align__(2 * sizeof(R)) cx {
  R x, y;
  cx() = default;
  __host__ __device__ constexpr cx(R re) : x(re), y(R(0)) {}
  __host__ __device__ constexpr cx(R re, R im) : x(re), y(im) {}
  __host__ __device__ cx &operator+=(const cx &o) { x += o.x; y += o.y; return *this; }
  __host__ __device__ cx &operator-=(const cx &o) { x -= o.x; y -= o.y; return *this; }
  __host__ __device__ cx &operator*=(const cx &o) { *this = *this * o; return *this; }
  friend __host__ __device__ cx operator+(cx a, const cx &b) { return cx(a.x + b.x, a.y + b.y); }
  friend __host__ __device__ cx operator-(cx a, const cx &b) { return cx(a.x - b.x, a.y - b.y); }
  friend __host__ __device__ cx operator-(const cx &a) { return cx(-a.x, -a.y); }
  friend __host__ __device__ cx operator*(const cx &a, const cx &b) {
    return cx(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
  }
  // Smith's algorithm (R. L. Smith, CACM 5(8), 1962): scales by the larger
  // component of the divisor, avoiding the overflow of |b|^2.
  friend __host__ __device__ cx operator/(const cx &a, const cx &b) {
    if (fabs(b.x) >= fabs(b.y)) {
      const R r = b.y / b.x, d = b.x + b.y * r;
      return cx((a.x + a.y * r) / d, (a.y - a.x * r) / d);
    }
    const R r = b.x / b.y, d = b.y + b.x * r;
    return cx((a.x * r + a.y) / d, (a.y * r - a.x) / d);
  }
  friend __host__ __device__ bool operator==(const cx &a, const cx &b) { return a.x == b.x && a.y == b.y; }
  friend __host__ __device__ bool operator!=(const cx &a, const cx &b) { return !(a == b); }
};

using cxf = cx<float>;
using cxd = cx<double>;

template <typename T> struct is_cx { static constexpr bool value = false; };
template <typename R> struct is_cx<cx<R>> { static constexpr bool value = true; };

// Principal square root, the textbook formula: t = sqrt((|x| + |z|) / 2);
// x >= 0: (t, y / 2t), else (|y| / 2t, sign(y) t). |z| by CUDA's hypot.
template <typename R>
__host__ __device__ inline cx<R> csqrt_principal(const cx<R> &z) {
  if (z.x == R(0) && z.y == R(0)) return cx<R>(R(0), R(0));
  const R t = sqrt((fabs(z.x) + hypot(z.x, z.y)) * R(0.5));
  if (z.x >= R(0)) return cx<R>(t, z.y / (R(2) * t));
  return cx<R>(fabs(z.y) / (R(2) * t), copysign(t, z.y));
}

// Complex-symmetric Cholesky pivot: usable unless zero or not finite (there
// is no definiteness test without conjugation).
template <typename R>
__device__ __forceinline__ bool is_pos_pivot(const cx<R> &d) {
  return (d.x != R(0) || d.y != R(0)) && isfinite(d.x) && isfinite(d.y);
}

// sqrt(d) and 1/sqrt(d) of a pivot.
template <typename R>
__device__ __forceinline__ void pivot_rs(const cx<R> &d, cx<R> &s, cx<R> &r) {
  s = csqrt_principal(d);
  r = cx<R>(R(1)) / s;
}

template <typename R>
__device__ __forceinline__ cx<R> pivot_sqrt(const cx<R> &d) { return csqrt_principal(d); }

// Warp shuffles of a complex value (both parts).
template <typename R>
__device__ __forceinline__ cx<R> shfl_xor_t(const cx<R> &v, int o) {
  return cx<R>(__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o));
}

}  // namespace kgb

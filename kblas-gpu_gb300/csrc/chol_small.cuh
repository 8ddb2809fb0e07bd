// chol_small.cuh -- register-resident POSV pieces for n <= 32: a segment of W
// lanes (W in {8, 16, 32}, W >= n) owns one system, lane i owns row i, columns
// are broadcast with width-W warp shuffles, and 32/W systems share a warp.
// The factor is written row-major to shared memory (stride W + 1, conflict
// free) by warp_chol_rot; both triangular sweeps read it from there.
#pragma once

#include "chol_panel.cuh"

namespace kgb {

// Stage row `lane` of the lower triangle of A (column-major, lda): FP32 with
// the power-of-two scaling of the mixed path, or plain. Loads of one column
// are coalesced across the lanes.
template <typename T, int W, bool SCALE>
__device__ __forceinline__ void small_load(int n, const double *A, int lda, int sh_lane,
                                           bool active, T (&v)[32])
{
  const int lane = threadIdx.x & (W - 1);
  double a[W];
#pragma unroll
  for (int c = 0; c < W; c++)
    a[c] = (active && c < n && c <= lane && lane < n) ? A[(size_t)lane + (size_t)c * lda] : 0.0;
#pragma unroll
  for (int c = 0; c < 32; c++) {
    if (c < W) {
      const int sh_c = __shfl_sync(0xffffffffu, sh_lane, c, W);
      v[c] = SCALE ? (T)f64_to_f32_scaled(a[c], sh_lane + sh_c) : (T)a[c];
    } else {
      v[c] = T(0);
    }
  }
}

// y := L^{-T} L^{-1} y, one entry of y per lane. Ls: row-major L (stride
// W + 1); rinv: per-column reciprocal pivots (shared).
template <typename T, int W>
__device__ __forceinline__ T small_llt_solve(int n, const T *Ls, const T *rinv, T y)
{
  const int lane = threadIdx.x & (W - 1);
  for (int c = 0; c < n; c++) {
    if (lane == c) y *= rinv[c];
    const T yc = __shfl_sync(0xffffffffu, y, c, W);
    if (lane > c && lane < n) y -= Ls[lane * (W + 1) + c] * yc;
  }
  for (int c = n - 1; c >= 0; c--) {
    if (lane == c) y *= rinv[c];
    const T xc = __shfl_sync(0xffffffffu, y, c, W);
    if (lane < c) y -= Ls[c * (W + 1) + lane] * xc;
  }
  return y;
}

// Width-W transpose-sum: on entry lane i holds v[j] for j < W; on exit lane j
// holds sum_i v[j] over the W lanes of the segment.
template <int W>
__device__ __forceinline__ double seg_transpose_sum(double (&v)[W])
{
  const int lane = threadIdx.x & (W - 1);
#pragma unroll
  for (int lvl = W / 2; lvl >= 1; lvl >>= 1) {
    const bool hi = (lane & lvl) != 0;
#pragma unroll
    for (int k = 0; k < lvl; k++) {
      const double send = hi ? v[k] : v[k + lvl];
      const double keep = hi ? v[k + lvl] : v[k];
      v[k] = keep + __shfl_xor_sync(0xffffffffu, send, lvl, W);
    }
  }
  return v[0];
}

// FP64 residual r_i = b_i - sum_j a_ij x_j for lane i; A symmetric from its
// lower triangle. Lane i loads row i of the lower triangle (coalesced per
// column); the mirrored upper part is summed per column with one
// transpose-sum, so every load is coalesced and every FMA is useful.
template <int W>
__device__ __forceinline__ double small_residual(int n, const double *A, int lda, double b,
                                                 double x, bool active)
{
  const int lane = threadIdx.x & (W - 1);
  double a[W];
#pragma unroll
  for (int j = 0; j < W; j++)
    a[j] = (active && lane < n && j <= lane) ? A[(size_t)lane + (size_t)j * lda] : 0.0;
  double s0 = 0.0, s1 = 0.0;
#pragma unroll
  for (int j = 0; j < W; j++) {
    const double xj = __shfl_sync(0xffffffffu, x, j, W);
    if (j & 1) s1 += a[j] * xj;
    else s0 += a[j] * xj;
    a[j] = (j < lane) ? a[j] * x : 0.0;
  }
  const double cs = seg_transpose_sum<W>(a);
  return b - (s0 + s1) - cs;
}

}  // namespace kgb

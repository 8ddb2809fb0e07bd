// chol_reg.cuh -- batched POTRS of uniform order n <= 32 (real types): each
// factor lives in the registers of a W-lane segment of a warp (W in {8, 16,
// 32}, W >= n; 32 / W systems per warp), lane i holding row i of L.
//
//  * load: when the factor is 16-byte aligned and lda * sizeof(T) is a
//    multiple of 16, the segment reads the lower triangle column by column in
//    coalesced 128-bit chunks (2 doubles / 4 floats, rows 0..round_up(n) - 1
//    of each column, which lie inside the column's lda rows) into a staging
//    square in shared memory, from which lane i takes its row; otherwise lane
//    i reads its row with coalesced scalar loads, column by column;
//  * solve: X L L^T = B for each right-hand side (a row of B), forward with
//    the rows in registers, backward with a row-major copy of L in shared
//    memory (stride W + 1), one width-W shuffle and one FMA per column.
//
// The factorization is not done this way: with a row per lane, only the rows
// below column c do useful work at column c, and an FP64 instruction costs
// its issue slot whether or not its lane is predicated off, so the team
// kernel (chol_kernels.cuh), which deals the trailing elements out to every
// lane, is faster for POTRF and POSV.
//
// Reference behaviour covered: POTRS src/batch_triangular/
// Xpotrs_batch_drivers.cuh:33-171 (side R, lower); the reference's own n <= 32
// register kernel is Xpotrf_batch_kernels.cuh:37-78.
#pragma once

#include "device_util.cuh"

namespace kgb {

// Shared memory per matrix: a W x (W + 1) square (staging with column stride
// W, later the row-major factor with row stride W + 1).
template <typename T, int W>
__host__ __device__ constexpr int reg_square_elems() {
  return W * (W + 1);
}

// Load the lower triangle of an n x n matrix (column-major, lda) into the
// rows v of the segment's lanes; sq: the segment's W x (W + 1) square. vec:
// the 128-bit path is allowed for this matrix. Every lane of the warp calls
// this (its __syncwarp needs the whole warp).
template <typename T, int W>
__device__ __forceinline__ void seg_load(const T *A, int lda, int n, bool active, bool vec, T *sq,
                                         T (&v)[W]) {
  constexpr int VEC = 16 / (int)sizeof(T);
  const int lane = threadIdx.x & (W - 1);
  if (vec) {
    const int nch = (n + VEC - 1) / VEC;  // chunks per column
    for (int q = lane; q < n * nch; q += W) {
      const int c = q / nch, g = q - c * nch;
      if (VEC * g + VEC - 1 < c) continue;  // wholly above the diagonal
      const T *src = A + (size_t)c * lda + VEC * g;
      if (sizeof(T) == 8)
        *reinterpret_cast<double2 *>(sq + c * W + VEC * g) = *reinterpret_cast<const double2 *>(src);
      else
        *reinterpret_cast<float4 *>(sq + c * W + VEC * g) = *reinterpret_cast<const float4 *>(src);
    }
    __syncwarp();
#pragma unroll
    for (int c = 0; c < W; c++) v[c] = (c < n && c <= lane && lane < n) ? sq[c * W + lane] : T(0);
  } else {
#pragma unroll
    for (int c = 0; c < W; c++)
      v[c] = (active && c < n && c <= lane && lane < n) ? A[(size_t)lane + (size_t)c * lda] : T(0);
  }
}

// X L L^T = B for rows [0, m) of B (m x n, column-major, ldb): forward with
// the rows v (v[c] = L(lane, c)), backward with the row-major copy Lr (stride
// W + 1); ri = 1 / L(lane, lane).
template <typename T, int W>
__device__ __forceinline__ void seg_solve(T *B, int ldb, int m, int n, bool go, const T (&v)[W],
                                          const T *Lr, T ri, int m_hi) {
  const int lane = threadIdx.x & (W - 1);
  for (int r = 0; r < m_hi; r++) {
    const bool act = go && r < m && lane < n;
    T y = act ? B[(size_t)r + (size_t)lane * ldb] : T(0);
#pragma unroll
    for (int c = 0; c < W; c++) {
      if (c < n) {
        if (lane == c) y *= ri;
        const T yc = __shfl_sync(0xffffffffu, y, c, W);
        if (lane > c) y -= v[c] * yc;
      }
    }
#pragma unroll
    for (int c = W - 1; c >= 0; c--) {
      if (c < n) {
        if (lane == c) y *= ri;
        const T xc = __shfl_sync(0xffffffffu, y, c, W);
        if (lane < c) y -= Lr[c * (W + 1) + lane] * xc;
      }
    }
    if (act) B[(size_t)r + (size_t)lane * ldb] = y;
  }
}

template <typename T, int W, int NT, class AccA, class AccB>
__global__ void __launch_bounds__(NT)
potrs_reg_kernel(int n, int m, AccA A, int lda, AccB B, int ldb, long long batch)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & (W - 1);
  const int seg = threadIdx.x / W;  // segment index in the CTA
  const long long b = (long long)blockIdx.x * (NT / W) + seg;
  const bool active = b < batch;
  T *sq = reinterpret_cast<T *>(smem_raw) + (size_t)seg * reg_square_elems<T, W>();
  const T *Ag = active ? A.get(b) : nullptr;
  const bool vec = active && ((reinterpret_cast<uintptr_t>(Ag) & 15u) == 0) &&
                   ((lda * (int)sizeof(T)) % 16 == 0);
  T v[W];
  seg_load<T, W>(Ag, lda, n, active, vec, sq, v);
  // the diagonal of L and the row-major copy for the backward sweep
  T diag = T(0);
#pragma unroll
  for (int c = 0; c < W; c++)
    if (c == lane) diag = v[c];
  const T ri = (lane < n) ? T(1) / diag : T(0);
  __syncwarp();
#pragma unroll
  for (int c = 0; c < W; c++)
    if (c <= lane) sq[lane * (W + 1) + c] = v[c];
  __syncwarp();
  // m is uniform: every segment of the warp runs the same number of solves
  seg_solve<T, W>(active ? B.get(b) : nullptr, ldb, m, n, active, v, sq, ri, m);
}

}  // namespace kgb

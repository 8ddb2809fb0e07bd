// gemm_tile.cuh -- the C-tile engine behind batched GEMM and the
// variable-size SYRK: one CTA of GT_NT threads computes GT x GT tiles of
//   C := alpha * op(A) * op(B) + beta * C
// staging GT_K-deep slabs of op(A) and op(B) through shared memory, each
// thread holding a 4 x 4 block of C in registers (rows 4ty..4ty+3, columns
// 4tx..4tx+3, read from shared memory as two 4-wide vectors per k step).
//
// A tile clipped by the matrix edge skips the FMAs of threads whose 4 x 4
// block lies wholly outside it: with rows split 16 per warp, a matrix of at
// most 16 rows leaves the second warp idle instead of issuing wasted FP64
// instructions (the FP64 pipe, 2 DFMA per clock per SM, bounds this kernel).
//
// Grids are (matrices, tile slots): the CTA at (b, y) takes tiles y,
// y + gridDim.y, ... of matrix b, so one launch serves uniform and
// variable-size batches and needs no per-matrix prefix sums; per-matrix
// sizes come through a dims accessor (DimsU: the same for every matrix,
// DimsV: device arrays indexed by matrix).
#pragma once

#include "device_util.cuh"
#include "kblas_internal.h"

namespace kgb {

constexpr int GT = 32;      // C tile edge
constexpr int GT_K = 16;    // k slab staged per step
constexpr int GT_NT = 64;   // 8 x 8 threads, 4 x 4 elements each
constexpr int GT_PAD = 4;   // keeps every row 16-byte aligned for 4-wide loads

template <typename T>
struct GemmSmem {
  T a[GT_K][GT + GT_PAD];   // a[l][i] = op(A)(I0 + i, l0 + l)
  T b[GT_K][GT + GT_PAD];   // b[l][j] = op(B)(l0 + l, J0 + j)
};

// Which part of the C tile is written: all of it, the lower (gi >= gj) or
// the upper (gi <= gj) triangle.
enum { TILE_FULL = 0, TILE_LOWER = 1, TILE_UPPER = 2 };

template <typename T>
struct TileJob {
  const T *A;
  const T *B;
  T *C;
  int lda, ldb, ldc;
  int m, n, k;      // C is m x n, op(A) m x k, op(B) k x n
  int ta, tb;       // op(A) = A^T if ta; op(B) = B^T if tb
  int I0, J0;       // tile origin in C
  int part;         // TILE_FULL / TILE_LOWER / TILE_UPPER
};

__device__ __forceinline__ void ld4(const float *p, float (&v)[4]) {
  const float4 q = *reinterpret_cast<const float4 *>(p);
  v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
}
__device__ __forceinline__ void ld4(const double *p, double (&v)[4]) {
  const double2 q0 = *reinterpret_cast<const double2 *>(p);
  const double2 q1 = *reinterpret_cast<const double2 *>(p + 2);
  v[0] = q0.x; v[1] = q0.y; v[2] = q1.x; v[3] = q1.y;
}

__device__ __forceinline__ void ld4(const cx<float> *p, cx<float> (&v)[4]) {
  const float4 q0 = *reinterpret_cast<const float4 *>(p);
  const float4 q1 = *reinterpret_cast<const float4 *>(p + 2);
  v[0] = cx<float>(q0.x, q0.y); v[1] = cx<float>(q0.z, q0.w);
  v[2] = cx<float>(q1.x, q1.y); v[3] = cx<float>(q1.z, q1.w);
}
__device__ __forceinline__ void ld4(const cx<double> *p, cx<double> (&v)[4]) {
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const double2 q = *reinterpret_cast<const double2 *>(p + i);
    v[i] = cx<double>(q.x, q.y);
  }
}

// One C tile. Every thread of the CTA calls it (it holds barriers). BLAS
// semantics: op(A), op(B) are not read when alpha == 0 or k == 0, C is not
// read when beta == 0.
template <typename T>
__device__ void gemm_tile(const TileJob<T> &j, T alpha, T beta, GemmSmem<T> &s) {
  const int tid = threadIdx.x, tx = tid & 7, ty = tid >> 3;
  const int r0 = 4 * ty, c0 = 4 * tx;
  const bool active = r0 < j.m - j.I0 && c0 < j.n - j.J0;
  T acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int c = 0; c < 4; c++) acc[a][c] = T(0);

  const bool prod = alpha != T(0) && j.k > 0;
  const int kend = prod ? j.k : 0;
  for (int l0 = 0; l0 < kend; l0 += GT_K) {
    for (int idx = tid; idx < GT_K * GT; idx += GT_NT) {
      // op(A)(i, l): A(i, l) is contiguous along i, A^T's along l
      int i, l;
      if (j.ta) { l = idx % GT_K; i = idx / GT_K; } else { i = idx % GT; l = idx / GT; }
      int gi = j.I0 + i, gl = l0 + l;
      T v = T(0);
      if (gi < j.m && gl < j.k)
        v = j.ta ? j.A[(size_t)gl + (size_t)gi * j.lda] : j.A[(size_t)gi + (size_t)gl * j.lda];
      s.a[l][i] = v;
      // op(B)(l, jj): B(l, jj) is contiguous along l, B^T's along jj
      int jj;
      if (j.tb) { jj = idx % GT; l = idx / GT; } else { l = idx % GT_K; jj = idx / GT_K; }
      const int gj = j.J0 + jj;
      gl = l0 + l;
      T w = T(0);
      if (gj < j.n && gl < j.k)
        w = j.tb ? j.B[(size_t)gj + (size_t)gl * j.ldb] : j.B[(size_t)gl + (size_t)gj * j.ldb];
      s.b[l][jj] = w;
    }
    __syncthreads();
    if (active) {
#pragma unroll
      for (int l = 0; l < GT_K; l++) {
        T av[4], bv[4];
        ld4(&s.a[l][r0], av);
        ld4(&s.b[l][c0], bv);
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
          for (int c = 0; c < 4; c++) acc[a][c] += av[a] * bv[c];
      }
    }
    __syncthreads();
  }
  if (!active) return;
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const int gi = j.I0 + r0 + a, gj = j.J0 + c0 + c;
      if (gi >= j.m || gj >= j.n) continue;
      if ((j.part == TILE_LOWER && gi < gj) || (j.part == TILE_UPPER && gi > gj)) continue;
      T *p = j.C + (size_t)gi + (size_t)gj * j.ldc;
      const T old = (beta == T(0)) ? T(0) : beta * *p;
      *p = prod ? alpha * acc[a][c] + old : old;
    }
}

// Tile t of the triangle of an nt x nt tile grid, enumerated row-major over
// the lower triangle (ti >= tj).
__device__ __forceinline__ void tri_tile(int t, int &ti, int &tj) {
  // ti = floor((sqrt(8t + 1) - 1) / 2), corrected for rounding
  int r = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
  while ((r + 1) * (r + 2) / 2 <= t) r++;
  while (r * (r + 1) / 2 > t) r--;
  ti = r;
  tj = t - r * (r + 1) / 2;
}

// C := alpha op(A) op(A)^T + beta C on one triangle; dims = (m, k, lda, ldc)
template <typename T, class AccA, class AccC, class Dims>
__global__ void __launch_bounds__(GT_NT)
syrk_batch_kernel(int upper, int trans, T alpha, AccA A, T beta, AccC Cm, Dims dims,
                  long long batch)
{
  __shared__ __align__(16) GemmSmem<T> s;
  const long long mat = blockIdx.x;
  if (mat >= batch) return;
  int d[4];
  dims.get(mat, d);
  const int m = d[0];
  if (m <= 0) return;
  const int nt = (m + GT - 1) / GT;
  TileJob<T> j;
  j.A = j.B = A.get(mat);
  j.C = Cm.get(mat);
  j.m = j.n = m;
  j.k = d[1];
  j.lda = j.ldb = d[2];
  j.ldc = d[3];
  j.ta = trans;    // op(A)
  j.tb = !trans;   // op(B) = op(A)^T
  j.part = upper ? TILE_UPPER : TILE_LOWER;
  for (int t = blockIdx.y; t < nt * (nt + 1) / 2; t += gridDim.y) {
    int ti, tj;
    tri_tile(t, ti, tj);
    j.I0 = (upper ? tj : ti) * GT;
    j.J0 = (upper ? ti : tj) * GT;
    gemm_tile<T>(j, alpha, beta, s);
  }
}

// Tile slots per matrix: enough CTAs to fill the GPU several times over
// when the batch alone does not, never more than the largest matrix has
// tiles (the hint; unknown -> capped at 64 slots).
static inline unsigned tile_slots(KBlasHandle *h, long long batch, long long tiles_hint) {
  ensure_device_props(h);
  const long long target = (long long)(h->sm_count > 0 ? h->sm_count : 152) * 16;
  long long y = (target + batch - 1) / batch;
  const long long cap = tiles_hint > 0 ? tiles_hint : 64;
  if (y > cap) y = cap;
  if (y < 1) y = 1;
  if (y > 65535) y = 65535;
  return (unsigned)y;
}

}  // namespace kgb

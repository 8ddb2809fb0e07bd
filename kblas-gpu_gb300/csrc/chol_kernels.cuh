// chol_kernels.cuh -- batched Cholesky factor / solve kernels (uniform n).
//
// Two size classes, both written for the GB300 balance of pipes: FP64 FMA is
// the scarce resource (an order of magnitude below the FP32 pipe), while
// shared memory, integer and shuffle throughput are plentiful. Both kernels
// therefore deal out FMA work so that nearly every issued FP64 instruction
// does useful work on every lane, and amortise the per-column pivot
// (reciprocal square root) over several matrices per warp.
//
//  * chol_team_kernel (n <= 32): a team of G lanes owns one matrix; a warp
//    holds 32/G matrices. The lower triangle lives in shared memory in packed
//    column-major form. Right-looking: per column, the team leader computes
//    the pivot, the team scales the column, then the (n-j-1)(n-j)/2 elements
//    of the trailing triangle are dealt round-robin to the G lanes.
//  * chol_blocked_kernel (n > 32): one CTA per matrix, left-looking by panels
//    of NB columns. Each panel (rows J..n-1) is staged in shared memory,
//    updated with the already final columns (read from the matrix itself,
//    i.e. from L2, with one row per thread and NB register accumulators),
//    its diagonal block is factored by one warp, the rows below are solved
//    against it, and the panel is written back.
//
// MODE 0: POTRF (factor, write L, info).
// MODE 1: POSV  (factor, write L, info, then solve X*A = B for the m rows of
//                B if the factorization succeeded; B is untouched otherwise).
// MODE 2: POTRS (A holds L on entry; solve X*L*L^T = B).
//
// Reference behaviour covered: POTRF = src/batch_triangular/
// Xpotrf_batch_drivers.cuh:31-135 (lower only), POTRS = Xpotrs_batch_drivers
// .cuh:33-171 (side R, lower), POSV = Xposv_batch_drivers.cuh:33-114, with
// LAPACK info semantics (first non-positive / NaN pivot, 1-based).
#pragma once

#include "device_util.cuh"

namespace kgb {

enum { MODE_POTRF = 0, MODE_POSV = 1, MODE_POTRS = 2 };

// Shared memory bytes of one team (matrix + reciprocals + RHS chunk).
template <typename T>
__host__ __device__ __forceinline__ size_t team_smem_elems(int n, int rc) {
  return (size_t)n * (n + 1) / 2 + n + (size_t)rc * n;
}

template <typename T, int G, int NT, int MODE, class AccA, class AccB>
__global__ void __launch_bounds__(NT)
chol_team_kernel(int n, int m, int rc, AccA A, int lda, AccB B, int ldb, long long batch, int *info)
{
  static_assert(32 % G == 0, "team size must divide the warp");
  constexpr int TPB = NT / G;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int team = threadIdx.x / G;
  const int r = threadIdx.x % G;
  const long long b = (long long)blockIdx.x * TPB + team;
  const bool active = b < batch;

  const size_t per_team = team_smem_elems<T>(n, rc);
  T *sL = reinterpret_cast<T *>(smem_raw) + (size_t)team * per_team;
  T *sR = sL + (size_t)n * (n + 1) / 2;
  T *sY = sR + n;

  T *Ag = active ? A.get(b) : nullptr;

  // ---- stage the lower triangle (column by column, lanes over rows) ----
  if (active) {
    for (int k = 0; k < n; k++) {
      const T *col = Ag + (size_t)k * lda;
      T *dst = sL + coff(k, n) - k;
      for (int i = k + r; i < n; i += G) dst[i] = col[i];
    }
  }
  __syncwarp();

  int failed = 0;  // 1-based failing column, identical on every lane of a team
  if (MODE != MODE_POTRS) {
    for (int j = 0; j < n; j++) {
      T *cj = sL + coff(j, n) - j;  // column j, indexed by row
      if (r == 0 && active && !failed) {
        T d = cj[j];
        if (is_pos_pivot(d)) {
          T s, rr;
          pivot_rs(d, s, rr);
          cj[j] = s;
          sR[j] = rr;
        } else {
          sR[j] = T(0);  // marks the failure for the other lanes of the team
        }
      }
      __syncwarp();
      // every lane of the team reads the verdict of column j
      if (active && !failed && !is_pos_pivot(sR[j])) failed = j + 1;
      if (active && !failed) {
        const T rj = sR[j];
        for (int i = j + 1 + r; i < n; i += G) cj[i] *= rj;
      }
      __syncwarp();
      if (active && !failed) {
        const int mm = n - 1 - j;  // trailing order
        int ii = 0, kk = r;
        tri_advance(ii, kk, 0);
        while (ii < mm) {
          const int i = j + 1 + ii, k = j + 1 + kk;
          T *ck = sL + coff(k, n) - k;
          ck[i] -= cj[i] * cj[k];
          tri_advance(ii, kk, G);
        }
      }
      __syncwarp();
    }
    if (active) {
      // write back the lower triangle (the strict upper triangle is untouched)
      for (int k = 0; k < n; k++) {
        T *col = Ag + (size_t)k * lda;
        const T *src = sL + coff(k, n) - k;
        for (int i = k + r; i < n; i += G) col[i] = src[i];
      }
      if (r == 0 && info) info[b] = failed;
    }
  } else {
    if (active)
      for (int j = r; j < n; j += G) sR[j] = T(1) / sL[coff(j, n)];
    __syncwarp();
  }

  if (MODE == MODE_POTRF) return;

  // ---- solve X * L * L^T = B for the m rows of B, rc rows at a time ----
  T *Bg = active ? B.get(b) : nullptr;
  const bool solve = active && !failed;
  for (int r0 = 0; r0 < m; r0 += rc) {
    const int mc = min(rc, m - r0);
    if (solve)
      for (int q = r; q < mc * n; q += G) {
        const int rr = q % mc, jj = q / mc;
        sY[rr * n + jj] = Bg[(r0 + rr) + (size_t)jj * ldb];
      }
    __syncwarp();
    // forward: L y^T = b^T
    for (int j = 0; j < n; j++) {
      if (solve)
        for (int rr = r; rr < mc; rr += G) sY[rr * n + j] *= sR[j];
      __syncwarp();
      if (solve) {
        const T *cj = sL + coff(j, n) - j;
        const int cnt = n - 1 - j;
        for (int q = r; q < mc * cnt; q += G) {
          const int rr = q % mc, i = j + 1 + q / mc;
          sY[rr * n + i] -= cj[i] * sY[rr * n + j];
        }
      }
      __syncwarp();
    }
    // backward: L^T x^T = y^T
    for (int j = n - 1; j >= 0; j--) {
      if (solve)
        for (int rr = r; rr < mc; rr += G) sY[rr * n + j] *= sR[j];
      __syncwarp();
      if (solve) {
        for (int q = r; q < mc * j; q += G) {
          const int rr = q % mc, i = q / mc;  // i < j
          sY[rr * n + i] -= sL[coff(i, n) + (j - i)] * sY[rr * n + j];
        }
      }
      __syncwarp();
    }
    if (solve)
      for (int q = r; q < mc * n; q += G) {
        const int rr = q % mc, jj = q / mc;
        Bg[(r0 + rr) + (size_t)jj * ldb] = sY[rr * n + jj];
      }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// Blocked (panel) kernel, one CTA per matrix, any n.
// Shared memory: panel P (ldp = n rows x NB), the NB x KC chunk of L rows
// J..J+jb-1, the n reciprocal pivots, and an rc x n RHS chunk.
// ---------------------------------------------------------------------------
template <typename T, int NB, int KC>
__host__ __device__ __forceinline__ size_t blocked_smem_elems(int n, int rc) {
  return (size_t)n * NB + (size_t)NB * KC + n + (size_t)rc * n;
}

template <typename T, int NB, int KC, int NT, int MODE, class AccA, class AccB>
__global__ void __launch_bounds__(NT)
chol_blocked_kernel(int n, int m, int rc, AccA A, int lda, AccB B, int ldb, long long batch, int *info)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *sP = reinterpret_cast<T *>(smem_raw);  // n x NB, ld = n (row index relative to J)
  T *sK = sP + (size_t)n * NB;              // NB x KC, ld = NB
  T *sR = sK + (size_t)NB * KC;             // n
  T *sY = sR + n;                           // rc x n
  __shared__ int s_fail;

  const long long b = blockIdx.x;
  if (b >= batch) return;
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  T *Ag = A.get(b);
  if (tid == 0) s_fail = 0;
  __syncthreads();

  if (MODE != MODE_POTRS) {
    for (int J = 0; J < n; J += NB) {
      const int jb = min(NB, n - J);
      const int rows = n - J;
      // 1. stage panel rows J..n-1, columns J..J+jb-1 (lower part)
      for (int idx = tid; idx < rows * jb; idx += NT) {
        const int c = idx / rows, i = idx - c * rows;
        if (i >= c) sP[i + (size_t)c * n] = Ag[(size_t)(J + i) + (size_t)(J + c) * lda];
      }
      // 2. panel -= L(J:n, 0:J) * L(J:J+jb, 0:J)^T, KC columns of L at a time
      for (int k0 = 0; k0 < J; k0 += KC) {
        const int kc = min(KC, J - k0);
        __syncthreads();
        for (int idx = tid; idx < jb * kc; idx += NT) {
          const int kk = idx / jb, c = idx - kk * jb;
          sK[c + kk * NB] = Ag[(size_t)(J + c) + (size_t)(k0 + kk) * lda];
        }
        __syncthreads();
        for (int i = tid; i < rows; i += NT) {
          T acc[NB];
#pragma unroll
          for (int c = 0; c < NB; c++) acc[c] = T(0);
          const T *arow = Ag + (size_t)(J + i) + (size_t)k0 * lda;
          for (int kk = 0; kk < kc; kk++) {
            const T a = arow[(size_t)kk * lda];
#pragma unroll
            for (int c = 0; c < NB; c++) acc[c] += a * sK[c + kk * NB];
          }
          const int cmax = min(jb, i + 1);
#pragma unroll
          for (int c = 0; c < NB; c++)
            if (c < cmax) sP[i + (size_t)c * n] -= acc[c];
        }
      }
      __syncthreads();
      // 3. factor the jb x jb diagonal block with warp 0
      if (warp == 0) {
        int fail = 0;
        for (int c = 0; c < jb; c++) {
          T *pc = sP + (size_t)c * n;
          if (lane == 0) {
            T d = pc[c];
            if (is_pos_pivot(d)) {
              T s, rr;
              pivot_rs(d, s, rr);
              pc[c] = s;
              sR[J + c] = rr;
            } else {
              sR[J + c] = T(0);
            }
          }
          __syncwarp();
          const T rr = sR[J + c];
          if (!is_pos_pivot(rr)) {
            fail = J + c + 1;
            break;
          }
          for (int i = c + 1 + lane; i < jb; i += 32) pc[i] *= rr;
          __syncwarp();
          for (int i = c + 1 + lane; i < jb; i += 32) {
            const T lic = pc[i];
            for (int k = c + 1; k <= i; k++) sP[i + (size_t)k * n] -= lic * pc[k];
          }
          __syncwarp();
        }
        if (lane == 0 && fail) s_fail = fail;
      }
      __syncthreads();
      const int fail = s_fail;
      // 4. rows below the diagonal block: x * L_JJ^T = p  (row by row)
      if (!fail) {
        for (int i = jb + tid; i < rows; i += NT) {
          for (int c = 0; c < jb; c++) {
            T x = sP[i + (size_t)c * n];
            for (int cc = 0; cc < c; cc++) x -= sP[i + (size_t)cc * n] * sP[c + (size_t)cc * n];
            sP[i + (size_t)c * n] = x * sR[J + c];
          }
        }
      }
      __syncthreads();
      // 5. write the panel back (lower part); on failure the failing column
      //    keeps the non-positive pivot in its diagonal entry
      const int jw = fail ? min(jb, fail - J) : jb;
      for (int idx = tid; idx < rows * jw; idx += NT) {
        const int c = idx / rows, i = idx - c * rows;
        if (i >= c) Ag[(size_t)(J + i) + (size_t)(J + c) * lda] = sP[i + (size_t)c * n];
      }
      __syncthreads();
      if (fail) break;
    }
    if (tid == 0 && info) info[b] = s_fail;
  } else {
    for (int j = tid; j < n; j += NT) sR[j] = T(1) / Ag[(size_t)j + (size_t)j * lda];
    __syncthreads();
  }

  if (MODE == MODE_POTRF) return;
  if (s_fail) return;

  // ---- solve X * L * L^T = B; L read from the matrix (L2 resident) ----
  T *Bg = B.get(b);
  for (int r0 = 0; r0 < m; r0 += rc) {
    const int mc = min(rc, m - r0);
    __syncthreads();
    for (int q = tid; q < mc * n; q += NT) {
      const int rr = q % mc, jj = q / mc;
      sY[rr * n + jj] = Bg[(r0 + rr) + (size_t)jj * ldb];
    }
    __syncthreads();
    for (int j = 0; j < n; j++) {
      for (int rr = tid; rr < mc; rr += NT) sY[rr * n + j] *= sR[j];
      __syncthreads();
      const T *cj = Ag + (size_t)j * lda;
      const int cnt = n - 1 - j;
      for (int q = tid; q < mc * cnt; q += NT) {
        const int i = j + 1 + q / mc, rr = q % mc;
        sY[rr * n + i] -= cj[i] * sY[rr * n + j];
      }
      __syncthreads();
    }
    for (int j = n - 1; j >= 0; j--) {
      for (int rr = tid; rr < mc; rr += NT) sY[rr * n + j] *= sR[j];
      __syncthreads();
      const T *cj = Ag + (size_t)j * lda;  // L(j, i) = A(j, i) for i < j: row j
      for (int q = tid; q < mc * j; q += NT) {
        const int i = q / mc, rr = q % mc;
        sY[rr * n + i] -= Ag[(size_t)j + (size_t)i * lda] * sY[rr * n + j];
      }
      (void)cj;
      __syncthreads();
    }
    for (int q = tid; q < mc * n; q += NT) {
      const int rr = q % mc, jj = q / mc;
      Bg[(r0 + rr) + (size_t)jj * ldb] = sY[rr * n + jj];
    }
  }
}

}  // namespace kgb

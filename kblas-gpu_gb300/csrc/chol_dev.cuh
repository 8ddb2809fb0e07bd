// chol_dev.cuh -- team-level Cholesky factor / solve / residual routines used
// by the persistent mixed-precision and variable-size POSV kernels.
//
// The factor lives in packed column-major lower storage (coff(), device_util
// .cuh) behind a generic pointer, so the same code runs with the factor in
// shared memory or, when it does not fit, in a per-CTA global scratch slot
// (L2 resident while the CTA works on it).
#pragma once

#include "device_util.cuh"
#include "team.cuh"

namespace kgb {

// Packed element (i, k), i >= k.
template <typename T>
__device__ __forceinline__ T &PL(T *Lp, int n, int i, int k) {
  return Lp[coff(k, n) + (i - k)];
}

// Right-looking Cholesky of the packed lower matrix Lp (order n), in place.
// A pivot d <= tol (or NaN, or +inf) stops the factorization; returns the
// 1-based failing column, 0 on success. rinv[j] = 1 / L(j,j).
// Per column: the team leader takes the pivot, the team scales the column,
// and the (n-j-1)(n-j)/2 trailing elements are dealt round-robin to the team
// so every lane does useful FMA work.
template <typename T>
__device__ int team_potrf_packed(const Team &t, int n, T *Lp, T *rinv, T tol, bool active)
{
  int fail = active ? 0 : -1;  // -1: idle team slot, runs the loop for the syncs only
  for (int j = 0; j < n; j++) {
    T *cj = Lp + coff(j, n) - j;
    if (t.tid == 0 && fail == 0) {
      T d = cj[j];
      if (d > tol) {
        T s, r;
        pivot_rs(d, s, r);
        cj[j] = s;
        rinv[j] = r;
      } else {
        rinv[j] = T(0);
      }
    }
    t.sync();
    if (fail == 0 && !(rinv[j] > T(0))) fail = j + 1;
    if (fail == 0) {
      const T rj = rinv[j];
      for (int i = j + 1 + t.tid; i < n; i += t.nt) cj[i] *= rj;
    }
    t.sync();
    if (fail == 0) {
      const int mm = n - 1 - j;
      int ii = 0, kk = t.tid;
      tri_advance(ii, kk, 0);
      while (ii < mm) {
        const int i = j + 1 + ii, k = j + 1 + kk;
        PL(Lp, n, i, k) -= cj[i] * cj[k];
        tri_advance(ii, kk, t.nt);
      }
    }
    t.sync();
  }
  return fail < 0 ? 0 : fail;
}

// y := L^{-T} L^{-1} y with L packed (solve of L L^T y = c), in place.
// Sub-warp teams sweep column by column; teams of whole warps go by blocks
// of 32: one warp solves each 32 x 32 diagonal block with shuffles, and the
// off-diagonal part is a coalesced matrix-vector update spread over the team.
template <typename T>
__device__ void team_llt_solve(const Team &t, int n, const T *Lp, const T *rinv, T *y, T *red,
                               bool active)
{
  if (t.nt < 32) {
    for (int j = 0; j < n; j++) {
      if (active && t.tid == 0) y[j] *= rinv[j];
      t.sync();
      if (active) {
        const T yj = y[j];
        const T *cj = Lp + coff(j, n) - j;
        for (int i = j + 1 + t.tid; i < n; i += t.nt) y[i] -= cj[i] * yj;
      }
      t.sync();
    }
    for (int j = n - 1; j >= 0; j--) {
      if (active && t.tid == 0) y[j] *= rinv[j];
      t.sync();
      if (active) {
        const T yj = y[j];
        for (int i = t.tid; i < j; i += t.nt) y[i] -= Lp[coff(i, n) + (j - i)] * yj;
      }
      t.sync();
    }
    return;
  }
  const int lane = t.lane(), w = t.warp(), nw = t.nwarps();
  // forward: L z = y
  for (int J = 0; J < n; J += 32) {
    const int jb = min(32, n - J);
    if (w == 0 && active) {
      T v = (lane < jb) ? y[J + lane] : T(0);
      for (int c = 0; c < jb; c++) {
        if (lane == c) v *= rinv[J + c];
        const T yc = __shfl_sync(0xffffffffu, v, c);
        if (lane > c && lane < jb) v -= PL(const_cast<T *>(Lp), n, J + lane, J + c) * yc;
      }
      if (lane < jb) y[J + lane] = v;
    }
    t.sync();
    if (active)
      for (int i = J + jb + t.tid; i < n; i += t.nt) {
        T s0 = T(0), s1 = T(0);
        int c = 0;
        for (; c + 1 < jb; c += 2) {
          s0 += PL(const_cast<T *>(Lp), n, i, J + c) * y[J + c];
          s1 += PL(const_cast<T *>(Lp), n, i, J + c + 1) * y[J + c + 1];
        }
        if (c < jb) s0 += PL(const_cast<T *>(Lp), n, i, J + c) * y[J + c];
        y[i] -= s0 + s1;
      }
    t.sync();
  }
  // backward: L^T x = z
  for (int J = ((n - 1) / 32) * 32; J >= 0; J -= 32) {
    const int jb = min(32, n - J);
    T s = T(0);
    if (active && lane < jb) {
      const T *col = Lp + coff(J + lane, n) - (J + lane);
      for (int k = J + jb + w; k < n; k += nw) s += col[k] * y[k];
    }
    red[w * 32 + lane] = s;
    t.sync();
    if (w == 0 && active) {
      T v = (lane < jb) ? y[J + lane] : T(0);
      for (int q = 0; q < nw; q++) v -= red[q * 32 + lane];
      for (int c = jb - 1; c >= 0; c--) {
        if (lane == c) v *= rinv[J + c];
        const T xc = __shfl_sync(0xffffffffu, v, c);
        if (lane < c) v -= PL(const_cast<T *>(Lp), n, J + c, J + lane) * xc;
      }
      if (lane < jb) y[J + lane] = v;
    }
    t.sync();
  }
}

// FP64 residual of up to MR right-hand sides (rows r0.. of the m x n matrix B,
// side 'R', X*A = B): r_q = b_q - A x_q, A symmetric given by its lower
// triangle (global memory, column-major). Each thread owns whole rows of A,
// so every DFMA issued is useful work.
template <int MR>
__device__ void team_residual(const Team &t, int n, const double *A, int lda, const double *B,
                              int ldb, int r0, int nr, const double *x, int ldx, double *r,
                              bool active)
{
  if (!active) return;
  for (int i = t.tid; i < n; i += t.nt) {
    double s[MR];
#pragma unroll
    for (int q = 0; q < MR; q++) s[q] = (q < nr) ? B[(size_t)(r0 + q) + (size_t)i * ldb] : 0.0;
    const double *row = A + i;  // A(i, j) = row[j * lda] for j <= i
    int j = 0;
    for (; j <= i; j++) {
      const double a = row[(size_t)j * lda];
#pragma unroll
      for (int q = 0; q < MR; q++) s[q] -= a * x[q * ldx + j];
    }
    const double *col = A + (size_t)i * lda;  // A(j, i) = col[j] for j > i
    for (; j < n; j++) {
      const double a = col[j];
#pragma unroll
      for (int q = 0; q < MR; q++) s[q] -= a * x[q * ldx + j];
    }
#pragma unroll
    for (int q = 0; q < MR; q++)
      if (q < nr) r[q * ldx + i] = s[q];
  }
}

}  // namespace kgb

// uplo_swap.cuh -- in-place transpose of the leading n x n block of every
// matrix of a batch, used to run the upper-triangle variants (uplo = 'U') of
// POTRF / POSV / TRTRI / LAUUM / POTRI / POTI on the lower-triangle kernels.
//
// With A^T in place, the upper triangle's data sits in the lower triangle and
// vice versa; the lower kernels read and write only the lower triangle, so
// transposing again afterwards returns the factor (or inverse) to the upper
// triangle and the untouched strict lower triangle to where it was, bit for
// bit. Cost: two extra passes over the n x n block (2 x 16 n^2 bytes).
//
// One CTA per (matrix, pair of 32 x 32 tiles (I, J), I >= J): both tiles are
// staged in shared memory and written back transposed into each other's place,
// so every element is owned by exactly one CTA.
#pragma once

#include "device_util.cuh"
#include "kblas_internal.h"

namespace kgb {

constexpr int TX_T = 32;

template <typename T, class Acc>
__global__ void __launch_bounds__(256) swap_uplo_kernel(int n, Acc A, int lda, long long batch) {
  __shared__ T s0[TX_T][TX_T + 1];
  __shared__ T s1[TX_T][TX_T + 1];
  const long long mat = blockIdx.x;
  if (mat >= batch) return;
  const int nt = (n + TX_T - 1) / TX_T;
  const int npairs = nt * (nt + 1) / 2;
  T *a = A.get(mat);
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 32 x 8
  for (int p = blockIdx.y; p < npairs; p += gridDim.y) {
    int I = 0, q = p;   // pair p -> (I, J), J <= I, row-major over the lower tile triangle
    while (q > I) { q -= I + 1; I++; }
    const int J = q;
    const int r0 = I * TX_T, c0 = J * TX_T;
    // s0 = tile (I, J), s1 = tile (J, I); element (r, c) of a tile at s[c][r]
    for (int c = ty; c < TX_T; c += 8) {
      const int gr = r0 + tx, gc = c0 + c;
      if (gr < n && gc < n) s0[c][tx] = a[(size_t)gr + (size_t)gc * lda];
      const int hr = c0 + tx, hc = r0 + c;
      if (I != J && hr < n && hc < n) s1[c][tx] = a[(size_t)hr + (size_t)hc * lda];
    }
    __syncthreads();
    // tile (I, J) := tile (J, I)^T, tile (J, I) := tile (I, J)^T
    for (int c = ty; c < TX_T; c += 8) {
      const int gr = r0 + tx, gc = c0 + c;     // (gr, gc) in tile (I, J) <- (gc, gr)
      if (gr < n && gc < n) a[(size_t)gr + (size_t)gc * lda] = (I == J) ? s0[tx][c] : s1[tx][c];
      const int hr = c0 + tx, hc = r0 + c;     // (hr, hc) in tile (J, I) <- (hc, hr)
      if (I != J && hr < n && hc < n) a[(size_t)hr + (size_t)hc * lda] = s0[tx][c];
    }
    __syncthreads();
  }
}

template <typename T, class Acc>
static int swap_uplo(KBlasHandle *h, int n, Acc A, int lda, long long batch) {
  if (n <= 1 || batch <= 0) return KBLAS_Success;
  if (batch > 0x7fffffffLL) return KBLAS_NotSupported;
  const long long nt = (n + TX_T - 1) / TX_T;
  long long pairs = nt * (nt + 1) / 2;
  ensure_device_props(h);
  const long long target = (long long)(h->sm_count > 0 ? h->sm_count : 152) * 16;
  long long y = (target + batch - 1) / batch;
  if (y > pairs) y = pairs;
  if (y > 65535) y = 65535;
  if (y < 1) y = 1;
  dim3 grid((unsigned)batch, (unsigned)y);
  swap_uplo_kernel<T><<<grid, 256, 0, h->stream>>>(n, A, lda, batch);
  KGB_LAUNCH_CHECK("swap_uplo_kernel");
  return KBLAS_Success;
}

}  // namespace kgb

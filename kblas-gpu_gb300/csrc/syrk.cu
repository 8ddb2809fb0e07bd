// syrk.cu -- batched SYRK (lower and upper), single and double precision, strided and
// pointer-array forms: C := alpha * op(A) * op(A)^T + beta * C.
//
// Entry points replace reference src/batch_triangular/Xsyrk_batch.cu:83-200
// (Upper is KBLAS_NotImplemented there, Xsyrk_batch_drivers.cuh:133-136; here
// it runs on the C-tile engine of gemm_tile.cuh). The
// reference builds pointer arrays and issues one cuBLAS gemmBatched per level
// of a flat recursion plus a diagonal-tile kernel; here one launch covers all
// lower tiles of every matrix: one CTA per (matrix, 32 x 32 lower tile), the
// two 32-row slabs of op(A) staged through shared memory KC columns at a
// time, and a 2 x 2 register tile of C per thread.
#include <stdio.h>

#include <cuComplex.h>

#include "device_util.cuh"
#include "gemm_tile.cuh"
#include "kblas_internal.h"
#include "launch_util.h"

namespace kgb {

constexpr int SY_TB = 32;   // C tile
constexpr int SY_KC = 32;   // k chunk
constexpr int SY_NT = 256;  // 16 x 16 threads, 2 x 2 elements each

template <typename T, class AccA, class AccC>
__global__ void __launch_bounds__(SY_NT)
syrk_lower_kernel(int m, int k, int trans, T alpha, AccA A, int lda, T beta, AccC Cm, int ldc,
                  int ntiles, long long batch)
{
  __shared__ T sI[SY_KC][SY_TB + 1];
  __shared__ T sJ[SY_KC][SY_TB + 1];
  const int ntri = ntiles * (ntiles + 1) / 2;
  const long long mat = blockIdx.x / ntri;
  if (mat >= batch) return;
  int t = blockIdx.x - (int)(mat * ntri);
  int ti = 0;  // tile row, tile col: enumerate the lower triangle row-major
  while (t > ti) { t -= ti + 1; ti++; }
  const int tj = t;
  const int I0 = ti * SY_TB, J0 = tj * SY_TB;
  const T *Ag = A.get(mat);
  T *Cg = Cm.get(mat);
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  T acc[2][2] = {{T(0), T(0)}, {T(0), T(0)}};

  const int kk_end = (alpha == T(0)) ? 0 : k;  // BLAS: A is not read when alpha == 0
  for (int l0 = 0; l0 < kk_end; l0 += SY_KC) {
    const int kc = min(SY_KC, k - l0);
    // op(A)(i, l) = trans ? A(l, i) : A(i, l)
    for (int idx = threadIdx.x; idx < SY_KC * SY_TB; idx += SY_NT) {
      int ll, ii;
      if (trans) { ll = idx % SY_KC; ii = idx / SY_KC; } else { ii = idx % SY_TB; ll = idx / SY_TB; }
      T vi = T(0), vj = T(0);
      if (ll < kc) {
        const int gi = I0 + ii, gj = J0 + ii, gl = l0 + ll;
        if (gi < m) vi = trans ? Ag[(size_t)gl + (size_t)gi * lda] : Ag[(size_t)gi + (size_t)gl * lda];
        if (gj < m) vj = trans ? Ag[(size_t)gl + (size_t)gj * lda] : Ag[(size_t)gj + (size_t)gl * lda];
      }
      sI[ll][ii] = vi;
      sJ[ll][ii] = vj;
    }
    __syncthreads();
    for (int ll = 0; ll < kc; ll++) {
      const T a0 = sI[ll][ty], a1 = sI[ll][ty + 16];
      const T b0 = sJ[ll][tx], b1 = sJ[ll][tx + 16];
      acc[0][0] += a0 * b0;
      acc[0][1] += a0 * b1;
      acc[1][0] += a1 * b0;
      acc[1][1] += a1 * b1;
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int c = 0; c < 2; c++) {
      const int gi = I0 + ty + 16 * a, gj = J0 + tx + 16 * c;
      if (gi < m && gj < m && gi >= gj) {
        T *p = Cg + (size_t)gi + (size_t)gj * ldc;
        *p = (beta == T(0)) ? alpha * acc[a][c] : alpha * acc[a][c] + beta * (*p);
      }
    }
}

// uplo 'U' (KBLAS_NotImplemented in the reference): the C-tile engine of
// gemm_tile.cuh on the upper tile triangle.
template <typename T, class AccA, class AccC>
static int launch_syrk_upper(KBlasHandle *h, int m, int k, bool trans, T alpha, AccA A, int lda,
                             T beta, AccC Cm, int ldc, long long batch) {
  if (batch > 0x7fffffffLL) return KBLAS_NotSupported;
  const long long nt = (m + GT - 1) / GT;
  dim3 grid((unsigned)batch, tile_slots(h, batch, nt * (nt + 1) / 2));
  syrk_batch_kernel<T><<<grid, GT_NT, 0, h->stream>>>(1, trans ? 1 : 0, alpha, A, beta, Cm,
                                                      DimsU<4>{{m, k, lda, ldc}}, batch);
  KGB_LAUNCH_CHECK("syrk_batch_kernel");
  return KBLAS_Success;
}

template <typename T, class AccA, class AccC>
static int launch_syrk(KBlasHandle *h, int m, int k, bool trans, T alpha, AccA A, int lda, T beta,
                       AccC Cm, int ldc, long long batch) {
  const int ntiles = (m + SY_TB - 1) / SY_TB;
  const long long grid = batch * (long long)(ntiles * (ntiles + 1) / 2);
  if (grid > 0x7fffffffLL) return KBLAS_NotSupported;
  syrk_lower_kernel<T><<<(unsigned)grid, SY_NT, 0, h->stream>>>(m, k, trans ? 1 : 0, alpha, A, lda,
                                                                beta, Cm, ldc, ntiles, batch);
  KGB_LAUNCH_CHECK("syrk_lower_kernel");
  return KBLAS_Success;
}

static inline int check_syrk(KBlasHandle *h, char uplo, char trans, int m, int n, int lda, int ldb,
                             int batch) {
  if (!h) return KBLAS_Error_NotInitialized;
  if (!(is_lower(uplo) || is_upper(uplo)) || !(is_trans(trans) || is_notrans(trans)))
    return KBLAS_Error_WrongInput;
  const int rows_a = is_notrans(trans) ? m : n;
  if (m < 0 || n < 0 || batch < 0 || lda < (rows_a > 1 ? rows_a : 1) || ldb < (m > 1 ? m : 1))
    return KBLAS_Error_WrongInput;
  return KBLAS_Success;
}

template <typename T>
static int syrk_strided(KBlasHandle *h, char uplo, char trans, int m, int n, T alpha, const T *A,
                        int lda, long long sA, T beta, T *B, int ldb, long long sB, int batch) {
  int st = check_syrk(h, uplo, trans, m, n, lda, ldb, batch);
  if (st != KBLAS_Success) return st;
  if (m == 0 || batch == 0) return KBLAS_Success;
  if (!B || (n > 0 && !A) || (batch > 1 && sB < (long long)ldb * m)) return KBLAS_Error_WrongInput;
  if (is_upper(uplo))
    return launch_syrk_upper<T>(h, m, n, is_trans(trans), alpha, Strided<T>{const_cast<T *>(A), sA},
                                lda, beta, Strided<T>{B, sB}, ldb, batch);
  return launch_syrk<T>(h, m, n, is_trans(trans), alpha, Strided<T>{const_cast<T *>(A), sA}, lda,
                        beta, Strided<T>{B, sB}, ldb, batch);
}

template <typename T>
static int syrk_array(KBlasHandle *h, char uplo, char trans, int m, int n, T alpha, const T **A,
                      int lda, T beta, T **B, int ldb, int batch) {
  int st = check_syrk(h, uplo, trans, m, n, lda, ldb, batch);
  if (st != KBLAS_Success) return st;
  if (m == 0 || batch == 0) return KBLAS_Success;
  if (!B || (n > 0 && !A)) return KBLAS_Error_WrongInput;
  if (is_upper(uplo))
    return launch_syrk_upper<T>(h, m, n, is_trans(trans), alpha, PtrArr<T>{const_cast<T **>(A)}, lda,
                                beta, PtrArr<T>{B}, ldb, batch);
  return launch_syrk<T>(h, m, n, is_trans(trans), alpha, PtrArr<T>{const_cast<T **>(A)}, lda, beta,
                        PtrArr<T>{B}, ldb, batch);
}

}  // namespace kgb

using namespace kgb;

extern "C" {

int kblasSsyrk_batch(kblasHandle_t h, char uplo, char trans, const int m, const int n,
                     const float alpha, const float **A, int lda, const float beta, float **B,
                     int ldb, int batchCount) {
  return syrk_array<float>(h, uplo, trans, m, n, alpha, A, lda, beta, B, ldb, batchCount);
}
int kblasDsyrk_batch(kblasHandle_t h, char uplo, char trans, const int m, const int n,
                     const double alpha, const double **A, int lda, const double beta, double **B,
                     int ldb, int batchCount) {
  return syrk_array<double>(h, uplo, trans, m, n, alpha, A, lda, beta, B, ldb, batchCount);
}
int kblasSsyrk_batch_strided(kblasHandle_t h, char uplo, char trans, const int m, const int n,
                             const float alpha, const float *A, int lda, long strideA,
                             const float beta, float *B, int ldb, long strideB, int batchCount) {
  return syrk_strided<float>(h, uplo, trans, m, n, alpha, A, lda, strideA, beta, B, ldb, strideB,
                             batchCount);
}
int kblasDsyrk_batch_strided(kblasHandle_t h, char uplo, char trans, const int m, const int n,
                             const double alpha, const double *A, int lda, long strideA,
                             const double beta, double *B, int ldb, long strideB,
                             int batchCount) {
  return syrk_strided<double>(h, uplo, trans, m, n, alpha, A, lda, strideA, beta, B, ldb, strideB,
                              batchCount);
}

// Complex precisions: C := alpha op(A) op(A)^T + beta C (complex-symmetric,
// the reference's kblas{C,Z}syrk_batch; no conjugation).
#define KGB_SYRK_CPLX(X, API, T)                                                                   \
  int kblas##X##syrk_batch(kblasHandle_t h, char uplo, char trans, const int m, const int n,       \
                           const API alpha, const API **A, int lda, const API beta, API **B,       \
                           int ldb, int batchCount) {                                              \
    return syrk_array<T>(h, uplo, trans, m, n, T(alpha.x, alpha.y),                                \
                         reinterpret_cast<const T **>(A), lda, T(beta.x, beta.y),                  \
                         reinterpret_cast<T **>(B), ldb, batchCount);                              \
  }                                                                                                \
  int kblas##X##syrk_batch_strided(kblasHandle_t h, char uplo, char trans, const int m,            \
                                   const int n, const API alpha, const API *A, int lda,            \
                                   long strideA, const API beta, API *B, int ldb, long strideB,    \
                                   int batchCount) {                                               \
    return syrk_strided<T>(h, uplo, trans, m, n, T(alpha.x, alpha.y),                              \
                           reinterpret_cast<const T *>(A), lda, strideA, T(beta.x, beta.y),        \
                           reinterpret_cast<T *>(B), ldb, strideB, batchCount);                    \
  }

KGB_SYRK_CPLX(C, cuFloatComplex, cxf)
KGB_SYRK_CPLX(Z, cuDoubleComplex, cxd)
#undef KGB_SYRK_CPLX

}  // extern "C"

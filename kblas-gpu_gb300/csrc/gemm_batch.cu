// gemm_batch.cu -- batched GEMM (uniform: strided and pointer-array;
// variable-size: per-matrix m, n, k and leading dimensions in device arrays)
// and the variable-size SYRK (lower and upper), single and double precision.
//
// Entry points replace reference src/batch_triangular/Xgemm_batch.cu:53-240
// (uniform GEMM through cuBLAS gemm(Strided)Batched, Xgemm_batch_core.cuh:
// 171-300 and 493-560; variable-size GEMM through MAGMA only,
// Xgemm_batch_core.cuh:386-470) and Xsyrk_batch.cu:100-200 (variable-size SYRK
// through MAGMA only, Xsyrk_batch_drivers.cuh:437-500). Here all of them run
// on one native tile kernel (gemm_tile.cuh), whatever the sizes.
//
// Argument conventions kept from the reference: batchCount < 1 is
// KBLAS_Error_WrongInput for GEMM (Xgemm_batch_core.cuh:181,386); for the
// variable-size calls max_m / max_n / max_k are hints, and "all zero" means
// the sizes are not known on the host (the reference then recomputes them on
// the device and synchronises; these kernels do not need them, so nothing is
// recomputed and no workspace is used). Per-matrix sizes in the device
// arrays are not validated (the reference calls MAGMA's _nocheck variants):
// a matrix with m <= 0 or n <= 0 is skipped.
#include <stdio.h>

#include <cuComplex.h>

#include "gemm_tile.cuh"
#include "kblas_internal.h"
#include "launch_util.h"

namespace kgb {

// C := alpha op(A) op(B) + beta C over a batch; dims = (m, n, k, lda, ldb, ldc)
template <typename T, class AccA, class AccB, class AccC, class Dims>
__global__ void __launch_bounds__(GT_NT)
gemm_batch_kernel(int ta, int tb, T alpha, AccA A, AccB B, T beta, AccC Cm, Dims dims,
                  long long batch)
{
  __shared__ __align__(16) GemmSmem<T> s;
  const long long mat = blockIdx.x;
  if (mat >= batch) return;
  int d[6];
  dims.get(mat, d);
  const int m = d[0], n = d[1];
  if (m <= 0 || n <= 0) return;
  const int tm = (m + GT - 1) / GT, tn = (n + GT - 1) / GT;
  TileJob<T> j;
  j.A = A.get(mat);
  j.B = B.get(mat);
  j.C = Cm.get(mat);
  j.m = m; j.n = n; j.k = d[2];
  j.lda = d[3]; j.ldb = d[4]; j.ldc = d[5];
  j.ta = ta; j.tb = tb;
  j.part = TILE_FULL;
  for (int t = blockIdx.y; t < tm * tn; t += gridDim.y) {
    j.I0 = (t % tm) * GT;
    j.J0 = (t / tm) * GT;
    gemm_tile<T>(j, alpha, beta, s);
  }
}

static inline bool trans_flag(char c, int &t) {
  if (is_trans(c)) { t = 1; return true; }
  if (is_notrans(c)) { t = 0; return true; }
  return false;
}

template <typename T, class AccA, class AccB, class AccC, class Dims>
static int launch_gemm(KBlasHandle *h, int ta, int tb, T alpha, AccA A, AccB B, T beta, AccC Cm,
                       Dims dims, long long batch, long long tiles_hint) {
  if (batch > 0x7fffffffLL) return KBLAS_NotSupported;
  dim3 grid((unsigned)batch, tile_slots(h, batch, tiles_hint));
  gemm_batch_kernel<T><<<grid, GT_NT, 0, h->stream>>>(ta, tb, alpha, A, B, beta, Cm, dims, batch);
  KGB_LAUNCH_CHECK("gemm_batch_kernel");
  return KBLAS_Success;
}

static inline long long ceil_div(long long a, long long b) { return (a + b - 1) / b; }

static int check_gemm(KBlasHandle *h, char transA, char transB, int m, int n, int k, int lda,
                      int ldb, int ldc, int batch, int &ta, int &tb) {
  if (!h) return KBLAS_Error_NotInitialized;
  if (batch < 1) return KBLAS_Error_WrongInput;
  if (!trans_flag(transA, ta) || !trans_flag(transB, tb)) return KBLAS_Error_WrongInput;
  const int rows_a = ta ? k : m, rows_b = tb ? n : k;
  if (m < 0 || n < 0 || k < 0 || lda < (rows_a > 1 ? rows_a : 1) ||
      ldb < (rows_b > 1 ? rows_b : 1) || ldc < (m > 1 ? m : 1))
    return KBLAS_Error_WrongInput;
  return KBLAS_Success;
}

template <typename T>
static int gemm_strided(KBlasHandle *h, char transA, char transB, int m, int n, int k, T alpha,
                        const T *A, int lda, long long sA, const T *B, int ldb, long long sB,
                        T beta, T *C, int ldc, long long sC, int batch) {
  int ta, tb;
  int st = check_gemm(h, transA, transB, m, n, k, lda, ldb, ldc, batch, ta, tb);
  if (st != KBLAS_Success) return st;
  if (m == 0 || n == 0) return KBLAS_Success;
  if (!C || (k > 0 && alpha != T(0) && (!A || !B))) return KBLAS_Error_WrongInput;
  DimsU<6> dims{{m, n, k, lda, ldb, ldc}};
  return launch_gemm<T>(h, ta, tb, alpha, Strided<T>{const_cast<T *>(A), sA},
                        Strided<T>{const_cast<T *>(B), sB}, beta, Strided<T>{C, sC}, dims, batch,
                        ceil_div(m, GT) * ceil_div(n, GT));
}

template <typename T>
static int gemm_array(KBlasHandle *h, char transA, char transB, int m, int n, int k, T alpha,
                      const T **A, int lda, const T **B, int ldb, T beta, T **C, int ldc,
                      int batch) {
  int ta, tb;
  int st = check_gemm(h, transA, transB, m, n, k, lda, ldb, ldc, batch, ta, tb);
  if (st != KBLAS_Success) return st;
  if (m == 0 || n == 0) return KBLAS_Success;
  if (!C || (k > 0 && alpha != T(0) && (!A || !B))) return KBLAS_Error_WrongInput;
  DimsU<6> dims{{m, n, k, lda, ldb, ldc}};
  return launch_gemm<T>(h, ta, tb, alpha, PtrArr<T>{const_cast<T **>(A)},
                        PtrArr<T>{const_cast<T **>(B)}, beta, PtrArr<T>{C}, dims, batch,
                        ceil_div(m, GT) * ceil_div(n, GT));
}

template <typename T>
static int gemm_vbatch(KBlasHandle *h, char transA, char transB, const int *m, const int *n,
                       const int *k, int max_m, int max_n, int max_k, T alpha, const T **A,
                       const int *lda, const T **B, const int *ldb, T beta, T **C, const int *ldc,
                       int batch) {
  (void)max_k;
  if (!h) return KBLAS_Error_NotInitialized;
  int ta, tb;
  if (batch < 1 || !trans_flag(transA, ta) || !trans_flag(transB, tb)) return KBLAS_Error_WrongInput;
  if (!m || !n || !k || !lda || !ldb || !ldc || !A || !B || !C) return KBLAS_Error_WrongInput;
  const long long hint = (max_m > 0 && max_n > 0) ? ceil_div(max_m, GT) * ceil_div(max_n, GT) : 0;
  DimsV<6> dims{{m, n, k, lda, ldb, ldc}};
  return launch_gemm<T>(h, ta, tb, alpha, PtrArr<T>{const_cast<T **>(A)},
                        PtrArr<T>{const_cast<T **>(B)}, beta, PtrArr<T>{C}, dims, batch, hint);
}

template <typename T>
static int syrk_vbatch(KBlasHandle *h, char uplo, char trans, const int *m, const int *n,
                       int max_m, int max_n, T alpha, const T **A, const int *lda, T beta, T **B,
                       const int *ldb, int batch) {
  (void)max_n;
  if (!h) return KBLAS_Error_NotInitialized;
  int tr;
  if (!(is_lower(uplo) || is_upper(uplo)) || !trans_flag(trans, tr) || batch < 0)
    return KBLAS_Error_WrongInput;
  if (batch == 0) return KBLAS_Success;
  if (!m || !n || !lda || !ldb || !A || !B) return KBLAS_Error_WrongInput;
  if (batch > 0x7fffffffLL) return KBLAS_NotSupported;
  long long hint = 0;
  if (max_m > 0) {
    const long long nt = ceil_div(max_m, GT);
    hint = nt * (nt + 1) / 2;
  }
  DimsV<4> dims{{m, n, lda, ldb}};
  dim3 grid((unsigned)batch, tile_slots(h, batch, hint));
  syrk_batch_kernel<T><<<grid, GT_NT, 0, h->stream>>>(is_upper(uplo) ? 1 : 0, tr, alpha,
                                                       PtrArr<T>{const_cast<T **>(A)}, beta,
                                                       PtrArr<T>{B}, dims, (long long)batch);
  KGB_LAUNCH_CHECK("syrk_batch_kernel");
  return KBLAS_Success;
}

}  // namespace kgb

using namespace kgb;

extern "C" {

int kblasSgemm_batch(kblasHandle_t h, char transA, char transB, const int m, const int n,
                     const int k, const float alpha, const float **A, int lda, const float **B,
                     int ldb, const float beta, float **C, int ldc, int batchCount) {
  return gemm_array<float>(h, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc,
                           batchCount);
}
int kblasDgemm_batch(kblasHandle_t h, char transA, char transB, const int m, const int n,
                     const int k, const double alpha, const double **A, int lda, const double **B,
                     int ldb, const double beta, double **C, int ldc, int batchCount) {
  return gemm_array<double>(h, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc,
                            batchCount);
}
int kblasSgemm_batch_strided(kblasHandle_t h, char transA, char transB, const int m, const int n,
                             const int k, const float alpha, const float *A, int lda,
                             long strideA, const float *B, int ldb, long strideB,
                             const float beta, float *C, int ldc, long strideC, int batchCount) {
  return gemm_strided<float>(h, transA, transB, m, n, k, alpha, A, lda, strideA, B, ldb, strideB,
                             beta, C, ldc, strideC, batchCount);
}
int kblasDgemm_batch_strided(kblasHandle_t h, char transA, char transB, const int m, const int n,
                             const int k, const double alpha, const double *A, int lda,
                             long strideA, const double *B, int ldb, long strideB,
                             const double beta, double *C, int ldc, long strideC,
                             int batchCount) {
  return gemm_strided<double>(h, transA, transB, m, n, k, alpha, A, lda, strideA, B, ldb, strideB,
                              beta, C, ldc, strideC, batchCount);
}

int kblasSgemm_vbatch(kblasHandle_t h, char transA, char transB, int *m, int *n, int *k,
                      int max_m, int max_n, int max_k, const float alpha, const float **A,
                      int *lda, const float **B, int *ldb, const float beta, float **C, int *ldc,
                      int batchCount) {
  return gemm_vbatch<float>(h, transA, transB, m, n, k, max_m, max_n, max_k, alpha, A, lda, B,
                            ldb, beta, C, ldc, batchCount);
}
int kblasDgemm_vbatch(kblasHandle_t h, char transA, char transB, int *m, int *n, int *k,
                      int max_m, int max_n, int max_k, const double alpha, const double **A,
                      int *lda, const double **B, int *ldb, const double beta, double **C,
                      int *ldc, int batchCount) {
  return gemm_vbatch<double>(h, transA, transB, m, n, k, max_m, max_n, max_k, alpha, A, lda, B,
                             ldb, beta, C, ldc, batchCount);
}

int kblasSsyrk_vbatch(kblasHandle_t h, char uplo, char trans, int *m, int *n, int max_m,
                      int max_n, const float alpha, const float **A, int *lda, const float beta,
                      float **B, int *ldb, int batchCount) {
  return syrk_vbatch<float>(h, uplo, trans, m, n, max_m, max_n, alpha, A, lda, beta, B, ldb,
                            batchCount);
}
int kblasDsyrk_vbatch(kblasHandle_t h, char uplo, char trans, int *m, int *n, int max_m,
                      int max_n, const double alpha, const double **A, int *lda,
                      const double beta, double **B, int *ldb, int batchCount) {
  return syrk_vbatch<double>(h, uplo, trans, m, n, max_m, max_n, alpha, A, lda, beta, B, ldb,
                             batchCount);
}

// Complex precisions (op = transpose, as the reference's KBLAS_Trans):
// uniform GEMM (reference kblas{C,Z}gemm_batch[_strided]) and the
// variable-size GEMM / SYRK (its complex non-uniform overloads).
#define KGB_GEMM_CPLX(X, API, T)                                                                   \
  int kblas##X##gemm_batch(kblasHandle_t h, char transA, char transB, const int m, const int n,    \
                           const int k, const API alpha, const API **A, int lda, const API **B,    \
                           int ldb, const API beta, API **C, int ldc, int batchCount) {            \
    return gemm_array<T>(h, transA, transB, m, n, k, T(alpha.x, alpha.y),                          \
                         reinterpret_cast<const T **>(A), lda, reinterpret_cast<const T **>(B),    \
                         ldb, T(beta.x, beta.y), reinterpret_cast<T **>(C), ldc, batchCount);      \
  }                                                                                                \
  int kblas##X##gemm_batch_strided(kblasHandle_t h, char transA, char transB, const int m,         \
                                   const int n, const int k, const API alpha, const API *A,        \
                                   int lda, long strideA, const API *B, int ldb, long strideB,     \
                                   const API beta, API *C, int ldc, long strideC,                  \
                                   int batchCount) {                                               \
    return gemm_strided<T>(h, transA, transB, m, n, k, T(alpha.x, alpha.y),                        \
                           reinterpret_cast<const T *>(A), lda, strideA,                           \
                           reinterpret_cast<const T *>(B), ldb, strideB, T(beta.x, beta.y),        \
                           reinterpret_cast<T *>(C), ldc, strideC, batchCount);                    \
  }                                                                                                \
  int kblas##X##gemm_vbatch(kblasHandle_t h, char transA, char transB, int *m, int *n, int *k,     \
                            int max_m, int max_n, int max_k, const API alpha, const API **A,       \
                            int *lda, const API **B, int *ldb, const API beta, API **C, int *ldc,  \
                            int batchCount) {                                                      \
    return gemm_vbatch<T>(h, transA, transB, m, n, k, max_m, max_n, max_k, T(alpha.x, alpha.y),    \
                          reinterpret_cast<const T **>(A), lda, reinterpret_cast<const T **>(B),   \
                          ldb, T(beta.x, beta.y), reinterpret_cast<T **>(C), ldc, batchCount);     \
  }                                                                                                \
  int kblas##X##syrk_vbatch(kblasHandle_t h, char uplo, char trans, int *m, int *n, int max_m,     \
                            int max_n, const API alpha, const API **A, int *lda, const API beta,   \
                            API **B, int *ldb, int batchCount) {                                   \
    return syrk_vbatch<T>(h, uplo, trans, m, n, max_m, max_n, T(alpha.x, alpha.y),                 \
                          reinterpret_cast<const T **>(A), lda, T(beta.x, beta.y),                 \
                          reinterpret_cast<T **>(B), ldb, batchCount);                             \
  }

KGB_GEMM_CPLX(C, cuFloatComplex, cxf)
KGB_GEMM_CPLX(Z, cuDoubleComplex, cxd)
#undef KGB_GEMM_CPLX

}  // extern "C"

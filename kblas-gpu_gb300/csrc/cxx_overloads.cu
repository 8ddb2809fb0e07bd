// cxx_overloads.cu -- the C++ overload set of the batch API
// (reference include/kblas_batch.h:493-576, 794-891, 1119-1177, 1396-1452,
// 2094-2152, 2790-2855), forwarding to the C entry points.
#include "kblas.h"

int kblas_potrf_batch(kblasHandle_t h, char uplo, const int n, float **A, int lda, int batchCount,
                      int *info) {
  return kblasSpotrf_batch(h, uplo, n, A, lda, batchCount, info);
}
int kblas_potrf_batch(kblasHandle_t h, char uplo, const int n, double **A, int lda, int batchCount,
                      int *info) {
  return kblasDpotrf_batch(h, uplo, n, A, lda, batchCount, info);
}
int kblas_potrf_batch(kblasHandle_t h, char uplo, const int n, float *A, int lda, long strideA,
                      int batchCount, int *info) {
  return kblasSpotrf_batch_strided(h, uplo, n, A, lda, strideA, batchCount, info);
}
int kblas_potrf_batch(kblasHandle_t h, char uplo, const int n, double *A, int lda, long strideA,
                      int batchCount, int *info) {
  return kblasDpotrf_batch_strided(h, uplo, n, A, lda, strideA, batchCount, info);
}

int kblas_potrs_batch(kblasHandle_t h, char side, char uplo, const int m, const int n,
                      const float **A, int lda, float **B, int ldb, int batchCount) {
  return kblasSpotrs_batch(h, side, uplo, m, n, A, lda, B, ldb, batchCount);
}
int kblas_potrs_batch(kblasHandle_t h, char side, char uplo, const int m, const int n,
                      const double **A, int lda, double **B, int ldb, int batchCount) {
  return kblasDpotrs_batch(h, side, uplo, m, n, A, lda, B, ldb, batchCount);
}
int kblas_potrs_batch(kblasHandle_t h, char side, char uplo, const int m, const int n,
                      const float *A, int lda, long strideA, float *B, int ldb, long strideB,
                      int batchCount) {
  return kblasSpotrs_batch_strided(h, side, uplo, m, n, A, lda, strideA, B, ldb, strideB, batchCount);
}
int kblas_potrs_batch(kblasHandle_t h, char side, char uplo, const int m, const int n,
                      const double *A, int lda, long strideA, double *B, int ldb, long strideB,
                      int batchCount) {
  return kblasDpotrs_batch_strided(h, side, uplo, m, n, A, lda, strideA, B, ldb, strideB, batchCount);
}

int kblas_posv_batch(kblasHandle_t h, char side, char uplo, const int m, const int n, float **A,
                     int lda, float **B, int ldb, int batchCount, int *info) {
  return kblasSposv_batch(h, side, uplo, m, n, A, lda, B, ldb, batchCount, info);
}
int kblas_posv_batch(kblasHandle_t h, char side, char uplo, const int m, const int n, double **A,
                     int lda, double **B, int ldb, int batchCount, int *info) {
  return kblasDposv_batch(h, side, uplo, m, n, A, lda, B, ldb, batchCount, info);
}
int kblas_posv_batch(kblasHandle_t h, char side, char uplo, const int m, const int n, float *A,
                     int lda, long strideA, float *B, int ldb, long strideB, int batchCount,
                     int *info) {
  return kblasSposv_batch_strided(h, side, uplo, m, n, A, lda, strideA, B, ldb, strideB, batchCount,
                                  info);
}
int kblas_posv_batch(kblasHandle_t h, char side, char uplo, const int m, const int n, double *A,
                     int lda, long strideA, double *B, int ldb, long strideB, int batchCount,
                     int *info) {
  return kblasDposv_batch_strided(h, side, uplo, m, n, A, lda, strideA, B, ldb, strideB, batchCount,
                                  info);
}

int kblas_trsm_batch(kblasHandle_t h, char side, char uplo, char trans, char diag, const int m,
                     const int n, const float alpha, const float **A, int lda, float **B, int ldb,
                     int batchCount) {
  return kblasStrsm_batch(h, side, uplo, trans, diag, m, n, alpha, A, lda, B, ldb, batchCount);
}
int kblas_trsm_batch(kblasHandle_t h, char side, char uplo, char trans, char diag, const int m,
                     const int n, const double alpha, const double **A, int lda, double **B,
                     int ldb, int batchCount) {
  return kblasDtrsm_batch(h, side, uplo, trans, diag, m, n, alpha, A, lda, B, ldb, batchCount);
}
int kblas_trsm_batch(kblasHandle_t h, char side, char uplo, char trans, char diag, const int m,
                     const int n, const float alpha, const float *A, int lda, long strideA,
                     float *B, int ldb, long strideB, int batchCount) {
  return kblasStrsm_batch_strided(h, side, uplo, trans, diag, m, n, alpha, A, lda, strideA, B, ldb,
                                  strideB, batchCount);
}
int kblas_trsm_batch(kblasHandle_t h, char side, char uplo, char trans, char diag, const int m,
                     const int n, const double alpha, const double *A, int lda, long strideA,
                     double *B, int ldb, long strideB, int batchCount) {
  return kblasDtrsm_batch_strided(h, side, uplo, trans, diag, m, n, alpha, A, lda, strideA, B, ldb,
                                  strideB, batchCount);
}

int kblas_trmm_batch(kblasHandle_t h, char side, char uplo, char trans, char diag, const int m,
                     const int n, const float alpha, const float **A, int lda, float **B, int ldb,
                     int batchCount) {
  return kblasStrmm_batch(h, side, uplo, trans, diag, m, n, alpha, A, lda, B, ldb, batchCount);
}
int kblas_trmm_batch(kblasHandle_t h, char side, char uplo, char trans, char diag, const int m,
                     const int n, const double alpha, const double **A, int lda, double **B,
                     int ldb, int batchCount) {
  return kblasDtrmm_batch(h, side, uplo, trans, diag, m, n, alpha, A, lda, B, ldb, batchCount);
}
int kblas_trmm_batch(kblasHandle_t h, char side, char uplo, char trans, char diag, const int m,
                     const int n, const float alpha, const float *A, int lda, long strideA,
                     float *B, int ldb, long strideB, int batchCount) {
  return kblasStrmm_batch_strided(h, side, uplo, trans, diag, m, n, alpha, A, lda, strideA, B, ldb,
                                  strideB, batchCount);
}
int kblas_trmm_batch(kblasHandle_t h, char side, char uplo, char trans, char diag, const int m,
                     const int n, const double alpha, const double *A, int lda, long strideA,
                     double *B, int ldb, long strideB, int batchCount) {
  return kblasDtrmm_batch_strided(h, side, uplo, trans, diag, m, n, alpha, A, lda, strideA, B, ldb,
                                  strideB, batchCount);
}

int kblas_syrk_batch(kblasHandle_t h, char uplo, char trans, const int m, const int n,
                     const float alpha, const float **A, int lda, const float beta, float **B,
                     int ldb, int batchCount) {
  return kblasSsyrk_batch(h, uplo, trans, m, n, alpha, A, lda, beta, B, ldb, batchCount);
}
int kblas_syrk_batch(kblasHandle_t h, char uplo, char trans, const int m, const int n,
                     const double alpha, const double **A, int lda, const double beta, double **B,
                     int ldb, int batchCount) {
  return kblasDsyrk_batch(h, uplo, trans, m, n, alpha, A, lda, beta, B, ldb, batchCount);
}
int kblas_syrk_batch(kblasHandle_t h, char uplo, char trans, const int m, const int n,
                     const float alpha, const float *A, int lda, long strideA, const float beta,
                     float *B, int ldb, long strideB, int batchCount) {
  return kblasSsyrk_batch_strided(h, uplo, trans, m, n, alpha, A, lda, strideA, beta, B, ldb, strideB,
                                  batchCount);
}
int kblas_syrk_batch(kblasHandle_t h, char uplo, char trans, const int m, const int n,
                     const double alpha, const double *A, int lda, long strideA,
                     const double beta, double *B, int ldb, long strideB, int batchCount) {
  return kblasDsyrk_batch_strided(h, uplo, trans, m, n, alpha, A, lda, strideA, beta, B, ldb, strideB,
                                  batchCount);
}

// GEMM, reference include/kblas_batch.h:82-190 (uniform) and :201-245
// (variable-size).
int kblas_gemm_batch(kblasHandle_t h, char transA, char transB, const int m, const int n,
                     const int k, const float alpha, const float **A, int lda, const float **B,
                     int ldb, const float beta, float **C, int ldc, int batchCount) {
  return kblasSgemm_batch(h, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc,
                          batchCount);
}
int kblas_gemm_batch(kblasHandle_t h, char transA, char transB, const int m, const int n,
                     const int k, const double alpha, const double **A, int lda, const double **B,
                     int ldb, const double beta, double **C, int ldc, int batchCount) {
  return kblasDgemm_batch(h, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc,
                          batchCount);
}
int kblas_gemm_batch(kblasHandle_t h, char transA, char transB, const int m, const int n,
                     const int k, const float alpha, const float *A, int lda, long strideA,
                     const float *B, int ldb, long strideB, const float beta, float *C, int ldc,
                     long strideC, int batchCount) {
  return kblasSgemm_batch_strided(h, transA, transB, m, n, k, alpha, A, lda, strideA, B, ldb,
                                  strideB, beta, C, ldc, strideC, batchCount);
}
int kblas_gemm_batch(kblasHandle_t h, char transA, char transB, const int m, const int n,
                     const int k, const double alpha, const double *A, int lda, long strideA,
                     const double *B, int ldb, long strideB, const double beta, double *C,
                     int ldc, long strideC, int batchCount) {
  return kblasDgemm_batch_strided(h, transA, transB, m, n, k, alpha, A, lda, strideA, B, ldb,
                                  strideB, beta, C, ldc, strideC, batchCount);
}
int kblas_gemm_batch(kblasHandle_t h, char transA, char transB, int *m, int *n, int *k,
                     int max_m, int max_n, int max_k, const float alpha, const float **A,
                     int *lda, const float **B, int *ldb, const float beta, float **C, int *ldc,
                     int batchCount) {
  return kblasSgemm_vbatch(h, transA, transB, m, n, k, max_m, max_n, max_k, alpha, A, lda, B, ldb,
                           beta, C, ldc, batchCount);
}
int kblas_gemm_batch(kblasHandle_t h, char transA, char transB, int *m, int *n, int *k,
                     int max_m, int max_n, int max_k, const double alpha, const double **A,
                     int *lda, const double **B, int *ldb, const double beta, double **C,
                     int *ldc, int batchCount) {
  return kblasDgemm_vbatch(h, transA, transB, m, n, k, max_m, max_n, max_k, alpha, A, lda, B, ldb,
                           beta, C, ldc, batchCount);
}

// Variable-size SYRK and TRSM, reference include/kblas_batch.h:524-550 and
// :829-860.
int kblas_syrk_batch(kblasHandle_t h, char uplo, char trans, int *m, int *n, int max_m, int max_n,
                     float alpha, float **A, int *lda, float beta, float **B, int *ldb,
                     int batchCount) {
  return kblasSsyrk_vbatch(h, uplo, trans, m, n, max_m, max_n, alpha, (const float **)A, lda, beta,
                           B, ldb, batchCount);
}
int kblas_syrk_batch(kblasHandle_t h, char uplo, char trans, int *m, int *n, int max_m, int max_n,
                     double alpha, double **A, int *lda, double beta, double **B, int *ldb,
                     int batchCount) {
  return kblasDsyrk_vbatch(h, uplo, trans, m, n, max_m, max_n, alpha, (const double **)A, lda,
                           beta, B, ldb, batchCount);
}
int kblas_trsm_batch(kblasHandle_t h, char side, char uplo, char trans, char diag, int *m, int *n,
                     int max_m, int max_n, float alpha, float **A, int *lda, float **B, int *ldb,
                     int batchCount) {
  return kblasStrsm_vbatch(h, side, uplo, trans, diag, m, n, max_m, max_n, alpha,
                           (const float **)A, lda, B, ldb, batchCount);
}
int kblas_trsm_batch(kblasHandle_t h, char side, char uplo, char trans, char diag, int *m, int *n,
                     int max_m, int max_n, double alpha, double **A, int *lda, double **B,
                     int *ldb, int batchCount) {
  return kblasDtrsm_vbatch(h, side, uplo, trans, diag, m, n, max_m, max_n, alpha,
                           (const double **)A, lda, B, ldb, batchCount);
}

// Complex precisions of every overload above (reference: the cuFloatComplex /
// cuDoubleComplex members of each overload set).
int kblas_potrf_batch(kblasHandle_t h, char uplo, const int n, cuFloatComplex **A, int lda, int batchCount,
                      int *info) {
  return kblasCpotrf_batch(h, uplo, n, A, lda, batchCount, info);
}
int kblas_potrf_batch(kblasHandle_t h, char uplo, const int n, cuDoubleComplex **A, int lda, int batchCount,
                      int *info) {
  return kblasZpotrf_batch(h, uplo, n, A, lda, batchCount, info);
}
int kblas_potrf_batch(kblasHandle_t h, char uplo, const int n, cuFloatComplex *A, int lda, long strideA,
                      int batchCount, int *info) {
  return kblasCpotrf_batch_strided(h, uplo, n, A, lda, strideA, batchCount, info);
}
int kblas_potrf_batch(kblasHandle_t h, char uplo, const int n, cuDoubleComplex *A, int lda, long strideA,
                      int batchCount, int *info) {
  return kblasZpotrf_batch_strided(h, uplo, n, A, lda, strideA, batchCount, info);
}
int kblas_potrs_batch(kblasHandle_t h, char side, char uplo, const int m, const int n,
                      const cuFloatComplex **A, int lda, cuFloatComplex **B, int ldb, int batchCount) {
  return kblasCpotrs_batch(h, side, uplo, m, n, A, lda, B, ldb, batchCount);
}
int kblas_potrs_batch(kblasHandle_t h, char side, char uplo, const int m, const int n,
                      const cuDoubleComplex **A, int lda, cuDoubleComplex **B, int ldb, int batchCount) {
  return kblasZpotrs_batch(h, side, uplo, m, n, A, lda, B, ldb, batchCount);
}
int kblas_potrs_batch(kblasHandle_t h, char side, char uplo, const int m, const int n,
                      const cuFloatComplex *A, int lda, long strideA, cuFloatComplex *B, int ldb, long strideB,
                      int batchCount) {
  return kblasCpotrs_batch_strided(h, side, uplo, m, n, A, lda, strideA, B, ldb, strideB, batchCount);
}
int kblas_potrs_batch(kblasHandle_t h, char side, char uplo, const int m, const int n,
                      const cuDoubleComplex *A, int lda, long strideA, cuDoubleComplex *B, int ldb, long strideB,
                      int batchCount) {
  return kblasZpotrs_batch_strided(h, side, uplo, m, n, A, lda, strideA, B, ldb, strideB, batchCount);
}
int kblas_posv_batch(kblasHandle_t h, char side, char uplo, const int m, const int n, cuFloatComplex **A,
                     int lda, cuFloatComplex **B, int ldb, int batchCount, int *info) {
  return kblasCposv_batch(h, side, uplo, m, n, A, lda, B, ldb, batchCount, info);
}
int kblas_posv_batch(kblasHandle_t h, char side, char uplo, const int m, const int n, cuDoubleComplex **A,
                     int lda, cuDoubleComplex **B, int ldb, int batchCount, int *info) {
  return kblasZposv_batch(h, side, uplo, m, n, A, lda, B, ldb, batchCount, info);
}
int kblas_posv_batch(kblasHandle_t h, char side, char uplo, const int m, const int n, cuFloatComplex *A,
                     int lda, long strideA, cuFloatComplex *B, int ldb, long strideB, int batchCount,
                     int *info) {
  return kblasCposv_batch_strided(h, side, uplo, m, n, A, lda, strideA, B, ldb, strideB, batchCount,
                                  info);
}
int kblas_posv_batch(kblasHandle_t h, char side, char uplo, const int m, const int n, cuDoubleComplex *A,
                     int lda, long strideA, cuDoubleComplex *B, int ldb, long strideB, int batchCount,
                     int *info) {
  return kblasZposv_batch_strided(h, side, uplo, m, n, A, lda, strideA, B, ldb, strideB, batchCount,
                                  info);
}
int kblas_trsm_batch(kblasHandle_t h, char side, char uplo, char trans, char diag, const int m,
                     const int n, const cuFloatComplex alpha, const cuFloatComplex **A, int lda, cuFloatComplex **B,
                     int ldb, int batchCount) {
  return kblasCtrsm_batch(h, side, uplo, trans, diag, m, n, alpha, A, lda, B, ldb, batchCount);
}
int kblas_trsm_batch(kblasHandle_t h, char side, char uplo, char trans, char diag, const int m,
                     const int n, const cuDoubleComplex alpha, const cuDoubleComplex **A, int lda, cuDoubleComplex **B,
                     int ldb, int batchCount) {
  return kblasZtrsm_batch(h, side, uplo, trans, diag, m, n, alpha, A, lda, B, ldb, batchCount);
}
int kblas_trsm_batch(kblasHandle_t h, char side, char uplo, char trans, char diag, const int m,
                     const int n, const cuFloatComplex alpha, const cuFloatComplex *A, int lda, long strideA,
                     cuFloatComplex *B, int ldb, long strideB, int batchCount) {
  return kblasCtrsm_batch_strided(h, side, uplo, trans, diag, m, n, alpha, A, lda, strideA, B, ldb,
                                  strideB, batchCount);
}
int kblas_trsm_batch(kblasHandle_t h, char side, char uplo, char trans, char diag, const int m,
                     const int n, const cuDoubleComplex alpha, const cuDoubleComplex *A, int lda, long strideA,
                     cuDoubleComplex *B, int ldb, long strideB, int batchCount) {
  return kblasZtrsm_batch_strided(h, side, uplo, trans, diag, m, n, alpha, A, lda, strideA, B, ldb,
                                  strideB, batchCount);
}
int kblas_trmm_batch(kblasHandle_t h, char side, char uplo, char trans, char diag, const int m,
                     const int n, const cuFloatComplex alpha, const cuFloatComplex **A, int lda, cuFloatComplex **B,
                     int ldb, int batchCount) {
  return kblasCtrmm_batch(h, side, uplo, trans, diag, m, n, alpha, A, lda, B, ldb, batchCount);
}
int kblas_trmm_batch(kblasHandle_t h, char side, char uplo, char trans, char diag, const int m,
                     const int n, const cuDoubleComplex alpha, const cuDoubleComplex **A, int lda, cuDoubleComplex **B,
                     int ldb, int batchCount) {
  return kblasZtrmm_batch(h, side, uplo, trans, diag, m, n, alpha, A, lda, B, ldb, batchCount);
}
int kblas_trmm_batch(kblasHandle_t h, char side, char uplo, char trans, char diag, const int m,
                     const int n, const cuFloatComplex alpha, const cuFloatComplex *A, int lda, long strideA,
                     cuFloatComplex *B, int ldb, long strideB, int batchCount) {
  return kblasCtrmm_batch_strided(h, side, uplo, trans, diag, m, n, alpha, A, lda, strideA, B, ldb,
                                  strideB, batchCount);
}
int kblas_trmm_batch(kblasHandle_t h, char side, char uplo, char trans, char diag, const int m,
                     const int n, const cuDoubleComplex alpha, const cuDoubleComplex *A, int lda, long strideA,
                     cuDoubleComplex *B, int ldb, long strideB, int batchCount) {
  return kblasZtrmm_batch_strided(h, side, uplo, trans, diag, m, n, alpha, A, lda, strideA, B, ldb,
                                  strideB, batchCount);
}
int kblas_syrk_batch(kblasHandle_t h, char uplo, char trans, const int m, const int n,
                     const cuFloatComplex alpha, const cuFloatComplex **A, int lda, const cuFloatComplex beta, cuFloatComplex **B,
                     int ldb, int batchCount) {
  return kblasCsyrk_batch(h, uplo, trans, m, n, alpha, A, lda, beta, B, ldb, batchCount);
}
int kblas_syrk_batch(kblasHandle_t h, char uplo, char trans, const int m, const int n,
                     const cuDoubleComplex alpha, const cuDoubleComplex **A, int lda, const cuDoubleComplex beta, cuDoubleComplex **B,
                     int ldb, int batchCount) {
  return kblasZsyrk_batch(h, uplo, trans, m, n, alpha, A, lda, beta, B, ldb, batchCount);
}
int kblas_syrk_batch(kblasHandle_t h, char uplo, char trans, const int m, const int n,
                     const cuFloatComplex alpha, const cuFloatComplex *A, int lda, long strideA,
                     const cuFloatComplex beta, cuFloatComplex *B, int ldb, long strideB, int batchCount) {
  return kblasCsyrk_batch_strided(h, uplo, trans, m, n, alpha, A, lda, strideA, beta, B, ldb, strideB,
                                  batchCount);
}
int kblas_syrk_batch(kblasHandle_t h, char uplo, char trans, const int m, const int n,
                     const cuDoubleComplex alpha, const cuDoubleComplex *A, int lda, long strideA,
                     const cuDoubleComplex beta, cuDoubleComplex *B, int ldb, long strideB, int batchCount) {
  return kblasZsyrk_batch_strided(h, uplo, trans, m, n, alpha, A, lda, strideA, beta, B, ldb, strideB,
                                  batchCount);
}
int kblas_gemm_batch(kblasHandle_t h, char transA, char transB, const int m, const int n,
                     const int k, const cuFloatComplex alpha, const cuFloatComplex **A, int lda, const cuFloatComplex **B,
                     int ldb, const cuFloatComplex beta, cuFloatComplex **C, int ldc, int batchCount) {
  return kblasCgemm_batch(h, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc,
                          batchCount);
}
int kblas_gemm_batch(kblasHandle_t h, char transA, char transB, const int m, const int n,
                     const int k, const cuDoubleComplex alpha, const cuDoubleComplex **A, int lda, const cuDoubleComplex **B,
                     int ldb, const cuDoubleComplex beta, cuDoubleComplex **C, int ldc, int batchCount) {
  return kblasZgemm_batch(h, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc,
                          batchCount);
}
int kblas_gemm_batch(kblasHandle_t h, char transA, char transB, const int m, const int n,
                     const int k, const cuFloatComplex alpha, const cuFloatComplex *A, int lda, long strideA,
                     const cuFloatComplex *B, int ldb, long strideB, const cuFloatComplex beta, cuFloatComplex *C,
                     int ldc, long strideC, int batchCount) {
  return kblasCgemm_batch_strided(h, transA, transB, m, n, k, alpha, A, lda, strideA, B, ldb,
                                  strideB, beta, C, ldc, strideC, batchCount);
}
int kblas_gemm_batch(kblasHandle_t h, char transA, char transB, const int m, const int n,
                     const int k, const cuDoubleComplex alpha, const cuDoubleComplex *A, int lda, long strideA,
                     const cuDoubleComplex *B, int ldb, long strideB, const cuDoubleComplex beta, cuDoubleComplex *C,
                     int ldc, long strideC, int batchCount) {
  return kblasZgemm_batch_strided(h, transA, transB, m, n, k, alpha, A, lda, strideA, B, ldb,
                                  strideB, beta, C, ldc, strideC, batchCount);
}
int kblas_gemm_batch(kblasHandle_t h, char transA, char transB, int *m, int *n, int *k,
                     int max_m, int max_n, int max_k, const cuFloatComplex alpha, const cuFloatComplex **A,
                     int *lda, const cuFloatComplex **B, int *ldb, const cuFloatComplex beta, cuFloatComplex **C,
                     int *ldc, int batchCount) {
  return kblasCgemm_vbatch(h, transA, transB, m, n, k, max_m, max_n, max_k, alpha, A, lda, B, ldb,
                           beta, C, ldc, batchCount);
}
int kblas_gemm_batch(kblasHandle_t h, char transA, char transB, int *m, int *n, int *k,
                     int max_m, int max_n, int max_k, const cuDoubleComplex alpha, const cuDoubleComplex **A,
                     int *lda, const cuDoubleComplex **B, int *ldb, const cuDoubleComplex beta, cuDoubleComplex **C,
                     int *ldc, int batchCount) {
  return kblasZgemm_vbatch(h, transA, transB, m, n, k, max_m, max_n, max_k, alpha, A, lda, B, ldb,
                           beta, C, ldc, batchCount);
}
int kblas_syrk_batch(kblasHandle_t h, char uplo, char trans, int *m, int *n, int max_m, int max_n,
                     cuFloatComplex alpha, cuFloatComplex **A, int *lda, cuFloatComplex beta, cuFloatComplex **B, int *ldb,
                     int batchCount) {
  return kblasCsyrk_vbatch(h, uplo, trans, m, n, max_m, max_n, alpha, (const cuFloatComplex **)A, lda,
                           beta, B, ldb, batchCount);
}
int kblas_syrk_batch(kblasHandle_t h, char uplo, char trans, int *m, int *n, int max_m, int max_n,
                     cuDoubleComplex alpha, cuDoubleComplex **A, int *lda, cuDoubleComplex beta, cuDoubleComplex **B, int *ldb,
                     int batchCount) {
  return kblasZsyrk_vbatch(h, uplo, trans, m, n, max_m, max_n, alpha, (const cuDoubleComplex **)A, lda,
                           beta, B, ldb, batchCount);
}
int kblas_trsm_batch(kblasHandle_t h, char side, char uplo, char trans, char diag, int *m, int *n,
                     int max_m, int max_n, cuFloatComplex alpha, cuFloatComplex **A, int *lda, cuFloatComplex **B,
                     int *ldb, int batchCount) {
  return kblasCtrsm_vbatch(h, side, uplo, trans, diag, m, n, max_m, max_n, alpha,
                           (const cuFloatComplex **)A, lda, B, ldb, batchCount);
}
int kblas_trsm_batch(kblasHandle_t h, char side, char uplo, char trans, char diag, int *m, int *n,
                     int max_m, int max_n, cuDoubleComplex alpha, cuDoubleComplex **A, int *lda, cuDoubleComplex **B,
                     int *ldb, int batchCount) {
  return kblasZtrsm_vbatch(h, side, uplo, trans, diag, m, n, max_m, max_n, alpha,
                           (const cuDoubleComplex **)A, lda, B, ldb, batchCount);
}

// TRTRI / LAUUM / POTRI / POTI, reference include/kblas_batch.h:1627-2729.
int kblas_trtri_batch(kblasHandle_t h, char uplo, char diag, const int n, float **A, int lda,
                      int batchCount, int *info) {
  return kblasStrtri_batch(h, uplo, diag, n, A, lda, batchCount, info);
}
int kblas_trtri_batch(kblasHandle_t h, char uplo, char diag, const int n, float *A, int lda,
                      long strideA, int batchCount, int *info) {
  return kblasStrtri_batch_strided(h, uplo, diag, n, A, lda, strideA, batchCount, info);
}
int kblas_lauum_batch(kblasHandle_t h, char uplo, const int n, float **A, int lda, int batchCount,
                      int *info) {
  return kblasSlauum_batch(h, uplo, n, A, lda, batchCount, info);
}
int kblas_lauum_batch(kblasHandle_t h, char uplo, const int n, float *A, int lda, long strideA,
                      int batchCount, int *info) {
  return kblasSlauum_batch_strided(h, uplo, n, A, lda, strideA, batchCount, info);
}
int kblas_potri_batch(kblasHandle_t h, char uplo, const int n, float **A, int lda, int batchCount,
                      int *info) {
  return kblasSpotri_batch(h, uplo, n, A, lda, batchCount, info);
}
int kblas_potri_batch(kblasHandle_t h, char uplo, const int n, float *A, int lda, long strideA,
                      int batchCount, int *info) {
  return kblasSpotri_batch_strided(h, uplo, n, A, lda, strideA, batchCount, info);
}
int kblas_poti_batch(kblasHandle_t h, char uplo, const int n, float **A, int lda, int batchCount,
                      int *info) {
  return kblasSpoti_batch(h, uplo, n, A, lda, batchCount, info);
}
int kblas_poti_batch(kblasHandle_t h, char uplo, const int n, float *A, int lda, long strideA,
                      int batchCount, int *info) {
  return kblasSpoti_batch_strided(h, uplo, n, A, lda, strideA, batchCount, info);
}
int kblas_trtri_batch(kblasHandle_t h, char uplo, char diag, const int n, double **A, int lda,
                      int batchCount, int *info) {
  return kblasDtrtri_batch(h, uplo, diag, n, A, lda, batchCount, info);
}
int kblas_trtri_batch(kblasHandle_t h, char uplo, char diag, const int n, double *A, int lda,
                      long strideA, int batchCount, int *info) {
  return kblasDtrtri_batch_strided(h, uplo, diag, n, A, lda, strideA, batchCount, info);
}
int kblas_lauum_batch(kblasHandle_t h, char uplo, const int n, double **A, int lda, int batchCount,
                      int *info) {
  return kblasDlauum_batch(h, uplo, n, A, lda, batchCount, info);
}
int kblas_lauum_batch(kblasHandle_t h, char uplo, const int n, double *A, int lda, long strideA,
                      int batchCount, int *info) {
  return kblasDlauum_batch_strided(h, uplo, n, A, lda, strideA, batchCount, info);
}
int kblas_potri_batch(kblasHandle_t h, char uplo, const int n, double **A, int lda, int batchCount,
                      int *info) {
  return kblasDpotri_batch(h, uplo, n, A, lda, batchCount, info);
}
int kblas_potri_batch(kblasHandle_t h, char uplo, const int n, double *A, int lda, long strideA,
                      int batchCount, int *info) {
  return kblasDpotri_batch_strided(h, uplo, n, A, lda, strideA, batchCount, info);
}
int kblas_poti_batch(kblasHandle_t h, char uplo, const int n, double **A, int lda, int batchCount,
                      int *info) {
  return kblasDpoti_batch(h, uplo, n, A, lda, batchCount, info);
}
int kblas_poti_batch(kblasHandle_t h, char uplo, const int n, double *A, int lda, long strideA,
                      int batchCount, int *info) {
  return kblasDpoti_batch_strided(h, uplo, n, A, lda, strideA, batchCount, info);
}
int kblas_trtri_batch(kblasHandle_t h, char uplo, char diag, const int n, cuFloatComplex **A, int lda,
                      int batchCount, int *info) {
  return kblasCtrtri_batch(h, uplo, diag, n, A, lda, batchCount, info);
}
int kblas_trtri_batch(kblasHandle_t h, char uplo, char diag, const int n, cuFloatComplex *A, int lda,
                      long strideA, int batchCount, int *info) {
  return kblasCtrtri_batch_strided(h, uplo, diag, n, A, lda, strideA, batchCount, info);
}
int kblas_lauum_batch(kblasHandle_t h, char uplo, const int n, cuFloatComplex **A, int lda, int batchCount,
                      int *info) {
  return kblasClauum_batch(h, uplo, n, A, lda, batchCount, info);
}
int kblas_lauum_batch(kblasHandle_t h, char uplo, const int n, cuFloatComplex *A, int lda, long strideA,
                      int batchCount, int *info) {
  return kblasClauum_batch_strided(h, uplo, n, A, lda, strideA, batchCount, info);
}
int kblas_potri_batch(kblasHandle_t h, char uplo, const int n, cuFloatComplex **A, int lda, int batchCount,
                      int *info) {
  return kblasCpotri_batch(h, uplo, n, A, lda, batchCount, info);
}
int kblas_potri_batch(kblasHandle_t h, char uplo, const int n, cuFloatComplex *A, int lda, long strideA,
                      int batchCount, int *info) {
  return kblasCpotri_batch_strided(h, uplo, n, A, lda, strideA, batchCount, info);
}
int kblas_poti_batch(kblasHandle_t h, char uplo, const int n, cuFloatComplex **A, int lda, int batchCount,
                      int *info) {
  return kblasCpoti_batch(h, uplo, n, A, lda, batchCount, info);
}
int kblas_poti_batch(kblasHandle_t h, char uplo, const int n, cuFloatComplex *A, int lda, long strideA,
                      int batchCount, int *info) {
  return kblasCpoti_batch_strided(h, uplo, n, A, lda, strideA, batchCount, info);
}
int kblas_trtri_batch(kblasHandle_t h, char uplo, char diag, const int n, cuDoubleComplex **A, int lda,
                      int batchCount, int *info) {
  return kblasZtrtri_batch(h, uplo, diag, n, A, lda, batchCount, info);
}
int kblas_trtri_batch(kblasHandle_t h, char uplo, char diag, const int n, cuDoubleComplex *A, int lda,
                      long strideA, int batchCount, int *info) {
  return kblasZtrtri_batch_strided(h, uplo, diag, n, A, lda, strideA, batchCount, info);
}
int kblas_lauum_batch(kblasHandle_t h, char uplo, const int n, cuDoubleComplex **A, int lda, int batchCount,
                      int *info) {
  return kblasZlauum_batch(h, uplo, n, A, lda, batchCount, info);
}
int kblas_lauum_batch(kblasHandle_t h, char uplo, const int n, cuDoubleComplex *A, int lda, long strideA,
                      int batchCount, int *info) {
  return kblasZlauum_batch_strided(h, uplo, n, A, lda, strideA, batchCount, info);
}
int kblas_potri_batch(kblasHandle_t h, char uplo, const int n, cuDoubleComplex **A, int lda, int batchCount,
                      int *info) {
  return kblasZpotri_batch(h, uplo, n, A, lda, batchCount, info);
}
int kblas_potri_batch(kblasHandle_t h, char uplo, const int n, cuDoubleComplex *A, int lda, long strideA,
                      int batchCount, int *info) {
  return kblasZpotri_batch_strided(h, uplo, n, A, lda, strideA, batchCount, info);
}
int kblas_poti_batch(kblasHandle_t h, char uplo, const int n, cuDoubleComplex **A, int lda, int batchCount,
                      int *info) {
  return kblasZpoti_batch(h, uplo, n, A, lda, batchCount, info);
}
int kblas_poti_batch(kblasHandle_t h, char uplo, const int n, cuDoubleComplex *A, int lda, long strideA,
                      int batchCount, int *info) {
  return kblasZpoti_batch_strided(h, uplo, n, A, lda, strideA, batchCount, info);
}

/*
 * kblas_batch.h -- batched Cholesky / triangular routines (uniform and
 * variable size) for GB300 (sm_103a).
 *
 * The uniform-size routines keep the reference names, argument lists, storage
 * conventions and return codes of include/kblas_batch.h in the reference
 * (citations beside each group). Storage is column-major. "Strided" forms take
 * one device buffer and a stride in elements between consecutive matrices;
 * the other forms take a DEVICE array of device pointers (the reference's
 * kernels dereference the array on the device, e.g.
 * src/batch_triangular/Xpotrf_batch_kernels.cuh:96).
 *
 * Conventions shared by every routine:
 *  - all work is queued on the handle's stream; nothing synchronises the host
 *    and nothing allocates memory, so the calls can be captured in CUDA graphs
 *    once the workspace is allocated;
 *  - info arrays are device int[batchCount]; 0 = success, +j = the leading
 *    minor of order j is not positive definite (LAPACK xPOTRF semantics, the
 *    meaning documented at reference include/kblas_batch.h:1482);
 *  - flag combinations the reference leaves unimplemented (it returns
 *    KBLAS_NotImplemented) run here: Upper POTRF / POTRS / POSV / SYRK /
 *    TRTRI / LAUUM / POTRI / POTI and side 'L' POTRS / POSV; TRSM/TRMM
 *    implement Upper, Unit and Right natively, which
 *    the reference only reaches through MAGMA.
 */
#ifndef KBLAS_GB300_BATCH_H
#define KBLAS_GB300_BATCH_H

#include <cuComplex.h>
#include <cuda_runtime_api.h>
#include "kblas_defs.h"

#ifdef __cplusplus
extern "C" {
#endif

struct KBlasHandle;
typedef struct KBlasHandle *kblasHandle_t;

/* ---------------------------------------------------------------------------
 * Workspace queries (reference include/kblas_batch.h:485,773,786,1100,1113,
 * 1380,1391,2077,2089,2772,2785). Each call raises the handle's requested
 * workspace to what the routine needs; kblasAllocateWorkspace then allocates.
 * SYRK, TRSM and TRMM need none (zero-byte requests, kept so KBLAS callers
 * link unchanged). The double-precision POTRF / POTRS / POSV of order 33..1024
 * request scratch for the persistent panel kernel and run on it once the
 * workspace is allocated; without it they run on a one-launch blocked kernel
 * that needs none but is several times slower at small orders (about 14% of
 * the FP64 peak at n = 64 against 33% with the workspace). Call the query and
 * kblasAllocateWorkspace, as KBLAS callers do, before timing these routines.
 * ------------------------------------------------------------------------- */
void kblas_syrk_batch_wsquery(kblasHandle_t handle, const int m, int batchCount);
void kblas_trsm_batch_wsquery(kblasHandle_t handle, char side, int m, int n, int batchCount);
void kblas_trsm_batch_strided_wsquery(kblasHandle_t handle, char side, int m, int n, int batchCount);
void kblas_trmm_batch_wsquery(kblasHandle_t handle, char side, int m, int n, int batchCount);
void kblas_trmm_batch_strided_wsquery(kblasHandle_t handle, char side, int m, int n, int batchCount);
void kblas_potrf_batch_wsquery(kblasHandle_t handle, const int n, int batchCount);
void kblas_potrf_batch_strided_wsquery(kblasHandle_t handle, const int n, int batchCount);
void kblas_potrs_batch_wsquery(kblasHandle_t handle, const int m, const int n, int batchCount);
void kblas_potrs_batch_strided_wsquery(kblasHandle_t handle, const int m, const int n, int batchCount);
void kblas_posv_batch_wsquery(kblasHandle_t handle, char side, const int m, const int n, int batchCount);
void kblas_posv_batch_strided_wsquery(kblasHandle_t handle, char side, const int m, const int n, int batchCount);

/* ---------------------------------------------------------------------------
 * SYRK: B := alpha*op(A)*op(A)^T + beta*B on the uplo triangle of B (m x m);
 * op(A) is m x n (trans = 'N') or A is n x m (trans = 'T').
 * reference include/kblas_batch.h:631-728 (uplo = 'U' is KBLAS_NotImplemented
 * there, src/batch_triangular/Xsyrk_batch_drivers.cuh:133-136; supported here).
 * ------------------------------------------------------------------------- */
int kblasSsyrk_batch(kblasHandle_t handle, char uplo, char trans, const int m, const int n,
                     const float alpha, const float **A_array, int lda,
                     const float beta, float **B_array, int ldb, int batchCount);
int kblasDsyrk_batch(kblasHandle_t handle, char uplo, char trans, const int m, const int n,
                     const double alpha, const double **A_array, int lda,
                     const double beta, double **B_array, int ldb, int batchCount);
int kblasSsyrk_batch_strided(kblasHandle_t handle, char uplo, char trans, const int m, const int n,
                             const float alpha, const float *A, int lda, long strideA,
                             const float beta, float *B, int ldb, long strideB, int batchCount);
int kblasDsyrk_batch_strided(kblasHandle_t handle, char uplo, char trans, const int m, const int n,
                             const double alpha, const double *A, int lda, long strideA,
                             const double beta, double *B, int ldb, long strideB, int batchCount);

/* ---------------------------------------------------------------------------
 * TRSM: solve op(A)*X = alpha*B (side 'L', A m x m) or X*op(A) = alpha*B
 * (side 'R', A n x n); B is m x n and is overwritten by X.
 * reference include/kblas_batch.h:948-1053.
 * ------------------------------------------------------------------------- */
int kblasStrsm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag,
                     const int m, const int n, const float alpha,
                     const float **A_array, int lda, float **B_array, int ldb, int batchCount);
int kblasDtrsm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag,
                     const int m, const int n, const double alpha,
                     const double **A_array, int lda, double **B_array, int ldb, int batchCount);
int kblasStrsm_batch_strided(kblasHandle_t handle, char side, char uplo, char trans, char diag,
                             const int m, const int n, const float alpha,
                             const float *A, int lda, long strideA,
                             float *B, int ldb, long strideB, int batchCount);
int kblasDtrsm_batch_strided(kblasHandle_t handle, char side, char uplo, char trans, char diag,
                             const int m, const int n, const double alpha,
                             const double *A, int lda, long strideA,
                             double *B, int ldb, long strideB, int batchCount);

/* ---------------------------------------------------------------------------
 * TRMM: B := alpha*op(A)*B (side 'L') or alpha*B*op(A) (side 'R').
 * reference include/kblas_batch.h:1232-1335.
 * ------------------------------------------------------------------------- */
int kblasStrmm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag,
                     const int m, const int n, const float alpha,
                     const float **A_array, int lda, float **B_array, int ldb, int batchCount);
int kblasDtrmm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag,
                     const int m, const int n, const double alpha,
                     const double **A_array, int lda, double **B_array, int ldb, int batchCount);
int kblasStrmm_batch_strided(kblasHandle_t handle, char side, char uplo, char trans, char diag,
                             const int m, const int n, const float alpha,
                             const float *A, int lda, long strideA,
                             float *B, int ldb, long strideB, int batchCount);
int kblasDtrmm_batch_strided(kblasHandle_t handle, char side, char uplo, char trans, char diag,
                             const int m, const int n, const double alpha,
                             const double *A, int lda, long strideA,
                             double *B, int ldb, long strideB, int batchCount);

/* ---------------------------------------------------------------------------
 * POTRF: A = L*L^T (uplo 'L') or A = U^T*U (uplo 'U', KBLAS_NotImplemented in
 * the reference) in place; only the uplo triangle is read and written.
 * reference include/kblas_batch.h:1486-1566.
 * ------------------------------------------------------------------------- */
int kblasSpotrf_batch(kblasHandle_t handle, char uplo, const int n,
                      float **A_array, int lda, int batchCount, int *info_array);
int kblasDpotrf_batch(kblasHandle_t handle, char uplo, const int n,
                      double **A_array, int lda, int batchCount, int *info_array);
int kblasSpotrf_batch_strided(kblasHandle_t handle, char uplo, const int n,
                              float *A, int lda, long strideA, int batchCount, int *info_array);
int kblasDpotrf_batch_strided(kblasHandle_t handle, char uplo, const int n,
                              double *A, int lda, long strideA, int batchCount, int *info_array);

/* ---------------------------------------------------------------------------
 * POTRS: solve X*A = B (side 'R', A n x n) or A*X = B (side 'L', A m x m)
 * with A = L*L^T or U^T*U given by its factor (uplo 'L' / 'U'); B is m x n
 * and is overwritten by X. reference include/kblas_batch.h:2190-2278 (side
 * 'R' + uplo 'L' only there; the other three run as two TRSM passes here).
 * ------------------------------------------------------------------------- */
int kblasSpotrs_batch(kblasHandle_t handle, char side, char uplo, const int m, const int n,
                      const float **A_array, int lda, float **B_array, int ldb, int batchCount);
int kblasDpotrs_batch(kblasHandle_t handle, char side, char uplo, const int m, const int n,
                      const double **A_array, int lda, double **B_array, int ldb, int batchCount);
int kblasSpotrs_batch_strided(kblasHandle_t handle, char side, char uplo, const int m, const int n,
                              const float *A, int lda, long strideA,
                              float *B, int ldb, long strideB, int batchCount);
int kblasDpotrs_batch_strided(kblasHandle_t handle, char side, char uplo, const int m, const int n,
                              const double *A, int lda, long strideA,
                              double *B, int ldb, long strideB, int batchCount);

/* ---------------------------------------------------------------------------
 * POSV: POTRF then POTRS, fused into one kernel per size class for side 'R'
 * (either uplo); side 'L' factors, then solves with two TRSM passes. On exit A
 * holds the factor and B holds X; for a matrix with info > 0, B is left
 * unchanged (LAPACK xPOSV). reference include/kblas_batch.h:2896-2988.
 * ------------------------------------------------------------------------- */
int kblasSposv_batch(kblasHandle_t handle, char side, char uplo, const int m, const int n,
                     float **A_array, int lda, float **B_array, int ldb,
                     int batchCount, int *info_array);
int kblasDposv_batch(kblasHandle_t handle, char side, char uplo, const int m, const int n,
                     double **A_array, int lda, double **B_array, int ldb,
                     int batchCount, int *info_array);
int kblasSposv_batch_strided(kblasHandle_t handle, char side, char uplo, const int m, const int n,
                             float *A, int lda, long strideA, float *B, int ldb, long strideB,
                             int batchCount, int *info_array);
int kblasDposv_batch_strided(kblasHandle_t handle, char side, char uplo, const int m, const int n,
                             double *A, int lda, long strideA, double *B, int ldb, long strideB,
                             int batchCount, int *info_array);

/* ---------------------------------------------------------------------------
 * Inversion: TRTRI (inverse of a triangular matrix), LAUUM (L^T L or U U^T),
 * POTRI (inverse of A from its Cholesky factor) and POTI (inverse of an SPD
 * A), either triangle (the reference: lower only), in place. reference include/kblas_batch.h:1611-2729.
 * info as LAPACK: TRTRI / POTRI give the first zero diagonal entry (A then
 * unchanged), POTI the first non-positive pivot of its Cholesky step. TRTRI
 * also accepts diag = 'U' (the reference: non-unit only). No workspace.
 * ------------------------------------------------------------------------- */
void kblas_trtri_batch_wsquery(kblasHandle_t handle, const int n, int batchCount);
void kblas_trtri_batch_strided_wsquery(kblasHandle_t handle, const int n, int batchCount);
void kblas_lauum_batch_wsquery(kblasHandle_t handle, const int n, int batchCount);
void kblas_lauum_batch_strided_wsquery(kblasHandle_t handle, const int n, int batchCount);
void kblas_potri_batch_wsquery(kblasHandle_t handle, const int n, int batchCount);
void kblas_potri_batch_strided_wsquery(kblasHandle_t handle, const int n, int batchCount);
void kblas_poti_batch_wsquery(kblasHandle_t handle, const int n, int batchCount);
void kblas_poti_batch_strided_wsquery(kblasHandle_t handle, const int n, int batchCount);
int kblasStrtri_batch(kblasHandle_t handle, char uplo, char diag, const int n, float **A_array,
                      int lda, int batchCount, int *info_array);
int kblasDtrtri_batch(kblasHandle_t handle, char uplo, char diag, const int n, double **A_array,
                      int lda, int batchCount, int *info_array);
int kblasStrtri_batch_strided(kblasHandle_t handle, char uplo, char diag, const int n, float *A,
                              int lda, long strideA, int batchCount, int *info_array);
int kblasDtrtri_batch_strided(kblasHandle_t handle, char uplo, char diag, const int n, double *A,
                              int lda, long strideA, int batchCount, int *info_array);
int kblasSlauum_batch(kblasHandle_t handle, char uplo, const int n, float **A_array, int lda,
                      int batchCount, int *info_array);
int kblasDlauum_batch(kblasHandle_t handle, char uplo, const int n, double **A_array, int lda,
                      int batchCount, int *info_array);
int kblasSlauum_batch_strided(kblasHandle_t handle, char uplo, const int n, float *A, int lda,
                              long strideA, int batchCount, int *info_array);
int kblasDlauum_batch_strided(kblasHandle_t handle, char uplo, const int n, double *A, int lda,
                              long strideA, int batchCount, int *info_array);
int kblasSpotri_batch(kblasHandle_t handle, char uplo, const int n, float **A_array, int lda,
                      int batchCount, int *info_array);
int kblasDpotri_batch(kblasHandle_t handle, char uplo, const int n, double **A_array, int lda,
                      int batchCount, int *info_array);
int kblasSpotri_batch_strided(kblasHandle_t handle, char uplo, const int n, float *A, int lda,
                              long strideA, int batchCount, int *info_array);
int kblasDpotri_batch_strided(kblasHandle_t handle, char uplo, const int n, double *A, int lda,
                              long strideA, int batchCount, int *info_array);
int kblasSpoti_batch(kblasHandle_t handle, char uplo, const int n, float **A_array, int lda,
                     int batchCount, int *info_array);
int kblasDpoti_batch(kblasHandle_t handle, char uplo, const int n, double **A_array, int lda,
                     int batchCount, int *info_array);
int kblasSpoti_batch_strided(kblasHandle_t handle, char uplo, const int n, float *A, int lda,
                             long strideA, int batchCount, int *info_array);
int kblasDpoti_batch_strided(kblasHandle_t handle, char uplo, const int n, double *A, int lda,
                             long strideA, int batchCount, int *info_array);

/* ---------------------------------------------------------------------------
 * GEMM: C := alpha*op(A)*op(B) + beta*C, op(A) m x k, op(B) k x n.
 * reference include/kblas_batch.h:35-36 (wsqueries), :309-460 (C names;
 * cuBLAS there, a native tile kernel here). batchCount < 1 ->
 * KBLAS_Error_WrongInput, as the reference. No workspace.
 * ------------------------------------------------------------------------- */
void kblas_gemm_batch_strided_wsquery(kblasHandle_t handle, int batchCount);
void kblas_gemm_batch_nonuniform_wsquery(kblasHandle_t handle);
int kblasSgemm_batch(kblasHandle_t handle, char transA, char transB, const int m, const int n,
                     const int k, const float alpha, const float **A, int lda, const float **B,
                     int ldb, const float beta, float **C, int ldc, int batchCount);
int kblasDgemm_batch(kblasHandle_t handle, char transA, char transB, const int m, const int n,
                     const int k, const double alpha, const double **A, int lda,
                     const double **B, int ldb, const double beta, double **C, int ldc,
                     int batchCount);
int kblasSgemm_batch_strided(kblasHandle_t handle, char transA, char transB, const int m,
                             const int n, const int k, const float alpha, const float *A, int lda,
                             long strideA, const float *B, int ldb, long strideB, const float beta,
                             float *C, int ldc, long strideC, int batchCount);
int kblasDgemm_batch_strided(kblasHandle_t handle, char transA, char transB, const int m,
                             const int n, const int k, const double alpha, const double *A,
                             int lda, long strideA, const double *B, int ldb, long strideB,
                             const double beta, double *C, int ldc, long strideC, int batchCount);

/* ---------------------------------------------------------------------------
 * Variable-size GEMM / SYRK / TRSM. The reference has these as C++ overloads
 * of kblas_{gemm,syrk,trsm}_batch taking per-matrix sizes and leading
 * dimensions in DEVICE int arrays (include/kblas_batch.h:201-245, :524-550,
 * :829-860; MAGMA-only there); these are their C names, and the overloads
 * below forward to them. max_* are host-side upper bounds of the sizes; all
 * of them <= 0 means "unknown". GEMM and SYRK need no bound (it only sizes
 * the grid) and no workspace. TRSM sizes its shared-memory layout from the
 * bound: when max_m and max_n are both <= 0 it recomputes them on the device
 * into the workspace kblas_trsm_batch_nonuniform_wsquery requests, and
 * synchronises the stream (as the reference). Per-matrix sizes are not
 * validated; matrices with a size <= 0 are skipped. SYRK accepts uplo 'L'
 * and 'U'; TRSM every side / uplo / trans / diag.
 * ------------------------------------------------------------------------- */
void kblas_syrk_batch_nonuniform_wsquery(kblasHandle_t handle);
void kblas_trsm_batch_nonuniform_wsquery(kblasHandle_t handle);
int kblasSgemm_vbatch(kblasHandle_t handle, char transA, char transB, int *m, int *n, int *k,
                      int max_m, int max_n, int max_k, const float alpha, const float **A,
                      int *lda, const float **B, int *ldb, const float beta, float **C, int *ldc,
                      int batchCount);
int kblasDgemm_vbatch(kblasHandle_t handle, char transA, char transB, int *m, int *n, int *k,
                      int max_m, int max_n, int max_k, const double alpha, const double **A,
                      int *lda, const double **B, int *ldb, const double beta, double **C,
                      int *ldc, int batchCount);
int kblasSsyrk_vbatch(kblasHandle_t handle, char uplo, char trans, int *m, int *n, int max_m,
                      int max_n, const float alpha, const float **A, int *lda, const float beta,
                      float **B, int *ldb, int batchCount);
int kblasDsyrk_vbatch(kblasHandle_t handle, char uplo, char trans, int *m, int *n, int max_m,
                      int max_n, const double alpha, const double **A, int *lda,
                      const double beta, double **B, int *ldb, int batchCount);
int kblasStrsm_vbatch(kblasHandle_t handle, char side, char uplo, char trans, char diag, int *m,
                      int *n, int max_m, int max_n, const float alpha, const float **A, int *lda,
                      float **B, int *ldb, int batchCount);
int kblasDtrsm_vbatch(kblasHandle_t handle, char side, char uplo, char trans, char diag, int *m,
                      int *n, int max_m, int max_n, const double alpha, const double **A,
                      int *lda, double **B, int *ldb, int batchCount);


/* ---------------------------------------------------------------------------
 * Complex precisions C (cuFloatComplex) and Z (cuDoubleComplex) of every
 * routine above, reference include/kblas_batch.h (kblas{C,Z}* names, e.g.
 * :339-354, :438-453 for GEMM). As in the reference, these are the
 * complex-symmetric forms: POTRF factors A = L*L^T (no conjugation; a pivot
 * fails when it is zero or not finite, and its square root is the principal
 * one), op = transpose for TRSM / TRMM / GEMM, SYRK forms A*A^T; the
 * reference's tests build complex-symmetric matrices
 * (testing/testing_helper.cu:405-414). Arguments, flags and return codes as
 * for the real routines.
 * ------------------------------------------------------------------------- */
int kblasCsyrk_batch(kblasHandle_t handle, char uplo, char trans, const int m, const int n,
                     const cuFloatComplex alpha, const cuFloatComplex **A_array, int lda,
                     const cuFloatComplex beta, cuFloatComplex **B_array, int ldb, int batchCount);
int kblasZsyrk_batch(kblasHandle_t handle, char uplo, char trans, const int m, const int n,
                     const cuDoubleComplex alpha, const cuDoubleComplex **A_array, int lda,
                     const cuDoubleComplex beta, cuDoubleComplex **B_array, int ldb, int batchCount);
int kblasCsyrk_batch_strided(kblasHandle_t handle, char uplo, char trans, const int m, const int n,
                             const cuFloatComplex alpha, const cuFloatComplex *A, int lda, long strideA,
                             const cuFloatComplex beta, cuFloatComplex *B, int ldb, long strideB, int batchCount);
int kblasZsyrk_batch_strided(kblasHandle_t handle, char uplo, char trans, const int m, const int n,
                             const cuDoubleComplex alpha, const cuDoubleComplex *A, int lda, long strideA,
                             const cuDoubleComplex beta, cuDoubleComplex *B, int ldb, long strideB, int batchCount);
int kblasCtrsm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag,
                     const int m, const int n, const cuFloatComplex alpha,
                     const cuFloatComplex **A_array, int lda, cuFloatComplex **B_array, int ldb, int batchCount);
int kblasZtrsm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag,
                     const int m, const int n, const cuDoubleComplex alpha,
                     const cuDoubleComplex **A_array, int lda, cuDoubleComplex **B_array, int ldb, int batchCount);
int kblasCtrsm_batch_strided(kblasHandle_t handle, char side, char uplo, char trans, char diag,
                             const int m, const int n, const cuFloatComplex alpha,
                             const cuFloatComplex *A, int lda, long strideA,
                             cuFloatComplex *B, int ldb, long strideB, int batchCount);
int kblasZtrsm_batch_strided(kblasHandle_t handle, char side, char uplo, char trans, char diag,
                             const int m, const int n, const cuDoubleComplex alpha,
                             const cuDoubleComplex *A, int lda, long strideA,
                             cuDoubleComplex *B, int ldb, long strideB, int batchCount);
int kblasCtrmm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag,
                     const int m, const int n, const cuFloatComplex alpha,
                     const cuFloatComplex **A_array, int lda, cuFloatComplex **B_array, int ldb, int batchCount);
int kblasZtrmm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag,
                     const int m, const int n, const cuDoubleComplex alpha,
                     const cuDoubleComplex **A_array, int lda, cuDoubleComplex **B_array, int ldb, int batchCount);
int kblasCtrmm_batch_strided(kblasHandle_t handle, char side, char uplo, char trans, char diag,
                             const int m, const int n, const cuFloatComplex alpha,
                             const cuFloatComplex *A, int lda, long strideA,
                             cuFloatComplex *B, int ldb, long strideB, int batchCount);
int kblasZtrmm_batch_strided(kblasHandle_t handle, char side, char uplo, char trans, char diag,
                             const int m, const int n, const cuDoubleComplex alpha,
                             const cuDoubleComplex *A, int lda, long strideA,
                             cuDoubleComplex *B, int ldb, long strideB, int batchCount);
int kblasCpotrf_batch(kblasHandle_t handle, char uplo, const int n,
                      cuFloatComplex **A_array, int lda, int batchCount, int *info_array);
int kblasZpotrf_batch(kblasHandle_t handle, char uplo, const int n,
                      cuDoubleComplex **A_array, int lda, int batchCount, int *info_array);
int kblasCpotrf_batch_strided(kblasHandle_t handle, char uplo, const int n,
                              cuFloatComplex *A, int lda, long strideA, int batchCount, int *info_array);
int kblasZpotrf_batch_strided(kblasHandle_t handle, char uplo, const int n,
                              cuDoubleComplex *A, int lda, long strideA, int batchCount, int *info_array);
int kblasCpotrs_batch(kblasHandle_t handle, char side, char uplo, const int m, const int n,
                      const cuFloatComplex **A_array, int lda, cuFloatComplex **B_array, int ldb, int batchCount);
int kblasZpotrs_batch(kblasHandle_t handle, char side, char uplo, const int m, const int n,
                      const cuDoubleComplex **A_array, int lda, cuDoubleComplex **B_array, int ldb, int batchCount);
int kblasCpotrs_batch_strided(kblasHandle_t handle, char side, char uplo, const int m, const int n,
                              const cuFloatComplex *A, int lda, long strideA,
                              cuFloatComplex *B, int ldb, long strideB, int batchCount);
int kblasZpotrs_batch_strided(kblasHandle_t handle, char side, char uplo, const int m, const int n,
                              const cuDoubleComplex *A, int lda, long strideA,
                              cuDoubleComplex *B, int ldb, long strideB, int batchCount);
int kblasCposv_batch(kblasHandle_t handle, char side, char uplo, const int m, const int n,
                     cuFloatComplex **A_array, int lda, cuFloatComplex **B_array, int ldb,
                     int batchCount, int *info_array);
int kblasZposv_batch(kblasHandle_t handle, char side, char uplo, const int m, const int n,
                     cuDoubleComplex **A_array, int lda, cuDoubleComplex **B_array, int ldb,
                     int batchCount, int *info_array);
int kblasCposv_batch_strided(kblasHandle_t handle, char side, char uplo, const int m, const int n,
                             cuFloatComplex *A, int lda, long strideA, cuFloatComplex *B, int ldb, long strideB,
                             int batchCount, int *info_array);
int kblasZposv_batch_strided(kblasHandle_t handle, char side, char uplo, const int m, const int n,
                             cuDoubleComplex *A, int lda, long strideA, cuDoubleComplex *B, int ldb, long strideB,
                             int batchCount, int *info_array);
int kblasCtrtri_batch(kblasHandle_t handle, char uplo, char diag, const int n, cuFloatComplex **A_array,
                      int lda, int batchCount, int *info_array);
int kblasZtrtri_batch(kblasHandle_t handle, char uplo, char diag, const int n, cuDoubleComplex **A_array,
                      int lda, int batchCount, int *info_array);
int kblasCtrtri_batch_strided(kblasHandle_t handle, char uplo, char diag, const int n, cuFloatComplex *A,
                              int lda, long strideA, int batchCount, int *info_array);
int kblasZtrtri_batch_strided(kblasHandle_t handle, char uplo, char diag, const int n, cuDoubleComplex *A,
                              int lda, long strideA, int batchCount, int *info_array);
int kblasClauum_batch(kblasHandle_t handle, char uplo, const int n, cuFloatComplex **A_array, int lda,
                      int batchCount, int *info_array);
int kblasZlauum_batch(kblasHandle_t handle, char uplo, const int n, cuDoubleComplex **A_array, int lda,
                      int batchCount, int *info_array);
int kblasClauum_batch_strided(kblasHandle_t handle, char uplo, const int n, cuFloatComplex *A, int lda,
                              long strideA, int batchCount, int *info_array);
int kblasZlauum_batch_strided(kblasHandle_t handle, char uplo, const int n, cuDoubleComplex *A, int lda,
                              long strideA, int batchCount, int *info_array);
int kblasCpotri_batch(kblasHandle_t handle, char uplo, const int n, cuFloatComplex **A_array, int lda,
                      int batchCount, int *info_array);
int kblasZpotri_batch(kblasHandle_t handle, char uplo, const int n, cuDoubleComplex **A_array, int lda,
                      int batchCount, int *info_array);
int kblasCpotri_batch_strided(kblasHandle_t handle, char uplo, const int n, cuFloatComplex *A, int lda,
                              long strideA, int batchCount, int *info_array);
int kblasZpotri_batch_strided(kblasHandle_t handle, char uplo, const int n, cuDoubleComplex *A, int lda,
                              long strideA, int batchCount, int *info_array);
int kblasCpoti_batch(kblasHandle_t handle, char uplo, const int n, cuFloatComplex **A_array, int lda,
                     int batchCount, int *info_array);
int kblasZpoti_batch(kblasHandle_t handle, char uplo, const int n, cuDoubleComplex **A_array, int lda,
                     int batchCount, int *info_array);
int kblasCpoti_batch_strided(kblasHandle_t handle, char uplo, const int n, cuFloatComplex *A, int lda,
                             long strideA, int batchCount, int *info_array);
int kblasZpoti_batch_strided(kblasHandle_t handle, char uplo, const int n, cuDoubleComplex *A, int lda,
                             long strideA, int batchCount, int *info_array);
int kblasCgemm_batch(kblasHandle_t handle, char transA, char transB, const int m, const int n,
                     const int k, const cuFloatComplex alpha, const cuFloatComplex **A, int lda,
                     const cuFloatComplex **B, int ldb, const cuFloatComplex beta, cuFloatComplex **C, int ldc,
                     int batchCount);
int kblasZgemm_batch(kblasHandle_t handle, char transA, char transB, const int m, const int n,
                     const int k, const cuDoubleComplex alpha, const cuDoubleComplex **A, int lda,
                     const cuDoubleComplex **B, int ldb, const cuDoubleComplex beta, cuDoubleComplex **C, int ldc,
                     int batchCount);
int kblasCgemm_batch_strided(kblasHandle_t handle, char transA, char transB, const int m,
                             const int n, const int k, const cuFloatComplex alpha, const cuFloatComplex *A,
                             int lda, long strideA, const cuFloatComplex *B, int ldb, long strideB,
                             const cuFloatComplex beta, cuFloatComplex *C, int ldc, long strideC, int batchCount);
int kblasZgemm_batch_strided(kblasHandle_t handle, char transA, char transB, const int m,
                             const int n, const int k, const cuDoubleComplex alpha, const cuDoubleComplex *A,
                             int lda, long strideA, const cuDoubleComplex *B, int ldb, long strideB,
                             const cuDoubleComplex beta, cuDoubleComplex *C, int ldc, long strideC, int batchCount);
int kblasCgemm_vbatch(kblasHandle_t handle, char transA, char transB, int *m, int *n, int *k,
                      int max_m, int max_n, int max_k, const cuFloatComplex alpha, const cuFloatComplex **A,
                      int *lda, const cuFloatComplex **B, int *ldb, const cuFloatComplex beta, cuFloatComplex **C,
                      int *ldc, int batchCount);
int kblasZgemm_vbatch(kblasHandle_t handle, char transA, char transB, int *m, int *n, int *k,
                      int max_m, int max_n, int max_k, const cuDoubleComplex alpha, const cuDoubleComplex **A,
                      int *lda, const cuDoubleComplex **B, int *ldb, const cuDoubleComplex beta, cuDoubleComplex **C,
                      int *ldc, int batchCount);
int kblasCsyrk_vbatch(kblasHandle_t handle, char uplo, char trans, int *m, int *n, int max_m,
                      int max_n, const cuFloatComplex alpha, const cuFloatComplex **A, int *lda,
                      const cuFloatComplex beta, cuFloatComplex **B, int *ldb, int batchCount);
int kblasZsyrk_vbatch(kblasHandle_t handle, char uplo, char trans, int *m, int *n, int max_m,
                      int max_n, const cuDoubleComplex alpha, const cuDoubleComplex **A, int *lda,
                      const cuDoubleComplex beta, cuDoubleComplex **B, int *ldb, int batchCount);
int kblasCtrsm_vbatch(kblasHandle_t handle, char side, char uplo, char trans, char diag, int *m,
                      int *n, int max_m, int max_n, const cuFloatComplex alpha, const cuFloatComplex **A,
                      int *lda, cuFloatComplex **B, int *ldb, int batchCount);
int kblasZtrsm_vbatch(kblasHandle_t handle, char side, char uplo, char trans, char diag, int *m,
                      int *n, int max_m, int max_n, const cuDoubleComplex alpha, const cuDoubleComplex **A,
                      int *lda, cuDoubleComplex **B, int *ldb, int batchCount);

/* ===========================================================================
 * Extensions with no reference counterpart.
 * ========================================================================= */

/* Mixed-precision POSV (semantics of LAPACK DSPOSV, batched). The factor is
 * computed in FP32 after symmetric diagonal scaling; each system is refined
 * in FP64 (residual b - A*x and the update of x) until its computed normwise
 * backward error certifies a true one of at most 10*n*eps64 (computed value
 * <= (9n-2)*eps64, eps64 = 2^-53); a system whose refinement stalls, or whose
 * FP32 factorization meets a non-positive or tiny pivot, is re-solved with
 * the FP64 factorization. iter_array (device int[batchCount], may be NULL):
 * >= 0 refinement steps taken (A is unchanged); < 0 the FP64 path was used
 * (A holds L): -1 FP32 pivot test failed, -2 refinement stalled (error not
 * halved by a step, or contracting too slowly for the remaining steps to cost
 * less than the FP64 factorization), -3 step cap, -4 routed to the FP64 path
 * before any refinement by the conditioning estimate of kblasSetPosvRouting.
 * info_array as for POSV. Needs workspace: kblas_posv_batch_mixed_wsquery. */
void kblas_posv_batch_mixed_wsquery(kblasHandle_t handle, char side, const int m, const int n,
                                    int batchCount);
int kblasDposv_batch_mixed_strided(kblasHandle_t handle, char side, char uplo,
                                   const int m, const int n,
                                   double *A, int lda, long strideA,
                                   double *B, int ldb, long strideB,
                                   int batchCount, int *info_array, int *iter_array);
int kblasDposv_batch_mixed(kblasHandle_t handle, char side, char uplo,
                           const int m, const int n,
                           double **A_array, int lda, double **B_array, int ldb,
                           int batchCount, int *info_array, int *iter_array);

/* Variable-size POSV in one persistent launch. m, n, lda, ldb are DEVICE
 * int[batchCount] (the non-uniform convention of reference
 * include/kblas_batch.h:829-845); max_m / max_n bound them. Matrices are
 * binned by size class on the device, then one persistent kernel pulls work
 * items from a device queue, factorizes, solves and (for _mixed) refines each
 * system while it is resident on chip. No host synchronisation: the sequence
 * can be captured in a CUDA graph. Needs workspace: kblas_posv_vbatch_wsquery.
 * A non-positive n or an out-of-range lda/ldb gives info = -(argument index). */
void kblas_posv_vbatch_wsquery(kblasHandle_t handle, const int max_n, int batchCount);
int kblasDposv_vbatch(kblasHandle_t handle, char side, char uplo,
                      int *m, int *n, int max_m, int max_n,
                      double **A_array, int *lda, double **B_array, int *ldb,
                      int batchCount, int *info_array);
int kblasDposv_vbatch_mixed(kblasHandle_t handle, char side, char uplo,
                            int *m, int *n, int max_m, int max_n,
                            double **A_array, int *lda, double **B_array, int *ldb,
                            int batchCount, int *info_array, int *iter_array);

/* Override the launch-shape table of the persistent POSV kernels (mixed != 0:
 * the mixed-precision table, else the plain FP64 one): per size class, the
 * largest order n of the class, the team size in threads (8..256, a power of
 * two) and the systems per work item. KBLAS_POSV_TUNING_CLASSES entries each;
 * NULL restores the table compiled into the library. Used by the committed
 * autotuner. */
#define KBLAS_POSV_TUNING_CLASSES 8
int kblasSetPosvTuning(int mixed, const int *nmax, const int *ts, const int *spi);

/* Routing constant of the mixed-precision POSV: after the FP32
 * factorization, a system whose predicted refinement (contraction estimated
 * as c * 2^-24 / d_min, d_min the smallest pivot of the scaled factor) would
 * cost more FP64 work than the FP64 factorization goes straight to the FP64
 * path (iter = -4). c > 0 sets the constant, c == 0 turns the routing off,
 * c < 0 restores the compiled one. Used by the committed autotuner. */
int kblasSetPosvRouting(double c);

/* Allocation-free mixed-precision POSV (no counterpart in the reference).
 * Same arguments, semantics and results as kblasDposv_batch_mixed_strided,
 * but it takes a CUDA stream instead of a handle and allocates nothing: its
 * scratch is one fixed array per device in the library's device image. For
 * callers that cannot allocate when they solve (a framework that owns all
 * device memory, a latency-bound loop where cudaMalloc / cudaFree would stall
 * or fail). Limits: n <= KBLAS_POSV_NOALLOC_MAX_N, else a message and
 * KBLAS_NotSupported; scratch KBLAS_POSV_NOALLOC_SCRATCH_BYTES per device.
 * Every call looks up the array's address in the calling thread's current
 * context (no address is cached across calls, so the routine stays correct
 * after cudaDeviceReset and under non-primary contexts); the first call in a
 * context loads that part of the library's image: make it before any stream
 * capture.
 * All calls on a device share the array, so calls that overlap in time
 * (different streams without ordering) race and give wrong results; calls in
 * one stream are safe. */
#define KBLAS_POSV_NOALLOC_MAX_N 256
#define KBLAS_POSV_NOALLOC_SCRATCH_BYTES (64u << 20)
int kblasDposv_batch_mixed_strided_noalloc(cudaStream_t stream, char side, char uplo,
                                           const int m, const int n,
                                           double *A, int lda, long strideA,
                                           double *B, int ldb, long strideB,
                                           int batchCount, int *info_array, int *iter_array);

/* Device status word of the handle's mixed-precision launches (no reference
 * counterpart): KBLAS_Success, or KBLAS_Error_Timeout if, in any launch since
 * the last read, a bounded device-side wait for the tensor-core MMAs ran out
 * (that launch stopped without writing its results). Synchronises the handle's
 * stream and clears the word. */
int kblasGetDeviceStatus(kblasHandle_t handle);

#ifdef __cplusplus
}
#endif

#ifdef __cplusplus
/* C++ overloads, reference include/kblas_batch.h:82-245 (GEMM), 493-576 (SYRK),
 * 794-891 (TRSM), 1119-1177 (TRMM), 1396-1452 (POTRF), 1627-2729 (TRTRI / LAUUM /
 * POTRI / POTI), 2094-2152 (POTRS), 2790-2855 (POSV); S, D, C, Z. */
int kblas_potrf_batch(kblasHandle_t handle, char uplo, const int n, float **A, int lda, int batchCount,
                      int *info);
int kblas_potrf_batch(kblasHandle_t handle, char uplo, const int n, double **A, int lda, int batchCount,
                      int *info);
int kblas_potrf_batch(kblasHandle_t handle, char uplo, const int n, float *A, int lda, long strideA,
                      int batchCount, int *info);
int kblas_potrf_batch(kblasHandle_t handle, char uplo, const int n, double *A, int lda, long strideA,
                      int batchCount, int *info);
int kblas_potrs_batch(kblasHandle_t handle, char side, char uplo, const int m, const int n,
                      const float **A, int lda, float **B, int ldb, int batchCount);
int kblas_potrs_batch(kblasHandle_t handle, char side, char uplo, const int m, const int n,
                      const double **A, int lda, double **B, int ldb, int batchCount);
int kblas_potrs_batch(kblasHandle_t handle, char side, char uplo, const int m, const int n,
                      const float *A, int lda, long strideA, float *B, int ldb, long strideB,
                      int batchCount);
int kblas_potrs_batch(kblasHandle_t handle, char side, char uplo, const int m, const int n,
                      const double *A, int lda, long strideA, double *B, int ldb, long strideB,
                      int batchCount);
int kblas_posv_batch(kblasHandle_t handle, char side, char uplo, const int m, const int n, float **A,
                     int lda, float **B, int ldb, int batchCount, int *info);
int kblas_posv_batch(kblasHandle_t handle, char side, char uplo, const int m, const int n, double **A,
                     int lda, double **B, int ldb, int batchCount, int *info);
int kblas_posv_batch(kblasHandle_t handle, char side, char uplo, const int m, const int n, float *A,
                     int lda, long strideA, float *B, int ldb, long strideB, int batchCount,
                     int *info);
int kblas_posv_batch(kblasHandle_t handle, char side, char uplo, const int m, const int n, double *A,
                     int lda, long strideA, double *B, int ldb, long strideB, int batchCount,
                     int *info);
int kblas_trsm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag, const int m,
                     const int n, const float alpha, const float **A, int lda, float **B, int ldb,
                     int batchCount);
int kblas_trsm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag, const int m,
                     const int n, const double alpha, const double **A, int lda, double **B,
                     int ldb, int batchCount);
int kblas_trsm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag, const int m,
                     const int n, const float alpha, const float *A, int lda, long strideA,
                     float *B, int ldb, long strideB, int batchCount);
int kblas_trsm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag, const int m,
                     const int n, const double alpha, const double *A, int lda, long strideA,
                     double *B, int ldb, long strideB, int batchCount);
int kblas_trmm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag, const int m,
                     const int n, const float alpha, const float **A, int lda, float **B, int ldb,
                     int batchCount);
int kblas_trmm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag, const int m,
                     const int n, const double alpha, const double **A, int lda, double **B,
                     int ldb, int batchCount);
int kblas_trmm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag, const int m,
                     const int n, const float alpha, const float *A, int lda, long strideA,
                     float *B, int ldb, long strideB, int batchCount);
int kblas_trmm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag, const int m,
                     const int n, const double alpha, const double *A, int lda, long strideA,
                     double *B, int ldb, long strideB, int batchCount);
int kblas_syrk_batch(kblasHandle_t handle, char uplo, char trans, const int m, const int n,
                     const float alpha, const float **A, int lda, const float beta, float **B,
                     int ldb, int batchCount);
int kblas_syrk_batch(kblasHandle_t handle, char uplo, char trans, const int m, const int n,
                     const double alpha, const double **A, int lda, const double beta, double **B,
                     int ldb, int batchCount);
int kblas_syrk_batch(kblasHandle_t handle, char uplo, char trans, const int m, const int n,
                     const float alpha, const float *A, int lda, long strideA, const float beta,
                     float *B, int ldb, long strideB, int batchCount);
int kblas_syrk_batch(kblasHandle_t handle, char uplo, char trans, const int m, const int n,
                     const double alpha, const double *A, int lda, long strideA,
                     const double beta, double *B, int ldb, long strideB, int batchCount);
int kblas_gemm_batch(kblasHandle_t handle, char transA, char transB, const int m, const int n,
                     const int k, const float alpha, const float **A, int lda, const float **B,
                     int ldb, const float beta, float **C, int ldc, int batchCount);
int kblas_gemm_batch(kblasHandle_t handle, char transA, char transB, const int m, const int n,
                     const int k, const double alpha, const double **A, int lda, const double **B,
                     int ldb, const double beta, double **C, int ldc, int batchCount);
int kblas_gemm_batch(kblasHandle_t handle, char transA, char transB, const int m, const int n,
                     const int k, const float alpha, const float *A, int lda, long strideA,
                     const float *B, int ldb, long strideB, const float beta, float *C, int ldc,
                     long strideC, int batchCount);
int kblas_gemm_batch(kblasHandle_t handle, char transA, char transB, const int m, const int n,
                     const int k, const double alpha, const double *A, int lda, long strideA,
                     const double *B, int ldb, long strideB, const double beta, double *C,
                     int ldc, long strideC, int batchCount);
int kblas_gemm_batch(kblasHandle_t handle, char transA, char transB, int *m, int *n, int *k,
                     int max_m, int max_n, int max_k, const float alpha, const float **A,
                     int *lda, const float **B, int *ldb, const float beta, float **C, int *ldc,
                     int batchCount);
int kblas_gemm_batch(kblasHandle_t handle, char transA, char transB, int *m, int *n, int *k,
                     int max_m, int max_n, int max_k, const double alpha, const double **A,
                     int *lda, const double **B, int *ldb, const double beta, double **C,
                     int *ldc, int batchCount);
int kblas_syrk_batch(kblasHandle_t handle, char uplo, char trans, int *m, int *n, int max_m, int max_n,
                     float alpha, float **A, int *lda, float beta, float **B, int *ldb,
                     int batchCount);
int kblas_syrk_batch(kblasHandle_t handle, char uplo, char trans, int *m, int *n, int max_m, int max_n,
                     double alpha, double **A, int *lda, double beta, double **B, int *ldb,
                     int batchCount);
int kblas_trsm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag, int *m, int *n,
                     int max_m, int max_n, float alpha, float **A, int *lda, float **B, int *ldb,
                     int batchCount);
int kblas_trsm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag, int *m, int *n,
                     int max_m, int max_n, double alpha, double **A, int *lda, double **B,
                     int *ldb, int batchCount);
int kblas_potrf_batch(kblasHandle_t handle, char uplo, const int n, cuFloatComplex **A, int lda, int batchCount,
                      int *info);
int kblas_potrf_batch(kblasHandle_t handle, char uplo, const int n, cuDoubleComplex **A, int lda, int batchCount,
                      int *info);
int kblas_potrf_batch(kblasHandle_t handle, char uplo, const int n, cuFloatComplex *A, int lda, long strideA,
                      int batchCount, int *info);
int kblas_potrf_batch(kblasHandle_t handle, char uplo, const int n, cuDoubleComplex *A, int lda, long strideA,
                      int batchCount, int *info);
int kblas_potrs_batch(kblasHandle_t handle, char side, char uplo, const int m, const int n,
                      const cuFloatComplex **A, int lda, cuFloatComplex **B, int ldb, int batchCount);
int kblas_potrs_batch(kblasHandle_t handle, char side, char uplo, const int m, const int n,
                      const cuDoubleComplex **A, int lda, cuDoubleComplex **B, int ldb, int batchCount);
int kblas_potrs_batch(kblasHandle_t handle, char side, char uplo, const int m, const int n,
                      const cuFloatComplex *A, int lda, long strideA, cuFloatComplex *B, int ldb, long strideB,
                      int batchCount);
int kblas_potrs_batch(kblasHandle_t handle, char side, char uplo, const int m, const int n,
                      const cuDoubleComplex *A, int lda, long strideA, cuDoubleComplex *B, int ldb, long strideB,
                      int batchCount);
int kblas_posv_batch(kblasHandle_t handle, char side, char uplo, const int m, const int n, cuFloatComplex **A,
                     int lda, cuFloatComplex **B, int ldb, int batchCount, int *info);
int kblas_posv_batch(kblasHandle_t handle, char side, char uplo, const int m, const int n, cuDoubleComplex **A,
                     int lda, cuDoubleComplex **B, int ldb, int batchCount, int *info);
int kblas_posv_batch(kblasHandle_t handle, char side, char uplo, const int m, const int n, cuFloatComplex *A,
                     int lda, long strideA, cuFloatComplex *B, int ldb, long strideB, int batchCount,
                     int *info);
int kblas_posv_batch(kblasHandle_t handle, char side, char uplo, const int m, const int n, cuDoubleComplex *A,
                     int lda, long strideA, cuDoubleComplex *B, int ldb, long strideB, int batchCount,
                     int *info);
int kblas_trsm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag, const int m,
                     const int n, const cuFloatComplex alpha, const cuFloatComplex **A, int lda, cuFloatComplex **B,
                     int ldb, int batchCount);
int kblas_trsm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag, const int m,
                     const int n, const cuDoubleComplex alpha, const cuDoubleComplex **A, int lda, cuDoubleComplex **B,
                     int ldb, int batchCount);
int kblas_trsm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag, const int m,
                     const int n, const cuFloatComplex alpha, const cuFloatComplex *A, int lda, long strideA,
                     cuFloatComplex *B, int ldb, long strideB, int batchCount);
int kblas_trsm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag, const int m,
                     const int n, const cuDoubleComplex alpha, const cuDoubleComplex *A, int lda, long strideA,
                     cuDoubleComplex *B, int ldb, long strideB, int batchCount);
int kblas_trmm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag, const int m,
                     const int n, const cuFloatComplex alpha, const cuFloatComplex **A, int lda, cuFloatComplex **B,
                     int ldb, int batchCount);
int kblas_trmm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag, const int m,
                     const int n, const cuDoubleComplex alpha, const cuDoubleComplex **A, int lda, cuDoubleComplex **B,
                     int ldb, int batchCount);
int kblas_trmm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag, const int m,
                     const int n, const cuFloatComplex alpha, const cuFloatComplex *A, int lda, long strideA,
                     cuFloatComplex *B, int ldb, long strideB, int batchCount);
int kblas_trmm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag, const int m,
                     const int n, const cuDoubleComplex alpha, const cuDoubleComplex *A, int lda, long strideA,
                     cuDoubleComplex *B, int ldb, long strideB, int batchCount);
int kblas_syrk_batch(kblasHandle_t handle, char uplo, char trans, const int m, const int n,
                     const cuFloatComplex alpha, const cuFloatComplex **A, int lda, const cuFloatComplex beta, cuFloatComplex **B,
                     int ldb, int batchCount);
int kblas_syrk_batch(kblasHandle_t handle, char uplo, char trans, const int m, const int n,
                     const cuDoubleComplex alpha, const cuDoubleComplex **A, int lda, const cuDoubleComplex beta, cuDoubleComplex **B,
                     int ldb, int batchCount);
int kblas_syrk_batch(kblasHandle_t handle, char uplo, char trans, const int m, const int n,
                     const cuFloatComplex alpha, const cuFloatComplex *A, int lda, long strideA,
                     const cuFloatComplex beta, cuFloatComplex *B, int ldb, long strideB, int batchCount);
int kblas_syrk_batch(kblasHandle_t handle, char uplo, char trans, const int m, const int n,
                     const cuDoubleComplex alpha, const cuDoubleComplex *A, int lda, long strideA,
                     const cuDoubleComplex beta, cuDoubleComplex *B, int ldb, long strideB, int batchCount);
int kblas_gemm_batch(kblasHandle_t handle, char transA, char transB, const int m, const int n,
                     const int k, const cuFloatComplex alpha, const cuFloatComplex **A, int lda, const cuFloatComplex **B,
                     int ldb, const cuFloatComplex beta, cuFloatComplex **C, int ldc, int batchCount);
int kblas_gemm_batch(kblasHandle_t handle, char transA, char transB, const int m, const int n,
                     const int k, const cuDoubleComplex alpha, const cuDoubleComplex **A, int lda, const cuDoubleComplex **B,
                     int ldb, const cuDoubleComplex beta, cuDoubleComplex **C, int ldc, int batchCount);
int kblas_gemm_batch(kblasHandle_t handle, char transA, char transB, const int m, const int n,
                     const int k, const cuFloatComplex alpha, const cuFloatComplex *A, int lda, long strideA,
                     const cuFloatComplex *B, int ldb, long strideB, const cuFloatComplex beta, cuFloatComplex *C,
                     int ldc, long strideC, int batchCount);
int kblas_gemm_batch(kblasHandle_t handle, char transA, char transB, const int m, const int n,
                     const int k, const cuDoubleComplex alpha, const cuDoubleComplex *A, int lda, long strideA,
                     const cuDoubleComplex *B, int ldb, long strideB, const cuDoubleComplex beta, cuDoubleComplex *C,
                     int ldc, long strideC, int batchCount);
int kblas_gemm_batch(kblasHandle_t handle, char transA, char transB, int *m, int *n, int *k,
                     int max_m, int max_n, int max_k, const cuFloatComplex alpha, const cuFloatComplex **A,
                     int *lda, const cuFloatComplex **B, int *ldb, const cuFloatComplex beta, cuFloatComplex **C,
                     int *ldc, int batchCount);
int kblas_gemm_batch(kblasHandle_t handle, char transA, char transB, int *m, int *n, int *k,
                     int max_m, int max_n, int max_k, const cuDoubleComplex alpha, const cuDoubleComplex **A,
                     int *lda, const cuDoubleComplex **B, int *ldb, const cuDoubleComplex beta, cuDoubleComplex **C,
                     int *ldc, int batchCount);
int kblas_syrk_batch(kblasHandle_t handle, char uplo, char trans, int *m, int *n, int max_m, int max_n,
                     cuFloatComplex alpha, cuFloatComplex **A, int *lda, cuFloatComplex beta, cuFloatComplex **B, int *ldb,
                     int batchCount);
int kblas_syrk_batch(kblasHandle_t handle, char uplo, char trans, int *m, int *n, int max_m, int max_n,
                     cuDoubleComplex alpha, cuDoubleComplex **A, int *lda, cuDoubleComplex beta, cuDoubleComplex **B, int *ldb,
                     int batchCount);
int kblas_trsm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag, int *m, int *n,
                     int max_m, int max_n, cuFloatComplex alpha, cuFloatComplex **A, int *lda, cuFloatComplex **B,
                     int *ldb, int batchCount);
int kblas_trsm_batch(kblasHandle_t handle, char side, char uplo, char trans, char diag, int *m, int *n,
                     int max_m, int max_n, cuDoubleComplex alpha, cuDoubleComplex **A, int *lda, cuDoubleComplex **B,
                     int *ldb, int batchCount);
int kblas_trtri_batch(kblasHandle_t handle, char uplo, char diag, const int n, float **A, int lda,
                      int batchCount, int *info);
int kblas_trtri_batch(kblasHandle_t handle, char uplo, char diag, const int n, float *A, int lda,
                      long strideA, int batchCount, int *info);
int kblas_lauum_batch(kblasHandle_t handle, char uplo, const int n, float **A, int lda, int batchCount,
                      int *info);
int kblas_lauum_batch(kblasHandle_t handle, char uplo, const int n, float *A, int lda, long strideA,
                      int batchCount, int *info);
int kblas_potri_batch(kblasHandle_t handle, char uplo, const int n, float **A, int lda, int batchCount,
                      int *info);
int kblas_potri_batch(kblasHandle_t handle, char uplo, const int n, float *A, int lda, long strideA,
                      int batchCount, int *info);
int kblas_poti_batch(kblasHandle_t handle, char uplo, const int n, float **A, int lda, int batchCount,
                      int *info);
int kblas_poti_batch(kblasHandle_t handle, char uplo, const int n, float *A, int lda, long strideA,
                      int batchCount, int *info);
int kblas_trtri_batch(kblasHandle_t handle, char uplo, char diag, const int n, double **A, int lda,
                      int batchCount, int *info);
int kblas_trtri_batch(kblasHandle_t handle, char uplo, char diag, const int n, double *A, int lda,
                      long strideA, int batchCount, int *info);
int kblas_lauum_batch(kblasHandle_t handle, char uplo, const int n, double **A, int lda, int batchCount,
                      int *info);
int kblas_lauum_batch(kblasHandle_t handle, char uplo, const int n, double *A, int lda, long strideA,
                      int batchCount, int *info);
int kblas_potri_batch(kblasHandle_t handle, char uplo, const int n, double **A, int lda, int batchCount,
                      int *info);
int kblas_potri_batch(kblasHandle_t handle, char uplo, const int n, double *A, int lda, long strideA,
                      int batchCount, int *info);
int kblas_poti_batch(kblasHandle_t handle, char uplo, const int n, double **A, int lda, int batchCount,
                      int *info);
int kblas_poti_batch(kblasHandle_t handle, char uplo, const int n, double *A, int lda, long strideA,
                      int batchCount, int *info);
int kblas_trtri_batch(kblasHandle_t handle, char uplo, char diag, const int n, cuFloatComplex **A, int lda,
                      int batchCount, int *info);
int kblas_trtri_batch(kblasHandle_t handle, char uplo, char diag, const int n, cuFloatComplex *A, int lda,
                      long strideA, int batchCount, int *info);
int kblas_lauum_batch(kblasHandle_t handle, char uplo, const int n, cuFloatComplex **A, int lda, int batchCount,
                      int *info);
int kblas_lauum_batch(kblasHandle_t handle, char uplo, const int n, cuFloatComplex *A, int lda, long strideA,
                      int batchCount, int *info);
int kblas_potri_batch(kblasHandle_t handle, char uplo, const int n, cuFloatComplex **A, int lda, int batchCount,
                      int *info);
int kblas_potri_batch(kblasHandle_t handle, char uplo, const int n, cuFloatComplex *A, int lda, long strideA,
                      int batchCount, int *info);
int kblas_poti_batch(kblasHandle_t handle, char uplo, const int n, cuFloatComplex **A, int lda, int batchCount,
                      int *info);
int kblas_poti_batch(kblasHandle_t handle, char uplo, const int n, cuFloatComplex *A, int lda, long strideA,
                      int batchCount, int *info);
int kblas_trtri_batch(kblasHandle_t handle, char uplo, char diag, const int n, cuDoubleComplex **A, int lda,
                      int batchCount, int *info);
int kblas_trtri_batch(kblasHandle_t handle, char uplo, char diag, const int n, cuDoubleComplex *A, int lda,
                      long strideA, int batchCount, int *info);
int kblas_lauum_batch(kblasHandle_t handle, char uplo, const int n, cuDoubleComplex **A, int lda, int batchCount,
                      int *info);
int kblas_lauum_batch(kblasHandle_t handle, char uplo, const int n, cuDoubleComplex *A, int lda, long strideA,
                      int batchCount, int *info);
int kblas_potri_batch(kblasHandle_t handle, char uplo, const int n, cuDoubleComplex **A, int lda, int batchCount,
                      int *info);
int kblas_potri_batch(kblasHandle_t handle, char uplo, const int n, cuDoubleComplex *A, int lda, long strideA,
                      int batchCount, int *info);
int kblas_poti_batch(kblasHandle_t handle, char uplo, const int n, cuDoubleComplex **A, int lda, int batchCount,
                      int *info);
int kblas_poti_batch(kblasHandle_t handle, char uplo, const int n, cuDoubleComplex *A, int lda, long strideA,
                      int batchCount, int *info);
#endif /* __cplusplus */

#endif /* KBLAS_GB300_BATCH_H */

/*
 * oracle_impl.h -- precision-generic body of the CPU oracle (TEST
 * INFRASTRUCTURE ONLY: included twice by kblas_oracle.c, once with
 * REAL = double / float, and for the complex routines with REAL = double
 * _Complex / float _Complex: the same loops, nothing conjugated).
 *
 * The reference library has no CPU implementation of the batched path; its
 * tests check every routine against host LAPACK/BLAS looped over the batch
 * (reference testing/batch_triangular/test_Xpotrf_batch.cpp:276-338,
 * test_Xposv_batch.cpp:301-338, test_Xtrsm_batch.cpp:330-360,
 * test_Xtrmm_batch.cpp:330-354, test_Xsyrk_batch.cpp:380-417). LAPACK and
 * BLAS are not part of the reference tree (MKL / OpenBLAS, linked at build
 * time); this file restates the published algorithms of the reference
 * implementations of LAPACK 3.x (xPOTF2 / xPOTRS, and for the inversion
 * routines xTRTI2 / xLAUU2 / xPOTRI) and BLAS (xTRSM, xTRMM, xSYRK) in plain C
 * loops, with no blocking.
 */

#define ORC_CAT_(a, b) a##b
#define ORC_CAT(a, b) ORC_CAT_(a, b)
#define ORC(name) ORC_CAT(ORC_CAT(oracle_, PFX), name)

#define AT(M, ld, i, j) (M)[(size_t)(i) + (size_t)(j) * (size_t)(ld)]

/* Pivot test and square root of the factorization: real types fail on a
 * pivot <= 0 or NaN (LAPACK); the complex instantiation (complex-symmetric,
 * A = L L^T without conjugation, the reference's complex batch routines)
 * fails on a zero or non-finite pivot and takes the principal root. */
#ifndef ORC_PIVOT_BAD
#define ORC_PIVOT_BAD(d) (!((d) > (REAL)0))  /* also catches NaN */
#define ORC_SQRT(d) ((REAL)sqrt((double)(d)))
#define ORC_DEFAULT_PIVOT 1
#endif

/* LAPACK xPOTF2, lower: column-by-column dot-product (left-looking) Cholesky.
 * info = j (1-based) for the first pivot that is <= 0 or NaN; A(j,j) then
 * holds that pivot value and the columns after it are untouched, as in
 * LAPACK. Same factor, in exact arithmetic, as the reference's right-looking
 * register kernel (src/batch_triangular/Xpotrf_batch_kernels.cuh:37-78). */
int ORC(potrf)(int n, REAL *A, int lda)
{
    for (int j = 0; j < n; j++) {
        REAL ajj = AT(A, lda, j, j);
        for (int k = 0; k < j; k++) ajj -= AT(A, lda, j, k) * AT(A, lda, j, k);
        if (ORC_PIVOT_BAD(ajj)) {
            AT(A, lda, j, j) = ajj;
            return j + 1;
        }
        ajj = ORC_SQRT(ajj);
        AT(A, lda, j, j) = ajj;
        for (int i = j + 1; i < n; i++) {
            REAL s = AT(A, lda, i, j);
            for (int k = 0; k < j; k++) s -= AT(A, lda, i, k) * AT(A, lda, j, k);
            AT(A, lda, i, j) = s / ajj;
        }
    }
    return 0;
}

/* Solve M*x = alpha*x for one vector x (stride incx), where M is the
 * triangle stored in A (lower if lower != 0) or its transpose (trans != 0),
 * unit diagonal if unit != 0. Reference BLAS xTRSM/xTRSV loop order. */
static void ORC(trsv_)(int lower, int trans, int unit, int n, const REAL *A, int lda,
                       REAL *x, long incx)
{
    /* effective triangle of M: lower iff (lower xor trans) */
    int mlower = (lower != 0) ^ (trans != 0);
#define MEL(i, j) (trans ? AT(A, lda, j, i) : AT(A, lda, i, j))
    if (mlower) { /* forward substitution */
        for (int i = 0; i < n; i++) {
            REAL s = x[i * incx];
            for (int k = 0; k < i; k++) s -= MEL(i, k) * x[k * incx];
            if (!unit) s /= MEL(i, i);
            x[i * incx] = s;
        }
    } else { /* backward substitution */
        for (int i = n - 1; i >= 0; i--) {
            REAL s = x[i * incx];
            for (int k = i + 1; k < n; k++) s -= MEL(i, k) * x[k * incx];
            if (!unit) s /= MEL(i, i);
            x[i * incx] = s;
        }
    }
#undef MEL
}

/* y = M*x in place (M as in trsv_). */
static void ORC(trmv_)(int lower, int trans, int unit, int n, const REAL *A, int lda,
                       REAL *x, long incx)
{
    int mlower = (lower != 0) ^ (trans != 0);
#define MEL(i, j) (trans ? AT(A, lda, j, i) : AT(A, lda, i, j))
    if (mlower) { /* y_i depends on x_0..x_i: go downwards */
        for (int i = n - 1; i >= 0; i--) {
            REAL s = unit ? x[i * incx] : MEL(i, i) * x[i * incx];
            for (int k = 0; k < i; k++) s += MEL(i, k) * x[k * incx];
            x[i * incx] = s;
        }
    } else {
        for (int i = 0; i < n; i++) {
            REAL s = unit ? x[i * incx] : MEL(i, i) * x[i * incx];
            for (int k = i + 1; k < n; k++) s += MEL(i, k) * x[k * incx];
            x[i * incx] = s;
        }
    }
#undef MEL
}

/* BLAS xTRSM: op(A)*X = alpha*B (side 'L') or X*op(A) = alpha*B (side 'R').
 * A row r of X*op(A) = b_r is the column system op(A)^T x_r^T = b_r^T. */
void ORC(trsm)(char side, char uplo, char trans, char diag, int m, int n, REAL alpha,
               const REAL *A, int lda, REAL *B, int ldb)
{
    int lower = (uplo == 'L' || uplo == 'l');
    int tr = (trans == 'T' || trans == 't' || trans == 'C' || trans == 'c');
    int unit = (diag == 'U' || diag == 'u');
    if (side == 'L' || side == 'l') {
        for (int j = 0; j < n; j++) {
            REAL *x = &AT(B, ldb, 0, j);
            for (int i = 0; i < m; i++) x[i] *= alpha;
            ORC(trsv_)(lower, tr, unit, m, A, lda, x, 1);
        }
    } else {
        for (int r = 0; r < m; r++) {
            REAL *x = &AT(B, ldb, r, 0);
            for (int i = 0; i < n; i++) x[(long)i * ldb] *= alpha;
            ORC(trsv_)(lower, !tr, unit, n, A, lda, x, ldb);
        }
    }
}

/* BLAS xTRMM: B := alpha*op(A)*B (side 'L') or alpha*B*op(A) (side 'R'). */
void ORC(trmm)(char side, char uplo, char trans, char diag, int m, int n, REAL alpha,
               const REAL *A, int lda, REAL *B, int ldb)
{
    int lower = (uplo == 'L' || uplo == 'l');
    int tr = (trans == 'T' || trans == 't' || trans == 'C' || trans == 'c');
    int unit = (diag == 'U' || diag == 'u');
    if (side == 'L' || side == 'l') {
        for (int j = 0; j < n; j++) {
            REAL *x = &AT(B, ldb, 0, j);
            ORC(trmv_)(lower, tr, unit, m, A, lda, x, 1);
            for (int i = 0; i < m; i++) x[i] *= alpha;
        }
    } else {
        for (int r = 0; r < m; r++) {
            REAL *x = &AT(B, ldb, r, 0);
            ORC(trmv_)(lower, !tr, unit, n, A, lda, x, ldb);
            for (int i = 0; i < n; i++) x[(long)i * ldb] *= alpha;
        }
    }
}

/* BLAS xSYRK: C := alpha*op(A)*op(A)^T + beta*C on the uplo triangle of the
 * m x m matrix C; op(A) is m x k. beta == 0 means C is not read. */
void ORC(syrk)(char uplo, char trans, int m, int k, REAL alpha, const REAL *A, int lda,
               REAL beta, REAL *C, int ldc)
{
    int lower = (uplo == 'L' || uplo == 'l');
    int tr = (trans == 'T' || trans == 't' || trans == 'C' || trans == 'c');
    for (int j = 0; j < m; j++) {
        int i0 = lower ? j : 0, i1 = lower ? m : j + 1;
        for (int i = i0; i < i1; i++) {
            REAL s = 0;
            for (int l = 0; l < k; l++) {
                REAL ai = tr ? AT(A, lda, l, i) : AT(A, lda, i, l);
                REAL aj = tr ? AT(A, lda, l, j) : AT(A, lda, j, l);
                s += ai * aj;
            }
            REAL c = (beta == (REAL)0) ? (REAL)0 : beta * AT(C, ldc, i, j);
            AT(C, ldc, i, j) = alpha * s + c;
        }
    }
}

/* BLAS xGEMM: C := alpha*op(A)*op(B) + beta*C, C m x n, op(A) m x k,
 * op(B) k x n; op(A), op(B) not read when alpha == 0 or k == 0, C not read
 * when beta == 0 (the reference BLAS rules, which the reference's cuBLAS
 * and MAGMA calls, src/batch_triangular/Xgemm_batch_core.cuh:171-470, keep). */
void ORC(gemm)(char transA, char transB, int m, int n, int k, REAL alpha, const REAL *A,
               int lda, const REAL *B, int ldb, REAL beta, REAL *C, int ldc)
{
    int ta = (transA == 'T' || transA == 't' || transA == 'C' || transA == 'c');
    int tb = (transB == 'T' || transB == 't' || transB == 'C' || transB == 'c');
    int prod = (alpha != (REAL)0 && k > 0);
    for (int j = 0; j < n; j++)
        for (int i = 0; i < m; i++) {
            REAL s = 0;
            if (prod)
                for (int l = 0; l < k; l++) {
                    REAL a = ta ? AT(A, lda, l, i) : AT(A, lda, i, l);
                    REAL b = tb ? AT(B, ldb, j, l) : AT(B, ldb, l, j);
                    s += a * b;
                }
            REAL c = (beta == (REAL)0) ? (REAL)0 : beta * AT(C, ldc, i, j);
            AT(C, ldc, i, j) = prod ? alpha * s + c : c;
        }
}

/* POTRS with side 'R', uplo 'L' (the only form of the reference,
 * src/batch_triangular/Xpotrs_batch_drivers.cuh:40-43): X*L*L^T = B, i.e.
 * B := B*L^{-T}*L^{-1}, the reference's TRSM(R,L,T,N) then TRSM(R,L,N,N)
 * sequence (Xpotrs_batch_drivers.cuh:94-171) in unblocked form. */
void ORC(potrs)(int m, int n, const REAL *L, int lda, REAL *B, int ldb)
{
    ORC(trsm)('R', 'L', 'T', 'N', m, n, (REAL)1, L, lda, B, ldb);
    ORC(trsm)('R', 'L', 'N', 'N', m, n, (REAL)1, L, lda, B, ldb);
}

/* POSV = POTRF + POTRS (reference Xposv_batch_drivers.cuh:83-114); B is left
 * unchanged when the factorization fails (LAPACK xPOSV). */
int ORC(posv)(int m, int n, REAL *A, int lda, REAL *B, int ldb)
{
    int info = ORC(potrf)(n, A, lda);
    if (info == 0) ORC(potrs)(m, n, A, lda, B, ldb);
    return info;
}

/* LAPACK xTRTRI (lower), unblocked as xTRTI2: in-place inverse of a lower
 * triangular matrix, columns from the last: X(j,j) = 1/L(j,j), then
 * X(j+1:n, j) = -X(j,j) * X(j+1:n, j+1:n) * L(j+1:n, j) (the trailing block
 * already inverted, a lower triangular matrix-vector product). unit != 0: unit
 * diagonal, not referenced. info = j (1-based) for the first L(j,j) == 0
 * (non-unit), A then unchanged, as LAPACK xTRTRI checks before it starts. */
int ORC(trtri)(int unit, int n, REAL *A, int lda)
{
    if (!unit)
        for (int j = 0; j < n; j++)
            if (AT(A, lda, j, j) == (REAL)0) return j + 1;
    for (int j = n - 1; j >= 0; j--) {
        REAL ajj;
        if (!unit) {
            AT(A, lda, j, j) = (REAL)1 / AT(A, lda, j, j);
            ajj = -AT(A, lda, j, j);
        } else {
            ajj = (REAL)-1;
        }
        if (j < n - 1) {
            /* x := X(j+1:n, j+1:n) * x, x = A(j+1:n, j), lower triangular (xTRMV) */
            for (int i = n - 1; i > j; i--) {
                REAL s = unit ? AT(A, lda, i, j) : AT(A, lda, i, i) * AT(A, lda, i, j);
                for (int k = j + 1; k < i; k++) s += AT(A, lda, i, k) * AT(A, lda, k, j);
                AT(A, lda, i, j) = s;
            }
            for (int i = j + 1; i < n; i++) AT(A, lda, i, j) *= ajj;
        }
    }
    return 0;
}

/* LAPACK xLAUUM (lower), unblocked as xLAUU2: the lower triangle of L^T L
 * overwrites L. Row i of the result needs rows >= i of L only, so rows are
 * produced top-down, the diagonal entry of a row last. */
void ORC(lauum)(int n, REAL *A, int lda)
{
    for (int i = 0; i < n; i++) {
        /* B(i, j) = sum_{k >= i} L(k, i) L(k, j), j <= i */
        for (int j = 0; j <= i; j++) {
            REAL s = 0;
            for (int k = i; k < n; k++) s += AT(A, lda, k, i) * AT(A, lda, k, j);
            if (j < i) AT(A, lda, i, j) = s;
            else {
                /* the diagonal last: row i's other entries read L(i, i) */
                AT(A, lda, i, i) = s;
            }
        }
    }
}

/* LAPACK xPOTRI (lower): inverse of A from its Cholesky factor L (in A):
 * xTRTRI then xLAUUM. info as xTRTRI. */
int ORC(potri)(int n, REAL *A, int lda)
{
    int info = ORC(trtri)(0, n, A, lda);
    if (info) return info;
    ORC(lauum)(n, A, lda);
    return 0;
}

/* POTI (the reference's kblas_poti_batch): inverse of an SPD matrix in place,
 * xPOTRF then xPOTRI; info from the first that fails. */
int ORC(poti)(int n, REAL *A, int lda)
{
    int info = ORC(potrf)(n, A, lda);
    if (info) return info;
    return ORC(potri)(n, A, lda);
}

/* ---------------------------- batched drivers ---------------------------- */
/* One matrix per loop iteration, dynamic schedule, as the reference tests'
 * CPU timing loop (test_Xposv_batch.cpp:301-326). */

void ORC(potrf_batch)(int n, REAL *A, int lda, long strideA, int batch, int *info, int nthreads)
{
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
    for (int b = 0; b < batch; b++) info[b] = ORC(potrf)(n, A + (size_t)b * strideA, lda);
}

void ORC(potrs_batch)(int m, int n, const REAL *A, int lda, long strideA, REAL *B, int ldb,
                      long strideB, int batch, int nthreads)
{
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
    for (int b = 0; b < batch; b++)
        ORC(potrs)(m, n, A + (size_t)b * strideA, lda, B + (size_t)b * strideB, ldb);
}

void ORC(posv_batch)(int m, int n, REAL *A, int lda, long strideA, REAL *B, int ldb, long strideB,
                     int batch, int *info, int nthreads)
{
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
    for (int b = 0; b < batch; b++)
        info[b] = ORC(posv)(m, n, A + (size_t)b * strideA, lda, B + (size_t)b * strideB, ldb);
}

void ORC(trsm_batch)(char side, char uplo, char trans, char diag, int m, int n, REAL alpha,
                     const REAL *A, int lda, long strideA, REAL *B, int ldb, long strideB,
                     int batch, int nthreads)
{
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
    for (int b = 0; b < batch; b++)
        ORC(trsm)(side, uplo, trans, diag, m, n, alpha, A + (size_t)b * strideA, lda,
                  B + (size_t)b * strideB, ldb);
}

void ORC(trmm_batch)(char side, char uplo, char trans, char diag, int m, int n, REAL alpha,
                     const REAL *A, int lda, long strideA, REAL *B, int ldb, long strideB,
                     int batch, int nthreads)
{
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
    for (int b = 0; b < batch; b++)
        ORC(trmm)(side, uplo, trans, diag, m, n, alpha, A + (size_t)b * strideA, lda,
                  B + (size_t)b * strideB, ldb);
}

void ORC(syrk_batch)(char uplo, char trans, int m, int k, REAL alpha, const REAL *A, int lda,
                     long strideA, REAL beta, REAL *C, int ldc, long strideC, int batch,
                     int nthreads)
{
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
    for (int b = 0; b < batch; b++)
        ORC(syrk)(uplo, trans, m, k, alpha, A + (size_t)b * strideA, lda, beta,
                  C + (size_t)b * strideC, ldc);
}

void ORC(gemm_batch)(char transA, char transB, int m, int n, int k, REAL alpha, const REAL *A,
                     int lda, long strideA, const REAL *B, int ldb, long strideB, REAL beta,
                     REAL *C, int ldc, long strideC, int batch, int nthreads)
{
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
    for (int b = 0; b < batch; b++)
        ORC(gemm)(transA, transB, m, n, k, alpha, A + (size_t)b * strideA, lda,
                  B + (size_t)b * strideB, ldb, beta, C + (size_t)b * strideC, ldc);
}

void ORC(trtri_batch)(int unit, int n, REAL *A, int lda, long strideA, int batch, int *info,
                      int nthreads)
{
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
    for (int b = 0; b < batch; b++) info[b] = ORC(trtri)(unit, n, A + (size_t)b * strideA, lda);
}

void ORC(lauum_batch)(int n, REAL *A, int lda, long strideA, int batch, int nthreads)
{
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
    for (int b = 0; b < batch; b++) ORC(lauum)(n, A + (size_t)b * strideA, lda);
}

void ORC(potri_batch)(int n, REAL *A, int lda, long strideA, int batch, int *info, int nthreads)
{
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
    for (int b = 0; b < batch; b++) info[b] = ORC(potri)(n, A + (size_t)b * strideA, lda);
}

void ORC(poti_batch)(int n, REAL *A, int lda, long strideA, int batch, int *info, int nthreads)
{
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
    for (int b = 0; b < batch; b++) info[b] = ORC(poti)(n, A + (size_t)b * strideA, lda);
}

/* Variable-size POSV over pointer arrays (host pointers here). */
void ORC(posv_vbatch)(const int *m, const int *n, REAL **A, const int *lda, REAL **B,
                      const int *ldb, int batch, int *info, int nthreads)
{
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
    for (int b = 0; b < batch; b++) info[b] = ORC(posv)(m[b], n[b], A[b], lda[b], B[b], ldb[b]);
}

#undef AT
#undef ORC
#undef ORC_CAT
#undef ORC_CAT_

#ifdef ORC_DEFAULT_PIVOT
#undef ORC_PIVOT_BAD
#undef ORC_SQRT
#undef ORC_DEFAULT_PIVOT
#endif

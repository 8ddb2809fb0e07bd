/*
 * kblas_oracle.c -- CPU oracle for the batched Cholesky / triangular path.
 *
 * TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and the CPU
 * baseline legs of bench.py load this library, as the checker and as the
 * timed CPU baseline; the product library never links or calls it.
 *
 * What it restates: the host LAPACK/BLAS checks of the reference's batch
 * tests (see oracle_impl.h for the per-routine citations), plus the error
 * measures used to judge a GPU result:
 *  - normwise backward error of X*A = B per right-hand side row,
 *      eta = ||b - x*A||_inf / (||A||_inf * ||x||_inf + ||b||_inf),
 *    accumulated in long double from the lower triangle of A (A symmetric);
 *  - the reference tests' relative factor difference
 *      max|L1 - L2| / max|L2| over the lower triangle
 *    (reference testing/batch_triangular/test_Xpotrf_batch.cpp:317-338).
 *
 * Parity pin: these routines are checked against LAPACK/BLAS outputs
 * (scipy's bundled OpenBLAS) stored as fixtures in tests/golden/, made by
 * tests/golden/make_golden.py.
 */
#include <math.h>
#include <stddef.h>
#include <stdlib.h>

#define REAL double
#define PFX d
#include "oracle_impl.h"
#undef REAL
#undef PFX

#define REAL float
#define PFX s
#include "oracle_impl.h"
#undef REAL
#undef PFX

/* complex-symmetric instantiations (C99 complex: the same layout as
 * cuDoubleComplex / cuFloatComplex and numpy complex128 / complex64) */
#include <complex.h>
#define ORC_PIVOT_BAD(d) ((d) == 0 || !isfinite(creal(d)) || !isfinite(cimag(d)))
#define ORC_SQRT(d) csqrt(d)
#define REAL double _Complex
#define PFX z
#include "oracle_impl.h"
#undef REAL
#undef PFX
#undef ORC_PIVOT_BAD
#undef ORC_SQRT

#define ORC_PIVOT_BAD(d) ((d) == 0 || !isfinite(crealf(d)) || !isfinite(cimagf(d)))
#define ORC_SQRT(d) csqrtf(d)
#define REAL float _Complex
#define PFX c
#include "oracle_impl.h"
#undef REAL
#undef PFX
#undef ORC_PIVOT_BAD
#undef ORC_SQRT

#define AT(M, ld, i, j) (M)[(size_t)(i) + (size_t)(j) * (size_t)(ld)]

/* A(i,j) of a symmetric matrix given by its lower triangle. */
static inline long double sym_lower(const double *A, int lda, int i, int j)
{
    return (i >= j) ? (long double)AT(A, lda, i, j) : (long double)AT(A, lda, j, i);
}

/* Backward error of X*A = B (side 'R'; X, B are m x n, A n x n symmetric given
 * by its lower triangle): returns the max over the m rows. */
double oracle_backward_error_r(int m, int n, const double *A, int lda, const double *X, int ldx,
                               const double *B, int ldb)
{
    long double anorm = 0;
    for (int i = 0; i < n; i++) {
        long double s = 0;
        for (int j = 0; j < n; j++) s += fabsl(sym_lower(A, lda, i, j));
        if (s > anorm) anorm = s;
    }
    double worst = 0;
    for (int r = 0; r < m; r++) {
        long double rmax = 0, xmax = 0, bmax = 0;
        for (int j = 0; j < n; j++) {
            long double s = (long double)AT(B, ldb, r, j);
            for (int k = 0; k < n; k++) s -= (long double)AT(X, ldx, r, k) * sym_lower(A, lda, k, j);
            if (fabsl(s) > rmax) rmax = fabsl(s);
            if (fabsl((long double)AT(X, ldx, r, j)) > xmax) xmax = fabsl((long double)AT(X, ldx, r, j));
            if (fabsl((long double)AT(B, ldb, r, j)) > bmax) bmax = fabsl((long double)AT(B, ldb, r, j));
        }
        long double den = anorm * xmax + bmax;
        double eta = (den > 0) ? (double)(rmax / den) : (rmax > 0 ? INFINITY : 0.0);
        if (!(eta <= worst)) worst = eta; /* propagates NaN */
    }
    return worst;
}

/* Batched backward errors for strided storage: eta[b] per system. */
void oracle_backward_error_r_batch(int m, int n, const double *A, int lda, long strideA,
                                   const double *X, int ldx, long strideX, const double *B,
                                   int ldb, long strideB, int batch, double *eta, int nthreads)
{
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
    for (int b = 0; b < batch; b++)
        eta[b] = oracle_backward_error_r(m, n, A + (size_t)b * strideA, lda, X + (size_t)b * strideX,
                                         ldx, B + (size_t)b * strideB, ldb);
}

/* Backward error of a Cholesky factor: ||A - L*L^T||_max / ||A||_max over the
 * lower triangle, accumulated in long double. */
double oracle_factor_backward_error(int n, const double *A, int lda, const double *L, int ldl)
{
    long double num = 0, den = 0;
    for (int j = 0; j < n; j++) {
        for (int i = j; i < n; i++) {
            long double s = 0;
            for (int k = 0; k <= j; k++) s += (long double)AT(L, ldl, i, k) * (long double)AT(L, ldl, j, k);
            long double d = fabsl((long double)AT(A, lda, i, j) - s);
            if (d > num) num = d;
            if (fabsl((long double)AT(A, lda, i, j)) > den) den = fabsl((long double)AT(A, lda, i, j));
        }
    }
    return den > 0 ? (double)(num / den) : (double)num;
}

/* Relative difference of two lower triangles, the reference tests' measure
 * (test_Xpotrf_batch.cpp:317-338): max|L1-L2| / max|L2|. */
double oracle_lower_rel_diff(int n, const double *L1, int ld1, const double *L2, int ld2)
{
    double num = 0, den = 0;
    for (int j = 0; j < n; j++)
        for (int i = j; i < n; i++) {
            double d = fabs(AT(L1, ld1, i, j) - AT(L2, ld2, i, j));
            if (!(d <= num)) num = d;
            if (fabs(AT(L2, ld2, i, j)) > den) den = fabs(AT(L2, ld2, i, j));
        }
    return den > 0 ? num / den : num;
}

/* Variable-size backward errors over host pointer arrays. */
void oracle_backward_error_r_vbatch(const int *m, const int *n, double *const *A, const int *lda,
                                    double *const *X, const int *ldx, double *const *B,
                                    const int *ldb, int batch, double *eta, int nthreads)
{
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
    for (int b = 0; b < batch; b++)
        eta[b] = oracle_backward_error_r(m[b], n[b], A[b], lda[b], X[b], ldx[b], B[b], ldb[b]);
}

int oracle_max_threads(void)
{
#ifdef _OPENMP
    extern int omp_get_max_threads(void);
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* The reference testers' CPU timing path with the host's own LAPACK
 * (test_Xposv_batch.cpp:301-326: one LAPACK call per matrix, OpenMP over the
 * batch): dpotrf + dpotrs through function pointers the caller supplies (an
 * optimized LAPACK, e.g. the one scipy links; Fortran calling convention,
 * 32-bit integers), over a variable-size batch with ONE right-hand side per
 * system stored as a contiguous column of n values (B[b][0..n-1]). info[b]
 * as dpotrf's; B[b] is solved in place only when info[b] == 0. */
typedef void (*orc_lapack_dpotrf_fn)(char *, int *, double *, int *, int *);
typedef void (*orc_lapack_dpotrs_fn)(char *, int *, int *, double *, int *, double *, int *, int *);

void oracle_lapack_dposv_vbatch(void *potrf, void *potrs, const int *n, int nrhs,
                                double *const *A, const int *lda, double *const *B,
                                const int *ldb, int batch, int *info, int nthreads);

void oracle_lapack_dposv1_vbatch(void *potrf, void *potrs, const int *n, double *const *A,
                                 const int *lda, double *const *B, int batch, int *info,
                                 int nthreads)
{
    oracle_lapack_dposv_vbatch(potrf, potrs, n, 1, A, lda, B, n, batch, info, nthreads);
}

/* The same with nrhs right-hand sides per system: B[b] is n x nrhs,
 * column-major with leading dimension ldb[b] (LAPACK's layout). */
void oracle_lapack_dposv_vbatch(void *potrf, void *potrs, const int *n, int nrhs,
                                double *const *A, const int *lda, double *const *B,
                                const int *ldb, int batch, int *info, int nthreads)
{
    const orc_lapack_dpotrf_fn f = (orc_lapack_dpotrf_fn)potrf;
    const orc_lapack_dpotrs_fn s = (orc_lapack_dpotrs_fn)potrs;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
    for (int b = 0; b < batch; b++) {
        char lo = 'L';
        int nn = n[b], ld = lda[b], nr = nrhs, inf = 0;
        if (nn > 0) f(&lo, &nn, A[b], &ld, &inf);
        if (inf == 0 && nn > 0 && nr > 0) {
            int lb = ldb[b], inf2 = 0;
            s(&lo, &nn, &nr, A[b], &ld, B[b], &lb, &inf2);
        }
        info[b] = inf;
    }
}

/*
 * kblas_c_driver.c -- a plain C host program that drives the batched
 * Cholesky / triangular path through the library's C ABI, the way a KBLAS
 * caller does (reference testing/batch_triangular/test_Xposv_batch.cpp and
 * test_Xpotrf_batch.cpp: kblasCreate, *_wsquery, kblasAllocateWorkspace,
 * device matrices with the leading dimension rounded up to 32, device pointer
 * arrays, kblasTimerTic/Toc, info read back from the device).
 *
 * TEST PROGRAM: it links the CPU oracle (oracle/liboracle.so) as the checker.
 * Every routine's output is compared with the oracle on the same inputs:
 *   - info codes: identical to the oracle's (integer, exact);
 *   - POSV / POTRS / mixed POSV: normwise backward error of X*A = B per
 *     system <= 10*n*eps64, and B unchanged for systems with info > 0;
 *   - POTRF: ||A - L*L^T||_max / ||A||_max <= 10*n*eps64;
 *   - TRSM: |A*X - alpha*B| <= 10*m*eps64 * (|A|*|X|) elementwise;
 *   - SYRK: |C_gpu - C_oracle| <= 10*k*eps64 * (|A|*|A|^T + |C|) elementwise.
 *
 * usage: kblas_c_driver [batch n nrhs vbatch vmax_n]   (defaults 600 48 3 400 130)
 * Prints one line per routine and "ALL PASS" (exit 0), or FAIL lines (exit 1).
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include "kblas.h"

/* CPU oracle (oracle/kblas_oracle.c, oracle/oracle_impl.h) */
int oracle_dpotrf(int n, double *A, int lda);
void oracle_dpotrf_batch(int n, double *A, int lda, long strideA, int batch, int *info, int nthreads);
void oracle_dposv_batch(int m, int n, double *A, int lda, long strideA, double *B, int ldb,
                        long strideB, int batch, int *info, int nthreads);
void oracle_dsyrk(char uplo, char trans, int m, int k, double alpha, const double *A, int lda,
                  double beta, double *C, int ldc);
double oracle_backward_error_r(int m, int n, const double *A, int lda, const double *X, int ldx,
                               const double *B, int ldb);
double oracle_factor_backward_error(int n, const double *A, int lda, const double *L, int ldl);
int oracle_max_threads(void);

#define EPS64 1.1102230246251565e-16 /* 2^-53 */
#define AT(M, ld, i, j) (M)[(size_t)(i) + (size_t)(j) * (size_t)(ld)]

static int g_fail = 0;

#define CUDA_OK(call)                                                                   \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            fprintf(stderr, "CUDA error %s at %s:%d: %s\n", cudaGetErrorName(e_),       \
                    __FILE__, __LINE__, #call);                                         \
            exit(2);                                                                    \
        }                                                                               \
    } while (0)

#define KBLAS_OK(call)                                                                  \
    do {                                                                                \
        int s_ = (call);                                                                \
        if (s_ != KBLAS_Success) {                                                      \
            fprintf(stderr, "KBLAS error %d (%s) at %s:%d: %s\n", s_,                   \
                    kblasGetErrorString(s_), __FILE__, __LINE__, #call);                \
            exit(2);                                                                    \
        }                                                                               \
    } while (0)

/* splitmix64 stream, uniform (0,1) and Box-Muller normals */
static uint64_t g_rng = 0x243F6A8885A308D3ull;
static double urand(void)
{
    uint64_t z = (g_rng += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return ((double)(z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}
static double nrand(void)
{
    const double u = urand(), v = urand();
    return sqrt(-2.0 * log(u)) * cos(6.283185307179586 * v);
}

static int round_up32(int x) { return ((x + 31) / 32) * 32; }

/* A = G*G^T + n*I (G n x n, N(0,1)), full symmetric storage, column-major. */
static void make_spd(int n, double *A, int lda, double *G)
{
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) AT(G, n, i, j) = nrand();
    for (int j = 0; j < n; j++)
        for (int i = j; i < n; i++) {
            double s = 0;
            for (int k = 0; k < n; k++) s += AT(G, n, i, k) * AT(G, n, j, k);
            if (i == j) s += n;
            AT(A, lda, i, j) = s;
            AT(A, lda, j, i) = s;
        }
}

/* every 9th system loses definiteness at a chosen column k: info = k + 1 */
static int planted_minor(int b, int n) { return (b % 9 == 4 && n > 0) ? (b * 7) % n : -1; }

static void report(const char *name, int ok, const char *fmt, double v)
{
    printf("%-36s %s ", name, ok ? "PASS" : "FAIL");
    printf(fmt, v);
    printf("\n");
    if (!ok) g_fail = 1;
}

/* The copies and memsets below run on the legacy default stream, the library
 * on the handle's non-blocking stream: wait for the uploads before a call. */
static void uploads_done(void) { CUDA_OK(cudaDeviceSynchronize()); }

/* host (ld = rows) <-> device (ld = dld) copies of `cols` consecutive columns */
static void to_dev(double *d, int dld, const double *h, int rows, long cols)
{
    CUDA_OK(cudaMemcpy2D(d, (size_t)dld * sizeof(double), h, (size_t)rows * sizeof(double),
                         (size_t)rows * sizeof(double), (size_t)cols, cudaMemcpyHostToDevice));
}
static void to_host(double *h, int rows, const double *d, int dld, long cols)
{
    CUDA_OK(cudaMemcpy2D(h, (size_t)rows * sizeof(double), d, (size_t)dld * sizeof(double),
                         (size_t)rows * sizeof(double), (size_t)cols, cudaMemcpyDeviceToHost));
}

static double **device_ptr_array(double *base, long stride, int batch)
{
    double **h = (double **)malloc(sizeof(double *) * (size_t)(batch > 0 ? batch : 1));
    for (int b = 0; b < batch; b++) h[b] = base + (size_t)b * stride;
    double **d = NULL;
    CUDA_OK(cudaMalloc((void **)&d, sizeof(double *) * (size_t)(batch > 0 ? batch : 1)));
    CUDA_OK(cudaMemcpy(d, h, sizeof(double *) * (size_t)batch, cudaMemcpyHostToDevice));
    free(h);
    return d;
}

/* Compare GPU POSV results (X in Bg, info in ig) with the oracle's. */
static void check_posv(const char *name, int m, int n, int batch, const double *A0, const double *B0,
                       const double *Bg, const int *ig, const int *io)
{
    int info_exact = 1, untouched = 1;
    double worst = 0;
    for (int b = 0; b < batch; b++) {
        const double *A = A0 + (size_t)b * n * n;
        const double *B = B0 + (size_t)b * m * n;
        const double *X = Bg + (size_t)b * m * n;
        if (ig[b] != io[b]) info_exact = 0;
        if (io[b] > 0) {
            if (memcmp(X, B, sizeof(double) * (size_t)m * n) != 0) untouched = 0;
            continue;
        }
        const double eta = oracle_backward_error_r(m, n, A, n, X, m, B, m) / (10.0 * n * EPS64);
        if (!(eta <= worst)) worst = eta;
    }
    char buf[160];
    snprintf(buf, sizeof buf, "batch %d n %d nrhs %d: info exact %d, failed systems' B untouched %d, "
             "max eta/(10 n eps64) %%.3g", batch, n, m, info_exact, untouched);
    report(name, info_exact && untouched && worst <= 1.0, buf, worst);
}

int main(int argc, char **argv)
{
    const int batch = argc > 1 ? atoi(argv[1]) : 600;
    const int n = argc > 2 ? atoi(argv[2]) : 48;
    const int m = argc > 3 ? atoi(argv[3]) : 3; /* right-hand sides: B is m x n (side 'R') */
    const int vbatch = argc > 4 ? atoi(argv[4]) : 400;
    const int vmax = argc > 5 ? atoi(argv[5]) : 130;
    if (batch < 1 || n < 1 || m < 1 || vbatch < 1 || vmax < 1) {
        fprintf(stderr, "usage: %s [batch n nrhs vbatch vmax_n] (all >= 1)\n", argv[0]);
        return 2;
    }
    const int nth = oracle_max_threads();
    const int ldda = round_up32(n), lddb = round_up32(m);
    const long sA = (long)ldda * n, sB = (long)lddb * n;

    /* host inputs: A (lda = n), B (ldb = m), both column-major and contiguous */
    double *hA = (double *)malloc(sizeof(double) * (size_t)n * n * batch);
    double *hB = (double *)malloc(sizeof(double) * (size_t)m * n * batch);
    double *G = (double *)malloc(sizeof(double) * (size_t)n * n);
    for (int b = 0; b < batch; b++) {
        double *A = hA + (size_t)b * n * n;
        make_spd(n, A, n, G);
        const int k = planted_minor(b, n);
        if (k >= 0) AT(A, n, k, k) = -AT(A, n, k, k);
    }
    for (size_t i = 0; i < (size_t)m * n * batch; i++) hB[i] = nrand();

    /* oracle: POSV on copies */
    double *oA = (double *)malloc(sizeof(double) * (size_t)n * n * batch);
    double *oB = (double *)malloc(sizeof(double) * (size_t)m * n * batch);
    int *oinfo = (int *)malloc(sizeof(int) * (size_t)batch);
    memcpy(oA, hA, sizeof(double) * (size_t)n * n * batch);
    memcpy(oB, hB, sizeof(double) * (size_t)m * n * batch);
    oracle_dposv_batch(m, n, oA, n, (long)n * n, oB, m, (long)m * n, batch, oinfo, nth);

    kblasHandle_t h;
    KBLAS_OK(kblasCreate(&h));
    cudaStream_t stream;
    CUDA_OK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    kblasSetStream(h, stream);

    double *dA, *dB;
    int *dinfo, *diter;
    CUDA_OK(cudaMalloc((void **)&dA, sizeof(double) * (size_t)sA * batch));
    CUDA_OK(cudaMalloc((void **)&dB, sizeof(double) * (size_t)sB * batch));
    CUDA_OK(cudaMalloc((void **)&dinfo, sizeof(int) * (size_t)batch));
    CUDA_OK(cudaMalloc((void **)&diter, sizeof(int) * (size_t)batch));

    kblas_posv_batch_strided_wsquery(h, 'R', m, n, batch);
    kblas_posv_batch_wsquery(h, 'R', m, n, batch);
    kblas_potrf_batch_wsquery(h, n, batch);
    kblas_potrs_batch_wsquery(h, m, n, batch);
    kblas_trsm_batch_strided_wsquery(h, 'L', n, n, batch);
    kblas_syrk_batch_wsquery(h, n, batch);
    kblas_posv_batch_mixed_wsquery(h, 'R', m, n, batch);
    kblas_posv_vbatch_wsquery(h, vmax, vbatch);
    KBLAS_OK(kblasAllocateWorkspace(h));

    double *gA = (double *)malloc(sizeof(double) * (size_t)n * n * batch);
    double *gB = (double *)malloc(sizeof(double) * (size_t)m * n * batch);
    int *ginfo = (int *)malloc(sizeof(int) * (size_t)batch);
    int *giter = (int *)malloc(sizeof(int) * (size_t)batch);

    /* 1. kblasDposv_batch_strided, timed with the handle's timer */
    to_dev(dA, ldda, hA, n, (long)n * batch);
    to_dev(dB, lddb, hB, m, (long)n * batch);
    CUDA_OK(cudaMemset(dinfo, 0xff, sizeof(int) * (size_t)batch));
    uploads_done();
    kblasTimerTic(h);
    KBLAS_OK(kblasDposv_batch_strided(h, 'R', 'L', m, n, dA, ldda, sA, dB, lddb, sB, batch, dinfo));
    const double ms = kblasTimerToc(h);
    CUDA_OK(cudaStreamSynchronize(stream));
    to_host(gB, m, dB, lddb, (long)n * batch);
    CUDA_OK(cudaMemcpy(ginfo, dinfo, sizeof(int) * (size_t)batch, cudaMemcpyDeviceToHost));
    check_posv("kblasDposv_batch_strided", m, n, batch, hA, hB, gB, ginfo, oinfo);
    const double flops = (double)n * n * n / 3.0 + (double)n * n / 2.0 + (double)n / 6.0 + 2.0 * m * n * n;
    printf("%-36s %.1f GFLOP/s (%.3f ms)\n", "  timed (kblasTimerTic/Toc)", flops * batch / (ms * 1e6), ms);

    /* 2. pointer-array kblasDpotrf_batch + kblasDpotrs_batch */
    double **dAarr = device_ptr_array(dA, sA, batch);
    double **dBarr = device_ptr_array(dB, sB, batch);
    to_dev(dA, ldda, hA, n, (long)n * batch);
    to_dev(dB, lddb, hB, m, (long)n * batch);
    CUDA_OK(cudaMemset(dinfo, 0xff, sizeof(int) * (size_t)batch));
    uploads_done();
    KBLAS_OK(kblasDpotrf_batch(h, 'L', n, dAarr, ldda, batch, dinfo));
    CUDA_OK(cudaStreamSynchronize(stream));
    to_host(gA, n, dA, ldda, (long)n * batch);
    CUDA_OK(cudaMemcpy(ginfo, dinfo, sizeof(int) * (size_t)batch, cudaMemcpyDeviceToHost));
    {
        int info_exact = 1;
        double worst = 0;
        for (int b = 0; b < batch; b++) {
            if (ginfo[b] != oinfo[b]) info_exact = 0;
            if (oinfo[b] != 0) continue;
            const double e = oracle_factor_backward_error(n, hA + (size_t)b * n * n, n,
                                                          gA + (size_t)b * n * n, n) / (10.0 * n * EPS64);
            if (!(e <= worst)) worst = e;
        }
        char buf[160];
        snprintf(buf, sizeof buf, "batch %d n %d: info exact %d, max ||A-LL^T||/||A||/(10 n eps64) %%.3g",
                 batch, n, info_exact);
        report("kblasDpotrf_batch (pointer array)", info_exact && worst <= 1.0, buf, worst);
    }
    /* POTRS only on the systems that factored: their pointers, compacted */
    {
        int good = 0;
        for (int b = 0; b < batch; b++) good += oinfo[b] == 0;
        double **hpa = (double **)malloc(sizeof(double *) * (size_t)good);
        double **hpb = (double **)malloc(sizeof(double *) * (size_t)good);
        for (int b = 0, g = 0; b < batch; b++)
            if (oinfo[b] == 0) {
                hpa[g] = dA + (size_t)b * sA;
                hpb[g] = dB + (size_t)b * sB;
                g++;
            }
        double **dpa, **dpb;
        CUDA_OK(cudaMalloc((void **)&dpa, sizeof(double *) * (size_t)(good > 0 ? good : 1)));
        CUDA_OK(cudaMalloc((void **)&dpb, sizeof(double *) * (size_t)(good > 0 ? good : 1)));
        CUDA_OK(cudaMemcpy(dpa, hpa, sizeof(double *) * (size_t)good, cudaMemcpyHostToDevice));
        CUDA_OK(cudaMemcpy(dpb, hpb, sizeof(double *) * (size_t)good, cudaMemcpyHostToDevice));
        uploads_done();
        KBLAS_OK(kblasDpotrs_batch(h, 'R', 'L', m, n, (const double **)dpa, ldda, dpb, lddb, good));
        CUDA_OK(cudaStreamSynchronize(stream));
        to_host(gB, m, dB, lddb, (long)n * batch);
        double worst = 0;
        for (int b = 0; b < batch; b++) {
            if (oinfo[b] != 0) continue;
            const double e = oracle_backward_error_r(m, n, hA + (size_t)b * n * n, n, gB + (size_t)b * m * n,
                                                     m, hB + (size_t)b * m * n, m) / (10.0 * n * EPS64);
            if (!(e <= worst)) worst = e;
        }
        char buf[160];
        snprintf(buf, sizeof buf, "%d systems n %d nrhs %d: max eta/(10 n eps64) %%.3g", good, n, m);
        report("kblasDpotrs_batch (pointer array)", worst <= 1.0, buf, worst);
        CUDA_OK(cudaFree(dpa));
        CUDA_OK(cudaFree(dpb));
        free(hpa);
        free(hpb);
    }

    /* 3. kblasDposv_batch_mixed_strided (FP32 factor, FP64 refinement) */
    to_dev(dA, ldda, hA, n, (long)n * batch);
    to_dev(dB, lddb, hB, m, (long)n * batch);
    CUDA_OK(cudaMemset(dinfo, 0xff, sizeof(int) * (size_t)batch));
    uploads_done();
    KBLAS_OK(kblasDposv_batch_mixed_strided(h, 'R', 'L', m, n, dA, ldda, sA, dB, lddb, sB, batch, dinfo, diter));
    CUDA_OK(cudaStreamSynchronize(stream));
    to_host(gB, m, dB, lddb, (long)n * batch);
    CUDA_OK(cudaMemcpy(ginfo, dinfo, sizeof(int) * (size_t)batch, cudaMemcpyDeviceToHost));
    CUDA_OK(cudaMemcpy(giter, diter, sizeof(int) * (size_t)batch, cudaMemcpyDeviceToHost));
    check_posv("kblasDposv_batch_mixed_strided", m, n, batch, hA, hB, gB, ginfo, oinfo);

    /* 4. kblasDtrsm_batch_strided L/L/N/N, alpha = 0.5: L off-diagonal N(0,1)/sqrt(n),
     *    diagonal U[1,2] (the 64 x 64 TRSM benchmark's recipe), B N(0,1) n x n */
    {
        const int nr = n; /* B is n x n */
        const double alpha = 0.5;
        double *hX = (double *)malloc(sizeof(double) * (size_t)n * nr * batch);
        double *hL = (double *)malloc(sizeof(double) * (size_t)n * n * batch);
        for (int b = 0; b < batch; b++) {
            double *L = hL + (size_t)b * n * n;
            for (int j = 0; j < n; j++)
                for (int i = 0; i < n; i++)
                    AT(L, n, i, j) = i > j ? nrand() / sqrt((double)n) : (i == j ? 1.0 + urand() : 0.0);
        }
        double *hR = (double *)malloc(sizeof(double) * (size_t)n * nr * batch);
        for (size_t i = 0; i < (size_t)n * nr * batch; i++) hR[i] = nrand();
        double *dL, *dX;
        CUDA_OK(cudaMalloc((void **)&dL, sizeof(double) * (size_t)sA * batch));
        CUDA_OK(cudaMalloc((void **)&dX, sizeof(double) * (size_t)sA * batch));
        to_dev(dL, ldda, hL, n, (long)n * batch);
        to_dev(dX, ldda, hR, n, (long)nr * batch);
        uploads_done();
        KBLAS_OK(kblasDtrsm_batch_strided(h, 'L', 'L', 'N', 'N', n, nr, alpha, dL, ldda, sA, dX, ldda, sA, batch));
        CUDA_OK(cudaStreamSynchronize(stream));
        to_host(hX, n, dX, ldda, (long)nr * batch);
        double worst = 0;
        for (int b = 0; b < batch; b++) {
            const double *L = hL + (size_t)b * n * n, *X = hX + (size_t)b * n * nr, *R = hR + (size_t)b * n * nr;
            for (int j = 0; j < nr; j++)
                for (int i = 0; i < n; i++) {
                    long double s = -(long double)alpha * AT(R, n, i, j), sc = 0;
                    for (int k = 0; k <= i; k++) {
                        s += (long double)AT(L, n, i, k) * AT(X, n, k, j);
                        sc += fabsl((long double)AT(L, n, i, k) * AT(X, n, k, j));
                    }
                    const double r = (double)(fabsl(s) / (10.0L * n * EPS64 * sc + 1e-300L));
                    if (!(r <= worst)) worst = r;
                }
        }
        char buf[160];
        snprintf(buf, sizeof buf, "batch %d, %d x %d, L/L/N/N: max |AX-aB|/(10 n eps64 |A||X|) %%.3g", batch, n, nr);
        report("kblasDtrsm_batch_strided", worst <= 1.0, buf, worst);

        /* 5. kblasDsyrk_batch_strided C <- C - A*A^T (lower), A = hR's first n columns */
        double *hC = (double *)malloc(sizeof(double) * (size_t)n * n * batch);
        double *gC = (double *)malloc(sizeof(double) * (size_t)n * n * batch);
        for (int b = 0; b < batch; b++) make_spd(n, hC + (size_t)b * n * n, n, G);
        to_dev(dL, ldda, hR, n, (long)n * batch); /* A: n x n */
        to_dev(dX, ldda, hC, n, (long)n * batch); /* C */
        uploads_done();
        KBLAS_OK(kblasDsyrk_batch_strided(h, 'L', 'N', n, n, -1.0, dL, ldda, sA, 1.0, dX, ldda, sA, batch));
        CUDA_OK(cudaStreamSynchronize(stream));
        to_host(gC, n, dX, ldda, (long)n * batch);
        worst = 0;
        int upper_untouched = 1;
        for (int b = 0; b < batch; b++) {
            const double *A = hR + (size_t)b * n * n, *C0 = hC + (size_t)b * n * n, *Cg = gC + (size_t)b * n * n;
            double *Co = (double *)malloc(sizeof(double) * (size_t)n * n);
            memcpy(Co, C0, sizeof(double) * (size_t)n * n);
            oracle_dsyrk('L', 'N', n, n, -1.0, A, n, 1.0, Co, n);
            for (int j = 0; j < n; j++)
                for (int i = 0; i < n; i++) {
                    if (i < j) {
                        if (AT(Cg, n, i, j) != AT(C0, n, i, j)) upper_untouched = 0;
                        continue;
                    }
                    double sc = fabs(AT(C0, n, i, j));
                    for (int k = 0; k < n; k++) sc += fabs(AT(A, n, i, k) * AT(A, n, j, k));
                    const double r = fabs(AT(Cg, n, i, j) - AT(Co, n, i, j)) / (10.0 * n * EPS64 * sc + 1e-300);
                    if (!(r <= worst)) worst = r;
                }
            free(Co);
        }
        snprintf(buf, sizeof buf, "batch %d, %d x %d, C - A A^T: upper untouched %d, max diff/(10 k eps64 scale) %%.3g",
                 batch, n, n, upper_untouched);
        report("kblasDsyrk_batch_strided", upper_untouched && worst <= 1.0, buf, worst);
        CUDA_OK(cudaFree(dL));
        CUDA_OK(cudaFree(dX));
        free(hX);
        free(hL);
        free(hR);
        free(hC);
        free(gC);
    }

    /* 6. kblasDposv_vbatch_mixed: variable n in 1..vmax, lda = n + (b % 3), one RHS */
    {
        int *vn = (int *)malloc(sizeof(int) * (size_t)vbatch), *vm = (int *)malloc(sizeof(int) * (size_t)vbatch);
        int *vlda = (int *)malloc(sizeof(int) * (size_t)vbatch), *vldb = (int *)malloc(sizeof(int) * (size_t)vbatch);
        size_t *offA = (size_t *)malloc(sizeof(size_t) * (size_t)vbatch), *offB = (size_t *)malloc(sizeof(size_t) * (size_t)vbatch);
        size_t totA = 0, totB = 0;
        for (int b = 0; b < vbatch; b++) {
            vn[b] = 1 + (int)(urand() * vmax);
            if (vn[b] > vmax) vn[b] = vmax;
            vm[b] = 1;
            vlda[b] = vn[b] + b % 3;
            vldb[b] = 1;
            offA[b] = totA;
            offB[b] = totB;
            totA += ((size_t)vlda[b] * vn[b] + 1) & ~(size_t)1; /* 16-byte aligned starts */
            totB += (size_t)vn[b] + (vn[b] & 1);
        }
        double *vA = (double *)calloc(totA, sizeof(double)), *vB = (double *)calloc(totB, sizeof(double));
        double *vX = (double *)malloc(sizeof(double) * totB);
        double *Gv = (double *)malloc(sizeof(double) * (size_t)vmax * vmax);
        int *vinfo_o = (int *)malloc(sizeof(int) * (size_t)vbatch), *vinfo_g = (int *)malloc(sizeof(int) * (size_t)vbatch);
        double *Aw = (double *)malloc(sizeof(double) * (size_t)vmax * vmax);
        for (int b = 0; b < vbatch; b++) {
            double *A = vA + offA[b];
            make_spd(vn[b], A, vlda[b], Gv);
            const int k = planted_minor(b, vn[b]);
            if (k >= 0) AT(A, vlda[b], k, k) = -AT(A, vlda[b], k, k);
            for (int j = 0; j < vn[b]; j++) vB[offB[b] + j] = nrand();
            for (int j = 0; j < vn[b]; j++)
                for (int i = 0; i < vn[b]; i++) AT(Aw, vn[b], i, j) = AT(A, vlda[b], i, j);
            vinfo_o[b] = oracle_dpotrf(vn[b], Aw, vn[b]);
        }
        double *dvA, *dvB, **dvAarr, **dvBarr;
        int *dvn, *dvm, *dvlda, *dvldb, *dvinfo, *dviter;
        CUDA_OK(cudaMalloc((void **)&dvA, sizeof(double) * totA));
        CUDA_OK(cudaMalloc((void **)&dvB, sizeof(double) * totB));
        CUDA_OK(cudaMemcpy(dvA, vA, sizeof(double) * totA, cudaMemcpyHostToDevice));
        CUDA_OK(cudaMemcpy(dvB, vB, sizeof(double) * totB, cudaMemcpyHostToDevice));
        double **hpa = (double **)malloc(sizeof(double *) * (size_t)vbatch), **hpb = (double **)malloc(sizeof(double *) * (size_t)vbatch);
        for (int b = 0; b < vbatch; b++) {
            hpa[b] = dvA + offA[b];
            hpb[b] = dvB + offB[b];
        }
        CUDA_OK(cudaMalloc((void **)&dvAarr, sizeof(double *) * (size_t)vbatch));
        CUDA_OK(cudaMalloc((void **)&dvBarr, sizeof(double *) * (size_t)vbatch));
        CUDA_OK(cudaMemcpy(dvAarr, hpa, sizeof(double *) * (size_t)vbatch, cudaMemcpyHostToDevice));
        CUDA_OK(cudaMemcpy(dvBarr, hpb, sizeof(double *) * (size_t)vbatch, cudaMemcpyHostToDevice));
        int **dints[6] = {&dvn, &dvm, &dvlda, &dvldb, &dvinfo, &dviter};
        for (int i = 0; i < 6; i++) CUDA_OK(cudaMalloc((void **)dints[i], sizeof(int) * (size_t)vbatch));
        CUDA_OK(cudaMemcpy(dvn, vn, sizeof(int) * (size_t)vbatch, cudaMemcpyHostToDevice));
        CUDA_OK(cudaMemcpy(dvm, vm, sizeof(int) * (size_t)vbatch, cudaMemcpyHostToDevice));
        CUDA_OK(cudaMemcpy(dvlda, vlda, sizeof(int) * (size_t)vbatch, cudaMemcpyHostToDevice));
        CUDA_OK(cudaMemcpy(dvldb, vldb, sizeof(int) * (size_t)vbatch, cudaMemcpyHostToDevice));
        CUDA_OK(cudaMemset(dvinfo, 0xff, sizeof(int) * (size_t)vbatch));
        uploads_done();
        KBLAS_OK(kblasDposv_vbatch_mixed(h, 'R', 'L', dvm, dvn, 1, vmax, dvAarr, dvlda, dvBarr, dvldb, vbatch,
                                         dvinfo, dviter));
        CUDA_OK(cudaStreamSynchronize(stream));
        CUDA_OK(cudaMemcpy(vX, dvB, sizeof(double) * totB, cudaMemcpyDeviceToHost));
        CUDA_OK(cudaMemcpy(vinfo_g, dvinfo, sizeof(int) * (size_t)vbatch, cudaMemcpyDeviceToHost));
        int info_exact = 1, untouched = 1, nfail = 0;
        double worst = 0;
        for (int b = 0; b < vbatch; b++) {
            if (vinfo_g[b] != vinfo_o[b]) info_exact = 0;
            if (vinfo_o[b] > 0) {
                nfail++;
                if (memcmp(vX + offB[b], vB + offB[b], sizeof(double) * (size_t)vn[b]) != 0) untouched = 0;
                continue;
            }
            const double e = oracle_backward_error_r(1, vn[b], vA + offA[b], vlda[b], vX + offB[b], 1,
                                                     vB + offB[b], 1) / (10.0 * vn[b] * EPS64);
            if (!(e <= worst)) worst = e;
        }
        char buf[200];
        snprintf(buf, sizeof buf, "%d systems n 1..%d (%d not SPD): info exact %d, B untouched %d, "
                 "max eta/(10 n eps64) %%.3g", vbatch, vmax, nfail, info_exact, untouched);
        report("kblasDposv_vbatch_mixed", info_exact && untouched && worst <= 1.0, buf, worst);
        for (int i = 0; i < 6; i++) CUDA_OK(cudaFree(*dints[i]));
        CUDA_OK(cudaFree(dvA));
        CUDA_OK(cudaFree(dvB));
        CUDA_OK(cudaFree(dvAarr));
        CUDA_OK(cudaFree(dvBarr));
        free(vn); free(vm); free(vlda); free(vldb); free(offA); free(offB);
        free(vA); free(vB); free(vX); free(Gv); free(vinfo_o); free(vinfo_g); free(Aw); free(hpa); free(hpb);
    }

    /* argument errors come back as return codes, as in the reference */
    {
        const int st = kblasDpotrf_batch_strided(h, 'L', n, dA, n - 1 > 0 ? n - 1 : 0, sA, batch, dinfo);
        report("lda < n rejected", st == KBLAS_Error_WrongInput, "(status %.0f)", (double)st);
    }

    CUDA_OK(cudaFree(dAarr));
    CUDA_OK(cudaFree(dBarr));
    CUDA_OK(cudaFree(dA));
    CUDA_OK(cudaFree(dB));
    CUDA_OK(cudaFree(dinfo));
    CUDA_OK(cudaFree(diter));
    KBLAS_OK(kblasDestroy(&h));
    CUDA_OK(cudaStreamDestroy(stream));
    free(hA); free(hB); free(G); free(oA); free(oB); free(oinfo); free(gA); free(gB); free(ginfo); free(giter);
    printf("%s\n", g_fail ? "FAIL" : "ALL PASS");
    return g_fail ? 1 : 0;
}

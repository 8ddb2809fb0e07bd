// inverse.cu -- batched TRTRI / LAUUM / POTRI / POTI, single and
// double precision, strided and pointer-array forms.
//
// Entry points replace reference src/batch_triangular/Xtrtri_batch.cu:86,
// Xlauum_batch.cu:86, Xpotri_batch.cu:86 and Xpoti_batch.cu:86 (names and
// arguments of include/kblas_batch.h:1611-2729). The reference returns
// KBLAS_NotImplemented for Upper; here Upper runs the lower kernel between two
// in-place transposes. TRTRI also takes a unit diagonal (a superset: the
// reference supports non-unit only). info follows LAPACK: TRTRI / POTRI
// report the first zero diagonal entry of the triangle (1-based) and leave A
// unchanged; POTI reports the first non-positive pivot of its Cholesky step and
// leaves A as LAPACK xPOTRF does.
//
// One CTA per matrix. The lower triangle is staged in shared memory as a dense
// column-major block with an odd leading dimension (conflict-free column and
// row walks) when it fits, else processed in place in global memory; the
// algorithms are LAPACK's unblocked ones with the rows spread over the threads:
//   TRTRI  columns from the last: X(j,j) = 1/L(j,j), X(i,j) = -X(j,j) *
//          sum_{k=j+1..i} X(i,k) L(k,j) for i > j (xTRTI2);
//   LAUUM  rows from the first: row i of L^T L from rows >= i of L (xLAUU2);
//   POTRI  TRTRI then LAUUM;  POTI  a left-looking Cholesky, then POTRI.
#include <stdio.h>

#include <cuComplex.h>

#include "device_util.cuh"
#include "kblas_internal.h"
#include "launch_util.h"
#include "uplo_swap.cuh"

namespace kgb {

enum { INV_TRTRI = 0, INV_LAUUM = 1, INV_POTRI = 2, INV_POTI = 3 };
constexpr int INV_ROWS = 4;        // rows (or columns) per thread and step
constexpr int INV_MAX_N = 1024;    // = INV_ROWS * 256 threads

template <typename T>
__device__ __forceinline__ T &el(T *M, int ld, int i, int j) { return M[(size_t)i + (size_t)j * ld]; }

// in-place inverse of the lower triangle (M, ld), all threads of the block
template <typename T>
__device__ void blk_trtri(T *M, int ld, int n, bool unit)
{
  for (int j = n - 1; j >= 0; j--) {
    T xjj = T(1);
    if (!unit) xjj = T(1) / el(M, ld, j, j);
    // t_i = sum_{k=j+1..i} X(i,k) L(k,j), X(i,i) already inverted (1 for unit)
    T t[INV_ROWS];
    int r = 0;
    for (int i = j + 1 + threadIdx.x; i < n && r < INV_ROWS; i += blockDim.x, r++) {
      T s0 = unit ? el(M, ld, i, j) : el(M, ld, i, i) * el(M, ld, i, j), s1 = T(0);
      int k = j + 1;
      for (; k + 1 < i; k += 2) {
        s0 += el(M, ld, i, k) * el(M, ld, k, j);
        s1 += el(M, ld, i, k + 1) * el(M, ld, k + 1, j);
      }
      if (k < i) s0 += el(M, ld, i, k) * el(M, ld, k, j);
      t[r] = s0 + s1;
    }
    __syncthreads();
    r = 0;
    for (int i = j + 1 + threadIdx.x; i < n && r < INV_ROWS; i += blockDim.x, r++) el(M, ld, i, j) = -xjj * t[r];
    if (threadIdx.x == 0 && !unit) el(M, ld, j, j) = xjj;
    __syncthreads();
  }
}

// in place: lower triangle of L^T L over L
template <typename T>
__device__ void blk_lauum(T *M, int ld, int n)
{
  for (int i = 0; i < n; i++) {
    T t[INV_ROWS];
    int r = 0;
    for (int j = threadIdx.x; j <= i && r < INV_ROWS; j += blockDim.x, r++) {
      T s0 = T(0), s1 = T(0);
      int k = i;
      for (; k + 1 < n; k += 2) {
        s0 += el(M, ld, k, i) * el(M, ld, k, j);
        s1 += el(M, ld, k + 1, i) * el(M, ld, k + 1, j);
      }
      if (k < n) s0 += el(M, ld, k, i) * el(M, ld, k, j);
      t[r] = s0 + s1;
    }
    __syncthreads();
    r = 0;
    for (int j = threadIdx.x; j <= i && r < INV_ROWS; j += blockDim.x, r++) el(M, ld, i, j) = t[r];
    __syncthreads();
  }
}

// left-looking Cholesky (xPOTF2 order); returns the 1-based failing column
// or 0; on failure M(j,j) holds the non-positive pivot and later columns are
// untouched, as LAPACK leaves them
template <typename T>
__device__ int blk_potrf(T *M, int ld, int n, int *s_flag)
{
  for (int j = 0; j < n; j++) {
    if (threadIdx.x < 32) {
      T s = T(0);
      for (int k = threadIdx.x; k < j; k += 32) s += el(M, ld, j, k) * el(M, ld, j, k);
      for (int o = 16; o > 0; o >>= 1) s += shfl_xor_t(s, o);
      if (threadIdx.x == 0) {
        const T d = el(M, ld, j, j) - s;
        const bool ok = is_pos_pivot(d);  // real: d > 0, false for NaN
        el(M, ld, j, j) = ok ? pivot_sqrt(d) : d;
        *s_flag = ok ? 0 : j + 1;
      }
    }
    __syncthreads();
    const int f = *s_flag;
    if (f) return f;
    const T rjj = T(1) / el(M, ld, j, j);
    for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) {
      T s0 = el(M, ld, i, j), s1 = T(0);
      int k = 0;
      for (; k + 1 < j; k += 2) {
        s0 -= el(M, ld, i, k) * el(M, ld, j, k);
        s1 -= el(M, ld, i, k + 1) * el(M, ld, j, k + 1);
      }
      if (k < j) s0 -= el(M, ld, i, k) * el(M, ld, j, k);
      el(M, ld, i, j) = (s0 + s1) * rjj;
    }
    __syncthreads();
  }
  return 0;
}

template <typename T, int OP, bool SMEM, class Acc>
__global__ void __launch_bounds__(256) inverse_kernel(int n, Acc A, int lda, long long batch,
                                                      int *info, int unit)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_flag;
  const long long b = blockIdx.x;
  if (b >= batch) return;
  T *G = A.get(b);
  T *M = G;
  int ld = lda;
  if (SMEM) {
    M = reinterpret_cast<T *>(smem_raw);
    ld = n | 1;  // odd leading dimension
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const int j = e / n, i = e - j * n;
      if (i >= j) el(M, ld, i, j) = el(G, lda, i, j);
    }
    __syncthreads();
  }
  int inf = 0;
  if (OP == INV_TRTRI || OP == INV_POTRI) {
    // a zero diagonal entry: report the first, change nothing (every thread
    // scans the diagonal, so all agree without a reduction)
    if (!(OP == INV_TRTRI && unit))
      for (int j = 0; j < n; j++)
        if (el(M, ld, j, j) == T(0)) {
          inf = j + 1;
          break;
        }
  }
  if (OP == INV_POTI) inf = blk_potrf<T>(M, ld, n, &s_flag);
  if (!inf) {
    if (OP == INV_TRTRI) blk_trtri<T>(M, ld, n, unit != 0);
    if (OP == INV_POTRI || OP == INV_POTI) blk_trtri<T>(M, ld, n, false);
    if (OP != INV_TRTRI) blk_lauum<T>(M, ld, n);
  }
  if (SMEM && (!inf || OP == INV_POTI)) {
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const int j = e / n, i = e - j * n;
      if (i >= j) el(G, lda, i, j) = el(M, ld, i, j);
    }
  }
  if (info && threadIdx.x == 0) info[b] = inf;
}

// checks of the reference drivers (Xtrtri_batch_drivers.cuh:91-99 and the
// uplo tests of the LAUUM / POTRI / POTI drivers)
static int check_inverse(KBlasHandle *h, char uplo, char diag, bool has_diag, int n, int lda,
                         int batch, const void *A, const char *name) {
  (void)name;
  if (!h) return KBLAS_Error_NotInitialized;
  if (!is_lower(uplo) && !is_upper(uplo)) return KBLAS_Error_WrongInput;
  if (has_diag && !is_unit(diag) && !is_nonunit(diag)) return KBLAS_Error_WrongInput;
  if (n < 0 || batch < 0 || lda < (n > 1 ? n : 1)) return KBLAS_Error_WrongInput;
  if (n > 0 && batch > 0 && !A) return KBLAS_Error_WrongInput;
  return KBLAS_Success;
}

template <typename T, int OP, class Acc>
static int launch_inverse(KBlasHandle *h, int n, Acc A, int lda, int batch, int *info, bool unit) {
  if (batch == 0) return KBLAS_Success;
  if (n == 0) return zero_info(h, info, batch);
  if (n > INV_MAX_N) return KBLAS_NotSupported;
  const int threads = n >= 256 ? 256 : ((n + 31) / 32) * 32;
  const size_t smem = (size_t)(n | 1) * n * sizeof(T);
  if ((long long)smem <= max_smem(h)) {
    auto kern = inverse_kernel<T, OP, true, Acc>;
    int st = set_smem(kern, smem);
    if (st != KBLAS_Success) return st;
    kern<<<(unsigned)batch, threads, smem, h->stream>>>(n, A, lda, batch, info, unit ? 1 : 0);
  } else {
    inverse_kernel<T, OP, false, Acc><<<(unsigned)batch, threads, 0, h->stream>>>(
        n, A, lda, batch, info, unit ? 1 : 0);
  }
  KGB_LAUNCH_CHECK("inverse_kernel");
  return KBLAS_Success;
}

// uplo 'U': the lower kernel between two in-place transposes (uplo_swap.cuh):
// the upper factor U is L^T of A^T, inv(U) = inv(L)^T, U U^T = (L^T L)^T
// stored as its upper triangle, inv(A) likewise.
template <typename T, int OP, class Acc>
static int launch_inverse_uplo(KBlasHandle *h, bool upper, int n, Acc A, int lda, int batch,
                               int *info, bool unit) {
  if (!upper || n <= 1 || batch == 0)
    return launch_inverse<T, OP>(h, n, A, lda, batch, info, unit);
  if (n > INV_MAX_N) return KBLAS_NotSupported;
  int st = swap_uplo<T>(h, n, A, lda, batch);
  if (st != KBLAS_Success) return st;
  st = launch_inverse<T, OP>(h, n, A, lda, batch, info, unit);
  const int st2 = swap_uplo<T>(h, n, A, lda, batch);
  return st != KBLAS_Success ? st : st2;
}

template <typename T, int OP>
static int inv_strided(KBlasHandle *h, char uplo, char diag, int n, T *A, int lda, long long sA,
                       int batch, int *info, const char *name) {
  int st = check_inverse(h, uplo, diag, OP == INV_TRTRI, n, lda, batch, A, name);
  if (st != KBLAS_Success) return st;
  if (batch > 1 && sA < (long long)lda * n) return KBLAS_Error_WrongInput;
  return launch_inverse_uplo<T, OP>(h, is_upper(uplo), n, Strided<T>{A, sA}, lda, batch, info,
                                    OP == INV_TRTRI && is_unit(diag));
}

template <typename T, int OP>
static int inv_array(KBlasHandle *h, char uplo, char diag, int n, T **A, int lda, int batch,
                     int *info, const char *name) {
  int st = check_inverse(h, uplo, diag, OP == INV_TRTRI, n, lda, batch, A, name);
  if (st != KBLAS_Success) return st;
  return launch_inverse_uplo<T, OP>(h, is_upper(uplo), n, PtrArr<T>{A}, lda, batch, info,
                                    OP == INV_TRTRI && is_unit(diag));
}

}  // namespace kgb

using namespace kgb;

extern "C" {

// no workspace: one launch per call
void kblas_trtri_batch_wsquery(kblasHandle_t, const int, int) {}
void kblas_trtri_batch_strided_wsquery(kblasHandle_t, const int, int) {}
void kblas_lauum_batch_wsquery(kblasHandle_t, const int, int) {}
void kblas_lauum_batch_strided_wsquery(kblasHandle_t, const int, int) {}
void kblas_potri_batch_wsquery(kblasHandle_t, const int, int) {}
void kblas_potri_batch_strided_wsquery(kblasHandle_t, const int, int) {}
void kblas_poti_batch_wsquery(kblasHandle_t, const int, int) {}
void kblas_poti_batch_strided_wsquery(kblasHandle_t, const int, int) {}

#define KGB_INV_ENTRIES(X, API, T)                                                                   \
  int kblas##X##trtri_batch(kblasHandle_t h, char uplo, char diag, const int n, API **A, int lda, \
                            int batchCount, int *info) {                                        \
    return inv_array<T, INV_TRTRI>(h, uplo, diag, n, reinterpret_cast<T **>(A), lda, batchCount, info, "TRTRI");         \
  }                                                                                             \
  int kblas##X##trtri_batch_strided(kblasHandle_t h, char uplo, char diag, const int n, API *A,   \
                                    int lda, long strideA, int batchCount, int *info) {         \
    return inv_strided<T, INV_TRTRI>(h, uplo, diag, n, reinterpret_cast<T *>(A), lda, strideA, batchCount, info,       \
                                     "TRTRI");                                                  \
  }                                                                                             \
  int kblas##X##lauum_batch(kblasHandle_t h, char uplo, const int n, API **A, int lda,             \
                            int batchCount, int *info) {                                        \
    return inv_array<T, INV_LAUUM>(h, uplo, 'N', n, reinterpret_cast<T **>(A), lda, batchCount, info, "LAUUM");          \
  }                                                                                             \
  int kblas##X##lauum_batch_strided(kblasHandle_t h, char uplo, const int n, API *A, int lda,     \
                                    long strideA, int batchCount, int *info) {                  \
    return inv_strided<T, INV_LAUUM>(h, uplo, 'N', n, reinterpret_cast<T *>(A), lda, strideA, batchCount, info,        \
                                     "LAUUM");                                                  \
  }                                                                                             \
  int kblas##X##potri_batch(kblasHandle_t h, char uplo, const int n, API **A, int lda,             \
                            int batchCount, int *info) {                                        \
    return inv_array<T, INV_POTRI>(h, uplo, 'N', n, reinterpret_cast<T **>(A), lda, batchCount, info, "POTRI");          \
  }                                                                                             \
  int kblas##X##potri_batch_strided(kblasHandle_t h, char uplo, const int n, API *A, int lda,     \
                                    long strideA, int batchCount, int *info) {                  \
    return inv_strided<T, INV_POTRI>(h, uplo, 'N', n, reinterpret_cast<T *>(A), lda, strideA, batchCount, info,        \
                                     "POTRI");                                                  \
  }                                                                                             \
  int kblas##X##poti_batch(kblasHandle_t h, char uplo, const int n, API **A, int lda,              \
                           int batchCount, int *info) {                                         \
    return inv_array<T, INV_POTI>(h, uplo, 'N', n, reinterpret_cast<T **>(A), lda, batchCount, info, "POTI");            \
  }                                                                                             \
  int kblas##X##poti_batch_strided(kblasHandle_t h, char uplo, const int n, API *A, int lda,      \
                                   long strideA, int batchCount, int *info) {                   \
    return inv_strided<T, INV_POTI>(h, uplo, 'N', n, reinterpret_cast<T *>(A), lda, strideA, batchCount, info,         \
                                    "POTI");                                                    \
  }

KGB_INV_ENTRIES(S, float, float)
KGB_INV_ENTRIES(D, double, double)
KGB_INV_ENTRIES(C, cuFloatComplex, cxf)
KGB_INV_ENTRIES(Z, cuDoubleComplex, cxd)
#undef KGB_INV_ENTRIES

}  // extern "C"

// potrf_posv.cu -- batched POTRF / POTRS / POSV, single and double precision,
// strided and pointer-array forms.
//
// Entry points replace reference src/batch_triangular/Xpotrf_batch.cu:86-160,
// Xpotrs_batch.cu:87-165 and Xposv_batch.cu:92-178 (same names, arguments,
// flag support and return codes). Unlike the reference (host recursion over
// TRSM + SYRK + cuBLAS GEMM, 4 launches at n = 32 and one HBM pass per level),
// every call is ONE kernel launch: for n <= 32 the team kernel (POTRS of real
// types: the register kernel, chol_reg.cuh) and, above,
// the persistent panel kernel (double precision, when the workspace the
// wsqueries request is allocated) or the blocked panel kernel (see
// chol_kernels.cuh).
#include <stdio.h>
#include <type_traits>

#include <cuComplex.h>

#include "chol_kernels.cuh"
#include "chol_reg.cuh"
#include "kblas_internal.h"
#include "launch_util.h"
#include "posv_launch.h"
#include "tri_internal.h"
#include "uplo_swap.cuh"

namespace kgb {

// Team size (lanes per matrix) for the n <= 32 kernel.
static inline int team_size_for(int n, bool dbl) {
  if (n <= 4) return 2;
  if (n <= 12) return 4;
  if (n <= 24) return dbl ? 8 : 8;
  return 8;
}

template <typename T, int G, int MODE, class AccA, class AccB>
static int launch_team(KBlasHandle *h, int n, int m, AccA A, int lda, AccB B, int ldb,
                       long long batch, int *info) {
  constexpr int NT = 128;
  constexpr int TPB = NT / G;
  int rc = (MODE == MODE_POTRF) ? 0 : (m < 8 ? m : 8);
  size_t smem = (size_t)TPB * team_smem_elems<T>(n, rc) * sizeof(T);
  auto kern = chol_team_kernel<T, G, NT, MODE, AccA, AccB>;
  int st = set_smem(kern, smem);
  if (st != KBLAS_Success) return st;
  long long grid = (batch + TPB - 1) / TPB;
  kern<<<(unsigned)grid, NT, smem, h->stream>>>(n, m, rc, A, lda, B, ldb, batch, info);
  KGB_LAUNCH_CHECK("chol_team_kernel");
  return KBLAS_Success;
}

// POTRS, n <= 32, real types: one factor per W-lane segment, rows in registers.
template <typename T, int W, class AccA, class AccB>
static int launch_potrs_reg(KBlasHandle *h, int n, int m, AccA A, int lda, AccB B, int ldb,
                            long long batch) {
  constexpr int NT = 128;
  constexpr int SPB = NT / W;  // systems per CTA
  const size_t smem = (size_t)SPB * reg_square_elems<T, W>() * sizeof(T);
  auto kern = potrs_reg_kernel<T, W, NT, AccA, AccB>;
  int st = set_smem(kern, smem);
  if (st != KBLAS_Success) return st;
  long long grid = (batch + SPB - 1) / SPB;
  kern<<<(unsigned)grid, NT, smem, h->stream>>>(n, m, A, lda, B, ldb, batch);
  KGB_LAUNCH_CHECK("potrs_reg_kernel");
  return KBLAS_Success;
}

template <typename T, int NB, int MODE, class AccA, class AccB>
static int launch_blocked_nb(KBlasHandle *h, int n, int m, AccA A, int lda, AccB B, int ldb,
                             long long batch, int *info, size_t smem, int rc) {
  constexpr int KC = 32;
  constexpr int NT = 256;
  auto kern = chol_blocked_kernel<T, NB, KC, NT, MODE, AccA, AccB>;
  int st = set_smem(kern, smem);
  if (st != KBLAS_Success) return st;
  kern<<<(unsigned)batch, NT, smem, h->stream>>>(n, m, rc, A, lda, B, ldb, batch, info);
  KGB_LAUNCH_CHECK("chol_blocked_kernel");
  return KBLAS_Success;
}

template <typename T, int MODE, class AccA, class AccB>
static int launch_chol(KBlasHandle *h, int n, int m, AccA A, int lda, AccB B, int ldb,
                       long long batch, int *info) {
  // POTRS of order <= 32 runs on the register kernel (real types). POTRF and
  // POSV stay on the team kernel: the register factorization keeps a row per
  // lane, so at column c only the rows below c do useful work, and on this
  // part an FP64 instruction costs its issue slot whether or not its lane is
  // predicated off -- it measured slower (n = 32, 10,000 matrices: POTRF 438
  // vs 310 us, POSV 605 vs 369 us; POTRS 105 vs 122 us).
  if constexpr (MODE == MODE_POTRS &&
                (std::is_same<T, double>::value || std::is_same<T, float>::value)) {
    if (n <= 8) return launch_potrs_reg<T, 8>(h, n, m, A, lda, B, ldb, batch);
    if (n <= 16) return launch_potrs_reg<T, 16>(h, n, m, A, lda, B, ldb, batch);
    if (n <= 32) return launch_potrs_reg<T, 32>(h, n, m, A, lda, B, ldb, batch);
  }
  if (n <= 32) {
    switch (team_size_for(n, std::is_same<T, double>::value)) {
      case 2: return launch_team<T, 2, MODE>(h, n, m, A, lda, B, ldb, batch, info);
      case 4: return launch_team<T, 4, MODE>(h, n, m, A, lda, B, ldb, batch, info);
      default: return launch_team<T, 8, MODE>(h, n, m, A, lda, B, ldb, batch, info);
    }
  }
  const int limit = max_smem(h);
  int rc = (MODE == MODE_POTRF) ? 0 : (m < 8 ? m : 8);
  size_t s32 = blocked_smem_elems<T, 32, 32>(n, rc) * sizeof(T);
  if ((long long)s32 <= limit)
    return launch_blocked_nb<T, 32, MODE>(h, n, m, A, lda, B, ldb, batch, info, s32, rc);
  if (rc > 1) rc = 1;
  size_t s16 = blocked_smem_elems<T, 16, 32>(n, rc) * sizeof(T);
  if ((long long)s16 <= limit)
    return launch_blocked_nb<T, 16, MODE>(h, n, m, A, lda, B, ldb, batch, info, s16, rc);
  fprintf(stderr, "KBLAS: batched Cholesky of order %d exceeds the on-chip panel limit\n", n);
  return KBLAS_NotSupported;
}

// Uniform FP64 orders 33..1024 go to the persistent panel path when the
// handle's workspace covers it (posv_vbatch.cu; the wsqueries request it): for
// 33 <= n <= 192 it is 1.3-2.9x faster than the one-launch blocked kernel
// below, which remains the path when no workspace was allocated.
size_t fp64_uniform_ws_bytes(KBlasHandle *h, int n, long long batch);
int fp64_uniform_persistent(KBlasHandle *h, int op, int m, int n, SysArgs sys, int batch, int *info);

template <typename T, class AccA, class AccB>
static int try_persistent(KBlasHandle *h, int op, int m, int n, AccA A, int lda, AccB B, int ldb,
                          int batch, int *info) {
  if (!std::is_same<T, double>::value || n <= 32 || n > PC_MAX_N) return KBLAS_InsufficientWorkspace;
  SysArgs s{};
  if constexpr (std::is_same<AccA, Strided<T>>::value) {
    s.mode = 0;
    s.A = reinterpret_cast<double *>(A.base);
    s.sA = A.stride;
    s.B = reinterpret_cast<double *>(B.base);
    s.sB = B.stride;
  } else {
    s.mode = 1;
    s.Aarr = reinterpret_cast<double *const *>(A.arr);
    s.Barr = reinterpret_cast<double *const *>(B.arr);
  }
  s.lda = lda;
  s.ldb = ldb;
  return fp64_uniform_persistent(h, op, m, n, s, batch, info);
}

// ------------------------------- checks ---------------------------------
static inline int check_potrf(KBlasHandle *h, char uplo, int n, const void *A, int lda,
                              int batch) {
  if (!h) return KBLAS_Error_NotInitialized;
  if (!is_lower(uplo) && !is_upper(uplo)) return KBLAS_Error_WrongInput;
  if (n < 0 || batch < 0 || lda < (n > 1 ? n : 1)) return KBLAS_Error_WrongInput;
  if (n > 0 && batch > 0 && !A) return KBLAS_Error_WrongInput;
  return KBLAS_Success;
}

// B is m x n in both sides; A is n x n for side 'R' (X A = B) and m x m for
// side 'L' (A X = B), the TRSM convention of the reference header.
static inline int check_potrs(KBlasHandle *h, char side, char uplo, int m, int n, const void *A,
                              int lda, const void *B, int ldb, int batch) {
  if (!h) return KBLAS_Error_NotInitialized;
  if (!(is_left(side) || is_right(side)) || !(is_lower(uplo) || is_upper(uplo)))
    return KBLAS_Error_WrongInput;
  const int order = is_left(side) ? m : n;
  if (m < 0 || n < 0 || batch < 0 || lda < (order > 1 ? order : 1) || ldb < (m > 1 ? m : 1))
    return KBLAS_Error_WrongInput;
  if (order > 0 && batch > 0 && (!A || (m > 0 && n > 0 && !B))) return KBLAS_Error_WrongInput;
  return KBLAS_Success;
}

// ------------------------------ drivers ---------------------------------
// Lower factorization of order n on the fastest path available.
template <typename T, class AccA>
static int potrf_lower(KBlasHandle *h, int n, AccA A, int lda, long long batch, int *info) {
  int st = try_persistent<T>(h, 1, 0, n, A, lda, AccA{}, 1, (int)batch, info);
  if (st != KBLAS_InsufficientWorkspace) return st;
  return launch_chol<T, MODE_POTRF>(h, n, 0, A, lda, AccA{}, 1, batch, info);
}

// uplo = 'U': the lower kernels run between two in-place transposes
// (uplo_swap.cuh); a kernel that did not launch leaves A as it was.
template <typename T, class AccA>
static int potrf_any(KBlasHandle *h, bool upper, int n, AccA A, int lda, long long batch,
                     int *info) {
  if (!upper) return potrf_lower<T>(h, n, A, lda, batch, info);
  int st = swap_uplo<T>(h, n, A, lda, batch);
  if (st != KBLAS_Success) return st;
  st = potrf_lower<T>(h, n, A, lda, batch, info);
  const int st2 = swap_uplo<T>(h, n, A, lda, batch);
  return st != KBLAS_Success ? st : st2;
}

// Solve with a Cholesky factor by two TRSM passes (every side / uplo but
// side 'R' + lower, which the fused kernels cover):
//   side R, L: X L L^T = B     -> B L^-T, then L^-1 (reference Xpotrs_batch_drivers.cuh:94-171)
//   side R, U: X U^T U = B     -> B U^-1, then U^-T
//   side L, L: L L^T X = B     -> L^-1 B, then L^-T
//   side L, U: U^T U X = B     -> U^-T B, then U^-1
// skip (device info or null): systems whose factorization failed are left as is.
template <typename T, class AccA, class AccB>
static int potrs_trsm(KBlasHandle *h, char side, char uplo, int m, int n, AccA A, int lda, AccB B,
                      int ldb, long long batch, const int *skip) {
  const bool left = is_left(side), lower = is_lower(uplo);
  const char first = (left == lower) ? 'N' : 'T';
  const char second = (first == 'N') ? 'T' : 'N';
  int st = trsm_batch_internal<T>(h, side, uplo, first, 'N', m, n, T(1), A, lda, B, ldb, batch, skip);
  if (st != KBLAS_Success) return st;
  return trsm_batch_internal<T>(h, side, uplo, second, 'N', m, n, T(1), A, lda, B, ldb, batch, skip);
}

template <typename T, class AccA, class AccB>
static int potrs_any(KBlasHandle *h, char side, char uplo, int m, int n, AccA A, int lda, AccB B,
                     int ldb, long long batch) {
  if (batch == 0 || n == 0 || m == 0) return KBLAS_Success;
  if (is_right(side) && is_lower(uplo)) {
    int st = try_persistent<T>(h, 2, m, n, A, lda, B, ldb, (int)batch, nullptr);
    if (st != KBLAS_InsufficientWorkspace) return st;
    return launch_chol<T, MODE_POTRS>(h, n, m, A, lda, B, ldb, batch, nullptr);
  }
  return potrs_trsm<T>(h, side, uplo, m, n, A, lda, B, ldb, batch, nullptr);
}

template <typename T, class AccA, class AccB>
static int posv_any(KBlasHandle *h, char side, char uplo, int m, int n, AccA A, int lda, AccB B,
                    int ldb, long long batch, int *info) {
  if (batch == 0) return KBLAS_Success;
  const bool left = is_left(side), upper = is_upper(uplo);
  const int order = left ? m : n, nrhs = left ? n : m;
  if (order == 0) return zero_info(h, info, batch);
  if (nrhs == 0) return potrf_any<T>(h, upper, order, A, lda, batch, info);
  if (!left) {
    // side R: the fused factor + solve kernels (on A^T for uplo 'U')
    if (upper) {
      int st = swap_uplo<T>(h, order, A, lda, batch);
      if (st != KBLAS_Success) return st;
    }
    int st = try_persistent<T>(h, 0, m, n, A, lda, B, ldb, (int)batch, info);
    if (st == KBLAS_InsufficientWorkspace)
      st = launch_chol<T, MODE_POSV>(h, n, m, A, lda, B, ldb, batch, info);
    if (upper) {
      const int st2 = swap_uplo<T>(h, order, A, lda, batch);
      if (st == KBLAS_Success) st = st2;
    }
    return st;
  }
  // side L: factor, then two TRSM passes that skip the systems whose info > 0
  int st = potrf_any<T>(h, upper, order, A, lda, batch, info);
  if (st != KBLAS_Success) return st;
  return potrs_trsm<T>(h, side, uplo, m, n, A, lda, B, ldb, batch, info);
}

template <typename T>
static int potrf_strided(KBlasHandle *h, char uplo, int n, T *A, int lda, long long sA, int batch,
                         int *info) {
  int st = check_potrf(h, uplo, n, A, lda, batch);
  if (st != KBLAS_Success) return st;
  if (batch > 1 && sA < (long long)lda * n) return KBLAS_Error_WrongInput;
  if (batch == 0) return KBLAS_Success;
  if (n == 0) return zero_info(h, info, batch);
  return potrf_any<T>(h, is_upper(uplo), n, Strided<T>{A, sA}, lda, batch, info);
}

template <typename T>
static int potrf_array(KBlasHandle *h, char uplo, int n, T **A, int lda, int batch, int *info) {
  int st = check_potrf(h, uplo, n, A, lda, batch);
  if (st != KBLAS_Success) return st;
  if (batch == 0) return KBLAS_Success;
  if (n == 0) return zero_info(h, info, batch);
  return potrf_any<T>(h, is_upper(uplo), n, PtrArr<T>{A}, lda, batch, info);
}

template <typename T>
static int potrs_strided(KBlasHandle *h, char side, char uplo, int m, int n, const T *A, int lda,
                         long long sA, T *B, int ldb, long long sB, int batch) {
  int st = check_potrs(h, side, uplo, m, n, A, lda, B, ldb, batch);
  if (st != KBLAS_Success) return st;
  const int order = is_left(side) ? m : n;
  if (batch > 1 && (sB < (long long)ldb * n || sA < (long long)lda * order))
    return KBLAS_Error_WrongInput;
  return potrs_any<T>(h, side, uplo, m, n, Strided<T>{const_cast<T *>(A), sA}, lda,
                      Strided<T>{B, sB}, ldb, batch);
}

template <typename T>
static int potrs_array(KBlasHandle *h, char side, char uplo, int m, int n, const T **A, int lda,
                       T **B, int ldb, int batch) {
  int st = check_potrs(h, side, uplo, m, n, A, lda, B, ldb, batch);
  if (st != KBLAS_Success) return st;
  return potrs_any<T>(h, side, uplo, m, n, PtrArr<T>{const_cast<T **>(A)}, lda, PtrArr<T>{B}, ldb,
                      batch);
}

template <typename T>
static int posv_strided(KBlasHandle *h, char side, char uplo, int m, int n, T *A, int lda,
                        long long sA, T *B, int ldb, long long sB, int batch, int *info) {
  int st = check_potrs(h, side, uplo, m, n, A, lda, B, ldb, batch);
  if (st != KBLAS_Success) return st;
  const int order = is_left(side) ? m : n;
  if (batch > 1 && (sA < (long long)lda * order || (m > 0 && n > 0 && sB < (long long)ldb * n)))
    return KBLAS_Error_WrongInput;
  return posv_any<T>(h, side, uplo, m, n, Strided<T>{A, sA}, lda, Strided<T>{B, sB}, ldb, batch,
                     info);
}

template <typename T>
static int posv_array(KBlasHandle *h, char side, char uplo, int m, int n, T **A, int lda, T **B,
                      int ldb, int batch, int *info) {
  int st = check_potrs(h, side, uplo, m, n, A, lda, B, ldb, batch);
  if (st != KBLAS_Success) return st;
  const int nrhs = is_left(side) ? n : m;
  return posv_any<T>(h, side, uplo, m, n, PtrArr<T>{A}, lda, PtrArr<T>{nrhs ? B : nullptr}, ldb,
                     batch, info);
}

}  // namespace kgb

using namespace kgb;

extern "C" {

int kblasSpotrf_batch(kblasHandle_t h, char uplo, const int n, float **A, int lda, int batchCount,
                      int *info) {
  return potrf_array<float>(h, uplo, n, A, lda, batchCount, info);
}
int kblasDpotrf_batch(kblasHandle_t h, char uplo, const int n, double **A, int lda, int batchCount,
                      int *info) {
  return potrf_array<double>(h, uplo, n, A, lda, batchCount, info);
}
int kblasSpotrf_batch_strided(kblasHandle_t h, char uplo, const int n, float *A, int lda,
                              long strideA, int batchCount, int *info) {
  return potrf_strided<float>(h, uplo, n, A, lda, strideA, batchCount, info);
}
int kblasDpotrf_batch_strided(kblasHandle_t h, char uplo, const int n, double *A, int lda,
                              long strideA, int batchCount, int *info) {
  return potrf_strided<double>(h, uplo, n, A, lda, strideA, batchCount, info);
}

int kblasSpotrs_batch(kblasHandle_t h, char side, char uplo, const int m, const int n,
                      const float **A, int lda, float **B, int ldb, int batchCount) {
  return potrs_array<float>(h, side, uplo, m, n, A, lda, B, ldb, batchCount);
}
int kblasDpotrs_batch(kblasHandle_t h, char side, char uplo, const int m, const int n,
                      const double **A, int lda, double **B, int ldb, int batchCount) {
  return potrs_array<double>(h, side, uplo, m, n, A, lda, B, ldb, batchCount);
}
int kblasSpotrs_batch_strided(kblasHandle_t h, char side, char uplo, const int m, const int n,
                              const float *A, int lda, long strideA, float *B, int ldb,
                              long strideB, int batchCount) {
  return potrs_strided<float>(h, side, uplo, m, n, A, lda, strideA, B, ldb, strideB, batchCount);
}
int kblasDpotrs_batch_strided(kblasHandle_t h, char side, char uplo, const int m, const int n,
                              const double *A, int lda, long strideA, double *B, int ldb,
                              long strideB, int batchCount) {
  return potrs_strided<double>(h, side, uplo, m, n, A, lda, strideA, B, ldb, strideB, batchCount);
}

int kblasSposv_batch(kblasHandle_t h, char side, char uplo, const int m, const int n, float **A,
                     int lda, float **B, int ldb, int batchCount, int *info) {
  return posv_array<float>(h, side, uplo, m, n, A, lda, B, ldb, batchCount, info);
}
int kblasDposv_batch(kblasHandle_t h, char side, char uplo, const int m, const int n, double **A,
                     int lda, double **B, int ldb, int batchCount, int *info) {
  return posv_array<double>(h, side, uplo, m, n, A, lda, B, ldb, batchCount, info);
}
int kblasSposv_batch_strided(kblasHandle_t h, char side, char uplo, const int m, const int n,
                             float *A, int lda, long strideA, float *B, int ldb, long strideB,
                             int batchCount, int *info) {
  return posv_strided<float>(h, side, uplo, m, n, A, lda, strideA, B, ldb, strideB, batchCount,
                             info);
}
int kblasDposv_batch_strided(kblasHandle_t h, char side, char uplo, const int m, const int n,
                             double *A, int lda, long strideA, double *B, int ldb, long strideB,
                             int batchCount, int *info) {
  return posv_strided<double>(h, side, uplo, m, n, A, lda, strideA, B, ldb, strideB, batchCount,
                              info);
}

// Complex precisions (the reference's kblas{C,Z}{potrf,potrs,posv}_batch[_strided],
// complex-symmetric: A = L L^T, nothing conjugated).
#define KGB_CHOL_CPLX(X, API, T)                                                                  \
  int kblas##X##potrf_batch(kblasHandle_t h, char uplo, const int n, API **A, int lda,            \
                            int batchCount, int *info) {                                          \
    return potrf_array<T>(h, uplo, n, reinterpret_cast<T **>(A), lda, batchCount, info);          \
  }                                                                                               \
  int kblas##X##potrf_batch_strided(kblasHandle_t h, char uplo, const int n, API *A, int lda,     \
                                    long strideA, int batchCount, int *info) {                    \
    return potrf_strided<T>(h, uplo, n, reinterpret_cast<T *>(A), lda, strideA, batchCount, info); \
  }                                                                                               \
  int kblas##X##potrs_batch(kblasHandle_t h, char side, char uplo, const int m, const int n,      \
                            const API **A, int lda, API **B, int ldb, int batchCount) {           \
    return potrs_array<T>(h, side, uplo, m, n, reinterpret_cast<const T **>(A), lda,              \
                          reinterpret_cast<T **>(B), ldb, batchCount);                            \
  }                                                                                               \
  int kblas##X##potrs_batch_strided(kblasHandle_t h, char side, char uplo, const int m,           \
                                    const int n, const API *A, int lda, long strideA, API *B,     \
                                    int ldb, long strideB, int batchCount) {                      \
    return potrs_strided<T>(h, side, uplo, m, n, reinterpret_cast<const T *>(A), lda, strideA,    \
                            reinterpret_cast<T *>(B), ldb, strideB, batchCount);                  \
  }                                                                                               \
  int kblas##X##posv_batch(kblasHandle_t h, char side, char uplo, const int m, const int n,       \
                           API **A, int lda, API **B, int ldb, int batchCount, int *info) {       \
    return posv_array<T>(h, side, uplo, m, n, reinterpret_cast<T **>(A), lda,                     \
                         reinterpret_cast<T **>(B), ldb, batchCount, info);                       \
  }                                                                                               \
  int kblas##X##posv_batch_strided(kblasHandle_t h, char side, char uplo, const int m,            \
                                   const int n, API *A, int lda, long strideA, API *B, int ldb,   \
                                   long strideB, int batchCount, int *info) {                     \
    return posv_strided<T>(h, side, uplo, m, n, reinterpret_cast<T *>(A), lda, strideA,           \
                           reinterpret_cast<T *>(B), ldb, strideB, batchCount, info);             \
  }

KGB_CHOL_CPLX(C, cuFloatComplex, cxf)
KGB_CHOL_CPLX(Z, cuDoubleComplex, cxd)
#undef KGB_CHOL_CPLX

}  // extern "C"

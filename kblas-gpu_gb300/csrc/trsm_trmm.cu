// trsm_trmm.cu -- batched TRSM and TRMM, single and double precision,
// strided and pointer-array forms, every side / uplo / trans / diag.
//
// Entry points replace reference src/batch_triangular/Xtrsm_batch.cu:97-262
// and Xtrmm_batch.cu:141-277. The reference implements Lower/NonUnit only
// (Xtrsm_batch_drivers.cuh:64-67) and sends Right/Upper/Unit TRMM to MAGMA
// (Xtrmm_batch.cu:63-106); here every combination runs natively.
//
// Design: every case is reduced to one lower-triangular kernel acting on
// independent vectors. Side 'L' acts on the n columns of B, side 'R' on the
// m rows of B (X*op(A) = B  <=>  op(A)^T x^T = b^T). The effective matrix
// M = op(A) (side L) or op(A)^T (side R) is upper or lower; an upper M is
// turned into a lower one by reversing the index order of both M and the
// vector while staging. One thread owns one vector (its K elements live in
// shared memory), so every FMA of every lane is useful work -- on GB300 the
// FP64 pipe is the bottleneck, and this layout issues no wasted FP64
// instruction. The triangle is staged once per CTA in packed row-major form
// (broadcast reads) when it fits, else read through L1 from global memory.
#include <stdio.h>

#include "device_util.cuh"
#include "kblas_internal.h"
#include "launch_util.h"

namespace kgb {

struct TriDesc {
  int K;          // order of the triangle
  int V;          // number of vectors per matrix
  int vstride;    // distance between consecutive vectors in B
  int estride;    // distance between consecutive elements of one vector
  int mtrans;     // M(i,k) = A(k,i) if set, else A(i,k)
  int rev;        // M is upper: reverse indices so it becomes lower
  int unit;       // unit diagonal
  int staged;     // triangle staged in shared memory
  int ldx;        // shared-memory stride between vectors
  int VC;         // vectors per CTA
  int nchunks;    // ceil(V / VC)
};

// op = 0: TRSM (x := M^{-1} * alpha * x),  op = 1: TRMM (x := alpha * M * x)
template <typename T, int OP, class AccA, class AccB>
__global__ void tri_vec_kernel(TriDesc d, T alpha, AccA A, int lda, AccB B, long long batch)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int K = d.K;
  const long long mat = blockIdx.x / d.nchunks;
  const int chunk = blockIdx.x - (int)(mat * d.nchunks);
  if (mat >= batch) return;
  const int v0 = chunk * d.VC;
  const int vc = min(d.VC, d.V - v0);
  const int tid = threadIdx.x, NT = blockDim.x;

  T *sX = reinterpret_cast<T *>(smem_raw);       // VC x ldx
  T *sD = sX + (size_t)d.VC * d.ldx;             // K diagonal entries (or reciprocals)
  T *sM = sD + K;                                // packed row-major lower triangle
  const T *Ag = A.get(mat);
  T *Bg = B.get(mat);

  auto Mval = [&](int i, int k) -> T {  // lower-normalised M(i,k), i >= k
    int a = d.rev ? K - 1 - i : i, c = d.rev ? K - 1 - k : k;
    return d.mtrans ? Ag[(size_t)c + (size_t)a * lda] : Ag[(size_t)a + (size_t)c * lda];
  };

  if (alpha == T(0)) {  // BLAS: B := 0 without reading A
    for (int idx = tid; idx < vc * K; idx += NT) {
      int v, e;
      if (d.vstride == 1) { v = idx % vc; e = idx / vc; } else { e = idx % K; v = idx / K; }
      Bg[(size_t)(v0 + v) * d.vstride + (size_t)e * d.estride] = T(0);
    }
    return;
  }

  // stage the vectors (coalesced along whichever index is contiguous in B)
  for (int idx = tid; idx < vc * K; idx += NT) {
    int v, e;
    if (d.vstride == 1) { v = idx % vc; e = idx / vc; } else { e = idx % K; v = idx / K; }
    const int i = d.rev ? K - 1 - e : e;
    T x = Bg[(size_t)(v0 + v) * d.vstride + (size_t)e * d.estride];
    sX[(size_t)v * d.ldx + i] = (OP == 0) ? alpha * x : x;
  }
  for (int i = tid; i < K; i += NT) {
    T dg = d.unit ? T(1) : Mval(i, i);
    sD[i] = (OP == 0) ? T(1) / dg : dg;
  }
  if (d.staged)
    for (int i = tid; i < K; i += NT) {
      T *row = sM + ((size_t)i * (i + 1) >> 1);
      for (int k = 0; k < i; k++) row[k] = Mval(i, k);
    }
  __syncthreads();

  if (tid < vc) {
    T *x = sX + (size_t)tid * d.ldx;
    if (OP == 0) {
      for (int i = 0; i < K; i++) {
        T s0 = x[i], s1 = T(0), s2 = T(0), s3 = T(0);
        int k = 0;
        if (d.staged) {
          const T *row = sM + ((size_t)i * (i + 1) >> 1);
          for (; k + 3 < i; k += 4) {
            s0 -= row[k] * x[k];
            s1 -= row[k + 1] * x[k + 1];
            s2 -= row[k + 2] * x[k + 2];
            s3 -= row[k + 3] * x[k + 3];
          }
          for (; k < i; k++) s0 -= row[k] * x[k];
        } else {
          for (; k < i; k++) s0 -= Mval(i, k) * x[k];
        }
        x[i] = ((s0 + s1) + (s2 + s3)) * sD[i];
      }
    } else {
      for (int i = K - 1; i >= 0; i--) {
        T s0 = sD[i] * x[i], s1 = T(0), s2 = T(0), s3 = T(0);
        int k = 0;
        if (d.staged) {
          const T *row = sM + ((size_t)i * (i + 1) >> 1);
          for (; k + 3 < i; k += 4) {
            s0 += row[k] * x[k];
            s1 += row[k + 1] * x[k + 1];
            s2 += row[k + 2] * x[k + 2];
            s3 += row[k + 3] * x[k + 3];
          }
          for (; k < i; k++) s0 += row[k] * x[k];
        } else {
          for (; k < i; k++) s0 += Mval(i, k) * x[k];
        }
        x[i] = alpha * ((s0 + s1) + (s2 + s3));
      }
    }
  }
  __syncthreads();
  for (int idx = tid; idx < vc * K; idx += NT) {
    int v, e;
    if (d.vstride == 1) { v = idx % vc; e = idx / vc; } else { e = idx % K; v = idx / K; }
    const int i = d.rev ? K - 1 - e : e;
    Bg[(size_t)(v0 + v) * d.vstride + (size_t)e * d.estride] = sX[(size_t)v * d.ldx + i];
  }
}

template <typename T, int OP, class AccA, class AccB>
static int launch_tri(KBlasHandle *h, char side, char uplo, char trans, char diag, int m, int n,
                      T alpha, AccA A, int lda, AccB B, int ldb, long long batch) {
  TriDesc d;
  const bool left = is_left(side);
  d.K = left ? m : n;
  d.V = left ? n : m;
  d.vstride = left ? ldb : 1;
  d.estride = left ? 1 : ldb;
  const bool tr = is_trans(trans);
  d.mtrans = left ? tr : !tr;
  const bool lower = is_lower(uplo);
  const bool mlower = lower != (bool)d.mtrans;
  d.rev = !mlower;
  d.unit = is_unit(diag);
  d.ldx = d.K | 1;
  const int limit = max_smem(h);
  const size_t tri_bytes = (size_t)d.K * (d.K + 1) / 2 * sizeof(T);
  d.staged = tri_bytes <= 64 * 1024;
  int VC = d.V < 64 ? d.V : 64;
  auto bytes = [&](int vc, bool st) {
    return ((size_t)vc * d.ldx + d.K) * sizeof(T) + (st ? tri_bytes : 0);
  };
  while (VC > 8 && bytes(VC, d.staged) > (size_t)limit / 2) VC /= 2;
  if (bytes(VC, d.staged) > (size_t)limit) d.staged = 0;
  while (VC > 1 && bytes(VC, d.staged) > (size_t)limit) VC /= 2;
  if (bytes(VC, d.staged) > (size_t)limit) {
    fprintf(stderr, "KBLAS: batched TRSM/TRMM with a triangle of order %d exceeds on-chip limits\n", d.K);
    return KBLAS_NotSupported;
  }
  d.VC = VC;
  d.nchunks = (d.V + VC - 1) / VC;
  const size_t smem = bytes(VC, d.staged);
  const int NT = VC < 32 ? 32 : VC;
  auto kern = tri_vec_kernel<T, OP, AccA, AccB>;
  int st = set_smem(kern, smem);
  if (st != KBLAS_Success) return st;
  const long long grid = batch * d.nchunks;
  if (grid > 0x7fffffffLL) return KBLAS_NotSupported;
  kern<<<(unsigned)grid, NT, smem, h->stream>>>(d, alpha, A, lda, B, batch);
  KGB_LAUNCH_CHECK(OP == 0 ? "trsm kernel" : "trmm kernel");
  return KBLAS_Success;
}

static inline int check_tri(KBlasHandle *h, char side, char uplo, char trans, char diag, int m,
                            int n, int lda, int ldb, int batch) {
  if (!h) return KBLAS_Error_NotInitialized;
  if (!(is_left(side) || is_right(side)) || !(is_lower(uplo) || is_upper(uplo)) ||
      !(is_trans(trans) || is_notrans(trans)) || !(is_unit(diag) || is_nonunit(diag)))
    return KBLAS_Error_WrongInput;
  const int ka = is_left(side) ? m : n;
  if (m < 0 || n < 0 || batch < 0 || lda < (ka > 1 ? ka : 1) || ldb < (m > 1 ? m : 1))
    return KBLAS_Error_WrongInput;
  return KBLAS_Success;
}

template <typename T, int OP>
static int tri_strided(KBlasHandle *h, char side, char uplo, char trans, char diag, int m, int n,
                       T alpha, const T *A, int lda, long long sA, T *B, int ldb, long long sB,
                       int batch) {
  int st = check_tri(h, side, uplo, trans, diag, m, n, lda, ldb, batch);
  if (st != KBLAS_Success) return st;
  if (m == 0 || n == 0 || batch == 0) return KBLAS_Success;
  if (!A || !B || (batch > 1 && sB < (long long)ldb * n) || sA < 0) return KBLAS_Error_WrongInput;
  return launch_tri<T, OP>(h, side, uplo, trans, diag, m, n, alpha, Strided<T>{const_cast<T *>(A), sA},
                           lda, Strided<T>{B, sB}, ldb, batch);
}

template <typename T, int OP>
static int tri_array(KBlasHandle *h, char side, char uplo, char trans, char diag, int m, int n,
                     T alpha, const T **A, int lda, T **B, int ldb, int batch) {
  int st = check_tri(h, side, uplo, trans, diag, m, n, lda, ldb, batch);
  if (st != KBLAS_Success) return st;
  if (m == 0 || n == 0 || batch == 0) return KBLAS_Success;
  if (!A || !B) return KBLAS_Error_WrongInput;
  return launch_tri<T, OP>(h, side, uplo, trans, diag, m, n, alpha, PtrArr<T>{const_cast<T **>(A)},
                           lda, PtrArr<T>{B}, ldb, batch);
}

}  // namespace kgb

using namespace kgb;

extern "C" {

int kblasStrsm_batch(kblasHandle_t h, char side, char uplo, char trans, char diag, const int m,
                     const int n, const float alpha, const float **A, int lda, float **B, int ldb,
                     int batchCount) {
  return tri_array<float, 0>(h, side, uplo, trans, diag, m, n, alpha, A, lda, B, ldb, batchCount);
}
int kblasDtrsm_batch(kblasHandle_t h, char side, char uplo, char trans, char diag, const int m,
                     const int n, const double alpha, const double **A, int lda, double **B,
                     int ldb, int batchCount) {
  return tri_array<double, 0>(h, side, uplo, trans, diag, m, n, alpha, A, lda, B, ldb, batchCount);
}
int kblasStrsm_batch_strided(kblasHandle_t h, char side, char uplo, char trans, char diag,
                             const int m, const int n, const float alpha, const float *A, int lda,
                             long strideA, float *B, int ldb, long strideB, int batchCount) {
  return tri_strided<float, 0>(h, side, uplo, trans, diag, m, n, alpha, A, lda, strideA, B, ldb,
                               strideB, batchCount);
}
int kblasDtrsm_batch_strided(kblasHandle_t h, char side, char uplo, char trans, char diag,
                             const int m, const int n, const double alpha, const double *A,
                             int lda, long strideA, double *B, int ldb, long strideB,
                             int batchCount) {
  return tri_strided<double, 0>(h, side, uplo, trans, diag, m, n, alpha, A, lda, strideA, B, ldb,
                                strideB, batchCount);
}

int kblasStrmm_batch(kblasHandle_t h, char side, char uplo, char trans, char diag, const int m,
                     const int n, const float alpha, const float **A, int lda, float **B, int ldb,
                     int batchCount) {
  return tri_array<float, 1>(h, side, uplo, trans, diag, m, n, alpha, A, lda, B, ldb, batchCount);
}
int kblasDtrmm_batch(kblasHandle_t h, char side, char uplo, char trans, char diag, const int m,
                     const int n, const double alpha, const double **A, int lda, double **B,
                     int ldb, int batchCount) {
  return tri_array<double, 1>(h, side, uplo, trans, diag, m, n, alpha, A, lda, B, ldb, batchCount);
}
int kblasStrmm_batch_strided(kblasHandle_t h, char side, char uplo, char trans, char diag,
                             const int m, const int n, const float alpha, const float *A, int lda,
                             long strideA, float *B, int ldb, long strideB, int batchCount) {
  return tri_strided<float, 1>(h, side, uplo, trans, diag, m, n, alpha, A, lda, strideA, B, ldb,
                               strideB, batchCount);
}
int kblasDtrmm_batch_strided(kblasHandle_t h, char side, char uplo, char trans, char diag,
                             const int m, const int n, const double alpha, const double *A,
                             int lda, long strideA, double *B, int ldb, long strideB,
                             int batchCount) {
  return tri_strided<double, 1>(h, side, uplo, trans, diag, m, n, alpha, A, lda, strideA, B, ldb,
                                strideB, batchCount);
}

}  // extern "C"

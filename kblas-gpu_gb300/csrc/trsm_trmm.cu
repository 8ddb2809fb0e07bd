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
//
// The same kernel serves the variable-size TRSM (kblas{S,D}trsm_vbatch, the
// reference's non-uniform kblas_trsm_batch overload, MAGMA-only there):
// per-matrix m, n, lda, ldb come from device arrays and the shared-memory
// layout is sized for the largest triangle.
#include <stdio.h>

#include <cuComplex.h>

#include "device_util.cuh"
#include "kblas_internal.h"
#include "launch_util.h"
#include "tri_internal.h"

namespace kgb {

struct TriDesc {
  int left;       // side L: the triangle is m x m and acts on the n columns of B
  int mtrans;     // M(i,k) = A(k,i) if set, else A(i,k)
  int rev;        // M is upper: reverse indices so it becomes lower
  int unit;       // unit diagonal
  int staged;     // triangle staged in shared memory
  int Kmax;       // largest triangle order the shared-memory layout holds
  int ldx;        // shared-memory stride between vectors (Kmax | 1)
  int VC;         // vectors per chunk
  const int *skip;  // device int[batch] or null: matrices with a non-zero entry are left as is
};

// op = 0: TRSM (x := M^{-1} * alpha * x),  op = 1: TRMM (x := alpha * M * x).
// dims = (m, n, lda, ldb) of each matrix. The CTA at (b, y) stages the
// triangle of matrix b once and then takes vector chunks y, y + gridDim.y, ...
template <typename T, int OP, class AccA, class AccB, class Dims>
__global__ void tri_vec_kernel(TriDesc d, T alpha, AccA A, AccB B, Dims dims, long long batch)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const long long mat = blockIdx.x;
  if (mat >= batch) return;
  int dd[4];
  dims.get(mat, dd);
  const int K = d.left ? dd[0] : dd[1], V = d.left ? dd[1] : dd[0];
  const int lda = dd[2], ldb = dd[3];
  if (K <= 0 || V <= 0 || K > d.Kmax) return;
  if (d.skip && d.skip[mat] != 0) return;
  const int vstride = d.left ? ldb : 1, estride = d.left ? 1 : ldb;
  const int nchunks = (V + d.VC - 1) / d.VC;
  if ((int)blockIdx.y >= nchunks) return;
  const int tid = threadIdx.x, NT = blockDim.x;

  T *sX = reinterpret_cast<T *>(smem_raw);       // VC x ldx
  T *sD = sX + (size_t)d.VC * d.ldx;             // K diagonal entries (or reciprocals)
  T *sM = sD + d.Kmax;                           // packed row-major lower triangle
  const T *Ag = A.get(mat);
  T *Bg = B.get(mat);

  auto Mval = [&](int i, int k) -> T {  // lower-normalised M(i,k), i >= k
    int a = d.rev ? K - 1 - i : i, c = d.rev ? K - 1 - k : k;
    return d.mtrans ? Ag[(size_t)c + (size_t)a * lda] : Ag[(size_t)a + (size_t)c * lda];
  };
  // element e of vector v of the chunk at v0, in B
  auto bidx = [&](int v0, int v, int e) -> size_t {
    return (size_t)(v0 + v) * vstride + (size_t)e * estride;
  };

  if (alpha == T(0)) {  // BLAS: B := 0 without reading A
    for (int c = blockIdx.y; c < nchunks; c += gridDim.y) {
      const int v0 = c * d.VC, vc = min(d.VC, V - v0);
      for (int idx = tid; idx < vc * K; idx += NT) {
        int v, e;
        if (vstride == 1) { v = idx % vc; e = idx / vc; } else { e = idx % K; v = idx / K; }
        Bg[bidx(v0, v, e)] = T(0);
      }
    }
    return;
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

  for (int c = blockIdx.y; c < nchunks; c += gridDim.y) {
    const int v0 = c * d.VC, vc = min(d.VC, V - v0);
    // stage the vectors (coalesced along whichever index is contiguous in B)
    for (int idx = tid; idx < vc * K; idx += NT) {
      int v, e;
      if (vstride == 1) { v = idx % vc; e = idx / vc; } else { e = idx % K; v = idx / K; }
      const int i = d.rev ? K - 1 - e : e;
      T x = Bg[bidx(v0, v, e)];
      sX[(size_t)v * d.ldx + i] = (OP == 0) ? alpha * x : x;
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
      if (vstride == 1) { v = idx % vc; e = idx / vc; } else { e = idx % K; v = idx / K; }
      const int i = d.rev ? K - 1 - e : e;
      Bg[bidx(v0, v, e)] = sX[(size_t)v * d.ldx + i];
    }
    __syncthreads();
  }
}

// Host-side plan shared by the uniform and variable-size launches: flags
// from side/uplo/trans/diag, the shared-memory layout from the largest
// triangle order Kmax and the largest vector count Vmax.
template <typename T>
static int plan_tri(KBlasHandle *h, char side, char uplo, char trans, char diag, int Kmax,
                    int Vmax, TriDesc &d, size_t &smem) {
  d.left = is_left(side);
  d.skip = nullptr;
  const bool tr = is_trans(trans);
  d.mtrans = d.left ? tr : !tr;
  const bool lower = is_lower(uplo);
  const bool mlower = lower != (bool)d.mtrans;
  d.rev = !mlower;
  d.unit = is_unit(diag);
  d.Kmax = Kmax;
  d.ldx = Kmax | 1;
  const int limit = max_smem(h);
  const size_t tri_bytes = (size_t)Kmax * (Kmax + 1) / 2 * sizeof(T);
  d.staged = tri_bytes <= 64 * 1024;
  int VC = Vmax < 64 ? Vmax : 64;
  if (VC < 1) VC = 1;
  auto bytes = [&](int vc, bool st) {
    return ((size_t)vc * d.ldx + Kmax) * sizeof(T) + (st ? tri_bytes : 0);
  };
  while (VC > 8 && bytes(VC, d.staged) > (size_t)limit / 2) VC /= 2;
  if (bytes(VC, d.staged) > (size_t)limit) d.staged = 0;
  while (VC > 1 && bytes(VC, d.staged) > (size_t)limit) VC /= 2;
  if (bytes(VC, d.staged) > (size_t)limit) {
    fprintf(stderr, "KBLAS: batched TRSM/TRMM with a triangle of order %d exceeds on-chip limits\n", Kmax);
    return KBLAS_NotSupported;
  }
  d.VC = VC;
  smem = bytes(VC, d.staged);
  return KBLAS_Success;
}

// Chunk slots per matrix: fill the GPU several times over when the batch
// alone does not, never more than the largest matrix has chunks.
static unsigned chunk_slots(KBlasHandle *h, long long batch, long long chunks_max) {
  ensure_device_props(h);
  const long long target = (long long)(h->sm_count > 0 ? h->sm_count : 152) * 16;
  long long y = (target + batch - 1) / batch;
  if (y > chunks_max) y = chunks_max;
  if (y < 1) y = 1;
  if (y > 65535) y = 65535;
  return (unsigned)y;
}

template <typename T, int OP, class AccA, class AccB, class Dims>
static int launch_tri_plan(KBlasHandle *h, const TriDesc &d, size_t smem, int Vmax, T alpha,
                           AccA A, AccB B, Dims dims, long long batch) {
  auto kern = tri_vec_kernel<T, OP, AccA, AccB, Dims>;
  int st = set_smem(kern, smem);
  if (st != KBLAS_Success) return st;
  if (batch > 0x7fffffffLL) return KBLAS_NotSupported;
  const int NT = d.VC < 32 ? 32 : d.VC;
  dim3 grid((unsigned)batch, chunk_slots(h, batch, (Vmax + d.VC - 1) / d.VC));
  kern<<<grid, NT, smem, h->stream>>>(d, alpha, A, B, dims, batch);
  KGB_LAUNCH_CHECK(OP == 0 ? "trsm kernel" : "trmm kernel");
  return KBLAS_Success;
}

template <typename T, int OP, class AccA, class AccB>
static int launch_tri(KBlasHandle *h, char side, char uplo, char trans, char diag, int m, int n,
                      T alpha, AccA A, int lda, AccB B, int ldb, long long batch,
                      const int *skip = nullptr) {
  const bool left = is_left(side);
  const int K = left ? m : n, V = left ? n : m;
  TriDesc d;
  size_t smem = 0;
  int st = plan_tri<T>(h, side, uplo, trans, diag, K, V, d, smem);
  if (st != KBLAS_Success) return st;
  d.skip = skip;
  return launch_tri_plan<T, OP>(h, d, smem, V, alpha, A, B, DimsU<4>{{m, n, lda, ldb}}, batch);
}

template <typename T, class AccA, class AccB>
int trsm_batch_internal(KBlasHandle *h, char side, char uplo, char trans, char diag, int m, int n,
                        T alpha, AccA A, int lda, AccB B, int ldb, long long batch,
                        const int *skip) {
  if (m <= 0 || n <= 0 || batch <= 0) return KBLAS_Success;
  return launch_tri<T, 0>(h, side, uplo, trans, diag, m, n, alpha, A, lda, B, ldb, batch, skip);
}
template int trsm_batch_internal<float, Strided<float>, Strided<float>>(
    KBlasHandle *, char, char, char, char, int, int, float, Strided<float>, int, Strided<float>, int,
    long long, const int *);
template int trsm_batch_internal<double, Strided<double>, Strided<double>>(
    KBlasHandle *, char, char, char, char, int, int, double, Strided<double>, int, Strided<double>,
    int, long long, const int *);
template int trsm_batch_internal<float, PtrArr<float>, PtrArr<float>>(
    KBlasHandle *, char, char, char, char, int, int, float, PtrArr<float>, int, PtrArr<float>, int,
    long long, const int *);
template int trsm_batch_internal<double, PtrArr<double>, PtrArr<double>>(
    KBlasHandle *, char, char, char, char, int, int, double, PtrArr<double>, int, PtrArr<double>,
    int, long long, const int *);
template int trsm_batch_internal<cxf, Strided<cxf>, Strided<cxf>>(
    KBlasHandle *, char, char, char, char, int, int, cxf, Strided<cxf>, int, Strided<cxf>, int,
    long long, const int *);
template int trsm_batch_internal<cxd, Strided<cxd>, Strided<cxd>>(
    KBlasHandle *, char, char, char, char, int, int, cxd, Strided<cxd>, int, Strided<cxd>, int,
    long long, const int *);
template int trsm_batch_internal<cxf, PtrArr<cxf>, PtrArr<cxf>>(
    KBlasHandle *, char, char, char, char, int, int, cxf, PtrArr<cxf>, int, PtrArr<cxf>, int,
    long long, const int *);
template int trsm_batch_internal<cxd, PtrArr<cxd>, PtrArr<cxd>>(
    KBlasHandle *, char, char, char, char, int, int, cxd, PtrArr<cxd>, int, PtrArr<cxd>, int,
    long long, const int *);

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

// Largest m and n of a variable-size batch (values <= 0 count as 0), into
// out[0], out[1] (zeroed by the caller).
__global__ void imax2_kernel(const int *m, const int *n, long long batch, int *out) {
  int mm = 0, nn = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < batch;
       i += (long long)gridDim.x * blockDim.x) {
    mm = max(mm, m[i]);
    nn = max(nn, n[i]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    mm = max(mm, __shfl_xor_sync(0xffffffffu, mm, o));
    nn = max(nn, __shfl_xor_sync(0xffffffffu, nn, o));
  }
  if ((threadIdx.x & 31) == 0) {
    if (mm > 0) atomicMax(out, mm);
    if (nn > 0) atomicMax(out + 1, nn);
  }
}

// Variable-size TRSM, reference Xtrsm_batch_drivers.cuh:278-340 (MAGMA
// vbatched there): max_m / max_n bound the sizes; when both are <= 0 they
// are recomputed on the device into the workspace that
// kblas_trsm_batch_nonuniform_wsquery requests, and read back with a stream
// synchronisation, as the reference does. A matrix whose triangle is larger
// than the bound is skipped (the reference's MAGMA _nocheck path leaves
// that case undefined).
template <typename T>
static int trsm_vbatch(KBlasHandle *h, char side, char uplo, char trans, char diag, const int *m,
                       const int *n, int max_m, int max_n, T alpha, const T **A, const int *lda,
                       T **B, const int *ldb, int batch) {
  if (!h) return KBLAS_Error_NotInitialized;
  if (!(is_left(side) || is_right(side)) || !(is_lower(uplo) || is_upper(uplo)) ||
      !(is_trans(trans) || is_notrans(trans)) || !(is_unit(diag) || is_nonunit(diag)) || batch < 0)
    return KBLAS_Error_WrongInput;
  if (batch == 0) return KBLAS_Success;
  if (!m || !n || !lda || !ldb || !A || !B) return KBLAS_Error_WrongInput;
  if (max_m <= 0 && max_n <= 0) {
    if (!h->ws.d_data || h->ws.allocated.d_data_bytes < 2 * sizeof(int))
      return KBLAS_InsufficientWorkspace;
    int *dmax = static_cast<int *>(h->ws.d_data);
    int hmax[2] = {0, 0};
    cudaError_t e = cudaMemsetAsync(dmax, 0, 2 * sizeof(int), h->stream);
    if (e != cudaSuccess) return cuda_check(e, "cudaMemsetAsync", __FILE__, __LINE__);
    ensure_device_props(h);
    const long long blocks = (batch + 255) / 256;
    const int grid = (int)(blocks < (long long)h->sm_count * 4 ? blocks : (long long)h->sm_count * 4);
    imax2_kernel<<<grid > 0 ? grid : 1, 256, 0, h->stream>>>(m, n, batch, dmax);
    KGB_LAUNCH_CHECK("imax2_kernel");
    e = cudaMemcpyAsync(hmax, dmax, 2 * sizeof(int), cudaMemcpyDeviceToHost, h->stream);
    if (e != cudaSuccess) return cuda_check(e, "cudaMemcpyAsync", __FILE__, __LINE__);
    e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_check(e, "cudaStreamSynchronize", __FILE__, __LINE__);
    max_m = hmax[0];
    max_n = hmax[1];
  }
  if (max_m <= 0 || max_n <= 0) return KBLAS_Success;
  const bool left = is_left(side);
  const int K = left ? max_m : max_n, V = left ? max_n : max_m;
  TriDesc d;
  size_t smem = 0;
  int st = plan_tri<T>(h, side, uplo, trans, diag, K, V, d, smem);
  if (st != KBLAS_Success) return st;
  return launch_tri_plan<T, 0>(h, d, smem, V, alpha, PtrArr<T>{const_cast<T **>(A)},
                               PtrArr<T>{B}, DimsV<4>{{m, n, lda, ldb}}, batch);
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

int kblasStrsm_vbatch(kblasHandle_t h, char side, char uplo, char trans, char diag, int *m, int *n,
                      int max_m, int max_n, const float alpha, const float **A, int *lda,
                      float **B, int *ldb, int batchCount) {
  return trsm_vbatch<float>(h, side, uplo, trans, diag, m, n, max_m, max_n, alpha, A, lda, B, ldb,
                            batchCount);
}
int kblasDtrsm_vbatch(kblasHandle_t h, char side, char uplo, char trans, char diag, int *m, int *n,
                      int max_m, int max_n, const double alpha, const double **A, int *lda,
                      double **B, int *ldb, int batchCount) {
  return trsm_vbatch<double>(h, side, uplo, trans, diag, m, n, max_m, max_n, alpha, A, lda, B,
                             ldb, batchCount);
}

// Complex precisions (op = transpose, never conjugate-transpose, as the
// reference's KBLAS_Trans; every side / uplo / trans / diag).
#define KGB_TRI_CPLX(X, API, T)                                                                    \
  int kblas##X##trsm_batch(kblasHandle_t h, char side, char uplo, char trans, char diag,           \
                           const int m, const int n, const API alpha, const API **A, int lda,      \
                           API **B, int ldb, int batchCount) {                                     \
    return tri_array<T, 0>(h, side, uplo, trans, diag, m, n, T(alpha.x, alpha.y),                  \
                           reinterpret_cast<const T **>(A), lda, reinterpret_cast<T **>(B), ldb,   \
                           batchCount);                                                            \
  }                                                                                                \
  int kblas##X##trsm_batch_strided(kblasHandle_t h, char side, char uplo, char trans, char diag,   \
                                   const int m, const int n, const API alpha, const API *A,        \
                                   int lda, long strideA, API *B, int ldb, long strideB,           \
                                   int batchCount) {                                               \
    return tri_strided<T, 0>(h, side, uplo, trans, diag, m, n, T(alpha.x, alpha.y),                \
                             reinterpret_cast<const T *>(A), lda, strideA,                         \
                             reinterpret_cast<T *>(B), ldb, strideB, batchCount);                  \
  }                                                                                                \
  int kblas##X##trmm_batch(kblasHandle_t h, char side, char uplo, char trans, char diag,           \
                           const int m, const int n, const API alpha, const API **A, int lda,      \
                           API **B, int ldb, int batchCount) {                                     \
    return tri_array<T, 1>(h, side, uplo, trans, diag, m, n, T(alpha.x, alpha.y),                  \
                           reinterpret_cast<const T **>(A), lda, reinterpret_cast<T **>(B), ldb,   \
                           batchCount);                                                            \
  }                                                                                                \
  int kblas##X##trmm_batch_strided(kblasHandle_t h, char side, char uplo, char trans, char diag,   \
                                   const int m, const int n, const API alpha, const API *A,        \
                                   int lda, long strideA, API *B, int ldb, long strideB,           \
                                   int batchCount) {                                               \
    return tri_strided<T, 1>(h, side, uplo, trans, diag, m, n, T(alpha.x, alpha.y),                \
                             reinterpret_cast<const T *>(A), lda, strideA,                         \
                             reinterpret_cast<T *>(B), ldb, strideB, batchCount);                  \
  }

#define KGB_TRSM_VB_CPLX(X, API, T)                                                                \
  int kblas##X##trsm_vbatch(kblasHandle_t h, char side, char uplo, char trans, char diag, int *m,  \
                            int *n, int max_m, int max_n, const API alpha, const API **A,          \
                            int *lda, API **B, int *ldb, int batchCount) {                         \
    return trsm_vbatch<T>(h, side, uplo, trans, diag, m, n, max_m, max_n, T(alpha.x, alpha.y),     \
                          reinterpret_cast<const T **>(A), lda, reinterpret_cast<T **>(B), ldb,    \
                          batchCount);                                                             \
  }
KGB_TRSM_VB_CPLX(C, cuFloatComplex, cxf)
KGB_TRSM_VB_CPLX(Z, cuDoubleComplex, cxd)
#undef KGB_TRSM_VB_CPLX

KGB_TRI_CPLX(C, cuFloatComplex, cxf)
KGB_TRI_CPLX(Z, cuDoubleComplex, cxd)
#undef KGB_TRI_CPLX

}  // extern "C"

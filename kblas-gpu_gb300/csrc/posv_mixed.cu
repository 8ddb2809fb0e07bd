// posv_mixed.cu -- mixed-precision batched DPOSV, uniform size (strided and
// pointer-array forms), and the tuning-table override used by the autotuner.
//
// No reference counterpart: KBLAS has only the plain FP64 POSV
// (src/batch_triangular/Xposv_batch.cu:92-178). The argument list follows
// kblasDposv_batch[_strided] plus an iteration/outcome array, the role of
// ITER in LAPACK DSPOSV. The work is one persistent launch (posv_core.cuh).
#include <stdio.h>

#include "posv_launch.h"
#include "workspace.h"

namespace kgb {

static_assert(PC_NCLS == KBLAS_POSV_TUNING_CLASSES, "size-class count of the tuning API");

TuneOverride &tune_override() {
  static TuneOverride o;
  return o;
}

size_t mixed_posv_ws_bytes(KBlasHandle *h, int n, long long batch) {
  if (batch <= 0 || n <= 0) return 0;
  PosvPlan pl;
  const int st = n > 32 ? plan_posv<true, 2>(h, n, pl) : plan_posv<true, 1>(h, n, pl);
  if (st != KBLAS_Success) return 0;
  return posv_ws_layout(n, batch, false, pl).total;
}

static int mixed_uniform(KBlasHandle *h, char side, char uplo, int m, int n, SysArgs sys, int batch,
                         int *info, int *iter) {
  if (!h) return KBLAS_Error_NotInitialized;
  if (is_left(side) || is_upper(uplo)) {
    printf("(Left | Upper) POSV_BATCH is not implemented yet\n");
    return KBLAS_NotImplemented;
  }
  if (!is_right(side) || !is_lower(uplo)) return KBLAS_Error_WrongInput;
  if (m < 0 || n < 0 || batch < 0 || sys.lda < (n > 1 ? n : 1) || sys.ldb < (m > 1 ? m : 1))
    return KBLAS_Error_WrongInput;
  if (batch == 0) return KBLAS_Success;
  if (n == 0) {
    int st = zero_info(h, info, batch);
    if (st == KBLAS_Success) st = zero_info(h, iter, batch);
    return st;
  }
  if (n > PC_MAX_N) return KBLAS_NotSupported;
  PosvPlan pl;
  int st = n > 32 ? plan_posv<true, 2>(h, n, pl) : plan_posv<true, 1>(h, n, pl);
  if (st != KBLAS_Success) return st;
  const PosvWs ws = posv_ws_layout(n, batch, false, pl);
  if (ws.total > h->ws.allocated.d_data_bytes || !h->ws.d_data) return KBLAS_InsufficientWorkspace;
  char *base = static_cast<char *>(h->ws.d_data);
  int *header = reinterpret_cast<int *>(base + ws.header);
  cudaError_t e = cudaMemsetAsync(header, 0, 64 * sizeof(int), h->stream);
  if (e != cudaSuccess) return cuda_check(e, "cudaMemsetAsync", __FILE__, __LINE__);
  ItemArgs it{};
  it.uniform = 1;
  it.batch = batch;
  it.n_uniform = n;
  it.queue = header;
  OutArgs out{info, iter, base + ws.scratch, (long long)pl.slot_bytes, pl.tc, h->d_status};
  sys.n = n;
  sys.m = m;
  if (n > 32 && pl.tc)
    posv_persistent_kernel<true, 6><<<pl.grid, PC_NT, pl.smem, h->stream>>>(sys, it, out, pl.cfg, pl.smem);
  else if (n > 32)
    posv_persistent_kernel<true, 2><<<pl.grid, PC_NT, pl.smem, h->stream>>>(sys, it, out, pl.cfg, pl.smem);
  else
    posv_persistent_kernel<true, 1><<<pl.grid, PC_NT, pl.smem, h->stream>>>(sys, it, out, pl.cfg, pl.smem);
  KGB_LAUNCH_CHECK("posv_persistent_kernel<mixed>");
  return KBLAS_Success;
}

// The launch behind the allocation-free entry point (posv_noalloc.cu): the
// checks and the kernel of mixed_uniform, on the caller's stream, with
// scratch the caller owns. scratch[0, 256) is the work counter, cleared here
// before the launch; the per-CTA slots follow it, and the grid is cut to the
// number of slots that fit in scratch_bytes. No memory is allocated.
int mixed_uniform_fixed_scratch(cudaStream_t stream, int device, int sm_count, int smem_optin,
                                char side, char uplo, int m, int n, double *A, int lda,
                                long long sA, double *B, int ldb, long long sB, int batch,
                                int *info, int *iter, char *scratch, size_t scratch_bytes) {
  if (is_left(side) || is_upper(uplo)) {
    printf("(Left | Upper) POSV_BATCH is not implemented yet\n");
    return KBLAS_NotImplemented;
  }
  if (!is_right(side) || !is_lower(uplo)) return KBLAS_Error_WrongInput;
  if (m < 0 || n < 0 || batch < 0 || lda < (n > 1 ? n : 1) || ldb < (m > 1 ? m : 1))
    return KBLAS_Error_WrongInput;
  if (batch > 1 && (sA < (long long)lda * n || (m > 0 && sB < (long long)ldb * n)))
    return KBLAS_Error_WrongInput;
  if (n > 0 && batch > 0 && (!A || (m > 0 && !B))) return KBLAS_Error_WrongInput;
  if (batch == 0) return KBLAS_Success;
  KBlasHandle hh;  // stand-in carrying the stream and device properties only
  hh.device_id = device;
  hh.stream = stream;
  hh.sm_count = sm_count;
  hh.max_smem_optin = smem_optin;
  if (n == 0) {
    int st = zero_info(&hh, info, batch);
    if (st == KBLAS_Success) st = zero_info(&hh, iter, batch);
    return st;
  }
  if (n > PC_MAX_N) return KBLAS_NotSupported;
  PosvPlan pl;
  int st = n > 32 ? plan_posv<true, 2>(&hh, n, pl) : plan_posv<true, 1>(&hh, n, pl);
  if (st != KBLAS_Success) return st;
  const size_t head = 256;
  if (!scratch || scratch_bytes < head) return KBLAS_InsufficientWorkspace;
  if (pl.slot_bytes > 0) {
    const size_t fit = (scratch_bytes - head) / pl.slot_bytes;
    if (fit < 1) return KBLAS_InsufficientWorkspace;
    if ((size_t)pl.grid > fit) pl.grid = (int)fit;
  }
  int *header = reinterpret_cast<int *>(scratch);
  cudaError_t e = cudaMemsetAsync(header, 0, head, stream);
  if (e != cudaSuccess) return cuda_check(e, "cudaMemsetAsync", __FILE__, __LINE__);
  SysArgs sys{};
  sys.mode = 0;
  sys.n = n;
  sys.m = m;
  sys.lda = lda;
  sys.ldb = ldb;
  sys.A = A;
  sys.sA = sA;
  sys.B = B;
  sys.sB = sB;
  ItemArgs it{};
  it.uniform = 1;
  it.batch = batch;
  it.n_uniform = n;
  it.queue = header;
  OutArgs out{info, iter, pl.slot_bytes ? scratch + head : nullptr, (long long)pl.slot_bytes,
              pl.tc, nullptr};
  if (n > 32 && pl.tc)
    posv_persistent_kernel<true, 6><<<pl.grid, PC_NT, pl.smem, stream>>>(sys, it, out, pl.cfg, pl.smem);
  else if (n > 32)
    posv_persistent_kernel<true, 2><<<pl.grid, PC_NT, pl.smem, stream>>>(sys, it, out, pl.cfg, pl.smem);
  else
    posv_persistent_kernel<true, 1><<<pl.grid, PC_NT, pl.smem, stream>>>(sys, it, out, pl.cfg, pl.smem);
  KGB_LAUNCH_CHECK("posv_persistent_kernel<mixed>");
  return KBLAS_Success;
}

}  // namespace kgb

using namespace kgb;

extern "C" {

int kblasDposv_batch_mixed_strided(kblasHandle_t h, char side, char uplo, const int m, const int n,
                                   double *A, int lda, long strideA, double *B, int ldb,
                                   long strideB, int batchCount, int *info, int *iter) {
  if (h && batchCount > 1 && (strideA < (long)lda * n || (m > 0 && strideB < (long)ldb * n)))
    return KBLAS_Error_WrongInput;
  if (h && n > 0 && batchCount > 0 && (!A || (m > 0 && !B))) return KBLAS_Error_WrongInput;
  SysArgs s{};
  s.mode = 0;
  s.lda = lda;
  s.ldb = ldb;
  s.A = A;
  s.sA = strideA;
  s.B = B;
  s.sB = strideB;
  return mixed_uniform(h, side, uplo, m, n, s, batchCount, info, iter);
}

int kblasDposv_batch_mixed(kblasHandle_t h, char side, char uplo, const int m, const int n,
                           double **A, int lda, double **B, int ldb, int batchCount, int *info,
                           int *iter) {
  if (h && n > 0 && batchCount > 0 && (!A || (m > 0 && !B))) return KBLAS_Error_WrongInput;
  SysArgs s{};
  s.mode = 1;
  s.lda = lda;
  s.ldb = ldb;
  s.Aarr = A;
  s.Barr = B;
  return mixed_uniform(h, side, uplo, m, n, s, batchCount, info, iter);
}

// Tuning-table override (used by the autotuner to time candidate shapes
// without rebuilding). mixed selects the table; nmax/ts/spi hold
// KBLAS_POSV_TUNING_CLASSES entries each. Passing NULL arrays restores the compiled table.
int kblasSetPosvTuning(int mixed, const int *nmax, const int *ts, const int *spi) {
  TuneOverride &o = tune_override();
  const int k = mixed ? 1 : 0;
  if (!nmax || !ts || !spi) {
    o.set[k] = 0;
    return KBLAS_Success;
  }
  PosvCfg c;
  for (int i = 0; i < PC_NCLS; i++) {
    c.nmax[i] = nmax[i];
    c.ts[i] = ts[i];
    c.spi[i] = spi[i];
  }
  c.nmax[PC_NCLS - 1] = PC_MAX_N;
  c.route_c = 0.f;  // taken from the routing override or the compiled constant
  if (!cfg_valid(c)) return KBLAS_Error_WrongInput;
  o.cfg[k] = c;
  o.set[k] = 1;
  return KBLAS_Success;
}

// Conditioning routing constant of the mixed-precision POSV (the constant c
// of the estimate rho = c * 2^-24 / d_min, see route_fp64): c > 0 sets it,
// c == 0 turns the routing off, c < 0 restores the compiled constant.
int kblasSetPosvRouting(double c) {
  TuneOverride &o = tune_override();
  if (c != c) return KBLAS_Error_WrongInput;
  if (c < 0.0) {
    o.route_set = 0;
  } else {
    o.route_set = 1;
    o.route_c = (float)c;
  }
  return KBLAS_Success;
}

}  // extern "C"

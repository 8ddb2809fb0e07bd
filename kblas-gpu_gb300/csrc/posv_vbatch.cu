// posv_vbatch.cu -- variable-size batched DPOSV (plain FP64 and mixed
// precision) in one persistent launch, preceded by on-device binning.
//
// KBLAS has no variable-size POTRF/POSV (its non-uniform TRSM/SYRK forward to
// MAGMA, src/batch_triangular/Xtrsm_batch_drivers.cuh:278); the argument
// convention (device arrays m, n, lda, ldb plus host bounds max_m, max_n) is
// the reference's non-uniform one (include/kblas_batch.h:829-845).
//
// Launch sequence (all on the handle's stream, no host synchronisation, no
// allocation -- capturable in a CUDA graph):
//   1. cudaMemsetAsync  -- zero the queue header, histogram and cursors
//   2. vb_count         -- validate each system (bad argument -> info = -i),
//                          histogram of the orders n
//   3. vb_plan (1 CTA)  -- orders sorted largest first; per order the slice of
//                          the permutation and the work items (groups of
//                          systems of equal n, sized by the tuning table)
//   4. vb_scatter       -- counting-sort the system indices into the slices
//   5. posv_persistent_kernel -- CTAs pull items from the queue
// Largest-first ordering keeps the tail of the persistent launch short (the
// cost per system spans n^3 over a 32x range of n).
#include <stdio.h>

#include "posv_launch.h"
#include "workspace.h"

namespace kgb {

__global__ void vb_count(long long batch, const int *n, const int *m, const int *lda,
                         const int *ldb, int max_m, int max_n, int *cnt, int *info, int *iter)
{
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < batch;
       b += (long long)gridDim.x * blockDim.x) {
    const int nn = n[b], mm = m[b], la = lda[b], lb = ldb[b];
    int bad = 0;
    // argument positions of kblasDposv_vbatch: 4 m, 5 n, 6 max_m, 7 max_n, 9 lda, 11 ldb
    if (mm < 0) bad = -4;
    else if (nn < 0) bad = -5;
    else if (mm > max_m) bad = -6;
    else if (nn > max_n) bad = -7;
    else if (la < (nn > 1 ? nn : 1)) bad = -9;
    else if (lb < (mm > 1 ? mm : 1)) bad = -11;
    if (bad || nn == 0) {
      if (info) info[b] = bad;
      if (iter) iter[b] = 0;
      continue;
    }
    atomicAdd(&cnt[nn], 1);
  }
}

__global__ void vb_plan(int max_n, const int *cnt, int *off, int *ioff, int4 *items, int *header,
                        PosvCfg cfg)
{
  // prefix sums over n, largest n first (max_n <= 1024: one thread suffices)
  if (threadIdx.x == 0) {
    int o = 0, io = 0, split = -1;
    for (int nn = max_n; nn >= 1; nn--) {
      if (split < 0 && nn <= 32) split = io;  // items of orders > 32 come first
      off[nn] = o;
      ioff[nn] = io;
      const int c = cnt[nn];
      const int spi = cfg.spi[pc_class(cfg, nn)];
      o += c;
      io += (c + spi - 1) / spi;
    }
    header[1] = io;
    header[3] = split < 0 ? io : split;
  }
  __syncthreads();
  for (int nn = 1 + threadIdx.x; nn <= max_n; nn += blockDim.x) {
    const int c = cnt[nn];
    if (!c) continue;
    const int spi = cfg.spi[pc_class(cfg, nn)];
    const int k = (c + spi - 1) / spi;
    for (int j = 0; j < k; j++)
      items[ioff[nn] + j] = make_int4(nn, off[nn] + j * spi, min(spi, c - j * spi), 0);
  }
}

__global__ void vb_scatter(long long batch, const int *n, const int *m, const int *lda,
                           const int *ldb, int max_m, int max_n, const int *off, int *cursor,
                           int *perm)
{
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < batch;
       b += (long long)gridDim.x * blockDim.x) {
    const int nn = n[b], mm = m[b], la = lda[b], lb = ldb[b];
    const bool ok = mm >= 0 && nn >= 1 && mm <= max_m && nn <= max_n && la >= nn &&
                    lb >= (mm > 1 ? mm : 1);
    if (!ok) continue;
    const int pos = atomicAdd(&cursor[nn], 1);
    perm[off[nn] + pos] = (int)b;
  }
}

// Plans of the two launches: the panel path (orders > 32; carries the
// per-CTA scratch) and the register path (orders <= 32).
template <bool MIXED>
static int plan_vbatch(KBlasHandle *h, int max_n, PosvPlan &panel, PosvPlan &reg) {
  int st = plan_posv<MIXED, 1>(h, max_n < 32 ? max_n : 32, reg);
  if (st != KBLAS_Success) return st;
  if (max_n > 32) return plan_posv<MIXED, 2>(h, max_n, panel);
  panel = reg;
  panel.slot_bytes = 0;
  return KBLAS_Success;
}

size_t vbatch_ws_bytes(KBlasHandle *h, int max_n, long long batch, bool mixed) {
  if (batch <= 0 || max_n <= 0 || max_n > PC_MAX_N) return 0;
  PosvPlan panel, reg;
  int st = mixed ? plan_vbatch<true>(h, max_n, panel, reg) : plan_vbatch<false>(h, max_n, panel, reg);
  if (st != KBLAS_Success) return 0;
  return posv_ws_layout(max_n, batch, true, panel).total;
}

// Uniform FP64 POSV / POTRF / POTRS (op 0 / 1 / 2) of order n > 32 on the
// persistent panel path: one launch, teams sized by the FP64 tuning table.
// Returns KBLAS_InsufficientWorkspace, launching nothing, when the handle's
// workspace is short of fp64_uniform_ws_bytes (the caller then uses the
// one-launch blocked kernel); arguments are checked by the caller.
size_t fp64_uniform_ws_bytes(KBlasHandle *h, int n, long long batch) {
  if (n <= 32 || n > PC_MAX_N || batch <= 0) return 0;
  PosvPlan pl;
  if (plan_posv<false, 2>(h, n, pl) != KBLAS_Success) return 0;
  return posv_ws_layout(n, batch, false, pl).total;
}

int fp64_uniform_persistent(KBlasHandle *h, int op, int m, int n, SysArgs sys, int batch,
                            int *info) {
  if (n <= 32 || n > PC_MAX_N) return KBLAS_NotSupported;
  PosvPlan pl;
  int st = plan_posv<false, 2>(h, n, pl);
  if (st != KBLAS_Success) return st;
  const PosvWs ws = posv_ws_layout(n, batch, false, pl);
  if (ws.total > h->ws.allocated.d_data_bytes || !h->ws.d_data) return KBLAS_InsufficientWorkspace;
  char *base = static_cast<char *>(h->ws.d_data);
  int *header = reinterpret_cast<int *>(base + ws.header);
  cudaError_t e = cudaMemsetAsync(header, 0, 64 * sizeof(int), h->stream);
  if (e != cudaSuccess) return cuda_check(e, "cudaMemsetAsync", __FILE__, __LINE__);
  sys.n = n;
  sys.m = (op == 1) ? 0 : m;
  sys.op = (op == 2) ? 2 : 0;
  ItemArgs it{};
  it.uniform = 1;
  it.batch = batch;
  it.n_uniform = n;
  it.queue = header;
  OutArgs out{op == 2 ? nullptr : info, nullptr, base + ws.scratch, (long long)pl.slot_bytes,
              0, h->d_status};
  posv_persistent_kernel<false, 2><<<pl.grid, PC_NT, pl.smem, h->stream>>>(sys, it, out, pl.cfg, pl.smem);
  KGB_LAUNCH_CHECK("posv_persistent_kernel<fp64>");
  return KBLAS_Success;
}

template <bool MIXED>
static int vbatch(KBlasHandle *h, char side, char uplo, int *m, int *n, int max_m, int max_n,
                  double **A, int *lda, double **B, int *ldb, int batch, int *info, int *iter) {
  if (!h) return KBLAS_Error_NotInitialized;
  if (is_left(side) || is_upper(uplo)) {
    printf("(Left | Upper) POSV_VBATCH is not implemented yet\n");
    return KBLAS_NotImplemented;
  }
  if (!is_right(side) || !is_lower(uplo) || batch < 0 || max_n < 0 || max_m < 0)
    return KBLAS_Error_WrongInput;
  if (batch == 0) return KBLAS_Success;
  if (!m || !n || !A || !lda || !B || !ldb) return KBLAS_Error_WrongInput;
  if (max_n > PC_MAX_N) return KBLAS_NotSupported;
  if (max_n == 0) {
    int st = zero_info(h, info, batch);
    return st == KBLAS_Success ? zero_info(h, iter, batch) : st;
  }
  PosvPlan pl, preg;
  int st = plan_vbatch<MIXED>(h, max_n, pl, preg);
  if (st != KBLAS_Success) return st;
  const PosvWs ws = posv_ws_layout(max_n, batch, true, pl);
  if (ws.total > h->ws.allocated.d_data_bytes || !h->ws.d_data) return KBLAS_InsufficientWorkspace;
  char *base = static_cast<char *>(h->ws.d_data);
  int *header = reinterpret_cast<int *>(base + ws.header);
  int *cnt = reinterpret_cast<int *>(base + ws.cnt);
  int *off = reinterpret_cast<int *>(base + ws.off);
  int *ioff = reinterpret_cast<int *>(base + ws.ioff);
  int *cursor = reinterpret_cast<int *>(base + ws.cursor);
  int *perm = reinterpret_cast<int *>(base + ws.perm);
  int4 *items = reinterpret_cast<int4 *>(base + ws.items);
  // header .. cursor are contiguous: one memset clears them
  cudaError_t e = cudaMemsetAsync(base, 0, ws.perm, h->stream);
  if (e != cudaSuccess) return cuda_check(e, "cudaMemsetAsync", __FILE__, __LINE__);
  const int tpb = 256;
  long long nb = (batch + tpb - 1) / tpb;
  const int blocks = (int)(nb < 4L * h->sm_count * 8 ? nb : 4L * h->sm_count * 8);
  vb_count<<<blocks, tpb, 0, h->stream>>>(batch, n, m, lda, ldb, max_m, max_n, cnt, info,
                                          MIXED ? iter : nullptr);
  KGB_LAUNCH_CHECK("vb_count");
  vb_plan<<<1, 256, 0, h->stream>>>(max_n, cnt, off, ioff, items, header, pl.cfg);
  KGB_LAUNCH_CHECK("vb_plan");
  vb_scatter<<<blocks, tpb, 0, h->stream>>>(batch, n, m, lda, ldb, max_m, max_n, off, cursor, perm);
  KGB_LAUNCH_CHECK("vb_scatter");
  SysArgs sys{};
  sys.mode = 2;
  sys.Aarr = A;
  sys.Barr = B;
  sys.narr = n;
  sys.marr = m;
  sys.ldaarr = lda;
  sys.ldbarr = ldb;
  ItemArgs it{};
  it.uniform = 0;
  it.batch = batch;
  it.items = items;
  it.perm = perm;
  it.nitems_p = header + 1;
  it.split_p = header + 3;
  OutArgs out{info, MIXED ? iter : nullptr, base + ws.scratch, (long long)pl.slot_bytes,
              pl.tc, h->d_status};
  // orders > 32 first (largest first), then orders <= 32 on the register path
  if (max_n > 32) {
    it.queue = header;
    bool launched = false;
    if constexpr (MIXED) {
      if (pl.tc) {
        posv_persistent_kernel<MIXED, 6><<<pl.grid, PC_NT, pl.smem, h->stream>>>(sys, it, out, pl.cfg, pl.smem);
        launched = true;
      }
    }
    if (!launched)
      posv_persistent_kernel<MIXED, 2><<<pl.grid, PC_NT, pl.smem, h->stream>>>(sys, it, out, pl.cfg, pl.smem);
    KGB_LAUNCH_CHECK("posv_persistent_kernel");
  }
  it.queue = header + 2;
  posv_persistent_kernel<MIXED, 1><<<preg.grid, PC_NT, preg.smem, h->stream>>>(sys, it, out, preg.cfg, preg.smem);
  KGB_LAUNCH_CHECK("posv_persistent_kernel");
  return KBLAS_Success;
}

}  // namespace kgb

using namespace kgb;

extern "C" {

int kblasDposv_vbatch(kblasHandle_t h, char side, char uplo, int *m, int *n, int max_m, int max_n,
                      double **A, int *lda, double **B, int *ldb, int batchCount, int *info) {
  return vbatch<false>(h, side, uplo, m, n, max_m, max_n, A, lda, B, ldb, batchCount, info, nullptr);
}

int kblasDposv_vbatch_mixed(kblasHandle_t h, char side, char uplo, int *m, int *n, int max_m,
                            int max_n, double **A, int *lda, double **B, int *ldb, int batchCount,
                            int *info, int *iter) {
  return vbatch<true>(h, side, uplo, m, n, max_m, max_n, A, lda, B, ldb, batchCount, info, iter);
}

}  // extern "C"

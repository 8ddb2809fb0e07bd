// posv_core.cuh -- the persistent batched POSV kernel behind the
// mixed-precision (kblasDposv_batch_mixed*) and variable-size
// (kblasDposv_vbatch*) entry points.
//
// One launch processes a whole batch. CTAs pull work items from a device
// queue (one atomicAdd per item, no waiting anywhere). A work item is a group
// of systems of the same order n; the CTA's threads are split into teams of
// TS threads, one system per team (TS and the systems per item come from the
// tuning table, per size class). Per system, everything happens while the
// system is on chip -- read A once, factor, solve, refine, write X:
//
//  MIXED (X*A = B, side 'R', lower; LAPACK DSPOSV semantics):
//   1. stage A's lower triangle as FP32 with power-of-two symmetric diagonal
//      scaling  As = S A S,  S = diag(2^-e_i),  e_i = floor(log2(a_ii) / 2),
//      so the factor stays in range (the scaling is exact);
//   2. FP32 Cholesky As = Ls Ls^T in shared memory (pivot test d > n*2^-24);
//   3. x = S Ls^-T Ls^-1 S b in FP32, then refine: r = b - A x in FP64 (A
//      re-read from L2), stop when ||r|| <= 2 sqrt(n) eps64 (||A|| ||x|| +
//      ||b||) -- with the residual's own rounding this certifies a backward
//      error below 10 n eps64 -- else x += S Ls^-T Ls^-1 S r (FP32 solve,
//      FP64 update);
//   4. a system whose FP32 factorization fails, or whose refinement stalls
//      (error not halved) or runs out of steps, is factored again in FP64 by
//      the same team (packed factor in a global scratch slot) and solved
//      directly; A then receives the FP64 factor and info the exact LAPACK
//      code. iter[] records the outcome.
//  PLAIN (FP64 POSV): FP64 factor in shared memory (or the scratch slot when
//   it does not fit), solve, write L and X -- LAPACK DPOSV semantics.
#pragma once

#include <stdint.h>

#include "chol_dev.cuh"
#include "team.cuh"

namespace kgb {

constexpr int PC_NT = 256;     // threads per persistent CTA
constexpr int PC_NCLS = 6;     // size classes
constexpr int PC_MR = 4;       // right-hand sides per residual sweep
constexpr int PC_ITMAX = 12;   // refinement step cap

struct PosvCfg {
  int nmax[PC_NCLS];  // class c holds n <= nmax[c] (ascending)
  int ts[PC_NCLS];    // team size (threads) of class c
  int spi[PC_NCLS];   // systems per work item of class c
};

__host__ __device__ __forceinline__ int pc_class(const PosvCfg &c, int n) {
  for (int k = 0; k < PC_NCLS; k++)
    if (n <= c.nmax[k]) return k;
  return PC_NCLS - 1;
}

// Describes where the systems are: uniform strided / pointer-array, or
// per-system arrays (variable size). All pointers are device pointers.
struct SysArgs {
  int mode;  // 0 uniform strided, 1 uniform pointer array, 2 variable size
  int n, m, lda, ldb;
  double *A;
  long long sA;
  double *B;
  long long sB;
  double *const *Aarr;
  double *const *Barr;
  const int *narr, *marr, *ldaarr, *ldbarr;
  __device__ __forceinline__ void get(long long b, int &nn, int &mm, double *&Ap, int &la,
                                      double *&Bp, int &lb) const {
    if (mode == 2) {
      nn = narr[b]; mm = marr[b]; la = ldaarr[b]; lb = ldbarr[b];
      Ap = Aarr[b]; Bp = Barr[b];
    } else {
      nn = n; mm = m; la = lda; lb = ldb;
      Ap = (mode == 0) ? A + b * sA : Aarr[b];
      Bp = (mode == 0) ? B + b * sB : Barr[b];
    }
  }
};

// Work items: uniform batches are cut into consecutive groups; binned
// variable-size batches use the item table written by the binning kernels.
struct ItemArgs {
  int uniform;          // 1: item q = systems [q*spi, (q+1)*spi)
  long long batch;
  int n_uniform;
  const int4 *items;    // (n, start, count, -) into perm
  const int *perm;
  const int *nitems_p;  // number of items (device), for binned batches
  int *queue;           // work counter (zeroed before the launch)
};

struct OutArgs {
  int *info;   // may be NULL
  int *iter;   // may be NULL (mixed only)
  char *scratch;         // per-CTA global scratch slots
  long long slot_bytes;  // bytes per CTA slot
};

// ---- per-team shared memory layout -------------------------------------
template <bool MIXED>
__host__ __device__ __forceinline__ size_t team_smem_bytes(int n, int ts, bool lp_in_smem) {
  const size_t P = (size_t)n * (n + 1) / 2;
  const int nw = ts >= 32 ? ts / 32 : 1;
  size_t b = 0;
  if (MIXED) {
    b += (lp_in_smem ? P : 0) * 4;        // FP32 factor
    b += 3 * (size_t)n * 4;               // rinv, scale, (spare)
    b += (size_t)PC_MR * n * 4;           // FP32 solve vectors
    b = (b + 7) / 8 * 8;
    b += 2 * (size_t)PC_MR * n * 8;       // x, r (FP64)
    b += (size_t)32 * nw * 8;             // reduction scratch
    b += 64;                              // flags
  } else {
    b += (lp_in_smem ? P : 0) * 8;        // FP64 factor
    b += (size_t)n * 8;                   // rinv
    b += (size_t)PC_MR * n * 8;           // solve vectors
    b += (size_t)32 * nw * 8;
    b += 64;
  }
  return (b + 15) / 16 * 16;
}

// Stage A's lower triangle (FP64) into the packed factor storage of type T,
// optionally as FP32 with the exponent shifts e[] applied.
template <typename T, bool SCALE>
__device__ __forceinline__ void team_load_lower(const Team &t, int n, const double *A, int lda,
                                                T *Lp, const float *scl)
{
  // columns one after the other, team lanes along the rows (coalesced)
  for (int k = 0; k < n; k++) {
    const double *col = A + (size_t)k * lda;
    T *dst = Lp + coff(k, n) - k;
    for (int i = k + t.tid; i < n; i += t.nt) {
      if (SCALE) dst[i] = (T)((float)col[i] * scl[i] * scl[k]);
      else dst[i] = (T)col[i];
    }
  }
}

// Loop bound that is uniform across every team sharing a warp: sub-warp
// teams must call the same sequence of __syncwarp, so loops whose trip count
// depends on per-system data run to the warp-wide maximum.
__device__ __forceinline__ int warp_uniform_max(const Team &t, int v) {
  if (t.nt >= 32) return v;
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__device__ __forceinline__ int group_any(const Team &t, int v, int *scratch) {
  if (t.nt < 32) return __any_sync(0xffffffffu, v);  // warp-wide: keeps sub-warp teams in step
  return team_any(t, v, scratch);
}

// FP64 factor + solve of one system (the plain path, and the mixed path's
// fallback). Lp64 is packed FP64 storage (shared or scratch). Solves the RHS
// rows [r_from, m) of B and writes L to A. Returns the info code.
static __device__ int team_fp64_posv(const Team &t, bool active, int n, int m, int r_from, double *A,
                              int lda, double *B, int ldb, double *Lp64, double *rinv64, double *y,
                              double *red)
{
  if (active) team_load_lower<double, false>(t, n, A, lda, Lp64, nullptr);
  t.sync();
  int info = team_potrf_packed<double>(t, n, Lp64, rinv64, 0.0, active);
  // write the factor back (columns before a failure are the true factor; the
  // failing column keeps its non-positive pivot, LAPACK xPOTRF style)
  if (active) {
    const int ncol = info ? info : n;
    for (int k = 0; k < ncol; k++) {
      double *col = A + (size_t)k * lda;
      const double *src = Lp64 + coff(k, n) - k;
      for (int i = k + t.tid; i < n; i += t.nt) col[i] = src[i];
    }
  }
  const bool solve = active && info == 0;
  const int m_hi = warp_uniform_max(t, active ? m : 0);
  for (int r0 = r_from; r0 < m_hi; r0++) {
    const bool go = solve && r0 < m;
    if (go)
      for (int i = t.tid; i < n; i += t.nt) y[i] = B[(size_t)r0 + (size_t)i * ldb];
    t.sync();
    team_llt_solve<double>(t, n, Lp64, rinv64, y, red, go);
    if (go)
      for (int i = t.tid; i < n; i += t.nt) B[(size_t)r0 + (size_t)i * ldb] = y[i];
    t.sync();
  }
  return info;
}

// Mixed-precision solve of one system by one team (see the file header).
static __device__ void team_mixed_posv(const Team &t, bool active, int n, int m, double *A, int lda,
                                double *B, int ldb, unsigned char *base, bool lp_smem,
                                float *Lp_scratch, double *Lp64_scratch, int *info_out,
                                int *iter_out)
{
  const size_t P = (size_t)n * (n + 1) / 2;
  float *Lp = lp_smem ? reinterpret_cast<float *>(base) : Lp_scratch;
  unsigned char *p = base + (lp_smem ? P * 4 : 0);
  float *rinv = reinterpret_cast<float *>(p); p += (size_t)n * 4;
  float *scl = reinterpret_cast<float *>(p); p += (size_t)n * 4;
  p += (size_t)n * 4;
  float *ys = reinterpret_cast<float *>(p); p += (size_t)PC_MR * n * 4;
  p = reinterpret_cast<unsigned char *>(((uintptr_t)p + 7) & ~(uintptr_t)7);
  double *x = reinterpret_cast<double *>(p); p += (size_t)PC_MR * n * 8;
  double *r = reinterpret_cast<double *>(p); p += (size_t)PC_MR * n * 8;
  double *red = reinterpret_cast<double *>(p);

  // ---- 1. power-of-two scaling from the FP64 diagonal ----
  int bad_diag = 0;
  if (active)
    for (int i = t.tid; i < n; i += t.nt) {
      const double d = A[(size_t)i + (size_t)i * lda];
      int e = 0;
      if (d > 0.0 && d < 1e300) {
        e = ilogb(d);
        e = (e >= 0) ? e / 2 : -((-e + 1) / 2);  // floor(log2(d) / 2)
        if (e > 120 || e < -120) bad_diag = 1;   // outside FP32 range: FP64 path
      } else {
        bad_diag = 1;  // non-positive / NaN / huge diagonal: the FP64 path decides
      }
      scl[i] = bad_diag ? 1.0f : ldexpf(1.0f, -e);
    }
  t.sync();
  // ---- 2. stage As = S A S in FP32 and factor it ----
  if (active) team_load_lower<float, true>(t, n, A, lda, Lp, scl);
  t.sync();
  const float ftol = (float)n * 5.9604645e-08f;  // n * 2^-24
  const int fail = team_potrf_packed<float>(t, n, Lp, rinv, ftol, active);
  // ||A||_inf (= ||A||_1 by symmetry); an FP32 sum is enough for a threshold
  double anorm = 0.0;
  if (active) {
    float rs_max = 0.f;
    for (int i = t.tid; i < n; i += t.nt) {
      float s = 0.f;
      for (int j = 0; j <= i; j++) s += fabsf((float)A[(size_t)i + (size_t)j * lda]);
      for (int j = i + 1; j < n; j++) s += fabsf((float)A[(size_t)j + (size_t)i * lda]);
      rs_max = fmaxf(rs_max, s);
    }
    anorm = (double)rs_max * (1.0 + 1e-6 * n);
  }
  anorm = team_max<double>(t, anorm, red);
  const int bad = team_any(t, active && (fail != 0 || bad_diag), reinterpret_cast<int *>(red));
  bool need_fb = active && bad;
  int fb_code = need_fb ? -1 : 0, fb_from = 0, steps_used = 0;
  const double tol_conv = 2.0 * sqrt((double)n) * 1.1102230246251565e-16;

  // ---- 3. solve and refine, PC_MR right-hand sides at a time ----
  const int m_hi = warp_uniform_max(t, active ? m : 0);
  for (int r0 = 0; r0 < m_hi; r0 += PC_MR) {
    const int nr = (active && r0 < m) ? min(PC_MR, m - r0) : 0;
    const bool go0 = active && !need_fb && nr > 0;
    for (int q = 0; q < PC_MR; q++) {
      const bool gq = go0 && q < nr;
      if (gq)
        for (int i = t.tid; i < n; i += t.nt)
          ys[q * n + i] = (float)B[(size_t)(r0 + q) + (size_t)i * ldb] * scl[i];
      t.sync();
      team_llt_solve<float>(t, n, Lp, rinv, ys + q * n, reinterpret_cast<float *>(red), gq);
      if (gq)
        for (int i = t.tid; i < n; i += t.nt) x[q * n + i] = (double)(ys[q * n + i] * scl[i]);
      t.sync();
    }
    double eta_prev = INFINITY;
    bool going = go0, converged = false;
    int step = 0;
    while (group_any(t, going, reinterpret_cast<int *>(red))) {
      team_residual<PC_MR>(t, n, A, lda, B, ldb, r0, nr, x, n, r, going);
      t.sync();
      double eta = 0.0;
      for (int q = 0; q < PC_MR; q++) {
        double rm = 0.0, xm = 0.0, bm = 0.0;
        if (going && q < nr)
          for (int i = t.tid; i < n; i += t.nt) {
            rm = fmax(rm, fabs(r[q * n + i]));
            xm = fmax(xm, fabs(x[q * n + i]));
            bm = fmax(bm, fabs(B[(size_t)(r0 + q) + (size_t)i * ldb]));
          }
        rm = team_max<double>(t, rm, red);
        xm = team_max<double>(t, xm, red);
        bm = team_max<double>(t, bm, red);
        if (going && q < nr) {
          const double den = anorm * xm + bm;
          const double e = (den > 0.0) ? rm / den : (rm > 0.0 ? INFINITY : 0.0);
          eta = (e > eta || e != e) ? e : eta;
        }
      }
      if (going) {
        if (eta <= tol_conv) {
          going = false;
          converged = true;
        } else if (!(eta <= 0.5 * eta_prev) || step >= PC_ITMAX) {
          going = false;  // stalled, NaN, or out of steps
        }
      }
      for (int q = 0; q < PC_MR; q++) {
        const bool gq = going && q < nr;
        if (gq)
          for (int i = t.tid; i < n; i += t.nt) ys[q * n + i] = (float)r[q * n + i] * scl[i];
        t.sync();
        team_llt_solve<float>(t, n, Lp, rinv, ys + q * n, reinterpret_cast<float *>(red), gq);
        if (gq)
          for (int i = t.tid; i < n; i += t.nt) x[q * n + i] += (double)(ys[q * n + i] * scl[i]);
        t.sync();
      }
      if (going) {
        eta_prev = eta;
        step++;
      }
    }
    if (go0) {
      steps_used = max(steps_used, step);
      if (converged) {
        for (int q = 0; q < nr; q++)
          for (int i = t.tid; i < n; i += t.nt) B[(size_t)(r0 + q) + (size_t)i * ldb] = x[q * n + i];
      } else {
        need_fb = true;
        fb_code = (step >= PC_ITMAX) ? -3 : -2;
        fb_from = r0;
      }
    }
    t.sync();
  }
  // ---- 4. FP64 fallback for the systems that need it ----
  int info = 0;
  if (group_any(t, need_fb, reinterpret_cast<int *>(red)))
    info = team_fp64_posv(t, need_fb, n, m, fb_from, A, lda, B, ldb, Lp64_scratch, r, x, red);
  if (active && t.tid == 0) {
    if (info_out) *info_out = need_fb ? info : 0;
    if (iter_out) *iter_out = need_fb ? fb_code : steps_used;
  }
}

template <bool MIXED>
__global__ void __launch_bounds__(PC_NT)
posv_persistent_kernel(SysArgs sys, ItemArgs it, OutArgs out, PosvCfg cfg, int smem_bytes)
{
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_item;
  long long nitems;
  if (it.uniform) {
    const int spi = cfg.spi[pc_class(cfg, it.n_uniform)];
    nitems = (it.batch + spi - 1) / spi;
  } else {
    nitems = *it.nitems_p;
  }
  char *slot = out.scratch ? out.scratch + (size_t)blockIdx.x * out.slot_bytes : nullptr;

  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(it.queue, 1);
    __syncthreads();
    const long long q = s_item;
    __syncthreads();
    if (q >= nitems) break;
    int n, start, count;
    if (it.uniform) {
      n = it.n_uniform;
      const int spi = cfg.spi[pc_class(cfg, n)];
      start = (int)(q * spi);
      count = (int)min((long long)spi, it.batch - q * spi);
    } else {
      const int4 e = it.items[q];
      n = e.x;
      start = e.y;
      count = e.z;
    }
    const int c = pc_class(cfg, n);
    const int TS = cfg.ts[c];
    const int team_id = threadIdx.x / TS;
    const int nteams = PC_NT / TS;
    const size_t P = (size_t)n * (n + 1) / 2;
    const bool lp_smem = (size_t)nteams * team_smem_bytes<MIXED>(n, TS, true) <= (size_t)smem_bytes;
    const size_t tb = team_smem_bytes<MIXED>(n, TS, lp_smem);
    const Team t{(int)(threadIdx.x % TS), TS, 1 + team_id};
    const bool active = team_id < count;
    // whole-warp teams without a system have nothing to synchronise with
    if (active || TS < 32) {
      long long sidx = 0;
      int nn = n, m = 0, lda = 1, ldb = 1;
      double *A = nullptr, *B = nullptr;
      if (active) {
        sidx = it.uniform ? (long long)start + team_id : (long long)it.perm[start + team_id];
        sys.get(sidx, nn, m, A, lda, B, ldb);
      }
      unsigned char *base = smem + (size_t)team_id * tb;
      // scratch slot: FP64 packed factors of all teams, then FP32 ones
      double *Lp64_scratch = slot ? reinterpret_cast<double *>(slot) + (size_t)team_id * P : nullptr;
      float *Lp32_scratch =
          slot ? reinterpret_cast<float *>(reinterpret_cast<double *>(slot) + (size_t)nteams * P) +
                     (size_t)team_id * P
               : nullptr;
      int *info_p = (active && out.info) ? out.info + sidx : nullptr;
      int *iter_p = (active && out.iter) ? out.iter + sidx : nullptr;
      if (MIXED) {
        team_mixed_posv(t, active, n, m, A, lda, B, ldb, base, lp_smem, Lp32_scratch, Lp64_scratch,
                        info_p, iter_p);
      } else {
        double *Lp64 = lp_smem ? reinterpret_cast<double *>(base) : Lp64_scratch;
        unsigned char *p = base + (lp_smem ? P * 8 : 0);
        double *rinv = reinterpret_cast<double *>(p); p += (size_t)n * 8;
        double *y = reinterpret_cast<double *>(p); p += (size_t)PC_MR * n * 8;
        double *red = reinterpret_cast<double *>(p);
        const int info = team_fp64_posv(t, active, n, m, 0, A, lda, B, ldb, Lp64, rinv, y, red);
        if (info_p && t.tid == 0) *info_p = info;
      }
    }
    __syncthreads();
  }
}

// Bytes of global scratch each persistent CTA needs: the packed FP64 factors
// of all teams of the largest item (mixed fallback / plain factors that do
// not fit in shared memory).
__host__ inline size_t posv_slot_bytes(const PosvCfg &cfg, int max_n) {
  size_t best = 0;
  for (int c = 0; c < PC_NCLS; c++) {
    const int nhi = min(cfg.nmax[c], max_n);
    const int nlo = c ? cfg.nmax[c - 1] + 1 : 1;
    if (nhi < nlo) continue;
    const size_t P = (size_t)nhi * (nhi + 1) / 2;
    const size_t b = (size_t)(PC_NT / cfg.ts[c]) * P * 12;  // FP64 + FP32 packed factors
    if (b > best) best = b;
  }
  return (best + 255) / 256 * 256;
}

}  // namespace kgb

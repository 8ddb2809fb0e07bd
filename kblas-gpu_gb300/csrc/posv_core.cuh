// posv_core.cuh -- the persistent batched POSV kernel behind the
// mixed-precision (kblasDposv_batch_mixed*) and variable-size
// (kblasDposv_vbatch*) entry points.
//
// One launch processes a whole batch. CTAs pull work items from a device
// queue (one atomicAdd per item; nothing ever waits on another CTA). A work
// item is a group of systems of the same order n; the CTA's threads are
// split into teams of TS threads, one system per team (TS and the systems per
// item come from the tuning table, per size class). Per system, everything
// happens while the system is on chip -- read A, factor, solve, refine,
// write X:
//
//  MIXED (X*A = B, side 'R', lower; LAPACK DSPOSV semantics):
//   1. power-of-two symmetric diagonal scaling As = S A S, S = diag(2^-e_i),
//      e_i = floor(log2(a_ii)/2): exact, and keeps the FP32 factor in range;
//   2. FP32 Cholesky As = Ls Ls^T on chip (pivot test d > n*2^-24);
//   3. x = S Ls^-T Ls^-1 S b in FP32, then refinement: r = b - A x in FP64 (A
//      re-read, L2 resident), stop when ||r|| <= (9n - 2) eps64 (||A|| ||x|| +
//      ||b||) -- with the residual's own rounding (< (n+1) eps64) this
//      certifies a normwise backward error below 10 n eps64 -- else
//      x += S Ls^-T Ls^-1 S r (FP32 solve, FP64 update);
//   4. a system whose FP32 factorization fails, or whose refinement stalls
//      (error not halved), converges too slowly to beat an FP64 re-solve
//      (refine_too_slow) or runs out of steps, is factored again in FP64 by
//      the same team and solved directly; A then receives the FP64 factor and
//      info the exact LAPACK code; iter[] records which path was taken.
//  PLAIN (FP64 POSV): FP64 factor, solve, write L and X (LAPACK DPOSV).
//
// n <= 32: register path (chol_small.cuh), W lanes per system (W >= n).
// n >  32: panel path (chol_panel.cuh), teams of whole warps; the factor in
//          shared memory, or in the CTA's global scratch slot when too big.
#pragma once

#include <stdint.h>

#include "chol_small.cuh"
#include "team.cuh"

namespace kgb {

constexpr int PC_NT = 256;     // threads per persistent CTA
constexpr int PC_NCLS = 8;     // size classes (KBLAS_POSV_TUNING_CLASSES)
constexpr int PC_MR = 4;       // right-hand sides per residual sweep (panel path)
// The mixed panel path runs its trailing updates on the tensor cores when a
// launch holds orders above this: at n = 512 (8 RHS) that measured +5.6%, on
// the n <= 256 distribution the kernel without tensor-core code was 1.5%
// faster (at n <= 256 a step's update is too small to pay for the staging).
constexpr int PC_TC_NMIN = 256;
constexpr int PC_ITMAX = 12;   // refinement step cap
constexpr double PC_EPS64 = 1.1102230246251565e-16;  // 2^-53, FP64 unit roundoff

// Refinement stops when the computed normwise backward error
// eta = ||b - A x|| / (||A|| ||x|| + ||b||) (infinity norms) is at most
// (9n - 2) u, u = 2^-53. The FP64 residual is computed with an error of at most
// gamma_{n+1} (||b|| + ||A|| ||x||) per component, gamma_{n+1} <= (n + 1.01) u,
// so the true backward error is then at most ((9n - 2) + (n + 1.01)) u < 10 n u,
// the accuracy the routine guarantees; ||A|| is taken from truncated FP32 row
// sums (never above the true norm, which only makes eta larger) or, on the
// register path, from rounded FP32 sums inflated by at most 1 + 4e-5 (n <= 32),
// which the 0.99 u of slack covers.
__host__ __device__ __forceinline__ double posv_eta_target(int n) {
  return (9.0 * n - 2.0) * PC_EPS64;
}

// Cost-model exit from refinement. A residual sweep over nr right-hand sides
// costs n^2 nr FP64 FMAs; re-solving in FP64 costs n^3/6 (factor) + n^2 nr
// (solve), i.e. n / (6 nr) + 1 sweeps. When the observed contraction
// eta / eta_prev predicts more sweeps than that before eta reaches the
// target, the FP64 path is the cheaper way to the same guarantee.
__device__ __forceinline__ bool refine_too_slow(double eta, double eta_prev, double tol, int n,
                                                int nr) {
  if (!(eta_prev < INFINITY) || !(eta > tol)) return false;
  const float rho = (float)(eta / eta_prev);   // in (0, 0.5] here
  const float need = log2f((float)(eta / tol)) / -log2f(rho);
  return need > (float)n / (6.0f * (float)nr) + 1.0f;
}

struct PosvCfg {
  int nmax[PC_NCLS];  // class c holds n <= nmax[c] (ascending)
  int ts[PC_NCLS];    // team size (threads) of class c
  int spi[PC_NCLS];   // systems per work item of class c
  float route_c;      // conditioning routing constant (route_fp64); <= 0: no routing
};

// Routing to FP64 before any refinement, from a conditioning estimate that
// the FP32 factorization gives for free. On the scaled matrix (unit
// diagonal) every pivot d_i = L_ii^2 lies in [lambda_min, lambda_max], so
// d_min = min d_i bounds lambda_min from above; the refinement contracts the
// error by about rho = ||A^-1 dA|| with ||dA|| ~ c u32 (u32 = 2^-24), so
// rho_hat = c u32 / d_min. From the first FP32 solve's backward error (~
// sqrt(n) u32) to the target (9n - 2) u64 takes
// k = log2(sqrt(n) u32 / ((9n - 2) u64)) / -log2(rho_hat) refinement steps,
// each one FP64 residual sweep (n^2 nr FMAs) after the first, against n^3 / 6
// + n^2 nr for the FP64 factor and solve: a system goes straight to the FP64
// path when rho_hat >= 1/2 or k > max(n / (6 nr), 1.5). The refinement's own
// cost-model exit (refine_too_slow) still catches what the estimate misses.
// Panel path only (n > 32): below that the FP64 factorization is not the
// cheaper path in practice (every step is latency, not FP64 work).
__device__ __forceinline__ bool route_fp64(float dmin, int n, int nr, float c) {
  if (!(c > 0.f)) return false;
  if (!(dmin > 0.f)) return true;
  const float rho = c * 5.9604645e-08f / dmin;
  if (!(rho < 0.5f)) return true;
  const float l = 29.0f + 0.5f * log2f((float)n) - log2f(9.0f * n - 2.0f);
  const float k = l / -log2f(rho);
  // a system that converges in one or two steps stays on the mixed path even
  // when many right-hand sides make the FP64 factorization cheap
  return k > fmaxf((float)n / (6.0f * (float)nr), 1.5f);
}

__host__ __device__ __forceinline__ int pc_class(const PosvCfg &c, int n) {
  for (int k = 0; k < PC_NCLS; k++)
    if (n <= c.nmax[k]) return k;
  return PC_NCLS - 1;
}

// Where the systems are: uniform strided / pointer array, or per-system arrays.
struct SysArgs {
  int mode;  // 0 uniform strided, 1 uniform pointer array, 2 variable size
  int op;    // plain FP64 panel path: 0 POSV (POTRF when m = 0), 2 POTRS (A holds L)
  int n, m, lda, ldb;
  double *A;
  long long sA;
  double *B;
  long long sB;
  double *const *Aarr;
  double *const *Barr;
  const int *narr, *marr, *ldaarr, *ldbarr;
  __device__ __forceinline__ void get(long long b, int &mm, double *&Ap, int &la, double *&Bp,
                                      int &lb) const {
    if (mode == 2) {
      mm = marr[b]; la = ldaarr[b]; lb = ldbarr[b];
      Ap = Aarr[b]; Bp = Barr[b];
    } else {
      mm = m; la = lda; lb = ldb;
      Ap = (mode == 0) ? A + b * sA : Aarr[b];
      Bp = (mode == 0) ? B + b * sB : (Barr ? Barr[b] : nullptr);  // no B for POTRF
    }
  }
};

struct ItemArgs {
  int uniform;          // 1: item q = systems [q*spi, (q+1)*spi)
  long long batch;
  int n_uniform;
  const int4 *items;    // (n, start, count, -) into perm
  const int *perm;
  const int *nitems_p;  // number of items (device), binned batches
  const int *split_p;   // binned: items [0, *split_p) have n > 32, the rest n <= 32
  int *queue;           // work counter (zeroed before the launch)
};

struct OutArgs {
  int *info;
  int *iter;
  char *scratch;         // per-CTA global scratch slots
  long long slot_bytes;
  int tc;                // mixed panel path: tensor-core trailing updates for whole-CTA teams
  int *status;           // device status word: set to 1 when a bounded wait ran out (may be null)
};

// ---------------------------------------------------------------------------
// shared-memory bytes of one team
// ---------------------------------------------------------------------------
// tc: a whole-CTA team of the mixed panel path stages the BF16 operands of
// its tensor-core trailing updates in the region of the solve / refinement
// vectors (free during the factorization), grown to the staging size.
template <bool MIXED>
__host__ __device__ __forceinline__ size_t team_smem_bytes(int n, int ts, bool fac_in_smem,
                                                           bool tc = false) {
  if (n <= 32) {
    // register path: row-major L (FP64; FP32 too for mixed), reciprocal
    // pivots, scales
    const int W = ts;
    size_t b = (size_t)W * (W + 1) * 8 + (size_t)W * 8;
    if (MIXED) b += (size_t)W * (W + 1) * 4 + 2 * (size_t)W * 4;
    return (b + 15) / 16 * 16;
  }
  const PanelLayout L = make_layout(n);
  const int nw = ts / 32;
  const size_t T = MIXED ? 4 : 8;
  size_t b = 0;
  b += (fac_in_smem ? L.total() : 0) * T;          // panels
  b += 32 * LDD * 8;                               // diagonal block (FP64 size: fallback too)
  b += (size_t)n * 8;                              // rinv (FP64 size: fallback too)
  if (MIXED) {
    b += (size_t)n * 8;                            // scales + exponent shifts
    b = (b + 15) / 16 * 16;
    size_t u = (size_t)PC_MR * n * 4;              // FP32 solve vectors
    u = (u + 7) / 8 * 8;
    u += 2 * (size_t)PC_MR * n * 8;                // x, r
    u += (size_t)nw * n * 8;                       // per-warp column sums of the residual
    if (tc && ts == PC_NT && u < tc_stage_bytes(n)) u = tc_stage_bytes(n);
    b += u;
  } else {
    b += (size_t)n * 8;                            // solve vector
  }
  b += (size_t)32 * nw * 8;                        // reductions / partial sums
  b += 16;                                         // flag
  return (b + 15) / 16 * 16;
}

// ---------------------------------------------------------------------------
// helpers keeping sub-warp teams in step
// ---------------------------------------------------------------------------
__device__ __forceinline__ int warp_uniform_max_w(int v, int W) {
  if (W >= 32) return v;
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__device__ __forceinline__ int seg_any(int v, int W) {
  const unsigned ball = __ballot_sync(0xffffffffu, v);
  if (W >= 32) return ball != 0u;
  const int base = (threadIdx.x & 31) & ~(W - 1);
  return ((ball >> base) & ((1u << W) - 1u)) != 0u;
}

// power-of-two scale 2^sh of row i from the FP64 diagonal (sh = -floor(
// log2(a_ii) / 2)); bad = outside the FP32 range
__device__ __forceinline__ float pow2_scale(double d, int &bad, int &sh) {
  sh = 0;
  if (d > 0.0 && d < 1e300) {
    int e = ilogb(d);
    e = (e >= 0) ? e / 2 : -((-e + 1) / 2);  // floor(log2(d) / 2)
    if (e > 120 || e < -120) {
      bad = 1;
      return 1.0f;
    }
    sh = -e;
    return ldexpf(1.0f, -e);
  }
  bad = 1;  // non-positive / NaN / huge diagonal: the FP64 path decides
  return 1.0f;
}

// ===========================================================================
// register path (n <= W <= 32); every segment of a warp runs every shuffle
// ===========================================================================

// FP64 factor + solve of RHS rows [r_from, m) -- plain path and fallback.
// Ls64: W x (W+1) doubles, rinv64: W doubles (segment-private shared).
template <int W>
__device__ int small_fp64_posv(bool active, int n, int m, int r_from, double *A, int lda, double *B,
                               int ldb, double *Ls64, double *rinv64)
{
  const int lane = threadIdx.x & (W - 1);
  double v[32];
  small_load<double, W, false>(n, active ? A : nullptr, lda, 0, active, v);
  const int fail = warp_chol_rot<double, W, false>(v, n, 0.0, Ls64, W + 1, rinv64);
  __syncwarp();
  if (active && lane < n) {
    const int ncol = fail ? fail - 1 : n;
    for (int c = 0; c <= lane && c < ncol; c++) A[(size_t)lane + (size_t)c * lda] = Ls64[lane * (W + 1) + c];
  }
  const bool solve = active && !fail;
  const int m_hi = warp_uniform_max_w(active ? m : 0, W);
  // Every lane of the warp runs the same trip count (small_llt_solve shuffles
  // over the full warp); r_from differs between the systems sharing a warp,
  // so each one solves only its own rows r_from..m-1.
  for (int r0 = 0; r0 < m_hi; r0++) {
    const bool go = solve && r0 >= r_from && r0 < m;
    double y = (go && lane < n) ? B[(size_t)r0 + (size_t)lane * ldb] : 0.0;
    y = small_llt_solve<double, W>(n, Ls64, rinv64, y);
    if (go && lane < n) B[(size_t)r0 + (size_t)lane * ldb] = y;
  }
  __syncwarp();
  return fail;
}

template <int W>
__device__ void small_mixed_posv(bool active, int n, int m, double *A, int lda, double *B, int ldb,
                                 unsigned char *base, int *info_out, int *iter_out)
{
  const int lane = threadIdx.x & (W - 1);
  double *Ls64 = reinterpret_cast<double *>(base);
  double *rinv64 = Ls64 + W * (W + 1);
  float *Ls = reinterpret_cast<float *>(rinv64 + W);
  float *rinv = Ls + W * (W + 1);
  float *scl = rinv + W;
  int bad = 0, shl = 0;
  float sc = 1.0f;
  if (active && lane < n) sc = pow2_scale(A[(size_t)lane + (size_t)lane * lda], bad, shl);
  scl[lane] = sc;
  float v[32];
  small_load<float, W, true>(n, active ? A : nullptr, lda, shl, active, v);
  // ||A||_inf from the staged values (|a_ij| = |as_ij| / (s_i s_j), exact)
#pragma unroll
  for (int c = 0; c < W; c++)
    if (c <= lane) Ls[lane * (W + 1) + c] = v[c];
  __syncwarp();
  float rs = 0.f;
  if (lane < n) {
    for (int c = 0; c <= lane; c++) rs += fabsf(Ls[lane * (W + 1) + c]) / scl[c];
    for (int j = lane + 1; j < n; j++) rs += fabsf(Ls[j * (W + 1) + lane]) / scl[j];
    rs /= sc;
  }
  const double anorm = (double)warp_max_width(rs, W) * (1.0 + 1e-6 * n);
  __syncwarp();
  const int fail = warp_chol_rot<float, W, true>(v, n, (float)n * 5.9604645e-08f, Ls, W + 1, rinv);
  __syncwarp();
  const int any_bad = seg_any(bad, W);
  bool need_fb = active && (fail != 0 || any_bad);
  int fb_code = need_fb ? -1 : 0, fb_from = 0, steps_used = 0;
  const double tol_conv = posv_eta_target(n);
  const int m_hi = warp_uniform_max_w(active ? m : 0, W);
  for (int r0 = 0; r0 < m_hi; r0++) {
    const bool go = active && !need_fb && r0 < m;
    const double b = (go && lane < n) ? B[(size_t)r0 + (size_t)lane * ldb] : 0.0;
    float y = small_llt_solve<float, W>(n, Ls, rinv, f64_to_f32_scaled(b, shl));
    double x = (double)(y * sc);
    double eta_prev = INFINITY;
    bool going = go, converged = false;
    int step = 0;
    while (__any_sync(0xffffffffu, going)) {
      const double r = small_residual<W>(n, A, lda, b, x, going);
      const double rm = warp_max_width(lane < n ? fabs(r) : 0.0, W);
      const double xm = warp_max_width(lane < n ? fabs(x) : 0.0, W);
      const double bm = warp_max_width(lane < n ? fabs(b) : 0.0, W);
      if (going) {
        const double den = anorm * xm + bm;
        const double eta = (den > 0.0) ? rm / den : (rm > 0.0 ? INFINITY : 0.0);
        if (eta <= tol_conv) {
          going = false;
          converged = true;
        } else if (!(eta <= 0.5 * eta_prev) || step >= PC_ITMAX ||
                   refine_too_slow(eta, eta_prev, tol_conv, n, 1)) {
          going = false;
        } else {
          eta_prev = eta;
        }
      }
      y = small_llt_solve<float, W>(n, Ls, rinv, going ? f64_to_f32_scaled(r, shl) : 0.0f);
      if (going) {
        x += (double)(y * sc);
        step++;
      }
    }
    if (go) {
      steps_used = max(steps_used, step);
      if (converged) {
        if (lane < n) B[(size_t)r0 + (size_t)lane * ldb] = x;
      } else {
        need_fb = true;
        fb_code = (step >= PC_ITMAX) ? -3 : -2;
        fb_from = r0;
      }
    }
  }
  int info = 0;
  if (__any_sync(0xffffffffu, need_fb))
    info = small_fp64_posv<W>(need_fb, n, m, fb_from, A, lda, B, ldb, Ls64, rinv64);
  if (active && lane == 0) {
    if (info_out) *info_out = need_fb ? info : 0;
    if (iter_out) *iter_out = need_fb ? fb_code : steps_used;
  }
}

// ===========================================================================
// panel path (n > 32, teams of whole warps)
// ===========================================================================

// FP64 factor + solve of RHS rows [r_from, m). Ps64: panel storage (shared or
// global scratch); Ld: 32x32 doubles; rinv, y: n doubles; red: 32 * nwarps
// doubles; flag: one int.
static __device__ int panel_fp64_posv(const Team &t, int n, int m, int r_from, double *A, int lda,
                               double *B, int ldb, double *Ps64, double *Ld, double *rinv, double *y,
                               double *red, int *flag)
{
  const PanelLayout L = make_layout(n);
  team_load_panels<double, false>(t, L, A, lda, Ps64, nullptr);
  t.sync();
  const int info = team_potrf_panel<double, false>(t, L, Ps64, Ld, rinv, 0.0, flag, true);
  team_store_panels<double>(t, L, Ps64, A, lda, info ? info - 1 : n);
  if (!info) {
    for (int r0 = r_from; r0 < m; r0++) {
      for (int i = t.tid; i < n; i += t.nt) y[i] = B[(size_t)r0 + (size_t)i * ldb];
      t.sync();
      team_llt_solve_panel<double>(t, L, Ps64, rinv, y, red, true);
      for (int i = t.tid; i < n; i += t.nt) B[(size_t)r0 + (size_t)i * ldb] = y[i];
      t.sync();
    }
  }
  t.sync();
  return info;
}

// FP32 solves of nr right-hand sides (ys, stride n) with an INV factor: with
// at least as many right-hand sides as warps, one warp per right-hand side
// (no team barriers); with fewer (but several), the whole team on all of
// them in one sweep when `wide` (wide_elems floats of team-shared scratch)
// holds the nr * nwarps * 32 partial sums (the sweep runs right-hand side q's
// diagonal blocks on warp q, so it needs nr < nwarps); otherwise the whole
// team on each in turn (a single warp is latency-bound on one solve).
static __device__ void team_solve_rhs(const Team &t, const PanelLayout &L, const float *Ps,
                                      const float *rinv, float *ys, int nr, float *red,
                                      float *wide, size_t wide_elems)
{
  const int nw = t.nwarps();
  if (nw > 1 && nr >= nw) {
    for (int q = t.warp(); q < nr; q += nw) warp_llt_solve_inv<float>(L, Ps, ys + (size_t)q * L.n);
    t.sync();
  } else if (nr >= 2 && nr < nw && nr <= PC_MR && (size_t)nr * nw * 32 <= wide_elems) {
    team_llt_solve_panel_inv_multi<float, PC_MR>(t, L, Ps, ys, nr, wide);
  } else {
    for (int q = 0; q < nr; q++) team_llt_solve_panel<float, true>(t, L, Ps, rinv, ys + (size_t)q * L.n, red, true);
  }
}

// Plain FP64 POSV of one team's system on the panel path; FAC_SMEM as for
// panel_mixed_posv (the FP64 factor in shared memory, else in the team's
// global scratch).
template <bool FAC_SMEM>
static __device__ void panel_plain_posv(const Team &t, int n, int m, double *A, int lda,
                                        double *B, int ldb, unsigned char *base,
                                        double *Ps_scratch, int *info_out)
{
  const PanelLayout L = make_layout(n);
  double *Ps = FAC_SMEM ? reinterpret_cast<double *>(base) : Ps_scratch;
  unsigned char *p = base + (FAC_SMEM ? L.total() * 8 : 0);
  double *Ld = reinterpret_cast<double *>(p); p += 32 * LDD * 8;
  double *rinv = reinterpret_cast<double *>(p); p += (size_t)n * 8;
  double *y = reinterpret_cast<double *>(p); p += (size_t)n * 8;
  double *red = reinterpret_cast<double *>(p); p += (size_t)32 * t.nwarps() * 8;
  int *flag = reinterpret_cast<int *>(p);
  const int inf_ = panel_fp64_posv(t, n, m, 0, A, lda, B, ldb, Ps, Ld, rinv, y, red, flag);
  if (info_out && t.tid == 0) *info_out = inf_;
}

// Plain FP64 POTRS of one team's system on the panel path: A holds the lower
// Cholesky factor L (as POTRF leaves it); every right-hand side row of B is
// replaced by the solution of X L L^T = B. FAC_SMEM as for panel_plain_posv.
template <bool FAC_SMEM>
static __device__ void panel_plain_potrs(const Team &t, int n, int m, const double *A, int lda,
                                         double *B, int ldb, unsigned char *base,
                                         double *Ps_scratch)
{
  const PanelLayout L = make_layout(n);
  double *Ps = FAC_SMEM ? reinterpret_cast<double *>(base) : Ps_scratch;
  unsigned char *p = base + (FAC_SMEM ? L.total() * 8 : 0);
  p += 32 * LDD * 8;  // diagonal-block buffer of the factorization, unused here
  double *rinv = reinterpret_cast<double *>(p); p += (size_t)n * 8;
  double *y = reinterpret_cast<double *>(p); p += (size_t)n * 8;
  double *red = reinterpret_cast<double *>(p);
  team_load_panels<double, false>(t, L, A, lda, Ps, nullptr);
  t.sync();
  for (int i = t.tid; i < n; i += t.nt) {
    const int pp = i / PNB, c = i - pp * PNB;
    rinv[i] = 1.0 / Ps[L.base(pp) + c + (size_t)c * L.ldp(pp)];
  }
  t.sync();
  for (int r0 = 0; r0 < m; r0++) {
    for (int i = t.tid; i < n; i += t.nt) y[i] = B[(size_t)r0 + (size_t)i * ldb];
    t.sync();
    team_llt_solve_panel<double>(t, L, Ps, rinv, y, red, true);
    for (int i = t.tid; i < n; i += t.nt) B[(size_t)r0 + (size_t)i * ldb] = y[i];
    t.sync();
  }
}

// Phase clock hooks of the mixed panel path for profiling builds; empty in
// the library.
#ifndef KGB_PHASE_BEGIN
#define KGB_PHASE_BEGIN(t)
#define KGB_PHASE_MARK(t, k)
#endif

// FAC_SMEM: the FP32 factor lives in the team's shared memory (else in its
// global scratch slot). A compile-time choice, so that every access to a
// shared-memory factor compiles to a shared-memory instruction rather than a
// generic one.
// tc (a team that is the whole CTA, else null): tensor-core trailing updates,
// operands staged in the solve / refinement region.
template <bool FAC_SMEM>
static __device__ void panel_mixed_posv(const Team &t, int n, int m, double *A, int lda, double *B,
                                 int ldb, unsigned char *base, float *Ps_scratch,
                                 double *Ps64_scratch, int *info_out, int *iter_out, TcCtx *tc,
                                 float route_c)
{
  const PanelLayout L = make_layout(n);
  const int nw = t.nwarps();
  float *Ps = FAC_SMEM ? reinterpret_cast<float *>(base) : Ps_scratch;
  unsigned char *p = base + (FAC_SMEM ? L.total() * 4 : 0);
  double *Ld64 = reinterpret_cast<double *>(p); p += 32 * LDD * 8;
  float *Ld = reinterpret_cast<float *>(Ld64);
  double *rinv64 = reinterpret_cast<double *>(p); p += (size_t)n * 8;
  float *rinv = reinterpret_cast<float *>(rinv64);
  float *scl = reinterpret_cast<float *>(p); p += (size_t)n * 4;
  int *sh = reinterpret_cast<int *>(p); p += (size_t)n * 4;
  p = base + (((size_t)(p - base) + 15) & ~(size_t)15);  // offset arithmetic keeps p shared
  unsigned char *region = p;  // ys, x, r, colsum; or the tensor-core staging
  float *ys = reinterpret_cast<float *>(p); p += (size_t)PC_MR * n * 4;
  p = base + (((size_t)(p - base) + 7) & ~(size_t)7);
  double *x = reinterpret_cast<double *>(p); p += (size_t)PC_MR * n * 8;
  double *r = reinterpret_cast<double *>(p); p += (size_t)PC_MR * n * 8;
  double *colsum = reinterpret_cast<double *>(p); p += (size_t)nw * n * 8;
  if (tc && (size_t)(p - region) < tc_stage_bytes(n)) p = region + tc_stage_bytes(n);
  if (tc) tc->stage = region;
  double *red = reinterpret_cast<double *>(p); p += (size_t)32 * nw * 8;
  int *flag = reinterpret_cast<int *>(p);
  KGB_PHASE_BEGIN(t);

  // 1. scales
  int bad = 0;
  for (int i = t.tid; i < n; i += t.nt) {
    int e;
    scl[i] = pow2_scale(A[(size_t)i + (size_t)i * lda], bad, e);
    sh[i] = e;
  }
  t.sync();
  // 2. stage As = S A S (FP32), factor
  team_load_panels<float, true>(t, L, A, lda, Ps, sh);
  t.sync();
  KGB_PHASE_MARK(t, 0);
  // ||A||_inf comes from the first residual (row sums of |A| on the spare
  // integer / FP32 issue slots of that FP64-bound pass); an underestimate
  // only makes the backward-error test stricter
  double anorm = -1.0;
  const float ftol = (float)n * 5.9604645e-08f;  // n * 2^-24
  const int fail = (t.nt >= 64)
                       ? team_potrf_panel_la<float, true, true>(t, L, Ps, Ld, rinv, ftol, flag, tc)
                       : team_potrf_panel<float, true, true>(t, L, Ps, Ld, rinv, ftol, flag, true);
  KGB_PHASE_MARK(t, 1);
  if (fail < 0) return;  // a tensor-core wait ran out: the launch stops, nothing is written
  const int any_bad = team_any(t, bad, reinterpret_cast<int *>(red));
  bool need_fb = fail != 0 || any_bad;
  int fb_code = need_fb ? -1 : 0, fb_from = 0, steps_used = 0;
  if (!need_fb && route_c > 0.f) {
    float rl = 0.f;
    for (int i = t.tid; i < n; i += t.nt) rl = fmaxf(rl, rinv[i]);
    const float rmax = team_max<float>(t, rl, reinterpret_cast<float *>(red));
    if (route_fp64(1.0f / (rmax * rmax), n, max(m, 1), route_c)) {
      need_fb = true;
      fb_code = -4;
    }
  }
  const double tol_conv = posv_eta_target(n);
  // 3. solve + refine, PC_MR right-hand sides at a time
  for (int r0 = 0; r0 < m && !need_fb; r0 += PC_MR) {
    const int nr = min(PC_MR, m - r0);
    // one warp per right-hand side for the FP32 solves
    for (int q = 0; q < nr; q++)
      for (int i = t.tid; i < n; i += t.nt)
        ys[q * n + i] = f64_to_f32_scaled(B[(size_t)(r0 + q) + (size_t)i * ldb], sh[i]);
    t.sync();
    team_solve_rhs(t, L, Ps, rinv, ys, nr, reinterpret_cast<float *>(red),
                   reinterpret_cast<float *>(colsum), (size_t)nw * n * 2);
    for (int q = 0; q < nr; q++)
      for (int i = t.tid; i < n; i += t.nt) x[q * n + i] = (double)(ys[q * n + i] * scl[i]);
    t.sync();
    KGB_PHASE_MARK(t, 2);
    double bmax[PC_MR];
    for (int q = 0; q < PC_MR; q++) {
      double bm = 0.0;
      if (q < nr)
        for (int i = t.tid; i < n; i += t.nt) bm = fmax(bm, fabs(B[(size_t)(r0 + q) + (size_t)i * ldb]));
      bmax[q] = team_max<double>(t, bm, red);
    }
    double eta_prev = INFINITY;
    bool converged = false;
    int step = 0;
    for (;;) {
      // the first residual of the call also sums the rows of |A| (right-hand
      // side 0 alone); the others go 2..4 at a time through one sweep of A
      int q = 0;
      if (anorm < 0.0 || nr == 1) {
        float *rowabs = (anorm < 0.0) ? ys : nullptr;  // ys is free here
        if (rowabs)
          for (int i = t.tid; i < n; i += t.nt) rowabs[i] = 0.f;
        team_residual_owner(t, n, A, lda, B + r0, ldb, x, r, colsum, rowabs);
        if (rowabs) {
          float an_local = 0.f;
          for (int i = t.tid; i < n; i += t.nt) an_local = fmaxf(an_local, rowabs[i]);
          anorm = (double)team_max<float>(t, an_local, reinterpret_cast<float *>(red));
        }
        q = 1;
      }
      switch (nr - q) {
        case 1: team_residual_owner(t, n, A, lda, B + (r0 + q), ldb, x + q * n, r + q * n, colsum, nullptr); break;
        case 2: team_residual_multi<2>(t, n, A, lda, B + (r0 + q), ldb, x + q * n, r + q * n); break;
        case 3: team_residual_multi<3>(t, n, A, lda, B + (r0 + q), ldb, x + q * n, r + q * n); break;
        case 4: team_residual_multi<4>(t, n, A, lda, B + (r0 + q), ldb, x + q * n, r + q * n); break;
        default: break;
      }
      KGB_PHASE_MARK(t, 3);
      double eta = 0.0;
      for (int q = 0; q < nr; q++) {
        double rm = 0.0, xm = 0.0;
        for (int i = t.tid; i < n; i += t.nt) {
          rm = fmax(rm, fabs(r[q * n + i]));
          xm = fmax(xm, fabs(x[q * n + i]));
        }
        // one reduction for both maxima: the residual is bounded by the
        // product, so pack (rm, xm) as two lanes of the scratch
        rm = team_max<double>(t, rm, red);
        xm = team_max<double>(t, xm, red);
        const double den = anorm * xm + bmax[q];
        const double e = (den > 0.0) ? rm / den : (rm > 0.0 ? INFINITY : 0.0);
        eta = (e > eta || e != e) ? e : eta;
      }
      if (eta <= tol_conv) {
        converged = true;
        break;
      }
      if (!(eta <= 0.5 * eta_prev) || step >= PC_ITMAX ||
          refine_too_slow(eta, eta_prev, tol_conv, n, nr))
        break;
      eta_prev = eta;
      for (int q = 0; q < nr; q++)
        for (int i = t.tid; i < n; i += t.nt) ys[q * n + i] = f64_to_f32_scaled(r[q * n + i], sh[i]);
      t.sync();
      team_solve_rhs(t, L, Ps, rinv, ys, nr, reinterpret_cast<float *>(red),
                   reinterpret_cast<float *>(colsum), (size_t)nw * n * 2);
      for (int q = 0; q < nr; q++)
        for (int i = t.tid; i < n; i += t.nt) x[q * n + i] += (double)(ys[q * n + i] * scl[i]);
      t.sync();
      KGB_PHASE_MARK(t, 4);
      step++;
    }
    steps_used = max(steps_used, step);
    if (converged) {
      for (int q = 0; q < nr; q++)
        for (int i = t.tid; i < n; i += t.nt) B[(size_t)(r0 + q) + (size_t)i * ldb] = x[q * n + i];
    } else {
      need_fb = true;
      fb_code = (step >= PC_ITMAX) ? -3 : -2;
      fb_from = r0;
    }
    t.sync();
  }
  // 4. FP64 fallback
  int info = 0;
  if (need_fb)
    info = panel_fp64_posv(t, n, m, fb_from, A, lda, B, ldb, Ps64_scratch, Ld64, rinv64, x, red,
                           flag);
  KGB_PHASE_MARK(t, 5);
  if (t.tid == 0) {
    if (info_out) *info_out = need_fb ? info : 0;
    if (iter_out) *iter_out = need_fb ? fb_code : steps_used;
  }
}

// ===========================================================================
// the persistent kernel
// ===========================================================================

__device__ __forceinline__ void item_decode(const ItemArgs &it, const PosvCfg &cfg, long long q,
                                            int &n, int &start, int &count) {
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
}

// Ask L2 for the lower triangles of the next item's matrices while the
// current item is being processed, so the next item's staging loads hit L2
// instead of waiting on HBM: one TMA bulk prefetch per column (rows j..n-1,
// contiguous), trimmed inward to 16-byte boundaries as the bulk operation
// requires, so it never reaches outside the column's own range.
__device__ __forceinline__ void prefetch_item(const SysArgs &sys, const ItemArgs &it,
                                              const PosvCfg &cfg, long long q) {
  int n, start, count;
  item_decode(it, cfg, q, n, start, count);
  const int pairs = count * n;  // (system, column) pairs
  for (int pc = threadIdx.x; pc < pairs; pc += blockDim.x) {
    const int k = pc / n, j = pc - k * n;
    const long long sidx = it.uniform ? (long long)start + k : (long long)it.perm[start + k];
    int m, lda, ldb;
    double *A, *B;
    sys.get(sidx, m, A, lda, B, ldb);
    const uintptr_t lo = reinterpret_cast<uintptr_t>(A + (size_t)j + (size_t)j * lda);
    const uintptr_t hi = reinterpret_cast<uintptr_t>(A + (size_t)n + (size_t)j * lda);
    const uintptr_t lo16 = (lo + 15) & ~(uintptr_t)15, hi16 = hi & ~(uintptr_t)15;
    if (hi16 > lo16)
      bulk_prefetch_l2(reinterpret_cast<const void *>(lo16), (uint32_t)(hi16 - lo16));
  }
}
// PATHS selects the code compiled in: bit 0 the register path (n <= 32), bit
// 1 the panel path (n > 32), bit 2 the tensor-core trailing update of the
// mixed panel path (a kernel without it carries none of its code, which
// measured 1.5% faster on batches whose orders stay at or below PC_TC_NMIN). A kernel holding one path only gets that path's
// register allocation (each path alone fits the register file; together they
// spill), so the binned launcher runs the two paths as two launches over the
// two item ranges: [0, *split_p) panel items, [*split_p, *nitems_p) register
// items.
template <bool MIXED, int PATHS = 3>
__global__ void __launch_bounds__(PC_NT, 1)
posv_persistent_kernel(SysArgs sys, ItemArgs it, OutArgs out, PosvCfg cfg, int smem_bytes)
{
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_item;
  __shared__ uint32_t s_tmem;
  __shared__ __align__(8) uint64_t s_tcbar;
  __shared__ int s_abort;
  // tensor-core trailing updates (mixed panel path): the CTA holds all TMEM
  // columns for the whole launch (one CTA per SM) and one mbarrier
  const bool use_tc = MIXED && (PATHS & 6) == 6 && out.tc != 0;
  if (threadIdx.x == 0) s_abort = 0;
  if (use_tc) {
    if (threadIdx.x < 32) {
      tmem_alloc(&s_tmem, TC_TMEM_COLS);
      tmem_relinquish();
    }
    if (threadIdx.x == 0) {
      mbar_init(&s_tcbar, 1);
      mbar_init_fence();
    }
    tc_fence_before_sync();
  }
  __syncthreads();
  if (use_tc) tc_fence_after_sync();
  TcCtx tcx{use_tc ? s_tmem : 0u, &s_tcbar, nullptr, &s_abort, out.status, 0u};
  long long first = 0, nitems;
  if (it.uniform) {
    const int spi = cfg.spi[pc_class(cfg, it.n_uniform)];
    nitems = (it.batch + spi - 1) / spi;
  } else {
    nitems = *it.nitems_p;
    if ((PATHS & 3) == 2) nitems = *it.split_p;
    if ((PATHS & 3) == 1) first = *it.split_p;
  }
  char *slot = out.scratch ? out.scratch + (size_t)blockIdx.x * out.slot_bytes : nullptr;

  if (threadIdx.x == 0) s_item = (int)first + atomicAdd(it.queue, 1);
  for (;;) {
    __syncthreads();
    const long long q = s_item;
    const bool stop = s_abort != 0;
    __syncthreads();
    if (q >= nitems || stop) break;
    // claim the next item now and warm L2 with its matrices
    if (threadIdx.x == 0) s_item = (int)first + atomicAdd(it.queue, 1);
    __syncthreads();
    if (s_item < nitems) prefetch_item(sys, it, cfg, s_item);
    int n, start, count;
    item_decode(it, cfg, q, n, start, count);
    const int c = pc_class(cfg, n);
    const int TS = cfg.ts[c];
    const int team_id = threadIdx.x / TS;
    const int nteams = PC_NT / TS;
    const bool item_tc = use_tc && nteams == 1 && n > 32;
    const bool fac_smem =
        (size_t)nteams * team_smem_bytes<MIXED>(n, TS, true, item_tc) <= (size_t)smem_bytes;
    const size_t tb = team_smem_bytes<MIXED>(n, TS, fac_smem, item_tc);
    const bool active = team_id < count;
    long long sidx = 0;
    int m = 0, lda = 1, ldb = 1;
    double *A = nullptr, *B = nullptr;
    if (active) {
      sidx = it.uniform ? (long long)start + team_id : (long long)it.perm[start + team_id];
      sys.get(sidx, m, A, lda, B, ldb);
    }
    unsigned char *base = smem + (size_t)team_id * tb;
    int *info_p = (active && out.info) ? out.info + sidx : nullptr;
    int *iter_p = (active && out.iter) ? out.iter + sidx : nullptr;
    if (n <= 32) {
      if constexpr ((PATHS & 1) != 0) {
      // register path: every segment of each warp runs, idle ones on no data
#define KGB_SMALL(WW)                                                                      \
  if (MIXED) {                                                                             \
    small_mixed_posv<WW>(active, n, m, A, lda, B, ldb, base, info_p, iter_p);              \
  } else {                                                                                 \
    double *ls_ = reinterpret_cast<double *>(base);                                        \
    const int inf_ = small_fp64_posv<WW>(active, n, m, 0, A, lda, B, ldb, ls_,             \
                                         ls_ + WW * (WW + 1));                             \
    if (info_p && (threadIdx.x & (WW - 1)) == 0) *info_p = inf_;                           \
  }
      if (TS == 8) {
        KGB_SMALL(8)
      } else if (TS == 16) {
        KGB_SMALL(16)
      } else {
        KGB_SMALL(32)
      }
#undef KGB_SMALL
      }
    } else if (active) {
      if constexpr ((PATHS & 2) != 0) {
      const Team t{(int)(threadIdx.x % TS), TS, 1 + team_id};
      const PanelLayout L = make_layout(n);
      // scratch slot: FP64 panels of every team, then FP32 ones
      double *P64s = slot ? reinterpret_cast<double *>(slot) + (size_t)team_id * L.total() : nullptr;
      float *P32s = slot ? reinterpret_cast<float *>(reinterpret_cast<double *>(slot) +
                                                       (size_t)nteams * L.total()) +
                               (size_t)team_id * L.total()
                         : nullptr;
      if (MIXED) {
        TcCtx *tcp = item_tc ? &tcx : nullptr;
        if (fac_smem)
          panel_mixed_posv<true>(t, n, m, A, lda, B, ldb, base, P32s, P64s, info_p, iter_p, tcp,
                                 cfg.route_c);
        else
          panel_mixed_posv<false>(t, n, m, A, lda, B, ldb, base, P32s, P64s, info_p, iter_p, tcp,
                                  cfg.route_c);
      } else {
        if (sys.op == 2) {
          if (fac_smem)
            panel_plain_potrs<true>(t, n, m, A, lda, B, ldb, base, P64s);
          else
            panel_plain_potrs<false>(t, n, m, A, lda, B, ldb, base, P64s);
        } else if (fac_smem) {
          panel_plain_posv<true>(t, n, m, A, lda, B, ldb, base, P64s, info_p);
        } else {
          panel_plain_posv<false>(t, n, m, A, lda, B, ldb, base, P64s, info_p);
        }
      }
      }
    }
    __syncthreads();
  }
  if (use_tc) {
    // every MMA was waited for (or its wait ran out and the loop stopped)
    tc_fence_before_sync();
    __syncthreads();
    tc_fence_after_sync();
    if (threadIdx.x < 32) tmem_dealloc(s_tmem, TC_TMEM_COLS);
  }
}

// Global scratch per CTA: FP64 + FP32 panel storage for every team of the
// largest item (mixed fallback; factors that do not fit in shared memory).
__host__ inline size_t posv_slot_bytes(const PosvCfg &cfg, int max_n) {
  size_t best = 0;
  for (int c = 0; c < PC_NCLS; c++) {
    const int nlo = c ? cfg.nmax[c - 1] + 1 : 1;
    const int nhi = min(cfg.nmax[c], max_n);
    if (nhi < nlo || nhi <= 32) continue;
    const size_t b = (size_t)(PC_NT / cfg.ts[c]) * make_layout(nhi).total() * 12;
    if (b > best) best = b;
  }
  return (best + 255) / 256 * 256;
}

}  // namespace kgb

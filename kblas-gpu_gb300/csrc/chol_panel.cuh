// chol_panel.cuh -- team-level blocked Cholesky, triangular solves and FP64
// residual on "panel" storage, for the persistent POSV kernels (n > 32).
//
// Storage of the lower triangle of one matrix of order n, block NB = 32:
// panel p (J = 32 p) holds rows J..n-1 of columns J..J+jb-1 (jb = min(32,
// n-J)), column-major with leading dimension ldp(p) = round_up(n - J, 4); the
// panels follow each other. Columns are contiguous and 16-byte aligned, so
// 4-row slices load as one 128-bit (FP32) or two 128-bit (FP64) accesses.
//
// Factorization (right-looking, one panel per step, 3 team barriers a step):
//   (a) the 32 x 32 diagonal block is factored in registers by one warp,
//       lane = row, columns broadcast by warp shuffles;
//   (b) the rows below it are solved against it, one row per thread, the
//       row held in registers and the block read as broadcast 128-bit loads
//       from a row-major copy;
//   (c) every later panel is updated with the new one: C -= P P^T, one 4 x 4
//       register tile per thread and step of k, i.e. two 128-bit shared
//       loads per 16 FMAs -- the one dense contraction of the factorization.
#pragma once

#include "device_util.cuh"
#include "tc_util.cuh"
#include "team.cuh"

namespace kgb {

// Sub-phase clock hooks for profiling builds; empty in the library.
#ifndef KGB_SUBPHASE_BEGIN
#define KGB_SUBPHASE_BEGIN(t)
#define KGB_SUBPHASE_MARK(t, k)
#define KGB_SUBPHASE_MARK1(t, k)
#endif

constexpr int PNB = 32;  // panel width
constexpr int LDD = 33;  // row stride of the diagonal-block copy (conflict free)

struct PanelLayout {
  int n, np;
  __host__ __device__ __forceinline__ int jb(int p) const { return min(PNB, n - p * PNB); }
  __host__ __device__ __forceinline__ int ldp(int p) const { return ((n - p * PNB) + 3) & ~3; }
  // element offset of panel p (sum of the sizes of the panels before it)
  __host__ __device__ __forceinline__ size_t base(int p) const {
    // sum_{q<p} round4(n - 32 q) * 32 ; closed form would need the rounding of
    // each term, a loop over <= 32 panels is cheap
    size_t s = 0;
    for (int q = 0; q < p; q++) s += (size_t)(((n - q * PNB) + 3) & ~3) * PNB;
    return s;
  }
  __host__ __device__ __forceinline__ size_t total() const { return base(np); }
};

__host__ __device__ __forceinline__ PanelLayout make_layout(int n) {
  PanelLayout L;
  L.n = n;
  L.np = (n + PNB - 1) / PNB;
  return L;
}

// ----------------------------------------------------------------------------
// Warp-register Cholesky of a jb x jb block (jb <= W <= 32), lane = row, in a
// segment of W lanes. Row `lane` arrives in v[0..31] (columns 0..jb-1). The
// column loop is rolled and the row registers rotate by one each step (the
// current column is always v[0]), so the code stays small: this runs on one
// warp while the rest of the team waits, and a fully unrolled 32 x 32 version
// is instruction-fetch bound. Column c of L is written to Lrow[lane * ldr + c]
// (row-major) and 1 / L(c,c) to rinv[c]. Every lane of the warp executes every
// shuffle (jb is uniform across the warp's segments); a failed segment keeps
// computing with a unit pivot, recording only its first failing column.
template <typename T, int W, bool CHECK_INF>
__device__ __forceinline__ int warp_chol_rot(T (&v)[32], int jb, T tol, T *Lrow, int ldr, T *rinv)
{
  const int lane = threadIdx.x & (W - 1);
  int fail = 0;
  for (int c = 0; c < jb; c++) {
    const T d = __shfl_sync(0xffffffffu, v[0], c, W);
    const bool ok = (d > tol) && (!CHECK_INF || d < T(INFINITY));
    if (!ok && fail == 0) fail = c + 1;
    T s, r;
    pivot_rs(ok ? d : T(1), s, r);
    const T l = (lane == c) ? s : v[0] * r;  // L(lane, c) for lane >= c
    if (lane >= c && lane < jb) Lrow[lane * ldr + c] = l;
    if (lane == c) rinv[c] = r;
#pragma unroll
    for (int k = 1; k < W; k++) {
      const T lk = __shfl_sync(0xffffffffu, l, (c + k) & (W - 1), W);  // L(c+k, c)
      if (lane >= c + k) v[k] -= l * lk;
    }
#pragma unroll
    for (int k = 1; k < W; k++) v[k - 1] = v[k];
    v[W - 1] = T(0);
  }
  return fail;
}

// The same factorization as warp_chol_rot<T, 32, CHECK_INF>, fully unrolled:
// the column index is a compile-time constant, so row `lane` stays in place
// (v[c] = A(lane, c)) and the updates need no register rotation and no lane
// predicate (entries above the diagonal take harmless values that are never
// stored or read back: every shuffle reads a lane at or below the current
// column). About 2 (31 - c) instructions per column c, ~21 KB of code: run by
// one warp per diagonal block, it still fits the instruction cache.
template <typename T, bool CHECK_INF>
__device__ __forceinline__ int warp_chol_unrolled(T (&v)[32], int jb, T tol, T *Lrow, int ldr,
                                                  T *rinv)
{
  const int lane = threadIdx.x & 31;
  int fail = 0;
#pragma unroll
  for (int c = 0; c < 32; c++) {
    if (c < jb) {
      const T d = __shfl_sync(0xffffffffu, v[c], c);
      const bool ok = (d > tol) && (!CHECK_INF || d < T(INFINITY));
      if (!ok && fail == 0) fail = c + 1;
      T sq, r;
      pivot_rs(ok ? d : T(1), sq, r);
      const T l = (lane == c) ? sq : v[c] * r;  // L(lane, c) for lane >= c
      v[c] = l;
      if (lane >= c && lane < jb) Lrow[lane * ldr + c] = l;
      if (lane == c) rinv[c] = r;
#pragma unroll
      for (int k = c + 1; k < 32; k++) v[k] -= l * __shfl_sync(0xffffffffu, l, k);
    }
  }
  return fail;
}

// Warp-level inverse of a factored diagonal block held in the panel's
// diagonal square (lower part, column-major, leading dimension ld a multiple
// of 4, 16-byte aligned columns): lane j computes column j of X = L^{-1} by a
// right-looking sweep in registers (x_i = b_i / L(i,i); b_r -= L(r,i) x_i for
// r > i), reading column i of L as broadcast 128-bit loads; then X replaces L
// in the lower part and X^T fills the strict upper part. The sweep is fully
// unrolled: it runs on every warp of a team at once (one block each), so the
// warps share the instruction fetch of the long straight-line code.
template <typename T>
__device__ __forceinline__ void warp_invert_diag(T *Pp, int ld, int jb, const T *rinvJ)
{
  const int lane = threadIdx.x & 31;
  T b[32];
#pragma unroll
  for (int i = 0; i < 32; i++) b[i] = (i == lane) ? T(1) : T(0);
#pragma unroll
  for (int i = 0; i < 32; i++) {
    if (i < jb) {
      const T xi = b[i] * rinvJ[i];
      b[i] = xi;
#pragma unroll
      for (int r0 = (i + 1) & ~3; r0 < 32; r0 += 4) {
        if (r0 < jb) {
          T q0, q1, q2, q3;
          if (sizeof(T) == 4) {
            const float4 q = *reinterpret_cast<const float4 *>(Pp + r0 + i * ld);
            q0 = q.x; q1 = q.y; q2 = q.z; q3 = q.w;
          } else {
            const double2 qa = *reinterpret_cast<const double2 *>(Pp + r0 + i * ld);
            const double2 qb = *reinterpret_cast<const double2 *>(Pp + r0 + 2 + i * ld);
            q0 = qa.x; q1 = qa.y; q2 = qb.x; q3 = qb.y;
          }
          if (r0 + 0 > i) b[r0 + 0] -= q0 * xi;
          if (r0 + 1 > i) b[r0 + 1] -= q1 * xi;
          if (r0 + 2 > i) b[r0 + 2] -= q2 * xi;
          if (r0 + 3 > i) b[r0 + 3] -= q3 * xi;
        }
      }
    }
  }
  __syncwarp();  // every lane is done reading L
  if (lane < jb) {
#pragma unroll
    for (int i = 0; i < 32; i++) {
      if (i < jb) {
        if (i > lane) Pp[lane + i * ld] = b[i];   // X^T, strict upper part
        if (i >= lane) Pp[i + lane * ld] = b[i];  // X, lower part
      }
    }
  }
  __syncwarp();
}

// Warp 0: factor the diagonal block of panel p in registers; L -> panel and
// -> Ldb (row-major copy, stride LDD); 1/L(c,c) -> rinv; *flag = failing
// column (global, 1-based) or 0. Inlined: as an out-of-line call (one copy
// of the ~21 KB of unrolled code for both panel factorizations) the mixed
// variable-size POSV measured ~1% slower.
template <typename T, bool CHECK_INF>
__device__ __forceinline__ void warp_factor_diag(const PanelLayout &L, int p, T *Ps, T *Ldb, T *rinv,
                                                 T tol, int *flag)
{
  const int lane = threadIdx.x & 31;
  const int J = p * PNB, jb = L.jb(p), ld = L.ldp(p);
  T *Pp = Ps + L.base(p);
  T v[32];
#pragma unroll
  for (int c = 0; c < 32; c++) v[c] = (c < jb && c <= lane && lane < jb) ? Pp[lane + c * ld] : T(0);
  const int f = warp_chol_unrolled<T, CHECK_INF>(v, jb, tol, Ldb, LDD, rinv + J);
  __syncwarp();
  for (int c = 0; c < jb; c++)
    if (lane >= c && lane < jb) Pp[lane + c * ld] = Ldb[lane * LDD + c];
  if (lane == 0) *flag = f ? J + f : 0;
  __syncwarp();
}

// ----------------------------------------------------------------------------
// Panel Cholesky of the team's matrix. Ps: panel storage (shared or global).
// Ld: 32 x 32 row-major scratch (shared) for the current diagonal block.
// rinv: n reciprocal pivots. flag: one int of team-shared scratch.
// Returns 1-based failing column or 0.
// INV: the diagonal 32 x 32 square of each panel receives the inverse of
// L_JJ instead of L_JJ (lower part), and its transpose in the strict upper
// part, so the triangular solves become two small matrix-vector products per
// panel (used by the FP32 refinement solves).
template <typename T, bool CHECK_INF, bool INV = false>
__device__ int team_potrf_panel(const Team &t, const PanelLayout &L, T *Ps, T *Ld, T *rinv, T tol,
                                int *flag, bool active)
{
  if (!active) return 0;
  const int lane = t.lane(), w = t.warp(), nw = t.nwarps();
  int fail = 0;
  for (int p = 0; p < L.np; p++) {
    const int J = p * PNB, jb = L.jb(p), ld = L.ldp(p);
    T *Pp = Ps + L.base(p);
    // (a) diagonal block, warp 0, lane = row: L -> Ld (row-major), then -> the
    // panel (with INV it is replaced by the inverse after the last step)
    if (w == 0) warp_factor_diag<T, CHECK_INF>(L, p, Ps, Ld, rinv, tol, flag);
    t.sync();
    fail = *flag;
    if (fail) break;
    // (b) rows below the diagonal block: x * L_JJ^T = p
    const int rows = L.n - J;
    for (int i = jb + t.tid; i < rows; i += t.nt) {
      T x[32];
#pragma unroll
      for (int c = 0; c < 32; c++) x[c] = (c < jb) ? Pp[i + c * ld] : T(0);
#pragma unroll
      for (int c = 0; c < 32; c++) {
        if (c < jb) {
          T s0 = x[c], s1 = T(0);
          const T *lrow = Ld + c * LDD;
#pragma unroll
          for (int q = 0; q < 32; q++) {
            if (q < c) {
              if (q & 1) s1 -= x[q] * lrow[q];
              else s0 -= x[q] * lrow[q];
            }
          }
          const T s = s0 + s1;
          x[c] = s * rinv[J + c];
        }
      }
#pragma unroll
      for (int c = 0; c < 32; c++)
        if (c < jb) Pp[i + c * ld] = x[c];
    }
    t.sync();
    // (c) trailing update of every later panel with this one, 4 x 4 tiles;
    // with INV, warp 0 meanwhile turns L_JJ into its inverse (it is not read
    // by the update, which only uses the rows below the diagonal block)
    {
      const int utid = t.tid, unt = t.nt;
      // count tiles per later panel: row tiles ceil(mq/4) x col tiles jbq/4 (jbq rounded up)
      int tile0 = 0;
      for (int q = p + 1; q < L.np; q++) {
        const int K = q * PNB, mq = L.n - K, jq = L.jb(q);
        const int rt = (mq + 3) >> 2, ct = (jq + 3) >> 2;
        const int ntile = rt * ct;
        T *Pq = Ps + L.base(q);
        const int ldq = L.ldp(q);
        const int start = ((utid - tile0) % unt + unt) % unt;
        for (int tt = start; tt < ntile; tt += unt) {
          const int c4 = tt / rt, r4 = tt - c4 * rt;
          const int i0 = r4 * 4, c0 = c4 * 4;  // rows K+i0.., cols c0.. of panel q
          if (i0 + 3 < c0) continue;           // entirely above the diagonal
          T acc[4][4];
#pragma unroll
          for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) acc[a][b] = T(0);
          const T *arow = Pp + (K - J) + i0;   // rows K+i0..K+i0+3 of panel p
          const T *brow = Pp + (K - J) + c0;   // rows K+c0..K+c0+3 of panel p
          for (int k = 0; k < jb; k++) {
            T a[4], b[4];
            if (sizeof(T) == 4) {
              const float4 av = *reinterpret_cast<const float4 *>(arow + (size_t)k * ld);
              const float4 bv = *reinterpret_cast<const float4 *>(brow + (size_t)k * ld);
              a[0] = av.x; a[1] = av.y; a[2] = av.z; a[3] = av.w;
              b[0] = bv.x; b[1] = bv.y; b[2] = bv.z; b[3] = bv.w;
            } else {
              const double2 a01 = *reinterpret_cast<const double2 *>(arow + (size_t)k * ld);
              const double2 a23 = *reinterpret_cast<const double2 *>(arow + (size_t)k * ld + 2);
              const double2 b01 = *reinterpret_cast<const double2 *>(brow + (size_t)k * ld);
              const double2 b23 = *reinterpret_cast<const double2 *>(brow + (size_t)k * ld + 2);
              a[0] = a01.x; a[1] = a01.y; a[2] = a23.x; a[3] = a23.y;
              b[0] = b01.x; b[1] = b01.y; b[2] = b23.x; b[3] = b23.y;
            }
#pragma unroll
            for (int x = 0; x < 4; x++)
#pragma unroll
              for (int y = 0; y < 4; y++) acc[x][y] += a[x] * b[y];
          }
#pragma unroll
          for (int y = 0; y < 4; y++) {
            if (c0 + y < jq) {
              T *col = Pq + (size_t)(c0 + y) * ldq + i0;
#pragma unroll
              for (int x = 0; x < 4; x++) col[x] -= acc[x][y];  // padding rows absorb the overhang
            }
          }
        }
        tile0 += ntile;
      }
    }
    t.sync();
  }
  if (INV && !fail) {
    // the diagonal blocks are independent now: each warp inverts its share
    for (int p = w; p < L.np; p += nw) warp_invert_diag<T>(Ps + L.base(p), L.ldp(p), L.jb(p), rinv + p * PNB);
    t.sync();
  }
  (void)lane;
  return fail;
}

// ----------------------------------------------------------------------------
// One 4 x 4 tile of the trailing update C -= P P^T: rows K+i0.., columns
// c0.. of the later panel q (Pq, ldq, jq columns) from rows of panel p.
template <typename T>
__device__ __forceinline__ void panel_tile_update(const T *Pp, int ld, int jb, int KmJ, int i0,
                                                  int c0, T *Pq, int ldq, int jq)
{
  T acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) acc[a][b] = T(0);
  const T *arow = Pp + KmJ + i0;
  const T *brow = Pp + KmJ + c0;
  for (int k = 0; k < jb; k++) {
    T a[4], b[4];
    if (sizeof(T) == 4) {
      const float4 av = *reinterpret_cast<const float4 *>(arow + (size_t)k * ld);
      const float4 bv = *reinterpret_cast<const float4 *>(brow + (size_t)k * ld);
      a[0] = av.x; a[1] = av.y; a[2] = av.z; a[3] = av.w;
      b[0] = bv.x; b[1] = bv.y; b[2] = bv.z; b[3] = bv.w;
    } else {
      const double2 a01 = *reinterpret_cast<const double2 *>(arow + (size_t)k * ld);
      const double2 a23 = *reinterpret_cast<const double2 *>(arow + (size_t)k * ld + 2);
      const double2 b01 = *reinterpret_cast<const double2 *>(brow + (size_t)k * ld);
      const double2 b23 = *reinterpret_cast<const double2 *>(brow + (size_t)k * ld + 2);
      a[0] = a01.x; a[1] = a01.y; a[2] = a23.x; a[3] = a23.y;
      b[0] = b01.x; b[1] = b01.y; b[2] = b23.x; b[3] = b23.y;
    }
#pragma unroll
    for (int x = 0; x < 4; x++)
#pragma unroll
      for (int y = 0; y < 4; y++) acc[x][y] += a[x] * b[y];
  }
#pragma unroll
  for (int y = 0; y < 4; y++) {
    if (c0 + y < jq) {
      T *col = Pq + (size_t)(c0 + y) * ldq + i0;
#pragma unroll
      for (int x = 0; x < 4; x++) col[x] -= acc[x][y];  // padding rows absorb the overhang
    }
  }
}


// The trailing update of step p by warps 1.. of a look-ahead team, FP32/FP64
// FMAs in 4 x 4 register tiles; the next panel's diagonal block (warp 0's)
// is skipped.
template <typename T>
__device__ __forceinline__ void trailing_update_ffma(const Team &t, const PanelLayout &L, int p, T *Ps)
{
  const int J = p * PNB, jb = L.jb(p), ld = L.ldp(p);
  const T *Pp = Ps + L.base(p);
  const int utid = t.tid - 32, unt = t.nt - 32;
  int tile0 = 0;
  for (int q = p + 1; q < L.np; q++) {
    const int K = q * PNB, mq = L.n - K, jq = L.jb(q);
    const int rt = (mq + 3) >> 2, ct = (jq + 3) >> 2;
    const int ntile = rt * ct;
    T *Pq = Ps + L.base(q);
    const int ldq = L.ldp(q);
    const int start = ((utid - tile0) % unt + unt) % unt;
    for (int tt = start; tt < ntile; tt += unt) {
      const int c4 = tt / rt, r4 = tt - c4 * rt;
      if (q == p + 1 && r4 < 8) continue;  // the next diagonal block: warp 0
      if (r4 * 4 + 3 < c4 * 4) continue;
      panel_tile_update<T>(Pp, ld, jb, K - J, r4 * 4, c4 * 4, Pq, ldq, jq);
    }
    tile0 += ntile;
  }
}

// ----------------------------------------------------------------------------
// Tensor-core trailing update (FP32 factor; a team that is the whole CTA).
//
// Step p's update of the trailing lower triangle, C -= P P^T with P the R =
// n - 32 (p + 1) rows of panel p below its diagonal block (K = 32), runs as
// BF16 products on the tensor cores with FP32 accumulation in TMEM. Each P
// entry is split into three BF16 terms, x = hi + mid + lo (to 2^-24 |x|), and
// the six products whose order is at most 2^-16 -- hi hi, hi mid, mid hi,
// hi lo, lo hi, mid mid -- are accumulated (the dropped terms are of order
// 2^-24 |x||y|): the hi + lo split of two BF16 terms extended by one term, so
// that the update stays close to FP32 accuracy and the refinement converges as
// with an FP32 FMA update (with two terms the factor would carry ~2^-16
// relative errors and need more FP64 refinement sweeps).
//
// Work split: warp 0 keeps its look-ahead (it updates and factors the next
// diagonal block with FP32 FMAs); warps 1.. stage P as the three BF16 terms
// in the no-swizzle K-major layout of tc_util.cuh, one of them issues the
// MMAs (M = 128 row tiles of the trailing matrix, N up to 256 columns per
// instruction, 2 x 6 instructions per tile and column chunk), and after the
// mbarrier reports completion every warp subtracts its TMEM lanes' results
// from the panel storage (lane = row: conflict-free column accesses).
// Row tiles start at multiples of 128; the last one starts at
// round_up8(R - 128) so that it ends at or past R (staged rows beyond R are
// zero and their results are dropped); tiles own disjoint row ranges. TMEM
// (512 columns) is filled with as many (tile, column chunk) pairs per round as
// fit; large orders take several rounds.
struct TcCtx {
  uint32_t tmem;         // TMEM address (lane 0, column 0) of the CTA's columns
  uint64_t *bar;         // MMA completion mbarrier (one arrival per round)
  unsigned char *stage;  // 3 x rows_pad x 64 bytes of shared memory, 16-byte aligned
  int *abort;            // shared flag: a bounded wait ran out
  int *status;           // device status word of the launch (may be null)
  uint32_t round;        // rounds completed (mbarrier phase parity)
};

// Rows of the staging buffer for a trailing matrix of R rows: at least one
// full M = 128 tile, and every column chunk a multiple of 16 rows.
__host__ __device__ __forceinline__ int tc_rows_pad(int R) {
  const int r16 = (R + 15) & ~15;
  return r16 > 128 ? r16 : 128;
}
// Shared-memory bytes of the staging buffer of a matrix of order n (step 0
// has the largest trailing matrix).
__host__ __device__ __forceinline__ size_t tc_stage_bytes(int n) {
  return n > PNB ? (size_t)3 * tc_rows_pad(n - PNB) * 64 : 0;
}

struct TcChunk {
  int m0, own_lo, own_hi, c0, nc;
};

// Enumerate the (row tile, column chunk) pairs of a trailing matrix of R rows
// in a fixed order; returns the number of pairs, fills `out` when non-null.
__device__ __forceinline__ int tc_chunk(int R, int idx, TcChunk *out) {
  const int ntiles = (R + 127) >> 7;
  int k = 0;
  for (int tile = 0; tile < ntiles; tile++) {
    const int last = (tile == ntiles - 1);
    int m0 = tile * 128;
    if (last && R > 128) m0 = min(m0, ((R - 128) + 7) & ~7);
    const int own_lo = tile * 128, own_hi = last ? R : (tile + 1) * 128;
    const int N = (own_hi + 15) & ~15;
    for (int c0 = 0; c0 < N; c0 += 256, k++) {
      if (k == idx && out) {
        out->m0 = m0;
        out->own_lo = own_lo;
        out->own_hi = own_hi;
        out->c0 = c0;
        out->nc = min(256, N - c0);
      }
    }
  }
  return k;
}

// Called by warps 1.. of a team that is the whole CTA (t.nt threads, t.nt >=
// 64), for step p < np - 1. Skips the next panel's diagonal block (rows and
// columns 0..31 of the trailing matrix): warp 0 updates it. Returns false if a
// bounded wait ran out (tc.abort is then set).
static __device__ bool team_trailing_tc(const Team &t, const PanelLayout &L, int p, float *Ps, TcCtx &tc)
{
  const int J = p * PNB, ld = L.ldp(p);
  const float *Pp = Ps + L.base(p);
  const int R = L.n - J - PNB;
  const int rows_pad = tc_rows_pad(R);
  const int utid = t.tid - 32, unt = t.nt - 32;
  const int w = t.warp();  // 1 .. nwarps-1
  const uint32_t term_bytes = (uint32_t)rows_pad * 64;
  // 1. stage the three BF16 terms of P (rows past R are zero)
  for (int e = utid; e < rows_pad * 4; e += unt) {
    const int k8 = e / rows_pad, i = e - k8 * rows_pad;
    uint32_t h[4], m[4], l[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const float x0 = (i < R) ? Pp[(PNB + i) + (size_t)(8 * k8 + 2 * q) * ld] : 0.f;
      const float x1 = (i < R) ? Pp[(PNB + i) + (size_t)(8 * k8 + 2 * q + 1) * ld] : 0.f;
      __nv_bfloat16 h0, m0, l0, h1, m1, l1;
      bf16_split3(x0, h0, m0, l0);
      bf16_split3(x1, h1, m1, l1);
      h[q] = pack_bf16(h0, h1);
      m[q] = pack_bf16(m0, m1);
      l[q] = pack_bf16(l0, l1);
    }
    const uint32_t off = (uint32_t)(i >> 3) * TC_SBO + (uint32_t)k8 * TC_LBO + (uint32_t)(i & 7) * 16;
    *reinterpret_cast<uint4 *>(tc.stage + off) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4 *>(tc.stage + term_bytes + off) = make_uint4(m[0], m[1], m[2], m[3]);
    *reinterpret_cast<uint4 *>(tc.stage + 2 * term_bytes + off) = make_uint4(l[0], l[1], l[2], l[3]);
  }
  fence_async_smem();
  asm volatile("bar.sync 15, %0;" ::"r"(unt) : "memory");
  // 2. rounds of MMAs + epilogue
  const int nchunks = tc_chunk(R, -1, nullptr);
  const uint32_t sbase = smem_addr(tc.stage);
  const int qd = w & 3;                     // TMEM lane quadrant of this warp
  const int nq = (qd == 0) ? 1 : 2;         // warps sharing it among warps 1..7
  const int qi = (qd == 0) ? 0 : (w >> 2);  // this warp's share
  // products (A term, B term), 0 = hi, 1 = mid, 2 = lo: the small ones first
  // and hi * hi last, so that the accumulator's alignment of each new partial
  // sum to the running total costs bits only at the final, large magnitude
  const int pa[6] = {1, 2, 0, 1, 0, 0}, pb[6] = {1, 0, 2, 0, 1, 0};
  bool ok = true;
  int c_first = 0;
  while (c_first < nchunks) {
    // chunks [c_first, c_end) fill at most TC_TMEM_COLS columns
    int c_end = c_first, cols = 0;
    while (c_end < nchunks) {
      TcChunk ch;
      tc_chunk(R, c_end, &ch);
      if (cols + ch.nc > TC_TMEM_COLS) break;
      cols += ch.nc;
      c_end++;
    }
    if (utid == 0) {
      tc_fence_after_sync();
      int tcol = 0;
      for (int c = c_first; c < c_end; c++) {
        TcChunk ch;
        tc_chunk(R, c, &ch);
        const uint32_t idesc = idesc_bf16_f32(128, ch.nc);
#pragma unroll
        for (int s = 0; s < 6; s++) {
#pragma unroll
          for (int hh = 0; hh < 2; hh++) {
            const uint32_t a = sbase + pa[s] * term_bytes + (uint32_t)(ch.m0 >> 3) * TC_SBO + hh * 256;
            const uint32_t b = sbase + pb[s] * term_bytes + (uint32_t)(ch.c0 >> 3) * TC_SBO + hh * 256;
            tc_mma_bf16(tc.tmem + tcol, smem_desc(a, TC_LBO, TC_SBO), smem_desc(b, TC_LBO, TC_SBO),
                        idesc, (s | hh) ? 1u : 0u);
          }
        }
        tcol += ch.nc;
      }
      tc_commit(tc.bar);
    }
    const bool done = mbar_wait_bounded(tc.bar, tc.round & 1u);
    tc.round++;
    if (!done) {
      ok = false;
      *tc.abort = 1;
      if (tc.status) atomicExch(tc.status, 1);
    }
    tc_fence_after_sync();
    if (done) {
      int tcol = 0;
      for (int c = c_first; c < c_end; c++) {
        TcChunk ch;
        tc_chunk(R, c, &ch);
        const int wlo = ch.m0 + 32 * qd;  // rows [wlo, wlo + 32) are this warp's lanes
        const int row = wlo + t.lane();
        const bool rok = row >= ch.own_lo && row < ch.own_hi && row < R;
        if (wlo + 32 > ch.own_lo && wlo < ch.own_hi && wlo < R) {
          for (int g = qi; g * 16 < ch.nc; g += nq) {
            const int cc = ch.c0 + g * 16;  // first trailing column of the group
            if (cc > wlo + 31) break;       // the rest lies above the diagonal
            if (wlo + 32 <= PNB && cc + 16 <= PNB) continue;  // warp 0's block
            float v[16];
            tmem_ld16(tc.tmem + ((uint32_t)(32 * qd) << 16) + (uint32_t)(tcol + g * 16), v);
            const int q = p + 1 + (cc >> 5);
            float *Pq = Ps + L.base(q);
            const int ldq = L.ldp(q);
            const int rq = row - 32 * (cc >> 5);  // row inside panel q
            if (rok) {
#pragma unroll
              for (int j = 0; j < 16; j++) {
                const int col = cc + j;
                if (col <= row && !(row < PNB && col < PNB))
                  Pq[rq + (size_t)(col & 31) * ldq] -= v[j];
              }
            }
          }
        }
        tcol += ch.nc;
      }
    }
    tc_fence_before_sync();
    asm volatile("bar.sync 15, %0;" ::"r"(unt) : "memory");
    if (*tc.abort) {
      // a wait ran out (the flag is read after the barrier, so every thread
      // decides alike): no more MMAs; wait once more, bounded, for the ones
      // in flight before the CTA stops and frees its TMEM
      mbar_wait_bounded(tc.bar, (tc.round - 1u) & 1u);
      return false;
    }
    c_first = c_end;
  }
  return ok;
}

// Panel Cholesky with look-ahead, for teams of at least two warps: while
// warps 1.. apply the trailing update of step p, warp 0 updates the next
// diagonal block first and factors it, so the 32-step dependent chain of each
// diagonal factorization overlaps the bulk update instead of stalling the
// team. Ld2 holds two row-major 32 x LDD copies (current and next block).
// INV: afterwards every diagonal square is replaced by its inverse (lower)
// and the transpose of the inverse (strict upper), one block per warp.
// tc (FP32 only, a team that is the whole CTA): the trailing update of warps
// 1.. runs on the tensor cores (team_trailing_tc); returns -1 if one of its
// bounded waits ran out.
template <typename T, bool CHECK_INF, bool INV>
__device__ int team_potrf_panel_la(const Team &t, const PanelLayout &L, T *Ps, T *Ld2, T *rinv,
                                   T tol, int *flag, TcCtx *tc = nullptr)
{
  const int lane = t.lane(), w = t.warp(), nw = t.nwarps();
  KGB_SUBPHASE_BEGIN(t);
  if (w == 0) warp_factor_diag<T, CHECK_INF>(L, 0, Ps, Ld2, rinv, tol, flag);
  t.sync();
  KGB_SUBPHASE_MARK(t, 8);
  int fail = *flag;
  for (int p = 0; p < L.np && !fail; p++) {
    const int J = p * PNB, jb = L.jb(p), ld = L.ldp(p);
    T *Pp = Ps + L.base(p);
    const T *Ld = Ld2 + (p & 1) * 32 * LDD;
    // (b) rows below the diagonal block: x * L_JJ^T = p
    const int rows = L.n - J;
    for (int i = jb + t.tid; i < rows; i += t.nt) {
      T x[32];
#pragma unroll
      for (int c = 0; c < 32; c++) x[c] = (c < jb) ? Pp[i + c * ld] : T(0);
#pragma unroll
      for (int c = 0; c < 32; c++) {
        if (c < jb) {
          T s0 = x[c], s1 = T(0);
          const T *lrow = Ld + c * LDD;
#pragma unroll
          for (int q = 0; q < 32; q++) {
            if (q < c) {
              if (q & 1) s1 -= x[q] * lrow[q];
              else s0 -= x[q] * lrow[q];
            }
          }
          x[c] = (s0 + s1) * rinv[J + c];
        }
      }
#pragma unroll
      for (int c = 0; c < 32; c++)
        if (c < jb) Pp[i + c * ld] = x[c];
    }
    t.sync();
    KGB_SUBPHASE_MARK(t, 9);
    // (c) trailing update; warp 0 takes the next diagonal block first
    if (w == 0) {
      if (p + 1 < L.np) {
        const int q = p + 1, K = q * PNB, mq = L.n - K, jq = L.jb(q);
        const int rt = min((mq + 3) >> 2, 8), ct = (jq + 3) >> 2;
        T *Pq = Ps + L.base(q);
        for (int tt = lane; tt < rt * ct; tt += 32) {
          const int c4 = tt / rt, r4 = tt - c4 * rt;
          if (r4 * 4 + 3 < c4 * 4) continue;
          panel_tile_update<T>(Pp, ld, jb, K - J, r4 * 4, c4 * 4, Pq, L.ldp(q), jq);
        }
        __syncwarp();
        KGB_SUBPHASE_MARK(t, 12);
        warp_factor_diag<T, CHECK_INF>(L, q, Ps, Ld2 + (q & 1) * 32 * LDD, rinv, tol, flag);
        KGB_SUBPHASE_MARK(t, 13);
      }
    } else if constexpr (sizeof(T) == 4) {
      KGB_SUBPHASE_MARK1(t, 15);
      if (tc && p + 1 < L.np) {
        team_trailing_tc(t, L, p, reinterpret_cast<float *>(Ps), *tc);
      } else {
        trailing_update_ffma<T>(t, L, p, Ps);
      }
      KGB_SUBPHASE_MARK1(t, 14);
    } else {
      trailing_update_ffma<T>(t, L, p, Ps);
    }
    t.sync();
    KGB_SUBPHASE_MARK(t, 10);
    if (tc && *tc->abort) return -1;
    fail = *flag;
  }
  if (INV && !fail) {
    for (int p = w; p < L.np; p += nw) warp_invert_diag<T>(Ps + L.base(p), L.ldp(p), L.jb(p), rinv + p * PNB);
    t.sync();
  }
  KGB_SUBPHASE_MARK(t, 11);
  (void)lane;
  return fail;
}

// ----------------------------------------------------------------------------
// y := L^{-T} L^{-1} y on panel storage (team of whole warps). red: nw * 32
// team-shared scratch.
// Sum over the 32 lanes of a warp for each of 32 columns at once: on entry
// lane i holds v[j] (contribution of lane i to column j); on exit lane j holds
// sum_i v[j]. Five butterfly rounds, 31 shuffles and 31 adds in total.
template <typename T>
__device__ __forceinline__ T warp_transpose_sum32(T (&v)[32])
{
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int lvl = 16; lvl >= 1; lvl >>= 1) {
    const bool hi = (lane & lvl) != 0;
#pragma unroll
    for (int k = 0; k < lvl; k++) {
      const T send = hi ? v[k] : v[k + lvl];
      const T keep = hi ? v[k + lvl] : v[k];
      v[k] = keep + __shfl_xor_sync(0xffffffffu, send, lvl);
    }
  }
  return v[0];
}

// y := L^{-T} L^{-1} y on panel storage (team of whole warps). red: nw * 32
// team-shared scratch.
//  forward, per panel: one warp sweeps the 32 x 32 diagonal block with its
//    row of L preloaded in registers (32 dependent steps of one shuffle and
//    one FMA), then each thread updates one row below (coalesced);
//  backward, per panel (last first): the off-diagonal products are summed per
//    column with lanes running down the rows (conflict-free reads) and one
//    warp transpose-sum, then one warp sweeps the diagonal block.
template <typename T, bool INV = false>
__device__ void team_llt_solve_panel(const Team &t, const PanelLayout &L, const T *Ps,
                                     const T *rinv, T *y, T *red, bool active)
{
  if (!active) return;
  const int lane = t.lane(), w = t.warp(), nw = t.nwarps();
  for (int p = 0; p < L.np; p++) {
    const int J = p * PNB, jb = L.jb(p), ld = L.ldp(p);
    const T *Pp = Ps + L.base(p);
    if (INV && w == 0) {
      // y_J := L_JJ^{-1} y_J: lane i takes row i of the inverse (lower part)
      T v0 = T(0), v1 = T(0);
      if (lane < jb) {
#pragma unroll
        for (int k = 0; k < 32; k += 2) {
          if (k <= lane && k < jb) v0 += Pp[lane + k * ld] * y[J + k];
          if (k + 1 <= lane && k + 1 < jb) v1 += Pp[lane + (k + 1) * ld] * y[J + k + 1];
        }
      }
      __syncwarp();
      if (lane < jb) y[J + lane] = v0 + v1;
    } else if (w == 0) {
      T lr[32];
#pragma unroll
      for (int c = 0; c < 32; c++) lr[c] = (c < lane && lane < jb) ? Pp[lane + c * ld] : T(0);
      T v = (lane < jb) ? y[J + lane] : T(0);
      const T ri = (lane < jb) ? rinv[J + lane] : T(0);
#pragma unroll
      for (int c = 0; c < 32; c++) {
        if (c < jb) {
          if (lane == c) v *= ri;
          const T yc = __shfl_sync(0xffffffffu, v, c);
          v -= lr[c] * yc;  // lr[c] = 0 unless lane > c
        }
      }
      if (lane < jb) y[J + lane] = v;
    }
    t.sync();
    for (int i = jb + t.tid; i < L.n - J; i += t.nt) {
      T s0 = T(0), s1 = T(0);
#pragma unroll 4
      for (int c = 0; c < jb; c += 2) {
        s0 += Pp[i + c * ld] * y[J + c];
        if (c + 1 < jb) s1 += Pp[i + (c + 1) * ld] * y[J + c + 1];
      }
      y[J + i] -= s0 + s1;
    }
    t.sync();
  }
  for (int p = L.np - 1; p >= 0; p--) {
    const int J = p * PNB, jb = L.jb(p), ld = L.ldp(p);
    const T *Pp = Ps + L.base(p);
    // partial[c] = sum over rows i >= J+jb of L(i, J+c) * y_i: warp w takes
    // row chunks w, w+nw, ... of 32 rows; lane = row
    T acc[32];
#pragma unroll
    for (int c = 0; c < 32; c++) acc[c] = T(0);
    for (int i0 = jb + w * 32; i0 < L.n - J; i0 += nw * 32) {
      const int i = i0 + lane;
      const T yi = (i < L.n - J) ? y[J + i] : T(0);
      const T *row = Pp + min(i, ld - 1);
#pragma unroll
      for (int c = 0; c < 32; c++)
        if (c < jb) acc[c] += row[(size_t)c * ld] * yi;
    }
    const T part = warp_transpose_sum32<T>(acc);
    red[w * 32 + lane] = part;
    t.sync();
    if (INV && w == 0) {
      // x_J := L_JJ^{-T} (y_J - partials): row i of the strict upper part
      // holds column i of the inverse
      T sv = (lane < jb) ? y[J + lane] : T(0);
      for (int q = 0; q < nw; q++) sv -= red[q * 32 + lane];
      if (lane < jb) y[J + lane] = sv;
      __syncwarp();
      T v0 = T(0), v1 = T(0);
      if (lane < jb) {
#pragma unroll
        for (int k = 0; k < 32; k += 2) {
          if (k >= lane && k < jb) v0 += Pp[lane + k * ld] * y[J + k];
          if (k + 1 >= lane && k + 1 < jb) v1 += Pp[lane + (k + 1) * ld] * y[J + k + 1];
        }
      }
      __syncwarp();
      if (lane < jb) y[J + lane] = v0 + v1;
    } else if (w == 0) {
      T lc[32];  // column `lane` of L_JJ: lc[c] = L(J+c, J+lane) for c > lane
#pragma unroll
      for (int c = 0; c < 32; c++) lc[c] = (c > lane && c < jb) ? Pp[c + lane * ld] : T(0);
      T v = (lane < jb) ? y[J + lane] : T(0);
      for (int q = 0; q < nw; q++) v -= red[q * 32 + lane];
      const T ri = (lane < jb) ? rinv[J + lane] : T(0);
#pragma unroll
      for (int c = 31; c >= 0; c--) {
        if (c < jb) {
          if (lane == c) v *= ri;
          const T xc = __shfl_sync(0xffffffffu, v, c);
          v -= lc[c] * xc;  // lc[c] = 0 unless c > lane
        }
      }
      if (lane < jb) y[J + lane] = v;
    }
    t.sync();
  }
}

// Y := L^{-T} L^{-1} Y for nr right-hand sides at once (y + q * n, q < nr,
// 2 <= nr < nwarps), on an INV factor, by the whole team: one sweep over the
// panels with the barriers of a single solve, every factor element loaded
// once per sweep step for all right-hand sides. Per right-hand side the
// arithmetic and its order are those of team_llt_solve_panel<T, true>, so
// the results are identical to nr solves in turn. The diagonal blocks run on
// warps 0..nr-1 in parallel, one right-hand side each. red: nr * nwarps * 32
// elements of team-shared scratch.
template <typename T, int NRMAX>
__device__ void team_llt_solve_panel_inv_multi(const Team &t, const PanelLayout &L, const T *Ps,
                                               T *y, int nr, T *red)
{
  const int lane = t.lane(), w = t.warp(), nw = t.nwarps();
  const int n = L.n;
  for (int p = 0; p < L.np; p++) {
    const int J = p * PNB, jb = L.jb(p), ld = L.ldp(p);
    const T *Pp = Ps + L.base(p);
    if (w < nr) {
      // y_J := L_JJ^{-1} y_J for right-hand side w
      T *yq = y + (size_t)w * n;
      T v0 = T(0), v1 = T(0);
      if (lane < jb) {
#pragma unroll
        for (int k = 0; k < 32; k += 2) {
          if (k <= lane && k < jb) v0 += Pp[lane + k * ld] * yq[J + k];
          if (k + 1 <= lane && k + 1 < jb) v1 += Pp[lane + (k + 1) * ld] * yq[J + k + 1];
        }
      }
      __syncwarp();
      if (lane < jb) yq[J + lane] = v0 + v1;
    }
    t.sync();
    for (int i = jb + t.tid; i < n - J; i += t.nt) {
      T s0[NRMAX], s1[NRMAX];
#pragma unroll
      for (int q = 0; q < NRMAX; q++) s0[q] = s1[q] = T(0);
#pragma unroll 4
      for (int c = 0; c < jb; c += 2) {
        const T a0 = Pp[i + c * ld];
        const T a1 = (c + 1 < jb) ? Pp[i + (c + 1) * ld] : T(0);
#pragma unroll
        for (int q = 0; q < NRMAX; q++) {
          if (q < nr) {
            const T *yq = y + (size_t)q * n;
            s0[q] += a0 * yq[J + c];
            if (c + 1 < jb) s1[q] += a1 * yq[J + c + 1];
          }
        }
      }
#pragma unroll
      for (int q = 0; q < NRMAX; q++)
        if (q < nr) y[(size_t)q * n + J + i] -= s0[q] + s1[q];
    }
    t.sync();
  }
  for (int p = L.np - 1; p >= 0; p--) {
    const int J = p * PNB, jb = L.jb(p), ld = L.ldp(p);
    const T *Pp = Ps + L.base(p);
    // partials of right-hand side q: warp w sums its row chunks (lane = row)
    for (int q = 0; q < nr; q++) {
      const T *yq = y + (size_t)q * n;
      T acc[32];
#pragma unroll
      for (int c = 0; c < 32; c++) acc[c] = T(0);
      for (int i0 = jb + w * 32; i0 < n - J; i0 += nw * 32) {
        const int i = i0 + lane;
        const T yi = (i < n - J) ? yq[J + i] : T(0);
        const T *row = Pp + min(i, ld - 1);
#pragma unroll
        for (int c = 0; c < 32; c++)
          if (c < jb) acc[c] += row[(size_t)c * ld] * yi;
      }
      const T part = warp_transpose_sum32<T>(acc);
      red[((size_t)q * nw + w) * 32 + lane] = part;
    }
    t.sync();
    if (w < nr) {
      // x_J := L_JJ^{-T} (y_J - partials) for right-hand side w
      T *yq = y + (size_t)w * n;
      const T *rq = red + (size_t)w * nw * 32;
      T sv = (lane < jb) ? yq[J + lane] : T(0);
      for (int q = 0; q < nw; q++) sv -= rq[q * 32 + lane];
      if (lane < jb) yq[J + lane] = sv;
      __syncwarp();
      T v0 = T(0), v1 = T(0);
      if (lane < jb) {
#pragma unroll
        for (int k = 0; k < 32; k += 2) {
          if (k >= lane && k < jb) v0 += Pp[lane + k * ld] * yq[J + k];
          if (k + 1 >= lane && k + 1 < jb) v1 += Pp[lane + (k + 1) * ld] * yq[J + k + 1];
        }
      }
      __syncwarp();
      if (lane < jb) yq[J + lane] = v0 + v1;
    }
    t.sync();
  }
}

// Stage the lower triangle of A (FP64, column-major, lda) into panel storage
// of type T (SCALE: FP32 a_ij * 2^(sh[i] + sh[j]), converted on the integer
// pipe, see f64_to_f32_scaled; sh = -e of the row scale 2^-e). One thread per
// panel row issues the 32 loads of the row before using any (32 loads in
// flight). Padding rows and the strict upper part of each diagonal block get
// zeros.
template <typename T, bool SCALE>
__device__ void team_load_panels(const Team &t, const PanelLayout &L, const double *__restrict__ A,
                                 int lda, T *Ps, const int *sh)
{
  for (int p = 0; p < L.np; p++) {
    const int J = p * PNB, jb = L.jb(p), ld = L.ldp(p);
    T *Pp = Ps + L.base(p);
    for (int ii = t.tid; ii < ld; ii += t.nt) {
      const int i = J + ii;
      const bool real = i < L.n;  // a row of the matrix (padding rows get zeros)
      const int si = (SCALE && real) ? sh[i] : 0;
      double a[32];
#pragma unroll
      for (int c = 0; c < 32; c++)
        a[c] = (real && c < jb && ii >= c) ? A[(size_t)i + (size_t)(J + c) * lda] : 0.0;
#pragma unroll
      for (int c = 0; c < 32; c++) {
        if (c < jb) {
          T v;
          if (SCALE) v = (T)f64_to_f32_scaled(a[c], si + sh[J + c]);
          else v = (T)a[c];
          Pp[ii + c * ld] = v;
        }
      }
    }
  }
}

// Write the factor held in panel storage back to A's lower triangle (columns
// 0..ncol-1).
template <typename T>
__device__ void team_store_panels(const Team &t, const PanelLayout &L, const T *Ps, double *A,
                                  int lda, int ncol)
{
  for (int p = 0; p < L.np; p++) {
    const int J = p * PNB, jb = L.jb(p), ld = L.ldp(p);
    if (J >= ncol) break;
    const T *Pp = Ps + L.base(p);
    const int rows = L.n - J;
    const int cols = min(jb, ncol - J);
    for (int e = t.tid; e < rows * cols; e += t.nt) {
      const int c = e / rows, ii = e - c * rows;
      if (ii >= c) A[(size_t)(J + ii) + (size_t)(J + c) * lda] = (double)Pp[ii + c * ld];
    }
  }
}

// |a| of an FP64 value as an FP32 number, from the high word only (integer
// pipe: the FP64 -> FP32 conversion shares the scarce FP64 pipe). The
// mantissa is truncated to 20 bits (a slight underestimate, relative error
// below 2^-20); values below the FP32 normal range give 0, above it +inf; a
// NaN gives NaN.
__device__ __forceinline__ float abs_f64_as_f32(double a)
{
  const unsigned hi = (unsigned)__double2hiint(a) & 0x7FFFFFFFu;
  const int e = (int)(hi >> 20);
  if (e >= 1023 + 128) return (e == 0x7FF && ((hi & 0xFFFFFu) | (unsigned)__double2loint(a))) ? __int_as_float(0x7FC00000) : __int_as_float(0x7F800000);
  if (e <= 1023 - 127) return 0.f;
  return __int_as_float((int)((unsigned)(e - 1023 + 127) << 23 | (hi & 0xFFFFFu) << 3));
}

// FP64 residual r = b - A x for one right-hand side; A symmetric, its lower
// triangle in global memory (column-major, lda). The rows are cut into blocks
// of 32; output block I needs the tiles (I, J), J <= I, read along their rows
// (lane = row I*32+lane, coalesced loads) and the tiles (K, I), K > I, read
// along their columns (lane = column I*32+lane: the mirrored upper part of row
// block I). A lane therefore accumulates its own row of the symmetric product
// in registers: no cross-lane reduction, no masked half of the diagonal tile
// (lane i takes a_ij from row i for j <= i and from column i for j > i), so
// the FP64 instruction count is exactly n^2 / 32 warp FMAs for n a multiple of
// 32. The nb^2 tile passes (nb = ceil(n / 32)) are split into equal contiguous
// ranges over the warps; each warp writes its partial rows to rowsum (nw x n
// doubles, team-shared), summed at the end.
// rowabs (may be NULL): rowabs[i] += sum_j |a_ij| (FP32, truncated from the
// FP64 high word, shared-memory atomics): the rows of the symmetric |A|,
// computed on the integer / FP32 pipes while the FP64 pipe does the products.
static __device__ void team_residual_owner(const Team &t, int n, const double *__restrict__ A,
                                           int lda, const double *__restrict__ b, int incb,
                                           const double *x, double *r, double *rowsum,
                                           float *rowabs)
{
  const int lane = t.lane(), w = t.warp(), nw = t.nwarps();
  const int nb = (n + 31) >> 5;
  const int units = nb * nb;
  const int u0 = (int)((long long)units * w / nw), u1 = (int)((long long)units * (w + 1) / nw);
  for (int i = t.tid; i < nw * n; i += t.nt) rowsum[i] = 0.0;
  t.sync();
  int u = u0;
  while (u < u1) {
    const int I = u / nb;
    const int uend = min(u1, (I + 1) * nb);
    const int row = I * 32 + lane;  // output row of this lane
    const bool rin = row < n;
    double s0 = 0.0, s1 = 0.0;
    float ra = 0.f;
    for (; u < uend; u++) {
      const int Tb = u - I * nb;  // tile column (Tb <= I) or tile row (Tb > I)
      const int c0 = Tb * 32;
      const double *xt = x + c0;
      const int cw = min(32, n - c0);
#pragma unroll
      for (int h = 0; h < 32; h += 16) {
        double a[16];
#pragma unroll
        for (int j = 0; j < 16; j++) {
          const int c = h + j, col = c0 + c;
          bool ok = rin && c < cw;
          size_t off;
          if (Tb < I || (Tb == I && c <= lane)) off = (size_t)row + (size_t)col * lda;  // a(row, col), lower
          else off = (size_t)col + (size_t)row * lda;                                   // a(col, row), lower
          a[j] = ok ? A[off] : 0.0;
        }
#pragma unroll
        for (int j = 0; j < 16; j += 2) {
          // x past n is not this vector's: mask it (0 * NaN would poison the sum)
          const double x0 = (h + j < cw) ? xt[h + j] : 0.0;
          const double x1 = (h + j + 1 < cw) ? xt[h + j + 1] : 0.0;
          s0 += a[j] * x0;
          s1 += a[j + 1] * x1;
        }
        if (rowabs) {
#pragma unroll
          for (int j = 0; j < 16; j++) ra += abs_f64_as_f32(a[j]);
        }
      }
    }
    if (rin) {
      rowsum[(size_t)w * n + row] = s0 + s1;
      if (rowabs) atomicAdd(&rowabs[row], ra);
    }
  }
  t.sync();
  for (int i = t.tid; i < n; i += t.nt) {
    double s = 0.0;
    for (int q = 0; q < nw; q++) s += rowsum[(size_t)q * n + i];
    r[i] = b[(size_t)i * incb] - s;
  }
  t.sync();
}

// The same residual for NR = 2..4 right-hand sides in one sweep over A: each
// element of A is loaded once and applied to every right-hand side, so a
// refinement step reads A once per group of right-hand sides rather than once
// per right-hand side (at n = 512 the systems in flight hold more of A than
// L2 does, and every extra sweep goes back to HBM). x, r: NR vectors of n
// (stride n); right-hand side q, element i at b[q + i * ldb].
// The tile ranges are split over nwr = min(nw, nb) warps, so that a range
// holds at least nb tiles and a row block is shared by at most two warps;
// each warp adds its partial rows into r (zeroed first) with shared-memory
// atomics. Two addends onto zero give the same sum in either order, so the
// result does not depend on which warp comes first.
template <int NR>
static __device__ void team_residual_multi(const Team &t, int n, const double *__restrict__ A,
                                           int lda, const double *__restrict__ b, int ldb,
                                           const double *x, double *r)
{
  const int lane = t.lane(), w = t.warp(), nw = t.nwarps();
  const int nb = (n + 31) >> 5;
  const int nwr = min(nw, nb);
  const int units = nb * nb;
  for (int i = t.tid; i < NR * n; i += t.nt) r[i] = 0.0;
  t.sync();
  if (w < nwr) {
    const int u0 = (int)((long long)units * w / nwr), u1 = (int)((long long)units * (w + 1) / nwr);
    int u = u0;
    while (u < u1) {
      const int I = u / nb;
      const int uend = min(u1, (I + 1) * nb);
      const int row = I * 32 + lane;  // output row of this lane
      const bool rin = row < n;
      double s[NR];
#pragma unroll
      for (int q = 0; q < NR; q++) s[q] = 0.0;
      for (; u < uend; u++) {
        const int Tb = u - I * nb;  // tile column (Tb <= I) or tile row (Tb > I)
        const int c0 = Tb * 32;
        const double *xt = x + c0;
        const int cw = min(32, n - c0);
#pragma unroll
        for (int h = 0; h < 32; h += 16) {
          double a[16];
#pragma unroll
          for (int j = 0; j < 16; j++) {
            const int c = h + j, col = c0 + c;
            const bool ok = rin && c < cw;
            size_t off;
            if (Tb < I || (Tb == I && c <= lane)) off = (size_t)row + (size_t)col * lda;  // a(row, col)
            else off = (size_t)col + (size_t)row * lda;  // a(col, row), the mirrored lower part
            a[j] = ok ? A[off] : 0.0;
          }
#pragma unroll
          for (int j = 0; j < 16; j++) {
            const bool xin = h + j < cw;  // x past n is not this vector's (0 * NaN)
#pragma unroll
            for (int q = 0; q < NR; q++) {
              const double xv = xin ? xt[(size_t)q * n + h + j] : 0.0;
              s[q] = fma(a[j], xv, s[q]);
            }
          }
        }
      }
      if (rin) {
#pragma unroll
        for (int q = 0; q < NR; q++) atomicAdd(&r[(size_t)q * n + row], s[q]);
      }
    }
  }
  t.sync();
  for (int i = t.tid; i < n; i += t.nt) {
#pragma unroll
    for (int q = 0; q < NR; q++) r[(size_t)q * n + i] = b[(size_t)q + (size_t)i * ldb] - r[(size_t)q * n + i];
  }
  t.sync();
}

// y := L^{-T} L^{-1} y on panel storage by ONE warp, for a factor whose
// diagonal squares hold the inverse of each diagonal block (lower part) and
// its transpose (strict upper part) -- the INV form of the panel
// factorizations. No team barrier is involved: the lanes take 32 rows at a
// time, the diagonal blocks become 32 x 32 matrix-vector products with the
// operand broadcast by shuffles, the updates below a block are dot products
// along panel rows (forward) and column sums folded by a warp transpose-sum
// (backward). Several right-hand sides run on several warps of a team at once.
template <typename T>
__device__ void warp_llt_solve_inv(const PanelLayout &L, const T *Ps, T *y)
{
  const int lane = threadIdx.x & 31;
  const int n = L.n;
  __syncwarp();
  for (int p = 0; p < L.np; p++) {
    const int J = p * PNB, jb = L.jb(p), ld = L.ldp(p);
    const T *Pp = Ps + L.base(p);
    const T v = (lane < jb) ? y[J + lane] : T(0);
    T o0 = T(0), o1 = T(0);
#pragma unroll
    for (int k = 0; k < 32; k += 2) {
      const T v0 = __shfl_sync(0xffffffffu, v, k), v1 = __shfl_sync(0xffffffffu, v, k + 1);
      if (k <= lane && lane < jb) o0 += Pp[lane + k * ld] * v0;
      if (k + 1 <= lane && lane < jb) o1 += Pp[lane + (k + 1) * ld] * v1;
    }
    const T yJ = o0 + o1;
    if (lane < jb) y[J + lane] = yJ;
    T yc[32];
#pragma unroll
    for (int c = 0; c < 32; c++) yc[c] = __shfl_sync(0xffffffffu, yJ, c);
    for (int i = J + jb + lane; i < n; i += 32) {
      const T *prow = Pp + (i - J);
      T s0 = T(0), s1 = T(0);
#pragma unroll
      for (int c = 0; c < 32; c += 2) {
        if (c < jb) s0 += prow[(size_t)c * ld] * yc[c];
        if (c + 1 < jb) s1 += prow[(size_t)(c + 1) * ld] * yc[c + 1];
      }
      y[i] -= s0 + s1;
    }
    __syncwarp();
  }
  for (int p = L.np - 1; p >= 0; p--) {
    const int J = p * PNB, jb = L.jb(p), ld = L.ldp(p);
    const T *Pp = Ps + L.base(p);
    T acc[32];
#pragma unroll
    for (int c = 0; c < 32; c++) acc[c] = T(0);
    for (int i0 = J + jb; i0 < n; i0 += 32) {
      const int i = i0 + lane;
      const T yi = (i < n) ? y[i] : T(0);
      const T *prow = Pp + min(i - J, ld - 1);
#pragma unroll
      for (int c = 0; c < 32; c++)
        if (c < jb) acc[c] += prow[(size_t)c * ld] * yi;
    }
    const T part = warp_transpose_sum32<T>(acc);
    const T v = (lane < jb) ? y[J + lane] - part : T(0);
    T o0 = T(0), o1 = T(0);
#pragma unroll
    for (int k = 0; k < 32; k += 2) {
      const T v0 = __shfl_sync(0xffffffffu, v, k), v1 = __shfl_sync(0xffffffffu, v, k + 1);
      if (k >= lane && k < jb) o0 += Pp[lane + k * ld] * v0;
      if (k + 1 >= lane && k + 1 < jb) o1 += Pp[lane + (k + 1) * ld] * v1;
    }
    __syncwarp();
    if (lane < jb) y[J + lane] = o0 + o1;
    __syncwarp();
  }
}

}  // namespace kgb

// posv_launch.h -- host-side planning of the persistent POSV launches:
// launch shape per size class, shared-memory budget, grid, workspace layout.
#pragma once

#include <stdlib.h>
#include <string.h>

#include "kblas_internal.h"
#include "launch_util.h"
#include "posv_core.cuh"
#include "tuning_table.h"

namespace kgb {

constexpr int PC_MAX_N = 1024;          // largest order the persistent kernels take
constexpr size_t PC_SMEM_BUDGET = 220 * 1024;

struct PosvPlan {
  PosvCfg cfg;
  int smem = 0;           // dynamic shared memory per CTA
  int grid = 0;           // persistent CTAs
  size_t slot_bytes = 0;  // global scratch per CTA
  int tc = 0;             // mixed panel path: tensor-core trailing updates for whole-CTA teams
};

// Tensor-core trailing updates are used by the mixed panel path when the
// launch holds orders above PC_TC_NMIN, a size class in range runs one team
// per CTA (the team then owns all of the SM's TMEM) and, with the BF16
// staging buffer, every class still fits the shared-memory budget with one
// CTA per SM; the launch then runs the kernel instantiation that carries the
// tensor-core code. KGB_NO_TC=1 in the environment turns them off (FP32 FMA
// updates), for comparisons.
static inline bool tc_disabled_by_env() {
  const char *e = getenv("KGB_NO_TC");
  return e && e[0] == '1';
}

// Process-wide override of the tuning table (set by the autotuner through
// kblasSetPosvTuning); zero entries mean "use the compiled table".
struct TuneOverride {
  int set[2] = {0, 0};
  PosvCfg cfg[2];
  int route_set = 0;
  float route_c = 0.f;
};
TuneOverride &tune_override();

static inline PosvCfg default_cfg(bool mixed) {
  PosvCfg c;
  const int mn[] = KGB_TUNE_MIXED_NMAX, mt[] = KGB_TUNE_MIXED_TS, ms[] = KGB_TUNE_MIXED_SPI;
  const int pn[] = KGB_TUNE_PLAIN_NMAX, pt[] = KGB_TUNE_PLAIN_TS, ps[] = KGB_TUNE_PLAIN_SPI;
  for (int k = 0; k < PC_NCLS; k++) {
    c.nmax[k] = mixed ? mn[k] : pn[k];
    c.ts[k] = mixed ? mt[k] : pt[k];
    c.spi[k] = mixed ? ms[k] : ps[k];
  }
  c.nmax[PC_NCLS - 1] = PC_MAX_N;
  c.route_c = KGB_TUNE_ROUTE_C;
  return c;
}

static inline PosvCfg current_cfg(bool mixed) {
  TuneOverride &o = tune_override();
  PosvCfg c = o.set[mixed ? 1 : 0] ? o.cfg[mixed ? 1 : 0] : default_cfg(mixed);
  c.route_c = o.route_set ? o.route_c : KGB_TUNE_ROUTE_C;
  return c;
}

// A class whose orders are all <= 32 runs the register path: team size W in
// {8, 16, 32} with W >= its largest order. A class with orders above 32 runs
// the panel path: whole warps (32..256); one that straddles 32 needs W = 32.
static inline bool cfg_valid(const PosvCfg &c) {
  for (int k = 0; k < PC_NCLS; k++) {
    const int ts = c.ts[k];
    const int nlo = k ? c.nmax[k - 1] + 1 : 1, nhi = c.nmax[k];
    if (k && nhi <= c.nmax[k - 1]) return false;
    if (!(ts == 8 || ts == 16 || ts == 32 || ts == 64 || ts == 128 || ts == 256)) return false;
    if (c.spi[k] < 1 || c.spi[k] * ts > PC_NT || (ts >= 64 && c.spi[k] > 15)) return false;
    if (nlo <= 32 && ts < (nhi < 32 ? nhi : 32)) return false;  // W >= n on the register path
    if (nlo <= 32 && nhi > 32 && ts != 32) return false;
    if (nhi > 32 && ts < 32) return false;
    if (ts < 32 && c.spi[k] * ts > PC_NT) return false;
  }
  return c.nmax[PC_NCLS - 1] >= PC_MAX_N;
}

// Launch plan of posv_persistent_kernel<MIXED, PATHS> for orders up to max_n:
// shared memory = the largest need over the size classes that kernel serves
// (register path: orders <= 32; panel path: orders > 32).
template <bool MIXED, int PATHS = 3>
static inline int plan_posv(KBlasHandle *h, int max_n, PosvPlan &pl) {
  pl.cfg = current_cfg(MIXED);
  if (!cfg_valid(pl.cfg)) return KBLAS_WrongConfig;
  const size_t budget = (size_t)(max_smem(h) < (int)PC_SMEM_BUDGET ? max_smem(h) : (int)PC_SMEM_BUDGET);
  // shared memory of the launch: the largest need over the classes in range
  auto need = [&](bool tc, size_t &out) -> bool {
    size_t smem = 0;
    for (int c = 0; c < PC_NCLS; c++) {
      const int nlo = c ? pl.cfg.nmax[c - 1] + 1 : 1;
      const int nhi = pl.cfg.nmax[c] < max_n ? pl.cfg.nmax[c] : max_n;
      if (nhi < nlo) continue;
      const int nteams = PC_NT / pl.cfg.ts[c];
      size_t b = 0;
      if ((PATHS & 1) && nlo <= 32) {
        const size_t b1 = (size_t)nteams * team_smem_bytes<MIXED>(nhi < 32 ? nhi : 32, pl.cfg.ts[c], true);
        if (b1 > b) b = b1;
      }
      if ((PATHS & 2) && nhi > 32) {
        const bool ctc = tc && nteams == 1;
        size_t b2 = (size_t)nteams * team_smem_bytes<MIXED>(nhi, pl.cfg.ts[c], true, ctc);
        if (b2 > budget) b2 = (size_t)nteams * team_smem_bytes<MIXED>(nhi, pl.cfg.ts[c], false, ctc);
        if (b2 > b) b = b2;
      }
      if (b > budget) return false;
      if (b > smem) smem = b;
    }
    out = smem;
    return true;
  };
  bool want_tc = false;
  if (MIXED && (PATHS & 2) && max_n > PC_TC_NMIN && !tc_disabled_by_env()) {
    for (int c = 0; c < PC_NCLS; c++) {
      const int nlo = c ? pl.cfg.nmax[c - 1] + 1 : 1;
      const int nhi = pl.cfg.nmax[c] < max_n ? pl.cfg.nmax[c] : max_n;
      if (nhi >= nlo && nhi > 32 && pl.cfg.ts[c] == PC_NT) want_tc = true;
    }
  }
  size_t smem = 0;
  if (want_tc && !need(true, smem)) want_tc = false;
  if (!want_tc && !need(false, smem)) return KBLAS_NotSupported;
  if (smem == 0) smem = 16;
  pl.smem = (int)smem;
  // the kernel instantiation launched: with the tensor-core code (PATHS bit
  // 2) only when the plan uses it
  auto occupancy = [&](bool tc, int bytes, int &per_sm) -> int {
    int st = KBLAS_Success;
    cudaError_t e = cudaSuccess;
    per_sm = 0;
    if constexpr (MIXED && (PATHS & 2) != 0) {
      if (tc) {
        auto kern = posv_persistent_kernel<MIXED, PATHS | 4>;
        st = set_smem(kern, bytes);
        if (st == KBLAS_Success) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, PC_NT, bytes);
      }
    }
    if (!tc) {
      auto kern = posv_persistent_kernel<MIXED, PATHS>;
      st = set_smem(kern, bytes);
      if (st == KBLAS_Success) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, PC_NT, bytes);
    }
    if (e != cudaSuccess || per_sm < 1) per_sm = 1;
    return st;
  };
  int per_sm = 0;
  int st = occupancy(want_tc, pl.smem, per_sm);
  if (st != KBLAS_Success) return st;
  // a CTA with tensor-core updates takes every TMEM column of its SM
  if (want_tc && per_sm > 1) {
    if (!need(false, smem)) return KBLAS_NotSupported;
    want_tc = false;
    pl.smem = (int)(smem ? smem : 16);
    st = occupancy(false, pl.smem, per_sm);
    if (st != KBLAS_Success) return st;
  }
  pl.tc = want_tc ? 1 : 0;
  pl.grid = h->sm_count * per_sm;
  pl.slot_bytes = (PATHS & 2) ? posv_slot_bytes(pl.cfg, max_n) : 0;
  return KBLAS_Success;
}

// Device workspace layout shared by the uniform mixed and the variable-size
// routines (offsets in bytes from the start of the handle's device data).
struct PosvWs {
  size_t header = 0;   // int[64]: [0] panel-path queue, [1] item count, [2] register-path
                       // queue, [3] panel items (items with n > 32 come first)
  size_t cnt = 0;      // int[max_n + 1]   systems per order n
  size_t off = 0;      // int[max_n + 1]   first slot of order n in perm
  size_t ioff = 0;     // int[max_n + 1]   first item of order n
  size_t cursor = 0;   // int[max_n + 1]
  size_t perm = 0;     // int[batch]
  size_t items = 0;    // int4[batch]
  size_t scratch = 0;  // grid * slot_bytes
  size_t total = 0;
};

static inline PosvWs posv_ws_layout(int max_n, long long batch, bool binned, const PosvPlan &pl) {
  PosvWs w;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t at = o;
    o += (bytes + 255) / 256 * 256;
    return at;
  };
  w.header = take(64 * sizeof(int));
  if (binned) {
    const size_t nb = (size_t)(max_n + 1) * sizeof(int);
    w.cnt = take(nb);
    w.off = take(nb);
    w.ioff = take(nb);
    w.cursor = take(nb);
    w.perm = take((size_t)batch * sizeof(int));
    w.items = take((size_t)batch * sizeof(int4));
  }
  w.scratch = take((size_t)pl.grid * pl.slot_bytes);
  w.total = o;
  return w;
}

}  // namespace kgb

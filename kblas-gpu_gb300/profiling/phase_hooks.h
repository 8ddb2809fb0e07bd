// phase_hooks.h -- clock64 phase timers for a profiling build of the library.
//
// The persistent POSV kernels carry KGB_PHASE_BEGIN / KGB_PHASE_MARK (mixed
// panel path: posv_core.cuh) and KGB_SUBPHASE_BEGIN / KGB_SUBPHASE_MARK (the
// look-ahead panel factorization: chol_panel.cuh), which compile to nothing
// in the library. phase_build.py force-includes this header into every unit
// of a separate build (libkblas_phase.so); there the first thread of each
// team adds the SM cycles since the previous mark to slot k of a device
// array and counts the visit in slot 16 + k. Each translation unit has its
// own array (no relocatable device code), so every unit registers a reader
// at load time and kgb_phase_all sums (or clears) all of them.
#pragma once
#include <cuda_runtime.h>

static __device__ unsigned long long kgb_phase_acc[32];

#define KGB_PHASE_TICK_(t, k, var)                                                       \
  do {                                                                                   \
    const long long now_ = clock64();                                                    \
    if ((t).tid == 0) {                                                                  \
      atomicAdd(&kgb_phase_acc[(k)], (unsigned long long)(now_ - var));                  \
      atomicAdd(&kgb_phase_acc[16 + (k)], 1ull);                                         \
    }                                                                                    \
    var = now_;                                                                          \
  } while (0)
#define KGB_PHASE_BEGIN(t) long long kgb_pt_ = clock64()
#define KGB_PHASE_MARK(t, k) KGB_PHASE_TICK_(t, k, kgb_pt_)
#define KGB_SUBPHASE_BEGIN(t) long long kgb_spt_ = clock64(), kgb_spt1_ = kgb_spt_
#define KGB_SUBPHASE_MARK(t, k) KGB_PHASE_TICK_(t, k, kgb_spt_)
// the same, counted by the team's thread 32 (the first lane of warp 1)
#define KGB_SUBPHASE_MARK1(t, k)                                                         \
  do {                                                                                   \
    const long long now_ = clock64();                                                    \
    if ((t).tid == 32) {                                                                 \
      atomicAdd(&kgb_phase_acc[(k)], (unsigned long long)(now_ - kgb_spt1_));            \
      atomicAdd(&kgb_phase_acc[16 + (k)], 1ull);                                         \
    }                                                                                    \
    kgb_spt1_ = now_;                                                                    \
  } while (0)

typedef int (*kgb_phase_fn)(unsigned long long *, int);
extern "C" __attribute__((weak)) kgb_phase_fn kgb_phase_fns[64] = {0};
extern "C" __attribute__((weak)) int kgb_phase_nfns = 0;

static int kgb_phase_rw(unsigned long long *buf, int clear) {
  if (clear) {
    unsigned long long z[32] = {0};
    return (int)cudaMemcpyToSymbol(kgb_phase_acc, z, sizeof z);
  }
  unsigned long long tmp[32];
  const int e = (int)cudaMemcpyFromSymbol(tmp, kgb_phase_acc, sizeof tmp);
  for (int i = 0; i < 32; i++) buf[i] += tmp[i];
  return e;
}
static int kgb_phase_reg_ = (kgb_phase_fns[kgb_phase_nfns++] = kgb_phase_rw, 0);

// buf: 32 slots, accumulated into (clear = 0), or every array zeroed (clear = 1).
extern "C" __attribute__((weak)) int kgb_phase_all(unsigned long long *buf, int clear) {
  int e = 0;
  for (int i = 0; i < kgb_phase_nfns; i++) e |= kgb_phase_fns[i](buf, clear);
  return e;
}

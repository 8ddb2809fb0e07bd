// team.cuh -- a "team" is the group of threads that owns one linear system
// inside a persistent CTA: either a slice of one warp (G lanes, G in
// {4, 8, 16}) or a set of whole warps synchronised by a named barrier.
#pragma once

#include <cuda_runtime.h>

namespace kgb {

struct Team {
  int tid;  // thread index inside the team
  int nt;   // team size (threads)
  int bar;  // named barrier id (1..15) for multi-warp teams
  __device__ __forceinline__ void sync() const {
    if (nt <= 32) {
      __syncwarp();
    } else {
      asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(nt) : "memory");
    }
  }
  __device__ __forceinline__ int lane() const { return tid & 31; }
  __device__ __forceinline__ int warp() const { return tid >> 5; }
  __device__ __forceinline__ int nwarps() const { return nt >= 32 ? nt >> 5 : 1; }
};

// Team-wide reductions through a shared scratch of at least nwarps() slots.
// Sub-warp teams reduce with width-limited shuffles inside their own lanes.
template <typename T>
__device__ __forceinline__ T warp_max_width(T v, int width) {
  for (int o = width >> 1; o > 0; o >>= 1) {
    T w = __shfl_xor_sync(0xffffffffu, v, o, width);
    v = (w > v || v != v) ? w : v;  // NaN-propagating max
  }
  return v;
}

template <typename T>
__device__ __forceinline__ T warp_sum_width(T v, int width) {
  for (int o = width >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, width);
  return v;
}

// max over the team; every thread of the team gets the result
template <typename T>
__device__ __forceinline__ T team_max(const Team &t, T v, T *scratch) {
  if (t.nt <= 32) return warp_max_width(v, t.nt);
  v = warp_max_width(v, 32);
  if (t.lane() == 0) scratch[t.warp()] = v;
  t.sync();
  T r = scratch[0];
  for (int w = 1; w < t.nwarps(); w++) {
    T x = scratch[w];
    r = (x > r || r != r) ? x : r;
  }
  t.sync();
  return r;
}

// logical OR over the team
__device__ __forceinline__ int team_any(const Team &t, int v, int *scratch) {
  if (t.nt <= 32) {
    const unsigned full = 0xffffffffu;
    unsigned ball = __ballot_sync(full, v);
    const int base = (t.nt < 32) ? (threadIdx.x & 31) / t.nt * t.nt : 0;
    unsigned mask = (t.nt == 32) ? full : (((1u << t.nt) - 1u) << base);
    return (ball & mask) != 0;
  }
  const int wv = __any_sync(0xffffffffu, v);
  if (t.lane() == 0) scratch[t.warp()] = wv;
  t.sync();
  int r = 0;
  for (int w = 0; w < t.nwarps(); w++) r |= scratch[w];
  t.sync();
  return r;
}

}  // namespace kgb

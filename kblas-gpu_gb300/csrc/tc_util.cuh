// tc_util.cuh -- the fifth-generation tensor-core (tcgen05) and mbarrier
// building blocks of the mixed-precision factorization, as inline PTX for
// sm_103a: tensor-memory (TMEM) allocation, shared-memory matrix descriptors,
// the BF16 x BF16 -> FP32 MMA issued by one thread, its completion through an
// mbarrier, and the TMEM -> register loads of the epilogue.
//
// Operand layout in shared memory (no swizzle, "K-major"): a matrix of R rows
// and K = 32 BF16 columns is stored as 8-row x 16-byte core matrices; row i,
// column k sits at byte
//     (i / 8) * TC_SBO + (k / 8) * TC_LBO + (i % 8) * 16 + (k % 8) * 2,
// with TC_LBO = 128 (next core matrix along K) and TC_SBO = 512 (next 8-row
// group). One MMA consumes K = 16 (two core matrices along K), so the second
// half of K starts 256 bytes further on.
//
// Every wait here is bounded: a wait that runs out reports failure to its
// caller, which records a status code and stops; nothing spins forever.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace kgb {

constexpr uint32_t TC_LBO = 128;   // bytes between core matrices adjacent along K
constexpr uint32_t TC_SBO = 512;   // bytes between 8-row groups (K = 32 per row)
constexpr int TC_TMEM_COLS = 512;  // TMEM columns a CTA takes (all of them)
constexpr long long TC_WAIT_LIMIT = 1ll << 22;  // polls before a wait gives up

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// ---- TMEM allocation (one full warp) ---------------------------------------
__device__ __forceinline__ void tmem_alloc(uint32_t *dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_addr(dst_smem)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

// ---- ordering between threads and the tensor core --------------------------
__device__ __forceinline__ void tc_fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy shared-memory writes -> visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ---- mbarrier ---------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Wait for the phase with the given parity to complete; false if it did not
// within TC_WAIT_LIMIT polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
  for (long long i = 0; i < TC_WAIT_LIMIT; i++) {
    if (mbar_try_wait(bar, parity)) return true;
    if (i > 64) __nanosleep(32);
  }
  return false;
}

// ---- bulk prefetch (TMA unit, no tensor map) --------------------------------
// Ask the TMA unit to bring [src, src + bytes) into L2 (a hint: nothing is
// waited for). src 16-byte aligned, bytes a positive multiple of 16.
__device__ __forceinline__ void bulk_prefetch_l2(const void *src, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

// ---- descriptors ------------------------------------------------------------
// Shared-memory matrix descriptor (tcgen05 form): start address, leading
// (K-direction) and stride (row-group) byte offsets, each >> 4; bits 46-47 =
// 1 (descriptor version of this architecture); base offset 0; no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::f16 with BF16 A and B (both K-major), FP32
// accumulator, dense, shape M x N (M = 128; N a multiple of 16, <= 256).
__host__ __device__ __forceinline__ uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4)                      // D format: F32
         | (1u << 7)                    // A format: BF16
         | (1u << 10)                   // B format: BF16
         | ((uint32_t)(N >> 3) << 17)   // N / 8
         | ((uint32_t)(M >> 4) << 24);  // M / 16
}

// D[tmem] (+)= A * B^T, issued by one thread.
__device__ __forceinline__ void tc_mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                            uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// The mbarrier receives one arrival once every MMA this thread issued so far
// has completed.
__device__ __forceinline__ void tc_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_addr(bar))
      : "memory");
}

// ---- TMEM -> registers --------------------------------------------------------
// 16 consecutive columns of this thread's TMEM lane (lane quadrant = warp % 4).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// ---- BF16 splitting ---------------------------------------------------------
// x = hi + mid + lo to within 2^-24 |x| (three BF16 terms, each rounded to
// nearest from the remainder of the previous ones).
__device__ __forceinline__ void bf16_split3(float x, __nv_bfloat16 &hi, __nv_bfloat16 &mid,
                                            __nv_bfloat16 &lo) {
  hi = __float2bfloat16_rn(x);
  const float r1 = x - __bfloat162float(hi);
  mid = __float2bfloat16_rn(r1);
  const float r2 = r1 - __bfloat162float(mid);
  lo = __float2bfloat16_rn(r2);
}

__device__ __forceinline__ uint32_t pack_bf16(__nv_bfloat16 a, __nv_bfloat16 b) {
  return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

}  // namespace kgb

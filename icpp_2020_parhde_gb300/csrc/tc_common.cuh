// tc_common.cuh -- helpers for the 5th-generation tensor-core kernels (tcgen05): mbarriers with bounded waits,
// TMEM allocation and loads, BF16 MMAs from shared-memory descriptors (K-major, no swizzle), and the
// three-part BF16 split of FP32 values (v = hi + mid + lo, 8 + 8 + 8 significand bits).
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

#include "common.cuh"

namespace {

constexpr int KC = 64;                     // K elements per staged operand block
constexpr int CORE_LBO = 128;              // bytes between core matrices adjacent in K
constexpr int CORE_SBO = (KC / 8) * 128;   // bytes between 8-row groups (1024)

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for the phase with the given parity; false on timeout, or when *fail is set by another thread.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint64_t timeout_ns,
                                          volatile int *fail) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_timer_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (fail && *fail) return false;
    if (global_timer_ns() - t0 > timeout_ns) return false;
  }
  return true;
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
// D[tmem] (+)= A[smem] * B[smem]^T, BF16 inputs, FP32 accumulator; accumulate == 0 overwrites D.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
// 16 consecutive accumulator columns of this thread's TMEM lane (the warp's 32-lane quarter), waited for.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor: K-major, no swizzle, LBO / SBO as above, descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(CORE_LBO >> 4) << 16) | ((uint64_t)(CORE_SBO >> 4) << 32) |
         (1ull << 46);
}
// Instruction descriptor, kind::f16: FP32 accumulator (bits 4-5 = 1), BF16 A and B (bits 7-9, 10-12 = 1),
// both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Byte offset of element (row, k) of a K-major operand in its stage buffer.
__device__ __forceinline__ uint32_t core_off(int row, int kgroup) {
  return (uint32_t)((row >> 3) * CORE_SBO + kgroup * CORE_LBO + (row & 7) * 16);
}

// Split 8 FP32 values (consecutive K) into three BF16 parts and store each as one 16-byte core-matrix row;
// pairs are converted together (the lower K index in the lower half of each 32-bit word).
__device__ __forceinline__ void store_split8(const float (&v)[8], uint8_t *hi, uint8_t *mid, uint8_t *lo) {
  uint32_t h[4], m[4], l[4];
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const __nv_bfloat162 hb = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
    const float2 hf = __bfloat1622float2(hb);
    const float ra = v[2 * i] - hf.x, rb = v[2 * i + 1] - hf.y;
    const __nv_bfloat162 mb = __floats2bfloat162_rn(ra, rb);
    const float2 mf = __bfloat1622float2(mb);
    const __nv_bfloat162 lb = __floats2bfloat162_rn(ra - mf.x, rb - mf.y);
    h[i] = *(const uint32_t *)&hb;
    m[i] = *(const uint32_t *)&mb;
    l[i] = *(const uint32_t *)&lb;
  }
  *(uint4 *)hi = make_uint4(h[0], h[1], h[2], h[3]);
  *(uint4 *)mid = make_uint4(m[0], m[1], m[2], m[3]);
  *(uint4 *)lo = make_uint4(l[0], l[1], l[2], l[3]);
}

}  // namespace

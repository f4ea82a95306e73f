// sg_tc.cuh -- 5th-generation tensor core primitives for sm_103a (inline PTX):
// tensor memory allocation, mbarriers, shared-memory matrix descriptors,
// tcgen05.mma (kind::f16, BF16 inputs, FP32 accumulate in tensor memory)
// and tcgen05.ld of the accumulators.
//
// Operand layout in shared memory (no swizzle, K-major): a tile of R rows x
// K elements is stored as 8x8 "core matrices" of 8 rows x 16 bytes each,
// 128 bytes contiguous; core matrices adjacent along K are 128 bytes apart
// (leading byte offset), groups of 8 rows are K/8 * 128 bytes apart (stride
// byte offset).  One tcgen05.mma consumes K = 16 (two core matrices).
//
// Every wait on an mbarrier is bounded: after about a second it gives up
// and the caller reports an error status instead of hanging.
#pragma once

#include <cuda_bf16.h>

#include <cstdint>

namespace sg {

__device__ inline uint32_t smem_u32(void const* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// byte offset of element (row, k) in a K-major core-matrix tile with K columns
__host__ __device__ constexpr uint32_t tile_off(uint32_t row, uint32_t k, uint32_t K) {
  return (row >> 3) * (K / 8) * 128 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

// tcgen05 shared-memory matrix descriptor: start address, leading and
// stride byte offsets (all >> 4), the descriptor version bits (46-48 =
// 0b001), no base offset, no swizzle.
__device__ inline uint64_t mat_desc(void const* base, uint32_t lbo, uint32_t sbo) {
  uint64_t const a = smem_u32(base);
  return ((a & 0x3FFFFull) >> 4) | (static_cast<uint64_t>((lbo & 0x3FFFFu) >> 4) << 16) |
         (static_cast<uint64_t>((sbo & 0x3FFFFu) >> 4) << 32) | (1ull << 46);
}
// descriptor of K-step `ks` (16 elements) of a K-major tile with K columns
__device__ inline uint64_t tile_desc(void const* base, uint32_t K, uint32_t ks) {
  return mat_desc(static_cast<uint8_t const*>(base) + ks * 256, 128, (K / 8) * 128);
}

// instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t M, uint32_t N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

// ---- mbarrier ----------------------------------------------------------------
__device__ inline void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ inline bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}
// Waits for the phase with parity `phase` to complete; false after ~1 s.
__device__ inline bool mbar_wait(uint64_t* bar, uint32_t phase) {
  long long const t0 = clock64();
  while (!mbar_try_wait(bar, phase))
    if (clock64() - t0 > 2000000000ll) return false;
  return true;
}

// ---- bulk copies (untiled TMA) --------------------------------------------------
// This thread's arrival on `bar`, which then also waits for `bytes` of copies.
__device__ inline void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// Copies `bytes` (a multiple of 16; both addresses 16-byte aligned) from
// global memory into this CTA's shared memory, completing on `bar`.
__device__ inline void bulk_g2s(void* dst, void const* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// ---- tensor memory -------------------------------------------------------------
// Allocates `ncols` columns (power of two, >= 32); one whole warp calls it.
__device__ inline void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ inline void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ inline void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ inline void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// makes this thread's shared-memory writes visible to the tensor cores
__device__ inline void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// D[tmem] (+)= A * B^T, one instruction (K = 16)
__device__ inline void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(acc)
      : "memory");
}
// arrives on `bar` once every MMA issued so far by this thread has completed
__device__ inline void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// 16 consecutive FP32 columns of this thread's row (lane) of tensor memory
__device__ inline void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ inline uint16_t bf16_bits(float f) { return __bfloat16_as_ushort(__float2bfloat16_rn(f)); }
__device__ inline float bf16_float(uint16_t b) { return __bfloat162float(__ushort_as_bfloat16(b)); }

}  // namespace sg

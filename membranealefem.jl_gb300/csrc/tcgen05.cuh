// tcgen05.cuh -- Blackwell (sm_100a / sm_103a) tensor-core and TMA helpers as
// inline PTX: Tensor Memory allocation, tcgen05.mma of kind::tf32 with
// shared-memory matrix descriptors, tcgen05.commit to an mbarrier, tcgen05.ld
// of the FP32 accumulators, and tiled TMA loads (cp.async.bulk.tensor) through
// a CUtensorMap.
//
// Operand layout used here (SWIZZLE_NONE, K-major): a core matrix is 8 rows x
// 16 bytes (8 rows x 4 TF32 values) stored as 128 contiguous bytes; the
// descriptor's leading byte offset (LBO) is the distance between the two core
// matrices one MMA reads along K (K = 8 TF32 = 32 bytes per instruction), its
// stride byte offset (SBO) the distance between core matrices 8 rows apart.
#pragma once

#include <cuda.h>  // CUtensorMap
#include <cuda_runtime.h>

#include <cstdint>

namespace mafem {
namespace tc {

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// ---- Tensor Memory (one warp executes each, all 32 lanes) ------------------------
// Allocates ncols columns (a power of two, 32..512) of the SM's 512 x 128-lane
// Tensor Memory and writes the base address to *holder (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t* holder, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(holder)), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
// order tcgen05 operations around a thread synchronisation (barrier or mbarrier)
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// ---- MMA -------------------------------------------------------------------------
// Shared-memory matrix descriptor (tcgen05 form): start address, LBO and SBO in
// 16-byte units, version 1 at bits 46-47, base offset 0, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}
// Instruction descriptor of kind::tf32: D FP32 (bits 4-5 = 1), A and B TF32
// (bits 7-9 and 10-12 = 2), both K-major (bits 15, 16 = 0), N / 8 at bits
// 17-22, M / 16 at bits 24-28.
__host__ __device__ constexpr uint32_t idesc_tf32(int m, int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}
// D (Tensor Memory, FP32) = A B + (accumulate ? D : 0); A M x 8 and B 8 x N
// TF32 from shared memory; issued by one thread.
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// The mbarrier receives one arrival when every MMA this thread issued before has completed.
__device__ __forceinline__ void commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(bar))
               : "memory");
}

// ---- accumulators -> registers ---------------------------------------------------
// 32 lanes x 8 consecutive columns starting at taddr (lane in bits 31-16,
// column in bits 15-0); lane i of the warp receives row (taddr lane + i).
__device__ __forceinline__ void ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr)
               : "memory");
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = __uint_as_float(r[k]);
}
__device__ __forceinline__ void wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// ---- TMA tiled load --------------------------------------------------------------
// 3-D box of `map` at coordinates (c0, c1, c2) into dst (shared, 128-byte
// aligned); the bytes complete on bar (whose expected transaction count the
// caller has raised).
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
          "r"(saddr(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(saddr(bar))
      : "memory");
}

}  // namespace tc
}  // namespace mafem

// Fifth-generation tensor cores (sm_100 family): tcgen05 MMA with the
// accumulator in tensor memory (TMEM), operands in shared memory described by
// 64-bit matrix descriptors, completion tracked by an mbarrier. Written from
// the PTX ISA's tcgen05 section; used by the guide network (k_guide.cu).
//
// Operand layout (both operands K-major, no swizzle): the canonical layout is
// built of core matrices of 8 rows x 16 bytes (8 halves), each stored as 128
// contiguous bytes. A row-major-by-K operand of R rows and K halves is kept as
//   byte offset(r, k) = (r / 8) * (K * 16) + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2
// so core matrices adjacent in K are 128 bytes apart (the descriptor's leading
// byte offset) and 8-row groups K * 16 bytes apart (its stride byte offset).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace rad {

__device__ __forceinline__ uint32_t SmemAddr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Byte offset of element (r, k) of a K-major operand with K halves per row.
__device__ __forceinline__ uint32_t TcOffset(uint32_t r, uint32_t k, uint32_t K) {
  return (r >> 3) * (K * 16u) + (k >> 3) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

// Shared-memory matrix descriptor: start address >> 4 (bits 0-13), leading
// byte offset >> 4 (bits 16-29), stride byte offset >> 4 (bits 32-45),
// descriptor version 1 (bits 46-47), base offset 0, no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t TcSmemDesc(uint32_t smemAddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((smemAddr >> 4) & 0x3fffu) | ((uint64_t)((lbo >> 4) & 0x3fffu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3fffu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: fp16 A and B, fp32 D, both K-major,
// N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t TcIdescF16(uint32_t M, uint32_t N) {
  return (1u << 4) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

// TMEM columns for this CTA (a power of two >= 32), by one full warp; the
// address is written to *slot (shared memory).
__device__ __forceinline__ void TcAlloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(SmemAddr(slot)),
               "r"(ncols));
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void TcDealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}

// D[tmem] (+)= A[smem] x B[smem]^T, issued by one thread.
__device__ __forceinline__ void TcMma(uint32_t dTmem, uint64_t aDesc, uint64_t bDesc, uint32_t idesc,
                                      bool accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dTmem),
      "l"(aDesc), "l"(bDesc), "r"(idesc), "r"(accumulate ? 1u : 0u));
}

// The mbarrier arrives once every tcgen05 operation this thread issued has completed.
__device__ __forceinline__ void TcCommit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   SmemAddr(mbar))
               : "memory");
}

__device__ __forceinline__ void TcFenceBefore() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void TcFenceAfter() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Shared-memory stores by threads become visible to the tensor cores' reads.
__device__ __forceinline__ void FenceProxyAsync() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void MbarInit(uint64_t* mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(SmemAddr(mbar)), "r"(count) : "memory");
}

// Waits until the phase with this parity has completed, for at most `limit`
// polls; returns false if it gave up.
__device__ __forceinline__ bool MbarWait(uint64_t* mbar, uint32_t parity, uint32_t limit) {
  const uint32_t a = SmemAddr(mbar);
  for (uint32_t i = 0; i < limit; i++) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// 16 consecutive fp32 columns of this thread's TMEM lane (32x32b shape: a warp
// reads the 32 lanes of its quarter of TMEM, warp w % 4 -> lanes 32 (w % 4) ..).
__device__ __forceinline__ void TcLoad16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  // the load and its completion wait in one statement: the registers are valid after the wait
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

}  // namespace rad

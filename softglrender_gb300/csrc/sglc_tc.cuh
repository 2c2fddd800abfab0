// Blackwell (sm_103a) tensor-core plumbing for the neural shader: tcgen05 MMA issued by one thread
// with operands in shared memory and the FP32 accumulator in tensor memory (TMEM), mbarrier
// completion, TMEM allocation and the TMEM -> register epilogue loads. Inline PTX only.
//
// Operand tiles use the SWIZZLE_NONE canonical layout built from 8x8 bf16 "core matrices" (8 rows of
// 16 bytes, 128 contiguous bytes). A tile of R rows x C columns (C a multiple of 8) stores core
// (rb, cb) = rows 8rb..8rb+7, columns 8cb..8cb+7 at byte offset (rb * C/8 + cb) * 128, row r % 8 at
// 16 * (r % 8), column c % 8 at 2 * (c % 8). The same bytes serve as a K-major operand (rows = M or
// N, columns = K: leading byte offset 128 between core matrices along K, stride byte offset C/8 * 128
// between 8-row groups along M/N) and as an MN-major operand (columns = M or N, rows = K: leading
// byte offset C/8 * 128 between 8-row groups along K, stride byte offset 128 between core matrices
// along M/N).
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace sglc {
namespace tc {

// byte offset of element (r, c) inside a core-matrix tile with C columns
__host__ __device__ constexpr uint32_t tileOffset(int r, int c, int C) {
  return (uint32_t) (((r >> 3) * (C >> 3) + (c >> 3)) * 128 + (r & 7) * 16 + (c & 7) * 2);
}

__device__ __forceinline__ uint32_t smemAddr(const void *p) {
  return (uint32_t) __cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor (tcgen05 format: version 1 at bits 46-47, SWIZZLE_NONE)
__device__ __forceinline__ uint64_t smemDesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t) ((addr & 0x3FFFFu) >> 4) | ((uint64_t) ((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t) ((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: BF16 A and B, FP32 accumulator, M x N, A/B K- or MN-major
__host__ __device__ constexpr uint32_t instrDesc(int M, int N, bool aMN, bool bMN) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((aMN ? 1u : 0u) << 15) | ((bMN ? 1u : 0u) << 16) |
         ((uint32_t) (N >> 3) << 17) | ((uint32_t) (M >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t dTmem, uint64_t aDesc, uint64_t bDesc, uint32_t idesc, bool accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dTmem),
      "l"(aDesc), "l"(bDesc), "r"(idesc), "r"((uint32_t) accumulate)
      : "memory");
}

// arrive once on the mbarrier when every MMA this thread issued so far has completed
__device__ __forceinline__ void commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smemAddr(bar))
               : "memory");
}

__device__ __forceinline__ void fenceBefore() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fenceAfter() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes become visible to the tensor core (async proxy)
__device__ __forceinline__ void fenceProxyAsync() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void barInit(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Bounded wait for the mbarrier phase with the given parity to complete. Returns false (and the
// caller records an error) after `limit` polls instead of spinning forever.
__device__ __forceinline__ bool barWait(uint64_t *bar, uint32_t parity, uint32_t limit = 1u << 24) {
  uint32_t a = smemAddr(bar);
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

// TMEM allocation: one full warp allocates `cols` columns (a power of two >= 32) and writes the
// base address to shared memory; the same warp frees them.
__device__ __forceinline__ void tmemAlloc(uint32_t *dst, uint32_t cols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(dst)), "r"(cols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmemFree(uint32_t base, uint32_t cols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base), "r"(cols) : "memory");
}

// Each thread of the warp reads 16 consecutive FP32 columns of its own TMEM lane
// (lane = 32 * (warp % 4) + laneid, encoded by the caller in bits 16-31 of taddr).
__device__ __forceinline__ void ld16(uint32_t taddr, float *v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}
// 32 consecutive FP32 columns of the thread's TMEM lane in one load (complete after ldWait)
__device__ __forceinline__ void ld32(uint32_t taddr, float *v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void ldWait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ uint32_t packBf16(float a, float b) {
  uint32_t lo = (uint32_t) __bfloat16_as_ushort(__float2bfloat16_rn(a));
  uint32_t hi = (uint32_t) __bfloat16_as_ushort(__float2bfloat16_rn(b));
  return lo | (hi << 16);
}

}  // namespace tc
}  // namespace sglc

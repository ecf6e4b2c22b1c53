// tc05.cuh — fifth-generation tensor-core primitives for sm_103a in inline PTX:
// tensor-memory (TMEM) allocation, shared-memory matrix descriptors, tcgen05.mma
// (kind::f16, BF16 inputs, FP32 accumulation, one issuing thread per CTA), commit
// to an mbarrier, bounded mbarrier waits and TMEM loads.
//
// Operand layout: every operand is K-major without swizzling, stored as 8 x 16-byte
// core matrices (8 rows x 8 BF16).  Element (r, k) of an R x K operand sits at byte
//   (r / 8) * (K * 16) + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2,
// so core matrices adjacent in K are 128 bytes apart (the descriptor's leading
// byte offset) and 8-row groups are K * 16 bytes apart (its stride byte offset).
// One MMA consumes K = 16, i.e. two core-matrix columns: slice s starts 256 * s
// bytes into the operand.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ckr {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Byte offset of element (r, k) in a K-major R x K BF16 operand.
__host__ __device__ __forceinline__ uint32_t kmaj(uint32_t r, uint32_t k, uint32_t K) {
  return (r >> 3) * (K * 16u) + (k >> 3) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

// Shared-memory matrix descriptor (no swizzle) for K-slice `s` of a K-major
// operand with K columns starting at shared address `base`.
__device__ __forceinline__ uint64_t sdesc(uint32_t base, uint32_t K, uint32_t s) {
  const uint32_t start = base + 256u * s;
  const uint64_t lbo = 128u >> 4, sbo = (K * 16u) >> 4;
  return (uint64_t)((start >> 4) & 0x3FFFu) | (lbo << 16) | (sbo << 32) | (1ull << 46);
}

// Instruction descriptor: D FP32, A and B BF16, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t M, uint32_t N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

// ---- TMEM allocation (one warp, all lanes) ----
__device__ __forceinline__ void tmem_alloc(uint32_t *dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Generic-proxy shared-memory writes made visible to the tensor core (async proxy).
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// ---- MMA ----
// D[tmem] (+)= A * B^T with A M x 16 and B N x 16 slices given by descriptors.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}
// Arrive on the mbarrier once every MMA issued so far by this thread has completed.
__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

// ---- mbarrier ----
__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// A bounded wait gives up after this long whatever its poll count: one try_wait may
// suspend the thread for an implementation-defined time, so a count alone does not
// bound the wait in time.
constexpr uint64_t kMbarWaitNs = 1000000000ull;  // 1 s; an MMA chain takes microseconds

// Waits for the phase with parity `parity` to complete; gives up after `tries`
// polls or kMbarWaitNs (returns false) so that a lost arrival cannot hang the GPU.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, uint32_t tries) {
  const uint64_t t0 = globaltimer_ns();
  for (uint32_t i = 0; i < tries; ++i) {
    if ((i & 255u) == 255u && globaltimer_ns() - t0 > kMbarWaitNs) return false;
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// ---- TMEM -> registers: 32 consecutive FP32 columns of this thread's lane ----
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc
}  // namespace ckr

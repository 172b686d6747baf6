/*
 * Fifth-generation tensor-core primitives for sm_103a, written as inline PTX:
 * TMEM allocation, tcgen05.mma (kind::f16, BF16 operands, FP32 accumulate,
 * A and B from shared memory, D in tensor memory), completion through an
 * mbarrier, and tcgen05.ld of the accumulator rows.
 *
 * Operand layout: K-major without swizzle.  A [rows x K] BF16 tile is stored
 * as 8 x 8 "core matrices" of 128 contiguous bytes (8 rows of 16 bytes);
 * element (row, k) lives at byte
 *     (row / 8) * SBO + (k / 8) * LBO + (row % 8) * 16 + (k % 8) * 2
 * with LBO = 128 (next core matrix along K) and SBO = K / 8 * 128 (next
 * group of 8 rows).  One MMA consumes K = 16, i.e. two core matrices along
 * K, so successive MMAs of a K loop advance the start address by 256 bytes.
 *
 * Every wait is bounded: a wait that runs out reports failure to the caller,
 * which records an error instead of hanging.
 */
#ifndef XMIMSIM_GB300_UMMA_CUH
#define XMIMSIM_GB300_UMMA_CUH

#include <cstdint>

namespace xmi {
namespace umma {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

/* byte offset of element (row, k) of a K-major tile with K columns */
__host__ __device__ __forceinline__ uint32_t kmajor_offset(int row, int k, int K) {
  return (uint32_t)((row >> 3) * (K >> 3) * 128 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

/* shared-memory matrix descriptor (no swizzle, K-major) */
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46; /* descriptor version of sm_100 family */
  /* base offset 0, layout type 0 = no swizzle */
  return d;
}

/* instruction descriptor: kind::f16, D = F32, A = B = BF16, both K-major */
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4)                        /* D format F32 */
         | (1u << 7)                      /* A format BF16 */
         | (1u << 10)                     /* B format BF16 */
         | ((uint32_t)(N >> 3) << 17)     /* N / 8 */
         | ((uint32_t)(M >> 4) << 24);    /* M / 16 */
}

/* ---- tensor memory ---- */
/* allocates ncols columns (power of two >= 32) for the CTA; whole warp */
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
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
/* generic-proxy shared-memory writes become visible to the tensor core */
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

/* ---- MMA ---- */
/* D[tmem] (+)= A[smem] * B[smem]^T, one instruction, issued by one thread */
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         bool accumulate) {
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "setp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"((uint32_t)accumulate)
      : "memory");
}

/* arrives on the mbarrier once every MMA this thread issued has completed */
__device__ __forceinline__ void mma_commit(uint64_t *mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
               : "memory");
}

/* ---- mbarrier ---- */
__device__ __forceinline__ void mbar_init(uint64_t *mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
}

/* waits for the phase with the given parity to complete; false when the
 * bound runs out */
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t parity, uint32_t max_tries = 1u << 22) {
  const uint32_t a = smem_u32(mbar);
  for (uint32_t i = 0; i < max_tries; i++) {
    uint32_t done;
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if (i > 64) __nanosleep(64);
  }
  return false;
}

/* ---- accumulator loads: 32 lanes x 32 columns (one row per thread); the
 * wait is in the same statement so no use of the registers can precede it ---- */
__device__ __forceinline__ void tmem_ld_32x32b_x32(uint32_t taddr, float *v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

}  // namespace umma
}  // namespace xmi
#endif

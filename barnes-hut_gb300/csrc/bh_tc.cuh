// bh_tc.cuh -- 5th-generation tensor-core (tcgen05) building blocks for sm_103a, inline PTX.
//
// Operand layout: K-major, no swizzle, "core matrices" of 8 rows x 16 bytes (8 BF16).  A tile
// of R rows x K columns keeps core matrix (r8, k8) at byte ((r8 * K/8) + k8) * 128, rows 16 bytes
// apart inside it, so the leading-dimension byte offset (next core matrix along K) is 128 and the
// stride byte offset (next 8-row group) is K/8 * 128.  One MMA consumes K = 16 (two core
// columns): the descriptor of K-step j starts 256 * j bytes into the tile.
//
// Accumulators live in tensor memory (TMEM): with M = 128 and cta_group::1, row i of D is TMEM
// lane i and column j is TMEM column (base + j), FP32.  Warp w reads lanes 32 (w % 4) .. +31.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace bh {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// byte offset of element (r, k) in a K-major no-swizzle tile with kc = K / 8 core columns
__host__ __device__ __forceinline__ uint32_t kmajor_off(int r, int k, int kc) {
    return (uint32_t)(((r >> 3) * kc + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// shared-memory matrix descriptor (tcgen05 format: version 1, no swizzle)
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}
// descriptor of K-step j of a K-major tile with kc core columns starting at saddr
__device__ __forceinline__ uint64_t kdesc(uint32_t saddr, int kc, int j) {
    return sdesc(saddr + 256u * (uint32_t)j, 128u, 128u * (uint32_t)kc);
}

// instruction descriptor, kind::f16: BF16 A and B (K-major), FP32 D, shape M x N
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
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

// D[tmem] (+)= A[smem] * B[smem]^T ; issued by one thread
__device__ __forceinline__ void mma(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                    uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// arrive on mbar when all tcgen05 operations issued so far by this thread complete
__device__ __forceinline__ void commit(uint64_t *mbar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(mbar))
        : "memory");
}

__device__ __forceinline__ void fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// make generic-proxy shared-memory writes visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t *m, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(m)), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t *m, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(m)), "r"(phase)
        : "memory");
    return ok != 0;
}
// Bounded wait for the given phase parity; false (and the caller raises an error flag) if the
// barrier did not complete within `limit` polls.
__device__ __forceinline__ bool mbar_wait(uint64_t *m, uint32_t phase, int limit = 1 << 22) {
    for (int i = 0; i < limit; i++)
        if (mbar_try(m, phase)) return true;
    return false;
}

// One arrival on mbar that also announces `bytes` of bulk-copy data to wait for.
__device__ __forceinline__ void mbar_expect_tx(uint64_t *m, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(m)), "r"(bytes)
                 : "memory");
}
// Bulk copy (TMA, untiled) global -> shared; completes `bytes` on mbar.  dst, src and bytes
// must be multiples of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *m) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(m))
        : "memory");
}

// 32 lanes x 16 consecutive FP32 columns: thread t of the warp gets lane (lane_base + t)
__device__ __forceinline__ void ld16(uint32_t taddr, float *v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void ld_wait() {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// GELU, tanh form (Hendrycks & Gimpel), with the hardware tanh approximation
__device__ __forceinline__ float tanh_approx(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
constexpr float GELU_C0 = 0.7978845608028654f;  // sqrt(2 / pi)
constexpr float GELU_C1 = 0.044715f;
__device__ __forceinline__ float gelu(float x) {
    float t = tanh_approx(GELU_C0 * (x + GELU_C1 * x * x * x));
    return 0.5f * x * (1.f + t);
}
__device__ __forceinline__ float gelu_grad(float x) {
    float u = GELU_C0 * (x + GELU_C1 * x * x * x);
    float t = tanh_approx(u);
    return 0.5f * (1.f + t) + 0.5f * x * (1.f - t * t) * GELU_C0 * (1.f + 3.f * GELU_C1 * x * x);
}

}  // namespace tc
}  // namespace bh

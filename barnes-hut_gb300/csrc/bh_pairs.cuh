// bh_pairs.cuh -- shared pieces of the force kernels: CTA shape and list capacities, packed
// FP32 pair arithmetic (sm_100-family f32x2 instructions) and the block-wide exclusive scan.
#pragma once
#include "bh_internal.cuh"

namespace bh {

constexpr int FT = FORCE_THREADS;
constexpr int FAR_CAP = 256;   // far entries per flush
constexpr int NEAR_CAP = 256;  // near boxes per flush
constexpr int SRC_CAP = 384;   // near sources per staging pass
constexpr int FR_CAP = FRONTIER_CAP;

__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Packed FP32 pairs (sm_100-family f32x2 instructions): two lanes of work per instruction.
typedef unsigned long long f2_t;
__device__ __forceinline__ f2_t f2_pack(float a, float b) {
    f2_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void f2_unpack(f2_t v, float &a, float &b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ f2_t f2_add(f2_t a, f2_t b) {
    f2_t r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2_t f2_mul(f2_t a, f2_t b) {
    f2_t r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2_t f2_fma(f2_t a, f2_t b, f2_t c) {
    f2_t r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
__device__ __forceinline__ f2_t f2_rcp(f2_t a) {
    f2_t r;
    asm("{\n.reg .f32 a0, a1, r0, r1;\nmov.b64 {a0, a1}, %1;\nrcp.approx.ftz.f32 r0, a0;\n"
        "rcp.approx.ftz.f32 r1, a1;\nmov.b64 %0, {r0, r1};\n}"
        : "=l"(r)
        : "l"(a));
    return r;
}

// Exclusive block scan of one int per thread; *total = block sum.
__device__ __forceinline__ int block_scan(int v, int *sh, int *total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    int pre = x - v, tot = 0;
    for (int k = 0; k < nw; k++) {
        int s = sh[k];
        if (k < w) pre += s;
        tot += s;
    }
    *total = tot;
    __syncthreads();
    return pre;
}

}  // namespace bh

// bh_mlp.cuh -- layout constants and tile helpers of the learned-correction MLP, shared by the
// standalone MLP kernels (bh_mlp.cu) and the fused correction kernels (bh_learned.cu).
#pragma once
#include <cuda_bf16.h>

#include "bh_internal.cuh"
#include "bh_tc.cuh"

namespace bh {

constexpr int MLP_IN = 6, MLP_K0 = 16, MLP_H = 64, MLP_NO = 16, MLP_OUT = 2;
constexpr int P_W1 = 0, P_B1 = 1024, P_W2 = 1088, P_B2 = 5184, P_W3 = 5248, P_B3 = 9344,
              P_W4 = 9408, P_B4 = 10432, P_TOTAL = 10448;
// image byte offsets
constexpr int I_B1 = 0, I_B2 = 2048, I_B3 = 10240, I_B4 = 18432, I_FWD = 20480;
constexpr int I_B2T = 20480, I_B3T = 28672, I_B4T = 36864, I_TOTAL = 38912;
static_assert(P_TOTAL == MLP_PARAMS && I_TOTAL == MLP_IMAGE_BYTES, "MLP layout");

__device__ __forceinline__ uint16_t bf16_bits(float v) {
    __nv_bfloat16 b = __float2bfloat16_rn(v);
    return *reinterpret_cast<uint16_t *>(&b);
}

__device__ __forceinline__ void copy_bytes(uint8_t *dst, const uint8_t *src, int bytes) {
    for (int i = threadIdx.x * 16; i < bytes; i += blockDim.x * 16)
        *reinterpret_cast<uint4 *>(dst + i) = *reinterpret_cast<const uint4 *>(src + i);
}

// write the 64 BF16 values of row r of a K-major 128 x 64 tile (8 core columns)
__device__ __forceinline__ void store_row64(uint8_t *tile, int r, const float *v) {
#pragma unroll
    for (int c = 0; c < 8; c++) {
        uint32_t w[4];
#pragma unroll
        for (int q = 0; q < 4; q++)
            w[q] = (uint32_t)bf16_bits(v[8 * c + 2 * q]) | ((uint32_t)bf16_bits(v[8 * c + 2 * q + 1]) << 16);
        *reinterpret_cast<uint4 *>(tile + tc::kmajor_off(r, 8 * c, 8)) = make_uint4(w[0], w[1], w[2], w[3]);
    }
}
__device__ __forceinline__ void store_row16(uint8_t *tile, int r, const float *v) {
#pragma unroll
    for (int c = 0; c < 2; c++) {
        uint32_t w[4];
#pragma unroll
        for (int q = 0; q < 4; q++)
            w[q] = (uint32_t)bf16_bits(v[8 * c + 2 * q]) | ((uint32_t)bf16_bits(v[8 * c + 2 * q + 1]) << 16);
        *reinterpret_cast<uint4 *>(tile + tc::kmajor_off(r, 8 * c, 2)) = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

// load 64 accumulator columns of this thread's lane starting at column col
__device__ __forceinline__ void ld64(uint32_t tbase, int col, float *v) {
    const uint32_t lane = (uint32_t)(threadIdx.x & 96) << 16;
#pragma unroll
    for (int c = 0; c < 4; c++) tc::ld16(tbase + lane + col + 16 * c, v + 16 * c);
    tc::ld_wait();
}

// one MMA round: issue (thread 0), commit, wait (all threads).  Returns false on timeout.
template <typename F>
__device__ __forceinline__ bool mma_round(uint64_t *mbar, uint32_t &phase, F issue) {
    tc::fence_async_smem();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (threadIdx.x == 0) {
        issue();
        tc::commit(mbar);
    }
    bool ok = tc::mbar_wait(mbar, phase);
    phase ^= 1u;
    tc::fence_after();
    return __syncthreads_and(ok ? 1 : 0) != 0;
}

// Forward of one 128-row tile whose input rows are already in A0 (K-major 128 x 16).  Thread t
// (of 128) owns row t and receives the two outputs in y[0..1].  W = forward images in shared
// memory, bias = 208 floats (b1, b2, b3, b4) in shared memory, ACT = 128 x 64 scratch tile,
// tmem = 64 allocated columns.  Returns false if a tensor-core wait timed out.
__device__ __forceinline__ bool mlp_tile_forward(uint32_t sW, uint32_t sA0, uint8_t *ACT,
                                                 const float *bias, uint32_t tmem, uint64_t *mbar,
                                                 uint32_t &phase, float *y) {
    const int tid = threadIdx.x;
    const uint32_t sACT = tc::smem_u32(ACT);
    float v[64];
    bool ok = mma_round(mbar, phase, [&] {
        tc::mma(tmem, tc::kdesc(sA0, 2, 0), tc::kdesc(sW + I_B1, 2, 0), tc::idesc_bf16(128, 64), 0);
    });
    if (!ok) return false;
    for (int layer = 0; layer < 3; layer++) {
        ld64(tmem, 0, v);
#pragma unroll
        for (int j = 0; j < 64; j++) v[j] = tc::gelu(v[j] + bias[64 * layer + j]);
        store_row64(ACT, tid, v);
        const uint32_t wimg = sW + (layer == 0 ? I_B2 : layer == 1 ? I_B3 : I_B4);
        const uint32_t idesc = layer < 2 ? tc::idesc_bf16(128, 64) : tc::idesc_bf16(128, 16);
        ok = mma_round(mbar, phase, [&] {
            for (int j = 0; j < 4; j++) tc::mma(tmem, tc::kdesc(sACT, 8, j), tc::kdesc(wimg, 8, j), idesc, j);
        });
        if (!ok) return false;
    }
    const uint32_t lane = (uint32_t)(tid & 96) << 16;
    tc::ld16(tmem + lane, v);
    tc::ld_wait();
    y[0] = v[0] + bias[192];
    y[1] = v[1] + bias[193];
    tc::fence_before();  // the next tile's MMA overwrites the columns just read
    return true;
}

}  // namespace bh

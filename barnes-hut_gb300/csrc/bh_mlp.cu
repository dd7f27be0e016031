// bh_mlp.cu -- learned far-field correction: a 6 -> 64 -> 64 -> 64 -> 2 GELU MLP on tcgen05.
//
// No reference counterpart (python-bh has no learned component).  BF16 weights and activations,
// FP32 accumulation in tensor memory, FP32 master weights and Adam moments in global memory.
//
// Master parameter layout (float, offsets below): W1[16][64] (rows >= 6 zero), b1[64],
// W2[64][64], b2[64], W3[64][64], b3[64], W4[64][16] (columns >= 2 zero), b4[16]; W_l[in][out].
// Packed images (BF16, K-major core-matrix tiles, see bh_tc.cuh):
//   forward  B1[64 out][16 in], B2[64][64], B3[64][64], B4[16 out][64 in]  (GEMM y = x W)
//   backward B2T[64 in][64 out], B3T[64][64], B4T[64 in][16 out]            (GEMM dx = dy W^T)
//
// Training tile = 128 (input, target) rows; per tile 4 forward GEMMs, 3 backward dA GEMMs and
// 2 weight-gradient GEMMs.  The weight gradients dW = A^T dH reduce over the rows of the tile,
// so the rows are the MMA's K dimension and the layer widths (16 or 64) its M dimension; two
// layers share one M = 128 MMA by stacking: [a1^T; a2^T] x [dh2^T; dh3^T]^T holds dW2 and dW3
// as diagonal blocks, [a0^T; a3^T; 0] x [dh1^T; dh4^T]^T holds dW1 and dW4.
#include "bh_mlp.cuh"

namespace bh {

constexpr int MT = 128;  // rows per tile = threads per CTA

// ------------------------------------------------------------------ packing
__global__ void k_mlp_pack(const float *p, uint8_t *img) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    // forward images
    if (t < 64 * 16) {  // B1[n][k] = W1[k][n]
        int n = t / 16, k = t % 16;
        float v = k < MLP_IN ? p[P_W1 + k * 64 + n] : 0.f;
        *reinterpret_cast<uint16_t *>(img + I_B1 + tc::kmajor_off(n, k, 2)) = bf16_bits(v);
    }
    if (t < 64 * 64) {
        int n = t / 64, k = t % 64;
        *reinterpret_cast<uint16_t *>(img + I_B2 + tc::kmajor_off(n, k, 8)) =
            bf16_bits(p[P_W2 + k * 64 + n]);
        *reinterpret_cast<uint16_t *>(img + I_B3 + tc::kmajor_off(n, k, 8)) =
            bf16_bits(p[P_W3 + k * 64 + n]);
        // backward: B2T[n = in][k = out] = W2[in][out]
        *reinterpret_cast<uint16_t *>(img + I_B2T + tc::kmajor_off(n, k, 8)) =
            bf16_bits(p[P_W2 + n * 64 + k]);
        *reinterpret_cast<uint16_t *>(img + I_B3T + tc::kmajor_off(n, k, 8)) =
            bf16_bits(p[P_W3 + n * 64 + k]);
    }
    if (t < 16 * 64) {  // B4[n][k] = W4[k][n] (n < 16 outputs)
        int n = t / 64, k = t % 64;
        float v = n < MLP_OUT ? p[P_W4 + k * 16 + n] : 0.f;
        *reinterpret_cast<uint16_t *>(img + I_B4 + tc::kmajor_off(n, k, 8)) = bf16_bits(v);
        // B4T[n = in (64)][k = out (16)] = W4[in][out]
        int n2 = t / 16, k2 = t % 16;
        float v2 = k2 < MLP_OUT ? p[P_W4 + n2 * 16 + k2] : 0.f;
        *reinterpret_cast<uint16_t *>(img + I_B4T + tc::kmajor_off(n2, k2, 2)) = bf16_bits(v2);
    }
}

// --------------------------------------------------------------- shared state
struct MlpSmemInfer {
    // byte offsets in dynamic shared memory (1024-aligned base)
    static constexpr int W = 0;                 // forward images, I_FWD bytes
    static constexpr int A0 = I_FWD;            // 128 x 16 BF16
    static constexpr int ACT = A0 + 4096;       // 128 x 64 BF16
    static constexpr int BIAS = ACT + 16384;    // 208 floats
    static constexpr int TOTAL = BIAS + 208 * 4;
};

// transposed store: value v[j] of row r goes to element (row0 + j, r) of a K-major tile with
// 16 core columns (K = 128 rows of the batch tile)
__device__ __forceinline__ void store_colT(uint8_t *tile, int row0, int r, const float *v, int n) {
    for (int j = 0; j < n; j++)
        *reinterpret_cast<uint16_t *>(tile + tc::kmajor_off(row0 + j, r, 16)) = bf16_bits(v[j]);
}

// ---------------------------------------------------------------- inference
// out[r] = MLP(feats[r][0..5]) for r < P; feats row stride fs floats, out row stride 2.
__global__ void __launch_bounds__(MT) k_mlp_infer(const float *feats, int fs, long long P,
                                                  const uint8_t *img, const float *params,
                                                  float *out, unsigned *err) {
    extern __shared__ __align__(1024) uint8_t sm[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tslot;
    uint8_t *W = sm + MlpSmemInfer::W, *A0 = sm + MlpSmemInfer::A0, *ACT = sm + MlpSmemInfer::ACT;
    float *bias = reinterpret_cast<float *>(sm + MlpSmemInfer::BIAS);
    const int tid = threadIdx.x;
    copy_bytes(W, img, I_FWD);
    for (int i = tid; i < 64; i += MT) {
        bias[i] = params[P_B1 + i];
        bias[64 + i] = params[P_B2 + i];
        bias[128 + i] = params[P_B3 + i];
    }
    if (tid < 16) bias[192 + tid] = params[P_B4 + tid];
    if (tid < 32) {
        tc::tmem_alloc(&tslot, 64);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        tc::mbar_init(&mbar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = tslot;
    const uint32_t sW = tc::smem_u32(W), sA0 = tc::smem_u32(A0);
    uint32_t phase = 0;
    bool ok = true;
    const long long ntiles = (P + MT - 1) / MT;
    for (long long t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        const long long row = t * MT + tid;
        float v[64];
#pragma unroll
        for (int k = 0; k < 16; k++) v[k] = 0.f;
        if (row < P) {
#pragma unroll
            for (int k = 0; k < MLP_IN; k++) v[k] = feats[row * fs + k];
        }
        store_row16(A0, tid, v);
        float y[2];
        ok = mlp_tile_forward(sW, sA0, ACT, bias, tmem, &mbar, phase, y);
        if (!ok) break;
        if (row < P) {
            out[row * 2 + 0] = y[0];
            out[row * 2 + 1] = y[1];
        }
    }
    if (!ok && tid == 0) atomicOr(err, 8u /*BH_DEV_WAIT_TIMEOUT*/);
    tc::fence_before();
    __syncthreads();
    if (tid < 32) tc::tmem_dealloc(tmem, 64);
}

// ----------------------------------------------------------------- training
struct MlpSmemTrain {
    static constexpr int W = 0;                  // all images, I_TOTAL bytes
    static constexpr int A0 = 38912;             // 128 x 16
    static constexpr int ACT = A0 + 4096;        // 128 x 64
    static constexpr int DH = ACT + 16384;       // 128 x 64
    static constexpr int DH4 = DH + 16384;       // 128 x 16
    static constexpr int AT23 = DH4 + 4096;      // 128 x 128 : [a1^T; a2^T]
    static constexpr int AT14 = AT23 + 32768;    // 128 x 128 : [a0^T; a3^T; 0]
    static constexpr int BT23 = AT14 + 32768;    // 128 x 128 : [dh2^T; dh3^T]
    static constexpr int BT14 = BT23 + 32768;    // 80 x 128  : [dh1^T; dh4^T]
    static constexpr int BIAS = BT14 + 20480;    // 208 floats
    static constexpr int GB = BIAS + 832;        // 208 floats of bias gradients
    static constexpr int TOTAL = GB + 832;
};
// TMEM columns
constexpr uint32_t T_H1 = 0, T_H2 = 64, T_H3 = 128, T_Y = 192, T_DA = 208, T_G23 = 288, T_G14 = 416;

// One pass over rows [0, P) of (feats, targets): accumulates d(loss)/d(params) into grad (FP32,
// atomics) and sum of squared errors into *loss.  loss = mean over rows and outputs of
// (y - target)^2 * scale, gradient scaled by 2 * scale / (P * 2).
__global__ void __launch_bounds__(MT, 1) k_mlp_train(const float *feats, int fs, const float *targets,
                                                     long long P, const uint8_t *img,
                                                     const float *params, float *grad, float *loss,
                                                     unsigned *err) {
    extern __shared__ __align__(1024) uint8_t sm[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tslot;
    __shared__ float s_loss;
    using L = MlpSmemTrain;
    uint8_t *W = sm + L::W;
    float *bias = reinterpret_cast<float *>(sm + L::BIAS);
    float *gb = reinterpret_cast<float *>(sm + L::GB);
    const int tid = threadIdx.x;
    copy_bytes(W, img, I_TOTAL);
    for (int i = tid; i < 64; i += MT) {
        bias[i] = params[P_B1 + i];
        bias[64 + i] = params[P_B2 + i];
        bias[128 + i] = params[P_B3 + i];
    }
    if (tid < 16) bias[192 + tid] = params[P_B4 + tid];
    for (int i = tid; i < 208; i += MT) gb[i] = 0.f;
    // zero the stacked transposes once (padding rows stay zero)
    for (int i = tid * 16; i < L::BIAS - L::AT23; i += MT * 16)
        *reinterpret_cast<uint4 *>(sm + L::AT23 + i) = make_uint4(0, 0, 0, 0);
    if (tid == 0) s_loss = 0.f;
    if (tid < 32) {
        tc::tmem_alloc(&tslot, 512);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        tc::mbar_init(&mbar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tm = tslot;
    const uint32_t sW = tc::smem_u32(W), sA0 = tc::smem_u32(sm + L::A0), sACT = tc::smem_u32(sm + L::ACT);
    const uint32_t sDH = tc::smem_u32(sm + L::DH), sDH4 = tc::smem_u32(sm + L::DH4);
    const uint32_t sAT23 = tc::smem_u32(sm + L::AT23), sAT14 = tc::smem_u32(sm + L::AT14);
    const uint32_t sBT23 = tc::smem_u32(sm + L::BT23), sBT14 = tc::smem_u32(sm + L::BT14);
    uint8_t *ACT = sm + L::ACT, *DH = sm + L::DH;
    uint32_t phase = 0;
    bool ok = true;
    int ntile_done = 0;
    const float gscale = 2.f / (float)(P * MLP_OUT);
    const long long ntiles = (P + MT - 1) / MT;
    float v[64], h[64];
    for (long long t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        const long long row = t * MT + tid;
        const bool valid = row < P;
        // ---- forward
#pragma unroll
        for (int k = 0; k < 16; k++) v[k] = 0.f;
        if (valid)
#pragma unroll
            for (int k = 0; k < MLP_IN; k++) v[k] = feats[row * fs + k];
        store_row16(sm + L::A0, tid, v);
        store_colT(sm + L::AT14, 0, tid, v, 16);
        ok = mma_round(&mbar, phase, [&] {
            tc::mma(tm + T_H1, tc::kdesc(sA0, 2, 0), tc::kdesc(sW + I_B1, 2, 0), tc::idesc_bf16(128, 64), 0);
        });
        if (!ok) break;
        ld64(tm, T_H1, v);
#pragma unroll
        for (int j = 0; j < 64; j++) v[j] = valid ? tc::gelu(v[j] + bias[j]) : 0.f;
        store_row64(ACT, tid, v);
        store_colT(sm + L::AT23, 0, tid, v, 64);
        ok = mma_round(&mbar, phase, [&] {
            for (int j = 0; j < 4; j++)
                tc::mma(tm + T_H2, tc::kdesc(sACT, 8, j), tc::kdesc(sW + I_B2, 8, j), tc::idesc_bf16(128, 64), j);
        });
        if (!ok) break;
        ld64(tm, T_H2, v);
#pragma unroll
        for (int j = 0; j < 64; j++) v[j] = valid ? tc::gelu(v[j] + bias[64 + j]) : 0.f;
        store_row64(ACT, tid, v);
        store_colT(sm + L::AT23, 64, tid, v, 64);
        ok = mma_round(&mbar, phase, [&] {
            for (int j = 0; j < 4; j++)
                tc::mma(tm + T_H3, tc::kdesc(sACT, 8, j), tc::kdesc(sW + I_B3, 8, j), tc::idesc_bf16(128, 64), j);
        });
        if (!ok) break;
        ld64(tm, T_H3, v);
#pragma unroll
        for (int j = 0; j < 64; j++) v[j] = valid ? tc::gelu(v[j] + bias[128 + j]) : 0.f;
        store_row64(ACT, tid, v);
        store_colT(sm + L::AT14, 16, tid, v, 64);
        ok = mma_round(&mbar, phase, [&] {
            for (int j = 0; j < 4; j++)
                tc::mma(tm + T_Y, tc::kdesc(sACT, 8, j), tc::kdesc(sW + I_B4, 8, j), tc::idesc_bf16(128, 16), j);
        });
        if (!ok) break;
        {
            const uint32_t lane = (uint32_t)(tid & ~31) << 16;
            tc::ld16(tm + lane + T_Y, v);
            tc::ld_wait();
        }
        // ---- loss and output gradient
        float dy[16];
#pragma unroll
        for (int k = 0; k < 16; k++) dy[k] = 0.f;
        if (valid) {
            float l = 0.f;
            for (int k = 0; k < MLP_OUT; k++) {
                float e = v[k] + bias[192 + k] - targets[row * 2 + k];
                l += e * e;
                dy[k] = gscale * e;
                atomicAdd(&gb[192 + k], dy[k]);
            }
            atomicAdd(&s_loss, l);
        }
        store_row16(sm + L::DH4, tid, dy);
        store_colT(sm + L::BT14, 64, tid, dy, 16);
        // da3 = dh4 W4^T
        ok = mma_round(&mbar, phase, [&] {
            tc::mma(tm + T_DA, tc::kdesc(sDH4, 2, 0), tc::kdesc(sW + I_B4T, 2, 0), tc::idesc_bf16(128, 64), 0);
        });
        if (!ok) break;
        // dh3 = da3 * gelu'(h3 + b3)
        ld64(tm, T_DA, v);
        ld64(tm, T_H3, h);
#pragma unroll
        for (int j = 0; j < 64; j++) {
            v[j] = valid ? v[j] * tc::gelu_grad(h[j] + bias[128 + j]) : 0.f;
            atomicAdd(&gb[128 + j], v[j]);
        }
        store_row64(DH, tid, v);
        store_colT(sm + L::BT23, 64, tid, v, 64);
        ok = mma_round(&mbar, phase, [&] {
            for (int j = 0; j < 4; j++)
                tc::mma(tm + T_DA, tc::kdesc(sDH, 8, j), tc::kdesc(sW + I_B3T, 8, j), tc::idesc_bf16(128, 64), j);
        });
        if (!ok) break;
        // dh2 = da2 * gelu'(h2 + b2)
        ld64(tm, T_DA, v);
        ld64(tm, T_H2, h);
#pragma unroll
        for (int j = 0; j < 64; j++) {
            v[j] = valid ? v[j] * tc::gelu_grad(h[j] + bias[64 + j]) : 0.f;
            atomicAdd(&gb[64 + j], v[j]);
        }
        store_row64(DH, tid, v);
        store_colT(sm + L::BT23, 0, tid, v, 64);
        const uint32_t acc = ntile_done > 0 ? 1u : 0u;
        ok = mma_round(&mbar, phase, [&] {
            for (int j = 0; j < 4; j++)
                tc::mma(tm + T_DA, tc::kdesc(sDH, 8, j), tc::kdesc(sW + I_B2T, 8, j), tc::idesc_bf16(128, 64), j);
            for (int j = 0; j < 8; j++)  // [a1^T; a2^T] x [dh2^T; dh3^T]^T, K = 128 rows
                tc::mma(tm + T_G23, tc::kdesc(sAT23, 16, j), tc::kdesc(sBT23, 16, j),
                        tc::idesc_bf16(128, 128), acc | (j > 0 ? 1u : 0u));
        });
        if (!ok) break;
        // dh1 = da1 * gelu'(h1 + b1)
        ld64(tm, T_DA, v);
        ld64(tm, T_H1, h);
#pragma unroll
        for (int j = 0; j < 64; j++) {
            v[j] = valid ? v[j] * tc::gelu_grad(h[j] + bias[j]) : 0.f;
            atomicAdd(&gb[j], v[j]);
        }
        store_colT(sm + L::BT14, 0, tid, v, 64);
        ok = mma_round(&mbar, phase, [&] {
            for (int j = 0; j < 8; j++)  // [a0^T; a3^T; 0] x [dh1^T; dh4^T]^T
                tc::mma(tm + T_G14, tc::kdesc(sAT14, 16, j), tc::kdesc(sBT14, 16, j),
                        tc::idesc_bf16(128, 80), acc | (j > 0 ? 1u : 0u));
        });
        if (!ok) break;
        ntile_done++;
    }
    // ---- flush gradients (this CTA's share) to global memory
    if (ok && ntile_done > 0) {
        const uint32_t lane = (uint32_t)(tid & ~31) << 16;
        float g[16];
        // G23: row tid; dW2 = rows 0..63 cols 0..63, dW3 = rows 64..127 cols 64..127
        const int c0 = tid < 64 ? 0 : 64;
        for (int c = 0; c < 4; c++) {
            tc::ld16(tm + lane + T_G23 + c0 + 16 * c, g);
            tc::ld_wait();
            for (int k = 0; k < 16; k++) {
                int out_n = 16 * c + k;
                if (tid < 64) atomicAdd(&grad[P_W2 + tid * 64 + out_n], g[k]);
                else atomicAdd(&grad[P_W3 + (tid - 64) * 64 + out_n], g[k]);
            }
        }
        // G14: dW1 = rows 0..15 (6 real) cols 0..63, dW4 = rows 16..79 cols 64..79 (2 real).
        // tcgen05.ld is warp-collective: every lane loads, each uses what belongs to it.
        for (int c = 0; c < 5; c++) {
            tc::ld16(tm + lane + T_G14 + 16 * c, g);
            tc::ld_wait();
            if (c < 4 && tid < MLP_IN)
                for (int k = 0; k < 16; k++) atomicAdd(&grad[P_W1 + tid * 64 + 16 * c + k], g[k]);
            if (c == 4 && tid >= 16 && tid < 80)
                for (int k = 0; k < MLP_OUT; k++) atomicAdd(&grad[P_W4 + (tid - 16) * 16 + k], g[k]);
        }
    }
    __syncthreads();
    if (ok) {
        for (int i = tid; i < 64; i += MT) {
            atomicAdd(&grad[P_B1 + i], gb[i]);
            atomicAdd(&grad[P_B2 + i], gb[64 + i]);
            atomicAdd(&grad[P_B3 + i], gb[128 + i]);
        }
        if (tid < MLP_OUT) atomicAdd(&grad[P_B4 + tid], gb[192 + tid]);
        if (tid == 0) atomicAdd(loss, s_loss);
    } else if (tid == 0) {
        atomicOr(err, 8u /*BH_DEV_WAIT_TIMEOUT*/);
    }
    tc::fence_before();
    __syncthreads();
    if (tid < 32) tc::tmem_dealloc(tm, 512);
}

// Adam (Kingma & Ba) on the master parameters; zeroes the gradient.
__global__ void k_mlp_adam(float *p, float *m, float *v, float *g, int step, float lr, float b1,
                           float b2, float eps) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P_TOTAL) return;
    // structurally zero entries stay zero
    bool fixed = (i >= P_W1 && i < P_B1 && (i - P_W1) / 64 >= MLP_IN) ||
                 (i >= P_W4 && i < P_B4 && (i - P_W4) % 16 >= MLP_OUT) || (i >= P_B4 + MLP_OUT);
    float gi = fixed ? 0.f : g[i];
    g[i] = 0.f;
    if (fixed) {
        p[i] = 0.f;
        return;
    }
    float mi = b1 * m[i] + (1.f - b1) * gi;
    float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    float mh = mi / (1.f - powf(b1, (float)step));
    float vh = vi / (1.f - powf(b2, (float)step));
    p[i] -= lr * mh / (sqrtf(vh) + eps);
}

// -------------------------------------------------------------------- launches
cudaError_t mlp_init() {
    cudaError_t e = cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         MlpSmemInfer::TOTAL + 1024);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                MlpSmemTrain::TOTAL + 1024);
}

cudaError_t mlp_pack(const float *params, uint8_t *img, cudaStream_t st) {
    k_mlp_pack<<<16, 256, 0, st>>>(params, img);
    return cudaGetLastError();
}

cudaError_t mlp_infer(const float *feats, int fs, long long P, const uint8_t *img,
                      const float *params, float *out, unsigned *err, cudaStream_t st) {
    if (P <= 0) return cudaSuccess;
    long long tiles = (P + MT - 1) / MT;
    const long long cap = device_sm_count() * 4LL;
    int grid = (int)(tiles < cap ? tiles : cap);
    k_mlp_infer<<<grid, MT, MlpSmemInfer::TOTAL + 1024, st>>>(feats, fs, P, img, params, out, err);
    return cudaGetLastError();
}

cudaError_t mlp_train(const float *feats, int fs, const float *targets, long long P,
                      const uint8_t *img, const float *params, float *grad, float *loss,
                      unsigned *err, cudaStream_t st) {
    if (P <= 0) return cudaSuccess;
    long long tiles = (P + MT - 1) / MT;
    const long long cap = device_sm_count();
    int grid = (int)(tiles < cap ? tiles : cap);
    k_mlp_train<<<grid, MT, MlpSmemTrain::TOTAL + 1024, st>>>(feats, fs, targets, P, img, params,
                                                            grad, loss, err);
    return cudaGetLastError();
}

cudaError_t mlp_adam(float *p, float *m, float *v, float *g, int step, float lr, cudaStream_t st) {
    k_mlp_adam<<<(P_TOTAL + 255) / 256, 256, 0, st>>>(p, m, v, g, step, lr, 0.9f, 0.999f, 1e-8f);
    return cudaGetLastError();
}

}  // namespace bh

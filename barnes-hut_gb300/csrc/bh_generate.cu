// bh_generate.cu -- particle generators on the device (the role of python-bh/bin/gen_input.py).
//
// gen_input.py:38-55 draws, per particle, x, y uniform in [0, DOMAIN_SIZE - 1) ("normal") or
// Gaussian around the domain centre with sigma (DOMAIN_SIZE - 1) / 12 ("gauss"; the reference's
// gauss branch calls an unimported module), velocities uniform in [-1, 1) and masses uniform in
// [0.5, 5).  Here the same distributions, plus the clustered mixture of this project's benchmark
// (8 Gaussian clusters with sigma 0.05 around centres uniform in [0.2, 0.8)^2, 20 % uniform
// background on [0, 1)^2, masses uniform in [1, 2), zero velocity), are drawn on the GPU from a
// counter-based generator, so any particle can be generated independently and the output is a
// pure function of (distribution, n, seed).
//
// Random numbers: Philox4x32-10 (J. Salmon, M. Moraes, R. Dror, D. Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC 2011): counter (particle index low, high, block, stream),
// key (seed low, seed high).  Two 32-bit outputs make one double in [0, 1) with 53 random bits;
// normal deviates come from the Box-Muller transform.  The uniform transforms are written with
// explicit rounding (no FMA contraction) so a CPU restatement reproduces them bit for bit.
#include <math.h>

#include "../../include/bh_gb300.h"
#include "bh_internal.cuh"

namespace bh {

struct U4 {
    unsigned a, b, c, d;
};

__device__ __forceinline__ U4 philox4x32_10(U4 ctr, unsigned k0, unsigned k1) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const unsigned lo0 = 0xD2511F53u * ctr.a, hi0 = __umulhi(0xD2511F53u, ctr.a);
        const unsigned lo1 = 0xCD9E8D57u * ctr.c, hi1 = __umulhi(0xCD9E8D57u, ctr.c);
        ctr = U4{hi1 ^ ctr.b ^ k0, lo1, hi0 ^ ctr.d ^ k1, lo0};
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return ctr;
}

// [0, 1) with 53 bits: 27 high bits of a, 26 of b (every step exact)
__device__ __forceinline__ double u53(unsigned a, unsigned b) {
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

// Box-Muller: two independent N(0, 1) from u, v in [0, 1)
__device__ __forceinline__ void box_muller(double u, double v, double *z0, double *z1) {
    const double r = sqrt(-2.0 * log(1.0 - u));
    double s, c;
    sincospi(2.0 * v, &s, &c);
    *z0 = r * c;
    *z1 = r * s;
}

constexpr double GEN_DOMAIN = 499.0;  // gen_input.py: DOMAIN_SIZE - 1

__global__ void k_generate(int dist, long long n, unsigned long long seed, double *x, double *y,
                           double *m, double *vx, double *vy) {
    const unsigned k0 = (unsigned)seed, k1 = (unsigned)(seed >> 32);
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const unsigned ilo = (unsigned)i, ihi = (unsigned)(i >> 32);
        const U4 r0 = philox4x32_10(U4{ilo, ihi, 0u, 0u}, k0, k1);
        const U4 r1 = philox4x32_10(U4{ilo, ihi, 1u, 0u}, k0, k1);
        const U4 r2 = philox4x32_10(U4{ilo, ihi, 2u, 0u}, k0, k1);
        const double u0 = u53(r0.a, r0.b), u1 = u53(r0.c, r0.d);
        const double u2 = u53(r1.a, r1.b), u3 = u53(r1.c, r1.d);
        const double u4 = u53(r2.a, r2.b);
        double px, py, pm, pvx = 0.0, pvy = 0.0;
        if (dist == BH_GEN_CLUSTER) {
            if (u0 < 0.2) {  // uniform background
                px = u2;
                py = u3;
            } else {
                const int c = min((int)(u1 * 8.0), 7);
                const U4 rc = philox4x32_10(U4{(unsigned)c, 0u, 0u, 1u}, k0, k1);  // centre c
                const double cx = 0.2 + 0.6 * u53(rc.a, rc.b), cy = 0.2 + 0.6 * u53(rc.c, rc.d);
                double z0, z1;
                box_muller(u2, u3, &z0, &z1);
                const double top = 1.0 - 5.9604644775390625e-8;  // 1 - 2^-24
                px = fmin(fmax(cx + 0.05 * z0, 0.0), top);
                py = fmin(fmax(cy + 0.05 * z1, 0.0), top);
            }
            pm = 1.0 + u4;
        } else {
            if (dist == BH_GEN_GAUSS) {
                double z0, z1;
                box_muller(u0, u1, &z0, &z1);
                px = 0.5 * GEN_DOMAIN + (GEN_DOMAIN / 12.0) * z0;
                py = 0.5 * GEN_DOMAIN + (GEN_DOMAIN / 12.0) * z1;
            } else {
                px = __dmul_rn(u0, GEN_DOMAIN);
                py = __dmul_rn(u1, GEN_DOMAIN);
            }
            pvx = __dmul_rn(__dsub_rn(u2, 0.5), 2.0);
            pvy = __dmul_rn(__dsub_rn(u3, 0.5), 2.0);
            pm = __dadd_rn(0.5, __dmul_rn(u4, 5.0 - 0.5));
        }
        x[i] = px;
        y[i] = py;
        m[i] = pm;
        vx[i] = pvx;
        vy[i] = pvy;
    }
}

}  // namespace bh

extern "C" int bh_generate(int distribution, long long n, unsigned long long seed, double *x, double *y,
                           double *m, double *vx, double *vy, void *stream) {
    if (distribution < BH_GEN_UNIFORM || distribution > BH_GEN_CLUSTER)
        return bh::bh_set_thread_error(BH_ERR_INVALID, "bh_generate: unknown distribution");
    if (n < 0) return bh::bh_set_thread_error(BH_ERR_INVALID, "bh_generate: n < 0");
    if (n == 0) return BH_OK;
    if (!x || !y || !m || !vx || !vy) return bh::bh_set_thread_error(BH_ERR_INVALID, "bh_generate: null array");
    long long blocks = (n + 255) / 256;
    const long long cap = bh::device_sm_count() * 16LL;
    if (blocks > cap) blocks = cap;
    bh::k_generate<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(distribution, n, seed, x, y, m, vx, vy);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return bh::bh_set_thread_error(BH_ERR_CUDA, cudaGetErrorString(e));
    return BH_OK;
}

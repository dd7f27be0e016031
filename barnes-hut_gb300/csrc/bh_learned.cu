// bh_learned.cu -- learned far-field correction in the step, and the generator of its training
// pairs.  No reference counterpart (python-bh has no learned component).
//
// Band: for a target group, the cells accepted by the opening criterion at theta (the step's
// looser angle) but rejected at correction_theta (the tighter angle whose plain monopole error
// the correction aims to match).  The force kernel has already added their monopoles; here the
// MLP adds, per (target particle, band cell) pair,  G M / s * MLP(u, v, qxx, qxy, qyy, w)  with
// u, v the offset from the target to the cell's centre of mass in cell edges s, q the cell's
// second moments about its centre of mass over M s^2, and w = 1 / |(u, v)|.
//
// Training pairs are made by the method itself: for sampled work items, the band cells up to a
// level cap, and a few targets per item, the exact FP64 sum over the cell's particles minus the
// FP64 monopole, in the same units.
#include "bh_mlp.cuh"

namespace bh {

constexpr int LT = 128;          // threads per CTA
constexpr int BAND_CAP = 1024;   // band cells per item
constexpr int LTMAX = TARGET_CHUNK;

struct BandCell {
    float rx, ry, M, s;   // centre of mass in the group frame, mass, cell edge
    float qxx, qxy, qyy;  // normalised second moments
    int cell;             // global cell index
};

__device__ __forceinline__ int lblock_scan(int v, int *sh, int *total) {
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

// Group geometry of a work item (the same mapping as the force kernel).
struct ItemGeom {
    int s, TG, G, gx0, gy0, gx1, gy1, ncol, nt, c0, T;
};

__device__ __forceinline__ void item_geom(const DevPlan &d, long long g, int chunk, int *col0,
                                          int *colpre, ItemGeom &ig) {
    const int tid = threadIdx.x;
    ig.s = find_seg(d.goff_tab, d.nsys, g);
    const SysDesc &sd = d.sys[ig.s];
    const long long lg = g - sd.goff;
    ig.TG = sd.TG;
    ig.G = sd.G;
    const int gi = (int)(lg / sd.NGs), gj = (int)(lg - (long long)gi * sd.NGs);
    ig.gx0 = gi * sd.TG;
    ig.gy0 = gj * sd.TG;
    ig.gx1 = min(sd.G, ig.gx0 + sd.TG);
    ig.gy1 = min(sd.G, ig.gy0 + sd.TG);
    ig.ncol = ig.gx1 - ig.gx0;
    if (tid < ig.ncol) {
        long long b0 = sd.boff + (long long)(ig.gx0 + tid) * sd.G + ig.gy0;
        int st = d.box_start[b0];
        col0[tid] = st;
        colpre[tid + 1] = d.box_start[b0 + (ig.gy1 - ig.gy0)] - st;
    }
    __syncthreads();
    if (tid == 0) {
        colpre[0] = 0;
        for (int c = 1; c <= ig.ncol; c++) colpre[c] += colpre[c - 1];
    }
    __syncthreads();
    ig.nt = colpre[ig.ncol];
    item_range(ig.nt, d.item_cnt[g], chunk, &ig.c0, &ig.T);
}

__device__ __forceinline__ int item_target(const ItemGeom &ig, const int *col0, const int *colpre,
                                           int v) {
    int u = ig.c0 + v, c = 0;
    while (c + 1 < ig.ncol && colpre[c + 1] <= u) c++;
    return col0[c] + (u - colpre[c]);
}

// Collect the band cells of a group (levels <= max_level).  Returns the block-uniform count;
// *ovf is set when the frontier or the band list overflowed (flagged by the caller).
__device__ int band_walk(const DevPlan &d, const ItemGeom &ig, float th2_hi, float th2_lo,
                         int max_level, BandCell *band, int *fr0, int *fr1, int *sh_scan,
                         bool *ovf) {
    const int tid = threadIdx.x;
    const SysDesc &sd = d.sys[ig.s];
    const SysDyn &dy = d.dyn[ig.s];
    const float step_f = __double2float_rn(dy.step);
    const float W_f = __fmul_rn((float)ig.TG, step_f);
    int *fr = fr0, *fn = fr1;
    if (tid == 0) fr[0] = 0;
    int nfr = 1, nband = 0;
    bool of = false;
    for (int l = sd.L - 1; l >= 1 && nfr > 0; l--) {  // leaves are never band cells' parents' children
        const int gl = sd.lvg[l];
        const int gc = sd.lvg[l - 1];
        int nnext = 0;
        __syncthreads();
        for (int q0 = 0; q0 < nfr; q0 += LT) {
            int q = q0 + tid;
            int isband = 0, nch = 0;
            int ci = 0, cj = 0;
            BandCell bc;
            int loc = q < nfr ? fr[q] : 0;
            if (q < nfr && (unsigned)loc >= (unsigned)(gl * gl)) {
                raise_err(d.glob, 4u /*BH_DEV_BAD_KEY*/);  // never expected: skip the cell
            } else if (q < nfr) {
                ci = loc / gl;
                cj = loc - ci * gl;
                long long cell = sd.coff + sd.lvoff[l] + loc;
                float4 rr = d.rec[cell];
                if (rr.z > 0.f) {
                    int lo_x = ci << l, hi_x = (ci + 1) << l, lo_y = cj << l, hi_y = (cj + 1) << l;
                    bool overlap = lo_x < ig.gx1 && hi_x > ig.gx0 && lo_y < ig.gy1 && hi_y > ig.gy0;
                    bool acc_hi = false, acc_lo = false;
                    float rx = 0.f, ry = 0.f, s_f = ldexpf(step_f, l);
                    if (!overlap) {
                        rx = __fadd_rn(__fmul_rn((float)(lo_x - ig.gx0), step_f), rr.x);
                        ry = __fadd_rn(__fmul_rn((float)(lo_y - ig.gy0), step_f), rr.y);
                        float dxo = fmaxf(0.f, fmaxf(-rx, __fsub_rn(rx, W_f)));
                        float dyo = fmaxf(0.f, fmaxf(-ry, __fsub_rn(ry, W_f)));
                        float d2 = __fadd_rn(__fmul_rn(dxo, dxo), __fmul_rn(dyo, dyo));
                        float s2 = __fmul_rn(s_f, s_f);
                        acc_hi = s2 < __fmul_rn(th2_hi, d2);
                        acc_lo = s2 < __fmul_rn(th2_lo, d2);
                    }
                    if (acc_hi) {
                        if (!acc_lo && l <= max_level) {
                            float4 q2 = d.rec2[cell];
                            bc.rx = rx; bc.ry = ry; bc.M = rr.z; bc.s = s_f;
                            bc.qxx = q2.x; bc.qxy = q2.y; bc.qyy = q2.z;
                            bc.cell = (int)cell;
                            isband = 1;
                        }
                    } else {
                        nch = (2 * ci + 1 < gc ? 2 : 1) * (2 * cj + 1 < gc ? 2 : 1);
                    }
                }
            }
            // level-0 band cells are leaves accepted at theta_hi; they come from level-1 children
            int tot;
            int pre = lblock_scan(isband | (nch << 12), sh_scan, &tot);
            if (isband) {
                int pos = nband + (pre & 4095);
                if (pos < BAND_CAP) band[pos] = bc;
            }
            if (nch) {
                int pos = nnext + (pre >> 12);
                if (pos + nch <= FRONTIER_CAP)
                    for (int a = 0; a < 2; a++)
                        for (int b = 0; b < 2; b++)
                            if (2 * ci + a < gc && 2 * cj + b < gc) fn[pos++] = (2 * ci + a) * gc + (2 * cj + b);
            }
            nband += tot & 4095;
            if (nnext + (tot >> 12) > FRONTIER_CAP) of = true;
            nnext += tot >> 12;
        }
        int *t = fr;
        fr = fn;
        fn = t;
        nfr = of ? 0 : nnext;
        // level 0: the children of rejected level-1 cells are leaves
        if (l == 1 && !of) {
            __syncthreads();
            for (int q0 = 0; q0 < nfr; q0 += LT) {
                int q = q0 + tid, isband = 0;
                BandCell bc;
                int loc = q < nfr ? fr[q] : 0;
                if (q < nfr && (unsigned)loc >= (unsigned)(gc * gc)) {
                    raise_err(d.glob, 4u /*BH_DEV_BAD_KEY*/);
                } else if (q < nfr) {
                    int ci0 = loc / gc, cj0 = loc - ci0 * gc;
                    long long cell = sd.coff + loc;
                    float4 rr = d.rec[cell];
                    if (rr.z > 0.f) {
                        bool overlap = ci0 < ig.gx1 && ci0 + 1 > ig.gx0 && cj0 < ig.gy1 && cj0 + 1 > ig.gy0;
                        if (!overlap) {
                            float rx = __fadd_rn(__fmul_rn((float)(ci0 - ig.gx0), step_f), rr.x);
                            float ry = __fadd_rn(__fmul_rn((float)(cj0 - ig.gy0), step_f), rr.y);
                            float dxo = fmaxf(0.f, fmaxf(-rx, __fsub_rn(rx, W_f)));
                            float dyo = fmaxf(0.f, fmaxf(-ry, __fsub_rn(ry, W_f)));
                            float d2 = __fadd_rn(__fmul_rn(dxo, dxo), __fmul_rn(dyo, dyo));
                            float s2 = __fmul_rn(step_f, step_f);
                            if (s2 < __fmul_rn(th2_hi, d2) && !(s2 < __fmul_rn(th2_lo, d2))) {
                                float4 q2 = d.rec2[cell];
                                bc.rx = rx; bc.ry = ry; bc.M = rr.z; bc.s = step_f;
                                bc.qxx = q2.x; bc.qxy = q2.y; bc.qyy = q2.z;
                                bc.cell = (int)cell;
                                isband = 1;
                            }
                        }
                    }
                }
                int tot;
                int pre = lblock_scan(isband, sh_scan, &tot);
                if (isband) {
                    int pos = nband + pre;
                    if (pos < BAND_CAP) band[pos] = bc;
                }
                nband += tot;
            }
        }
    }
    if (nband > BAND_CAP) {
        of = true;
        nband = BAND_CAP;
    }
    *ovf = of;
    __syncthreads();
    return nband;
}

__device__ __forceinline__ void band_features(const BandCell &b, float tx, float ty, float *f) {
    float inv_s = 1.f / b.s;
    float u = (b.rx - tx) * inv_s, v = (b.ry - ty) * inv_s;
    f[0] = u;
    f[1] = v;
    f[2] = b.qxx;
    f[3] = b.qxy;
    f[4] = b.qyy;
    f[5] = rsqrtf(u * u + v * v);
}

// ----------------------------------------------------------------- correction in the step
struct LSmem {
    static constexpr int W = 0;                      // forward images
    static constexpr int A0 = I_FWD;                 // 128 x 16 BF16
    static constexpr int ACT = A0 + 4096;            // 128 x 64 BF16
    static constexpr int BAND = ACT + 16384;         // BAND_CAP x 32 B
    static constexpr int TPOS = BAND + BAND_CAP * 32;  // LTMAX float2
    static constexpr int CORR = TPOS + LTMAX * 8;    // LTMAX float2
    static constexpr int FR = CORR + LTMAX * 8;      // 2 x FRONTIER_CAP int
    static constexpr int BIAS = FR + 2 * FRONTIER_CAP * 4;  // 208 floats
    static constexpr int TOTAL = BIAS + 208 * 4;
};

__global__ void __launch_bounds__(LT) k_learned_correct(DevPlan d, float th2_lo, const uint8_t *img,
                                                        const float *params, int tick) {
    extern __shared__ __align__(1024) uint8_t sm[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tslot;
    __shared__ int sh_scan[32], s_item, s_col0[9], s_colpre[9];
    BandCell *band = reinterpret_cast<BandCell *>(sm + LSmem::BAND);
    float2 *tpos = reinterpret_cast<float2 *>(sm + LSmem::TPOS);
    float2 *corr = reinterpret_cast<float2 *>(sm + LSmem::CORR);
    int *fr0 = reinterpret_cast<int *>(sm + LSmem::FR), *fr1 = fr0 + FRONTIER_CAP;
    float *bias = reinterpret_cast<float *>(sm + LSmem::BIAS);
    const int tid = threadIdx.x;
    copy_bytes(sm + LSmem::W, img, I_FWD);
    for (int i = tid; i < 64; i += LT) {
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
    const uint32_t tmem = tslot, sW = tc::smem_u32(sm + LSmem::W), sA0 = tc::smem_u32(sm + LSmem::A0);
    uint32_t phase = 0;
    bool ok = true;
    const int nxt = (d.glob->epoch + 1) & 1;
    const long long nitems = d.item_off[d.NG_total];
    for (;;) {
        if (tid == 0) s_item = (int)atomicAdd(&d.glob->item_next2, 1u);
        __syncthreads();
        const int item = s_item;
        if (item >= nitems || !ok) break;
        const long long g = d.item_group[item];
        ItemGeom ig;
        item_geom(d, g, item - d.item_off[g], s_col0, s_colpre, ig);
        const SysDyn &dy = d.dyn[ig.s];
        const float step_f = __double2float_rn(dy.step);
        bool of;
        const int nb = band_walk(d, ig, d.theta2_f, th2_lo, 64, band, fr0, fr1, sh_scan, &of);
        if (of && tid == 0) raise_err(d.glob, 2u /*BH_DEV_LIST_OVERFLOW*/);
        for (int v = tid; v < ig.T; v += LT) {
            int ti = item_target(ig, s_col0, s_colpre, v);
            const float4 p = d.PD[2 * (long long)ti];  // (x, x, y, y) box-relative
            int lb = d.skey[ti] - (int)d.sys[ig.s].boff;
            int kx = lb / ig.G, ky = lb - kx * ig.G;
            tpos[v] = make_float2(__fadd_rn(__fmul_rn((float)(kx - ig.gx0), step_f), p.x),
                                  __fadd_rn(__fmul_rn((float)(ky - ig.gy0), step_f), p.z));
            corr[v] = make_float2(0.f, 0.f);
        }
        __syncthreads();
        const long long npairs = (long long)ig.T * nb;
        if (tid == 0) atomicAdd(&d.glob->corr_pairs, (unsigned long long)npairs);
        for (long long p0 = 0; p0 < npairs && ok; p0 += 128) {
            const long long p = p0 + tid;
            float f[16];
#pragma unroll
            for (int k = 0; k < 16; k++) f[k] = 0.f;
            int t = 0, k = 0;
            if (p < npairs) {
                t = (int)(p / nb);
                k = (int)(p - (long long)t * nb);
                band_features(band[k], tpos[t].x, tpos[t].y, f);
            }
            store_row16(sm + LSmem::A0, tid, f);
            float y[2];
            ok = mlp_tile_forward(sW, sA0, sm + LSmem::ACT, bias, tmem, &mbar, phase, y);
            if (ok && p < npairs) {
                float scale = band[k].M / band[k].s;
                atomicAdd(&corr[t].x, scale * y[0]);
                atomicAdd(&corr[t].y, scale * y[1]);
            }
        }
        __syncthreads();
        for (int v = tid; v < ig.T && ok; v += LT) {
            int ti = item_target(ig, s_col0, s_colpre, v);
            double ax = d.AX[ti] + d.gconst * (double)corr[v].x;
            double ay = d.AY[ti] + d.gconst * (double)corr[v].y;
            d.AX[ti] = ax;
            d.AY[ti] = ay;
            if (tick) {
                double vx = d.VX[nxt][ti] + ax * d.dt, vy = d.VY[nxt][ti] + ay * d.dt;
                d.VX[nxt][ti] = vx;
                d.VY[nxt][ti] = vy;
                d.X[nxt][ti] = d.X[nxt][ti] + vx * d.dt;
                d.Y[nxt][ti] = d.Y[nxt][ti] + vy * d.dt;
            }
        }
        __syncthreads();
    }
    if (!ok && tid == 0) raise_err(d.glob, 8u /*BH_DEV_WAIT_TIMEOUT*/);
    tc::fence_before();
    __syncthreads();
    if (tid < 32) tc::tmem_dealloc(tmem, 64);
}

// ------------------------------------------------------------------- training pairs
struct PSmem {
    static constexpr int BAND = 0;
    static constexpr int FR = BAND_CAP * 32;
    static constexpr int TOTAL = FR + 2 * FRONTIER_CAP * 4;
};

// For items item_offset + k * item_stride: band cells at levels <= max_level, up to tpi targets
// per item spread over the item, one warp per (target, cell) pair: exact FP64 sum over the
// cell's particles minus the FP64 monopole, times s / M.  Rows appended at atomicAdd(counter).
__global__ void __launch_bounds__(LT) k_learned_pairs(DevPlan d, float th2_hi, float th2_lo,
                                                      int max_level, long long item_offset,
                                                      long long item_stride, int tpi, float *feats,
                                                      float *targets, unsigned *counter,
                                                      long long capacity) {
    extern __shared__ __align__(1024) uint8_t sm[];
    __shared__ int sh_scan[32], s_col0[9], s_colpre[9];
    BandCell *band = reinterpret_cast<BandCell *>(sm + PSmem::BAND);
    int *fr0 = reinterpret_cast<int *>(sm + PSmem::FR), *fr1 = fr0 + FRONTIER_CAP;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nxt = (d.glob->epoch + 1) & 1;
    const double *X = d.X[nxt], *Y = d.Y[nxt], *Mm = d.M[nxt];
    const long long nitems = d.item_off[d.NG_total];
    __shared__ int s_stop;
    for (long long it = item_offset + (long long)blockIdx.x * item_stride; it < nitems;
         it += (long long)gridDim.x * item_stride) {
        // one thread decides for the whole block (every thread must take the same branch)
        if (tid == 0) s_stop = *(volatile unsigned *)counter >= capacity;
        __syncthreads();
        const bool stop = s_stop != 0;
        __syncthreads();
        if (stop) break;
        const long long g = d.item_group[it];
        ItemGeom ig;
        item_geom(d, g, (int)(it - d.item_off[g]), s_col0, s_colpre, ig);
        bool of;
        const int nb = band_walk(d, ig, th2_hi, th2_lo, max_level, band, fr0, fr1, sh_scan, &of);
        const SysDesc &sd = d.sys[ig.s];
        const SysDyn &dy = d.dyn[ig.s];
        const int nt = min(tpi, ig.T);
        const int npair = nt * nb;
        for (int p = warp; p < npair; p += LT / 32) {
            const int tsel = p / nb, k = p - tsel * nb;
            const int ti = item_target(ig, s_col0, s_colpre, (int)((long long)tsel * ig.T / nt));
            const double xt = X[ti], yt = Y[ti];
            const BandCell bc = band[k];
            // cell geometry from its index
            const long long loc_all = bc.cell - sd.coff;
            int l = 0;
            while (l + 1 < sd.L && sd.lvoff[l + 1] <= loc_all) l++;
            const long long loc = loc_all - sd.lvoff[l];
            const int ci = (int)(loc / sd.lvg[l]), cj = (int)(loc - (long long)ci * sd.lvg[l]);
            const int kx0 = ci << l, kx1 = min(sd.G, (ci + 1) << l);
            const int ky0 = cj << l, ky1 = min(sd.G, (cj + 1) << l);
            double sx = 0.0, sy = 0.0;
            for (int kx = kx0; kx < kx1; kx++) {
                const long long b0 = sd.boff + (long long)kx * sd.G;
                const int st = d.box_start[b0 + ky0], en = d.box_start[b0 + ky1];
                for (int j = st + lane; j < en; j += 32) {
                    double dx = X[j] - xt, dyy = Y[j] - yt;
                    double w = Mm[j] / (dx * dx + dyy * dyy + d.eps2);
                    sx += w * dx;
                    sy += w * dyy;
                }
            }
            for (int o = 16; o; o >>= 1) {
                sx += __shfl_xor_sync(0xffffffffu, sx, o);
                sy += __shfl_xor_sync(0xffffffffu, sy, o);
            }
            if (lane == 0) {
                const double *q = d.mom + 6 * (long long)bc.cell;
                const double M = q[0];
                const double cx = box_origin(dy.minx, kx0, dy.step) + q[1] / M;
                const double cy = box_origin(dy.miny, ky0, dy.step) + q[2] / M;
                const double dx = cx - xt, dyy = cy - yt;
                const double w = M / (dx * dx + dyy * dyy + d.eps2);
                const double s = (double)(1 << l) * dy.step;
                const double rx = (sx - w * dx) * s / M, ry = (sy - w * dyy) * s / M;
                unsigned row = atomicAdd(counter, 1u);
                if (row < capacity) {
                    const double u = dx / s, v = dyy / s;
                    float *f = feats + 8 * (long long)row;
                    f[0] = (float)u;
                    f[1] = (float)v;
                    f[2] = bc.qxx;
                    f[3] = bc.qxy;
                    f[4] = bc.qyy;
                    f[5] = (float)(1.0 / sqrt(u * u + v * v));
                    f[6] = (float)l;
                    f[7] = 0.f;
                    targets[2 * (long long)row] = (float)rx;
                    targets[2 * (long long)row + 1] = (float)ry;
                }
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------------ launches
cudaError_t learned_init() {
    cudaError_t e = cudaFuncSetAttribute(k_learned_correct, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         LSmem::TOTAL + 1024);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_learned_pairs, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                PSmem::TOTAL + 16);
}

cudaError_t launch_learned_correct(const DevPlan &d, double theta_lo, const uint8_t *img,
                                   const float *params, bool tick, cudaStream_t st) {
    if (d.n_total == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(&d.glob->item_next2, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    long long items_max = d.NG_total + d.n_total / d.chunk + 1;
    long long grid = (long long)d.nsm * 2;
    if (grid > items_max) grid = items_max;
    k_learned_correct<<<(unsigned)grid, LT, LSmem::TOTAL + 1024, st>>>(
        d, (float)(theta_lo * theta_lo), img, params, tick ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_learned_pairs(const DevPlan &d, double theta_hi, double theta_lo, int max_level,
                                 long long item_offset, long long item_stride, int tpi,
                                 float *feats, float *targets, unsigned *counter, long long capacity,
                                 cudaStream_t st) {
    if (d.n_total == 0) return cudaSuccess;
    k_learned_pairs<<<d.nsm * 4, LT, PSmem::TOTAL + 16, st>>>(
        d, (float)(theta_hi * theta_hi), (float)(theta_lo * theta_lo), max_level, item_offset,
        item_stride, tpi, feats, targets, counter, capacity);
    return cudaGetLastError();
}

}  // namespace bh

// bh_fstream.cu -- list-streaming force evaluation with the tick fused into its epilogue.
//
// Replaces g_evaluate_boxes (python-bh/barneshut/kernels/grid_decomposition/gpu/grid.py:116-157)
// and, fused, g_tick_particles (gpu/grid.py:159-174) for the theta-mode production case: FP32
// pair arithmetic (plain or Kahan-compensated far field), Plummer softening > 0, no r^2 cutoff.
// The interaction lists come from k_lists (one pyramid walk per target group); this kernel only
// streams them.
//
// Work items are a group's targets split into near-equal chunks of at most STREAM_CHUNK, pulled
// from a device queue.  Per item:
//   * far field: the group's far codes are decoded (level, cell -> record; centre of mass shifted
//     into the group frame) into shared memory as packed (x, x, y, y) + (M, M) entries, FAR_CAP
//     at a time, and swept with Kahan compensation;
//   * near field: the near boxes' 32-byte packed records (x, x, y, y), (m, m, index, 0) are copied
//     box by box into shared memory by bulk asynchronous copies (TMA) completing on one mbarrier,
//     SRC_CAP sources per pass, and swept box piece by box piece with the piece's shift folded
//     into the targets (the slices split every piece, so the CTA's warps stay converged).
// Each thread owns FORCE_R targets as two packed pairs (one f32x2 instruction serves two targets);
// the CTA's threads form slices that sweep disjoint parts of every staged list, and the slice
// partials are reduced in shared memory before the FP64 write-back and the fused tick.
#include "bh_internal.cuh"
#include "bh_pairs.cuh"
#include "bh_tc.cuh"

namespace bh {

constexpr int NR = FORCE_R;
constexpr size_t FS_SMEM = (size_t)FAR_CAP * 24 + (size_t)SRC_CAP * 32 + (size_t)(NEAR_CAP + 1) * 16;
static_assert(2 * FT * NR * sizeof(float) <= (size_t)FAR_CAP * 24, "slice partials alias the far staging");
static_assert(FT * NR >= STREAM_CHUNK, "a CTA must cover every target of a work item");

template <bool KAHAN, int MINB>
__global__ void __launch_bounds__(FT, MINB) k_fstream(DevPlan d, int tick, int accumulate) {
    extern __shared__ __align__(128) unsigned char smem[];
    float4 *farxy = reinterpret_cast<float4 *>(smem);                 // FAR_CAP x (x, x, y, y)
    float2 *farm = reinterpret_cast<float2 *>(farxy + FAR_CAP);       // FAR_CAP x (M, M)
    unsigned char *src = smem + FAR_CAP * 24;                         // SRC_CAP x 32 bytes
    float2 *nshift = reinterpret_cast<float2 *>(src + SRC_CAP * 32);  // NEAR_CAP + 1
    int *nbox = reinterpret_cast<int *>(nshift + NEAR_CAP + 1);       // first particle of a box
    int *npre = nbox + NEAR_CAP + 1;                                  // NEAR_CAP + 1
    float *red = reinterpret_cast<float *>(smem);                     // aliases farxy / farm
    __shared__ uint64_t s_mbar;  // completion of the near-source bulk copies
    __shared__ int s_item;
    __shared__ int s_col0[MAX_TG + 1], s_colpre[MAX_TG + 1];

    const int tid = threadIdx.x;
    const int nxt = (d.glob->epoch + 1) & 1;
    const double *Xs = d.X[nxt], *Ys = d.Y[nxt];
    const long long nitems = d.item_off[d.NG_total];
    unsigned long long npairs = 0, fpairs = 0;  // counted by thread 0
    uint32_t tphase = 0;                        // parity of s_mbar's current phase
    bool tma_ok = true;  // block-uniform; cleared (and flagged) when a copy wait times out
    if (tid == 0) {
        tc::mbar_init(&s_mbar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    for (;;) {
        if (tid == 0) s_item = (int)atomicAdd(&d.glob->item_next, 1u);
        __syncthreads();
        const int item = s_item;
        if (item >= nitems) break;
        const long long g = d.item_group[item];
        const int chunk = item - d.item_off[g];
        const int s = find_seg(d.goff_tab, d.nsys, g);
        const SysDesc &sd = d.sys[s];
        const SysDyn &dy = d.dyn[s];
        const long long lg = g - sd.goff;
        const int TG = sd.TG, G = sd.G;
        const int gi = (int)(lg / sd.NGs), gj = (int)(lg - (long long)gi * sd.NGs);
        const int gx0 = gi * TG, gy0 = gj * TG;
        const int gx1 = min(G, gx0 + TG), gy1 = min(G, gy0 + TG);
        const int ncol = gx1 - gx0;
        if (tid < ncol) {
            const long long b0 = sd.boff + (long long)(gx0 + tid) * G + gy0;
            const int st = d.box_start[b0];
            s_col0[tid] = st;
            s_colpre[tid + 1] = d.box_start[b0 + (gy1 - gy0)] - st;
        }
        __syncthreads();
        if (tid == 0) {
            s_colpre[0] = 0;
            for (int c = 1; c <= ncol; c++) s_colpre[c] += s_colpre[c - 1];
        }
        __syncthreads();
        const int nt = s_colpre[ncol];
        int c0, T;
        item_range(nt, d.item_cnt[g], chunk, &c0, &T);
        const float step_f = __double2float_rn(dy.step);
        const float eps2 = d.eps2_f;

        // ---- thread -> (slice, NR targets)
        const int nthr = (T + NR - 1) / NR;
        const int nslice = FT / nthr;
        const bool active = tid < nslice * nthr;
        const int slice = active ? tid / nthr : 0, tl = active ? tid % nthr : 0;
        int ti[NR];
        bool tv[NR];
        float tx[NR], ty[NR];
#pragma unroll
        for (int r = 0; r < NR; r++) {
            const int v = tl * NR + r;
            tv[r] = v < T;
            const int u = c0 + (tv[r] ? v : 0);
            int c = 0;
            while (c + 1 < ncol && s_colpre[c + 1] <= u) c++;
            ti[r] = s_col0[c] + (u - s_colpre[c]);
            const float4 p = d.P[ti[r]];
            const int lb = d.skey[ti[r]] - (int)sd.boff;
            const int kx = lb / G, ky = lb - kx * G;
            tx[r] = __fadd_rn(__fmul_rn((float)(kx - gx0), step_f), p.x);
            ty[r] = __fadd_rn(__fmul_rn((float)(ky - gy0), step_f), p.y);
        }
        // negated target coordinates, near accumulators, far sums and compensations, in pairs
        f2_t ntx2[NR / 2], nty2[NR / 2], nax2[NR / 2], nay2[NR / 2];
        f2_t fsx2[NR / 2], fsy2[NR / 2], fcx2[NR / 2], fcy2[NR / 2];
        const f2_t eps2x2 = f2_pack(eps2, eps2);
        const f2_t m1x2 = f2_pack(-1.f, -1.f);
#pragma unroll
        for (int k = 0; k < NR / 2; k++) {
            ntx2[k] = f2_pack(-tx[2 * k], -tx[2 * k + 1]);
            nty2[k] = f2_pack(-ty[2 * k], -ty[2 * k + 1]);
            nax2[k] = nay2[k] = f2_pack(0.f, 0.f);
            fsx2[k] = fsy2[k] = fcx2[k] = fcy2[k] = f2_pack(0.f, 0.f);
        }
        const int2 cnt = d.lcnt[g];
        const int *lf = d.lfar + sd.lfoff + lg * sd.lfcap;
        const int4 *ln = d.lnear + sd.lnoff + lg * (sd.lncap + 1);

        // ---- far field
        for (int f0 = 0; f0 < cnt.x; f0 += FAR_CAP) {
            const int nf = min(FAR_CAP, cnt.x - f0);
            for (int k = tid; k < nf; k += FT) {
                const unsigned code = (unsigned)lf[f0 + k];
                const int l = (int)(code >> 28), loc = (int)(code & 0x0FFFFFFFu);
                const int gl = sd.lvg[l];
                const int ci = loc / gl, cj = loc - ci * gl;
                const float4 rr = d.rec[sd.coff + sd.lvoff[l] + loc];
                const float rx = __fadd_rn(__fmul_rn((float)((ci << l) - gx0), step_f), rr.x);
                const float ry = __fadd_rn(__fmul_rn((float)((cj << l) - gy0), step_f), rr.y);
                farxy[k] = make_float4(rx, rx, ry, ry);
                farm[k] = make_float2(rr.z, rr.z);
            }
            __syncthreads();
            if (active) {
                const ulonglong2 *fp = reinterpret_cast<const ulonglong2 *>(farxy);
                const f2_t *fm = reinterpret_cast<const f2_t *>(farm);
                for (int k = slice; k < nf; k += nslice) {
                    const ulonglong2 rxy = fp[k];  // (rx, rx), (ry, ry)
                    const f2_t mm = fm[k];         // (M, M)
#pragma unroll
                    for (int kk = 0; kk < NR / 2; kk++) {
                        const f2_t dx = f2_add(rxy.x, ntx2[kk]), dyy = f2_add(rxy.y, nty2[kk]);
                        const f2_t w = f2_mul(mm, f2_rcp(f2_fma(dx, dx, f2_fma(dyy, dyy, eps2x2))));
                        const f2_t fx = f2_mul(w, dx), fy = f2_mul(w, dyy);
                        if (KAHAN) {  // y = f - c; t = s + y; c = (t - s) - y; s = t
                            const f2_t yx = f2_fma(fcx2[kk], m1x2, fx), t1 = f2_add(fsx2[kk], yx);
                            fcx2[kk] = f2_fma(yx, m1x2, f2_fma(fsx2[kk], m1x2, t1));
                            fsx2[kk] = t1;
                            const f2_t yy = f2_fma(fcy2[kk], m1x2, fy), t2 = f2_add(fsy2[kk], yy);
                            fcy2[kk] = f2_fma(yy, m1x2, f2_fma(fsy2[kk], m1x2, t2));
                            fsy2[kk] = t2;
                        } else {
                            fsx2[kk] = f2_add(fsx2[kk], fx);
                            fsy2[kk] = f2_add(fsy2[kk], fy);
                        }
                    }
                }
            }
            fpairs += (unsigned long long)T * nf;
            __syncthreads();  // farxy / farm are restaged by the next pass
        }
        // compensated far sums s - c; the compensations are dead from here on
#pragma unroll
        for (int kk = 0; kk < NR / 2; kk++) {
            fsx2[kk] = f2_fma(fcx2[kk], m1x2, fsx2[kk]);
            fsy2[kk] = f2_fma(fcy2[kk], m1x2, fsy2[kk]);
        }

        // ---- near field: boxes in batches of NEAR_CAP, sources in bulk-copy passes of SRC_CAP.
        // Descriptor k of the group's near list is (first particle, exclusive prefix of the
        // particle counts, shift of the box origin in the group frame); entry nnb holds the total.
        for (int b0 = 0; b0 < cnt.y && tma_ok; b0 += NEAR_CAP) {
            const int nn = min(NEAR_CAP, cnt.y - b0);
            for (int k = tid; k <= nn; k += FT) {
                const int4 e = ln[b0 + k];
                nbox[k] = e.x;
                npre[k] = e.y;
                nshift[k] = make_float2(__int_as_float(e.z), __int_as_float(e.w));
            }
            __syncthreads();
            const int pend = npre[nn];
            int kfirst = 0;  // first box of the batch overlapping the current pass (block-uniform)
            for (int s0 = npre[0]; s0 < pend; s0 += SRC_CAP) {
                const int ns = min(SRC_CAP, pend - s0);
                // every box piece inside [s0, s0 + ns) is one bulk copy; all complete on s_mbar
                if (tid == 0) tc::mbar_expect_tx(&s_mbar, (uint32_t)ns * 32u);
                tc::fence_async_smem();
                for (int k = tid; k < nn; k += FT) {
                    const int lo = max(npre[k], s0), hi = min(npre[k + 1], s0 + ns);
                    if (lo < hi)
                        tc::bulk_g2s(src + 32 * (lo - s0), d.PD + 2 * (long long)(nbox[k] + (lo - npre[k])),
                                     (uint32_t)(hi - lo) * 32u, &s_mbar);
                }
                const bool ok = tc::mbar_wait(&s_mbar, tphase);
                tphase ^= 1u;
                if (!__syncthreads_and(ok ? 1 : 0)) {
                    // flagged; give the copies in flight a second bounded wait, then stage
                    // nothing more in this launch (the barrier phase is no longer known)
                    if (tid == 0) raise_err(d.glob, 8u /*BH_DEV_WAIT_TIMEOUT*/);
                    tc::mbar_wait(&s_mbar, tphase ^ 1u);
                    tma_ok = false;
                    __syncthreads();
                    break;
                }
                while (kfirst + 1 < nn && npre[kfirst + 1] <= s0) kfirst++;
                if (active) {
                    // every thread walks the same box pieces; the slices split each piece, and
                    // the piece's shift is folded into the (negated) target coordinates
                    const float4 *s4 = reinterpret_cast<const float4 *>(src);
                    for (int k = kfirst; k < nn && npre[k] < s0 + ns; k++) {
                        const int lo = max(npre[k], s0) - s0, hi = min(npre[k + 1], s0 + ns) - s0;
                        const float2 sh = nshift[k];
                        const f2_t shx = f2_pack(sh.x, sh.x), shy = f2_pack(sh.y, sh.y);
                        f2_t bx[NR / 2], by[NR / 2];
#pragma unroll
                        for (int kk = 0; kk < NR / 2; kk++) {
                            bx[kk] = f2_add(ntx2[kk], shx);
                            by[kk] = f2_add(nty2[kk], shy);
                        }
#pragma unroll 2
                        for (int j = lo + slice; j < hi; j += nslice) {
                            const ulonglong2 sxy = *reinterpret_cast<const ulonglong2 *>(s4 + 2 * j);
                            const f2_t mm = *reinterpret_cast<const f2_t *>(s4 + 2 * j + 1);
#pragma unroll
                            for (int kk = 0; kk < NR / 2; kk++) {
                                const f2_t dx = f2_add(sxy.x, bx[kk]), dyy = f2_add(sxy.y, by[kk]);
                                const f2_t r2 = f2_fma(dx, dx, f2_fma(dyy, dyy, eps2x2));
                                const f2_t w = f2_mul(mm, f2_rcp(r2));
                                nax2[kk] = f2_fma(w, dx, nax2[kk]);
                                nay2[kk] = f2_fma(w, dyy, nay2[kk]);
                            }
                        }
                    }
                }
                npairs += (unsigned long long)T * ns;
                __syncthreads();  // the staging buffer is refilled by the next pass
            }
            __syncthreads();  // the descriptors are rewritten by the next batch
        }
        __syncthreads();  // red aliases the far staging

        // ---- reduce slice partials and write
        if (active) {
#pragma unroll
            for (int k = 0; k < NR / 2; k++) {
                float a0, a1, b0, b1, s0, s1, t0, t1;
                f2_unpack(nax2[k], a0, a1);
                f2_unpack(nay2[k], b0, b1);
                f2_unpack(fsx2[k], s0, s1);
                f2_unpack(fsy2[k], t0, t1);
                float *o = red + 2 * ((slice * nthr + tl) * NR + 2 * k);
                o[0] = a0 + s0;
                o[1] = b0 + t0;
                o[2] = a1 + s1;
                o[3] = b1 + t1;
            }
        }
        __syncthreads();
        if (active && slice == 0) {
#pragma unroll
            for (int r = 0; r < NR; r++) {
                if (!tv[r]) continue;
                float sx = 0.f, sy = 0.f;
                for (int k = 0; k < nslice; k++) {
                    const float *o = red + 2 * ((k * nthr + tl) * NR + r);
                    sx += o[0];
                    sy += o[1];
                }
                const int t = ti[r];
                double ax = d.gconst * (double)sx, ay = d.gconst * (double)sy;
                if (accumulate) {
                    ax += d.AX[t];
                    ay += d.AY[t];
                }
                d.AX[t] = ax;
                d.AY[t] = ay;
                if (tick) {
                    const double vx = d.VX[nxt][t] + ax * d.dt, vy = d.VY[nxt][t] + ay * d.dt;
                    d.VX[nxt][t] = vx;
                    d.VY[nxt][t] = vy;
                    d.X[nxt][t] = Xs[t] + vx * d.dt;
                    d.Y[nxt][t] = Ys[t] + vy * d.dt;
                }
            }
        }
        __syncthreads();  // red and s_item are reused by the next item
    }
    if (tid == 0) {
        atomicAdd(&d.glob->near_pairs, npairs);
        atomicAdd(&d.glob->far_pairs, fpairs);
    }
}

template <bool KAHAN, int MINB>
static cudaError_t launch_fstream_t(const DevPlan &d, bool tick, bool accumulate, cudaStream_t st) {
    long long items_max = d.NG_total + d.n_total / d.chunk + 1;
    long long grid = 152LL * MINB;
    if (grid > items_max) grid = items_max;
    if (grid < 1) grid = 1;
    cudaError_t e = cudaMemsetAsync(&d.glob->item_next, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    k_fstream<KAHAN, MINB><<<(unsigned)grid, FT, FS_SMEM, st>>>(d, tick ? 1 : 0, accumulate ? 1 : 0);
    return cudaGetLastError();
}

template <bool KAHAN, int MINB>
static cudaError_t init_fstream_t() {
    return cudaFuncSetAttribute(k_fstream<KAHAN, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)FS_SMEM);
}

cudaError_t fstream_init() {
    cudaError_t e;
    if ((e = init_fstream_t<true, 8>()) != cudaSuccess) return e;
    if ((e = init_fstream_t<true, 6>()) != cudaSuccess) return e;
    if ((e = init_fstream_t<false, 8>()) != cudaSuccess) return e;
    return init_fstream_t<false, 6>();
}

cudaError_t launch_fstream(const DevPlan &d, bool tick, bool accumulate, cudaStream_t st) {
    if (d.n_total == 0) return cudaSuccess;
    if (d.prec == 1)
        return d.tune == 1 ? launch_fstream_t<true, 6>(d, tick, accumulate, st)
                           : launch_fstream_t<true, 8>(d, tick, accumulate, st);
    return d.tune == 1 ? launch_fstream_t<false, 6>(d, tick, accumulate, st)
                       : launch_fstream_t<false, 8>(d, tick, accumulate, st);
}

}  // namespace bh

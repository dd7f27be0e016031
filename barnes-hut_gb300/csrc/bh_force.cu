// bh_force.cu -- box-tiled force evaluation with the tick fused into its epilogue.
//
// Replaces g_evaluate_boxes (python-bh/barneshut/kernels/grid_decomposition/gpu/grid.py:116-157,
// with d_self_self_grav / d_self_other_grav / d_self_COM_grav at :211-268) and, when the tick is
// fused, g_tick_particles (gpu/grid.py:159-174).  The interaction semantics follow the reference
// CPU path (kernels/grid_decomposition/sequential/evaluation.py:73-109 with
// kernels/gravity/cpu_numba.py:30-92) in flat mode, and this project's opening-angle rule in
// theta mode.
//
// Work decomposition: a target group is TG x TG leaf boxes; its nt targets are split into work
// items of at most TARGET_CHUNK targets (built after the box scan), which CTAs pull from a device
// queue, so dense groups spread over many SMs.  Per item the CTA walks the cell pyramid level by
// level (every thread tests one frontier cell; accepted cells, rejected leaves and children are
// compacted with a block scan, so list order is deterministic), stages far entries (centre of
// mass in the group frame, mass) and near-box particles (float4 shifted into the group frame) in
// shared memory, and evaluates them: each thread owns R targets in registers and sweeps a slice of
// the staged entries (one shared-memory load feeds R pair interactions).  Lists that outgrow
// shared memory are evaluated and emptied on the fly; slice partials are reduced in shared memory.
//
// Pair arithmetic: a += m_j (x_j - x_t) * rcp(r^2 + eps^2) in FP32 (rcp.approx), far-field
// contributions Kahan-compensated when requested; BH_PREC_FP64 runs the same lists in FP64.
// Positions are box-relative offsets rounded once from FP64, so dx keeps ~1e-7 of a box edge.
#include "bh_internal.cuh"
#include "bh_pairs.cuh"
#include "bh_tc.cuh"

namespace bh {

template <typename R> struct Src;
template <> struct Src<float> { using T = float4; };
template <> struct Src<double> { struct T { double x, y, m; int idx, pad; }; };

template <typename R> __device__ __forceinline__ R rinv(R x);
template <> __device__ __forceinline__ float rinv<float>(float x) { return rcp_approx(x); }
template <> __device__ __forceinline__ double rinv<double>(double x) { return 1.0 / x; }

__device__ __forceinline__ void src_get(const float4 &e, float &x, float &y, float &m, int &idx) {
    x = e.x; y = e.y; m = e.z; idx = __float_as_int(e.w);
}
__device__ __forceinline__ void src_get(const Src<double>::T &e, double &x, double &y, double &m,
                                        int &idx) {
    x = e.x; y = e.y; m = e.m; idx = e.idx;
}


// bytes per staged far entry: the record, or (x, x, y, y) + (M, M) for the packed path
template <typename R> __host__ __device__ constexpr int far_bytes() {
    return sizeof(typename Src<R>::T) > 24 ? (int)sizeof(typename Src<R>::T) : 24;
}
// bytes per staged near source: the record, or the 32-byte PD record (x, x, y, y), (m, m, i, box)
template <typename R> __host__ __device__ constexpr int src_bytes() {
    return sizeof(typename Src<R>::T) > 32 ? (int)sizeof(typename Src<R>::T) : 32;
}

template <typename R, int NR, bool KAHAN, bool TEST, bool EXACT, int MINB>
__global__ void __launch_bounds__(FT, MINB)
k_force(DevPlan d, int tick, int accumulate) {
    using S = typename Src<R>::T;
    // packed FP32 near field (no cutoff test): sources staged as (x, x, y, y) + (m, m)
    constexpr bool PACKED = sizeof(R) == 4 && !TEST && NR % 2 == 0;
    extern __shared__ __align__(16) unsigned char smem[];
    S *far = reinterpret_cast<S *>(smem);                     // FAR_CAP x far_bytes<R>()
    float2 *farm = reinterpret_cast<float2 *>(reinterpret_cast<float4 *>(far) + FAR_CAP);
    S *src = reinterpret_cast<S *>(smem + FAR_CAP * far_bytes<R>());  // SRC_CAP x src_bytes<R>()
    __shared__ uint64_t s_mbar;  // bulk-copy completion of the near-source staging
    R *red = reinterpret_cast<R *>(smem);                     // aliases far/src at the end
    float2 *nshift = reinterpret_cast<float2 *>(reinterpret_cast<unsigned char *>(src) +
                                                SRC_CAP * src_bytes<R>());  // NEAR_CAP
    int *nbox = reinterpret_cast<int *>(nshift + NEAR_CAP);   // first particle of near box
    int *ncnt = nbox + NEAR_CAP;
    int *npre = ncnt + NEAR_CAP;                              // NEAR_CAP + 4
    int *front0 = npre + NEAR_CAP + 4;                        // FR_CAP
    int *front1 = front0 + FR_CAP;                            // FR_CAP
    __shared__ int sh_scan[32];
    __shared__ int s_item;
    __shared__ int s_col0[MAX_TG + 1], s_colpre[MAX_TG + 1];

    const int tid = threadIdx.x;
    const int nxt = (d.glob->epoch + 1) & 1;
    const double *Xs = d.X[nxt], *Ys = d.Y[nxt], *Ms = d.M[nxt];
    const long long nitems = d.item_off[d.NG_total];
    unsigned long long npairs = 0, fpairs = 0;  // counted by thread 0
    uint32_t tphase = 0;                        // parity of s_mbar's current phase
    bool tma_ok = true;  // block-uniform; cleared (and flagged) when a staging wait times out
    if (PACKED) {
        if (tid == 0) {
            tc::mbar_init(&s_mbar, 1);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        __syncthreads();
    }

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
            long long b0 = sd.boff + (long long)(gx0 + tid) * G + gy0;
            int st = d.box_start[b0];
            s_col0[tid] = st;
            s_colpre[tid + 1] = d.box_start[b0 + (gy1 - gy0)] - st;
        }
        __syncthreads();
        if (tid == 0) {
            s_colpre[0] = 0;
            for (int c = 1; c <= ncol; c++) s_colpre[c] += s_colpre[c - 1];
        }
        __syncthreads();
        // list counters: block-uniform registers, advanced by every thread from the
        // block scan's totals (no shared counter, no extra barrier)
        int nfar = 0, nnear = 0, nnext = 0;
        bool ovf = false;
        const int nt = s_colpre[ncol];
        int c0, T;
        item_range(nt, d.item_cnt[g], chunk, &c0, &T);
        const float step_f = __double2float_rn(dy.step);
        const float W_f = __fmul_rn((float)TG, step_f);
        const double gox = box_origin(dy.minx, gx0, dy.step), goy = box_origin(dy.miny, gy0, dy.step);
        const R eps2 = (R)(sizeof(R) == 4 ? (double)d.eps2_f : d.eps2);
        const R cut = (R)(sizeof(R) == 4 ? (double)d.cut_f : d.cutoff);

        // ---- thread -> (slice, NR targets)
        const int nthr = (T + NR - 1) / NR;
        const int nslice = FT / nthr;
        const bool active = tid < nslice * nthr;
        const int slice = active ? tid / nthr : 0, tl = active ? tid % nthr : 0;
        int ti[NR];
        R tx[NR], ty[NR];
        double txd[NR], tyd[NR];
        bool tv[NR];
#pragma unroll
        for (int r = 0; r < NR; r++) {
            int v = tl * NR + r;
            tv[r] = v < T;
            int u = c0 + (tv[r] ? v : 0), c = 0;
            while (c + 1 < ncol && s_colpre[c + 1] <= u) c++;
            ti[r] = s_col0[c] + (u - s_colpre[c]);
            if (sizeof(R) == 4) {
                const float4 p = d.PD[2 * (long long)ti[r]];  // (x, x, y, y) box-relative
                int lb = d.skey[ti[r]] - (int)sd.boff;
                int kx = lb / G, ky = lb - kx * G;
                tx[r] = (R)__fadd_rn(__fmul_rn((float)(kx - gx0), step_f), p.x);
                ty[r] = (R)__fadd_rn(__fmul_rn((float)(ky - gy0), step_f), p.z);
            } else {
                tx[r] = (R)(Xs[ti[r]] - gox);
                ty[r] = (R)(Ys[ti[r]] - goy);
            }
            txd[r] = EXACT ? Xs[ti[r]] : 0.0;
            tyd[r] = EXACT ? Ys[ti[r]] : 0.0;
        }
        R anx[NR], any_[NR], afx[NR], afy[NR], acx[NR], acy[NR];
#pragma unroll
        for (int r = 0; r < NR; r++) anx[r] = any_[r] = afx[r] = afy[r] = acx[r] = acy[r] = 0;
        // packed near-field state: negated target coordinates and accumulators, pairs of targets
        f2_t ntx2[NR / 2], nty2[NR / 2], nax2[NR / 2], nay2[NR / 2];
        // packed far-field sums and Kahan compensations
        f2_t fsx2[NR / 2], fsy2[NR / 2], fcx2[NR / 2], fcy2[NR / 2];
        const f2_t eps2x2 = f2_pack((float)eps2, (float)eps2);
        const f2_t m1x2 = f2_pack(-1.f, -1.f);
        if (PACKED) {
#pragma unroll
            for (int k = 0; k < NR / 2; k++) {
                ntx2[k] = f2_pack(-(float)tx[2 * k], -(float)tx[2 * k + 1]);
                nty2[k] = f2_pack(-(float)ty[2 * k], -(float)ty[2 * k + 1]);
                nax2[k] = nay2[k] = f2_pack(0.f, 0.f);
                fsx2[k] = fsy2[k] = fcx2[k] = fcy2[k] = f2_pack(0.f, 0.f);
            }
        }

        // 1 / (r^2 + eps^2) with the cutoff predicate on the unsoftened r^2
        auto pair_inv = [&](R dx, R dyy, int r, int sidx) -> R {
            if (!TEST) return rinv<R>(dx * dx + (dyy * dyy + eps2));
            R r2 = dx * dx + dyy * dyy;
            R inv = rinv<R>(r2 + eps2);
            bool keep = r2 > cut;
            if (EXACT && sidx >= 0) {
                R band = cut * (R)1e-3;
                R diff = r2 - cut;
                if (diff <= band && diff >= -band) {
                    double ex = __dsub_rn(txd[r], Xs[sidx]), ey = __dsub_rn(tyd[r], Ys[sidx]);
                    double e2 = __dmul_rn(ex, ex);
                    e2 = __dadd_rn(e2, __dmul_rn(ey, ey));
                    keep = e2 > d.cutoff;
                }
            }
            return keep ? inv : (R)0;
        };

        // evaluate and empty the far list (entries were written before the last barrier of
        // the block scan that appended them; the next append's scan barriers order the reuse)
        auto flush_far = [&]() {
            __syncthreads();
            const int nf = nfar;
            if (active && PACKED) {
                const ulonglong2 *fp = reinterpret_cast<const ulonglong2 *>(far);
                const f2_t *fm = reinterpret_cast<const f2_t *>(farm);
                for (int k = slice; k < nf; k += nslice) {
                    const ulonglong2 rxy = fp[k];  // (rx, rx), (ry, ry)
                    const f2_t mm = fm[k];         // (M, M)
#pragma unroll
                    for (int kk = 0; kk < NR / 2; kk++) {
                        f2_t dx = f2_add(rxy.x, ntx2[kk]), dyy = f2_add(rxy.y, nty2[kk]);
                        f2_t w = f2_mul(mm, f2_rcp(f2_fma(dx, dx, f2_fma(dyy, dyy, eps2x2))));
                        f2_t fx = f2_mul(w, dx), fy = f2_mul(w, dyy);
                        if (KAHAN) {  // y = f - c; t = s + y; c = (t - s) - y; s = t
                            f2_t yx = f2_fma(fcx2[kk], m1x2, fx), t1 = f2_add(fsx2[kk], yx);
                            fcx2[kk] = f2_fma(yx, m1x2, f2_fma(fsx2[kk], m1x2, t1));
                            fsx2[kk] = t1;
                            f2_t yy = f2_fma(fcy2[kk], m1x2, fy), t2 = f2_add(fsy2[kk], yy);
                            fcy2[kk] = f2_fma(yy, m1x2, f2_fma(fsy2[kk], m1x2, t2));
                            fsy2[kk] = t2;
                        } else {
                            fsx2[kk] = f2_add(fsx2[kk], fx);
                            fsy2[kk] = f2_add(fsy2[kk], fy);
                        }
                    }
                }
            } else if (active) {
                for (int k = slice; k < nf; k += nslice) {
                    R sx, sy, sm;
                    int sidx;
                    src_get(far[k], sx, sy, sm, sidx);
#pragma unroll
                    for (int r = 0; r < NR; r++) {
                        R dx = sx - tx[r], dyy = sy - ty[r];
                        R w = sm * pair_inv(dx, dyy, r, -1);
                        R fx = w * dx, fy = w * dyy;
                        if (KAHAN) {
                            R yx = fx - acx[r], t1 = afx[r] + yx;
                            acx[r] = (t1 - afx[r]) - yx;
                            afx[r] = t1;
                            R yy = fy - acy[r], t2 = afy[r] + yy;
                            acy[r] = (t2 - afy[r]) - yy;
                            afy[r] = t2;
                        } else {
                            afx[r] += fx;
                            afy[r] += fy;
                        }
                    }
                }
            }
            fpairs += (unsigned long long)T * nf;
            nfar = 0;
        };

        auto flush_near = [&]() {
            __syncthreads();
            const int nn = nnear;
            int total;
            {
                constexpr int IT = NEAR_CAP / FT;
                int v[IT], sum = 0;
#pragma unroll
                for (int k = 0; k < IT; k++) {
                    int e = tid * IT + k;
                    v[k] = e < nn ? ncnt[e] : 0;
                    sum += v[k];
                }
                int pre = block_scan(sum, sh_scan, &total);
#pragma unroll
                for (int k = 0; k < IT; k++) {
                    int e = tid * IT + k;
                    if (e < nn) npre[e] = pre;
                    pre += v[k];
                }
                if (tid == 0) npre[nn] = total;
            }
            __syncthreads();
            for (int s0 = 0; s0 < total && tma_ok; s0 += SRC_CAP) {
                const int ns = min(SRC_CAP, total - s0);
                if (PACKED) {
                    // Bulk copies (TMA) of the 32-byte PD records of every near-box piece
                    // that falls into [s0, s0 + ns), all completing on one mbarrier phase.
                    if (tid == 0) tc::mbar_expect_tx(&s_mbar, (uint32_t)ns * 32u);
                    tc::fence_async_smem();
                    unsigned char *sbase = reinterpret_cast<unsigned char *>(src);
                    for (int k = tid; k < nn; k += FT) {
                        const int lo = max(npre[k], s0), hi = min(npre[k] + ncnt[k], s0 + ns);
                        if (lo < hi)
                            tc::bulk_g2s(sbase + 32 * (lo - s0), d.PD + 2 * (long long)(nbox[k] + (lo - npre[k])),
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
                    // a slice takes an equal contiguous range [j0, j1) of the staged sources and
                    // walks the boxes it overlaps; each box's shift is folded into the targets
                    const int per = (ns + nslice - 1) / nslice;
                    const int j0 = min(ns, slice * per), j1 = min(ns, j0 + per);
                    if (active && j0 < j1) {
                        const float4 *s4 = reinterpret_cast<const float4 *>(src);
                        int k = 0;
                        {
                            int hi = nn;  // npre[k] <= s0 + j0 < npre[hi]
                            while (hi - k > 1) {
                                const int mid = (k + hi) >> 1;
                                if (npre[mid] <= s0 + j0) k = mid; else hi = mid;
                            }
                        }
                        for (int lo = j0; lo < j1 && k < nn; k++) {
                            const int hi = min(npre[k] + ncnt[k] - s0, j1);
                            if (lo >= hi) continue;
                            const float2 sh = nshift[k];
                            const f2_t shx = f2_pack(sh.x, sh.x), shy = f2_pack(sh.y, sh.y);
                            f2_t bx[NR / 2], by[NR / 2];
#pragma unroll
                            for (int kk = 0; kk < NR / 2; kk++) {
                                bx[kk] = f2_add(ntx2[kk], shx);
                                by[kk] = f2_add(nty2[kk], shy);
                            }
#pragma unroll 2
                            for (int j = lo; j < hi; j++) {
                                const ulonglong2 sxy = *reinterpret_cast<const ulonglong2 *>(s4 + 2 * j);
                                const f2_t mm = *reinterpret_cast<const f2_t *>(s4 + 2 * j + 1);
#pragma unroll
                                for (int kk = 0; kk < NR / 2; kk++) {
                                    f2_t dx = f2_add(sxy.x, bx[kk]), dyy = f2_add(sxy.y, by[kk]);
                                    f2_t r2 = f2_fma(dx, dx, f2_fma(dyy, dyy, eps2x2));
                                    f2_t w = f2_mul(mm, f2_rcp(r2));
                                    nax2[kk] = f2_fma(w, dx, nax2[kk]);
                                    nay2[kk] = f2_fma(w, dyy, nay2[kk]);
                                }
                            }
                            lo = hi;
                        }
                    }
                    npairs += (unsigned long long)T * ns;
                    __syncthreads();  // the staging buffer is refilled by the next pass
                    continue;
                }
                for (int j = tid; j < ns; j += FT) {
                    int J = s0 + j;
                    int lo = 0, hi = nn;  // npre[lo] <= J < npre[hi]
                    while (hi - lo > 1) {
                        int mid = (lo + hi) >> 1;
                        if (npre[mid] <= J) lo = mid; else hi = mid;
                    }
                    int idx = nbox[lo] + (J - npre[lo]);
                    if (sizeof(R) == 4) {
                        const float4 pxy = d.PD[2 * (long long)idx], pm = d.PD[2 * (long long)idx + 1];
                        float2 sh = nshift[lo];
                        reinterpret_cast<float4 *>(src)[j] =
                            make_float4(__fadd_rn(sh.x, pxy.x), __fadd_rn(sh.y, pxy.z), pm.x, pm.z);
                    } else {
                        typename Src<double>::T q;
                        q.x = Xs[idx] - gox;
                        q.y = Ys[idx] - goy;
                        q.m = Ms[idx];
                        q.idx = idx;
                        q.pad = 0;
                        reinterpret_cast<typename Src<double>::T *>(src)[j] = q;
                    }
                }
                __syncthreads();
                if (active) {
                    for (int j = slice; j < ns; j += nslice) {
                        R sx, sy, sm;
                        int sidx;
                        src_get(src[j], sx, sy, sm, sidx);
#pragma unroll
                        for (int r = 0; r < NR; r++) {
                            R dx = sx - tx[r], dyy = sy - ty[r];
                            R w = sm * pair_inv(dx, dyy, r, sidx);
                            anx[r] += w * dx;
                            any_[r] += w * dyy;
                        }
                    }
                }
                npairs += (unsigned long long)T * ns;
                __syncthreads();  // src is restaged by the next pass
            }
            nnear = 0;
        };

        // kind: 0 none, 1 far, 2 near, 3 open (children into front_next).  One block scan
        // places every thread's entries; all threads advance the counters from its total.
        auto emit = [&](int kind, int id, int l, int ci, int cj, float rx, float ry, float M,
                        int *front_next, int gc) {
            int nch = 0;
            if (kind == 3) nch = (2 * ci + 1 < gc ? 2 : 1) * (2 * cj + 1 < gc ? 2 : 1);
            int packed = (kind == 1 ? 1 : 0) | ((kind == 2 ? 1 : 0) << 10) | (nch << 20);
            int tot;
            int pre = block_scan(packed, sh_scan, &tot);
            if (kind == 1) {
                int pos = nfar + (pre & 1023);
                if (sizeof(R) == 4) {
                    if (PACKED) {
                        reinterpret_cast<float4 *>(far)[pos] = make_float4(rx, rx, ry, ry);
                        farm[pos] = make_float2(M, M);
                    } else {
                        reinterpret_cast<float4 *>(far)[pos] = make_float4(rx, ry, M, __int_as_float(id));
                    }
                } else {
                    const double *q = d.mom + 6 * (long long)id;
                    typename Src<double>::T e;
                    double ox = box_origin(dy.minx, ci << l, dy.step) - gox;
                    double oy = box_origin(dy.miny, cj << l, dy.step) - goy;
                    e.x = ox + q[1] / q[0];
                    e.y = oy + q[2] / q[0];
                    e.m = q[0];
                    e.idx = id;
                    e.pad = 0;
                    reinterpret_cast<typename Src<double>::T *>(far)[pos] = e;
                }
            } else if (kind == 2) {
                int pos = nnear + ((pre >> 10) & 1023);
                int st = d.box_start[id];
                nbox[pos] = st;
                ncnt[pos] = d.box_start[id + 1] - st;
                int lb = id - (int)sd.boff;
                int kx = lb / G, ky = lb - kx * G;
                nshift[pos] = make_float2(__fmul_rn((float)(kx - gx0), step_f),
                                          __fmul_rn((float)(ky - gy0), step_f));
            } else if (kind == 3) {
                int pos = nnext + (pre >> 20);
                if (pos + nch <= FR_CAP) {
                    for (int a = 0; a < 2; a++)
                        for (int b = 0; b < 2; b++)
                            if (2 * ci + a < gc && 2 * cj + b < gc)
                                front_next[pos++] = (2 * ci + a) * gc + (2 * cj + b);
                }
            }
            nfar += tot & 1023;
            nnear += (tot >> 10) & 1023;
            if (nnext + (tot >> 20) > FR_CAP) ovf = true;
            nnext += tot >> 20;
        };

        if (d.flat) {
            const long long B = (long long)G * G;
            for (long long q0 = 0; q0 < B; q0 += FT) {
                if (nfar + FT > FAR_CAP) flush_far();
                if (nnear + FT > NEAR_CAP) flush_near();
                long long b = q0 + tid;
                int kind = 0, bx = 0, byy = 0, id = 0;
                float rx = 0, ry = 0, M = 0;
                if (b < B) {
                    bx = (int)(b / G);
                    byy = (int)(b - (long long)bx * G);
                    long long gb = sd.boff + b;
                    // near boxes by their particles, far boxes by their moments (a plan over one
                    // rank's part of a system holds the other boxes' moments, not their particles)
                    if (abs(bx - gx0) <= 1 && abs(byy - gy0) <= 1) {
                        if (d.box_start[gb + 1] > d.box_start[gb]) {
                            kind = 2;
                            id = (int)gb;
                        }
                    } else {
                        float4 rr = d.rec[sd.coff + b];
                        if (rr.z > 0.f) {
                            rx = __fadd_rn(__fmul_rn((float)(bx - gx0), step_f), rr.x);
                            ry = __fadd_rn(__fmul_rn((float)(byy - gy0), step_f), rr.y);
                            M = rr.z;
                            kind = 1;
                            id = (int)(sd.coff + b);
                        }
                    }
                }
                emit(kind, id, 0, bx, byy, rx, ry, M, front1, 0);
            }
        } else {
            int *fr = front0, *fn = front1;
            if (tid == 0) fr[0] = 0;
            int nfr = 1;
            const float theta2 = d.theta2_f;
            for (int l = sd.L - 1; l >= 0 && nfr > 0; l--) {
                const int gl = sd.lvg[l];
                const int gc = l > 0 ? sd.lvg[l - 1] : 0;
                nnext = 0;
                __syncthreads();  // frontier entries of the previous level are visible
                for (int q0 = 0; q0 < nfr; q0 += FT) {
                    if (nfar + FT > FAR_CAP) flush_far();
                    if (nnear + FT > NEAR_CAP) flush_near();
                    int q = q0 + tid;
                    int kind = 0, ci = 0, cj = 0, id = 0;
                    float rx = 0, ry = 0, M = 0;
                    int loc = q < nfr ? fr[q] : 0;
                    if (q < nfr && (unsigned)loc >= (unsigned)(gl * gl)) {
                        raise_err(d.glob, 4u /*BH_DEV_BAD_KEY*/);  // never expected: skip the cell
                    } else if (q < nfr) {
                        ci = loc / gl;
                        cj = loc - ci * gl;
                        long long cell = sd.coff + sd.lvoff[l] + loc;
                        float4 rr = d.rec[cell];
                        if (rr.z > 0.f) {
                            int lo_x = ci << l, hi_x = (ci + 1) << l;
                            int lo_y = cj << l, hi_y = (cj + 1) << l;
                            bool overlap = lo_x < gx1 && hi_x > gx0 && lo_y < gy1 && hi_y > gy0;
                            bool accept = false;
                            if (!overlap) {
                                rx = __fadd_rn(__fmul_rn((float)(lo_x - gx0), step_f), rr.x);
                                ry = __fadd_rn(__fmul_rn((float)(lo_y - gy0), step_f), rr.y);
                                float dxo = fmaxf(0.f, fmaxf(-rx, __fsub_rn(rx, W_f)));
                                float dyo = fmaxf(0.f, fmaxf(-ry, __fsub_rn(ry, W_f)));
                                float d2 = __fadd_rn(__fmul_rn(dxo, dxo), __fmul_rn(dyo, dyo));
                                float s_f = ldexpf(step_f, l);
                                accept = __fmul_rn(s_f, s_f) < __fmul_rn(theta2, d2);
                            }
                            M = rr.z;
                            if (accept) {
                                kind = 1;
                                id = (int)cell;
                            } else if (l == 0) {
                                kind = 2;
                                id = (int)(sd.boff + loc);
                            } else {
                                kind = 3;
                            }
                        }
                    }
                    emit(kind, id, l, ci, cj, rx, ry, M, fn, gc);
                }
                int *t = fr;
                fr = fn;
                fn = t;
                // an overflowed frontier may hold unwritten slots: abandon the walk
                // (flagged; the host bounds theta and group size so this cannot happen)
                nfr = ovf ? 0 : nnext;
                if (ovf && tid == 0) raise_err(d.glob, 2u /*BH_DEV_LIST_OVERFLOW*/);
            }
        }
        flush_far();
        flush_near();
        __syncthreads();  // the reduction below reuses the staging buffers

        // ---- reduce slice partials and write
        if (PACKED) {
#pragma unroll
            for (int k = 0; k < NR / 2; k++) {
                float a0, a1, b0, b1;
                f2_unpack(nax2[k], a0, a1);
                f2_unpack(nay2[k], b0, b1);
                anx[2 * k] = (R)a0;
                anx[2 * k + 1] = (R)a1;
                any_[2 * k] = (R)b0;
                any_[2 * k + 1] = (R)b1;
                f2_unpack(fsx2[k], a0, a1);
                f2_unpack(fsy2[k], b0, b1);
                afx[2 * k] = (R)a0;
                afx[2 * k + 1] = (R)a1;
                afy[2 * k] = (R)b0;
                afy[2 * k + 1] = (R)b1;
                f2_unpack(fcx2[k], a0, a1);
                f2_unpack(fcy2[k], b0, b1);
                acx[2 * k] = (R)a0;
                acx[2 * k + 1] = (R)a1;
                acy[2 * k] = (R)b0;
                acy[2 * k + 1] = (R)b1;
            }
        }
        if (active) {
#pragma unroll
            for (int r = 0; r < NR; r++) {
                R *o = red + 2 * ((slice * nthr + tl) * NR + r);
                o[0] = anx[r] + (afx[r] - acx[r]);
                o[1] = any_[r] + (afy[r] - acy[r]);
            }
        }
        __syncthreads();
        if (active && slice == 0) {
#pragma unroll
            for (int r = 0; r < NR; r++) {
                if (!tv[r]) continue;
                R sx = 0, sy = 0;
                for (int k = 0; k < nslice; k++) {
                    const R *o = red + 2 * ((k * nthr + tl) * NR + r);
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
                    double vx = d.VX[nxt][t] + ax * d.dt, vy = d.VY[nxt][t] + ay * d.dt;
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

template <typename R>
static size_t force_smem() {
    using S = typename Src<R>::T;
    return (size_t)far_bytes<R>() * FAR_CAP + (size_t)src_bytes<R>() * SRC_CAP + sizeof(float2) * NEAR_CAP +
           sizeof(int) * (3 * NEAR_CAP + 4) + sizeof(int) * 2 * FR_CAP;
}

template <typename R, int NR, bool KAHAN, bool TEST, bool EXACT,
          int MINB = (sizeof(R) == 4 ? 8 : 4)>
static cudaError_t launch_force_t(const DevPlan &d, bool tick, bool accumulate, cudaStream_t st) {
    static_assert(sizeof(R) * 2 * FT * NR <= (size_t)far_bytes<R>() * FAR_CAP + (size_t)src_bytes<R>() * SRC_CAP,
                  "reduction buffer must fit in the staging buffers");
    static_assert(FT * NR >= TARGET_CHUNK, "a CTA must cover every target of a work item");
    auto k = k_force<R, NR, KAHAN, TEST, EXACT, MINB>;
    size_t sm = force_smem<R>();
    long long items_max = d.NG_total + d.n_total / d.chunk + 1;
    long long grid = (long long)d.nsm * MINB;
    if (grid > items_max) grid = items_max;
    if (grid < 1) grid = 1;
    cudaError_t e = cudaMemsetAsync(&d.glob->item_next, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    k<<<(unsigned)grid, FT, sm, st>>>(d, tick ? 1 : 0, accumulate ? 1 : 0);
    return cudaGetLastError();
}

template <typename R, int NR, bool KAHAN, bool TEST, bool EXACT,
          int MINB = (sizeof(R) == 4 ? 8 : 4)>
static cudaError_t init_force_t() {
    return cudaFuncSetAttribute(k_force<R, NR, KAHAN, TEST, EXACT, MINB>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)force_smem<R>());
}

// Raise the dynamic shared-memory limit of every instantiation once (outside
// any stream capture).
cudaError_t force_init() {
    cudaError_t e;
    if ((e = fstream_init()) != cudaSuccess) return e;
    if ((e = init_force_t<double, FORCE_R, false, true, false>()) != cudaSuccess) return e;
    if ((e = init_force_t<double, FORCE_R, false, false, false>()) != cudaSuccess) return e;
    if ((e = init_force_t<float, FORCE_R, true, true, true>()) != cudaSuccess) return e;
    if ((e = init_force_t<float, FORCE_R, true, true, false>()) != cudaSuccess) return e;
    if ((e = init_force_t<float, FORCE_R, true, false, false>()) != cudaSuccess) return e;
    if ((e = init_force_t<float, FORCE_R, false, true, true>()) != cudaSuccess) return e;
    if ((e = init_force_t<float, FORCE_R, false, true, false>()) != cudaSuccess) return e;
    if ((e = init_force_t<float, FORCE_R, true, false, false, 6>()) != cudaSuccess) return e;
    if ((e = init_force_t<float, FORCE_R, false, false, false, 6>()) != cudaSuccess) return e;
    return init_force_t<float, FORCE_R, false, false, false>();
}

cudaError_t launch_force(const DevPlan &d, bool tick, bool accumulate, cudaStream_t st,
                         const cudaEvent_t *ev) {
    if (d.n_total == 0) return cudaSuccess;
    if (d.stream) {  // prebuilt interaction lists, streamed (bh_lists.cu, bh_fstream.cu)
        cudaError_t e = launch_lists(d, st);
        if (e != cudaSuccess) return e;
        return launch_fstream(d, tick, accumulate, st, ev);
    }
    // The walk reads source positions from the FP64 state that the fused tick would update in
    // place while other CTAs still read them, so here the tick runs as its own kernel.
    const bool fused_tick = tick;
    tick = false;
    cudaError_t e = cudaSuccess;
    if (ev && (e = cudaEventRecord(ev[0], st)) != cudaSuccess) return e;
    const bool test = d.cutoff > 0.0 || d.eps2 == 0.0;
    const bool exact = d.cutoff > 0.0;
    if (d.prec == 2) {
        if (test) e = launch_force_t<double, FORCE_R, false, true, false>(d, tick, accumulate, st);
        else e = launch_force_t<double, FORCE_R, false, false, false>(d, tick, accumulate, st);
    } else if (d.prec == 1) {
        if (exact) e = launch_force_t<float, FORCE_R, true, true, true>(d, tick, accumulate, st);
        else if (test) e = launch_force_t<float, FORCE_R, true, true, false>(d, tick, accumulate, st);
        else if (d.tune == 1) e = launch_force_t<float, FORCE_R, true, false, false, 6>(d, tick, accumulate, st);
        else e = launch_force_t<float, FORCE_R, true, false, false>(d, tick, accumulate, st);
    } else {
        if (exact) e = launch_force_t<float, FORCE_R, false, true, true>(d, tick, accumulate, st);
        else if (test) e = launch_force_t<float, FORCE_R, false, true, false>(d, tick, accumulate, st);
        else if (d.tune == 1) e = launch_force_t<float, FORCE_R, false, false, false, 6>(d, tick, accumulate, st);
        else e = launch_force_t<float, FORCE_R, false, false, false>(d, tick, accumulate, st);
    }
    if (e != cudaSuccess) return e;
    if (ev && (e = cudaEventRecord(ev[1], st)) != cudaSuccess) return e;
    return fused_tick ? launch_tick(d, st, true) : cudaSuccess;
}

}  // namespace bh

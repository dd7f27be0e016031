// bh_fstream.cu -- list-streaming force evaluation with the tick fused into its epilogue.
//
// Replaces g_evaluate_boxes (python-bh/barneshut/kernels/grid_decomposition/gpu/grid.py:116-157)
// and, fused, g_tick_particles (gpu/grid.py:159-174) for the theta-mode production case: FP32
// pair arithmetic (plain or Kahan-compensated far field), Plummer softening > 0, no r^2 cutoff.
// The interaction lists come from k_lists (one pyramid walk per target group); this kernel only
// streams them.
//
// One warp owns one work item at a time (a full chunk of STREAM_CHUNK targets of a target set or
// a piece of its remainder, sitem_range; pulled from a device queue); the warps of a CTA share
// nothing but the CTA's shared memory carve-up, so there is no CTA-wide barrier and a warp
// waiting on memory leaves the SM to the other warps.  Per item:
//   * far field: the group's far entries (centre of mass in the group frame, mass) are widened
//     into the warp's staging as packed (x, x, y, y) + (M, M) entries, WFAR at a time, and
//     swept; each pass's plain FP32 sum enters the running total through a Kahan-compensated
//     addition (BH_PREC_FP32_KAHAN) or a plain one (BH_PREC_FP32);
//   * near field: the near boxes' 32-byte packed records (x, x, y, y), (m, m, index, box) are
//     copied piece by piece (a piece: a run of listed boxes whose particles are contiguous, as
//     neighbouring boxes of one column are) into the warp's staging by bulk asynchronous copies
//     (TMA),
//     WSRC sources per pass, double-buffered on two mbarriers so the copy of pass p + 1 overlaps
//     the sweep of pass p; the lanes shift each staged source from its box frame into the group
//     frame in place before the sweep, the shift following from the box coordinates that the
//     record carries.
// Each lane owns FORCE_R targets as two packed pairs (one f32x2 instruction serves two targets);
// the lanes form slices that split every staged list; slice partials are reduced through the
// warp's staging before the FP64 write-back and the fused tick.
#include "bh_internal.cuh"
#include "bh_pairs.cuh"
#include "bh_tc.cuh"

namespace bh {

constexpr int NR = FORCE_R;
constexpr int FW = 4;       // warps per CTA
constexpr int WDESC = 64;   // near descriptors per batch (per warp)
constexpr int NRUN = MAX_TG * MAX_TG;                // target runs (boxes) of a work item

// Per-warp shared-memory carve-up (bytes) of the build with MINB CTAs per SM.  The far phase of an
// item ends before its near phase starts, and the slice reduction follows both, so the far staging
// and the reduction buffer share the two near-source buffers.  WSRC near sources per bulk-copy
// pass: the largest pass that keeps MINB CTAs of FW warps within the SM's shared memory (the
// 8-CTA build, which spills, also leaves L1 room for its spills): 88 at 8 CTAs, 120 at 6.  WFAR
// far entries per pass: two raw 16-byte buffers (bulk copies of the group's far list, the next
// pass in flight while this one is swept) and the widened staging fit in the same space.
template <int MINB>
struct FsLayout {
    static constexpr int WSRC = MINB >= 8 ? 88 : 120;
    static constexpr int WFAR = MINB >= 8 ? 96 : 128;
    static constexpr int W_SRC = 0;                             // 2 x WSRC x 32 bytes
    static constexpr int W_FRAW = 0;                            // 2 x WFAR x float4 (x, y, M, 0)
    static constexpr int W_FARXY = W_FRAW + 2 * WFAR * 16;      // WFAR x float4 (x, x, y, y)
    static constexpr int W_FARM = W_FARXY + WFAR * 16;          // WFAR x float2 (M, M)
    static constexpr int W_NBOX = W_SRC + 2 * WSRC * 32;        // (WDESC + 1) x int
    static constexpr int W_NPRE = W_NBOX + (WDESC + 1) * 4;     // (WDESC + 1) x int
    static constexpr int W_RUN = W_NPRE + (WDESC + 1) * 4;      // 2 x (NRUN + 1) x int
    static constexpr int W_MBAR = (W_RUN + 2 * (NRUN + 1) * 4 + 7) / 8 * 8;  // 2 x uint64
    static constexpr int W_CNT = W_MBAR + 16;   // 2 x uint64: the warp's near, far pair counts
    static constexpr int W_BYTES = (W_CNT + 16 + 127) / 128 * 128;
    static constexpr size_t SMEM = (size_t)FW * W_BYTES;
    static_assert(W_FARM + WFAR * 8 <= W_NBOX, "far staging must fit in the near-source buffers");
    static_assert(2 * 32 * NR * sizeof(float) <= (size_t)W_NBOX, "slice partials alias the source buffers");
    static_assert((WSRC * 32) % 16 == 0 && W_BYTES % 128 == 0, "bulk-copy destinations must be 16-byte aligned");
    static_assert(MINB * (SMEM + 1024) <= 228 * 1024, "MINB CTAs must fit in the SM's shared memory");
    static_assert(WFAR % 32 == 0, "far staging passes are whole lane rounds");
};
static_assert(32 * NR >= STREAM_CHUNK, "a warp must cover every target of a work item");

template <bool KAHAN, int MINB>
__global__ void __launch_bounds__(FW * 32, MINB) k_fstream(DevPlan d, int tick, int accumulate) {
    extern __shared__ __align__(128) unsigned char smem[];
    using Ly = FsLayout<MINB>;
    constexpr int WSRC = Ly::WSRC, WFAR = Ly::WFAR;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned char *ws = smem + warp * Ly::W_BYTES;
    float4 *farxy = reinterpret_cast<float4 *>(ws + Ly::W_FARXY);
    float2 *farm = reinterpret_cast<float2 *>(ws + Ly::W_FARM);
    unsigned char *srcb = ws + Ly::W_SRC;
    unsigned char *fraw = ws + Ly::W_FRAW;
    int *nbox = reinterpret_cast<int *>(ws + Ly::W_NBOX);
    int *npre = reinterpret_cast<int *>(ws + Ly::W_NPRE);
    int *rstart = reinterpret_cast<int *>(ws + Ly::W_RUN);  // first particle of target run r
    int *rpre = rstart + NRUN + 1;                       // exclusive prefix of the run lengths
    uint64_t *mbar = reinterpret_cast<uint64_t *>(ws + Ly::W_MBAR);
    float *red = reinterpret_cast<float *>(ws);  // aliases the source buffers

    const int nxt = (d.glob->epoch + 1) & 1;
    const double *Xs = d.X[nxt], *Ys = d.Y[nxt];
    const long long nitems = d.sitem_off[d.NG_total];
    unsigned long long *wcnt = reinterpret_cast<unsigned long long *>(ws + Ly::W_CNT);  // lane 0 counts
    uint32_t phases = 0u;  // bit b: parity of buffer b's current mbarrier phase
    bool tma_ok = true;  // warp-uniform; cleared (and flagged) when a copy wait times out
    if (lane == 0) {
        wcnt[0] = wcnt[1] = 0ull;
        tc::mbar_init(&mbar[0], 1);
        tc::mbar_init(&mbar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();

    // lane 0 takes the queue slot of its next item one item ahead (the atomic's latency hides
    // behind the current item)
    int qnext = 0;
    if (lane == 0) qnext = (int)atomicAdd(&d.glob->item_next, 1u);
    for (;;) {
        int item = 0;
        if (lane == 0) {
            const int q = qnext;
            item = q < nitems ? d.item_order[q] : q;  // heaviest items first
            if (q < nitems) qnext = (int)atomicAdd(&d.glob->item_next, 1u);
        }
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= nitems) break;
        const long long g = d.sitem_group[item];
        const int sub = d.sitem_sub[item];  // box within the group, or -1: the sparse boxes
        const int2 ck = d.sitem_chunk[item];
        const int s = find_seg(d.goff_tab, d.nsys, g);
        const SysDesc &sd = d.sys[s];
        const SysDyn &dy = d.dyn[s];
        const long long lg = g - sd.goff;
        const int TG = sd.TG, G = sd.G;
        const int tgs = __ffs(TG) - 1;  // TG is a power of two
        // a system has fewer than 2^31 groups (G <= LIST_MAX_G)
        const int gi = (int)lg / sd.NGs, gj = (int)lg - gi * sd.NGs;
        const int gx0 = gi * TG, gy0 = gj * TG;
        // the item's targets: runs of box-sorted particles, one per box of the group (column-major;
        // a box outside the item's set is an empty run; a quadrant item's box run is the quadrant)
        const int nrun = TG * TG;
        const int qbox = sub >= nrun ? (sub - nrun) >> 2 : -1, quad = sub >= nrun ? (sub - nrun) & 3 : 0;
        const int2 cnt = d.lcnt[g];
        const float4 *lf = d.lfar + sd.lfoff + lg * sd.lfcap;
        const int nfp = (cnt.x + WFAR - 1) / WFAR;  // far passes
        // far pass p: one bulk copy of the list's entries into raw buffer p & 1 (the buffer's
        // previous contents, if any, were widened before; lane 0 announces the bytes and copies)
        auto issue_far = [&](int p) {
            const int f0 = p * WFAR, nf = min(WFAR, cnt.x - f0);
            __syncwarp();
            tc::fence_async_smem();
            if (lane == 0) {
                tc::mbar_expect_tx(&mbar[p & 1], (uint32_t)nf * 16u);
                tc::bulk_g2s(fraw + (p & 1) * (WFAR * 16), lf + f0, (uint32_t)nf * 16u, &mbar[p & 1]);
            }
        };
        if (tma_ok && nfp > 0) issue_far(0);
        if (tma_ok && nfp > 1) issue_far(1);
        {
            int carry = 0;
            for (int b0 = 0; b0 < nrun; b0 += 32) {
                const int b = b0 + lane;
                int st = 0, len = 0;
                if (b < nrun) {
                    const int cx = b >> tgs, cy = b & (TG - 1);
                    if (gx0 + cx < G && gy0 + cy < G) {
                        const long long bb = sd.boff + (long long)(gx0 + cx) * G + gy0 + cy;
                        st = d.box_start[bb];
                        len = d.box_start[bb + 1] - st;
                        if (qbox >= 0) {
                            if (b != qbox) {
                                len = 0;
                            } else {
                                const int4 qc = reinterpret_cast<const int4 *>(d.qcounts)[bb];
                                st += (quad > 0 ? qc.x : 0) + (quad > 1 ? qc.y : 0) + (quad > 2 ? qc.z : 0);
                                len = quad == 0 ? qc.x : quad == 1 ? qc.y : quad == 2 ? qc.z : qc.w;
                            }
                        } else if (sub >= 0 ? b != sub : box_item_kind(len, d.dense_min, d.quad_min) != 0) {
                            len = 0;
                        }
                    }
                }
                int inc = len;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, inc, o);
                    if (lane >= o) inc += y;
                }
                if (b < nrun) {
                    rstart[b] = st;
                    rpre[b + 1] = carry + inc;
                }
                carry += __shfl_sync(0xffffffffu, inc, 31);
            }
            if (lane == 0) rpre[0] = 0;
        }
        __syncwarp();
        const int nt = rpre[nrun];
        int c0, T;
        sitem_range(nt, ck.x, &c0, &T);
        const float step_f = __double2float_rn(dy.step);
        const float eps2 = d.eps2_f;

        // ---- lane -> (slice, NR targets)
        const int nthr = (T + NR - 1) / NR;
        const int nslice = 32 / nthr;
        const bool active = lane < nslice * nthr;
        const int slice = active ? lane / nthr : 0, tl = active ? lane % nthr : 0;
        // sorted index of the lane's target r (recomputed in the epilogue rather than kept live)
        // (the run is the target's box within the group, column-major)
        auto target_index = [&](int r, int &run) {
            const int v = tl * NR + r;
            const int u = c0 + (v < T ? v : 0);
            int lo = 0, hi = nrun;  // the run r with rpre[r] <= u < rpre[r + 1]
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (rpre[mid] <= u) lo = mid; else hi = mid;
            }
            run = lo;
            return rstart[lo] + (u - rpre[lo]);
        };
        float tx[NR], ty[NR];
#pragma unroll
        for (int r = 0; r < NR; r++) {
            int run;
            const int ti = target_index(r, run);
            const float4 p = d.PD[2 * (long long)ti];  // (x, x, y, y) box-relative
            tx[r] = __fadd_rn(__fmul_rn((float)(run >> tgs), step_f), p.x);
            ty[r] = __fadd_rn(__fmul_rn((float)(run & (TG - 1)), step_f), p.z);
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
        const int4 *ln = d.lnear + sd.lnoff + lg * 2 * (sd.lncap + 1);

        // sweep nf staged far entries; the pass's plain FP32 sum enters the far total through a
        // Kahan-compensated addition (compensate: the group's far list), or the near accumulators
        // by a plain one (the far entries a dense item's own opening test accepts)
        auto far_sweep = [&](int nf, bool compensate) {
            if (active) {
                const ulonglong2 *fp = reinterpret_cast<const ulonglong2 *>(farxy);
                const f2_t *fm = reinterpret_cast<const f2_t *>(farm);
                f2_t px2[NR / 2], py2[NR / 2];
#pragma unroll
                for (int kk = 0; kk < NR / 2; kk++) px2[kk] = py2[kk] = f2_pack(0.f, 0.f);
#pragma unroll 4
                for (int k = slice; k < nf; k += nslice) {
                    const ulonglong2 rxy = fp[k];  // (rx, rx), (ry, ry)
                    const f2_t mm = fm[k];         // (M, M)
#pragma unroll
                    for (int kk = 0; kk < NR / 2; kk++) {
                        const f2_t dx = f2_add(rxy.x, ntx2[kk]), dyy = f2_add(rxy.y, nty2[kk]);
                        const f2_t w = f2_mul(mm, f2_rcp(f2_fma(dx, dx, f2_fma(dyy, dyy, eps2x2))));
                        px2[kk] = f2_fma(w, dx, px2[kk]);
                        py2[kk] = f2_fma(w, dyy, py2[kk]);
                    }
                }
#pragma unroll
                for (int kk = 0; kk < NR / 2; kk++) {
                    if (KAHAN && compensate) {  // y = f - c; t = s + y; c = (t - s) - y; s = t
                        const f2_t yx = f2_fma(fcx2[kk], m1x2, px2[kk]), t1 = f2_add(fsx2[kk], yx);
                        fcx2[kk] = f2_fma(yx, m1x2, f2_fma(fsx2[kk], m1x2, t1));
                        fsx2[kk] = t1;
                        const f2_t yy = f2_fma(fcy2[kk], m1x2, py2[kk]), t2 = f2_add(fsy2[kk], yy);
                        fcy2[kk] = f2_fma(yy, m1x2, f2_fma(fsy2[kk], m1x2, t2));
                        fsy2[kk] = t2;
                    } else if (compensate) {
                        fsx2[kk] = f2_add(fsx2[kk], px2[kk]);
                        fsy2[kk] = f2_add(fsy2[kk], py2[kk]);
                    } else {
                        nax2[kk] = f2_add(nax2[kk], px2[kk]);
                        nay2[kk] = f2_add(nay2[kk], py2[kk]);
                    }
                }
            }
            if (lane == 0) wcnt[1] += (unsigned long long)T * nf;
            __syncwarp();  // the staging is rewritten next
        };

        // ---- far field: the group's accepted cells, pass by pass from the raw buffers (the
        // entries, centre of mass in the group frame and mass, widen into the packed staging)
        for (int p = 0; p < nfp && tma_ok; p++) {
            const int nf = min(WFAR, cnt.x - p * WFAR);
            const int buf = p & 1;
            const bool ok = tc::mbar_wait(&mbar[buf], (phases >> buf) & 1u);
            phases ^= 1u << buf;
            if (!__all_sync(0xffffffffu, ok)) {
                // flagged; give the copies in flight a second bounded wait, then stage nothing
                // more in this launch (the barrier phases are no longer known)
                if (lane == 0) raise_err(d.glob, 8u /*BH_DEV_WAIT_TIMEOUT*/);
                tc::mbar_wait(&mbar[buf], ((phases >> buf) & 1u) ^ 1u);
                if (p + 1 < nfp) tc::mbar_wait(&mbar[buf ^ 1], (phases >> (buf ^ 1)) & 1u);
                tma_ok = false;
                break;
            }
            const float4 *raw = reinterpret_cast<const float4 *>(fraw + buf * (WFAR * 16));
#pragma unroll
            for (int u = 0; u < WFAR / 32; u++) {
                const int k = lane + 32 * u;
                if (k < nf) {
                    const float4 e = raw[k];
                    farxy[k] = make_float4(e.x, e.x, e.y, e.y);
                    farm[k] = make_float2(e.z, e.z);
                }
            }
            if (p + 2 < nfp) issue_far(p + 2);  // (its syncwarp also publishes the staging)
            else __syncwarp();
            far_sweep(nf, true);
        }
        // the compensated far sums s - c start the near accumulators; the far sums and their
        // compensations are dead from here on
#pragma unroll
        for (int kk = 0; kk < NR / 2; kk++) {
            nax2[kk] = f2_fma(fcx2[kk], m1x2, fsx2[kk]);
            nay2[kk] = f2_fma(fcy2[kk], m1x2, fsy2[kk]);
        }

        // ---- near field: descriptors in batches of WDESC; sources in double-buffered passes.
        // Descriptor k is (first particle, exclusive prefix of the boxes' particle counts, box
        // shift in the group frame); entry [count] carries the total.
        for (int b0 = 0; b0 < cnt.y && tma_ok; b0 += WDESC) {
            int nn = min(WDESC, cnt.y - b0);
            if (sub < 0) {
                for (int k = lane; k <= nn; k += 32) {
                    const int2 e = *reinterpret_cast<const int2 *>(ln + 2 * (b0 + k));
                    nbox[k] = e.x;
                    npre[k] = e.y;
                }
                __syncwarp();
            } else {
                // a dense box's (or quadrant's) own lists: a near leaf of the group that passes the
                // opening test against the single box or quadrant (its offsets taken relative to
                // that rectangle's origin) is swept as a far entry; the others stay near and are
                // re-prefixed
                const int bsel = qbox >= 0 ? qbox : sub;
                const int bcx = bsel >> tgs, bcy = bsel & (TG - 1);
                float oxb, oyb, wr;  // rectangle origin in the group frame, edge
                if (qbox >= 0) {
                    const float half_f = 0.5f * step_f;
                    oxb = __fmul_rn((float)(2 * bcx + (quad >> 1)), half_f);
                    oyb = __fmul_rn((float)(2 * bcy + (quad & 1)), half_f);
                    wr = half_f;
                } else {
                    oxb = __fmul_rn((float)bcx, step_f);
                    oyb = __fmul_rn((float)bcy, step_f);
                    wr = step_f;
                }
                const float s2 = __fmul_rn(step_f, step_f), theta2 = d.theta2_f;
                const int own = (gx0 + bcx) * G + (gy0 + bcy);
                int nkeep = 0, nacc = 0, base = 0;
                // the batch's descriptors (WDESC = 2 rounds of 32) are loaded together
                int4 pe0[WDESC / 32], pe1[WDESC / 32];
                int pnx[WDESC / 32];
#pragma unroll
                for (int u = 0; u < WDESC / 32; u++) {
                    const int k = 32 * u + lane;
                    pe0[u] = make_int4(0, 0, 0, 0);
                    pe1[u] = make_int4(-1, 0, 0, 0);
                    pnx[u] = 0;
                    if (k < nn) {
                        pe0[u] = ln[2 * (b0 + k)];
                        pe1[u] = ln[2 * (b0 + k) + 1];
                        pnx[u] = ln[2 * (b0 + k + 1)].y;
                    }
                }
#pragma unroll
                for (int u = 0; u < WDESC / 32; u++) {
                    const int k0 = 32 * u;
                    if (k0 >= nn) break;
                    const int k = k0 + lane;
                    const int4 e0 = pe0[u], e1 = pe1[u];
                    const int c = k < nn ? pnx[u] - e0.y : 0;
                    bool acc = false;
                    if (k < nn) {
                        if (e1.x != own) {
                            const float rxb = __fsub_rn(__int_as_float(e1.z), oxb);
                            const float ryb = __fsub_rn(__int_as_float(e1.w), oyb);
                            const float dxo = fmaxf(0.f, fmaxf(-rxb, __fsub_rn(rxb, wr)));
                            const float dyo = fmaxf(0.f, fmaxf(-ryb, __fsub_rn(ryb, wr)));
                            const float d2 = __fadd_rn(__fmul_rn(dxo, dxo), __fmul_rn(dyo, dyo));
                            acc = s2 < __fmul_rn(theta2, d2);
                        }
                    }
                    const bool keep = k < nn && !acc;
                    const unsigned mk = __ballot_sync(0xffffffffu, keep), ma = __ballot_sync(0xffffffffu, acc);
                    const unsigned lt = (1u << lane) - 1u;
                    int inc = keep ? c : 0;  // inclusive scan of the kept particle counts
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int y = __shfl_up_sync(0xffffffffu, inc, o);
                        if (lane >= o) inc += y;
                    }
                    if (keep) {
                        const int q = nkeep + __popc(mk & lt);
                        nbox[q] = e0.x;
                        npre[q] = base + inc - c;
                    } else if (acc) {
                        const int q = nacc + __popc(ma & lt);
                        const float rx = __int_as_float(e1.z), ry = __int_as_float(e1.w), m = __int_as_float(e1.y);
                        farxy[q] = make_float4(rx, rx, ry, ry);
                        farm[q] = make_float2(m, m);
                    }
                    nkeep += __popc(mk);
                    nacc += __popc(ma);
                    base += __shfl_sync(0xffffffffu, inc, 31);
                }
                if (lane == 0) npre[nkeep] = base;
                __syncwarp();
                if (nacc > 0) far_sweep(nacc, false);  // (also orders the staging for the copies)
                nn = nkeep;
            }
            // boxes listed one after another whose particles are contiguous (neighbours in one
            // column of the near region) become one piece, copied at once
            {
                int bx[WDESC / 32], px[WDESC / 32];
                bool head[WDESC / 32];
#pragma unroll
                for (int u = 0; u < WDESC / 32; u++) {
                    const int k = lane + 32 * u;
                    bx[u] = k < nn ? nbox[k] : 0;
                    px[u] = k < nn ? npre[k] : 0;
                    head[u] = k < nn && (k == 0 || nbox[k - 1] + (px[u] - npre[k - 1]) != bx[u]);
                }
                const int total = npre[nn];
                __syncwarp();
                int np = 0;
#pragma unroll
                for (int u = 0; u < WDESC / 32; u++) {
                    const unsigned hm = __ballot_sync(0xffffffffu, head[u]);
                    if (head[u]) {
                        const int q = np + __popc(hm & ((1u << lane) - 1u));
                        nbox[q] = bx[u];
                        npre[q] = px[u];
                    }
                    np += __popc(hm);
                }
                if (lane == 0) npre[np] = total;
                __syncwarp();
                nn = np;
            }
            const int pbeg = npre[0], pend = npre[nn];
            const int npass = (pend - pbeg + WSRC - 1) / WSRC;
            // issue pass p into buffer p & 1: one bulk copy per box piece, all on that buffer's
            // mbarrier (lane 0 announces the bytes before any lane copies)
            auto issue = [&](int p) {
                const int s0 = pbeg + p * WSRC, ns = min(WSRC, pend - s0);
                unsigned char *dst = srcb + (p & 1) * (WSRC * 32);
                if (lane == 0) tc::mbar_expect_tx(&mbar[p & 1], (uint32_t)ns * 32u);
                __syncwarp();
                tc::fence_async_smem();
                for (int k = lane; k < nn; k += 32) {
                    const int lo = max(npre[k], s0), hi = min(npre[k + 1], s0 + ns);
                    if (lo < hi)
                        tc::bulk_g2s(dst + 32 * (lo - s0), d.PD + 2 * (long long)(nbox[k] + (lo - npre[k])),
                                     (uint32_t)(hi - lo) * 32u, &mbar[p & 1]);
                }
            };
            if (npass > 0) issue(0);
            if (npass > 1) issue(1);
            for (int p = 0; p < npass; p++) {
                const int s0 = pbeg + p * WSRC, ns = min(WSRC, pend - s0);
                const int buf = p & 1;
                const bool ok = tc::mbar_wait(&mbar[buf], (phases >> buf) & 1u);
                phases ^= 1u << buf;
                if (!__all_sync(0xffffffffu, ok)) {
                    // flagged; give the copies in flight a second bounded wait, then stage
                    // nothing more in this launch (the barrier phases are no longer known)
                    if (lane == 0) raise_err(d.glob, 8u /*BH_DEV_WAIT_TIMEOUT*/);
                    tc::mbar_wait(&mbar[buf], ((phases >> buf) & 1u) ^ 1u);
                    if (p + 1 < npass) tc::mbar_wait(&mbar[buf ^ 1], (phases >> (buf ^ 1)) & 1u);
                    tma_ok = false;
                    break;
                }
                // shift the staged sources into the group frame in place, lane-strided over the
                // pass: the shift of box (kx, ky) is (kx - gx0, ky - gy0) x step, as in the lists
                float4 *s4 = reinterpret_cast<float4 *>(srcb + buf * (WSRC * 32));
#pragma unroll 3
                for (int j = lane; j < ns; j += 32) {
                    float4 v = s4[2 * j];
                    const int code = __float_as_int(s4[2 * j + 1].w);
                    const float shx = __fmul_rn((float)((code >> 16) - gx0), step_f);
                    const float shy = __fmul_rn((float)((code & 0xffff) - gy0), step_f);
                    v.x = __fadd_rn(shx, v.x);
                    v.y = v.x;
                    v.z = __fadd_rn(shy, v.z);
                    v.w = v.z;
                    s4[2 * j] = v;
                }
                __syncwarp();
                if (active) {
#pragma unroll 4
                    for (int j = slice; j < ns; j += nslice) {
                        const ulonglong2 sxy = *reinterpret_cast<const ulonglong2 *>(s4 + 2 * j);
                        const f2_t mm = *reinterpret_cast<const f2_t *>(s4 + 2 * j + 1);
#pragma unroll
                        for (int kk = 0; kk < NR / 2; kk++) {
                            const f2_t dx = f2_add(sxy.x, ntx2[kk]), dyy = f2_add(sxy.y, nty2[kk]);
                            const f2_t r2 = f2_fma(dx, dx, f2_fma(dyy, dyy, eps2x2));
                            const f2_t w = f2_mul(mm, f2_rcp(r2));
                            nax2[kk] = f2_fma(w, dx, nax2[kk]);
                            nay2[kk] = f2_fma(w, dyy, nay2[kk]);
                        }
                    }
                }
                if (lane == 0) wcnt[0] += (unsigned long long)T * ns;
                __syncwarp();  // every lane is done with this buffer
                if (p + 2 < npass) issue(p + 2);
            }
            __syncwarp();  // the descriptors are rewritten by the next batch
        }


        // ---- reduce slice partials (through the source buffers) and write
        if (active) {
#pragma unroll
            for (int k = 0; k < NR / 2; k++) {
                float a0, a1, b0, b1;
                f2_unpack(nax2[k], a0, a1);
                f2_unpack(nay2[k], b0, b1);
                float *o = red + 2 * ((slice * nthr + tl) * NR + 2 * k);
                o[0] = a0;
                o[1] = b0;
                o[2] = a1;
                o[3] = b1;
            }
        }
        __syncwarp();
        // every lane takes targets v = lane, lane + 32, ... (not only the first slice's lanes)
        for (int v = lane; v < T; v += 32) {
            {
                const int vt = v / NR, r = v - vt * NR;  // the lane and register that held it
                float sx = 0.f, sy = 0.f;
                for (int k = 0; k < nslice; k++) {
                    const float *o = red + 2 * ((k * nthr + vt) * NR + r);
                    sx += o[0];
                    sy += o[1];
                }
                const int u = c0 + v;
                int lo = 0, hi = nrun;  // the run with rpre[lo] <= u < rpre[lo + 1]
                while (hi - lo > 1) {
                    const int mid = (lo + hi) >> 1;
                    if (rpre[mid] <= u) lo = mid; else hi = mid;
                }
                const int t = rstart[lo] + (u - rpre[lo]);
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
        __syncwarp();  // the staging and the column table are reused by the next item
    }
    if (lane == 0) {
        atomicAdd(&d.glob->near_pairs, wcnt[0]);
        atomicAdd(&d.glob->far_pairs, wcnt[1]);
    }
}

template <bool KAHAN, int MINB>
static cudaError_t launch_fstream_t(const DevPlan &d, bool tick, bool accumulate, cudaStream_t st,
                                    const cudaEvent_t *ev) {
    long long items_max = d.NG_total + d.n_total / d.dense_min +
                          (d.quad_min > 0 ? 4 * (d.n_total / d.quad_min) : 0) + d.n_total / STREAM_ITEM_DIV + 1;
    long long grid = (long long)d.nsm * MINB;
    if (grid * FW > items_max) grid = (items_max + FW - 1) / FW;
    if (grid < 1) grid = 1;
    cudaError_t e = cudaMemsetAsync(&d.glob->item_next, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    if (ev && (e = cudaEventRecord(ev[0], st)) != cudaSuccess) return e;
    k_fstream<KAHAN, MINB><<<(unsigned)grid, FW * 32, FsLayout<MINB>::SMEM, st>>>(d, tick ? 1 : 0, accumulate ? 1 : 0);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    return ev ? cudaEventRecord(ev[1], st) : cudaSuccess;
}

template <bool KAHAN, int MINB>
static cudaError_t init_fstream_t() {
    return cudaFuncSetAttribute(k_fstream<KAHAN, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)FsLayout<MINB>::SMEM);
}

cudaError_t fstream_init() {
    cudaError_t e;
    if ((e = init_fstream_t<true, 8>()) != cudaSuccess) return e;
    if ((e = init_fstream_t<true, 6>()) != cudaSuccess) return e;
    if ((e = init_fstream_t<false, 8>()) != cudaSuccess) return e;
    return init_fstream_t<false, 6>();
}

cudaError_t launch_fstream(const DevPlan &d, bool tick, bool accumulate, cudaStream_t st,
                           const cudaEvent_t *ev) {
    if (d.n_total == 0) return cudaSuccess;
    if (d.prec == 1)
        return d.tune == 1 ? launch_fstream_t<true, 8>(d, tick, accumulate, st, ev)
                           : launch_fstream_t<true, 6>(d, tick, accumulate, st, ev);
    return d.tune == 1 ? launch_fstream_t<false, 8>(d, tick, accumulate, st, ev)
                       : launch_fstream_t<false, 6>(d, tick, accumulate, st, ev);
}

}  // namespace bh

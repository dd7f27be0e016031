// bh_lists.cu -- interaction lists of every target group, for the list-streaming force kernel.
//
// The reference evaluates every box against its 3 x 3 neighbourhood and the centre of mass of
// every other box (kernels/grid_decomposition/gpu/grid.py:116-157,
// sequential/evaluation.py:73-109); in theta mode this project replaces the flat far field with
// a walk of the cell pyramid, and this kernel does that walk once per target group instead of
// once per work item.  One warp per group (grid-stride over groups) walks the pyramid level by
// level, each lane testing LU frontier cells per round (their records loaded together): a
// cell whose centre of mass lies at distance d from the group's box rectangle is accepted when
// s^2 < theta^2 d^2 (s = cell edge) and goes to the far list, a rejected leaf goes to the near
// list, any other rejected cell opens into its children.  Ballots and a warp scan place the
// entries in frontier order, so list order is deterministic and matches the walking force
// kernel's; the test is the same FP32 arithmetic, so both paths accept the same cells.
//
// Output per group g of system s: far entries (the accepted cell's centre of mass in the group
// frame, as the opening test computed it, and its mass) at lfar[s.lfoff + lg * s.lfcap ..]; near descriptors -- (first particle, exclusive prefix of the
// boxes' particle counts, box-origin shift in the group frame) and (box index, mass, centre of
// mass in the group frame) -- at lnear[s.lnoff + lg * 2 * (s.lncap + 1) ..] with the total in
// descriptor [count]; lcnt[g] = (far count, near count).  The slots are
// sized on the host so that a level's accepted cells never exceed FRONTIER_CAP; the kernel still
// checks and raises BH_DEV_LIST_OVERFLOW.
#include "bh_internal.cuh"
#include "bh_pairs.cuh"

namespace bh {

constexpr int LW = 4;  // warps per list-building CTA; one warp walks one group
constexpr int LU = 1;  // frontier cells per lane per round (a level's frontier averages ~47 cells)
constexpr int LISTS_MINB = 12;  // CTAs per SM (40 registers): the walk is latency-bound

__global__ void __launch_bounds__(LW * 32, LISTS_MINB) k_lists(DevPlan d) {
    __shared__ int front[LW][2][FR_CAP];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int(*fb)[FR_CAP] = front[warp];
    const float theta2 = d.theta2_f;
    const unsigned lt_mask = (1u << lane) - 1u;
    for (long long g = (long long)blockIdx.x * LW + warp; g < d.NG_total; g += (long long)gridDim.x * LW) {
        const int s = find_seg(d.goff_tab, d.nsys, g);
        const SysDesc &sd = d.sys[s];
        const SysDyn &dy = d.dyn[s];
        const long long lg = g - sd.goff;
        const int TG = sd.TG;
        const int gi = (int)(lg / sd.NGs), gj = (int)(lg - (long long)gi * sd.NGs);
        const int gx0 = gi * TG, gy0 = gj * TG;
        const int gx1 = min(sd.G, gx0 + TG), gy1 = min(sd.G, gy0 + TG);
        const float step_f = __double2float_rn(dy.step);
        const float W_f = __fmul_rn((float)TG, step_f);
        float4 *far_out = d.lfar + sd.lfoff + lg * sd.lfcap;
        int4 *near_out = d.lnear + sd.lnoff + lg * 2 * (sd.lncap + 1);
        int nfar = 0, nnear = 0, nfr = 1, cur = 0;
        bool ovf = false;
        __syncwarp();  // the previous group is done with front[]
        if (lane == 0) fb[0][0] = 0;
        __syncwarp();
        for (int l = sd.L - 1; l >= 0 && nfr > 0; l--) {
            const int gl = sd.lvg[l];
            const int gc = l > 0 ? sd.lvg[l - 1] : 0;
            const float s_f = ldexpf(step_f, l);
            const float s2 = __fmul_rn(s_f, s_f);
            const int *fr = fb[cur];
            int *fn = fb[cur ^ 1];  // next frontier; at the leaf level, the near boxes
            int nnext = 0;
            for (int q0 = 0; q0 < nfr; q0 += 32 * LU) {
                int loc[LU];
                float4 rr[LU];
#pragma unroll
                for (int u = 0; u < LU; u++) {  // issue the round's record loads together
                    const int q = q0 + u * 32 + lane;
                    loc[u] = -1;
                    rr[u] = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (q < nfr) {
                        const int c = fr[q];
                        if ((unsigned)c >= (unsigned)(gl * gl)) {
                            raise_err(d.glob, 4u /*BH_DEV_BAD_KEY*/);  // never expected: skip it
                        } else {
                            loc[u] = c;
                            rr[u] = d.rec[sd.coff + sd.lvoff[l] + c];
                        }
                    }
                }
#pragma unroll
                for (int u = 0; u < LU; u++) {  // classify and append in frontier order
                    int kind = 0, ci = 0, cj = 0;
                    float rx = 0.f, ry = 0.f;  // centre of mass in the group frame
                    if (loc[u] >= 0 && rr[u].z > 0.f) {
                        ci = loc[u] / gl;
                        cj = loc[u] - ci * gl;
                        const int lo_x = ci << l, hi_x = (ci + 1) << l;
                        const int lo_y = cj << l, hi_y = (cj + 1) << l;
                        const bool overlap = lo_x < gx1 && hi_x > gx0 && lo_y < gy1 && hi_y > gy0;
                        bool accept = false;
                        if (!overlap) {
                            rx = __fadd_rn(__fmul_rn((float)(lo_x - gx0), step_f), rr[u].x);
                            ry = __fadd_rn(__fmul_rn((float)(lo_y - gy0), step_f), rr[u].y);
                            const float dxo = fmaxf(0.f, fmaxf(-rx, __fsub_rn(rx, W_f)));
                            const float dyo = fmaxf(0.f, fmaxf(-ry, __fsub_rn(ry, W_f)));
                            const float d2 = __fadd_rn(__fmul_rn(dxo, dxo), __fmul_rn(dyo, dyo));
                            accept = s2 < __fmul_rn(theta2, d2);
                        }
                        kind = accept ? 1 : (l == 0 ? 2 : 3);
                    }
                    const unsigned mf = __ballot_sync(0xffffffffu, kind == 1);
                    const unsigned mn = __ballot_sync(0xffffffffu, kind == 2);
                    int nch = 0;
                    if (kind == 3) nch = (2 * ci + 1 < gc ? 2 : 1) * (2 * cj + 1 < gc ? 2 : 1);
                    int inc = nch;  // inclusive warp scan of the children counts
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int y = __shfl_up_sync(0xffffffffu, inc, o);
                        if (lane >= o) inc += y;
                    }
                    const int ntot = __shfl_sync(0xffffffffu, inc, 31);
                    if (kind == 1) {
                        const int pos = nfar + __popc(mf & lt_mask);
                        if (pos < sd.lfcap) far_out[pos] = make_float4(rx, ry, rr[u].z, 0.f);
                    } else if (kind == 2) {
                        const int pos = nnear + __popc(mn & lt_mask);
                        if (pos < sd.lncap) fn[pos] = loc[u];
                    } else if (kind == 3) {
                        int pos = nnext + inc - nch;
                        if (pos + nch <= FR_CAP) {
                            for (int a = 0; a < 2; a++)
                                for (int b = 0; b < 2; b++)
                                    if (2 * ci + a < gc && 2 * cj + b < gc) fn[pos++] = (2 * ci + a) * gc + (2 * cj + b);
                        }
                    }
                    nfar += __popc(mf);
                    nnear += __popc(mn);
                    if (nnext + ntot > FR_CAP) ovf = true;
                    nnext += ntot;
                }
            }
            __syncwarp();  // the next frontier (or the near list) is complete
            cur ^= 1;
            // an overflowed frontier may hold unwritten slots: abandon the walk (flagged)
            nfr = ovf ? 0 : nnext;
        }
        // near descriptors: first particle, exclusive prefix of the particle counts, box shift.
        // The near boxes were appended at the leaf level into the buffer that is now fb[cur]
        // (children in (0, 0), (0, 1), (1, 0), (1, 1) order, so a pair of boxes of one column
        // often follows each other: the force kernel copies such a run at once).
        const int nn = min(nnear, sd.lncap);
        const int *nl = fb[cur];
        int base = 0;
        // LU rounds of 32 boxes at a time: their particle ranges and records are loaded together
        for (int k0 = 0; k0 <= nn; k0 += 32 * LU) {
            int loc[LU], st[LU], c[LU];
            float4 rr[LU];
#pragma unroll
            for (int u = 0; u < LU; u++) {
                const int k = k0 + 32 * u + lane;
                loc[u] = k < nn ? nl[k] : 0;
            }
#pragma unroll
            for (int u = 0; u < LU; u++) {
                const int k = k0 + 32 * u + lane;
                st[u] = c[u] = 0;
                rr[u] = make_float4(0.f, 0.f, 0.f, 0.f);
                if (k < nn) {
                    st[u] = d.box_start[sd.boff + loc[u]];
                    c[u] = d.box_start[sd.boff + loc[u] + 1] - st[u];
                    rr[u] = d.rec[sd.coff + loc[u]];  // the leaf's record (level 0)
                }
            }
#pragma unroll
            for (int u = 0; u < LU; u++) {
                const int k = k0 + 32 * u + lane;
                int inc = c[u];
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, inc, o);
                    if (lane >= o) inc += y;
                }
                const int pre = base + inc - c[u];
                if (k < nn) {
                    const int kx = loc[u] / sd.G, ky = loc[u] - kx * sd.G;
                    const float shx = __fmul_rn((float)(kx - gx0), step_f), shy = __fmul_rn((float)(ky - gy0), step_f);
                    near_out[2 * k] = make_int4(st[u], pre, __float_as_int(shx), __float_as_int(shy));
                    near_out[2 * k + 1] = make_int4(loc[u], __float_as_int(rr[u].z), __float_as_int(__fadd_rn(shx, rr[u].x)),
                                                    __float_as_int(__fadd_rn(shy, rr[u].y)));
                } else if (k == nn) {
                    near_out[2 * k] = make_int4(0, pre, 0, 0);
                    near_out[2 * k + 1] = make_int4(0, 0, 0, 0);
                }
                base += __shfl_sync(0xffffffffu, inc, 31);
            }
        }
        if (lane == 0) {
            if (ovf || nfar > sd.lfcap || nnear > sd.lncap) raise_err(d.glob, 2u /*BH_DEV_LIST_OVERFLOW*/);
            d.lcnt[g] = make_int2(min(nfar, sd.lfcap), nn);
        }
    }
}

// ---------------------------------------------------------------- heaviest-first item order
// A warp of the force kernel owns one work item, so an item's duration grows with its pair count
// and the launch ends with its slowest warp.  Items are therefore handed out heaviest first:
// bucket b holds the items whose estimated cost (STREAM_CHUNK / slices) x (near sources + 2 x far
// cells) lies in [2^b, 2^(b+1)); buckets are laid out from the top down.  Order inside a bucket
// follows atomic arrival, which changes only which warp evaluates an item, not its result.
__device__ __forceinline__ int item_cost_bucket(const DevPlan &d, long long item) {
    const long long g = d.sitem_group[item];
    const int sub = d.sitem_sub[item];
    const int2 ck = d.sitem_chunk[item];
    const int s = find_seg(d.goff_tab, d.nsys, g);
    const SysDesc &sd = d.sys[s];
    const long long lg = g - sd.goff;
    const int2 cnt = d.lcnt[g];
    const int near_total = d.lnear[sd.lnoff + lg * 2 * (sd.lncap + 1) + 2 * cnt.y].y;
    const int gi = (int)(lg / sd.NGs), gj = (int)(lg - (long long)gi * sd.NGs);
    const int gx0 = gi * sd.TG, gy0 = gj * sd.TG;
    const int gx1 = min(sd.G, gx0 + sd.TG), gy1 = min(sd.G, gy0 + sd.TG);
    const int nbox = sd.TG * sd.TG;
    int nt = 0;  // the item's target set: a quadrant, one dense box, or the group's sparse boxes
    for (int c = gx0; c < gx1; c++)
        for (int r = gy0; r < gy1; r++) {
            const long long b = sd.boff + (long long)c * sd.G + r;
            const int nb = d.box_start[b + 1] - d.box_start[b];
            const int bi = (c - gx0) * sd.TG + (r - gy0);
            if (sub >= nbox) {
                if (bi == (sub - nbox) >> 2) nt += d.qcounts[4 * b + ((sub - nbox) & 3)];
            } else if (sub >= 0 ? bi == sub : box_item_kind(nb, d.dense_min, d.quad_min) == 0) {
                nt += nb;
            }
        }
    int c0, T;
    sitem_range(nt, ck.x, &c0, &T);
    // a sweep of T targets runs 32 / ceil(T / FORCE_R) slices; cost in full-warp target units
    const int nslice = 32 / max(1, (T + FORCE_R - 1) / FORCE_R);
    const unsigned long long cost =
        (unsigned long long)(STREAM_CHUNK / nslice) * (unsigned long long)(near_total + 2 * cnt.x) + 1ull;
    const int b = 63 - __clzll((long long)cost);
    return min(b, ITEM_BUCKETS - 1);
}

__global__ void __launch_bounds__(256) k_item_hist(DevPlan d) {
    __shared__ int h[ITEM_BUCKETS];
    if (threadIdx.x < ITEM_BUCKETS) h[threadIdx.x] = 0;
    __syncthreads();
    const long long nitems = d.sitem_off[d.NG_total];
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nitems; i += (long long)gridDim.x * blockDim.x) {
        const int b = item_cost_bucket(d, i);
        d.item_cost[i] = (unsigned char)b;  // for k_item_order
        atomicAdd(&h[b], 1);
    }
    __syncthreads();
    if (threadIdx.x < ITEM_BUCKETS && h[threadIdx.x]) atomicAdd(&d.item_bucket[threadIdx.x], h[threadIdx.x]);
}

__global__ void __launch_bounds__(256) k_item_order(DevPlan d) {
    __shared__ int off[ITEM_BUCKETS], h[ITEM_BUCKETS], base[ITEM_BUCKETS];
    if (threadIdx.x == 0) {
        int o = 0;
        for (int b = ITEM_BUCKETS - 1; b >= 0; b--) {  // heaviest bucket first
            off[b] = o;
            o += d.item_bucket[b];
        }
    }
    if (threadIdx.x < ITEM_BUCKETS) h[threadIdx.x] = 0;
    __syncthreads();
    const long long nitems = d.sitem_off[d.NG_total];
    const long long stride = (long long)gridDim.x * blockDim.x;
    // one pass of the grid per round; each round reserves a range per bucket for its block
    for (long long r0 = (long long)blockIdx.x * blockDim.x; r0 < nitems; r0 += stride) {
        const long long i = r0 + threadIdx.x;
        int b = -1, rank = 0;
        if (i < nitems) {
            b = d.item_cost[i];
            rank = atomicAdd(&h[b], 1);
        }
        __syncthreads();
        if (threadIdx.x < ITEM_BUCKETS) {
            base[threadIdx.x] = h[threadIdx.x] ? atomicAdd(&d.item_bucket[ITEM_BUCKETS + threadIdx.x], h[threadIdx.x]) : 0;
            h[threadIdx.x] = 0;
        }
        __syncthreads();
        if (b >= 0) d.item_order[off[b] + base[b] + rank] = (int)i;
        __syncthreads();
    }
}

cudaError_t launch_lists(const DevPlan &d, cudaStream_t st) {
    if (d.NG_total == 0) return cudaSuccess;
    long long grid = (long long)d.nsm * LISTS_MINB;
    if (grid * LW > d.NG_total) grid = (d.NG_total + LW - 1) / LW;
    k_lists<<<(unsigned)grid, LW * 32, 0, st>>>(d);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(d.item_bucket, 0, sizeof(int) * 2 * ITEM_BUCKETS, st);
    if (e != cudaSuccess) return e;
    long long items_max = d.NG_total + d.n_total / d.dense_min +
                          (d.quad_min > 0 ? 4 * (d.n_total / d.quad_min) : 0) + d.n_total / STREAM_ITEM_DIV + 1;  // >= items
    long long ig = (items_max + 255) / 256;
    if (ig > (long long)d.nsm * 8) ig = (long long)d.nsm * 8;
    k_item_hist<<<(unsigned)ig, 256, 0, st>>>(d);
    k_item_order<<<(unsigned)ig, 256, 0, st>>>(d);
    return cudaGetLastError();
}

}  // namespace bh

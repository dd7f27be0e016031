// bh_tree.cu -- create_tree and summarize kernels.
//
// create_tree = prologue -> bbox -> place -> scan (3 phases) -> scatter.
//   Replaces set_particles_bounding_box (python-bh/barneshut/implementations/base.py:211-239),
//   g_place_particles, g_calculate_box_cumm, g_sort_particles
//   (python-bh/barneshut/kernels/grid_decomposition/gpu/grid.py:15-76).
// summarize = leaf moments (segmented warp reduction) -> pyramid levels -> records.
//   Replaces g_summarize (gpu/grid.py:78-114) and calc_COM (internals/cloud.py:9-17).
#include "bh_internal.cuh"

namespace bh {

constexpr int TPB = 256;
constexpr int SCAN_TILE = 4096;  // counts per scan tile (256 threads x 16)

static inline unsigned grid_for(long long n, int tpb, long long cap) {
    long long b = (n + tpb - 1) / tpb;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return (unsigned)b;
}

// ----------------------------------------------------------------- prologue
// Zero the box histogram and the leaf moments, reset the bounding-box
// accumulators and pair counters, advance the state epoch.
__global__ void k_prologue(DevPlan d) {
    long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long stride = (long long)gridDim.x * blockDim.x;
    if (tid == 0) {
        d.glob->epoch += 1;
        d.glob->near_pairs = 0;
        d.glob->far_pairs = 0;
        d.glob->corr_pairs = 0;
    }
    if (tid < d.nsys) {
        d.dyn[tid].bbmin[0] = d.dyn[tid].bbmin[1] = ~0ull;
        d.dyn[tid].bbmax[0] = d.dyn[tid].bbmax[1] = 0ull;
    }
    for (long long b = tid; b < d.B_total; b += stride) {
        d.counts[b] = 0;
        reinterpret_cast<int4 *>(d.qcounts)[b] = make_int4(0, 0, 0, 0);
        int s = find_seg(d.boff_tab, d.nsys, b);
        long long c = d.sys[s].coff + (b - d.sys[s].boff);
        double *q = d.mom + 6 * c;
#pragma unroll
        for (int k = 0; k < 6; k++) q[k] = 0.0;
    }
}

// --------------------------------------------------------------------- bbox
// Min / max of x and y per system on the ordered-integer image of the doubles
// (integer min/max, no FP64 pipe work).  Each block reduces a contiguous tile.
__global__ void __launch_bounds__(TPB) k_bbox(DevPlan d) {
    const int cur = d.glob->epoch & 1;
    const double *X = d.X[cur], *Y = d.Y[cur];
    __shared__ unsigned long long red[4][TPB / 32];
    __shared__ int sys0;
    const long long tile = (long long)TPB * 16;
    for (long long t0 = (long long)blockIdx.x * tile; t0 < d.n_total; t0 += (long long)gridDim.x * tile) {
        long long t1 = t0 + tile < d.n_total ? t0 + tile : d.n_total;
        if (threadIdx.x == 0) sys0 = find_seg(d.poff_tab, d.nsys, t0);
        __syncthreads();
        int s_first = sys0;
        bool one_sys = d.poff_tab[s_first + 1] >= t1;
        unsigned long long mn0 = ~0ull, mn1 = ~0ull, mx0 = 0, mx1 = 0;
        int cs = s_first;
        for (long long i = t0 + threadIdx.x; i < t1; i += TPB) {
            if (!one_sys) {
                int s = find_seg(d.poff_tab, d.nsys, i);
                if (s != cs) {
                    if (mx0 | mx1) {
                        atomicMin(&d.dyn[cs].bbmin[0], mn0); atomicMin(&d.dyn[cs].bbmin[1], mn1);
                        atomicMax(&d.dyn[cs].bbmax[0], mx0); atomicMax(&d.dyn[cs].bbmax[1], mx1);
                    }
                    mn0 = mn1 = ~0ull; mx0 = mx1 = 0; cs = s;
                }
            }
            unsigned long long ux = ord_bits(X[i]), uy = ord_bits(Y[i]);
            mn0 = ux < mn0 ? ux : mn0; mx0 = ux > mx0 ? ux : mx0;
            mn1 = uy < mn1 ? uy : mn1; mx1 = uy > mx1 ? uy : mx1;
        }
        if (!one_sys) {
            if (mx0 | mx1) {
                atomicMin(&d.dyn[cs].bbmin[0], mn0); atomicMin(&d.dyn[cs].bbmin[1], mn1);
                atomicMax(&d.dyn[cs].bbmax[0], mx0); atomicMax(&d.dyn[cs].bbmax[1], mx1);
            }
        } else {
            for (int o = 16; o; o >>= 1) {
                unsigned long long a = __shfl_xor_sync(0xffffffffu, mn0, o); mn0 = a < mn0 ? a : mn0;
                a = __shfl_xor_sync(0xffffffffu, mn1, o); mn1 = a < mn1 ? a : mn1;
                a = __shfl_xor_sync(0xffffffffu, mx0, o); mx0 = a > mx0 ? a : mx0;
                a = __shfl_xor_sync(0xffffffffu, mx1, o); mx1 = a > mx1 ? a : mx1;
            }
            int w = threadIdx.x >> 5, l = threadIdx.x & 31;
            if (l == 0) { red[0][w] = mn0; red[1][w] = mn1; red[2][w] = mx0; red[3][w] = mx1; }
            __syncthreads();
            if (threadIdx.x == 0) {
                for (int k = 1; k < TPB / 32; k++) {
                    mn0 = red[0][k] < mn0 ? red[0][k] : mn0; mn1 = red[1][k] < mn1 ? red[1][k] : mn1;
                    mx0 = red[2][k] > mx0 ? red[2][k] : mx0; mx1 = red[3][k] > mx1 ? red[3][k] : mx1;
                }
                atomicMin(&d.dyn[s_first].bbmin[0], mn0); atomicMin(&d.dyn[s_first].bbmin[1], mn1);
                atomicMax(&d.dyn[s_first].bbmax[0], mx0); atomicMax(&d.dyn[s_first].bbmax[1], mx1);
            }
        }
        __syncthreads();
    }
}

// One thread per system: the square bounding box (helpers/grid.py:10-26), its
// box edge step = edge / G (base.py:233) and 1 / step, once per step.
__device__ void bbox_finalize_sys(const DevPlan &d, int s) {
    SysDyn &dy = d.dyn[s];
    double mnx = unord_bits(dy.bbmin[0]), mny = unord_bits(dy.bbmin[1]);
    double mxx = unord_bits(dy.bbmax[0]), mxy = unord_bits(dy.bbmax[1]);
    if (d.sys[s].fixed_grid) {  // part of a larger system: the whole system's extents
        mnx = d.sys[s].fg_ext[0];
        mny = d.sys[s].fg_ext[1];
        mxx = d.sys[s].fg_ext[2];
        mxy = d.sys[s].fg_ext[3];
    }
    double step;
    square_bbox(mnx, mny, mxx, mxy, d.sys[s].G, &step);
    dy.minx = mnx;
    dy.miny = mny;
    dy.step = step;
    dy.inv_step = step > 0.0 ? 1.0 / step : 0.0;
    // float key estimate: p and mn rounded to float (relative error 2^-24 each), their
    // difference and the product with float(1 / step) rounded (2^-24 each); in box edges the
    // error is at most ((|p| + |mn|) / step + 2 q) 2^-24 <= ((2 |mn| + |edge|) / step + 2 G) 2^-24;
    // a factor 4 covers the remaining roundings
    dy.minx_f = __double2float_rn(mnx);
    dy.miny_f = __double2float_rn(mny);
    dy.inv_step_f = __double2float_rn(dy.inv_step);
    if (step > 0.0 && isfinite(step)) {
        const double am = fmax(fabs(mnx), fabs(mny)), G = (double)d.sys[s].G;
        const double tol = 4.0 * ((2.0 * am + G * step) / step + 2.0 * G) * 5.9604644775390625e-8;
        dy.key_tol = tol < 0.25 ? (float)tol : 1.f;
    } else {
        dy.key_tol = 1.f;  // the FP64 key for every particle
    }
}

// One CTA per system: thread 0 squares the bounding box and derives the grid; then the CTA
// tabulates the box origins mn + k step (FP64), which the scatter reads instead of forming
// them per particle on the slow FP64 pipe.
__global__ void k_bbox_finalize(DevPlan d) {
    const int s = blockIdx.x;
    SysDyn &dy = d.dyn[s];
    if (d.sys[s].n == 0) return;
    if (threadIdx.x == 0) bbox_finalize_sys(d, s);
    __syncthreads();
    const int G = d.sys[s].G;
    double *org = d.org + d.sys[s].ooff;
    for (int k = threadIdx.x; k < G; k += blockDim.x) {
        org[k] = box_origin(dy.minx, k, dy.step);
        org[G + k] = box_origin(dy.miny, k, dy.step);
    }
}

// -------------------------------------------------------------------- place
// Box keys bit-exact with the reference's FP64 keys (computed at twice the box resolution, so
// each particle also gets its quadrant within the box), and a warp-aggregated histogram of
// boxes and of (box, quadrant) pairs; a particle's slot is its rank within its quadrant.
__global__ void __launch_bounds__(TPB) k_place(DevPlan d) {
    const int cur = d.glob->epoch & 1;
    const double *X = d.X[cur], *Y = d.Y[cur];
    const int lane = threadIdx.x & 31;
    long long stride = (long long)gridDim.x * blockDim.x;
    long long base = (long long)blockIdx.x * blockDim.x;
    for (; base < d.n_total; base += stride) {
        long long i = base + threadIdx.x;
        int key = -1;
        if (i < d.n_total) {
            int s = find_seg(d.poff_tab, d.nsys, i);
            const SysDesc &sd = d.sys[s];
            const SysDyn &dy = d.dyn[s];
            double x = X[i], y = Y[i];
            // finite test on the exponent bits (no FP64 operation)
            const unsigned hx = (unsigned)(__double_as_longlong(x) >> 52) & 0x7FFu;
            const unsigned hy = (unsigned)(__double_as_longlong(y) >> 52) & 0x7FFu;
            if (hx == 0x7FFu || hy == 0x7FFu) raise_err(d.glob, 1u /*BH_DEV_NAN_POSITION*/);
            // keys at twice the box resolution: box key and quadrant within the box
            const int k2x = half_key1_f32(x, dy.minx, dy.step, dy.inv_step, dy.minx_f, dy.inv_step_f, dy.key_tol, sd.G);
            const int k2y = half_key1_f32(y, dy.miny, dy.step, dy.inv_step, dy.miny_f, dy.inv_step_f, dy.key_tol, sd.G);
            const int box = (int)(sd.boff + (long long)(k2x >> 1) * sd.G + (k2y >> 1));
            key = 4 * box + (k2x & 1) * 2 + (k2y & 1);
        }
        // lanes with the same (box, quadrant) elect one leader that adds the group's size to the
        // box count (the scan's input) and to the quadrant count, whose old value is the group's
        // first slot in the quadrant
        unsigned peers = __match_any_sync(0xffffffffu, key);
        int leader = __ffs(peers) - 1;
        int rank = __popc(peers & ((1u << lane) - 1u));
        int old = 0;
        if (lane == leader && key >= 0) {
            atomicAdd(&d.counts[key >> 2], __popc(peers));
            old = atomicAdd(&d.qcounts[key], __popc(peers));
        }
        old = __shfl_sync(0xffffffffu, old, leader);
        if (i < d.n_total) {
            d.key[i] = key;  // 4 * box + quadrant
            d.slot[i] = old + rank;
        }
    }
}

// --------------------------------------------------------------------- scan
// Exclusive scan of the box histogram (all systems concatenated; systems are
// laid out in particle order, so the global prefix is the global particle
// index of each box's first particle).  Phase 1: per-tile sums; phase 2: one
// block scans the tile sums; phase 3: per-tile scan plus carry.
__device__ __forceinline__ int block_excl_scan(int v, int *sh, int *total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        int t = lane < nw ? sh[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < nw) sh[lane] = t;
    }
    __syncthreads();
    int pre = (w ? sh[w - 1] : 0) + x - v;
    if (total) *total = sh[nw - 1];
    __syncthreads();
    return pre;
}

// Generic over (in, out, n): out[i] = sum(in[0..i)), out[n] = total.
__global__ void __launch_bounds__(TPB) k_scan_tiles(const int *in, long long n, int *tiles) {
    __shared__ int sh[32];
    long long t0 = (long long)blockIdx.x * SCAN_TILE;
    int s = 0;
    for (int k = threadIdx.x; k < SCAN_TILE; k += TPB) {
        long long b = t0 + k;
        if (b < n) s += in[b];
    }
    int tot;
    block_excl_scan(s, sh, &tot);
    if (threadIdx.x == 0) tiles[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(1024) k_scan_sums(int *tiles, int ntiles, int *out, long long n) {
    __shared__ int sh[32];
    int carry = 0;
    for (int t0 = 0; t0 < ntiles; t0 += 1024) {
        int t = t0 + threadIdx.x;
        int v = t < ntiles ? tiles[t] : 0;
        int tot;
        int p = block_excl_scan(v, sh, &tot);
        if (t < ntiles) tiles[t] = carry + p;
        carry += tot;
    }
    if (threadIdx.x == 0) out[n] = carry;
}

__global__ void __launch_bounds__(TPB) k_scan_apply(const int *in, long long n, const int *tiles,
                                                   int *out) {
    __shared__ int sh[32];
    long long t0 = (long long)blockIdx.x * SCAN_TILE;
    // each thread owns 16 consecutive entries
    long long b0 = t0 + (long long)threadIdx.x * 16;
    int v[16], s = 0;
#pragma unroll
    for (int k = 0; k < 16; k++) {
        v[k] = (b0 + k < n) ? in[b0 + k] : 0;
        s += v[k];
    }
    int pre = block_excl_scan(s, sh, nullptr) + tiles[blockIdx.x];
#pragma unroll
    for (int k = 0; k < 16; k++) {
        if (b0 + k < n) out[b0 + k] = pre;
        pre += v[k];
    }
}

static cudaError_t scan_excl(const int *in, int *out, long long n, int *tiles, cudaStream_t st) {
    int ntiles = (int)((n + SCAN_TILE - 1) / SCAN_TILE);
    if (ntiles < 1) ntiles = 1;
    k_scan_tiles<<<ntiles, TPB, 0, st>>>(in, n, tiles);
    k_scan_sums<<<1, 1024, 0, st>>>(tiles, ntiles, out, n);
    k_scan_apply<<<ntiles, TPB, 0, st>>>(in, n, tiles, out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- work items
// Force work items: a target group with nt targets is split into
// ceil(nt / TARGET_CHUNK) items so that dense groups spread over many CTAs.
__global__ void __launch_bounds__(TPB) k_group_items(DevPlan d) {
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < d.NG_total; g += stride) {
        int s = find_seg(d.goff_tab, d.nsys, g);
        const SysDesc &sd = d.sys[s];
        long long lg = g - sd.goff;
        int gi = (int)(lg / sd.NGs), gj = (int)(lg - (long long)gi * sd.NGs);
        int gx0 = gi * sd.TG, gy0 = gj * sd.TG;
        int gx1 = min(sd.G, gx0 + sd.TG), gy1 = min(sd.G, gy0 + sd.TG);
        int nt = 0;
        for (int c = gx0; c < gx1; c++) {
            long long b0 = sd.boff + (long long)c * sd.G + gy0;
            nt += d.box_start[b0 + (gy1 - gy0)] - d.box_start[b0];
        }
        d.item_cnt[g] = (nt + d.chunk - 1) / d.chunk;
    }
}

__global__ void __launch_bounds__(TPB) k_fill_items(DevPlan d) {
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < d.NG_total; g += stride) {
        int o = d.item_off[g], c = d.item_cnt[g];
        for (int k = 0; k < c; k++) d.item_group[o + k] = (int)g;
    }
}

// List-streaming work items.  Per group: the boxes holding fewer than dense_min particles share
// ceil(n_sparse / chunk) items (sub = -1); every denser box gets ceil(n_box / chunk) items of its
// own (sub = cx * TG + cy), which use per-box refined near lists, and a box holding at least
// quad_min particles gets items per quadrant instead (sub = TG^2 + 4 (cx * TG + cy) + quadrant),
// which use per-quadrant refined near lists.  A set of nt targets splits into sitem_count(nt)
// items: full chunks of STREAM_CHUNK and the remainder's pieces (sitem_range).
__global__ void __launch_bounds__(TPB) k_sitem_count(DevPlan d) {
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < d.NG_total; g += stride) {
        int s = find_seg(d.goff_tab, d.nsys, g);
        const SysDesc &sd = d.sys[s];
        long long lg = g - sd.goff;
        int gi = (int)(lg / sd.NGs), gj = (int)(lg - (long long)gi * sd.NGs);
        int gx0 = gi * sd.TG, gy0 = gj * sd.TG;
        int gx1 = min(sd.G, gx0 + sd.TG), gy1 = min(sd.G, gy0 + sd.TG);
        int sparse = 0, cnt = 0;
        for (int c = gx0; c < gx1; c++)
            for (int r = gy0; r < gy1; r++) {
                const long long b = sd.boff + (long long)c * sd.G + r;
                const int nb = d.box_start[b + 1] - d.box_start[b];
                const int kind = box_item_kind(nb, d.dense_min, d.quad_min);
                if (kind == 2) {
                    for (int q = 0; q < 4; q++) cnt += sitem_count(d.qcounts[4 * b + q]);
                } else if (kind == 1) {
                    cnt += sitem_count(nb);
                } else {
                    sparse += nb;
                }
            }
        d.sitem_cnt[g] = cnt + sitem_count(sparse);
    }
}

__global__ void __launch_bounds__(TPB) k_sitem_fill(DevPlan d) {
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < d.NG_total; g += stride) {
        int s = find_seg(d.goff_tab, d.nsys, g);
        const SysDesc &sd = d.sys[s];
        long long lg = g - sd.goff;
        int gi = (int)(lg / sd.NGs), gj = (int)(lg - (long long)gi * sd.NGs);
        int gx0 = gi * sd.TG, gy0 = gj * sd.TG;
        int gx1 = min(sd.G, gx0 + sd.TG), gy1 = min(sd.G, gy0 + sd.TG);
        const int nbox = sd.TG * sd.TG;
        int o = d.sitem_off[g];
        int sparse = 0;
        for (int c = gx0; c < gx1; c++)
            for (int r = gy0; r < gy1; r++) {
                const long long b = sd.boff + (long long)c * sd.G + r;
                const int nb = d.box_start[b + 1] - d.box_start[b];
                if (box_item_kind(nb, d.dense_min, d.quad_min) == 0) sparse += nb;
            }
        const int ns = sitem_count(sparse);
        for (int k = 0; k < ns; k++, o++) {
            d.sitem_group[o] = (int)g;
            d.sitem_sub[o] = -1;
            d.sitem_chunk[o] = make_int2(k, ns);
        }
        for (int c = gx0; c < gx1; c++)
            for (int r = gy0; r < gy1; r++) {
                const long long b = sd.boff + (long long)c * sd.G + r;
                const int nb = d.box_start[b + 1] - d.box_start[b];
                const int kind = box_item_kind(nb, d.dense_min, d.quad_min);
                const int bi = (c - gx0) * sd.TG + (r - gy0);
                if (kind == 1) {
                    const int nk = sitem_count(nb);
                    for (int k = 0; k < nk; k++, o++) {
                        d.sitem_group[o] = (int)g;
                        d.sitem_sub[o] = bi;
                        d.sitem_chunk[o] = make_int2(k, nk);
                    }
                } else if (kind == 2) {
                    for (int q = 0; q < 4; q++) {
                        const int nk = sitem_count(d.qcounts[4 * b + q]);
                        for (int k = 0; k < nk; k++, o++) {
                            d.sitem_group[o] = (int)g;
                            d.sitem_sub[o] = nbox + 4 * bi + q;
                            d.sitem_chunk[o] = make_int2(k, nk);
                        }
                    }
                }
            }
    }
}

// ------------------------------------------------------------------ scatter
// Counting-sort scatter into box order, each box's particles quadrant by quadrant:
// destination = box_start[box] + (particles of the box's earlier quadrants) + slot.
// Writes the FP64 state of the next buffer, the packed float4 record (offsets
// from the box origin computed in FP64, rounded once to float) and the
// per-sorted-particle key.
__global__ void __launch_bounds__(TPB) k_scatter(DevPlan d) {
    const int cur = d.glob->epoch & 1, nxt = cur ^ 1;
    // SU particles per thread per round, each stage's loads issued for all of them before the
    // next stage uses them (the chain key -> box start and quadrant counts -> destination, and
    // the state loads, would otherwise run one particle at a time)
    constexpr int SU = 4;
    const long long n = d.n_total, stride = (long long)gridDim.x * blockDim.x;
    for (long long i0 = (long long)blockIdx.x * blockDim.x + threadIdx.x; i0 < n; i0 += SU * stride) {
        int key4[SU], dst[SU];
#pragma unroll
        for (int u = 0; u < SU; u++) {
            const long long i = i0 + u * stride;
            key4[u] = i < n ? d.key[i] : 0;
        }
#pragma unroll
        for (int u = 0; u < SU; u++) {
            const long long i = i0 + u * stride;
            dst[u] = 0;
            if (i < n) {
                const int key = key4[u] >> 2, quad = key4[u] & 3;
                const int4 qc = reinterpret_cast<const int4 *>(d.qcounts)[key];
                const int qpre = (quad > 0 ? qc.x : 0) + (quad > 1 ? qc.y : 0) + (quad > 2 ? qc.z : 0);
                dst[u] = d.box_start[key] + qpre + d.slot[i];
            }
        }
        double x[SU], y[SU], m[SU], vx[SU], vy[SU];
        int pid[SU];
#pragma unroll
        for (int u = 0; u < SU; u++) {
            const long long i = i0 + u * stride;
            if (i < n) {
                x[u] = d.X[cur][i];
                y[u] = d.Y[cur][i];
                m[u] = d.M[cur][i];
                vx[u] = d.VX[cur][i];
                vy[u] = d.VY[cur][i];
                pid[u] = d.PID[cur][i];
            }
        }
#pragma unroll
        for (int u = 0; u < SU; u++) {
            const long long i = i0 + u * stride;
            if (i >= n) continue;
            const int key = key4[u] >> 2, t = dst[u];
            const int s = find_seg(d.boff_tab, d.nsys, key);
            const SysDesc &sd = d.sys[s];
            const int lb = (int)(key - sd.boff);
            const int kx = lb / sd.G, ky = lb - kx * sd.G;
            d.X[nxt][t] = x[u];
            d.Y[nxt][t] = y[u];
            d.VX[nxt][t] = vx[u];
            d.VY[nxt][t] = vy[u];
            d.M[nxt][t] = m[u];
            d.PID[nxt][t] = pid[u];
            const double *org = d.org + sd.ooff;  // box origins (k_bbox_finalize)
            const float ox = f64_to_f32_rn(__dsub_rn(x[u], org[kx]));
            const float oy = f64_to_f32_rn(__dsub_rn(y[u], org[sd.G + ky]));
            const float mf = f64_to_f32_rn(m[u]);
            d.P[t] = make_float4(ox, oy, mf, __int_as_float(t));
            d.PD[2 * (long long)t] = make_float4(ox, ox, oy, oy);
            d.PD[2 * (long long)t + 1] = make_float4(mf, mf, __int_as_float(t), __int_as_float((kx << 16) | ky));
            d.skey[t] = key;
        }
    }
}

// ------------------------------------------------------------- leaf moments
// Segmented warp reduction over the box-sorted particles: lanes holding the
// same box key are contiguous; an inclusive segmented scan of the float
// contributions (offsets are box-relative, so 32 terms in FP32 are exact to
// ~1e-7 of a box) ends in the segment's last lane, which adds the partial
// into the box's FP64 moments with FP64 atomics.
__global__ void __launch_bounds__(TPB) k_leaf_moments(DevPlan d) {
    const int lane = threadIdx.x & 31;
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long base = (long long)blockIdx.x * blockDim.x; base < d.n_total; base += stride) {
        long long i = base + threadIdx.x;
        int key = -1;
        float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (i < d.n_total) {
            key = d.skey[i];
            float4 p = d.P[i];
            v[0] = p.z;
            v[1] = p.z * p.x;
            v[2] = p.z * p.y;
            v[3] = v[1] * p.x;
            v[4] = v[1] * p.y;
            v[5] = v[2] * p.y;
        }
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int k2 = __shfl_up_sync(0xffffffffu, key, o);
#pragma unroll
            for (int c = 0; c < 6; c++) {
                float y = __shfl_up_sync(0xffffffffu, v[c], o);
                if (lane >= o && k2 == key) v[c] += y;
            }
        }
        int knext = __shfl_down_sync(0xffffffffu, key, 1);
        bool tail = (lane == 31) || (knext != key);
        if (tail && key >= 0) {
            int s = find_seg(d.boff_tab, d.nsys, key);
            long long c = d.sys[s].coff + (key - d.sys[s].boff);
            double *q = d.mom + 6 * c;
#pragma unroll
            for (int k = 0; k < 6; k++) atomicAdd(q + k, (double)v[k]);
        }
    }
}

// ------------------------------------------------------------------ pyramid
// Level-l cell = sum of its (up to) four level-(l-1) children, moments shifted
// from the child origin to the parent origin (FP64).
__device__ __forceinline__ void pyramid_cell(const DevPlan &d, int l, long long t) {
    const long long *tab = d.lvl_tab + (long long)l * (d.nsys + 1);
    int s = find_seg(tab, d.nsys, t);
    const SysDesc &sd = d.sys[s];
    double step = d.dyn[s].step;
    long long loc = t - tab[s];
    int gl = sd.lvg[l], gc = sd.lvg[l - 1];
    int i = (int)(loc / gl), j = (int)(loc - (long long)i * gl);
    double p[6] = {0, 0, 0, 0, 0, 0};
    for (int a = 0; a < 2; a++)
        for (int b = 0; b < 2; b++) {
            int ci = 2 * i + a, cj = 2 * j + b;
            if (ci >= gc || cj >= gc) continue;
            const double *c = d.mom + 6 * (sd.coff + sd.lvoff[l - 1] + (long long)ci * gc + cj);
            double dx = (double)(a << (l - 1)) * step, dy = (double)(b << (l - 1)) * step;
            double M = c[0], Sx = c[1], Sy = c[2];
            p[0] += M;
            p[1] += Sx + M * dx;
            p[2] += Sy + M * dy;
            p[3] += c[3] + 2.0 * dx * Sx + M * dx * dx;
            p[4] += c[4] + dx * Sy + dy * Sx + M * dx * dy;
            p[5] += c[5] + 2.0 * dy * Sy + M * dy * dy;
        }
    double *q = d.mom + 6 * (sd.coff + sd.lvoff[l] + loc);
#pragma unroll
    for (int k = 0; k < 6; k++) q[k] = p[k];
}

__global__ void __launch_bounds__(TPB) k_pyramid_level(DevPlan d, int l) {
    const long long total = d.lvl_tab[(long long)l * (d.nsys + 1) + d.nsys];
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += stride)
        pyramid_cell(d, l, t);
}

// Levels l0 .. Lmax - 1 in one CTA (their cells are few): level by level, a barrier between.
constexpr int TAIL_THREADS = 1024;
constexpr long long TAIL_MAX_CELLS = 256;  // the first level given to the single CTA (FP64 work on one SM)
__global__ void __launch_bounds__(TAIL_THREADS) k_pyramid_tail(DevPlan d, int l0) {
    for (int l = l0; l < d.Lmax; l++) {
        const long long total = d.lvl_tab[(long long)l * (d.nsys + 1) + d.nsys];
        for (long long t = threadIdx.x; t < total; t += blockDim.x) pyramid_cell(d, l, t);
        __syncthreads();  // level l is complete before level l + 1 reads it
    }
}

// Float records: centre of mass relative to the cell origin and mass; second
// moments about the centre of mass normalised by M s^2 (s = cell edge).
__global__ void __launch_bounds__(TPB) k_records(DevPlan d, int second) {
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < d.C_total; c += stride) {
        const double *q = d.mom + 6 * c;
        double M = q[0];
        if (M > 0.0) {
            double cx = q[1] / M, cy = q[2] / M;
            d.rec[c] = make_float4(f64_to_f32_rn(cx), f64_to_f32_rn(cy), f64_to_f32_rn(M), 0.f);
            if (!second) continue;
            int s = find_seg(d.coff_tab, d.nsys, c);
            const SysDesc &sd = d.sys[s];
            long long loc = c - sd.coff;
            int l = 0;
            while (l + 1 < sd.L && sd.lvoff[l + 1] <= loc) l++;
            double sz = (double)(1 << l) * d.dyn[s].step;
            double nrm = 1.0 / (M * sz * sz);
            double ixx = q[3] - q[1] * cx, ixy = q[4] - q[1] * cy, iyy = q[5] - q[2] * cy;
            d.rec2[c] = make_float4(f64_to_f32_rn(ixx * nrm), f64_to_f32_rn(ixy * nrm),
                                    f64_to_f32_rn(iyy * nrm), 0.f);
        } else {
            d.rec[c] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (second) d.rec2[c] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
}

// ------------------------------------------------------------------ launches
cudaError_t launch_prologue(const DevPlan &d, cudaStream_t st) {
    long long n = d.B_total > d.nsys ? d.B_total : d.nsys;
    k_prologue<<<grid_for(n, TPB, d.nsm * 16LL), TPB, 0, st>>>(d);
    return cudaGetLastError();
}
cudaError_t launch_bbox(const DevPlan &d, cudaStream_t st) {
    if (d.n_total == 0) return cudaSuccess;
    k_bbox<<<grid_for(d.n_total, TPB * 16, d.nsm * 8LL), TPB, 0, st>>>(d);
    return cudaGetLastError();
}
cudaError_t launch_place(const DevPlan &d, cudaStream_t st) {
    if (d.n_total == 0) return cudaSuccess;
    k_bbox_finalize<<<d.nsys, 128, 0, st>>>(d);
    k_place<<<grid_for(d.n_total, TPB, d.nsm * 8LL), TPB, 0, st>>>(d);
    return cudaGetLastError();
}
cudaError_t launch_scan(const DevPlan &d, cudaStream_t st) {
    return scan_excl(d.counts, d.box_start, d.B_total, d.tile_sums, st);
}
// Work items of the walk kernel and of the learned correction (group, target chunk).
cudaError_t launch_walk_items(const DevPlan &d, cudaStream_t st) {
    unsigned g = grid_for(d.NG_total, TPB, d.nsm * 8LL);
    k_group_items<<<g, TPB, 0, st>>>(d);
    cudaError_t e = scan_excl(d.item_cnt, d.item_off, d.NG_total, d.tile_sums, st);
    if (e != cudaSuccess) return e;
    k_fill_items<<<g, TPB, 0, st>>>(d);
    return cudaGetLastError();
}
// The step's work items: the walk items where the walk or the learned correction runs, the
// list-streaming items where the lists are streamed (a streaming plan builds walk items only
// with the learned correction, or on demand for bh_learned_pairs).
cudaError_t launch_items(const DevPlan &d, cudaStream_t st) {
    cudaError_t e;
    if (!d.stream || d.learned) {
        e = launch_walk_items(d, st);
        if (e != cudaSuccess) return e;
    }
    if (d.stream) {
        unsigned g = grid_for(d.NG_total, TPB, d.nsm * 8LL);
        k_sitem_count<<<g, TPB, 0, st>>>(d);
        e = scan_excl(d.sitem_cnt, d.sitem_off, d.NG_total, d.tile_sums, st);
        if (e != cudaSuccess) return e;
        k_sitem_fill<<<g, TPB, 0, st>>>(d);
    }
    return cudaGetLastError();
}
cudaError_t launch_scatter(const DevPlan &d, cudaStream_t st) {
    if (d.n_total == 0) return cudaSuccess;
    k_scatter<<<grid_for(d.n_total, TPB, d.nsm * 8LL), TPB, 0, st>>>(d);
    return cudaGetLastError();
}
cudaError_t launch_summarize(const DevPlan &d, cudaStream_t st) {
    if (d.n_total > 0) k_leaf_moments<<<grid_for(d.n_total, TPB, d.nsm * 8LL), TPB, 0, st>>>(d);
    return launch_pyramid(d, st);
}
cudaError_t launch_pyramid(const DevPlan &d, cudaStream_t st) {
    for (int l = 1; l < d.Lmax; l++) {
        // the level's cell count over all systems is known on the host: one thread per cell
        // while the level is large, then one CTA for all the remaining (small) levels
        if (d.lvl_cells[l] <= TAIL_MAX_CELLS) {
            k_pyramid_tail<<<1, TAIL_THREADS, 0, st>>>(d, l);
            break;
        }
        k_pyramid_level<<<grid_for(d.lvl_cells[l], TPB, d.nsm * 4LL), TPB, 0, st>>>(d, l);
    }
    // the normalised second moments feed only the learned correction
    return launch_records(d, d.learned != 0, st);
}
cudaError_t launch_records(const DevPlan &d, bool second, cudaStream_t st) {
    k_records<<<grid_for(d.C_total, TPB, d.nsm * 8LL), TPB, 0, st>>>(d, second ? 1 : 0);
    return cudaGetLastError();
}

}  // namespace bh

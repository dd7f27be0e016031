// bh_tree.cu -- create_tree and summarize kernels.
//
// create_tree = prologue -> bbox (its last block squares the box) -> place -> scan (one pass)
//   -> scatter (permutation, per-quadrant sort, gather) -> work items (one pass).
//   Replaces set_particles_bounding_box (python-bh/barneshut/implementations/base.py:211-239),
//   g_place_particles, g_calculate_box_cumm, g_sort_particles
//   (python-bh/barneshut/kernels/grid_decomposition/gpu/grid.py:15-76).
// summarize = one kernel over tiles of leaf boxes: leaf moments, pyramid, records.
//   Replaces g_summarize (gpu/grid.py:78-114) and calc_COM (internals/cloud.py:9-17).
#include "bh_internal.cuh"

namespace bh {

constexpr int TPB = 256;

static inline unsigned grid_for(long long n, int tpb, long long cap) {
    long long b = (n + tpb - 1) / tpb;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return (unsigned)b;
}

// ----------------------------------------------------------------- prologue
// Zero the box and quadrant histograms, reset the bounding-box accumulators and
// pair counters, advance the state epoch.
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
        reinterpret_cast<int4 *>(d.qcounts)[b] = make_int4(0, 0, 0, 0);
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

// --------------------------------------------------------------------- bbox
// Min / max of x and y per system on the ordered-integer image of the doubles
// (integer min/max, no FP64 pipe work).  Each block reduces a contiguous tile.
__device__ __forceinline__ void minmax_ord(unsigned long long u, unsigned long long &mn, unsigned long long &mx) {
    mn = u < mn ? u : mn;
    mx = u > mx ? u : mx;
}

__device__ __forceinline__ void bbox_block_commit(const DevPlan &d, int s, unsigned long long mn0,
                                                  unsigned long long mn1, unsigned long long mx0,
                                                  unsigned long long mx1, unsigned long long (*red)[TPB / 32]) {
    for (int o = 16; o; o >>= 1) {
        unsigned long long a = __shfl_xor_sync(0xffffffffu, mn0, o); mn0 = a < mn0 ? a : mn0;
        a = __shfl_xor_sync(0xffffffffu, mn1, o); mn1 = a < mn1 ? a : mn1;
        a = __shfl_xor_sync(0xffffffffu, mx0, o); mx0 = a > mx0 ? a : mx0;
        a = __shfl_xor_sync(0xffffffffu, mx1, o); mx1 = a > mx1 ? a : mx1;
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { red[0][w] = mn0; red[1][w] = mn1; red[2][w] = mx0; red[3][w] = mx1; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < TPB / 32; k++) {
            mn0 = red[0][k] < mn0 ? red[0][k] : mn0; mn1 = red[1][k] < mn1 ? red[1][k] : mn1;
            mx0 = red[2][k] > mx0 ? red[2][k] : mx0; mx1 = red[3][k] > mx1 ? red[3][k] : mx1;
        }
        if (mx0 | mx1) {
            atomicMin(&d.dyn[s].bbmin[0], mn0); atomicMin(&d.dyn[s].bbmin[1], mn1);
            atomicMax(&d.dyn[s].bbmax[0], mx0); atomicMax(&d.dyn[s].bbmax[1], mx1);
        }
    }
    __syncthreads();
}

__global__ void __launch_bounds__(TPB) k_bbox(DevPlan d) {
    const int cur = d.glob->epoch & 1;
    const double *X = d.X[cur], *Y = d.Y[cur];
    __shared__ unsigned long long red[4][TPB / 32];
    __shared__ int sys0;
    if (d.nsys == 1) {
        // one system: a grid-stride sweep over 16-byte pairs, four pairs of each array in flight
        // per thread (the state arrays are 256-byte aligned)
        const long long n2 = d.n_total >> 1, stride = (long long)gridDim.x * TPB;
        const double2 *X2 = reinterpret_cast<const double2 *>(X), *Y2 = reinterpret_cast<const double2 *>(Y);
        unsigned long long mn0 = ~0ull, mn1 = ~0ull, mx0 = 0, mx1 = 0;
        long long i = (long long)blockIdx.x * TPB + threadIdx.x;
        for (; i + 3 * stride < n2; i += 4 * stride) {
            double2 a[4], b[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                a[u] = X2[i + u * stride];
                b[u] = Y2[i + u * stride];
            }
#pragma unroll
            for (int u = 0; u < 4; u++) {
                minmax_ord(ord_bits(a[u].x), mn0, mx0);
                minmax_ord(ord_bits(a[u].y), mn0, mx0);
                minmax_ord(ord_bits(b[u].x), mn1, mx1);
                minmax_ord(ord_bits(b[u].y), mn1, mx1);
            }
        }
        for (; i < n2; i += stride) {
            const double2 a = X2[i], b = Y2[i];
            minmax_ord(ord_bits(a.x), mn0, mx0);
            minmax_ord(ord_bits(a.y), mn0, mx0);
            minmax_ord(ord_bits(b.x), mn1, mx1);
            minmax_ord(ord_bits(b.y), mn1, mx1);
        }
        if ((d.n_total & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
            minmax_ord(ord_bits(X[d.n_total - 1]), mn0, mx0);
            minmax_ord(ord_bits(Y[d.n_total - 1]), mn1, mx1);
        }
        bbox_block_commit(d, 0, mn0, mn1, mx0, mx1, red);
    }
    const long long tile = (long long)TPB * 16;
    for (long long t0 = (long long)blockIdx.x * tile; d.nsys > 1 && t0 < d.n_total; t0 += (long long)gridDim.x * tile) {
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
            bbox_block_commit(d, s_first, mn0, mn1, mx0, mx1, red);
        }
        __syncthreads();
    }
    // the last block to finish squares every system's box and tabulates the box origins
    __shared__ unsigned ticket;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) ticket = atomicAdd(&d.glob->bbox_done, 1u);
    __syncthreads();
    if (ticket != gridDim.x - 1) return;
    __threadfence();
    if (threadIdx.x == 0) {
        for (int s = 0; s < d.nsys; s++)
            if (d.sys[s].n > 0) bbox_finalize_sys(d, s);
        d.glob->bbox_done = 0u;
    }
    __syncthreads();
    for (int s = 0; s < d.nsys; s++) {
        if (d.sys[s].n == 0) continue;
        const SysDyn &dy = d.dyn[s];
        const int G = d.sys[s].G;
        double *org = d.org + d.sys[s].ooff;
        for (int k = threadIdx.x; k < G; k += blockDim.x) {
            org[k] = box_origin(dy.minx, k, dy.step);
            org[G + k] = box_origin(dy.miny, k, dy.step);
        }
    }
}

// -------------------------------------------------------------------- place
// Box keys bit-exact with the reference's FP64 keys (computed at twice the box resolution, so
// each particle also gets its quadrant within the box), and a histogram of (box, quadrant)
// pairs aggregated over runs of equal keys in the block (a box's count is the sum of its
// four); a particle's slot is its rank within its quadrant.
constexpr int PLACE_PP = 4;  // consecutive particles per thread

// (64 registers: 4 CTAs per SM)
__global__ void __launch_bounds__(TPB, 4) k_place(DevPlan d) {
    constexpr int PT = TPB * PLACE_PP;  // particles per block round
    __shared__ int skeys[PT + 1], runold[PT], wmax[TPB / 32];
    const int cur = d.glob->epoch & 1;
    const double *X = d.X[cur], *Y = d.Y[cur];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int e0 = (int)threadIdx.x * PLACE_PP;  // the thread's first particle in the round
    for (long long base = (long long)blockIdx.x * PT; base < d.n_total; base += (long long)gridDim.x * PT) {
        const long long i0 = base + e0;
        double x[PLACE_PP], y[PLACE_PP];
        if (i0 + PLACE_PP <= d.n_total && (i0 & 1) == 0) {  // (always, but for a ragged end)
            const double2 *X2 = reinterpret_cast<const double2 *>(X + i0);
            const double2 *Y2 = reinterpret_cast<const double2 *>(Y + i0);
#pragma unroll
            for (int j = 0; j < PLACE_PP / 2; j++) {
                const double2 a = X2[j], b = Y2[j];
                x[2 * j] = a.x; x[2 * j + 1] = a.y;
                y[2 * j] = b.x; y[2 * j + 1] = b.y;
            }
        } else {
#pragma unroll
            for (int j = 0; j < PLACE_PP; j++) {
                x[j] = i0 + j < d.n_total ? X[i0 + j] : 0.0;
                y[j] = i0 + j < d.n_total ? Y[i0 + j] : 0.0;
            }
        }
        int key[PLACE_PP];
        // the thread's particles usually lie in one system: its constants are loaded once
        const int s_first = find_seg(d.poff_tab, d.nsys, i0 < d.n_total ? i0 : d.n_total - 1);
        const bool one_sys = d.poff_tab[s_first + 1] >= i0 + PLACE_PP;
        if (one_sys) {
            const SysDesc &sd = d.sys[s_first];
            const SysDyn &dy = d.dyn[s_first];
            const double mnx = dy.minx, mny = dy.miny, st = dy.step, inv = dy.inv_step;
            const float mnxf = dy.minx_f, mnyf = dy.miny_f, invf = dy.inv_step_f, tol = dy.key_tol;
            const int G = sd.G;
            const long long boff = sd.boff;
#pragma unroll
            for (int j = 0; j < PLACE_PP; j++) {
                const unsigned hx = (unsigned)(__double_as_longlong(x[j]) >> 52) & 0x7FFu;
                const unsigned hy = (unsigned)(__double_as_longlong(y[j]) >> 52) & 0x7FFu;
                if (hx == 0x7FFu || hy == 0x7FFu) raise_err(d.glob, 1u /*BH_DEV_NAN_POSITION*/);
                const int k2x = half_key1_f32(x[j], mnx, st, inv, mnxf, invf, tol, G);
                const int k2y = half_key1_f32(y[j], mny, st, inv, mnyf, invf, tol, G);
                const int box = (int)(boff + (long long)(k2x >> 1) * G + (k2y >> 1));
                key[j] = 4 * box + (k2x & 1) * 2 + (k2y & 1);
                skeys[e0 + j] = key[j];
            }
        } else
#pragma unroll
        for (int j = 0; j < PLACE_PP; j++) {
            const long long i = i0 + j;
            key[j] = -1;
            if (i < d.n_total) {
                const int s = find_seg(d.poff_tab, d.nsys, i);
                const SysDesc &sd = d.sys[s];
                const SysDyn &dy = d.dyn[s];
                // finite test on the exponent bits (no FP64 operation)
                const unsigned hx = (unsigned)(__double_as_longlong(x[j]) >> 52) & 0x7FFu;
                const unsigned hy = (unsigned)(__double_as_longlong(y[j]) >> 52) & 0x7FFu;
                if (hx == 0x7FFu || hy == 0x7FFu) raise_err(d.glob, 1u /*BH_DEV_NAN_POSITION*/);
                // keys at twice the box resolution: box key and quadrant within the box
                const int k2x = half_key1_f32(x[j], dy.minx, dy.step, dy.inv_step, dy.minx_f, dy.inv_step_f, dy.key_tol, sd.G);
                const int k2y = half_key1_f32(y[j], dy.miny, dy.step, dy.inv_step, dy.miny_f, dy.inv_step_f, dy.key_tol, sd.G);
                const int box = (int)(sd.boff + (long long)(k2x >> 1) * sd.G + (k2y >> 1));
                key[j] = 4 * box + (k2x & 1) * 2 + (k2y & 1);
            }
            skeys[e0 + j] = key[j];
        }
        if (threadIdx.x == 0) skeys[PT] = INT_MIN;
        // runs of consecutive particles of the round with the same (box, quadrant): the run's
        // last particle adds the run's length to the quadrant count, whose old value is the run's
        // first slot, so a quadrant whose particles lie in one round gets its slots in input
        // order (the common case when the input is the previous step's order); k_segsort puts
        // the runs of different blocks in order
        __syncthreads();
        int h[PLACE_PP];  // the first particle of each particle's run: a max-scan of run heads
        int hm = 0;
#pragma unroll
        for (int j = 0; j < PLACE_PP; j++) {
            const int e = e0 + j;
            const int kp = e > 0 ? skeys[e - 1] : INT_MIN;
            if (key[j] != kp) hm = e;
            h[j] = hm;
        }
        int hx = hm;  // inclusive max over the threads before and including this one
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) hx = max(hx, __shfl_up_sync(0xffffffffu, hx, o) * (lane >= o));
        if (lane == 31) wmax[warp] = hx;
        int hb = __shfl_up_sync(0xffffffffu, hx, 1) * (lane >= 1);  // exclusive, within the warp
        __syncthreads();
        for (int w = 0; w < warp; w++) hb = max(hb, wmax[w]);
#pragma unroll
        for (int j = 0; j < PLACE_PP; j++) {
            h[j] = max(h[j], hb);
            const int e = e0 + j;
            if (key[j] >= 0 && key[j] != skeys[e + 1]) runold[h[j]] = atomicAdd(&d.qcounts[key[j]], e - h[j] + 1);
        }
        __syncthreads();
        int kv[PLACE_PP], sv[PLACE_PP];
#pragma unroll
        for (int j = 0; j < PLACE_PP; j++) {
            kv[j] = key[j];  // 4 * box + quadrant
            sv[j] = key[j] >= 0 ? runold[h[j]] + (e0 + j - h[j]) : 0;
        }
        if (i0 + PLACE_PP <= d.n_total && (i0 & 3) == 0) {
            *reinterpret_cast<int4 *>(d.key + i0) = make_int4(kv[0], kv[1], kv[2], kv[3]);
            *reinterpret_cast<int4 *>(d.slot + i0) = make_int4(sv[0], sv[1], sv[2], sv[3]);
        } else {
#pragma unroll
            for (int j = 0; j < PLACE_PP; j++)
                if (i0 + j < d.n_total) {
                    d.key[i0 + j] = kv[j];
                    d.slot[i0 + j] = sv[j];
                }
        }
        __syncthreads();  // the block's shared arrays are reused in the next round
    }
}

// --------------------------------------------------------------------- scan
// Exclusive scans in one pass (decoupled look-back): tiles are numbered in the order their CTAs
// start (a ticket), so every tile's predecessors are already running; a tile publishes its sum,
// then its inclusive prefix once it has read its predecessors' (a predecessor's inclusive prefix
// ends the look-back).  A tile state is gen << 34 | flag << 32 | value (flag 1 = the tile's sum,
// 2 = inclusive prefix); a state of another generation is not yet written, and the scan's last
// tile bumps the generation, so the states need no clearing between scans.  Waits are bounded:
// on timeout the tile raises BH_DEV_WAIT_TIMEOUT and carries on (the result is then invalid).
constexpr unsigned long long SST_AGG = 1ull << 32, SST_PRE = 2ull << 32;
constexpr long long LOOKBACK_SPIN = 1ll << 22;

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

// Generations run 1 .. 2^30 - 1 (30 bits in a state); 0 never tags a state, so the zeroed
// states of a freshly bound plan read as not yet written.
__device__ __forceinline__ unsigned next_gen(unsigned g) { return g >= 0x3FFFFFFFu ? 1u : g + 1u; }

// Warp 0 of the CTA: publish the tile's sum `agg`, look back, publish the inclusive prefix and
// return the tile's exclusive prefix (to lane 0; the caller broadcasts through shared memory).
__device__ int lookback(unsigned long long *state, int tile, unsigned gen, int agg, Globals *glob) {
    const int lane = threadIdx.x & 31;
    volatile unsigned long long *vs = state;
    const unsigned long long tag = (unsigned long long)(gen & 0x3FFFFFFFu) << 34;
    if (tile == 0) {
        if (lane == 0) {
            __threadfence();
            vs[0] = tag | SST_PRE | (unsigned)agg;
        }
        return 0;
    }
    if (lane == 0) {
        __threadfence();
        vs[tile] = tag | SST_AGG | (unsigned)agg;
    }
    int excl = 0;
    int k = tile - 1;  // the nearest predecessor not yet read
    bool timed_out = false;
    while (k >= 0) {
        const int idx = k - lane;
        unsigned long long st = idx >= 0 ? 0ull : (tag | SST_PRE);  // before tile 0: prefix 0
        long long it = 0;
        for (;;) {
            if (idx >= 0) st = vs[idx];
            const bool ready = (st >> 34) == (tag >> 34) && (st & (3ull << 32)) != 0;
            if (__all_sync(0xffffffffu, ready)) break;
            if (++it > LOOKBACK_SPIN) {
                timed_out = true;
                break;
            }
        }
        if (timed_out) break;
        const unsigned pre_mask = __ballot_sync(0xffffffffu, (st & SST_PRE) == SST_PRE);
        const int stop = pre_mask ? __ffs(pre_mask) - 1 : 31;  // nearest inclusive prefix
        int v = lane <= stop ? (int)(unsigned)(st & 0xFFFFFFFFull) : 0;
#pragma unroll
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        excl += v;
        if (pre_mask) break;
        k -= 32;
    }
    if (lane == 0) {
        if (timed_out) raise_err(glob, 8u /*BH_DEV_WAIT_TIMEOUT*/);
        __threadfence();
        vs[tile] = tag | SST_PRE | (unsigned)(excl + agg);
    }
    return excl;
}

// out[i] = sum(in[0..i)) for i < n, out[n] = sum(in[0..n)); scan k of the plan's three.  QSUM:
// element i is the sum of the four quadrant counts in[4 i .. 4 i + 3] (a box's particles).
template <bool QSUM>
__global__ void __launch_bounds__(TPB) k_scan_lookback(const int *in, long long n, int *out,
                                                      unsigned long long *state, Globals *glob, int k) {
    __shared__ int sh[32];
    __shared__ int s_tile, s_excl;
    __shared__ unsigned s_gen;
    const long long ntiles = (n + SCAN_TILE - 1) / SCAN_TILE > 0 ? (n + SCAN_TILE - 1) / SCAN_TILE : 1;
    if (threadIdx.x == 0) {
        s_tile = (int)atomicAdd(&glob->scan_ticket[k], 1u);
        s_gen = *(volatile unsigned *)&glob->scan_gen[k];
    }
    __syncthreads();
    const int tile = s_tile;
    const long long b0 = (long long)tile * SCAN_TILE + (long long)threadIdx.x * 16;
    int v[16], sum = 0;
#pragma unroll
    for (int q = 0; q < 16; q++) {
        v[q] = 0;
        if (b0 + q < n) {
            if (QSUM) {
                const int4 c = reinterpret_cast<const int4 *>(in)[b0 + q];
                v[q] = c.x + c.y + c.z + c.w;
            } else {
                v[q] = in[b0 + q];
            }
        }
        sum += v[q];
    }
    int tot;
    int pre = block_excl_scan(sum, sh, &tot);
    if (threadIdx.x < 32) {
        const int e = lookback(state, tile, s_gen, tot, glob);
        if (threadIdx.x == 0) s_excl = e;
    }
    __syncthreads();
    pre += s_excl;
#pragma unroll
    for (int q = 0; q < 16; q++) {
        if (b0 + q < n) out[b0 + q] = pre;
        pre += v[q];
    }
    if (tile == ntiles - 1 && threadIdx.x == 0) {
        out[n] = s_excl + tot;
        glob->scan_ticket[k] = 0u;  // every tile has its ticket: ready for the next scan
        glob->scan_gen[k] = next_gen(s_gen);
    }
}

static cudaError_t scan_excl(const int *in, int *out, long long n, unsigned long long *state,
                             Globals *glob, int k, cudaStream_t st, bool qsum = false) {
    long long ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (ntiles < 1) ntiles = 1;
    if (qsum)
        k_scan_lookback<true><<<(unsigned)ntiles, TPB, 0, st>>>(in, n, out, state, glob, k);
    else
        k_scan_lookback<false><<<(unsigned)ntiles, TPB, 0, st>>>(in, n, out, state, glob, k);
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
// items: full chunks of STREAM_CHUNK and the remainder's pieces (sitem_range).  A group's items
// are the sparse ones, then the boxes' in (cx, cy) order, quadrant by quadrant.  One kernel: a
// warp per group (a lane per box) counts the group's items, the CTA scans its SITEM_TILE groups,
// a look-back over the preceding tiles gives their offset, and the lanes write their boxes'
// items.
constexpr int SITEM_WARPS = SITEM_TILE;  // one group per warp
static_assert(MAX_TG * MAX_TG <= 64, "a lane holds at most two boxes of a group");

__global__ void __launch_bounds__(SITEM_WARPS * 32) k_sitems(DevPlan d) {
    __shared__ int wtot[SITEM_WARPS], wpre[SITEM_WARPS];
    __shared__ int s_tile, s_excl;
    __shared__ unsigned s_gen;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long ntiles = (d.NG_total + SITEM_TILE - 1) / SITEM_TILE;
    if (threadIdx.x == 0) {
        s_tile = (int)atomicAdd(&d.glob->scan_ticket[2], 1u);
        s_gen = *(volatile unsigned *)&d.glob->scan_gen[2];
    }
    __syncthreads();
    const int tile = s_tile;
    const long long g = (long long)tile * SITEM_TILE + warp;
    // the lane's boxes bi = lane, lane + 32 of the group (bi = cx * TG + cy)
    int nb[2] = {0, 0}, kind[2] = {0, 0}, cnt[2] = {0, 0};
    int4 qc[2] = {make_int4(0, 0, 0, 0), make_int4(0, 0, 0, 0)};
    int sparse = 0, nbox = 0;
    if (g < d.NG_total) {
        const int s = find_seg(d.goff_tab, d.nsys, g);
        const SysDesc &sd = d.sys[s];
        const long long lg = g - sd.goff;
        const int gi = (int)(lg / sd.NGs), gj = (int)(lg - (long long)gi * sd.NGs);
        const int TG = sd.TG, tgs = __ffs(TG) - 1;
        nbox = TG * TG;
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const int bi = lane + 32 * u;
            const int cx = bi >> tgs, cy = bi & (TG - 1);
            if (bi < nbox && gi * TG + cx < sd.G && gj * TG + cy < sd.G) {
                const long long b = sd.boff + (long long)(gi * TG + cx) * sd.G + gj * TG + cy;
                nb[u] = d.box_start[b + 1] - d.box_start[b];
                kind[u] = box_item_kind(nb[u], d.dense_min, d.quad_min);
                if (kind[u] == 2) {
                    qc[u] = reinterpret_cast<const int4 *>(d.qcounts)[b];
                    cnt[u] = sitem_count(qc[u].x) + sitem_count(qc[u].y) + sitem_count(qc[u].z) + sitem_count(qc[u].w);
                } else if (kind[u] == 1) {
                    cnt[u] = sitem_count(nb[u]);
                } else {
                    sparse += nb[u];
                }
            }
        }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) sparse += __shfl_xor_sync(0xffffffffu, sparse, o);
    const int ns = sitem_count(sparse);
    // exclusive prefix of the boxes' item counts in bi order (lane's first box, then second)
    int inc0 = cnt[0], inc1 = cnt[1];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y0 = __shfl_up_sync(0xffffffffu, inc0, o), y1 = __shfl_up_sync(0xffffffffu, inc1, o);
        if (lane >= o) {
            inc0 += y0;
            inc1 += y1;
        }
    }
    const int tot0 = __shfl_sync(0xffffffffu, inc0, 31), tot1 = __shfl_sync(0xffffffffu, inc1, 31);
    const int gtot = g < d.NG_total ? ns + tot0 + tot1 : 0;
    if (lane == 0) wtot[warp] = gtot;
    __syncthreads();
    if (threadIdx.x < 32) {
        int v = lane < SITEM_WARPS ? wtot[lane] : 0, x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane < SITEM_WARPS) wpre[lane] = x - v;
        const int tot = __shfl_sync(0xffffffffu, x, 31);
        const int e = lookback(d.sst_sitem, tile, s_gen, tot, d.glob);
        if (threadIdx.x == 0) {
            s_excl = e;
            if (tile == ntiles - 1) {
                d.sitem_off[d.NG_total] = e + tot;
                d.glob->scan_ticket[2] = 0u;
                d.glob->scan_gen[2] = next_gen(s_gen);
            }
        }
    }
    __syncthreads();
    if (g >= d.NG_total) return;
    const int off = s_excl + wpre[warp];
    if (lane == 0) d.sitem_off[g] = off;
    for (int k = lane; k < ns; k += 32) {  // the sparse boxes' items
        d.sitem_group[off + k] = (int)g;
        d.sitem_sub[off + k] = -1;
        d.sitem_chunk[off + k] = make_int2(k, ns);
    }
#pragma unroll
    for (int u = 0; u < 2; u++) {
        const int bi = lane + 32 * u;
        int o = off + ns + (u ? tot0 : 0) + (u ? inc1 : inc0) - cnt[u];
        if (kind[u] == 1) {
            const int nk = cnt[u];
            for (int k = 0; k < nk; k++, o++) {
                d.sitem_group[o] = (int)g;
                d.sitem_sub[o] = bi;
                d.sitem_chunk[o] = make_int2(k, nk);
            }
        } else if (kind[u] == 2) {
            const int qv[4] = {qc[u].x, qc[u].y, qc[u].z, qc[u].w};
            for (int q = 0; q < 4; q++) {
                const int nk = sitem_count(qv[q]);
                for (int k = 0; k < nk; k++, o++) {
                    d.sitem_group[o] = (int)g;
                    d.sitem_sub[o] = nbox + 4 * bi + q;
                    d.sitem_chunk[o] = make_int2(k, nk);
                }
            }
        }
    }
}

// ------------------------------------------------------------------ scatter
// Counting sort into box order, each box's particles quadrant by quadrant, and within a quadrant
// in input order (the order the previous step left, or the caller's), so the step does not depend
// on the order in which k_place's atomics handed out slots:
//   k_perm     perm[box_start + earlier quadrants + slot] = input index (slots: k_place);
//   k_segsort  each quadrant's stretch of perm sorted ascending -- up to SEG_REG entries in a
//              thread's registers, longer ones listed for k_segsort_big (up to SEG_WARP entries
//              a warp each, a bitonic network in its slice of shared memory; longer ones a CTA
//              each, four stable 8-bit radix passes through the dead slot array);
//   k_gather   output particle t takes input perm[t]: the FP64 state of the next buffer, the
//              32-byte packed record (offsets from the box origin computed in FP64, rounded
//              once to float) and the sorted key; and it sums the leaves (below).
constexpr int SEG_REG = 16;
constexpr int SEG_WARP = 1024;
constexpr int SEG_CHECK = 128;  // stretches up to this long are checked for order by their thread

__device__ __forceinline__ int quad_first(const DevPlan &d, int key4) {
    const int box = key4 >> 2, quad = key4 & 3;
    const int4 qc = reinterpret_cast<const int4 *>(d.qcounts)[box];
    return d.box_start[box] + (quad > 0 ? qc.x : 0) + (quad > 1 ? qc.y : 0) + (quad > 2 ? qc.z : 0);
}

__global__ void __launch_bounds__(TPB) k_perm(DevPlan d) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < d.n_total; i += stride)
        d.perm[quad_first(d, d.key[i]) + d.slot[i]] = (int)i;
}

__global__ void __launch_bounds__(TPB) k_segsort(DevPlan d) {
    const long long nq = 4 * d.B_total, stride = (long long)gridDim.x * blockDim.x;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += stride) {
        const int n = d.qcounts[q];
        if (n < 2) continue;
        const int s0 = quad_first(d, (int)q);
        if (n > SEG_REG && n <= SEG_CHECK) {  // listed only when out of order
            bool sorted = true;
            int prev = d.perm[s0];
            for (int k0 = 1; k0 < n && sorted; k0 += 8) {
                int v[8];
#pragma unroll
                for (int k = 0; k < 8; k++) v[k] = k0 + k < n ? d.perm[s0 + k0 + k] : 0x7FFFFFFF;
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    sorted &= prev < v[k] || k0 + k >= n;
                    prev = v[k];
                }
            }
            if (sorted) continue;
        }
        if (n > SEG_WARP) {  // listed from the far end of the same array
            const unsigned k = atomicAdd(&d.glob->nhuge, 1u);
            d.bigseg[d.bigseg_cap - 1 - k] = make_int2(s0, n);
            continue;
        }
        if (n > SEG_REG) {
            const unsigned k = atomicAdd(&d.glob->nbig, 1u);
            d.bigseg[k] = make_int2(s0, n);
            continue;
        }
        int v[SEG_REG];
#pragma unroll
        for (int k = 0; k < SEG_REG; k++) v[k] = k < n ? d.perm[s0 + k] : 0x7FFFFFFF;
        bool sorted = true;  // (padding sorts after every index)
#pragma unroll
        for (int k = 0; k + 1 < SEG_REG; k++) sorted &= v[k] <= v[k + 1];
        if (sorted) continue;
        // odd-even transposition network: SEG_REG rounds sort SEG_REG entries
#pragma unroll
        for (int r = 0; r < SEG_REG; r++)
#pragma unroll
            for (int k = r & 1; k + 1 < SEG_REG; k += 2) {
                const int lo = min(v[k], v[k + 1]), hi = max(v[k], v[k + 1]);
                v[k] = lo;
                v[k + 1] = hi;
            }
#pragma unroll
        for (int k = 0; k < SEG_REG; k++)
            if (k < n) d.perm[s0 + k] = v[k];
    }
}

__global__ void __launch_bounds__(TPB) k_segsort_big(DevPlan d) {
    __shared__ int sv[TPB / 32][SEG_WARP];
    __shared__ int hist[256], base[256], run[256], wcnt[TPB / 32][256];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // stretches of SEG_REG + 1 .. SEG_WARP entries: a warp each, a bitonic network over the next
    // power of two (padded with INT_MAX) in the warp's slice of shared memory
    const unsigned nbig = d.glob->nbig;
    int *w = sv[warp];
    for (unsigned e = (unsigned)(blockIdx.x * (TPB / 32) + warp); e < nbig; e += gridDim.x * (TPB / 32)) {
        const int2 sg = d.bigseg[e];
        const int s0 = sg.x, n = sg.y;
        int m = 32;
        while (m < n) m <<= 1;
        // a stretch whose slots the atomics happened to hand out in input order is done already
        // (the common case when the input is the previous step's order)
        bool sorted = true;
        for (int k = lane; k < m; k += 32) {
            const int v = k < n ? d.perm[s0 + k] : 0x7FFFFFFF;
            w[k] = v;
        }
        __syncwarp();
        for (int k = lane; k + 1 < n; k += 32) sorted &= w[k] < w[k + 1];
        if (__all_sync(0xffffffffu, sorted)) {
            __syncwarp();
            continue;
        }
        for (int size = 2; size <= m; size <<= 1)
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                for (int k = lane; k < m; k += 32) {
                    const int j = k ^ stride;
                    if (j > k) {
                        const bool up = (k & size) == 0;
                        const int x = w[k], y = w[j];
                        if ((x > y) == up) {
                            w[k] = y;
                            w[j] = x;
                        }
                    }
                }
                __syncwarp();
            }
        for (int k = lane; k < n; k += 32) d.perm[s0 + k] = w[k];
        __syncwarp();
    }
    // longer stretches: a CTA each, four stable 8-bit radix passes perm -> slot -> perm -> slot
    // -> perm (the slot array is dead once k_perm has run)
    const unsigned nhuge = d.glob->nhuge;
    for (unsigned b = blockIdx.x; b < nhuge; b += gridDim.x) {
        const int2 sg = d.bigseg[d.bigseg_cap - 1 - b];
        const int s0 = sg.x, n = sg.y;
        int *src = d.perm + s0, *dst = d.slot + s0;
        for (int pass = 0; pass < 4; pass++) {
            const int sh = 8 * pass;
            for (int k = tid; k < 256; k += TPB) {
                hist[k] = 0;
                run[k] = 0;
            }
            __syncthreads();
            for (int k = tid; k < n; k += TPB) atomicAdd(&hist[(src[k] >> sh) & 255], 1);
            __syncthreads();
            if (tid == 0) {
                int acc = 0;
                for (int k = 0; k < 256; k++) {
                    base[k] = acc;
                    acc += hist[k];
                }
            }
            __syncthreads();
            for (int c0 = 0; c0 < n; c0 += TPB) {
                const int k = c0 + tid;
                const bool ok = k < n;
                const int v = ok ? src[k] : 0;
                const int dg = ok ? (v >> sh) & 255 : 256 + lane;  // invalid lanes match nobody
                for (int q = tid; q < (TPB / 32) * 256; q += TPB) (&wcnt[0][0])[q] = 0;
                __syncthreads();
                const unsigned peers = __match_any_sync(0xffffffffu, dg);
                const int rank = __popc(peers & ((1u << lane) - 1u));
                if (ok && rank == 0) wcnt[warp][dg] = __popc(peers);
                __syncthreads();
                if (ok) {
                    int pos = base[dg] + run[dg] + rank;
                    for (int q = 0; q < warp; q++) pos += wcnt[q][dg];
                    dst[pos] = v;
                }
                __syncthreads();
                for (int q = tid; q < 256; q += TPB) {
                    int t = 0;
                    for (int ww = 0; ww < TPB / 32; ww++) t += wcnt[ww][q];
                    run[q] += t;
                }
                __syncthreads();
            }
            int *t = src;
            src = dst;
            dst = t;
            __threadfence_block();
            __syncthreads();
        }
    }
}

// The leaf-moment terms of one particle (offsets from its box origin, mass), the segmented scan
// of a warp's chunk of 32 box-sorted particles and the write of its sums: the box inside the
// chunk gets its FP64 moments in mom, a box that starts before the chunk leaves its part in the
// chunk's head partial, one that runs past it in the tail partial (k_summarize adds a multi-chunk
// box's partials in chunk order).  The products are rounded one by one (no contraction), so the
// fused pass in k_gather and the stand-alone k_leaf give the same sums.  The second moments
// (Sxx, Sxy, Syy) are summed only with SECOND (a plan with the learned correction, or training
// pairs on demand); otherwise they are zeros.
template <bool SECOND>
__device__ __forceinline__ void leaf_terms(float ox, float oy, float mf, float v[6]) {
    v[0] = mf;
    v[1] = __fmul_rn(mf, ox);
    v[2] = __fmul_rn(mf, oy);
    v[3] = SECOND ? __fmul_rn(v[1], ox) : 0.f;
    v[4] = SECOND ? __fmul_rn(v[1], oy) : 0.f;
    v[5] = SECOND ? __fmul_rn(v[2], oy) : 0.f;
}

// key: the lane's box (-1 past the end); c: the chunk (its first particle is 32 c)
template <bool SECOND>
__device__ __forceinline__ void leaf_chunk(const DevPlan &d, long long c, int key, float v[6]) {
    constexpr int NL = SECOND ? 6 : 3;  // moments summed
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int k2 = __shfl_up_sync(0xffffffffu, key, o);
#pragma unroll
        for (int q = 0; q < NL; q++) {
            const float y = __shfl_up_sync(0xffffffffu, v[q], o);
            if (lane >= o && k2 == key) v[q] = __fadd_rn(v[q], y);
        }
    }
    const int knext = __shfl_down_sync(0xffffffffu, key, 1);
    const int kfirst = __shfl_sync(0xffffffffu, key, 0);
    const bool last = key >= 0 && (lane == 31 || knext != key);  // the segment's last lane
    if (!last) return;
    const long long i0 = c << 5;
    const bool head = key == kfirst && d.box_start[key] < i0;              // began in an earlier chunk
    const bool tail = lane == 31 && d.box_start[key + 1] > i0 + 32;        // goes on in a later chunk
    if (head || tail) {
        float *pt = d.leafpart + 12 * c;
        if (head)
#pragma unroll
            for (int q = 0; q < NL; q++) pt[q] = v[q];
        if (tail)
#pragma unroll
            for (int q = 0; q < NL; q++) pt[6 + q] = v[q];
    } else {
        const int s = find_seg(d.boff_tab, d.nsys, key);
        double *m = d.mom + 6 * (d.sys[s].coff + (key - d.sys[s].boff));
#pragma unroll
        for (int q = 0; q < 6; q++) m[q] = q < NL ? f32_to_f64(v[q]) : 0.0;
    }
}

// Output particle t takes input perm[t]; each warp's 32 consecutive outputs form a leaf chunk,
// whose moments are summed on the spot (the stand-alone k_leaf repeats this from the packed
// records when the leaf moments were overwritten since).
template <bool SECOND>
__global__ void __launch_bounds__(TPB) k_gather(DevPlan d) {
    const int cur = d.glob->epoch & 1, nxt = cur ^ 1;
    const int lane = threadIdx.x & 31;
    // SU particles per thread per round, each stage's loads issued for all of them before the
    // next stage uses them; the loop runs per warp (its first lane's index), for the scans.
    // Two per round keep the kernel at 58 registers, 4 CTAs per SM (four: 93, 2 CTAs, 9% slower)
    constexpr int SU = 2;
    const long long n = d.n_total, stride = (long long)gridDim.x * blockDim.x;
    // one system (the common case): its grid constants once, no search per particle
    const bool one = d.nsys == 1;
    const int G0 = d.sys[0].G;
    const long long boff0 = d.sys[0].boff, ooff0 = d.sys[0].ooff;
    for (long long w0 = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); w0 < n; w0 += SU * stride) {
        const long long t0 = w0 + lane;
        int src[SU], key4[SU];
#pragma unroll
        for (int u = 0; u < SU; u++) {
            const long long t = t0 + u * stride;
            src[u] = t < n ? d.perm[t] : 0;
        }
#pragma unroll
        for (int u = 0; u < SU; u++) {
            const long long t = t0 + u * stride;
            key4[u] = t < n ? d.key[src[u]] : 0;
        }
        double x[SU], y[SU], m[SU], vx[SU], vy[SU];
        int pid[SU];
#pragma unroll
        for (int u = 0; u < SU; u++) {
            const long long t = t0 + u * stride;
            if (t < n) {
                const int i = src[u];
                x[u] = d.X[cur][i];
                y[u] = d.Y[cur][i];
                m[u] = d.M[cur][i];
                vx[u] = d.VX[cur][i];
                vy[u] = d.VY[cur][i];
                pid[u] = d.PID[cur][i];
            }
        }
        float lx[SU], ly[SU], lm[SU];
#pragma unroll
        for (int u = 0; u < SU; u++) {
            const long long t = t0 + u * stride;
            lx[u] = ly[u] = lm[u] = 0.f;
            if (t >= n) continue;
            const int key = key4[u] >> 2;
            const int s = one ? 0 : find_seg(d.boff_tab, d.nsys, key);
            const int G = one ? G0 : d.sys[s].G;
            const long long boff = one ? boff0 : d.sys[s].boff, ooff = one ? ooff0 : d.sys[s].ooff;
            const int lb = (int)(key - boff);
            const int kx = lb / G, ky = lb - kx * G;
            d.X[nxt][t] = x[u];
            d.Y[nxt][t] = y[u];
            d.VX[nxt][t] = vx[u];
            d.VY[nxt][t] = vy[u];
            d.M[nxt][t] = m[u];
            d.PID[nxt][t] = pid[u];
            const double *org = d.org + ooff;  // box origins (tabulated by k_bbox's last block)
            const float ox = f64_to_f32_rn(__dsub_rn(x[u], org[kx]));
            const float oy = f64_to_f32_rn(__dsub_rn(y[u], org[G + ky]));
            const float mf = f64_to_f32_rn(m[u]);
            d.PD[2 * t] = make_float4(ox, ox, oy, oy);
            d.PD[2 * t + 1] = make_float4(mf, mf, __int_as_float((int)t), __int_as_float((kx << 16) | ky));
            d.skey[t] = key;
            lx[u] = ox;
            ly[u] = oy;
            lm[u] = mf;
        }
#pragma unroll
        for (int u = 0; u < SU; u++) {
            const long long wu = w0 + u * stride;  // the chunk's first particle
            if (wu >= n) break;                    // (warp-uniform)
            const long long t = wu + lane;
            float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            if (t < n) leaf_terms<SECOND>(lx[u], ly[u], lm[u], v);
            leaf_chunk<SECOND>(d, wu >> 5, t < n ? key4[u] >> 2 : -1, v);
        }
    }
}

// ---------------------------------------------------------------- summarize
// One CTA per tile of SUM_TILE x SUM_TILE leaf boxes: the boxes' moments (M, Sx, Sy, Sxx, Sxy,
// Syy about the box origin; k_gather summed them per chunk of 32 box-sorted particles), then
// pyramid levels 1..4 inside the tile, then the cell records of all of them.  Above the tiles
// (cells of 2^5 boxes and larger) a cell is built by the CTA that finishes its last child: each
// cell counts its children's arrivals, so the levels above rise along a reduction tree instead of
// waiting for one CTA.  Every sum runs in a fixed order, so the moments do not depend on
// scheduling.  Pyramid cells carry the second moments only for the learned correction (SECOND);
// the leaves always carry all six.
constexpr int SUM_THREADS = 128;  // 7 CTAs per SM: the 1,024 tiles of G = 512 in one wave
constexpr int SUM_CELLS = 256 + 64 + 16 + 4 + 1;  // a tile's cells at levels 0..4
constexpr int SUM_UP = 5;                         // the first level above the tiles (2^5 boxes)
static_assert(SUM_TILE == 1 << (SUM_UP - 1), "a tile is one cell of level SUM_UP - 1");

// The moments of child (a, b) of a level-l cell (q, FP64 about the child's origin) shifted to the
// cell origin, into o[6] (o[0..2] without SECOND); zeros when the child lies outside the grid.
template <bool SECOND>
__device__ __forceinline__ void child_terms(const double *q, bool has, int a, int b, int l, double step,
                                            double *o) {
    if (!has) {
#pragma unroll
        for (int k = 0; k < 6; k++) o[k] = 0.0;
        return;
    }
    const double dx = (double)(a << (l - 1)) * step, dy = (double)(b << (l - 1)) * step;
    const double M = q[0], Sx = q[1], Sy = q[2];
    o[0] = M;
    o[1] = Sx + M * dx;
    o[2] = Sy + M * dy;
    if (SECOND) {
        o[3] = q[3] + 2.0 * dx * Sx + M * dx * dx;
        o[4] = q[4] + dx * Sy + dy * Sx + M * dx * dy;
        o[5] = q[5] + 2.0 * dy * Sy + M * dy * dy;
    }
}

// a cell's four shifted children added in (0, 0), (0, 1), (1, 0), (1, 1) order
template <bool SECOND>
__device__ __forceinline__ void sum_children(const double *t, double *p) {
#pragma unroll
    for (int k = 0; k < (SECOND ? 6 : 3); k++) p[k] = ((t[k] + t[6 + k]) + t[12 + k]) + t[18 + k];
}

// Float records of cell c (level l): centre of mass relative to the cell origin and mass; with
// SECOND, the second moments about the centre of mass normalised by M s^2.
template <bool SECOND>
__device__ __forceinline__ void cell_record(const DevPlan &d, long long c, int l, double step,
                                            const double *q) {
    const double M = q[0];
    if (M > 0.0) {
        const double cx = q[1] / M, cy = q[2] / M;
        d.rec[c] = make_float4(f64_to_f32_rn(cx), f64_to_f32_rn(cy), f64_to_f32_rn(M), 0.f);
        if (SECOND) {
            const double sz = (double)(1 << l) * step;
            const double nrm = 1.0 / (M * sz * sz);
            const double ixx = q[3] - q[1] * cx, ixy = q[4] - q[1] * cy, iyy = q[5] - q[2] * cy;
            d.rec2[c] = make_float4(f64_to_f32_rn(ixx * nrm), f64_to_f32_rn(ixy * nrm),
                                    f64_to_f32_rn(iyy * nrm), 0.f);
        }
    } else {
        d.rec[c] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (SECOND) d.rec2[c] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

// Leaf moments from the packed records, balanced over the particles: a warp per chunk of 32
// box-sorted particles (k_gather does the same while it writes the records; this pass runs when
// the leaf moments have been overwritten since, bh_set_leaf_moments).  No atomics: fixed
// summation order.
template <bool SECOND>
__global__ void __launch_bounds__(TPB) k_leaf(DevPlan d) {
    const int lane = threadIdx.x & 31;
    const long long nch = (d.n_total + 31) >> 5;
    for (long long c = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < nch;
         c += ((long long)gridDim.x * blockDim.x) >> 5) {
        const long long i = (c << 5) + lane;
        int key = -1;
        float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (i < d.n_total) {
            key = d.skey[i];
            const float4 pxy = d.PD[2 * i], pm = d.PD[2 * i + 1];  // (x, x, y, y), (m, m, ., .)
            leaf_terms<SECOND>(pxy.x, pxy.z, pm.x, v);
        }
        leaf_chunk<SECOND>(d, c, key, v);
    }
}

// (s, c) += x, Kahan-compensated in FP32
__device__ __forceinline__ void kahan_add(float &s, float &c, float x) {
    const float y = __fsub_rn(x, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
}

// leaves_given: the leaf moments are already in d.mom (bh_set_leaf_moments); build the rest.
template <bool SECOND>
__global__ void __launch_bounds__(SUM_THREADS, 7) k_summarize(DevPlan d, int leaves_given) {
    constexpr int NM = SECOND ? 6 : 3;  // moments a pyramid cell carries
    __shared__ double cm[SUM_CELLS * 6];  // the tile's cells, level by level
    __shared__ double chm[4 * 64 * 6];    // shifted child moments: 64 cells x 4 children
    const int tid = threadIdx.x;
    const int loff[5] = {0, 256, 320, 336, 340};
    for (long long t = blockIdx.x; t < d.T_total; t += gridDim.x) {
        const int s = find_seg(d.toff_tab, d.nsys, t);
        const SysDesc &sd = d.sys[s];
        const double step = d.dyn[s].step;
        const int G = sd.G, lt = (int)(t - sd.toff), ti = lt / sd.tps, tj = lt - ti * sd.tps;
        const int bx0 = ti * SUM_TILE, by0 = tj * SUM_TILE;
        const int nbx = min(SUM_TILE, G - bx0), nby = min(SUM_TILE, G - by0);
        const int lmax = min(SUM_UP - 1, sd.L - 1);  // the tile's top level
        // ---- level 0: the tile's boxes (zeros outside the grid)
        for (int k = tid; k < 6 * SUM_TILE * SUM_TILE; k += SUM_THREADS) {
            const int box = k / 6, cx = box / SUM_TILE, cy = box - cx * SUM_TILE;
            double v = 0.0;
            if (leaves_given && cx < nbx && cy < nby)
                v = d.mom[6 * (sd.coff + (long long)(bx0 + cx) * G + (by0 + cy)) + (k - 6 * box)];
            cm[k] = v;
        }
        __syncthreads();
        if (!leaves_given) {
            // a box inside one chunk has its moments from the chunk's sums; a box over several
            // chunks adds its partials in chunk order (the first chunk's tail, whole middle
            // chunks, the last chunk's head) and writes the sum to mom, as an empty box its zeros
            for (int k = tid; k < SUM_TILE * SUM_TILE; k += SUM_THREADS) {
                const int cx = k / SUM_TILE, cy = k - cx * SUM_TILE;
                if (cx >= nbx || cy >= nby) continue;
                const long long lb = (long long)(bx0 + cx) * G + (by0 + cy);
                const int i0 = d.box_start[sd.boff + lb], i1 = d.box_start[sd.boff + lb + 1];
                double *mb = d.mom + 6 * (sd.coff + lb);
                if (i1 == i0) {  // empty: zeros
#pragma unroll
                    for (int q = 0; q < 6; q++) mb[q] = 0.0;
                    continue;
                }
                const long long c0 = i0 >> 5, c1 = (long long)(i1 - 1) >> 5;
                if (c0 == c1) {
#pragma unroll
                    for (int q = 0; q < 6; q++) cm[6 * k + q] = mb[q];
                    continue;
                }
                float sm_[6], cc_[6];
#pragma unroll
                for (int q = 0; q < 6; q++) {
                    sm_[q] = q < NM ? d.leafpart[12 * c0 + 6 + q] : 0.f;
                    cc_[q] = 0.f;
                }
                for (long long c = c0 + 1; c <= c1; c++)
#pragma unroll
                    for (int q = 0; q < NM; q++) kahan_add(sm_[q], cc_[q], d.leafpart[12 * c + q]);
#pragma unroll
                for (int q = 0; q < 6; q++) {
                    const double v = f32_to_f64(__fsub_rn(sm_[q], cc_[q]));
                    cm[6 * k + q] = v;
                    mb[q] = v;
                }
            }
            __syncthreads();
        }
        // ---- levels 1..lmax inside the tile: a thread per (cell, child) shifts the child's
        // moments to the cell origin, then a thread per cell adds its four children in order
        for (int l = 1; l <= lmax; l++) {
            const int nl = SUM_TILE >> l, nc = nl << 1;  // cells per side at l and l - 1
            const int gl = sd.lvg[l], gc = sd.lvg[l - 1];
            const int I0 = bx0 >> l, J0 = by0 >> l;
            for (int t = tid; t < 4 * nl * nl; t += SUM_THREADS) {
                const int cell = t >> 2, a = (t >> 1) & 1, b = t & 1;
                const int ci = cell / nl, cj = cell - ci * nl;
                const bool has = 2 * (I0 + ci) + a < gc && 2 * (J0 + cj) + b < gc;
                child_terms<SECOND>(cm + 6 * (loff[l - 1] + (2 * ci + a) * nc + (2 * cj + b)), has, a, b,
                                    l, step, chm + 6 * t);
            }
            __syncthreads();
            for (int c = tid; c < nl * nl; c += SUM_THREADS) {
                const int ci = c / nl, cj = c - ci * nl;
                const bool inside = I0 + ci < gl && J0 + cj < gl;
                double p[6];
                sum_children<SECOND>(chm + 24 * c, p);
#pragma unroll
                for (int k = 0; k < NM; k++) cm[6 * (loff[l] + c) + k] = inside ? p[k] : 0.0;
                if (inside) {
                    const long long cc = sd.coff + sd.lvoff[l] + (long long)(I0 + ci) * gl + (J0 + cj);
#pragma unroll
                    for (int k = 0; k < NM; k++) d.mom[6 * cc + k] = p[k];
                    cell_record<SECOND>(d, cc, l, step, p);
                }
            }
            __syncthreads();
        }
        // ---- records of the tile's boxes
        for (int k = tid; k < SUM_TILE * SUM_TILE; k += SUM_THREADS) {
            const int cx = k / SUM_TILE, cy = k - cx * SUM_TILE;
            if (cx >= nbx || cy >= nby) continue;
            cell_record<SECOND>(d, sd.coff + (long long)(bx0 + cx) * G + (by0 + cy), 0, step, cm + 6 * k);
        }
        // ---- above the tiles: the tile's top cell arrives at its parent; the CTA whose child
        // arrives last builds the parent (children in (0, 0), (0, 1), (1, 0), (1, 1) order, the
        // order of sum_children) and arrives at the next level
        if (sd.L > SUM_UP) {
            __threadfence();
            __syncthreads();
            if (tid == 0) {
                int I = ti, J = tj;
                for (int l = SUM_UP; l < sd.L; l++) {
                    I >>= 1;
                    J >>= 1;
                    const int gl = sd.lvg[l], gc = sd.lvg[l - 1];
                    const int nch = (2 * I + 1 < gc ? 2 : 1) * (2 * J + 1 < gc ? 2 : 1);
                    const long long cl = sd.lvoff[l] + (long long)I * gl + J;  // relative to coff
                    unsigned *cnt = d.upcnt + sd.upoff + (cl - sd.lvoff[SUM_UP]);
                    if (atomicAdd(cnt, 1u) != (unsigned)nch - 1u) break;
                    __threadfence();
                    *cnt = 0u;  // ready for the next step
                    double p[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
                    for (int a = 0; a < 2; a++)
                        for (int b = 0; b < 2; b++) {
                            const bool has = 2 * I + a < gc && 2 * J + b < gc;
                            double q[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, o[6];
                            if (has) {
                                const double *src =
                                    d.mom + 6 * (sd.coff + sd.lvoff[l - 1] + (long long)(2 * I + a) * gc + (2 * J + b));
#pragma unroll
                                for (int k = 0; k < NM; k++) q[k] = __ldcg(src + k);
                            }
                            child_terms<SECOND>(q, has, a, b, l, step, o);
#pragma unroll
                            for (int k = 0; k < NM; k++) p[k] = (a | b) ? p[k] + o[k] : o[k];
                        }
                    const long long cc = sd.coff + cl;
#pragma unroll
                    for (int k = 0; k < NM; k++) d.mom[6 * cc + k] = p[k];
                    cell_record<SECOND>(d, cc, l, step, p);
                    __threadfence();
                }
            }
        }
        __syncthreads();
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
    k_bbox<<<d.nsys == 1 ? (unsigned)(d.nsm * 4) : grid_for(d.n_total, TPB * 16, d.nsm * 8LL), TPB, 0, st>>>(d);
    return cudaGetLastError();
}
cudaError_t launch_place(const DevPlan &d, cudaStream_t st) {
    if (d.n_total == 0) return cudaSuccess;
    k_place<<<grid_for(d.n_total, TPB * PLACE_PP, d.nsm * 8LL), TPB, 0, st>>>(d);
    return cudaGetLastError();
}
cudaError_t launch_scan(const DevPlan &d, cudaStream_t st) {
    return scan_excl(d.qcounts, d.box_start, d.B_total, d.sst_box, d.glob, 0, st, true);
}
// Work items of the walk kernel and of the learned correction (group, target chunk).
cudaError_t launch_walk_items(const DevPlan &d, cudaStream_t st) {
    unsigned g = grid_for(d.NG_total, TPB, d.nsm * 8LL);
    k_group_items<<<g, TPB, 0, st>>>(d);
    cudaError_t e = scan_excl(d.item_cnt, d.item_off, d.NG_total, d.sst_witem, d.glob, 1, st);
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
    if (d.stream && d.NG_total > 0) {
        k_sitems<<<(unsigned)((d.NG_total + SITEM_TILE - 1) / SITEM_TILE), SITEM_WARPS * 32, 0, st>>>(d);
    }
    return cudaGetLastError();
}
cudaError_t launch_scatter(const DevPlan &d, cudaStream_t st) {
    if (d.n_total == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(&d.glob->nbig, 0, 2 * sizeof(unsigned), st);  // nbig, nhuge
    if (e != cudaSuccess) return e;
    k_perm<<<grid_for(d.n_total, TPB, d.nsm * 8LL), TPB, 0, st>>>(d);
    k_segsort<<<grid_for(4 * d.B_total, TPB, d.nsm * 8LL), TPB, 0, st>>>(d);
    k_segsort_big<<<(unsigned)(d.nsm * 4), TPB, 0, st>>>(d);
    if (d.learned) k_gather<true><<<grid_for(d.n_total, TPB, d.nsm * 8LL), TPB, 0, st>>>(d);
    else k_gather<false><<<grid_for(d.n_total, TPB, d.nsm * 8LL), TPB, 0, st>>>(d);
    return cudaGetLastError();
}
// leaves: the leaf sums of k_gather were overwritten since (bh_set_leaf_moments): redo them
cudaError_t launch_summarize(const DevPlan &d, bool leaves, cudaStream_t st) {
    if (leaves && d.n_total > 0) {
        const unsigned g = grid_for((d.n_total + 31) / 32, TPB / 32, d.nsm * 8LL);
        if (d.learned) k_leaf<true><<<g, TPB, 0, st>>>(d);
        else k_leaf<false><<<g, TPB, 0, st>>>(d);
    }
    // the second moments of the pyramid cells feed only the learned correction
    const unsigned g = grid_for(d.T_total, 1, d.nsm * 8LL);
    if (d.learned) k_summarize<true><<<g, SUM_THREADS, 0, st>>>(d, 0);
    else k_summarize<false><<<g, SUM_THREADS, 0, st>>>(d, 0);
    return cudaGetLastError();
}
cudaError_t launch_pyramid(const DevPlan &d, cudaStream_t st, bool second) {
    const unsigned g = grid_for(d.T_total, 1, d.nsm * 8LL);
    if (second && !d.learned) {
        // a plan without the learned correction sums no second moments: the leaves again from
        // the particles with them, then the pyramid
        if (d.n_total > 0) k_leaf<true><<<grid_for((d.n_total + 31) / 32, TPB / 32, d.nsm * 8LL), TPB, 0, st>>>(d);
        k_summarize<true><<<g, SUM_THREADS, 0, st>>>(d, 0);
    } else if (d.learned) {
        k_summarize<true><<<g, SUM_THREADS, 0, st>>>(d, 1);
    } else {
        k_summarize<false><<<g, SUM_THREADS, 0, st>>>(d, 1);
    }
    return cudaGetLastError();
}

}  // namespace bh

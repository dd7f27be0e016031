// bh_internal.cuh -- device-side layout shared by the kernels and the host
// layer of libbh_gb300.
//
// Data layout in HBM (one workspace, carved by bh_api.cu):
//   * particle state, double-buffered, box-sorted between steps (within a box,
//     quadrant by quadrant), SoA FP64:
//       X[2], Y[2], VX[2], VY[2], M[2] (n_total doubles each), PID[2] (int32)
//     The up-to-date state is buffer (epoch + 1) & 1; the step prologue
//     increments epoch, placement reads buffer epoch & 1 and scatters into
//     buffer (epoch + 1) & 1, which summarize / force / tick then use.  The
//     buffer choice is read on the device, so a captured CUDA graph of one
//     step replays correctly any number of times.
//   * PD: per box-sorted particle (x, x, y, y), (m, m, index, kx << 16 | ky)
//     with x, y the offsets from the box origin (formed in FP64, rounded once),
//     duplicated for packed f32x2 arithmetic, 32 bytes -- the list-streaming
//     kernel's near sources (copied into shared memory by bulk asynchronous
//     copies), every kernel's targets and the walking kernel's near sources.
//   * AX, AY: FP64 accelerations, box-sorted order (aligned with the state).
//   * key / slot: 4 * box key + quadrant, and rank in the quadrant, per particle
//     (placement output); skey: box key per box-sorted particle.
//   * counts, box_start: per-box histogram and exclusive prefix (int32),
//     concatenated over systems; box_start[b] is a global particle index;
//     qcounts: the four quadrant counts of every box.
//   * interaction lists, streaming work items and their order (list streaming):
//     see DevPlan.
//   * mom: FP64 moments (M, Sx, Sy, Sxx, Sxy, Syy about the cell origin) for
//     every pyramid cell; rec / rec2: float records the force kernel reads
//     (centre of mass relative to the cell origin, mass; normalised second
//     moments about the centre of mass, formed only for the learned correction).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/bh_gb300.h"

namespace bh {

constexpr int MAX_LEVELS = 16;  // G <= 32768
constexpr int FORCE_THREADS = 128;
constexpr int FORCE_R = 4;                                   // targets per thread (FP32)
constexpr int TARGET_CHUNK = FORCE_THREADS * FORCE_R;        // targets per work item
constexpr int FRONTIER_CAP = 512;                            // traversal frontier per level
constexpr int SCAN_TILE = 4096;   // counts per tile of the single-pass scans (256 threads x 16)
constexpr int MAX_TG = 8;          // largest target group (boxes per side)
constexpr int SITEM_TILE = 8;     // target groups per tile of the streaming work-item kernel (a warp each)
constexpr int SUM_TILE = 16;      // leaf boxes per side of a summarize tile (pyramid levels 0..4)
constexpr int STREAM_CHUNK = 128;  // targets per work item of the list-streaming force kernel
constexpr int LIST_MAX_G = 16384;  // largest G of the list-streaming path (32-bit group indices)
constexpr int ITEM_BUCKETS = 32;   // log2 cost buckets of the heaviest-first item order

struct SysDesc {
    long long n, poff;  // particle count, first particle (concatenated)
    long long boff;     // first box in counts / box_start
    long long coff;     // first pyramid cell (leaves first)
    long long goff;     // first target group
    int G, L, TG, NGs;  // boxes per side, pyramid levels, group dim, groups per side
    int lvg[MAX_LEVELS];         // cells per side per level
    long long lvoff[MAX_LEVELS]; // first cell of each level, relative to coff
    long long lfoff, lnoff;      // first far / near list slot of the system's groups
    int lfcap, lncap;            // far / near list slots per group
    long long ooff;              // first entry of the system's box-origin table (G x, then G y)
    int tps;                     // summarize tiles (SUM_TILE x SUM_TILE leaf boxes) per side
    long long toff;              // first summarize tile of the system
    long long upoff;             // first arrival counter of the system's cells above the tiles
    int fixed_grid;              // 1: the square box comes from fg_ext, not from the particles
    double fg_ext[4];            // min x, min y, max x, max y of the whole system (bh_set_grid)
};

struct SysDyn {
    unsigned long long bbmin[2];  // ordered bits of min x, min y (atomicMin)
    unsigned long long bbmax[2];  // ordered bits of max x, max y (atomicMax)
    double minx, miny, step;      // square bounding box origin and box edge
    double inv_step;              // 1 / step (0 when step is not positive)
    float minx_f, miny_f;         // the origin rounded to float
    float inv_step_f;             // 1 / step rounded to float
    float key_tol;                // bound on |float quotient - exact quotient| (box edges)
};

struct Globals {
    unsigned int epoch;
    unsigned int err;
    unsigned long long near_pairs, far_pairs;
    unsigned int item_next;   // force work queue head (zeroed before each force launch)
    unsigned int item_next2;  // learned-correction work queue head
    unsigned long long corr_pairs;  // (target, cell) pairs the learned correction evaluated
    unsigned int scan_ticket[3];    // next tile of each single-pass scan (its last tile resets it)
    unsigned int scan_gen[3];       // generation of each scan's tile states (its last tile bumps it)
    unsigned int bbox_done;         // bounding-box blocks finished (the last one finalises)
    unsigned int nbig;              // entries of the long-quadrant list (k_segsort)
    unsigned int nhuge;             // entries of the very-long-quadrant list, from its far end
};

struct DevPlan {
    int nsys, Lmax;
    long long n_total, B_total, C_total, NG_total;
    const SysDesc *sys;
    SysDyn *dyn;
    Globals *glob;
    const long long *poff_tab;  // nsys + 1 particle offsets
    const long long *boff_tab;  // nsys + 1 box offsets
    const long long *coff_tab;  // nsys + 1 cell offsets
    const long long *goff_tab;  // nsys + 1 group offsets
    const long long *toff_tab;  // nsys + 1 summarize-tile offsets
    long long T_total;          // summarize tiles over all systems
    const long long *lvl_tab;   // Lmax x (nsys + 1): prefix of level-l cells over systems
    long long lvl_cells[MAX_LEVELS];  // level-l cells over all systems (host copy, sizes grids)
    double *X[2], *Y[2], *VX[2], *VY[2], *M[2];
    int *PID[2];
    double *AX, *AY;  // accelerations, box-sorted order
    float4 *PD;  // per box-sorted particle: (x, x, y, y), (m, m, index, kx << 16 | ky) -- the
                 // packed near-field record (offsets from the box origin; box coordinates),
                 // staged into shared memory by bulk copies
    int *key, *slot, *skey;
    int *perm;     // box-sorted position -> input index (k_perm, k_segsort)
    int2 *bigseg;  // quadrant stretches too long for a thread's registers: (first, count)
    long long bigseg_cap;
    int *box_start;
    // single-pass scans (decoupled look-back): per-tile states of the box scan, the walk items'
    // scan and the streaming items' scan (generation << 34 | flag << 32 | value)
    unsigned long long *sst_box, *sst_witem, *sst_sitem;
    int *qcounts;  // per box, particles in each quadrant (x half * 2 + y half); a box's particles
                   // are stored quadrant by quadrant
    int *item_cnt, *item_off, *item_group;  // force work items (group, target chunk)
    double *org;  // per system: box origins mn + k step along x (k < G), then along y, FP64
    double *mom;
    unsigned *upcnt;  // per pyramid cell above the summarize tiles (levels >= 5): children done
                      // this step (the last child's CTA builds the cell and resets it)
    float *leafpart;  // per chunk of 32 box-sorted particles: head and tail partial moments (k_leaf)
    float4 *rec, *rec2;
    // interaction lists of every target group (list-streaming path), in fixed per-group slots
    // (SysDesc lfcap far entries, lncap + 1 near descriptors), counts in lcnt (x far, y near):
    //   far entry: the accepted cell's centre of mass in the group frame and its mass, float4
    //   (x, y, M, 0), formed with the opening test's own arithmetic;
    //   near descriptor: two int4 -- (first particle, exclusive prefix of the boxes' particle
    //   counts, shift of the box origin from the group origin as float bits x, y) and (box index
    //   in the system, mass, centre of mass in the group frame x, y as float bits); descriptor
    //   [count] carries the total in .y of its first int4
    float4 *lfar;
    int4 *lnear;
    int2 *lcnt;
    // list-streaming work items (per group: its sparse boxes together, then every dense box or
    // its quadrants): group, sub (-1: the sparse boxes; b = cx * TG + cy: box b; TG^2 + 4 b + q:
    // quadrant q of box b), (chunk, chunks)
    int *sitem_cnt, *sitem_off, *sitem_group, *sitem_sub;
    int2 *sitem_chunk;
    int dense_min;
    int quad_min;  // list streaming: boxes with at least this many particles get per-quadrant
                   // work items and near lists (0: none)
    int *item_order;  // list-streaming work items, heaviest cost bucket first
    int *item_bucket;  // ITEM_BUCKETS counts + ITEM_BUCKETS cursors
    unsigned char *item_cost;  // per list-streaming work item, its cost bucket (k_item_hist)
    int nsm;     // streaming multiprocessors of the plan's device (queried at bh_bind): sizes the
                 // persistent and grid-stride launches
    int stream;  // 1: lists are built by k_lists and streamed by k_fstream
    int chunk;   // targets per work item (TARGET_CHUNK, or STREAM_CHUNK when stream)
    // parameters
    double gconst, dt, eps2, cutoff;
    float theta2_f, eps2_f, cut_f;
    int flat, prec, learned, tune;
    double correction_theta;
};

// ---------------------------------------------------------------- helpers
__device__ __forceinline__ unsigned long long ord_bits(double d) {
    unsigned long long u = (unsigned long long)__double_as_longlong(d);
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double unord_bits(unsigned long long u) {
    u = (u & 0x8000000000000000ull) ? (u & ~0x8000000000000000ull) : ~u;
    return __longlong_as_double((long long)u);
}

// index of the segment containing v in a sorted offset table tab[0..n]
// (tab[0] = 0 <= v < tab[n]); n is small (systems).
__device__ __forceinline__ int find_seg(const long long *tab, int n, long long v) {
    int lo = 0, hi = n;  // invariant tab[lo] <= v < tab[hi]
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (tab[mid] <= v) lo = mid; else hi = mid;
    }
    return lo;
}

// Square bounding box exactly as python-bh/barneshut/kernels/helpers/grid.py:10-26
// and base.py:233-239 compute it (no FMA contraction).
__device__ __forceinline__ void square_bbox(double mnx, double mny, double mxx, double mxy, int G,
                                            double *step) {
    double xe = __dsub_rn(mxx, mnx), ye = __dsub_rn(mxy, mny);
    if (xe > ye) mxy = __dadd_rn(mxy, __dsub_rn(xe, ye));
    else if (ye > xe) mxx = __dadd_rn(mxx, __dsub_rn(ye, xe));
    *step = __ddiv_rn(__dsub_rn(mxx, mnx), (double)G);
}

// Box index of one coordinate: clip(floor((p - mn) / step), 0, G - 1)
// (implementations/sequential.py:32-34; gpu/grid.py:37-40).
__device__ __forceinline__ int box_key1(double p, double mn, double step, int G) {
    if (!(step > 0.0)) return 0;
    double k = floor(__ddiv_rn(__dsub_rn(p, mn), step));
    k = fmin(fmax(k, 0.0), (double)(G - 1));
    return (int)k;
}

// Same key, computed as floor((p - mn) * inv_step).  The product differs from the correctly
// rounded quotient by at most ~3 ulp, so the floors can differ only when the quotient lies
// within ~3 ulp of an integer (< 1e-10 for G <= 32768); only then is the IEEE division taken.
// FP64 -> FP32 rounded to nearest, ties to even (the IEEE 754 narrowing conversion), on the
// integer pipes: bit-identical to __double2float_rn
// whenever the result is a normal float (a mantissa carry rounds into the exponent, and past the
// largest float into infinity, as IEEE rounding does); zero, subnormal and out-of-range inputs
// take __double2float_rn.  GB300 executes that conversion on its slow FP64 pipe.
__device__ __forceinline__ float f64_to_f32_rn(double p) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(p);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const int e = (int)((hi >> 20) & 0x7FFu) - 1023 + 127;  // biased float exponent
    if (e < 1 || e > 254) return __double2float_rn(p);
    // the float fraction: hi's 20 fraction bits and lo's top 3; the 29 dropped bits round it
    const unsigned m = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    const unsigned rest = lo & 0x1FFFFFFFu, half = 0x10000000u;
    const unsigned up = (rest > half || (rest == half && (m & 1u))) ? 1u : 0u;
    return __uint_as_float(((hi & 0x80000000u) | ((unsigned)e << 23) | m) + up);
}

__device__ __forceinline__ int box_key1_fast(double p, double mn, double step, double inv, int G) {
    if (!(step > 0.0)) return 0;
    double d = __dsub_rn(p, mn);
    double q = __dmul_rn(d, inv);
    double k = floor(q);
    double fr = q - k;
    if (fr < 1e-10 || fr > 1.0 - 1e-10) k = floor(__ddiv_rn(d, step));
    k = fmin(fmax(k, 0.0), (double)(G - 1));
    return (int)k;
}

// float -> double on the integer pipes: exact for normal floats and zeros (rebias the exponent,
// widen the mantissa); subnormal, infinite and NaN inputs take the hardware conversion, which
// GB300 runs on its slow FP64 pipe.
__device__ __forceinline__ double f32_to_f64(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xFFu;
    if (e == 0u) {
        if ((u & 0x7FFFFFu) == 0u) return __longlong_as_double((long long)(u & 0x80000000u) << 32);
        return (double)f;
    }
    if (e == 0xFFu) return (double)f;
    const unsigned long long bits = ((unsigned long long)(u & 0x80000000u) << 32) |
                                    ((unsigned long long)(e + 896u) << 52) |
                                    ((unsigned long long)(u & 0x7FFFFFu) << 29);
    return __longlong_as_double((long long)bits);
}

// The same key with a float estimate first: q_f = (float(p) - float(mn)) * float(1 / step) is
// within tol of the FP64 quotient (tol from the system's extent, set in k_bbox_finalize), so
// floor(q_f) is the exact key unless q_f lies within tol of an integer; only then (and for an
// unusable tol) is the FP64 key computed.  GB300 runs FP64 at 1/64 of the FP32 rate, and the
// FP64 key costs about nine FP64 operations per coordinate.
__device__ __forceinline__ int box_key1_f32(double p, double mn, double step, double inv, float mn_f,
                                            float inv_f, float tol, int G) {
    const float q = __fmul_rn(__fsub_rn(f64_to_f32_rn(p), mn_f), inv_f);
    const float k = floorf(q);
    const float fr = q - k;
    if (!(tol < 0.25f) || fr < tol || fr > 1.f - tol) return box_key1_fast(p, mn, step, inv, G);
    return min(max((int)k, 0), G - 1);
}

// Key of one coordinate at twice the box resolution: clip(floor(2 q), 0, 2 G - 1) with q the
// FP64 quotient (p - mn) / step of box_key1.  Its high part (>> 1) is box_key1's key (floor(2 q)
// >> 1 = floor(q) for q >= 0, and the clips agree), its low bit the half of the box.
__device__ __forceinline__ int half_key1_fast(double p, double mn, double step, double inv, int G) {
    if (!(step > 0.0)) return 0;
    double d = __dsub_rn(p, mn);
    double q = __dmul_rn(__dmul_rn(d, inv), 2.0);
    double k = floor(q);
    double fr = q - k;
    if (fr < 1e-10 || fr > 1.0 - 1e-10) k = floor(__dmul_rn(__ddiv_rn(d, step), 2.0));
    k = fmin(fmax(k, 0.0), (double)(2 * G - 1));
    return (int)k;
}
// The same from the float estimate (2 q_f carries twice box_key1_f32's error bound).
__device__ __forceinline__ int half_key1_f32(double p, double mn, double step, double inv, float mn_f,
                                             float inv_f, float tol, int G) {
    const float q = 2.f * __fmul_rn(__fsub_rn(f64_to_f32_rn(p), mn_f), inv_f);
    const float k = floorf(q);
    const float fr = q - k;
    const float tol2 = 2.f * tol;
    if (!(tol2 < 0.25f) || fr < tol2 || fr > 1.f - tol2) return half_key1_fast(p, mn, step, inv, G);
    return min(max((int)k, 0), 2 * G - 1);
}

// Work-item kind of a box with nb particles (list streaming): 2 per-quadrant items, 1 own items,
// 0 shared with the group's other sparse boxes.
__device__ __forceinline__ int box_item_kind(int nb, int dense_min, int quad_min) {
    if (quad_min > 0 && nb >= quad_min) return 2;
    return nb >= dense_min ? 1 : 0;
}

// Streaming multiprocessors of the current device (the runtime caches the attribute); grid-stride
// launches that have no plan size their grids with it.
inline int device_sm_count() {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1)
        return 1;
    return n;
}

// Origin of leaf box k along one axis: mn + k * step, FP64, no contraction.
__device__ __forceinline__ double box_origin(double mn, int k, double step) {
    return __dadd_rn(mn, __dmul_rn((double)k, step));
}

// Targets [c0, c0 + T) of work item k of a group whose nt targets are split into nch items of
// near-equal size (each at most ceil(nt / nch)).
__device__ __forceinline__ void item_range(int nt, int nch, int k, int *c0, int *T) {
    const int a = (int)((long long)k * nt / nch), b = (int)((long long)(k + 1) * nt / nch);
    *c0 = a;
    *T = b - a;
}

// List-streaming work items of a target set of nt particles: full chunks of STREAM_CHUNK, then
// the remainder r = nt mod STREAM_CHUNK cut into pieces that keep a warp's lanes busy.  A piece of
// T targets occupies ceil(T / FORCE_R) lanes per slice and 32 / ceil(T / FORCE_R) slices (each
// slice sweeps its share of the sources), so its sweep takes sources / slices lane-passes for
// T x sources pairs: 128, 64 and 32 targets use every lane, while 65..127 targets run a single
// slice on 17..32 lanes.  The remainder therefore yields a piece of 64 first when r > 64, then a
// piece of 32 when 41..48 targets are left (two slices of 11..12 lanes become four of 8 plus a
// small piece), then the rest.  An extra piece needs at least 41 targets, so a set of nt targets
// has at most 1 + nt / 40 items.
constexpr int STREAM_ITEM_DIV = 32;  // items <= sets + n / STREAM_ITEM_DIV

__host__ __device__ __forceinline__ int sitem_count(int nt) {
    int r = nt % STREAM_CHUNK, n = nt / STREAM_CHUNK;
    if (r > 64) { n++; r -= 64; }
    if (r > 40 && r <= 48) { n++; r -= 32; }
    return n + (r > 0 ? 1 : 0);
}

// Targets [c0, c0 + T) of item k of a target set of nt particles (k < sitem_count(nt)).
__device__ __forceinline__ void sitem_range(int nt, int k, int *c0, int *T) {
    const int full = nt / STREAM_CHUNK;
    int c = k < full ? k * STREAM_CHUNK : full * STREAM_CHUNK, r = nt - c, j = k - full;
    if (j >= 0 && r > 64) {
        if (j == 0) r = 64;
        else { c += 64; r -= 64; j--; }
    }
    if (j >= 0 && r > 40 && r <= 48) {
        if (j == 0) r = 32;
        else { c += 32; r -= 32; }
    }
    *c0 = c;
    *T = min(STREAM_CHUNK, r);
}

__device__ __forceinline__ void raise_err(Globals *g, unsigned f) {
    if ((atomicOr(&g->err, 0u) & f) == 0) atomicOr(&g->err, f);
}

}  // namespace bh

// kernel launch wrappers (bh_tree.cu, bh_force.cu, bh_misc.cu)
namespace bh {
cudaError_t launch_prologue(const DevPlan &d, cudaStream_t st);
cudaError_t launch_bbox(const DevPlan &d, cudaStream_t st);
cudaError_t launch_place(const DevPlan &d, cudaStream_t st);
cudaError_t launch_scan(const DevPlan &d, cudaStream_t st);
cudaError_t launch_items(const DevPlan &d, cudaStream_t st);
cudaError_t launch_walk_items(const DevPlan &d, cudaStream_t st);
cudaError_t launch_scatter(const DevPlan &d, cudaStream_t st);
cudaError_t launch_summarize(const DevPlan &d, bool leaves, cudaStream_t st);
// the pyramid levels above the leaves and the cell records, from the leaf moments
// second: also the second moments and their records (always with the learned correction; a plan
// without it sums its leaves again from the particles for them)
cudaError_t launch_pyramid(const DevPlan &d, cudaStream_t st, bool second = false);
// ev (optional): two events recorded on st right before and after the force kernel proper
cudaError_t launch_force(const DevPlan &d, bool tick, bool accumulate, cudaStream_t st,
                         const cudaEvent_t *ev = nullptr);
cudaError_t launch_lists(const DevPlan &d, cudaStream_t st);
cudaError_t launch_fstream(const DevPlan &d, bool tick, bool accumulate, cudaStream_t st,
                           const cudaEvent_t *ev = nullptr);
cudaError_t fstream_init();
cudaError_t force_init();
cudaError_t launch_tick(const DevPlan &d, cudaStream_t st, bool keep_acc = false);
cudaError_t launch_load(const DevPlan &d, const double *x, const double *y, const double *m,
                        const double *vx, const double *vy, long long rec_stride,
                        cudaStream_t st);
cudaError_t launch_store(const DevPlan &d, int has_tree, bool has_acc, double *rec, double *x, double *y, double *vx,
                         double *vy, double *ax, double *ay, cudaStream_t st);
cudaError_t launch_direct(const DevPlan &d, int sys, const long long *targets, long long nt,
                          double *ax, double *ay, cudaStream_t st);
cudaError_t launch_diag(const DevPlan &d, int sys, int want_pot, double *out, cudaStream_t st);
cudaError_t launch_box_com(const DevPlan &d, int sys, double *out, cudaStream_t st);
// record a failure of a call without a plan (read by bh_last_error(NULL)); returns code
int bh_set_thread_error(int code, const char *msg);
// learned correction (bh_mlp.cu)
constexpr int MLP_PARAMS = 10448;
constexpr int MLP_IMAGE_BYTES = 38912;
cudaError_t mlp_init();
cudaError_t mlp_pack(const float *params, uint8_t *img, cudaStream_t st);
cudaError_t mlp_infer(const float *feats, int fs, long long P, const uint8_t *img,
                      const float *params, float *out, unsigned *err, cudaStream_t st);
cudaError_t mlp_train(const float *feats, int fs, const float *targets, long long P,
                      const uint8_t *img, const float *params, float *grad, float *loss,
                      unsigned *err, cudaStream_t st);
cudaError_t mlp_adam(float *p, float *m, float *v, float *g, int step, float lr, cudaStream_t st);
cudaError_t learned_init();
cudaError_t launch_learned_correct(const DevPlan &d, double theta_lo, const uint8_t *img,
                                   const float *params, bool tick, cudaStream_t st);
cudaError_t launch_learned_pairs(const DevPlan &d, double theta_hi, double theta_lo, int max_level,
                                 long long item_offset, long long item_stride, int tpi,
                                 float *feats, float *targets, unsigned *counter, long long capacity,
                                 cudaStream_t st);
}  // namespace bh

// bh_api.cu -- host side of the C ABI declared in include/bh_gb300.h.
//
// A plan is a host object: the system table, the workspace layout and the
// launch sequence of each step phase.  It allocates no device memory; the
// caller binds one workspace buffer.  Kernels read the plan's device tables
// and a device-side epoch that selects the current state buffer, so a step
// captured into a CUDA graph replays correctly.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>
#include <new>
#include <vector>

#include "../../include/bh_gb300.h"
#include "bh_internal.cuh"

using namespace bh;

struct bh_plan {
    bh_params params;
    int nsys = 0;
    std::vector<SysDesc> sys;
    std::vector<long long> poff, boff, coff, goff, toff, lvl;
    int Lmax = 1;
    long long n_total = 0, B_total = 0, C_total = 0, NG_total = 0;
    long long org_total = 0;  // entries of the box-origin tables (2 G per system)
    // workspace layout (byte offsets)
    size_t ws_bytes = 0;
    size_t o_sys, o_dyn, o_glob, o_poff, o_boff, o_coff, o_goff, o_toff, o_lvl;
    size_t o_X[2], o_Y[2], o_VX[2], o_VY[2], o_M[2], o_PID[2];
    size_t o_AX, o_AY, o_key, o_slot, o_skey, o_bstart, o_sst, o_leafpart, o_perm, o_bigseg, o_icnt, o_ioff, o_igrp, o_mom, o_rec, o_PD,
        o_rec2, o_org, o_lfar, o_lnear, o_lcnt, o_iord, o_icost, o_ibkt, o_sicnt, o_sioff, o_sigrp, o_sisub, o_sichk, o_qcnt;
    bool stream = false;  // theta-mode interaction lists built once per group and streamed
    int chunk = TARGET_CHUNK;
    int dense_min = BH_STREAM_DENSE_MIN;
    int quad_min = BH_STREAM_QUAD_MIN;
    void *ws = nullptr;
    int device = -1;
    int nsm = 1;  // streaming multiprocessors of `device`
    DevPlan dev;
    bool has_tree = false;
    bool acc_stale = true;  // next bh_evaluate overwrites instead of accumulating
    bool acc_valid = false;  // AX/AY hold accelerations (else they are zero by definition: a load
                             // or a generation does not write them)
    bool leaves_stale = false;  // leaf moments overwritten since the last create_tree
    // graph cache
    cudaGraphExec_t gexec = nullptr;
    size_t sst_bytes = 0;  // the single-pass scans' tile states
    size_t o_upcnt = 0;
    long long up_total = 0;  // pyramid cells above the summarize tiles, over all systems
    cudaEvent_t tev[2] = {nullptr, nullptr};  // bh_set_kernel_timing: around the force kernel
    bool timing = false;
    bool tev_recorded = false;
    int gkernels = -1;  // kernel nodes of the captured step graph
    int gsteps = 0;
    cudaStream_t gstream = nullptr;
    // create_tree's side branch: the work items (they need only the box scan) run on `side`
    // while the scatter runs on the caller's stream; fork and join through two events, which
    // a stream capture turns into graph edges
    cudaStream_t side = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    // learned correction (caller-owned device buffers)
    const uint8_t *mlp_img = nullptr;
    const float *mlp_params = nullptr;
    char err[512];
};

static int fail(bh_plan *p, int code, const char *fmt, ...) {
    if (p) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(p->err, sizeof(p->err), fmt, ap);
        va_end(ap);
    }
    return code;
}

static int cuda_fail(bh_plan *p, cudaError_t e, const char *what) {
    return fail(p, BH_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(p, call, what)                                  \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return cuda_fail(p, e_, what); \
    } while (0)

static size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

static thread_local char g_create_err[256] = "";

int bh::bh_set_thread_error(int code, const char *msg) {
    snprintf(g_create_err, sizeof(g_create_err), "%s", msg);
    return code;
}

extern "C" int bh_grid_dim(long long n, int ppb) {
    // base.py:223-231 with helpers/grid.py:5-8 (next_perfect_square)
    if (n <= 0) return 0;
    double nleaves = ppb == 1 ? 1.0 : (double)n / (0.7 * (double)ppb);
    double r = std::sqrt(nleaves);
    if (r == 0.0 || std::fmod(nleaves, r) != 0.0) {
        double c = std::ceil(r);
        nleaves = c * c;
    }
    return (int)std::sqrt(nleaves);
}

static int auto_group(long long n, int G) {
    double nb = G > 0 ? (double)n / ((double)G * G) : 0.0;
    if (nb >= 32.0) return 1;
    if (nb >= 8.0) return 2;
    if (nb >= 2.0) return 4;
    return 8;
}

extern "C" int bh_plan_create(bh_plan **out, int nsys, const long long *n, const int *grid_dim,
                              const bh_params *params) {
    if (!out) return BH_ERR_INVALID;
    *out = nullptr;
    if (nsys < 1 || !n || !params) {
        snprintf(g_create_err, sizeof(g_create_err), "bh_plan_create: nsys < 1 or null argument");
        return BH_ERR_INVALID;
    }
    bh_plan *p = new (std::nothrow) bh_plan();
    if (!p) return BH_ERR_INVALID;
    p->err[0] = 0;
    p->params = *params;
    const bh_params &pr = p->params;
    auto bad = [&](const char *msg) {
        snprintf(g_create_err, sizeof(g_create_err), "bh_plan_create: %s", msg);
        delete p;
        return BH_ERR_INVALID;
    };
    if (!(pr.tick_seconds == pr.tick_seconds) || !std::isfinite(pr.grav_constant)) return bad("bad constants");
    if (!(pr.softening >= 0.0) || !(pr.cutoff_r2 >= 0.0)) return bad("negative softening/cutoff");
    if (pr.precision < 0 || pr.precision > 2) return bad("precision");
    if (pr.group_dim < 0 || pr.group_dim > 8 || (pr.group_dim & (pr.group_dim - 1))) return bad("group_dim");
    const bool flat = !(pr.theta > 0.0);
    p->nsys = nsys;
    p->sys.resize(nsys);
    p->poff.assign(nsys + 1, 0);
    p->boff.assign(nsys + 1, 0);
    p->coff.assign(nsys + 1, 0);
    p->goff.assign(nsys + 1, 0);
    p->toff.assign(nsys + 1, 0);
    for (int s = 0; s < nsys; s++) {
        if (n[s] < 0 || n[s] > (1LL << 30)) return bad("particle count out of range [0, 2^30]");
        int G = grid_dim && grid_dim[s] > 0 ? grid_dim[s] : bh_grid_dim(n[s], 1000);
        if (G < 1) G = 1;
        if (G > 32768) return bad("grid_dim > 32768");
        SysDesc &d = p->sys[s];
        memset(&d, 0, sizeof(d));
        d.n = n[s];
        d.poff = p->poff[s];
        d.G = G;
        int L = 0;
        long long cells = 0;
        for (int g = G;;) {
            d.lvg[L] = g;
            d.lvoff[L] = cells;
            cells += (long long)g * g;
            L++;
            if (g == 1) break;
            g = (g + 1) / 2;
        }
        d.L = L;
        int TG = flat ? 1 : (pr.group_dim > 0 ? pr.group_dim : auto_group(n[s], G));
        if (!flat) {
            // children of cells rejected at level l+1 (edge s >= 2 boxes): a rejected cell
            // intersects the group widened by s/theta, so at most (TG/2 + 2/theta + 2)^2 of
            // them, four children each.  Keep that within the kernel's frontier.
            double bound = 4.0 * std::pow(TG / 2.0 + 2.0 / pr.theta + 2.0, 2.0);
            while (bound > (double)FRONTIER_CAP && TG > 1) {
                TG /= 2;
                bound = 4.0 * std::pow(TG / 2.0 + 2.0 / pr.theta + 2.0, 2.0);
            }
            if (bound > (double)FRONTIER_CAP) return bad("theta too small for the traversal frontier (theta >= 0.25)");
        }
        d.TG = TG;
        d.NGs = (G + TG - 1) / TG;
        d.ooff = p->org_total;
        p->org_total += 2LL * G;
        d.boff = p->boff[s];
        d.coff = p->coff[s];
        d.goff = p->goff[s];
        d.tps = (G + SUM_TILE - 1) / SUM_TILE;
        d.toff = p->toff[s];
        d.upoff = p->up_total;
        p->up_total += L > 5 ? cells - d.lvoff[5] : 0;
        p->poff[s + 1] = p->poff[s] + n[s];
        p->boff[s + 1] = p->boff[s] + (long long)G * G;
        p->coff[s + 1] = p->coff[s] + cells;
        p->goff[s + 1] = p->goff[s] + (long long)d.NGs * d.NGs;
        p->toff[s + 1] = p->toff[s] + (long long)d.tps * d.tps;
        if (L > p->Lmax) p->Lmax = L;
    }
    p->n_total = p->poff[nsys];
    // list-streaming force path: theta mode, FP32 pairs, softening > 0, no cutoff, G <= 16384
    int maxG = 0;
    for (int s = 0; s < nsys; s++) maxG = std::max(maxG, p->sys[s].G);
    p->stream = !flat && pr.precision != BH_PREC_FP64 && pr.cutoff_r2 == 0.0 && pr.softening > 0.0 &&
                !(pr.flags & BH_FLAG_WALK) && maxG <= LIST_MAX_G;
    p->chunk = p->stream ? STREAM_CHUNK : TARGET_CHUNK;
    if (pr.dense_min < 0) return bad("dense_min < 0");
    p->dense_min = pr.dense_min > 0 ? pr.dense_min : BH_STREAM_DENSE_MIN;
    p->quad_min = pr.quad_min > 0 ? pr.quad_min : (pr.quad_min == 0 ? BH_STREAM_QUAD_MIN : 0);
    long long lf_total = 0, ln_total = 0;
    if (p->stream) {
        // a level's accepted cells are a subset of its frontier, and the near boxes a subset of
        // the leaf level's frontier; a frontier holds the children of the cells rejected one level
        // up, at most 4 (TG/2 + 2/theta + 2)^2 (the bound checked against FRONTIER_CAP above)
        for (int s = 0; s < nsys; s++) {
            SysDesc &d = p->sys[s];
            const double fb = 4.0 * std::pow(d.TG / 2.0 + 2.0 / pr.theta + 2.0, 2.0);
            const long long lvcap = std::min<long long>(FRONTIER_CAP, (long long)std::ceil(fb));
            long long cap = 0;
            for (int l = 0; l < d.L; l++) cap += std::min<long long>(lvcap, (long long)d.lvg[l] * d.lvg[l]);
            d.lfcap = (int)cap;
            // a near leaf is rejected for the group rectangle, so its centre of mass lies within
            // 1/theta box edges of it: at most floor(1/theta) + 1 boxes away (one more for rounding)
            const long long reach = (long long)std::floor(1.0 / pr.theta) + 2;
            const long long side = std::min<long long>(d.G, d.TG + 2 * reach);
            d.lncap = (int)std::min<long long>(FRONTIER_CAP, side * side);
            d.lfoff = lf_total;
            d.lnoff = ln_total;
            lf_total += (long long)d.NGs * d.NGs * d.lfcap;
            ln_total += (long long)d.NGs * d.NGs * 2 * (d.lncap + 1);
        }
    }
    p->B_total = p->boff[nsys];
    p->C_total = p->coff[nsys];
    p->NG_total = p->goff[nsys];
    if (p->n_total >= (1LL << 31) || p->C_total >= (1LL << 31) || p->B_total >= (1LL << 29))
        return bad("total particles or cells >= 2^31, or boxes >= 2^29");
    // level tables: prefix of level-l cell counts over systems
    p->lvl.assign((size_t)p->Lmax * (nsys + 1), 0);
    for (int l = 0; l < p->Lmax; l++)
        for (int s = 0; s < nsys; s++) {
            long long c = l < p->sys[s].L ? (long long)p->sys[s].lvg[l] * p->sys[s].lvg[l] : 0;
            p->lvl[(size_t)l * (nsys + 1) + s + 1] = p->lvl[(size_t)l * (nsys + 1) + s] + c;
        }
    // workspace layout
    size_t o = 0;
    auto take = [&](size_t bytes) {
        size_t r = o;
        o = align_up(o + (bytes ? bytes : 1), 256);
        return r;
    };
    const size_t N = (size_t)p->n_total, B = (size_t)p->B_total, C = (size_t)p->C_total;
    p->o_sys = take(sizeof(SysDesc) * nsys);
    p->o_dyn = take(sizeof(SysDyn) * nsys);
    p->o_glob = take(sizeof(Globals));
    p->o_poff = take(sizeof(long long) * (nsys + 1));
    p->o_boff = take(sizeof(long long) * (nsys + 1));
    p->o_coff = take(sizeof(long long) * (nsys + 1));
    p->o_goff = take(sizeof(long long) * (nsys + 1));
    p->o_toff = take(sizeof(long long) * (nsys + 1));
    p->o_lvl = take(sizeof(long long) * p->lvl.size());
    for (int b = 0; b < 2; b++) {
        p->o_X[b] = take(8 * N);
        p->o_Y[b] = take(8 * N);
        p->o_VX[b] = take(8 * N);
        p->o_VY[b] = take(8 * N);
        p->o_M[b] = take(8 * N);
        p->o_PID[b] = take(4 * N);
    }
    p->o_AX = take(8 * N);
    p->o_AY = take(8 * N);
    p->o_PD = take(32 * N);
    p->o_key = take(4 * N);
    p->o_slot = take(4 * N);
    p->o_skey = take(4 * N);
    p->o_perm = take(4 * N);
    p->o_bigseg = take(8 * (N / 17 + 1));  // quadrants of more than 16 particles: at most N / 17
    p->o_qcnt = take(16 * B);
    p->o_bstart = take(4 * (B + 1));
    p->sst_bytes = 8 * (B / SCAN_TILE + 2 + (size_t)p->NG_total / SCAN_TILE + 2 + (size_t)p->NG_total / SITEM_TILE + 2);
    p->o_sst = take(p->sst_bytes);
    p->o_icnt = take(4 * (size_t)p->NG_total);
    p->o_ioff = take(4 * ((size_t)p->NG_total + 1));
    p->o_igrp = take(4 * ((size_t)p->NG_total + N / p->chunk + 1));
    p->o_lfar = take(16 * (size_t)lf_total);
    p->o_lnear = take(16 * (size_t)ln_total);
    p->o_lcnt = take(p->stream ? 8 * (size_t)p->NG_total : 0);
    // target sets: a sparse set per group, each dense box, each quadrant of a quadrant box; a
    // set of nt targets has at most 1 + nt / 40 items (sitem_count)
    const size_t sitems = p->stream ? (size_t)p->NG_total + N / p->dense_min +
                                          (p->quad_min > 0 ? 4 * (N / p->quad_min) : 0) + N / STREAM_ITEM_DIV + 1
                                    : 0;
    p->o_iord = take(4 * sitems);
    p->o_icost = take(sitems);
    p->o_sicnt = take(p->stream ? 4 * (size_t)p->NG_total : 0);
    p->o_sioff = take(p->stream ? 4 * ((size_t)p->NG_total + 1) : 0);
    p->o_sigrp = take(4 * sitems);
    p->o_sisub = take(4 * sitems);
    p->o_sichk = take(8 * sitems);
    p->o_ibkt = take(p->stream ? 4 * 2 * ITEM_BUCKETS : 0);
    p->o_mom = take(48 * C);
    p->o_upcnt = take(4 * (size_t)p->up_total);
    p->o_leafpart = take(48 * (N / 32 + 1));
    p->o_rec = take(16 * C);
    p->o_rec2 = take(16 * C);
    p->o_org = take(8 * (size_t)p->org_total);
    p->ws_bytes = o;
    *out = p;
    return BH_OK;
}

extern "C" int bh_plan_destroy(bh_plan *p) {
    if (!p) return BH_ERR_INVALID;
    if (p->gexec) cudaGraphExecDestroy(p->gexec);
    if (p->gstream) cudaStreamDestroy(p->gstream);
    if (p->side) cudaStreamDestroy(p->side);
    for (cudaEvent_t e : {p->fork_ev, p->join_ev, p->tev[0], p->tev[1]})
        if (e) cudaEventDestroy(e);
    delete p;
    return BH_OK;
}

// bh_last_error(NULL) reports the last bh_plan_create failure of this thread.
extern "C" const char *bh_last_error(const bh_plan *p) { return p ? p->err : g_create_err; }

extern "C" int bh_workspace_size(const bh_plan *p, size_t *bytes) {
    if (!p || !bytes) return BH_ERR_INVALID;
    *bytes = p->ws_bytes;
    return BH_OK;
}

static void fill_dev(bh_plan *p) {
    char *w = (char *)p->ws;
    DevPlan &d = p->dev;
    memset(&d, 0, sizeof(d));
    d.nsys = p->nsys;
    d.Lmax = p->Lmax;
    d.n_total = p->n_total;
    d.B_total = p->B_total;
    d.C_total = p->C_total;
    d.NG_total = p->NG_total;
    d.sys = (const SysDesc *)(w + p->o_sys);
    d.dyn = (SysDyn *)(w + p->o_dyn);
    d.glob = (Globals *)(w + p->o_glob);
    d.poff_tab = (const long long *)(w + p->o_poff);
    d.boff_tab = (const long long *)(w + p->o_boff);
    d.coff_tab = (const long long *)(w + p->o_coff);
    d.goff_tab = (const long long *)(w + p->o_goff);
    d.toff_tab = (const long long *)(w + p->o_toff);
    d.T_total = p->toff[p->nsys];
    d.lvl_tab = (const long long *)(w + p->o_lvl);
    for (int l = 0; l < p->Lmax && l < MAX_LEVELS; l++) d.lvl_cells[l] = p->lvl[(size_t)l * (p->nsys + 1) + p->nsys];
    for (int b = 0; b < 2; b++) {
        d.X[b] = (double *)(w + p->o_X[b]);
        d.Y[b] = (double *)(w + p->o_Y[b]);
        d.VX[b] = (double *)(w + p->o_VX[b]);
        d.VY[b] = (double *)(w + p->o_VY[b]);
        d.M[b] = (double *)(w + p->o_M[b]);
        d.PID[b] = (int *)(w + p->o_PID[b]);
    }
    d.AX = (double *)(w + p->o_AX);
    d.AY = (double *)(w + p->o_AY);
    d.PD = (float4 *)(w + p->o_PD);
    d.key = (int *)(w + p->o_key);
    d.slot = (int *)(w + p->o_slot);
    d.skey = (int *)(w + p->o_skey);
    d.perm = (int *)(w + p->o_perm);
    d.bigseg = (int2 *)(w + p->o_bigseg);
    d.bigseg_cap = p->n_total / 17 + 1;
    d.qcounts = (int *)(w + p->o_qcnt);
    d.box_start = (int *)(w + p->o_bstart);
    d.sst_box = (unsigned long long *)(w + p->o_sst);
    d.sst_witem = d.sst_box + p->B_total / SCAN_TILE + 2;
    d.sst_sitem = d.sst_witem + p->NG_total / SCAN_TILE + 2;
    d.item_cnt = (int *)(w + p->o_icnt);
    d.item_off = (int *)(w + p->o_ioff);
    d.item_group = (int *)(w + p->o_igrp);
    d.mom = (double *)(w + p->o_mom);
    d.leafpart = (float *)(w + p->o_leafpart);
    d.upcnt = (unsigned *)(w + p->o_upcnt);
    d.rec = (float4 *)(w + p->o_rec);
    d.rec2 = (float4 *)(w + p->o_rec2);
    d.org = (double *)(w + p->o_org);
    d.lfar = (float4 *)(w + p->o_lfar);
    d.lnear = (int4 *)(w + p->o_lnear);
    d.lcnt = (int2 *)(w + p->o_lcnt);
    d.item_order = (int *)(w + p->o_iord);
    d.sitem_cnt = (int *)(w + p->o_sicnt);
    d.sitem_off = (int *)(w + p->o_sioff);
    d.sitem_group = (int *)(w + p->o_sigrp);
    d.sitem_sub = (int *)(w + p->o_sisub);
    d.sitem_chunk = (int2 *)(w + p->o_sichk);
    d.dense_min = p->dense_min;
    d.quad_min = p->quad_min;
    d.item_bucket = (int *)(w + p->o_ibkt);
    d.item_cost = (unsigned char *)(w + p->o_icost);
    d.nsm = p->nsm;
    d.stream = p->stream ? 1 : 0;
    d.chunk = p->chunk;
    const bh_params &pr = p->params;
    d.gconst = pr.grav_constant;
    d.dt = pr.tick_seconds;
    d.eps2 = pr.softening * pr.softening;
    d.cutoff = pr.cutoff_r2;
    d.theta2_f = (float)(pr.theta * pr.theta);
    d.eps2_f = (float)d.eps2;
    d.cut_f = (float)d.cutoff;
    d.flat = pr.theta > 0.0 ? 0 : 1;
    d.prec = pr.precision;
    d.learned = (pr.flags & BH_FLAG_LEARNED) ? 1 : 0;
    d.tune = pr.tune;
    d.correction_theta = pr.correction_theta;
}

extern "C" int bh_bind(bh_plan *p, void *workspace, size_t bytes, void *stream) {
    if (!p) return BH_ERR_INVALID;
    if (!workspace || bytes < p->ws_bytes)
        return fail(p, BH_ERR_WORKSPACE, "workspace of %zu bytes < required %zu", bytes, p->ws_bytes);
    if (((uintptr_t)workspace) & 255) return fail(p, BH_ERR_WORKSPACE, "workspace not 256-byte aligned");
    cudaStream_t st = (cudaStream_t)stream;
    CK(p, cudaGetDevice(&p->device), "cudaGetDevice");
    CK(p, cudaDeviceGetAttribute(&p->nsm, cudaDevAttrMultiProcessorCount, p->device), "SM count");
    if (p->nsm < 1) p->nsm = 1;
    CK(p, force_init(), "force kernel attributes");
    CK(p, learned_init(), "learned kernel attributes");
    if (!p->side) CK(p, cudaStreamCreateWithFlags(&p->side, cudaStreamNonBlocking), "side stream");
    if (!p->fork_ev) CK(p, cudaEventCreateWithFlags(&p->fork_ev, cudaEventDisableTiming), "fork event");
    if (!p->join_ev) CK(p, cudaEventCreateWithFlags(&p->join_ev, cudaEventDisableTiming), "join event");
    p->ws = workspace;
    fill_dev(p);
    char *w = (char *)workspace;
    CK(p, cudaMemcpyAsync(w + p->o_sys, p->sys.data(), sizeof(SysDesc) * p->nsys, cudaMemcpyHostToDevice, st), "upload sys");
    CK(p, cudaMemcpyAsync(w + p->o_poff, p->poff.data(), 8 * (p->nsys + 1), cudaMemcpyHostToDevice, st), "upload poff");
    CK(p, cudaMemcpyAsync(w + p->o_boff, p->boff.data(), 8 * (p->nsys + 1), cudaMemcpyHostToDevice, st), "upload boff");
    CK(p, cudaMemcpyAsync(w + p->o_coff, p->coff.data(), 8 * (p->nsys + 1), cudaMemcpyHostToDevice, st), "upload coff");
    CK(p, cudaMemcpyAsync(w + p->o_goff, p->goff.data(), 8 * (p->nsys + 1), cudaMemcpyHostToDevice, st), "upload goff");
    CK(p, cudaMemcpyAsync(w + p->o_toff, p->toff.data(), 8 * (p->nsys + 1), cudaMemcpyHostToDevice, st), "upload toff");
    CK(p, cudaMemcpyAsync(w + p->o_lvl, p->lvl.data(), 8 * p->lvl.size(), cudaMemcpyHostToDevice, st), "upload lvl");
    CK(p, cudaMemsetAsync(w + p->o_dyn, 0, sizeof(SysDyn) * p->nsys, st), "zero dyn");
    CK(p, cudaMemsetAsync(w + p->o_glob, 0, sizeof(Globals), st), "zero globals");
    {  // scan generations start at 1 over zeroed tile states
        const unsigned one[3] = {1u, 1u, 1u};
        CK(p, cudaMemcpyAsync(w + p->o_glob + offsetof(Globals, scan_gen), one, sizeof(one),
                              cudaMemcpyHostToDevice, st), "scan generations");
        CK(p, cudaMemsetAsync(w + p->o_sst, 0, p->sst_bytes, st), "zero scan states");
    }
    CK(p, cudaMemsetAsync(w + p->o_upcnt, 0, 4 * (size_t)p->up_total, st), "zero arrival counters");
    CK(p, cudaStreamSynchronize(st), "bind sync");
    p->has_tree = false;
    p->acc_stale = true;
    p->acc_valid = false;
    if (p->gexec) {
        cudaGraphExecDestroy(p->gexec);
        p->gexec = nullptr;
        p->gsteps = 0;
    }
    return BH_OK;
}

static int need_bound(bh_plan *p) {
    if (!p) return BH_ERR_INVALID;
    if (!p->ws) return fail(p, BH_ERR_WORKSPACE, "no workspace bound (call bh_bind)");
    return BH_OK;
}

extern "C" int bh_load(bh_plan *p, const double *x, const double *y, const double *m,
                       const double *vx, const double *vy, void *stream) {
    int r = need_bound(p);
    if (r) return r;
    if (p->n_total && (!x || !y || !m || !vx || !vy)) return fail(p, BH_ERR_INVALID, "null input array");
    CK(p, launch_load(p->dev, x, y, m, vx, vy, 0, (cudaStream_t)stream), "load");
    p->has_tree = false;
    p->acc_stale = true;
    p->acc_valid = false;
    return BH_OK;
}

extern "C" int bh_load_records(bh_plan *p, const double *rec, void *stream) {
    int r = need_bound(p);
    if (r) return r;
    if (p->n_total && !rec) return fail(p, BH_ERR_INVALID, "null records");
    CK(p, launch_load(p->dev, rec + 0, rec + 1, rec + 2, rec + 3, rec + 4, 10, (cudaStream_t)stream), "load records");
    p->has_tree = false;
    p->acc_stale = true;
    p->acc_valid = false;
    return BH_OK;
}

extern "C" int bh_store_records(bh_plan *p, double *rec, void *stream) {
    int r = need_bound(p);
    if (r) return r;
    if (p->n_total && !rec) return fail(p, BH_ERR_INVALID, "null records");
    CK(p, launch_store(p->dev, p->has_tree ? 1 : 0, p->acc_valid, rec, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                       (cudaStream_t)stream), "store records");
    return BH_OK;
}

extern "C" int bh_store(bh_plan *p, double *x, double *y, double *vx, double *vy, double *ax,
                        double *ay, void *stream) {
    int r = need_bound(p);
    if (r) return r;
    CK(p, launch_store(p->dev, p->has_tree ? 1 : 0, p->acc_valid, nullptr, x, y, vx, vy, ax, ay, (cudaStream_t)stream),
       "store");
    return BH_OK;
}

static int enqueue_tree(bh_plan *p, cudaStream_t st) {
    CK(p, launch_prologue(p->dev, st), "prologue");
    CK(p, launch_bbox(p->dev, st), "bbox");
    CK(p, launch_place(p->dev, st), "place");
    CK(p, launch_scan(p->dev, st), "scan");
    // the work items need the box scan only: they run beside the scatter
    CK(p, cudaEventRecord(p->fork_ev, st), "fork");
    CK(p, cudaStreamWaitEvent(p->side, p->fork_ev, 0), "fork wait");
    CK(p, launch_items(p->dev, p->side), "work items");
    CK(p, cudaEventRecord(p->join_ev, p->side), "join");
    CK(p, launch_scatter(p->dev, st), "scatter");  // (and the leaf sums)
    p->leaves_stale = false;
    CK(p, cudaStreamWaitEvent(st, p->join_ev, 0), "join wait");
    return BH_OK;
}

extern "C" int bh_create_tree(bh_plan *p, void *stream) {
    int r = need_bound(p);
    if (r) return r;
    r = enqueue_tree(p, (cudaStream_t)stream);
    if (r) return r;
    p->has_tree = true;
    p->acc_stale = true;
    return BH_OK;
}

extern "C" int bh_summarize(bh_plan *p, void *stream) {
    int r = need_bound(p);
    if (r) return r;
    if (!p->has_tree) return fail(p, BH_ERR_INVALID, "summarize before create_tree");
    CK(p, launch_summarize(p->dev, p->leaves_stale, (cudaStream_t)stream), "summarize");
    p->leaves_stale = false;
    return BH_OK;
}

extern "C" int bh_evaluate(bh_plan *p, void *stream) {
    int r = need_bound(p);
    if (r) return r;
    if (!p->has_tree) return fail(p, BH_ERR_INVALID, "evaluate before create_tree");
    if (p->dev.learned && !p->mlp_img) return fail(p, BH_ERR_INVALID, "BH_FLAG_LEARNED without bh_set_correction");
    CK(p, launch_force(p->dev, false, !p->acc_stale, (cudaStream_t)stream, p->timing ? p->tev : nullptr),
       "evaluate");
    if (p->timing) p->tev_recorded = true;
    if (p->dev.learned)
        CK(p, launch_learned_correct(p->dev, p->params.correction_theta, p->mlp_img, p->mlp_params,
                                     false, (cudaStream_t)stream), "learned correction");
    p->acc_stale = false;
    p->acc_valid = true;
    return BH_OK;
}

extern "C" int bh_timestep(bh_plan *p, void *stream) {
    int r = need_bound(p);
    if (r) return r;
    if (!p->acc_valid) {  // no evaluation since the load: the tick sees zero accelerations
        const size_t nb = 8 * (size_t)p->n_total;
        CK(p, cudaMemsetAsync(p->dev.AX, 0, nb, (cudaStream_t)stream), "zero accelerations");
        CK(p, cudaMemsetAsync(p->dev.AY, 0, nb, (cudaStream_t)stream), "zero accelerations");
    }
    CK(p, launch_tick(p->dev, (cudaStream_t)stream), "timestep");
    p->acc_stale = true;
    p->acc_valid = true;  // (zeroed by the tick)
    return BH_OK;
}

static int enqueue_steps(bh_plan *p, int nsteps, cudaStream_t st) {
    for (int k = 0; k < nsteps; k++) {
        int r = enqueue_tree(p, st);
        if (r) return r;
        CK(p, launch_summarize(p->dev, false, st), "summarize");
        if (p->dev.learned) {
            if (!p->mlp_img) return fail(p, BH_ERR_INVALID, "BH_FLAG_LEARNED without bh_set_correction");
            CK(p, launch_force(p->dev, false, false, st), "force");
            CK(p, launch_learned_correct(p->dev, p->params.correction_theta, p->mlp_img,
                                         p->mlp_params, true, st), "learned correction+tick");
        } else {
            CK(p, launch_force(p->dev, true, false, st), "force+tick");
        }
    }
    return BH_OK;
}

extern "C" int bh_step(bh_plan *p, int nsteps, void *stream) {
    int r = need_bound(p);
    if (r) return r;
    if (nsteps < 0) return fail(p, BH_ERR_INVALID, "nsteps < 0");
    r = enqueue_steps(p, nsteps, (cudaStream_t)stream);
    if (r) return r;
    if (nsteps > 0) {
        p->has_tree = true;
        p->acc_stale = true;
        p->acc_valid = true;
    }
    return BH_OK;
}

extern "C" int bh_step_graph(bh_plan *p, int nsteps, void *stream) {
    int r = need_bound(p);
    if (r) return r;
    if (nsteps < 0) return fail(p, BH_ERR_INVALID, "nsteps < 0");
    if (nsteps == 0) return BH_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (!p->gexec || p->gsteps != nsteps) {
        if (p->gexec) {
            cudaGraphExecDestroy(p->gexec);
            p->gexec = nullptr;
        }
        if (!p->gstream) CK(p, cudaStreamCreateWithFlags(&p->gstream, cudaStreamNonBlocking), "graph stream");
        cudaGraph_t g;
        CK(p, cudaStreamBeginCapture(p->gstream, cudaStreamCaptureModeThreadLocal), "begin capture");
        int er = enqueue_steps(p, nsteps, p->gstream);
        cudaError_t e = cudaStreamEndCapture(p->gstream, &g);
        if (er) return er;
        if (e != cudaSuccess) return cuda_fail(p, e, "end capture");
        size_t nn = 0;
        e = cudaGraphGetNodes(g, nullptr, &nn);
        if (e == cudaSuccess) {
            std::vector<cudaGraphNode_t> nodes(nn);
            e = cudaGraphGetNodes(g, nodes.data(), &nn);
            int nk = 0;
            for (size_t k = 0; e == cudaSuccess && k < nn; k++) {
                cudaGraphNodeType t;
                e = cudaGraphNodeGetType(nodes[k], &t);
                if (t == cudaGraphNodeTypeKernel) nk++;
            }
            p->gkernels = nk;
        }
        if (e != cudaSuccess) {
            cudaGraphDestroy(g);
            return cuda_fail(p, e, "graph nodes");
        }
        e = cudaGraphInstantiate(&p->gexec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_fail(p, e, "graph instantiate");
        p->gsteps = nsteps;
    }
    CK(p, cudaGraphLaunch(p->gexec, st), "graph launch");
    p->has_tree = true;
    p->acc_stale = true;
    p->acc_valid = true;
    return BH_OK;
}

extern "C" int bh_set_kernel_timing(bh_plan *p, int enable) {
    if (!p) return BH_ERR_INVALID;
    if (enable)
        for (cudaEvent_t &e : p->tev)
            if (!e) CK(p, cudaEventCreate(&e), "timing event");
    p->timing = enable != 0;
    p->tev_recorded = false;
    return BH_OK;
}

extern "C" int bh_force_kernel_ms(bh_plan *p, float *ms) {
    if (!p || !ms) return BH_ERR_INVALID;
    if (!p->tev_recorded) return fail(p, BH_ERR_INVALID, "no timed bh_evaluate since bh_set_kernel_timing");
    CK(p, cudaEventSynchronize(p->tev[1]), "timing sync");
    CK(p, cudaEventElapsedTime(ms, p->tev[0], p->tev[1]), "elapsed time");
    return BH_OK;
}

extern "C" int bh_kernels_per_step(const bh_plan *p, int *count) {
    if (!p || !count) return BH_ERR_INVALID;
    // prologue, box scan, summarize tiles; with particles also bbox (which finalises the box),
    // place, the scatter's four kernels (permutation, quadrant sort, long quadrants, gather with
    // the leaf sums), force (and before it, when streaming, the list build and the two kernels of
    // the heaviest-first item order); work items: count, scan, fill for the walk or the learned
    // correction, one kernel for list streaming
    const bool walk_items = !p->stream || (p->params.flags & BH_FLAG_LEARNED);
    // (a walking plan's tick is a kernel of its own: the walk reads the state the tick writes)
    *count = 1 + 1 + (walk_items ? 3 : 0) + 1 + (p->n_total > 0 ? 7 : 0) + (p->stream ? 1 : 0) +
             (p->stream && p->n_total > 0 ? 3 : 0) + (!p->stream && p->n_total > 0 ? 1 : 0);
    return BH_OK;
}

extern "C" int bh_graph_kernel_nodes(const bh_plan *p, int *count) {
    if (!p || !count) return BH_ERR_INVALID;
    if (p->gkernels < 0) return BH_ERR_INVALID;  // no step graph captured yet
    *count = p->gkernels;
    return BH_OK;
}

extern "C" int bh_error_flags(bh_plan *p, unsigned *flags, void *stream) {
    int r = need_bound(p);
    if (r) return r;
    if (!flags) return fail(p, BH_ERR_INVALID, "null flags");
    cudaStream_t st = (cudaStream_t)stream;
    Globals g;
    CK(p, cudaMemcpyAsync(&g, (char *)p->ws + p->o_glob, sizeof(g), cudaMemcpyDeviceToHost, st), "read flags");
    CK(p, cudaStreamSynchronize(st), "sync");
    CK(p, cudaMemsetAsync((char *)p->ws + p->o_glob + offsetof(Globals, err), 0, sizeof(unsigned), st), "clear flags");
    *flags = g.err;
    return g.err ? fail(p, BH_ERR_DEVICE, "device error flags 0x%x", g.err) : BH_OK;
}

extern "C" int bh_pair_counts(bh_plan *p, long long *near_pairs, long long *far_pairs, void *stream) {
    int r = need_bound(p);
    if (r) return r;
    cudaStream_t st = (cudaStream_t)stream;
    Globals g;
    CK(p, cudaMemcpyAsync(&g, (char *)p->ws + p->o_glob, sizeof(g), cudaMemcpyDeviceToHost, st), "read counts");
    CK(p, cudaStreamSynchronize(st), "sync");
    if (near_pairs) *near_pairs = (long long)g.near_pairs;
    if (far_pairs) *far_pairs = (long long)g.far_pairs;
    return BH_OK;
}

extern "C" int bh_corrected_pairs(bh_plan *p, long long *pairs, void *stream) {
    int r = need_bound(p);
    if (r) return r;
    if (!pairs) return fail(p, BH_ERR_INVALID, "null pairs");
    cudaStream_t st = (cudaStream_t)stream;
    Globals g;
    CK(p, cudaMemcpyAsync(&g, (char *)p->ws + p->o_glob, sizeof(g), cudaMemcpyDeviceToHost, st), "read counts");
    CK(p, cudaStreamSynchronize(st), "sync");
    *pairs = (long long)g.corr_pairs;
    return BH_OK;
}

extern "C" int bh_direct_sample(bh_plan *p, int sys, const long long *targets, long long nt,
                                double *ax, double *ay, void *stream) {
    int r = need_bound(p);
    if (r) return r;
    if (sys < 0 || sys >= p->nsys) return fail(p, BH_ERR_INVALID, "system %d out of range", sys);
    if (nt < 0 || (nt > 0 && (!targets || !ax || !ay))) return fail(p, BH_ERR_INVALID, "bad targets");
    CK(p, launch_direct(p->dev, sys, targets, nt, ax, ay, (cudaStream_t)stream), "direct sample");
    return BH_OK;
}

extern "C" int bh_set_grid(bh_plan *p, int sys, const double *ext, void *stream) {
    if (!p || sys < 0 || sys >= p->nsys) return BH_ERR_INVALID;
    SysDesc &d = p->sys[sys];
    if (ext) {
        if (!(ext[2] >= ext[0]) || !(ext[3] >= ext[1]) || !std::isfinite(ext[0]) || !std::isfinite(ext[1]) ||
            !std::isfinite(ext[2]) || !std::isfinite(ext[3]))
            return fail(p, BH_ERR_INVALID, "bh_set_grid: extents must be finite with max >= min");
        d.fixed_grid = 1;
        for (int k = 0; k < 4; k++) d.fg_ext[k] = ext[k];
    } else {
        d.fixed_grid = 0;
    }
    if (p->ws) {  // bound: update the device copy of the system table (graphs replay from it)
        CK(p, cudaMemcpyAsync((char *)p->ws + p->o_sys + sizeof(SysDesc) * sys, &d, sizeof(SysDesc),
                              cudaMemcpyHostToDevice, (cudaStream_t)stream), "upload grid");
        CK(p, cudaStreamSynchronize((cudaStream_t)stream), "sync");
    }
    return BH_OK;
}

extern "C" int bh_leaf_moments(bh_plan *p, int sys, double *out, void *stream) {
    int r = need_bound(p);
    if (r) return r;
    if (sys < 0 || sys >= p->nsys || !out) return fail(p, BH_ERR_INVALID, "bad leaf_moments args");
    if (!p->has_tree) return fail(p, BH_ERR_INVALID, "leaf_moments before create_tree/summarize");
    const SysDesc &d = p->sys[sys];
    CK(p, cudaMemcpyAsync(out, (char *)p->ws + p->o_mom + 48 * d.coff, 48 * (size_t)d.G * d.G,
                          cudaMemcpyDeviceToDevice, (cudaStream_t)stream), "copy leaf moments");
    return BH_OK;
}

extern "C" int bh_set_leaf_moments(bh_plan *p, int sys, const double *in, void *stream) {
    int r = need_bound(p);
    if (r) return r;
    if (sys < 0 || sys >= p->nsys || !in) return fail(p, BH_ERR_INVALID, "bad set_leaf_moments args");
    if (!p->has_tree) return fail(p, BH_ERR_INVALID, "set_leaf_moments before create_tree");
    const SysDesc &d = p->sys[sys];
    cudaStream_t st = (cudaStream_t)stream;
    CK(p, cudaMemcpyAsync((char *)p->ws + p->o_mom + 48 * d.coff, in, 48 * (size_t)d.G * d.G,
                          cudaMemcpyDeviceToDevice, st), "copy leaf moments");
    p->leaves_stale = true;  // a later bh_summarize sums the leaves from the particles again
    CK(p, launch_pyramid(p->dev, st), "pyramid");
    return BH_OK;
}

extern "C" int bh_box_moments(bh_plan *p, int sys, double *out, void *stream) {
    int r = need_bound(p);
    if (r) return r;
    if (sys < 0 || sys >= p->nsys || !out) return fail(p, BH_ERR_INVALID, "bad box_moments args");
    if (!p->has_tree) return fail(p, BH_ERR_INVALID, "box_moments before create_tree/summarize");
    CK(p, launch_box_com(p->dev, sys, out, (cudaStream_t)stream), "box moments");
    return BH_OK;
}

extern "C" int bh_grid_info(bh_plan *p, int sys, double *out, void *stream) {
    int r = need_bound(p);
    if (r) return r;
    if (sys < 0 || sys >= p->nsys || !out) return fail(p, BH_ERR_INVALID, "bad grid_info args");
    cudaStream_t st = (cudaStream_t)stream;
    SysDyn dy;
    CK(p, cudaMemcpyAsync(&dy, (char *)p->ws + p->o_dyn + sizeof(SysDyn) * sys, sizeof(dy),
                          cudaMemcpyDeviceToHost, st), "read grid info");
    CK(p, cudaStreamSynchronize(st), "sync");
    out[0] = dy.minx;
    out[1] = dy.miny;
    out[2] = dy.step;
    out[3] = (double)p->sys[sys].G;
    out[4] = (double)p->sys[sys].n;
    return BH_OK;
}

extern "C" int bh_diagnostics(bh_plan *p, int sys, int want_potential, double *out, void *stream) {
    int r = need_bound(p);
    if (r) return r;
    if (sys < 0 || sys >= p->nsys || !out) return fail(p, BH_ERR_INVALID, "bad diagnostics args");
    CK(p, launch_diag(p->dev, sys, want_potential, out, (cudaStream_t)stream), "diagnostics");
    return BH_OK;
}

// ------------------------------------------------------------ learned correction
static int mlp_ready() {
    static int state = 0;  // 0 unknown, 1 ready, 2 failed (idempotent attribute setting)
    if (state == 0) state = mlp_init() == cudaSuccess ? 1 : 2;
    return state == 1;
}

extern "C" int bh_mlp_param_count(void) { return MLP_PARAMS; }
extern "C" int bh_mlp_image_bytes(void) { return MLP_IMAGE_BYTES; }

extern "C" int bh_mlp_pack(const float *params, void *image, void *stream) {
    if (!params || !image) return BH_ERR_INVALID;
    if (((uintptr_t)image) & 15) return BH_ERR_INVALID;
    return mlp_pack(params, (uint8_t *)image, (cudaStream_t)stream) == cudaSuccess ? BH_OK : BH_ERR_CUDA;
}

extern "C" int bh_mlp_forward(const float *feats, int fs, long long rows, const void *image,
                              const float *params, float *out, unsigned *err, void *stream) {
    if (rows < 0 || fs < 6 || (rows > 0 && (!feats || !image || !params || !out || !err)))
        return BH_ERR_INVALID;
    if (((uintptr_t)image) & 15) return BH_ERR_INVALID;
    if (!mlp_ready()) return BH_ERR_CUDA;
    return mlp_infer(feats, fs, rows, (const uint8_t *)image, params, out, err,
                     (cudaStream_t)stream) == cudaSuccess ? BH_OK : BH_ERR_CUDA;
}

extern "C" int bh_mlp_train_batch(const float *feats, int fs, const float *targets, long long rows,
                                  const void *image, const float *params, float *grad, float *loss,
                                  unsigned *err, void *stream) {
    if (rows < 0 || fs < 6 ||
        (rows > 0 && (!feats || !targets || !image || !params || !grad || !loss || !err)))
        return BH_ERR_INVALID;
    if (((uintptr_t)image) & 15) return BH_ERR_INVALID;
    if (!mlp_ready()) return BH_ERR_CUDA;
    return mlp_train(feats, fs, targets, rows, (const uint8_t *)image, params, grad, loss, err,
                     (cudaStream_t)stream) == cudaSuccess ? BH_OK : BH_ERR_CUDA;
}

extern "C" int bh_mlp_adam(float *params, float *m, float *v, float *grad, int step, float lr,
                           void *stream) {
    if (!params || !m || !v || !grad || step < 1) return BH_ERR_INVALID;
    return mlp_adam(params, m, v, grad, step, lr, (cudaStream_t)stream) == cudaSuccess ? BH_OK
                                                                                     : BH_ERR_CUDA;
}

extern "C" int bh_set_correction(bh_plan *p, const void *image, const float *params) {
    if (!p) return BH_ERR_INVALID;
    if (!image || !params || (((uintptr_t)image) & 15)) return fail(p, BH_ERR_INVALID, "bad MLP buffers");
    p->mlp_img = (const uint8_t *)image;
    p->mlp_params = params;
    if (p->gexec) {  // a captured step must pick up the new buffers
        cudaGraphExecDestroy(p->gexec);
        p->gexec = nullptr;
        p->gsteps = 0;
    }
    return BH_OK;
}

extern "C" int bh_learned_pairs(bh_plan *p, double theta_hi, double theta_lo, int max_level,
                                long long item_offset, long long item_stride, int tpi, float *feats,
                                float *targets, unsigned *counter, long long capacity,
                                void *stream) {
    int r = need_bound(p);
    if (r) return r;
    if (!p->has_tree) return fail(p, BH_ERR_INVALID, "learned_pairs before create_tree/summarize");
    if (!(theta_hi > theta_lo) || !(theta_lo > 0.0) || item_stride < 1 || item_offset < 0 ||
        tpi < 1 || capacity < 0 || !feats || !targets || !counter)
        return fail(p, BH_ERR_INVALID, "bad learned_pairs arguments");
    // a plan without the learned correction builds neither the pyramid's second moments nor
    // (when streaming) the walk items in its step: rebuild the pyramid above the summed leaves
    // with them (the same centres of mass and masses)
    if (!p->dev.learned) CK(p, launch_pyramid(p->dev, (cudaStream_t)stream, true), "second moments");
    if (p->dev.stream && !p->dev.learned) CK(p, launch_walk_items(p->dev, (cudaStream_t)stream), "work items");
    CK(p, launch_learned_pairs(p->dev, theta_hi, theta_lo, max_level, item_offset, item_stride, tpi,
                               feats, targets, counter, capacity, (cudaStream_t)stream),
       "learned pairs");
    return BH_OK;
}

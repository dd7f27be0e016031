/*
 * bh_oracle.c -- CPU oracle for the 2D grid-decomposition Barnes-Hut step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the tests, the smoke
 * check and the CPU-baseline leg of bench.py call it; the product (the CUDA
 * library and its Python host layer) never links, loads or calls it.
 *
 * Parity is pinned: the reference CPU path (python-bh, run unmodified under a
 * numba stub) produced the golden vectors in tests/golden/ref_*.npz, and
 * tests/test_oracle_golden.py checks this file against every one of them.
 *
 * Contents
 *   1. oref_grid_dim      grid sizing      python-bh/barneshut/implementations/base.py:13,211-239,
 *                                          python-bh/barneshut/kernels/helpers/grid.py:5-8
 *   2. oref_bbox          square bbox      kernels/helpers/grid.py:10-26, base.py:233-239
 *   3. oref_keys          box keys         implementations/sequential.py:32-34
 *   4. oref_reference_evaluate
 *                         the reference CPU evaluation, same loop and
 *                         accumulation order:
 *                           sort            implementations/sequential.py:37-52
 *                           COM             internals/cloud.py:9-17,93-104
 *                           com_concat_dedup kernels/grid_decomposition/sequential/evaluation.py:73-109
 *                           neighbours      kernels/helpers/grid.py:28-48
 *                           pair kernels    kernels/gravity/cpu_numba.py:30-92 (r^2 <= 1e-5 -> 0)
 *   5. oref_tick          kick-drift tick  kernels/grid_decomposition/gpu/grid.py:159-174
 *                         (the reference CPU tick never runs: grid_decomposition/box.py:26-30)
 *   6. oref_direct        FP64 direct sum  implementations/base.py:16-32 (optionally softened)
 *   7. oref_moments / oref_theta_evaluate
 *                         FP64 restatement of this project's opening-angle
 *                         (theta) far field.  It has no reference counterpart
 *                         (the only related reference item is the unused
 *                         `theta` key, configs/pykokkos.ini:11).  The cell
 *                         acceptance test is evaluated in float exactly as the
 *                         CUDA kernel evaluates it, so both sides build the same
 *                         interaction lists; the pair arithmetic here is FP64.
 *   8. oref_gpu_evaluate  the reference GPU evaluation (flat far field over every
 *                         box, no cutoff): kernels/grid_decomposition/gpu/grid.py:15-268
 *
 * Build: gcc -O2 -fopenmp -ffp-contract=off -fPIC -shared (no FMA contraction:
 * the reference is plain IEEE double arithmetic).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define REF_EPS 1e-5 /* cpu_numba.py:36,59,81 */

/* ------------------------------------------------------------------ 1 -- */
int oref_grid_dim(long long n, int ppb)
{
    /* base.py:223-231: nleaves = n / (0.7 * ppb) (or 1 when ppb == 1),
     * next_perfect_square (helpers/grid.py:5-8), G = int(sqrt(nleaves)). */
    double nleaves;
    if (ppb == 1)
        nleaves = 1.0;
    else
        nleaves = (double)n / (0.7 * (double)ppb);
    double r = sqrt(nleaves);
    if (fmod(nleaves, r) != 0.0 || r == 0.0) {
        double c = ceil(r);
        nleaves = c * c;
    }
    return (int)sqrt(nleaves);
}

/* ------------------------------------------------------------------ 2 -- */
void oref_bbox(long long n, const double *x, const double *y, int G, double *out)
{
    /* out = {min_x, min_y, max_x, max_y, step} after squaring the box. */
    double mnx = x[0], mny = y[0], mxx = x[0], mxy = y[0];
    for (long long i = 1; i < n; i++) {
        if (x[i] < mnx) mnx = x[i];
        if (x[i] > mxx) mxx = x[i];
        if (y[i] < mny) mny = y[i];
        if (y[i] > mxy) mxy = y[i];
    }
    double xe = mxx - mnx, ye = mxy - mny;
    if (xe > ye)
        mxy += (xe - ye);
    else if (ye > xe)
        mxx += (ye - xe);
    out[0] = mnx;
    out[1] = mny;
    out[2] = mxx;
    out[3] = mxy;
    out[4] = (mxx - mnx) / (double)G;
}

/* ------------------------------------------------------------------ 3 -- */
static inline int ref_key1(double p, double mn, double step, int G)
{
    double k = floor((p - mn) / step);
    if (k < 0.0) k = 0.0;
    if (k > (double)(G - 1)) k = (double)(G - 1);
    return (int)k;
}

void oref_keys(long long n, const double *x, const double *y, int G, const double *bb,
               int *kx, int *ky)
{
    for (long long i = 0; i < n; i++) {
        kx[i] = ref_key1(x[i], bb[0], bb[4], G);
        ky[i] = ref_key1(y[i], bb[1], bb[4], G);
    }
}

/* ------------------------------------------------------------------ 4 -- */
typedef struct {
    double gx, gy, px, py, m, vx, vy, ax, ay, pid;
} rrec;

static int cmp_rrec(const void *pa, const void *pb)
{
    /* numpy structured sort with order=[gx, gy]: ties are broken by the
     * remaining fields in field order (px, py, mass, vx, vy, ax, ay, pid). */
    const double *a = (const double *)pa, *b = (const double *)pb;
    for (int k = 0; k < 10; k++) {
        if (a[k] < b[k]) return -1;
        if (a[k] > b[k]) return 1;
    }
    return 0;
}

static inline void ref_pair_fk(double dx0, double dx1, double G, double *f0, double *f1)
{
    /* cpu_numba.py: distSqr = 0.; distSqr += dx[k]**2; fk = G*dx[k]*distSqr**-1
     * if distSqr > eps else 0 */
    double d2 = 0.0;
    d2 = d2 + dx0 * dx0;
    d2 = d2 + dx1 * dx1;
    if (d2 > REF_EPS) {
        double inv = pow(d2, -1.0);
        *f0 = (G * dx0) * inv;
        *f1 = (G * dx1) * inv;
    } else {
        *f0 = 0.0;
        *f1 = 0.0;
    }
}

/*
 * One reference evaluation.  Inputs in particle (pid) order.  Outputs:
 * ax/ay (pid order), kx/ky (pid order), coms[G*G*3] (cx, cy, M; zeros for an
 * empty box), bb[5] (see oref_bbox).  G <= 0 derives G from ppb.  Returns G.
 */
int oref_reference_evaluate(long long n, const double *x, const double *y, const double *m,
                            const double *vx, const double *vy, int G, int ppb, double gconst,
                            double *ax, double *ay, int *kx, int *ky, double *coms, double *bb)
{
    if (n <= 0) return 0;
    if (G <= 0) G = oref_grid_dim(n, ppb);
    oref_bbox(n, x, y, G, bb);
    rrec *r = (rrec *)malloc(sizeof(rrec) * (size_t)n);
    for (long long i = 0; i < n; i++) {
        r[i].gx = (double)ref_key1(x[i], bb[0], bb[4], G);
        r[i].gy = (double)ref_key1(y[i], bb[1], bb[4], G);
        r[i].px = x[i];
        r[i].py = y[i];
        r[i].m = m[i];
        r[i].vx = vx[i];
        r[i].vy = vy[i];
        r[i].ax = 0.0;
        r[i].ay = 0.0;
        r[i].pid = (double)i;
    }
    qsort(r, (size_t)n, sizeof(rrec), cmp_rrec);
    long long B = (long long)G * G;
    long long *start = (long long *)calloc((size_t)B + 1, sizeof(long long));
    long long *cnt = (long long *)calloc((size_t)B, sizeof(long long));
    for (long long i = 0; i < n; i++) cnt[(long long)r[i].gx * G + (long long)r[i].gy]++;
    for (long long b = 0; b < B; b++) start[b + 1] = start[b] + cnt[b];
    /* COMs: cloud.py:9-17 */
    for (long long b = 0; b < B; b++) {
        double M = 0.0, sx = 0.0, sy = 0.0;
        if (cnt[b] == 0) {
            coms[3 * b] = coms[3 * b + 1] = coms[3 * b + 2] = 0.0;
            continue;
        }
        for (long long i = start[b]; i < start[b + 1]; i++) {
            double mass = r[i].m;
            sx += r[i].px * mass;
            sy += r[i].py * mass;
            M += mass;
        }
        coms[3 * b] = sx / M;
        coms[3 * b + 1] = sy / M;
        coms[3 * b + 2] = M;
    }
    long long maxc = 1;
    for (long long b = 0; b < B; b++)
        if (cnt[b] > maxc) maxc = cnt[b];
    double *f1 = (double *)malloc(sizeof(double) * 2 * (size_t)(maxc > B ? maxc : B));
    double *f2 = (double *)malloc(sizeof(double) * 2 * (size_t)maxc);
    int *nb = (int *)malloc(sizeof(int) * 8 * 2);
    long long *coml = (long long *)malloc(sizeof(long long) * (size_t)B);

    for (int bx = 0; bx < G; bx++) {
        for (int by = 0; by < G; by++) {
            long long b = (long long)bx * G + by;
            if (cnt[b] == 0) continue;
            long long s0 = start[b], na = cnt[b];
            /* get_neighbor_cells (helpers/grid.py:28-37) */
            int xs = bx > 0 ? bx - 1 : bx, xe = bx < G - 1 ? bx + 1 : bx;
            int ys = by > 0 ? by - 1 : by, ye = by < G - 1 ? by + 1 : by;
            int nnb = 0;
            for (int i = xs; i <= xe; i++)
                for (int j = ys; j <= ye; j++)
                    if (!(i == bx && j == by)) {
                        nb[2 * nnb] = i;
                        nb[2 * nnb + 1] = j;
                        nnb++;
                    }
            /* COM list of every other non-empty, non-neighbour box */
            long long ncom = 0;
            for (int i = 0; i < G; i++)
                for (int j = 0; j < G; j++) {
                    long long c = (long long)i * G + j;
                    if (cnt[c] == 0 || c == b) continue;
                    int isnb = 0;
                    for (int k = 0; k < nnb; k++)
                        if (nb[2 * k] == i && nb[2 * k + 1] == j) isnb = 1;
                    if (!isnb) coml[ncom++] = c;
                }
            if (ncom) {
                /* self_other_numba_1 (cpu_numba.py:72-92) */
                for (long long j = 0; j < na; j++) f1[2 * j] = f1[2 * j + 1] = 0.0;
                for (long long ii = 0; ii < ncom; ii++) {
                    const double *c = coms + 3 * coml[ii];
                    for (long long j = 0; j < na; j++) {
                        double fa, fb;
                        ref_pair_fk(r[s0 + j].px - c[0], r[s0 + j].py - c[1], gconst, &fa, &fb);
                        f1[2 * j] = f1[2 * j] - fa * c[2];
                        f1[2 * j + 1] = f1[2 * j + 1] - fb * c[2];
                    }
                }
                for (long long j = 0; j < na; j++) {
                    r[s0 + j].ax = r[s0 + j].ax + f1[2 * j];
                    r[s0 + j].ay = r[s0 + j].ay + f1[2 * j + 1];
                }
            }
            /* remove_bottom_left_neighbors (helpers/grid.py:39-48), then the
             * mutual update self_other_numba_2 (cpu_numba.py:49-70) */
            for (int k = 0; k < nnb; k++) {
                int i2 = nb[2 * k], j2 = nb[2 * k + 1];
                if ((i2 == bx - 1 && j2 == by - 1) || (i2 == bx - 1 && j2 == by) ||
                    (i2 == bx && j2 == by - 1) || (i2 == bx + 1 && j2 == by - 1))
                    continue;
                long long c = (long long)i2 * G + j2;
                if (cnt[c] == 0) continue;
                long long t0 = start[c], nbb = cnt[c];
                for (long long j = 0; j < na; j++) f1[2 * j] = f1[2 * j + 1] = 0.0;
                for (long long i = 0; i < nbb; i++) f2[2 * i] = f2[2 * i + 1] = 0.0;
                for (long long i = 0; i < nbb; i++) {
                    for (long long j = 0; j < na; j++) {
                        double fa, fb;
                        ref_pair_fk(r[s0 + j].px - r[t0 + i].px, r[s0 + j].py - r[t0 + i].py,
                                    gconst, &fa, &fb);
                        f1[2 * j] = f1[2 * j] - fa * r[t0 + i].m;
                        f2[2 * i] = f2[2 * i] + fa * r[s0 + j].m;
                        f1[2 * j + 1] = f1[2 * j + 1] - fb * r[t0 + i].m;
                        f2[2 * i + 1] = f2[2 * i + 1] + fb * r[s0 + j].m;
                    }
                }
                for (long long j = 0; j < na; j++) {
                    r[s0 + j].ax = r[s0 + j].ax + f1[2 * j];
                    r[s0 + j].ay = r[s0 + j].ay + f1[2 * j + 1];
                }
                for (long long i = 0; i < nbb; i++) {
                    r[t0 + i].ax = r[t0 + i].ax + f2[2 * i];
                    r[t0 + i].ay = r[t0 + i].ay + f2[2 * i + 1];
                }
            }
            /* self_self_numba (cpu_numba.py:30-47) */
            for (long long j = 0; j < na; j++) f1[2 * j] = f1[2 * j + 1] = 0.0;
            for (long long i = 0; i < na; i++) {
                for (long long j = i + 1; j < na; j++) {
                    double fa, fb;
                    ref_pair_fk(r[s0 + j].px - r[s0 + i].px, r[s0 + j].py - r[s0 + i].py, gconst,
                                &fa, &fb);
                    f1[2 * i] = f1[2 * i] + fa * r[s0 + j].m;
                    f1[2 * j] = f1[2 * j] - fa * r[s0 + i].m;
                    f1[2 * i + 1] = f1[2 * i + 1] + fb * r[s0 + j].m;
                    f1[2 * j + 1] = f1[2 * j + 1] - fb * r[s0 + i].m;
                }
            }
            for (long long j = 0; j < na; j++) {
                r[s0 + j].ax = r[s0 + j].ax + f1[2 * j];
                r[s0 + j].ay = r[s0 + j].ay + f1[2 * j + 1];
            }
        }
    }
    for (long long i = 0; i < n; i++) {
        long long p = (long long)r[i].pid;
        ax[p] = r[i].ax;
        ay[p] = r[i].ay;
        kx[p] = (int)r[i].gx;
        ky[p] = (int)r[i].gy;
    }
    free(r);
    free(start);
    free(cnt);
    free(f1);
    free(f2);
    free(nb);
    free(coml);
    return G;
}

/*
 * Timed, bounded sample of one reference CPU step on a large system (the CPU
 * baseline).  Runs the O(N) phases in full (bounding box, keys, the sort by
 * (gx, gy, px, ...), per-box COM) and the com_concat_dedup evaluation for
 * `nsample` non-empty target boxes drawn with a fixed stride (starting at `offset` within the
 * stride, so successive calls with offsets 0, 1, 2, ... sample disjoint boxes), with OpenMP over
 * the sampled boxes.  Each sampled box does the reference's work: build its
 * COM list over all boxes, the far field against it, the four dedup
 * neighbours with mutual update, and the self interaction.
 * out[0] = seconds of the O(N) phases, out[1] = seconds of the sampled
 * evaluation, out[2] = non-empty boxes, out[3] = boxes sampled,
 * out[4] = estimated seconds per step = out[0] + out[1] * out[2] / out[3].
 */
static double wall_seconds(void)
{
#ifdef _OPENMP
    return omp_get_wtime();
#else
    return (double)clock() / CLOCKS_PER_SEC;
#endif
}

void oref_reference_sample_time(long long n, const double *x, const double *y, const double *m,
                                int G, long long nsample, long long offset, int nthreads, double *out)
{
    double t0 = wall_seconds();
    double bb[5];
    oref_bbox(n, x, y, G, bb);
    rrec *r = (rrec *)malloc(sizeof(rrec) * (size_t)n);
    for (long long i = 0; i < n; i++) {
        r[i].gx = (double)ref_key1(x[i], bb[0], bb[4], G);
        r[i].gy = (double)ref_key1(y[i], bb[1], bb[4], G);
        r[i].px = x[i];
        r[i].py = y[i];
        r[i].m = m[i];
        r[i].vx = r[i].vy = r[i].ax = r[i].ay = 0.0;
        r[i].pid = (double)i;
    }
    qsort(r, (size_t)n, sizeof(rrec), cmp_rrec);
    long long B = (long long)G * G;
    long long *start = (long long *)calloc((size_t)B + 1, sizeof(long long));
    for (long long i = 0; i < n; i++) start[(long long)r[i].gx * G + (long long)r[i].gy + 1]++;
    for (long long b = 0; b < B; b++) start[b + 1] += start[b];
    double *coms = (double *)calloc(3 * (size_t)B, sizeof(double));
    long long nonempty = 0;
    for (long long b = 0; b < B; b++) {
        if (start[b + 1] == start[b]) continue;
        nonempty++;
        double M = 0.0, sx = 0.0, sy = 0.0;
        for (long long i = start[b]; i < start[b + 1]; i++) {
            sx += r[i].px * r[i].m;
            sy += r[i].py * r[i].m;
            M += r[i].m;
        }
        coms[3 * b] = sx / M;
        coms[3 * b + 1] = sy / M;
        coms[3 * b + 2] = M;
    }
    long long *ne = (long long *)malloc(sizeof(long long) * (size_t)(nonempty ? nonempty : 1));
    long long k = 0;
    for (long long b = 0; b < B; b++)
        if (start[b + 1] > start[b]) ne[k++] = b;
    double t1 = wall_seconds();
    if (nsample > nonempty) nsample = nonempty;
    long long strd = nsample ? nonempty / nsample : 1;
    double sink = 0.0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : sink)
#endif
    for (long long q = 0; q < nsample; q++) {
        long long b = ne[(q * strd + (strd > 1 ? offset % strd : 0)) % (nonempty ? nonempty : 1)];
        int bx = (int)(b / G), by = (int)(b % G);
        long long s0 = start[b], na = start[b + 1] - s0;
        double *f1 = (double *)calloc(2 * (size_t)na, sizeof(double));
        long long *coml = (long long *)malloc(sizeof(long long) * (size_t)B);
        long long ncom = 0;
        for (int i = 0; i < G; i++)
            for (int j = 0; j < G; j++) {
                long long c = (long long)i * G + j;
                if (start[c + 1] == start[c] || c == b) continue;
                if (abs(i - bx) <= 1 && abs(j - by) <= 1) continue;
                coml[ncom++] = c;
            }
        for (long long ii = 0; ii < ncom; ii++) {
            const double *c = coms + 3 * coml[ii];
            for (long long j = 0; j < na; j++) {
                double fa, fb;
                ref_pair_fk(r[s0 + j].px - c[0], r[s0 + j].py - c[1], 1.0, &fa, &fb);
                f1[2 * j] -= fa * c[2];
                f1[2 * j + 1] -= fb * c[2];
            }
        }
        const int nbx[4] = {1, -1, 0, 1}, nby[4] = {0, 1, 1, 1};
        for (int t = 0; t < 4; t++) {
            int i2 = bx + nbx[t], j2 = by + nby[t];
            if (i2 < 0 || i2 >= G || j2 < 0 || j2 >= G) continue;
            long long c = (long long)i2 * G + j2, t0 = start[c], nbb = start[c + 1] - t0;
            for (long long i = 0; i < nbb; i++)
                for (long long j = 0; j < na; j++) {
                    double fa, fb;
                    ref_pair_fk(r[s0 + j].px - r[t0 + i].px, r[s0 + j].py - r[t0 + i].py, 1.0, &fa, &fb);
                    f1[2 * j] -= fa * r[t0 + i].m;
                    f1[2 * j + 1] -= fb * r[t0 + i].m;
                    sink += fa * r[s0 + j].m + fb;
                }
        }
        for (long long i = 0; i < na; i++)
            for (long long j = i + 1; j < na; j++) {
                double fa, fb;
                ref_pair_fk(r[s0 + j].px - r[s0 + i].px, r[s0 + j].py - r[s0 + i].py, 1.0, &fa, &fb);
                f1[2 * i] += fa * r[s0 + j].m;
                f1[2 * j] -= fa * r[s0 + i].m;
            }
        for (long long j = 0; j < na; j++) sink += f1[2 * j] + f1[2 * j + 1];
        free(f1);
        free(coml);
    }
    double t2 = wall_seconds();
    out[0] = t1 - t0;
    out[1] = t2 - t1;
    out[2] = (double)nonempty;
    out[3] = (double)nsample;
    out[4] = out[0] + (nsample ? out[1] * (double)nonempty / (double)nsample : 0.0);
    out[5] = sink;
    free(r);
    free(start);
    free(coms);
    free(ne);
}

/* ------------------------------------------------------------------ 5 -- */
void oref_tick(long long n, double *x, double *y, double *vx, double *vy, const double *ax,
               const double *ay, double dt)
{
    for (long long i = 0; i < n; i++) {
        vx[i] = vx[i] + ax[i] * dt;
        vy[i] = vy[i] + ay[i] * dt;
        x[i] = x[i] + vx[i] * dt;
        y[i] = y[i] + vy[i] * dt;
    }
}

/* Multi-step reference run: per step evaluate + restated tick.  State is
 * updated in place (pid order); ax/ay hold the last step's accelerations. */
int oref_reference_run(long long n, double *x, double *y, const double *m, double *vx,
                       double *vy, int G, int ppb, double gconst, double dt, int nsteps,
                       double *ax, double *ay)
{
    int *kx = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    int *ky = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    int Gd = G > 0 ? G : oref_grid_dim(n, ppb);
    double *coms = (double *)malloc(sizeof(double) * 3 * (size_t)Gd * (size_t)Gd);
    double bb[5];
    for (int s = 0; s < nsteps; s++) {
        oref_reference_evaluate(n, x, y, m, vx, vy, Gd, ppb, gconst, ax, ay, kx, ky, coms, bb);
        oref_tick(n, x, y, vx, vy, ax, ay, dt);
    }
    free(kx);
    free(ky);
    free(coms);
    return Gd;
}

/* ------------------------------------------------------------------ 6 -- */
/* a_t = G sum_{j != t, r^2 > cutoff} m_j (x_j - x_t) / (r^2 + eps2).  With
 * cutoff < 0 only j == t is skipped (base.py:16-32, no cutoff). */
void oref_direct(long long n, const double *x, const double *y, const double *m, double gconst,
                 double eps2, double cutoff, long long nt, const long long *targets, double *ax,
                 double *ay, int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (long long k = 0; k < nt; k++) {
        long long t = targets ? targets[k] : k;
        double xt = x[t], yt = y[t], sx = 0.0, sy = 0.0;
        for (long long j = 0; j < n; j++) {
            if (j == t) continue;
            double dx = x[j] - xt, dy = y[j] - yt;
            double r2 = dx * dx + dy * dy;
            if (cutoff >= 0.0 && !(r2 > cutoff)) continue;
            double w = m[j] / (r2 + eps2);
            sx += w * dx;
            sy += w * dy;
        }
        ax[k] = gconst * sx;
        ay[k] = gconst * sy;
    }
}

/* Direct FP64 potential energy: sum_{i<j} G m_i m_j * 0.5*ln(r^2 + eps2). */
double oref_potential(long long n, const double *x, const double *y, const double *m,
                      double gconst, double eps2, int nthreads)
{
    double tot = 0.0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : tot)
#endif
    for (long long i = 0; i < n; i++) {
        double s = 0.0;
        for (long long j = i + 1; j < n; j++) {
            double dx = x[j] - x[i], dy = y[j] - y[i];
            s += m[j] * 0.5 * log(dx * dx + dy * dy + eps2);
        }
        tot += m[i] * s;
    }
    return gconst * tot;
}

/* ------------------------------------------------------------------ 7 -- */
/*
 * Cell pyramid.  Level 0 is the G x G leaf grid; level l has
 * G_l = ceil(G_{l-1} / 2) cells per side; the top level has one cell.  Cell
 * (l, i, j) covers leaves [i 2^l, (i+1) 2^l) x [j 2^l, (j+1) 2^l) clipped to
 * the grid and has origin (min_x + (i 2^l) step, min_y + (j 2^l) step).
 * Moments (FP64) are relative to the cell origin: M, Sx, Sy, Sxx, Sxy, Syy.
 * Cells are stored level by level, column-major in i (index i*G_l + j).
 */
int oref_num_levels(int G)
{
    int L = 0, g = G;
    while (g > 1) {
        g = (g + 1) / 2;
        L++;
    }
    return L + 1;
}

long long oref_pyramid_cells(int G)
{
    long long tot = 0;
    int g = G;
    for (;;) {
        tot += (long long)g * g;
        if (g == 1) break;
        g = (g + 1) / 2;
    }
    return tot;
}

static void shift_moments(const double *c, double dx, double dy, double *p)
{
    double M = c[0], Sx = c[1], Sy = c[2];
    p[0] += M;
    p[1] += Sx + M * dx;
    p[2] += Sy + M * dy;
    p[3] += c[3] + 2.0 * dx * Sx + M * dx * dx;
    p[4] += c[4] + dx * Sy + dy * Sx + M * dx * dy;
    p[5] += c[5] + 2.0 * dy * Sy + M * dy * dy;
}

/*
 * Leaf moments + pyramid.  kx/ky: box keys per particle (pid order), bb from
 * oref_bbox.  mom: pyramid_cells*6 doubles.  rec: pyramid_cells*4 floats
 * {cx_off, cy_off, M, 0} where cx_off = (float)(Sx/M) is the centre of mass
 * relative to the cell origin (zeros for an empty cell).
 */
static void build_pyramid(int G, double step, double *mom, float *rec);

void oref_moments(long long n, const double *x, const double *y, const double *m, int G,
                  const double *bb, const int *kx, const int *ky, double *mom, float *rec)
{
    long long ncell = oref_pyramid_cells(G);
    memset(mom, 0, sizeof(double) * 6 * (size_t)ncell);
    double step = bb[4];
    for (long long i = 0; i < n; i++) {
        long long b = (long long)kx[i] * G + ky[i];
        double ox = bb[0] + (double)kx[i] * step, oy = bb[1] + (double)ky[i] * step;
        double dx = x[i] - ox, dy = y[i] - oy, mm = m[i];
        double *q = mom + 6 * b;
        q[0] += mm;
        q[1] += mm * dx;
        q[2] += mm * dy;
        q[3] += mm * dx * dx;
        q[4] += mm * dx * dy;
        q[5] += mm * dy * dy;
    }
    build_pyramid(G, step, mom, rec);
}

/* Levels above the leaves (each cell the sum of its up to four children, shifted to its origin)
 * and the float records, from the leaf moments in mom[0 .. G*G*6). */
static void build_pyramid(int G, double step, double *mom, float *rec)
{
    long long ncell = oref_pyramid_cells(G);
    memset(mom + 6 * (size_t)G * (size_t)G, 0, sizeof(double) * 6 * (size_t)(ncell - (long long)G * G));
    long long off = 0, poff;
    int g = G, l = 0;
    while (g > 1) {
        int gp = (g + 1) / 2;
        poff = off + (long long)g * g;
        for (int i = 0; i < gp; i++)
            for (int j = 0; j < gp; j++) {
                double *p = mom + 6 * (poff + (long long)i * gp + j);
                for (int a = 0; a < 2; a++)
                    for (int c = 0; c < 2; c++) {
                        int ci = 2 * i + a, cj = 2 * j + c;
                        if (ci >= g || cj >= g) continue;
                        double dxs = (double)(a << l) * step, dys = (double)(c << l) * step;
                        shift_moments(mom + 6 * (off + (long long)ci * g + cj), dxs, dys, p);
                    }
            }
        off = poff;
        g = gp;
        l++;
    }
    for (long long c = 0; c < ncell; c++) {
        double *q = mom + 6 * c;
        if (q[0] > 0.0) {
            rec[4 * c] = (float)(q[1] / q[0]);
            rec[4 * c + 1] = (float)(q[2] / q[0]);
            rec[4 * c + 2] = (float)q[0];
        } else {
            rec[4 * c] = rec[4 * c + 1] = rec[4 * c + 2] = 0.0f;
        }
        rec[4 * c + 3] = 0.0f;
    }
}

/*
 * Opening-angle evaluation, FP64 pair arithmetic.  Target groups are TG x TG
 * leaf boxes (TG a power of two).  For every group the pyramid is walked from
 * the top; a non-empty cell that does not overlap the group is accepted as a
 * monopole when (2^l step)^2 < theta^2 d^2, d the distance from the group's
 * square [0, TG step]^2 to the cell's centre of mass; the test is evaluated
 * in float with the same operation order as the CUDA kernel.  Rejected leaf
 * boxes are summed particle by particle.  theta <= 0 selects the flat mode of
 * the reference (TG must be 1): the 3x3 neighbourhood directly, every other
 * non-empty leaf box as a monopole.  Pairs whose unsoftened r^2 <= cutoff are
 * skipped (cutoff = 1e-5 reproduces cpu_numba.py; 0 skips coincident points).
 * Output ax/ay in pid order.  counts[0..1] = near / far pair interactions.
 * mask (optional, one byte per particle): forces are computed only for targets whose byte is
 * non-zero (the others keep their ax/ay); the pair counts always cover every target.
 */
/*
 * dense_min > 0 (theta mode): the targets of a box holding at least dense_min particles use
 * per-box lists refined from their group's lists -- a near leaf whose centre of mass passes the
 * opening test against the single box (same float arithmetic as the CUDA list-streaming kernel:
 * offsets in the group frame, then relative to the box origin) becomes a far entry for those
 * targets.  quad_min > 0: a box holding at least quad_min particles is refined quadrant by
 * quadrant instead (the test against the quarter of the box that holds the target; a particle's
 * quadrant is the low bit of its FP64 key at twice the box resolution).  dense_min <= 0 and
 * quad_min <= 0 keep the group lists for every target (the walking force kernel).
 */
static int theta_eval_core(long long n, const double *x, const double *y, const double *m, int G,
                           int TG, double theta, double eps2, double cutoff, double gconst,
                           double *ax, double *ay, long long *counts, int nthreads, int dense_min,
                           int quad_min, const unsigned char *mask, const double *bb_in,
                           const double *leaf_in);

int oref_theta_evaluate(long long n, const double *x, const double *y, const double *m, int G,
                        int TG, double theta, double eps2, double cutoff, double gconst,
                        double *ax, double *ay, long long *counts, int nthreads, int dense_min,
                        int quad_min, const unsigned char *mask)
{
    return theta_eval_core(n, x, y, m, G, TG, theta, eps2, cutoff, gconst, ax, ay, counts, nthreads,
                           dense_min, quad_min, mask, NULL, NULL);
}

/*
 * The same evaluation on a part of a system (one rank's slab of boxes plus the halo boxes its
 * near field reaches), with the grid and the far field of the whole system given: bb_in[5] the
 * whole system's square box (oref_bbox layout) and leaf_in[G*G*6] its leaf moments (M, Sx, Sy,
 * Sxx, Sxy, Syy about each box origin).  Pass the targets to evaluate in mask; the particles
 * present must include every near box of those targets.  Pair counts cover the masked targets
 * only.
 */
int oref_theta_evaluate_part(long long n, const double *x, const double *y, const double *m, int G,
                             int TG, double theta, double eps2, double cutoff, double gconst,
                             double *ax, double *ay, long long *counts, int nthreads, int dense_min,
                             int quad_min, const unsigned char *mask, const double *bb_in,
                             const double *leaf_in)
{
    return theta_eval_core(n, x, y, m, G, TG, theta, eps2, cutoff, gconst, ax, ay, counts, nthreads,
                           dense_min, quad_min, mask, bb_in, leaf_in);
}

/* Leaf moments of boxes (M, Sx, Sy, Sxx, Sxy, Syy about each box origin, FP64, particles summed
 * in index order) of the given particles on the grid bb (oref_bbox layout).  out[G*G*6]. */
void oref_leaf_moments(long long n, const double *x, const double *y, const double *m, int G,
                       const double *bb, double *out)
{
    memset(out, 0, sizeof(double) * 6 * (size_t)G * (size_t)G);
    for (long long i = 0; i < n; i++) {
        int kx = ref_key1(x[i], bb[0], bb[4], G), ky = ref_key1(y[i], bb[1], bb[4], G);
        double ox = bb[0] + (double)kx * bb[4], oy = bb[1] + (double)ky * bb[4];
        double dx = x[i] - ox, dy = y[i] - oy, mm = m[i];
        double *q = out + 6 * ((long long)kx * G + ky);
        q[0] += mm;
        q[1] += mm * dx;
        q[2] += mm * dy;
        q[3] += mm * dx * dx;
        q[4] += mm * dx * dy;
        q[5] += mm * dy * dy;
    }
}

static int theta_eval_core(long long n, const double *x, const double *y, const double *m, int G,
                           int TG, double theta, double eps2, double cutoff, double gconst,
                           double *ax, double *ay, long long *counts, int nthreads, int dense_min,
                           int quad_min, const unsigned char *mask, const double *bb_in,
                           const double *leaf_in)
{
    if (n <= 0) return 0;
    double bb[5];
    if (bb_in)
        memcpy(bb, bb_in, sizeof(bb));
    else
        oref_bbox(n, x, y, G, bb);
    int *kx = (int *)malloc(sizeof(int) * (size_t)n), *ky = (int *)malloc(sizeof(int) * (size_t)n);
    oref_keys(n, x, y, G, bb, kx, ky);
    /* quadrant of each particle within its box: the low bits of the keys at twice the box
     * resolution, clip(floor(2 (p - min) / step), 0, 2 G - 1) (x half * 2 + y half) */
    int *quad = (int *)malloc(sizeof(int) * (size_t)n);
    for (long long i = 0; i < n; i++) {
        double k2x = floor(2.0 * ((x[i] - bb[0]) / bb[4])), k2y = floor(2.0 * ((y[i] - bb[1]) / bb[4]));
        if (k2x < 0.0) k2x = 0.0;
        if (k2x > 2.0 * G - 1.0) k2x = 2.0 * G - 1.0;
        if (k2y < 0.0) k2y = 0.0;
        if (k2y > 2.0 * G - 1.0) k2y = 2.0 * G - 1.0;
        quad[i] = ((int)k2x & 1) * 2 + ((int)k2y & 1);
    }
    long long B = (long long)G * G, ncell = oref_pyramid_cells(G);
    int L = oref_num_levels(G);
    double *mom = (double *)malloc(sizeof(double) * 6 * (size_t)ncell);
    float *rec = (float *)malloc(sizeof(float) * 4 * (size_t)ncell);
    if (leaf_in) {
        memcpy(mom, leaf_in, sizeof(double) * 6 * (size_t)B);
        build_pyramid(G, bb[4], mom, rec);
    } else {
        oref_moments(n, x, y, m, G, bb, kx, ky, mom, rec);
    }
    long long *lvoff = (long long *)malloc(sizeof(long long) * (size_t)(L + 1));
    int *lvg = (int *)malloc(sizeof(int) * (size_t)(L + 1));
    {
        long long off = 0;
        int g = G;
        for (int l = 0; l < L; l++) {
            lvoff[l] = off;
            lvg[l] = g;
            off += (long long)g * g;
            g = (g + 1) / 2;
        }
    }
    /* particles grouped by box (pid lists) */
    long long *bstart = (long long *)calloc((size_t)B + 1, sizeof(long long));
    long long *order = (long long *)malloc(sizeof(long long) * (size_t)n);
    for (long long i = 0; i < n; i++) bstart[(long long)kx[i] * G + ky[i] + 1]++;
    for (long long b = 0; b < B; b++) bstart[b + 1] += bstart[b];
    {
        long long *cur = (long long *)malloc(sizeof(long long) * (size_t)B);
        memcpy(cur, bstart, sizeof(long long) * (size_t)B);
        for (long long i = 0; i < n; i++) order[cur[(long long)kx[i] * G + ky[i]]++] = i;
        free(cur);
    }
    const float step_f = (float)bb[4];
    const float theta2_f = (float)(theta * theta);
    const int flat = theta <= 0.0;
    if (flat) TG = 1;
    const int NGs = (G + TG - 1) / TG;
    const float W_f = (float)TG * step_f;
    long long cnt_near = 0, cnt_far = 0;

#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : cnt_near, cnt_far)
#endif
    for (long long gidx = 0; gidx < (long long)NGs * NGs; gidx++) {
        int gi = (int)(gidx / NGs), gj = (int)(gidx % NGs);
        int gx0 = gi * TG, gy0 = gj * TG;
        int gx1 = gx0 + TG < G ? gx0 + TG : G, gy1 = gy0 + TG < G ? gy0 + TG : G;
        long long nt = 0;
        for (int bx = gx0; bx < gx1; bx++) nt += bstart[(long long)bx * G + gy1] - bstart[(long long)bx * G + gy0];
        if (nt == 0) continue;
        /* interaction lists: far cells (level, index) and near leaf boxes */
        long long cap = 4 * ncell + 16;
        long long *far = (long long *)malloc(sizeof(long long) * (size_t)cap);
        long long *near = (long long *)malloc(sizeof(long long) * (size_t)B);
        long long nfar = 0, nnear = 0;
        if (flat) {
            for (int i = 0; i < G; i++)
                for (int j = 0; j < G; j++) {
                    long long c = (long long)i * G + j;
                    /* a part of a system knows the other boxes by their moments only */
                    const int nonempty = bstart[c + 1] > bstart[c] || (leaf_in && mom[6 * c] > 0.0);
                    if (!nonempty) continue;
                    if (abs(i - gx0) <= 1 && abs(j - gy0) <= 1)
                        near[nnear++] = c;
                    else
                        far[nfar++] = c;
                }
        } else {
            long long *fr = (long long *)malloc(sizeof(long long) * (size_t)cap);
            long long *nx = (long long *)malloc(sizeof(long long) * (size_t)cap);
            long long nfr = 1, nnx;
            fr[0] = 0; /* the single top cell, index within its level */
            for (int l = L - 1; l >= 0; l--) {
                nnx = 0;
                int gl = lvg[l];
                for (long long q = 0; q < nfr; q++) {
                    long long ci_ = fr[q];
                    int ci = (int)(ci_ / gl), cj = (int)(ci_ % gl);
                    long long cell = lvoff[l] + ci_;
                    if (!(mom[6 * cell] > 0.0)) continue;
                    int lo_x = ci << l, hi_x = (ci + 1) << l, lo_y = cj << l, hi_y = (cj + 1) << l;
                    int overlap = lo_x < gx1 && hi_x > gx0 && lo_y < gy1 && hi_y > gy0;
                    int accept = 0;
                    if (!overlap) {
                        float rx = (float)(lo_x - gx0) * step_f + rec[4 * cell];
                        float ry = (float)(lo_y - gy0) * step_f + rec[4 * cell + 1];
                        float dxo = fmaxf(0.0f, fmaxf(-rx, rx - W_f));
                        float dyo = fmaxf(0.0f, fmaxf(-ry, ry - W_f));
                        float d2 = dxo * dxo + dyo * dyo;
                        float s_f = ldexpf(step_f, l);
                        accept = (s_f * s_f) < (theta2_f * d2);
                    }
                    if (accept) {
                        far[nfar++] = cell;
                    } else if (l == 0) {
                        near[nnear++] = ci_;
                    } else {
                        int gc = lvg[l - 1];
                        for (int a = 0; a < 2; a++)
                            for (int c = 0; c < 2; c++) {
                                int ch_i = 2 * ci + a, ch_j = 2 * cj + c;
                                if (ch_i < gc && ch_j < gc) nx[nnx++] = (long long)ch_i * gc + ch_j;
                            }
                    }
                }
                long long *t = fr;
                fr = nx;
                nx = t;
                nfr = nnx;
            }
            free(fr);
            free(nx);
        }
        long long *bnear = (long long *)malloc(sizeof(long long) * (size_t)(nnear + 1));
        long long *bfar = (long long *)malloc(sizeof(long long) * (size_t)(nnear + 1));
        for (int bx = gx0; bx < gx1; bx++) {
            for (int by = gy0; by < gy1; by++) {
                const long long bb0 = (long long)bx * G + by;
                const long long nb = bstart[bb0 + 1] - bstart[bb0];
                if (nb == 0) continue;
                /* the box's target sets: the whole box with the group's lists (sparse box) or with
                 * per-box refined lists (dense box), or its four quadrants, each with lists refined
                 * against the quadrant (box with at least quad_min particles) */
                int kind = 0;
                if (!flat && quad_min > 0 && nb >= quad_min)
                    kind = 2;
                else if (!flat && dense_min > 0 && nb >= dense_min)
                    kind = 1;
                for (int part = 0; part < (kind == 2 ? 4 : 1); part++) {
                    long long nt_part = 0, nt_cnt = 0;
                    for (long long k = bstart[bb0]; k < bstart[bb0 + 1]; k++)
                        if (kind != 2 || quad[order[k]] == part) {
                            nt_part++;
                            if (!bb_in || !mask || mask[order[k]]) nt_cnt++;
                        }
                    if (nt_part == 0) continue;
                    const long long *nl = near;
                    long long nnl = nnear, nacc = 0;
                    if (kind > 0) {
                        float ox, oy, wr;  /* rectangle origin in the group frame, edge */
                        if (kind == 2) {
                            const float half_f = 0.5f * step_f;
                            ox = (float)(2 * (bx - gx0) + (part >> 1)) * half_f;
                            oy = (float)(2 * (by - gy0) + (part & 1)) * half_f;
                            wr = half_f;
                        } else {
                            ox = (float)(bx - gx0) * step_f;
                            oy = (float)(by - gy0) * step_f;
                            wr = step_f;
                        }
                        nnl = 0;
                        for (long long q = 0; q < nnear; q++) {
                            const long long c = near[q];
                            const int qi = (int)(c / G), qj = (int)(c % G);
                            int acc = 0;
                            if (!(qi == bx && qj == by)) {
                                float rx = (float)(qi - gx0) * step_f + rec[4 * c];
                                float ry = (float)(qj - gy0) * step_f + rec[4 * c + 1];
                                float rxb = rx - ox, ryb = ry - oy;
                                float dxo = fmaxf(0.0f, fmaxf(-rxb, rxb - wr));
                                float dyo = fmaxf(0.0f, fmaxf(-ryb, ryb - wr));
                                float d2 = dxo * dxo + dyo * dyo;
                                acc = (step_f * step_f) < (theta2_f * d2);
                            }
                            if (acc)
                                bfar[nacc++] = c; /* a leaf: level 0, cell index = box index */
                            else
                                bnear[nnl++] = c;
                        }
                        nl = bnear;
                    }
                    long long nsrc = 0;
                    for (long long q = 0; q < nnl; q++) nsrc += bstart[nl[q] + 1] - bstart[nl[q]];
                    cnt_near += nt_cnt * nsrc;
                    cnt_far += nt_cnt * (nfar + nacc);
                    for (long long k = bstart[bb0]; k < bstart[bb0 + 1]; k++) {
                        long long t = order[k];
                        if (kind == 2 && quad[t] != part) continue;
                        if (mask && !mask[t]) continue;
                        double xt = x[t], yt = y[t], sx = 0.0, sy = 0.0;
                        for (long long q = 0; q < nacc; q++) {
                            long long cell = bfar[q];
                            int ci = (int)(cell / G), cj = (int)(cell % G);
                            const double *qm = mom + 6 * cell;
                            double cx = (bb[0] + (double)ci * bb[4]) + qm[1] / qm[0];
                            double cy = (bb[1] + (double)cj * bb[4]) + qm[2] / qm[0];
                            double dx = cx - xt, dy = cy - yt;
                            double r2 = dx * dx + dy * dy;
                            if (!(r2 > cutoff)) continue;
                            double w = qm[0] / (r2 + eps2);
                            sx += w * dx;
                            sy += w * dy;
                        }
                        for (long long q = 0; q < nnl; q++)
                            for (long long kk = bstart[nl[q]]; kk < bstart[nl[q] + 1]; kk++) {
                                long long j = order[kk];
                                double dx = x[j] - xt, dy = y[j] - yt;
                                double r2 = dx * dx + dy * dy;
                                if (!(r2 > cutoff)) continue;
                                double w = m[j] / (r2 + eps2);
                                sx += w * dx;
                                sy += w * dy;
                            }
                        for (long long q = 0; q < nfar; q++) {
                            long long cell = far[q];
                            int l = 0;
                            while (l + 1 < L && lvoff[l + 1] <= cell) l++;
                            long long ci_ = cell - lvoff[l];
                            int ci = (int)(ci_ / lvg[l]), cj = (int)(ci_ % lvg[l]);
                            const double *qm = mom + 6 * cell;
                            double cx = (bb[0] + (double)(ci << l) * bb[4]) + qm[1] / qm[0];
                            double cy = (bb[1] + (double)(cj << l) * bb[4]) + qm[2] / qm[0];
                            double dx = cx - xt, dy = cy - yt;
                            double r2 = dx * dx + dy * dy;
                            if (!(r2 > cutoff)) continue;
                            double w = qm[0] / (r2 + eps2);
                            sx += w * dx;
                            sy += w * dy;
                        }
                        ax[t] = gconst * sx;
                        ay[t] = gconst * sy;
                    }
                }
            }
        }
        free(bnear);
        free(bfar);
        free(far);
        free(near);
    }
    if (counts) {
        counts[0] = cnt_near;
        counts[1] = cnt_far;
    }
    free(kx);
    free(quad);
    free(ky);
    free(mom);
    free(rec);
    free(lvoff);
    free(lvg);
    free(bstart);
    free(order);
    return G;
}

/* ------------------------------------------------------------------ 8 -- */
/*
 * The reference GPU evaluation (python-bh kernels/grid_decomposition/gpu/grid.py), FP64:
 *   keys      g_place_particles (:15-50): min(floor((p - min) / step), G - 1)
 *   COMs      g_summarize (:78-114): sum of p * m and m over the box; (0, 0, 0) for an empty box
 *   evaluate  g_evaluate_boxes (:116-157) with d_self_self_grav (:211-229), d_self_other_grav
 *             (:231-248), d_self_COM_grav (:250-268): for every target, a loop over all G x G
 *             boxes in (gx, gy) order -- its own box pair by pair skipping only itself (j != i),
 *             the 8 neighbours pair by pair, every other box (empty ones included) through its
 *             COM -- with f = (G m_i m_j) / (dist * dist), dist = sqrt(dx^2 + dy^2), and
 *             a -= f * dx / m_i, dx = x_i - x_j.  No cutoff, no softening.
 * The reference GPU path divides by zero for two particles at the same position (and for a
 * particle at exactly (0, 0) against an empty box's zero COM), which gives NaN; skip_zero != 0
 * drops every pair with dist == 0 instead (the rule of this project's CUDA path).  cutoff >= 0
 * also drops pairs with dx^2 + dy^2 <= cutoff (1e-5 gives the CPU path's physics: used to pin
 * this restatement against the reference CPU path's golden vectors).  mask: see
 * oref_theta_evaluate.  Output ax/ay in pid order.
 */
static inline void gpu_pair(double xi, double yi, double mi, double ox, double oy, double mj,
                            double G, double cutoff, int skip_zero, double *ax, double *ay)
{
    double xdif = xi - ox, ydif = yi - oy;
    double r2 = xdif * xdif + ydif * ydif;
    if (cutoff >= 0.0 && !(r2 > cutoff)) return;
    double dist = sqrt(r2);
    if (skip_zero && dist == 0.0) return;
    double f = (G * mi * mj) / (dist * dist);
    *ax = *ax - (f * xdif / mi);
    *ay = *ay - (f * ydif / mi);
}

void oref_gpu_evaluate(long long n, const double *x, const double *y, const double *m, int G,
                       double gconst, double cutoff, int skip_zero, const unsigned char *mask,
                       double *ax, double *ay, int nthreads)
{
    if (n <= 0) return;
    double bb[5];
    oref_bbox(n, x, y, G, bb);
    int *kx = (int *)malloc(sizeof(int) * (size_t)n), *ky = (int *)malloc(sizeof(int) * (size_t)n);
    for (long long i = 0; i < n; i++) {
        double qx = floor((x[i] - bb[0]) / bb[4]), qy = floor((y[i] - bb[1]) / bb[4]);
        kx[i] = (int)(qx < (double)(G - 1) ? qx : (double)(G - 1));
        ky[i] = (int)(qy < (double)(G - 1) ? qy : (double)(G - 1));
    }
    long long B = (long long)G * G;
    long long *bstart = (long long *)calloc((size_t)B + 1, sizeof(long long));
    long long *order = (long long *)malloc(sizeof(long long) * (size_t)n);
    for (long long i = 0; i < n; i++) bstart[(long long)kx[i] * G + ky[i] + 1]++;
    for (long long b = 0; b < B; b++) bstart[b + 1] += bstart[b];
    {
        long long *cur = (long long *)malloc(sizeof(long long) * (size_t)B);
        memcpy(cur, bstart, sizeof(long long) * (size_t)B);
        for (long long i = 0; i < n; i++) order[cur[(long long)kx[i] * G + ky[i]]++] = i;
        free(cur);
    }
    double *com = (double *)calloc(3 * (size_t)B, sizeof(double));
    for (long long b = 0; b < B; b++) {
        if (bstart[b + 1] == bstart[b]) continue;
        double M = 0.0, sx = 0.0, sy = 0.0;
        for (long long k = bstart[b]; k < bstart[b + 1]; k++) {
            long long j = order[k];
            sx += x[j] * m[j];
            sy += y[j] * m[j];
            M += m[j];
        }
        if (M != 0.0) {
            com[3 * b] = sx / M;
            com[3 * b + 1] = sy / M;
            com[3 * b + 2] = M;
        }
    }
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (long long i = 0; i < n; i++) {
        if (mask && !mask[i]) continue;
        const int bx = kx[i], by = ky[i];
        const double xi = x[i], yi = y[i], mi = m[i];
        double sx = 0.0, sy = 0.0;
        for (int gx = 0; gx < G; gx++)
            for (int gy = 0; gy < G; gy++) {
                long long c = (long long)gx * G + gy;
                if (abs(gx - bx) <= 1 && abs(gy - by) <= 1) {
                    for (long long k = bstart[c]; k < bstart[c + 1]; k++) {
                        long long j = order[k];
                        if (j == i) continue;
                        gpu_pair(xi, yi, mi, x[j], y[j], m[j], gconst, cutoff, skip_zero, &sx, &sy);
                    }
                } else {
                    gpu_pair(xi, yi, mi, com[3 * c], com[3 * c + 1], com[3 * c + 2], gconst, cutoff,
                             skip_zero, &sx, &sy);
                }
            }
        ax[i] = sx;
        ay[i] = sy;
    }
    free(kx);
    free(ky);
    free(bstart);
    free(order);
    free(com);
}

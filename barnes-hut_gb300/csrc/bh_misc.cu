// bh_misc.cu -- state upload / download, unfused tick, FP64 direct-sum sampler, diagnostics.
#include "bh_internal.cuh"

namespace bh {

constexpr int MT = 256;

static inline unsigned grid_of(long long n, int tpb, int nsm) {
    long long b = (n + tpb - 1) / tpb;
    if (b < 1) b = 1;
    if (b > nsm * 16LL) b = nsm * 16LL;
    return (unsigned)b;
}

// Upload: state buffer (epoch + 1) & 1 receives the particles in the given
// order; pid = concatenated index.  rec_stride = 0: SoA arrays; 10: the
// reference's N x 10 record (internals/particle.py:3-15), x points at row 0.
// The accelerations are not written: until the next evaluation they read as
// zero (the host tracks it; k_store then writes zeros).
__global__ void k_load(DevPlan d, const double *x, const double *y, const double *m,
                       const double *vx, const double *vy, long long rs) {
    const int b = (d.glob->epoch + 1) & 1;
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < d.n_total; i += stride) {
        long long k = rs ? i * rs : i;
        d.X[b][i] = x[k];
        d.Y[b][i] = y[k];
        d.M[b][i] = m[k];
        d.VX[b][i] = vx[k];
        d.VY[b][i] = vy[k];
        d.PID[b][i] = (int)i;
    }
}

// Download in pid order.  rec: N x 10 records (px, py, mass, vx, vy, ax, ay,
// gx, gy, pid) or NULL; SoA outputs may be NULL.  gx/gy come from the box
// keys of the last create_tree (skey), 0 before the first one; ax/ay are 0
// when no evaluation followed the last load (has_acc = 0).
__global__ void k_store(DevPlan d, double *rec, double *x, double *y, double *vx, double *vy,
                        double *ax, double *ay, int has_tree, int has_acc) {
    const int b = (d.glob->epoch + 1) & 1;
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < d.n_total; i += stride) {
        long long p = d.PID[b][i];
        double px = d.X[b][i], py = d.Y[b][i], pvx = d.VX[b][i], pvy = d.VY[b][i];
        const double pax = has_acc ? d.AX[i] : 0.0, pay = has_acc ? d.AY[i] : 0.0;
        if (rec) {
            double *r = rec + 10 * p;
            double gx = 0.0, gy = 0.0;
            if (has_tree) {
                int key = d.skey[i];
                int s = find_seg(d.boff_tab, d.nsys, key);
                int lb = (int)(key - d.sys[s].boff);
                gx = (double)(lb / d.sys[s].G);
                gy = (double)(lb % d.sys[s].G);
            }
            r[0] = px; r[1] = py; r[2] = d.M[b][i]; r[3] = pvx; r[4] = pvy;
            r[5] = pax; r[6] = pay; r[7] = gx; r[8] = gy; r[9] = (double)p;
        }
        if (x) x[p] = px;
        if (y) y[p] = py;
        if (vx) vx[p] = pvx;
        if (vy) vy[p] = pvy;
        if (ax) ax[p] = pax;
        if (ay) ay[p] = pay;
    }
}

// v += a dt; a = 0; x += v dt  (gpu/grid.py:159-174)
// keep_acc: leave the accelerations in place (the fused step's tick, which keeps the last
// evaluation's accelerations; the reference's tick, gpu/grid.py:159-174, zeroes them)
__global__ void k_tick(DevPlan d, int keep_acc) {
    const int b = (d.glob->epoch + 1) & 1;
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < d.n_total; i += stride) {
        double ax = d.AX[i], ay = d.AY[i];
        double vx = d.VX[b][i] + ax * d.dt, vy = d.VY[b][i] + ay * d.dt;
        d.VX[b][i] = vx;
        d.VY[b][i] = vy;
        if (!keep_acc) {
            d.AX[i] = 0.f;
            d.AY[i] = 0.f;
        }
        d.X[b][i] = d.X[b][i] + vx * d.dt;
        d.Y[b][i] = d.Y[b][i] + vy * d.dt;
    }
}

// inverse permutation pid -> current index, written into the key array
__global__ void k_inverse_pid(DevPlan d) {
    const int b = (d.glob->epoch + 1) & 1;
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < d.n_total; i += stride)
        d.key[d.PID[b][i]] = (int)i;
}

// FP64 direct sum, one CTA per target (base.py:16-32 without its self-skip by
// pid replaced: j == t is skipped by index).
__global__ void __launch_bounds__(MT) k_direct(DevPlan d, int sys, const long long *targets,
                                               double *oax, double *oay) {
    const int b = (d.glob->epoch + 1) & 1;
    const SysDesc &sd = d.sys[sys];
    __shared__ double rx[MT / 32], ry[MT / 32];
    long long t = targets[blockIdx.x];
    if (t < sd.poff || t >= sd.poff + sd.n) {  // not a particle of this system
        if (threadIdx.x == 0) oax[blockIdx.x] = oay[blockIdx.x] = __longlong_as_double(0x7ff8000000000000ll);
        return;
    }
    int ti = d.key[t];
    double xt = d.X[b][ti], yt = d.Y[b][ti];
    double sx = 0.0, sy = 0.0;
    for (long long j = sd.poff + threadIdx.x; j < sd.poff + sd.n; j += MT) {
        if (j == ti) continue;
        double dx = d.X[b][j] - xt, dy = d.Y[b][j] - yt;
        double w = d.M[b][j] / (dx * dx + dy * dy + d.eps2);
        sx += w * dx;
        sy += w * dy;
    }
    for (int o = 16; o; o >>= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, o);
        sy += __shfl_xor_sync(0xffffffffu, sy, o);
    }
    if ((threadIdx.x & 31) == 0) { rx[threadIdx.x >> 5] = sx; ry[threadIdx.x >> 5] = sy; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, c = 0.0;
        for (int k = 0; k < MT / 32; k++) { a += rx[k]; c += ry[k]; }
        oax[blockIdx.x] = d.gconst * a;
        oay[blockIdx.x] = d.gconst * c;
    }
}

// out = {kinetic, momentum x, momentum y, potential}; FP64 block reductions.
__global__ void __launch_bounds__(MT) k_diag(DevPlan d, int sys, int want_pot, double *out) {
    const int b = (d.glob->epoch + 1) & 1;
    const SysDesc &sd = d.sys[sys];
    __shared__ double red[4][MT / 32];
    double ke = 0, px = 0, py = 0, pe = 0;
    long long n = sd.n;
    for (long long i = (long long)blockIdx.x * MT + threadIdx.x; i < n; i += (long long)gridDim.x * MT) {
        long long k = sd.poff + i;
        double m = d.M[b][k], vx = d.VX[b][k], vy = d.VY[b][k];
        ke += 0.5 * m * (vx * vx + vy * vy);
        px += m * vx;
        py += m * vy;
        if (want_pot) {
            double xi = d.X[b][k], yi = d.Y[b][k], s = 0.0;
            for (long long j = sd.poff; j < sd.poff + n; j++) {
                if (j == k) continue;
                double dx = d.X[b][j] - xi, dy = d.Y[b][j] - yi;
                s += d.M[b][j] * 0.5 * log(dx * dx + dy * dy + d.eps2);
            }
            pe += 0.5 * m * s;  // each pair counted twice
        }
    }
    double v[4] = {ke, px, py, pe * d.gconst};
    for (int c = 0; c < 4; c++)
        for (int o = 16; o; o >>= 1) v[c] += __shfl_xor_sync(0xffffffffu, v[c], o);
    if ((threadIdx.x & 31) == 0)
        for (int c = 0; c < 4; c++) red[c][threadIdx.x >> 5] = v[c];
    __syncthreads();
    if (threadIdx.x < 4) {
        double a = 0;
        for (int k = 0; k < MT / 32; k++) a += red[threadIdx.x][k];
        atomicAdd(out + threadIdx.x, a);
    }
}

// Leaf centres of mass in the reference layout (G x G x 3: cx, cy, M).
__global__ void k_box_com(DevPlan d, int sys, double *out) {
    const SysDesc &sd = d.sys[sys];
    const SysDyn &dy = d.dyn[sys];
    long long B = (long long)sd.G * sd.G;
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x; b < B; b += stride) {
        const double *q = d.mom + 6 * (sd.coff + b);
        double M = q[0];
        double *o = out + 3 * b;
        if (M > 0.0) {
            int kx = (int)(b / sd.G), ky = (int)(b % sd.G);
            o[0] = box_origin(dy.minx, kx, dy.step) + q[1] / M;
            o[1] = box_origin(dy.miny, ky, dy.step) + q[2] / M;
            o[2] = M;
        } else {
            o[0] = o[1] = o[2] = 0.0;
        }
    }
}

cudaError_t launch_box_com(const DevPlan &d, int sys, double *out, cudaStream_t st) {
    k_box_com<<<d.nsm * 4, MT, 0, st>>>(d, sys, out);
    return cudaGetLastError();
}

cudaError_t launch_load(const DevPlan &d, const double *x, const double *y, const double *m,
                        const double *vx, const double *vy, long long rs, cudaStream_t st) {
    if (d.n_total == 0) return cudaSuccess;
    k_load<<<grid_of(d.n_total, MT, d.nsm), MT, 0, st>>>(d, x, y, m, vx, vy, rs);
    return cudaGetLastError();
}

cudaError_t launch_store(const DevPlan &d, int has_tree, bool has_acc, double *rec, double *x, double *y,
                         double *vx, double *vy, double *ax, double *ay, cudaStream_t st) {
    if (d.n_total == 0) return cudaSuccess;
    k_store<<<grid_of(d.n_total, MT, d.nsm), MT, 0, st>>>(d, rec, x, y, vx, vy, ax, ay, has_tree, has_acc ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_tick(const DevPlan &d, cudaStream_t st, bool keep_acc) {
    if (d.n_total == 0) return cudaSuccess;
    k_tick<<<grid_of(d.n_total, MT, d.nsm), MT, 0, st>>>(d, keep_acc ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_direct(const DevPlan &d, int sys, const long long *targets, long long nt,
                          double *ax, double *ay, cudaStream_t st) {
    if (d.n_total == 0 || nt == 0) return cudaSuccess;
    k_inverse_pid<<<grid_of(d.n_total, MT, d.nsm), MT, 0, st>>>(d);
    for (long long t0 = 0; t0 < nt; t0 += (1LL << 30)) {
        long long c = nt - t0 < (1LL << 30) ? nt - t0 : (1LL << 30);
        k_direct<<<(unsigned)c, MT, 0, st>>>(d, sys, targets + t0, ax + t0, ay + t0);
    }
    return cudaGetLastError();
}

cudaError_t launch_diag(const DevPlan &d, int sys, int want_pot, double *out, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(out, 0, 4 * sizeof(double), st);
    if (e != cudaSuccess) return e;
    k_diag<<<d.nsm * 2, MT, 0, st>>>(d, sys, want_pot, out);
    return cudaGetLastError();
}

}  // namespace bh

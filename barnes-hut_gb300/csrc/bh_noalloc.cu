// bh_noalloc.cu -- FP64 direct-sum sampler for callers that cannot allocate device memory.
//
// bh_direct_sample (bh_misc.cu) needs a plan, and a plan needs a workspace the caller
// allocates.  Some callers have no way to do that: code running inside another framework that
// has reserved the whole device for its own memory pool, or a control loop that must not call
// the CUDA allocator once it is running.  bh_direct_sum_noalloc serves them: it takes plain
// device arrays (positions and masses in any order, target indices, outputs) and keeps its
// scratch -- the per-chunk partial sums of every target -- in the file-scope array below,
// which every GPU that loads the library holds until the process exits.
#include <cuda.h>

#include <mutex>

#include "../../include/bh_gb300.h"
#include "bh_internal.cuh"

namespace bh {

constexpr int NA_THREADS = 256;
// partial sums: target k, source chunk c -> (ax, ay)
static __device__ __align__(256) double g_noalloc_partials[BH_NOALLOC_MAX_TARGETS * BH_NOALLOC_CHUNKS * 2];

// Phase 1: block (c, k) sums source chunk c for target k.  Every slot phase 2 reads is written
// here first, so nothing from an earlier call survives into the result.
__global__ void __launch_bounds__(NA_THREADS) k_direct_partials(const double *x, const double *y,
                                                               const double *m, long long n,
                                                               const long long *targets,
                                                               double eps2, double *scratch) {
    __shared__ double rx[NA_THREADS / 32], ry[NA_THREADS / 32];
    const int c = blockIdx.x, k = blockIdx.y;
    const long long t = targets[k];
    const long long per = (n + BH_NOALLOC_CHUNKS - 1) / BH_NOALLOC_CHUNKS;
    const long long j0 = (long long)c * per, j1 = j0 + per < n ? j0 + per : n;
    double sx = 0.0, sy = 0.0;
    if (t >= 0 && t < n) {
        const double xt = x[t], yt = y[t];
        for (long long j = j0 + threadIdx.x; j < j1; j += NA_THREADS) {
            if (j == t) continue;
            double dx = x[j] - xt, dy = y[j] - yt;
            double w = m[j] / (dx * dx + dy * dy + eps2);
            sx += w * dx;
            sy += w * dy;
        }
    }
    for (int o = 16; o; o >>= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, o);
        sy += __shfl_xor_sync(0xffffffffu, sy, o);
    }
    if ((threadIdx.x & 31) == 0) {
        rx[threadIdx.x >> 5] = sx;
        ry[threadIdx.x >> 5] = sy;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < NA_THREADS / 32; w++) {
            a += rx[w];
            b += ry[w];
        }
        double *o = scratch + 2 * ((long long)k * BH_NOALLOC_CHUNKS + c);
        o[0] = a;
        o[1] = b;
    }
}

// Phase 2: one thread per target adds its chunk partials in chunk order.
__global__ void k_direct_finish(const long long *targets, long long nt, long long n, double gconst,
                                const double *scratch, double *ax, double *ay) {
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nt) return;
    const long long t = targets[k];
    if (t < 0 || t >= n) {  // not a particle index: NaN, as bh_direct_sample reports it
        ax[k] = ay[k] = __longlong_as_double(0x7ff8000000000000ll);
        return;
    }
    double a = 0.0, b = 0.0;
    for (int c = 0; c < BH_NOALLOC_CHUNKS; c++) {
        a += scratch[2 * (k * BH_NOALLOC_CHUNKS + c)];
        b += scratch[2 * (k * BH_NOALLOC_CHUNKS + c) + 1];
    }
    ax[k] = gconst * a;
    ay[k] = gconst * b;
}

// Device address of the scratch array.  The address belongs to one CUDA context (the module is
// loaded once per context), so it is looked up once per context, with that context current, and
// cached under the context's ID -- unique for the life of the process, so a context created after
// cudaDeviceReset, or a framework's own driver-API context on the same device, never finds an
// address that belongs to another context.
constexpr int NA_CACHE = 64;
static std::mutex g_na_mutex;
static unsigned long long g_na_ctx[NA_CACHE];
static double *g_na_ptr[NA_CACHE];
static int g_na_next;

// The two driver calls are resolved through the runtime, so the library needs no link against
// the driver library (it loads on machines without a GPU driver, for its host-side checks).
typedef CUresult (*ctx_get_current_fn)(CUcontext *);
typedef CUresult (*ctx_get_id_fn)(CUcontext, unsigned long long *);
static ctx_get_current_fn g_ctx_get_current;
static ctx_get_id_fn g_ctx_get_id;

static cudaError_t noalloc_driver_calls() {
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (g_ctx_get_current && g_ctx_get_id) return cudaSuccess;
    void *a = nullptr, *b = nullptr;
    cudaDriverEntryPointQueryResult qa, qb;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa);
    if (e != cudaSuccess) return e;
    e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb);
    if (e != cudaSuccess) return e;
    if (qa != cudaDriverEntryPointSuccess || qb != cudaDriverEntryPointSuccess || !a || !b)
        return cudaErrorSymbolNotFound;
    g_ctx_get_current = (ctx_get_current_fn)a;
    g_ctx_get_id = (ctx_get_id_fn)b;
    return cudaSuccess;
}

static cudaError_t noalloc_scratch(double **out) {
    cudaError_t de = noalloc_driver_calls();
    if (de != cudaSuccess) return de;
    ctx_get_current_fn cuCtxGetCurrent = g_ctx_get_current;
    ctx_get_id_fn cuCtxGetId = g_ctx_get_id;
    CUcontext ctx = nullptr;
    CUresult r = cuCtxGetCurrent(&ctx);
    if (r == CUDA_ERROR_NOT_INITIALIZED)
        ctx = nullptr;
    else if (r != CUDA_SUCCESS)
        return cudaErrorDeviceUninitialized;
    double *p = nullptr;
    if (!ctx) {  // no context current yet: the runtime's lookup makes the primary context current
        cudaError_t e = cudaGetSymbolAddress((void **)&p, g_noalloc_partials);
        if (e != cudaSuccess) return e;
        if (cuCtxGetCurrent(&ctx) != CUDA_SUCCESS || !ctx) return cudaErrorDeviceUninitialized;
    }
    unsigned long long id = 0;
    if (cuCtxGetId(ctx, &id) != CUDA_SUCCESS) return cudaErrorDeviceUninitialized;
    std::lock_guard<std::mutex> lock(g_na_mutex);
    for (int i = 0; i < NA_CACHE; i++)
        if (g_na_ptr[i] && g_na_ctx[i] == id) {
            *out = g_na_ptr[i];
            return cudaSuccess;
        }
    if (!p) {
        cudaError_t e = cudaGetSymbolAddress((void **)&p, g_noalloc_partials);
        if (e != cudaSuccess) return e;
    }
    const int slot = g_na_next;  // oldest entry out first once the table is full
    g_na_next = (g_na_next + 1) % NA_CACHE;
    g_na_ctx[slot] = id;
    g_na_ptr[slot] = p;
    *out = p;
    return cudaSuccess;
}

}  // namespace bh

extern "C" int bh_direct_sum_noalloc(const double *x, const double *y, const double *m,
                                     long long n, const long long *targets, long long nt,
                                     double grav_constant, double softening, double *ax,
                                     double *ay, void *stream) {
    using namespace bh;
    if (n < 0 || nt < 0 || (nt > 0 && (!targets || !ax || !ay)) ||
        (n > 0 && nt > 0 && (!x || !y || !m)) || !(softening >= 0.0))
        return bh_set_thread_error(BH_ERR_INVALID, "bh_direct_sum_noalloc: invalid argument");
    if (nt > BH_NOALLOC_MAX_TARGETS)
        return bh_set_thread_error(BH_ERR_INVALID,
                                   "bh_direct_sum_noalloc: more than BH_NOALLOC_MAX_TARGETS (4096) "
                                   "targets; split the call or use bh_direct_sample");
    if (nt == 0) return BH_OK;
    double *scratch = nullptr;
    cudaError_t e = noalloc_scratch(&scratch);
    if (e != cudaSuccess)
        return bh_set_thread_error(BH_ERR_CUDA, "bh_direct_sum_noalloc: cudaGetSymbolAddress failed");
    cudaStream_t st = (cudaStream_t)stream;
    dim3 grid(BH_NOALLOC_CHUNKS, (unsigned)nt);
    k_direct_partials<<<grid, NA_THREADS, 0, st>>>(x, y, m, n, targets, softening * softening, scratch);
    k_direct_finish<<<(unsigned)((nt + 127) / 128), 128, 0, st>>>(targets, nt, n, grav_constant,
                                                                   scratch, ax, ay);
    e = cudaGetLastError();
    if (e != cudaSuccess) return bh_set_thread_error(BH_ERR_CUDA, "bh_direct_sum_noalloc: launch failed");
    return BH_OK;
}

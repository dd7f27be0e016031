/*
 * bh_gb300.h -- C ABI of the GB300-native 2D grid-decomposition Barnes-Hut step.
 *
 * The reference (ut-parla/barnes-hut, python-bh) has no native FFI: its
 * single-GPU implementation calls Numba CUDA kernels from Python.  The entry
 * points below are the calls that implementation makes, one per step phase
 * of its step interface (python-bh/barneshut/implementations/base.py:94-135):
 * each declaration cites the reference code it replaces.
 *
 * Conventions
 *  - Every function returns an int status (BH_OK == 0) and never aborts;
 *    bh_last_error(plan) gives a one-line message for the last failure.
 *  - All device work is asynchronous on the stream passed as `void *stream`
 *    (a cudaStream_t; NULL is the legacy default stream).
 *  - The library allocates no device memory.  The caller queries
 *    bh_workspace_size() and passes one device buffer to bh_bind(); all
 *    per-system state lives inside it.  A plan holds no global state, so
 *    several plans may be used concurrently from different host threads
 *    (python-bh/bin/run_2d_concurrent.py:53-87 runs instances in threads).
 *  - A plan steps `nsys` independent systems at once (particles, boxes and
 *    pyramid cells are concatenated); nsys = 1 is the reference's case.
 *  - Device pointers passed in are plain `double *` arrays of the
 *    concatenated particles in original particle (pid) order.
 */
#ifndef BH_GB300_H
#define BH_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BH_OK 0
#define BH_ERR_INVALID 1   /* invalid argument (checked on the host) */
#define BH_ERR_CUDA 2      /* a CUDA runtime call failed */
#define BH_ERR_WORKSPACE 3 /* no workspace bound, or too small */
#define BH_ERR_DEVICE 4    /* a kernel raised a device error flag */
#define BH_ERR_TIMEOUT 5   /* a bounded device wait gave up */

/* device error flags (bh_error_flags) */
#define BH_DEV_NAN_POSITION 1u   /* a non-finite position reached placement */
#define BH_DEV_LIST_OVERFLOW 2u  /* an interaction-list frontier overflowed */
#define BH_DEV_BAD_KEY 4u        /* a box key fell outside [0, G*G) */
#define BH_DEV_WAIT_TIMEOUT 8u   /* a bounded spin-wait expired */

/* precision of the pairwise force arithmetic */
#define BH_PREC_FP32 0       /* FP32 pairs, plain far-field sum */
#define BH_PREC_FP32_KAHAN 1 /* FP32 pairs, Kahan-compensated far-field sum */
#define BH_PREC_FP64 2       /* FP64 pairs (precision study) */

/* bh_params.flags */
#define BH_FLAG_LEARNED 1 /* apply the learned far-field correction (weights bound) */
/* List streaming (the theta-mode default): a box holding at least bh_params.dense_min particles
   (default below) is evaluated with its own near list, refined from its group's -- a near leaf
   whose centre of mass passes the opening test against the single box becomes a far entry for
   that box's particles. */
#define BH_STREAM_DENSE_MIN 64
/* ... and a box holding at least bh_params.quad_min particles is evaluated quadrant by
   quadrant (its particles are stored quadrant by quadrant), each quadrant with the near leaves
   that fail the opening test against that quarter of the box. */
#define BH_STREAM_QUAD_MIN 128
#define BH_FLAG_WALK 2    /* theta mode: walk the cell pyramid inside the force kernel for
                           every work item instead of building each target group's
                           interaction lists once and streaming them (the default for
                           FP32 pairs with softening > 0, no cutoff and grid_dim <= 16384) */

typedef struct bh_params {
    double grav_constant; /* [bh] grav_constant (python-bh/configs/default.ini) */
    double tick_seconds;  /* [bh] tick_seconds: dt of v += a dt; x += v dt */
    double softening;     /* Plummer epsilon; 0 = none (the reference has none) */
    double cutoff_r2;     /* pairs with unsoftened r^2 <= cutoff_r2 contribute 0.
                             1e-5 = the reference CPU kernels (cpu_numba.py:36);
                             0 = skip only coincident points (reference GPU). */
    double theta;         /* opening angle; <= 0 = the reference's flat far field
                             (3x3 neighbourhood direct, every other box's COM) */
    int group_dim;        /* target group = group_dim^2 leaf boxes (1, 2, 4, 8;
                             0 = automatic); forced to 1 in flat mode */
    int precision;        /* BH_PREC_* */
    int flags;            /* BH_FLAG_* */
    int tune;             /* force-kernel build, picked by the autotuner: 0 the path's
                             default (list streaming: 6 CTAs per SM, 80 registers; walk:
                             8 CTAs per SM), 1 the other (list streaming: 8 CTAs per SM,
                             64 registers; walk: 6 CTAs per SM) */
    double correction_theta; /* with BH_FLAG_LEARNED: cells accepted at theta but
                                not at correction_theta get the learned correction */
    int dense_min;        /* list streaming: boxes with at least this many particles get
                             per-box refined near lists (0 = BH_STREAM_DENSE_MIN) */
    int quad_min;         /* list streaming: boxes with at least this many particles get
                             per-quadrant refined near lists (0 = BH_STREAM_QUAD_MIN,
                             < 0 = none) */
} bh_params;

typedef struct bh_plan bh_plan;

/* Grid sizing of the reference: nleaves = n / (0.7 * ppb), rounded up to a
 * perfect square, G = sqrt(nleaves).
 * Replaces python-bh/barneshut/implementations/base.py:211-231 and
 * kernels/helpers/grid.py:5-8. */
int bh_grid_dim(long long n, int max_particles_per_box);

/* Create a plan for nsys systems with n[s] particles and grid_dim[s] boxes per
 * side (grid_dim[s] <= 0: bh_grid_dim(n[s], 1000)).  Host only, no CUDA call.
 * Replaces SingleGPUBarnesHut.__init__ (implementations/singlegpu.py:18-26). */
int bh_plan_create(bh_plan **plan, int nsys, const long long *n, const int *grid_dim,
                   const bh_params *params);
int bh_plan_destroy(bh_plan *plan);
/* Message of the last failure on this plan; bh_last_error(NULL) gives the
 * last bh_plan_create failure of the calling thread. */
const char *bh_last_error(const bh_plan *plan);

/* Device bytes the plan needs (state double buffers, keys, box table, cell
 * pyramid, tables).  Host only. */
int bh_workspace_size(const bh_plan *plan, size_t *bytes);

/* Bind a device workspace (>= bh_workspace_size bytes, 256-byte aligned) on
 * the current device, upload the system tables and zero the counters.
 * Replaces the device allocations of singlegpu.py:28-39 (__init_device_arrays). */
int bh_bind(bh_plan *plan, void *workspace, size_t bytes, void *stream);

/* Upload the particle state from device arrays in pid order (concatenated
 * over systems): positions x, y, masses m, velocities vx, vy (each n_total
 * doubles).  Accelerations start at zero.
 * Replaces cuda.to_device(self.particles) (singlegpu.py:37) of the file
 * reader's N x 10 record (base.py:47-72). */
int bh_load(bh_plan *plan, const double *x, const double *y, const double *m, const double *vx,
            const double *vy, void *stream);

/* Same, from the reference's N x 10 float64 particle record (field order
 * px, py, mass, vx, vy, ax, ay, gx, gy, pid: internals/particle.py:3-15),
 * as a device array in row order.  Rows are loaded in order; pid = row. */
int bh_load_records(bh_plan *plan, const double *records, void *stream);

/* Write the current state as N x 10 float64 records in pid order (gx, gy =
 * the particle's box, ax, ay = the last accelerations) into a device array.
 * Replaces ensure_particles_id_ordered (singlegpu.py:101-103). */
int bh_store_records(bh_plan *plan, double *records, void *stream);

/* Same as SoA arrays (any pointer may be NULL to skip that field). */
int bh_store(bh_plan *plan, double *x, double *y, double *vx, double *vy, double *ax,
             double *ay, void *stream);

/* Square bounding box, box keys, box histogram, exclusive scan and the
 * counting-sort scatter into box order (FP64 keys, bit-exact with the
 * reference: box index (gx, gy) = clip(floor((p - min) / step), 0, G-1)).
 * Replaces create_tree (singlegpu.py:41-67): set_particles_bounding_box
 * (base.py:211-239), g_place_particles, g_calculate_box_cumm and
 * g_sort_particles (kernels/grid_decomposition/gpu/grid.py:15-76). */
int bh_create_tree(bh_plan *plan, void *stream);

/* Per-box FP64 mass, centre of mass and second moments (segmented warp
 * reduction over the box-sorted particles), the cell pyramid and the float
 * cell records the force kernel reads.
 * Replaces summarize (singlegpu.py:69-77) and g_summarize (gpu/grid.py:78-114). */
int bh_summarize(bh_plan *plan, void *stream);

/* a += forces (reference semantics: accelerations accumulate until the tick
 * zeroes them).  Replaces evaluate (singlegpu.py:79-92) and g_evaluate_boxes
 * (gpu/grid.py:116-157) with the CPU path's semantics selected by params
 * (evaluation.py:73-109, cpu_numba.py:30-92). */
int bh_evaluate(bh_plan *plan, void *stream);

/* v += a dt; a = 0; x += v dt.  Replaces timestep (singlegpu.py:94-99) and
 * g_tick_particles (gpu/grid.py:159-174). */
int bh_timestep(bh_plan *plan, void *stream);

/* nsteps rounds of create_tree, summarize, evaluate with the tick fused into
 * the force epilogue (accelerations are overwritten, not accumulated, and
 * kept for bh_store).  Replaces the round loop of BaseBarnesHut.run
 * (base.py:104-127) with evaluation_rounds = 1. */
int bh_step(bh_plan *plan, int nsteps, void *stream);

/* bh_step captured once into a CUDA graph (per nsteps value) and replayed. */
int bh_step_graph(bh_plan *plan, int nsteps, void *stream);

/* Number of kernels one bh_step round launches (host only; no reference
 * counterpart: the reference launches 6 Numba kernels per round,
 * singlegpu.py:41-99). */
int bh_kernels_per_step(const bh_plan *plan, int *count);

/* Kernel nodes of the step graph bh_step_graph captured last (its nsteps
 * rounds); BH_ERR_INVALID before the first capture.  Host only; no reference
 * counterpart. */
int bh_graph_kernel_nodes(const bh_plan *plan, int *count);

/* Synchronise the stream and read (then clear) the device error flags. */
int bh_error_flags(bh_plan *plan, unsigned *flags, void *stream);

/* Pair interactions of the last force evaluation, counted exactly by the
 * force kernel: near = particle-particle, far = particle-cell (synchronises). */
int bh_pair_counts(bh_plan *plan, long long *near_pairs, long long *far_pairs, void *stream);

/* (target, cell) pairs the learned correction evaluated in the last step or evaluate
 * (synchronises); no reference counterpart. */
int bh_corrected_pairs(bh_plan *plan, long long *pairs, void *stream);

/* Leaf-box centres of mass of system `sys` from the last bh_summarize, in the
 * reference's layout: out[(gx * G + gy) * 3 + {0, 1, 2}] = (cx, cy, M), zeros
 * for an empty box (device array of G*G*3 doubles).  Replaces reading the
 * COM grid d_COMs (singlegpu.py:38,69-77; gpu/grid.py:78-114). */
int bh_box_moments(bh_plan *plan, int sys, double *out, void *stream);

/* A plan over one rank's part of a larger system (the box-slab step that replaces
 * implementations/multigpu.py:264-310).  bh_set_grid fixes system `sys`'s grid: from the next
 * bh_create_tree on, the square box comes from ext[4] = {min x, min y, max x, max y} of the
 * whole system (host doubles; the all-reduce of the ranks' extents) instead of from the
 * plan's own particles; ext = NULL returns to the plan's own box.  bh_leaf_moments copies the
 * last summarize's leaf moments of `sys` -- per box, x-major, (M, Sx, Sy, Sxx, Sxy, Syy) about
 * the box origin, FP64; the second moments only for a plan with BH_FLAG_LEARNED, zeros
 * otherwise -- into out (device, G*G*6 doubles); bh_set_leaf_moments replaces them
 * with `in` (device, same layout: the sum over ranks of their own boxes' moments) and rebuilds
 * the pyramid levels above the leaves and the cell records, so the next bh_evaluate takes its
 * far field from the whole system (multigpu.py:149-155, 303-306). */
int bh_set_grid(bh_plan *plan, int sys, const double *ext, void *stream);
int bh_leaf_moments(bh_plan *plan, int sys, double *out, void *stream);
int bh_set_leaf_moments(bh_plan *plan, int sys, const double *in, void *stream);

/* Square bounding box of system `sys` from the last bh_create_tree into host
 * out[5] = {min_x, min_y, step, grid_dim, n} (synchronises).  Replaces the
 * attributes min_xy, step, grid_dim that set_particles_bounding_box sets
 * (base.py:211-239). */
int bh_grid_info(bh_plan *plan, int sys, double *out, void *stream);

/* Kernel timing, no reference counterpart (the reference's Timer measures whole phases,
 * timer/timer.py).  With enable != 0, each later eager bh_evaluate records two CUDA events on
 * its stream, right before and after the force kernel proper (after the interaction lists and
 * the work-item order of the list-streaming path); bh_force_kernel_ms waits for the second
 * event and returns the last such launch's duration in milliseconds.  Graph replays
 * (bh_step_graph) and bh_step record nothing. */
int bh_set_kernel_timing(bh_plan *plan, int enable);
int bh_force_kernel_ms(bh_plan *plan, float *ms);

/* FP64 direct sum on the device for nt targets (indices into the
 * concatenated pid order, device array) of system `sys`, no cutoff, the
 * plan's softening: a_t = G sum_{j != t} m_j (x_j - x_t) / (r^2 + eps^2).
 * Outputs ax, ay (device, nt doubles).  Replaces nsquared_acc_check
 * (base.py:16-32) of the --check accuracy sampler (base.py:149-205). */
int bh_direct_sample(bh_plan *plan, int sys, const long long *targets, long long nt,
                     double *ax, double *ay, void *stream);

/* Direct-sum sampler that allocates nothing.  No counterpart in the reference:
 * it is the FP64 direct sum of bh_direct_sample for callers that cannot
 * allocate device memory (and so cannot bind a plan workspace) -- e.g. code
 * inside another framework that has reserved the whole device for its own
 * memory pool.  Inputs are plain device arrays: positions x, y and masses m
 * of n particles (any order), nt target indices into them (device
 * long longs); outputs ax, ay (device, nt doubles):
 *   a_t = grav_constant * sum_{j != t} m_j (x_j - x_t) / (r^2 + softening^2).
 * Scratch (the per-chunk partial sums of every target) lives in a static
 * device array of BH_NOALLOC_MAX_TARGETS x BH_NOALLOC_CHUNKS x 2 doubles (4 MiB)
 * that every GPU loading the library holds until the process exits; more
 * than BH_NOALLOC_MAX_TARGETS targets is rejected with BH_ERR_INVALID.  The
 * array's device address belongs to one CUDA context: the first call in a
 * context (the current one, or the device's primary context if none is
 * current) looks it up with that context current and caches it under the
 * context's process-unique ID, so a context made after cudaDeviceReset looks
 * it up again; make the first call in a context before any stream capture.  All
 * calls share the array: calls that overlap on the GPU (e.g. on two streams)
 * race and must be ordered by the caller.  bh_last_error(NULL) describes a
 * failure. */
#define BH_NOALLOC_MAX_TARGETS 4096
#define BH_NOALLOC_CHUNKS 64
int bh_direct_sum_noalloc(const double *x, const double *y, const double *m, long long n,
                          const long long *targets, long long nt, double grav_constant,
                          double softening, double *ax, double *ay, void *stream);

/* FP64 diagnostics of system `sys` into out[4] (device doubles):
 * kinetic energy, momentum x, momentum y, and the potential energy
 * sum_{i<j} G m_i m_j ln(sqrt(r^2 + eps^2)) by an FP64 direct sum (O(n^2):
 * pass want_potential = 0 to skip it for large n).  No reference
 * counterpart (the reference reports no energies). */
int bh_diagnostics(bh_plan *plan, int sys, int want_potential, double *out, void *stream);

/* ---- learned far-field correction (no reference counterpart: python-bh has
 * no learned component).  A 6 -> 64 -> 64 -> 64 -> 2 GELU MLP with BF16
 * weights and activations and FP32 accumulation on the 5th-generation tensor
 * cores.  Parameters are FP32 "master" values in global memory
 * (bh_mlp_param_count floats); bh_mlp_pack converts them to the BF16 operand
 * images (bh_mlp_image_bytes bytes) the kernels stage into shared memory.
 * Feature rows are 6 floats at a stride of feat_stride floats; outputs and
 * targets are 2 floats per row.  err points at a device unsigned that
 * receives BH_DEV_WAIT_TIMEOUT if a bounded tensor-core wait gave up. */
int bh_mlp_param_count(void);
int bh_mlp_image_bytes(void);
int bh_mlp_pack(const float *params, void *image, void *stream);
int bh_mlp_forward(const float *feats, int feat_stride, long long rows, const void *image,
                   const float *params, float *out, unsigned *err, void *stream);
/* Accumulate d(loss)/d(params) of loss = mean((y - target)^2) over the rows
 * into grad (FP32, device, zeroed by bh_mlp_adam) and the summed squared
 * error into *loss (device float). */
int bh_mlp_train_batch(const float *feats, int feat_stride, const float *targets,
                       long long rows, const void *image, const float *params, float *grad,
                       float *loss, unsigned *err, void *stream);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8) on params with moments m, v;
 * zeroes grad.  step counts from 1. */
int bh_mlp_adam(float *params, float *m, float *v, float *grad, int step, float lr, void *stream);

/* Bind the MLP (image from bh_mlp_pack, FP32 parameters; the caller keeps
 * both alive) that bh_evaluate and bh_step apply when params.flags has
 * BH_FLAG_LEARNED: the cells accepted at params.theta but not at
 * params.correction_theta get a += G M / s * MLP(features) per target. */
int bh_set_correction(bh_plan *plan, const void *image, const float *params);

/* Training pairs made by the method on the current state (after
 * bh_create_tree and bh_summarize): for work items item_offset + k *
 * item_stride, the cells accepted at theta_hi but not at theta_lo up to
 * pyramid level max_level, and targets_per_item targets of each item, one
 * row per (target, cell): 8 features (u, v, qxx, qxy, qyy, w, level, 0) and 2
 * targets ((exact sum over the cell's particles - monopole) * s / M, FP64
 * sums), appended at rows atomicAdd(counter) < capacity. */
int bh_learned_pairs(bh_plan *plan, double theta_hi, double theta_lo, int max_level,
                     long long item_offset, long long item_stride, int targets_per_item,
                     float *feats, float *targets, unsigned *counter, long long capacity,
                     void *stream);

/* ------------------------------------------------------------ input generators
 * Replaces python-bh/bin/gen_input.py:38-55 (per-particle host loop) with a device
 * generator: n particles into caller-owned device arrays (FP64), a pure function of
 * (distribution, n, seed) -- Philox4x32-10 counters per particle.
 *   BH_GEN_UNIFORM: x, y uniform in [0, 499) (gen_input.py "normal"), v uniform in
 *                   [-1, 1), m uniform in [0.5, 5)
 *   BH_GEN_GAUSS:   x, y ~ N(249.5, (499 / 12)^2) (gen_input.py "gauss"), v and m as above
 *   BH_GEN_CLUSTER: 8 Gaussian clusters (sigma 0.05, centres uniform in [0.2, 0.8)^2) with
 *                   20 % uniform background on [0, 1)^2, m uniform in [1, 2), v = 0
 * No plan needed; asynchronous on stream; errors via bh_last_error(NULL). */
#define BH_GEN_UNIFORM 0
#define BH_GEN_GAUSS 1
#define BH_GEN_CLUSTER 2
int bh_generate(int distribution, long long n, unsigned long long seed, double *x, double *y,
                double *m, double *vx, double *vy, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* BH_GB300_H */

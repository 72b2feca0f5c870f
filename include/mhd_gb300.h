/*
 * mhd_gb300 — GB300 (sm_103a) implementation of the relaxing-TVD split MHD
 * step of uelipen/Heterogeneous_MHD, behind the reference's own C call
 * surface.
 *
 * Data layout everywhere (C/array_definition.h:12-13): u(5,nx,ny,nz) holds
 * (rho, rho vx, rho vy, rho vz, E) and b(3,nx,ny,nz) the face-staggered field,
 * Fortran order with the component innermost: element ((k*ny+j)*nx+i)*nc+c.
 * Boundaries are periodic.
 *
 * Two layers:
 *   1. Drop-in functions with the reference's names and signatures
 *      (C/spu_function.h:1-15).  A C driver written against the reference
 *      (C/mhd.c) links against this library unchanged.  Pointers may be
 *      device pointers (fast) or host pointers (staged through a cached
 *      device mirror, for correctness only).  Each call is synchronous, like
 *      the reference.  Errors never exit(): they are recorded for
 *      mhd_last_error().
 *   2. A context API (mhd_create ... mhd_step) that owns device state,
 *      runs the whole Strang step asynchronously on one stream, optionally as
 *      a captured CUDA graph, with dt kept on the device.
 */
#ifndef MHD_GB300_H
#define MHD_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define MHD_API __attribute__((visibility("default")))

/* ------------------------------------------------------------ status codes */
#define MHD_OK 0
#define MHD_ERR_ARG 1         /* bad argument (null pointer, bad size, nx != nz for transpose13) */
#define MHD_ERR_CUDA 2        /* a CUDA runtime call failed */
#define MHD_ERR_TIMEOUT 3     /* a bounded device-side wait gave up */
#define MHD_ERR_NONFINITE 4   /* the CFL reduction met a NaN cell */
#define MHD_ERR_UNSUPPORTED 5 /* shape or mode not supported by this build */
#define MHD_ERR_NOMEM 6       /* device allocation failed */

/* ------------------------------------------------------- 1. drop-in layer */

/* fluidx (C/spu_function.h:1, C/fluidx.c:19): u <- relaxing-TVD x-sweep of
 * update_u, with the cell-centred field built from update_b.  b and iter are
 * unused, as in the reference. */
MHD_API void fluidx(float *u, float *b, int *nx, int *ny, int *nz, float *dt, float *update_u,
                    float *update_b, int iter);

/* copy_matrix (C/spu_function.h:3, C/copy_matrix.c:9): update_u <- u, update_b <- b. */
MHD_API void copy_matrix(float *u, float *b, int *nx, int *ny, int *nz, float *update_u,
                         float *update_b);

/* advectbyzx (C/spu_function.h:5, C/advectbyzx.c:14): constrained-transport
 * advection of b(2) and b(3) along x (A1/A2/B1/B2).  Reads update_u and
 * update_b; b(1) is read from b itself and updated in place, b(2), b(3) are
 * overwritten.  u is unused. */
MHD_API void advectbyzx(float *u, float *b, int *nx, int *ny, int *nz, float *dt, float *update_u,
                        float *update_b);

/* transpose12 (C/spu_function.h:7, C/transpose12.c:7): (u,b) with dims
 * (ny,nx,nz) <- update_* with dims (nx,ny,nz), x<->y swapped, components
 * permuted u:(1,3,2,4,5) b:(2,1,3). */
MHD_API void transpose12(float *u, float *b, float *update_u, float *update_b, int *nx, int *ny,
                         int *nz, int iter);

/* transpose13 (C/spu_function.h:9, C/transpose13.c:9): x<->z swap, u:(1,4,3,2,5)
 * b:(3,2,1).  Only nx == nz, like the reference; otherwise the outputs are
 * left untouched and MHD_ERR_ARG is recorded. */
MHD_API void transpose13(float *u, float *b, float *update_u, float *update_b, int *nx, int *ny,
                         int *nz);

/* calcfl (C/spu_function.h:15, C/calcfl.c:13): returns 1/max_c over all cells. */
MHD_API float calcfl(float *u, float *b, int *nx, int *ny, int *nz);

/* Status of the last drop-in call made by this thread (MHD_OK or an error). */
MHD_API int mhd_last_error(void);
MHD_API const char *mhd_error_string(int status);

/* Arithmetic of the drop-in calls: MHD_MODE_FAST (default) or MHD_MODE_EXACT.
 * The environment variable MHD_GB300_MODE=exact selects EXACT at first use. */
MHD_API int mhd_set_dropin_mode(int mode);

/* ------------------------------------------------------ 2. context layer */

typedef struct mhd_ctx mhd_ctx;

/* flags for mhd_create */
#define MHD_F32 0         /* float state (the reference's type) */
#define MHD_F64 1         /* double state (the reference built with -Dfloat=double) */
#define MHD_MODE_FAST 0   /* FP32 with FMA contraction and reciprocal multiplies */
#define MHD_MODE_EXACT 2  /* reproduces the reference's float/double promotions and
                             evaluation order bit for bit (no contraction) */

/* where a buffer lives */
#define MHD_HOST 0
#define MHD_DEVICE 1

/* step variants */
#define MHD_PLAIN 0 /* drop-in kernel sequence with ping-pong buffers */
#define MHD_FUSED 1 /* transpose-free sweep kernels (shared-memory transposes) */

MHD_API int mhd_create(mhd_ctx **out, int nx, int ny, int nz, int flags);
MHD_API int mhd_destroy(mhd_ctx *ctx);
MHD_API void *mhd_stream(mhd_ctx *ctx); /* the cudaStream_t all work is queued on */
MHD_API int mhd_sync(mhd_ctx *ctx);

/* Per-operator calls on device pointers, queued on the context stream.  The
 * element type is the context's precision.  Semantics as the drop-in layer. */
MHD_API int mhd_op_fluidx(mhd_ctx *ctx, void *u, const void *update_u, const void *update_b, int nx,
                          int ny, int nz, double dt);
MHD_API int mhd_op_advectbyzx(mhd_ctx *ctx, void *b, const void *update_u, const void *update_b,
                              int nx, int ny, int nz, double dt);
MHD_API int mhd_op_transpose12(mhd_ctx *ctx, void *u, void *b, const void *update_u,
                               const void *update_b, int nx, int ny, int nz);
MHD_API int mhd_op_transpose13(mhd_ctx *ctx, void *u, void *b, const void *update_u,
                               const void *update_b, int nx, int ny, int nz);
MHD_API int mhd_op_copy(mhd_ctx *ctx, const void *u, const void *b, void *update_u, void *update_b,
                        int nx, int ny, int nz);
/* Synchronous: writes 1/max_c (as the reference returns it) to *inv_cmax. */
MHD_API int mhd_op_calcfl(mhd_ctx *ctx, const void *u, const void *b, int nx, int ny, int nz,
                          double *inv_cmax);

/* Owned state.  mhd_set_state copies (u,b) in (from host or device memory)
 * and resets the clock to t = 0. */
MHD_API int mhd_set_state(mhd_ctx *ctx, const void *u, const void *b, int where);
MHD_API int mhd_get_state(mhd_ctx *ctx, void *u, void *b, int where);
/* Device pointers of the current state (valid until the next mhd_step). */
MHD_API int mhd_state_ptrs(mhd_ctx *ctx, void **u, void **b);
/* device address of the step clock: 4 values of the state's precision (t, tf, dt, 1/c),
 * written on the context stream by every step */
MHD_API int mhd_clock_ptr(mhd_ctx *ctx, void **clock);

/* nsteps full Strang steps x(F,A) T12 y(F,A) T13 z(F,A,A,F) T13 y(A,F) T12 x(A,F)
 * (C/mhd.c:59-124) with dt = cfl * calcfl, clamped so that t never passes tf
 * (set by mhd_set_time; +inf by default).  Asynchronous. */
MHD_API int mhd_step(mhd_ctx *ctx, int nsteps, double cfl, int variant);
/* nsteps steps (as mhd_step) on a state held in host memory, which is what
 * the reference's loop does (C/mhd.c:59-124 on the host arrays u, b): u
 * (5*nx*ny*nz) and b (3*nx*ny*nz) are copied in, stepped, and the result is
 * written back into them before the call returns.  The copies overlap the
 * step (the first CFL pass runs on each chunk of the state as it arrives, b
 * goes back out while the last fluidx runs); pinned host memory gives the
 * full host-link bandwidth.  Equivalent to mhd_set_state, mhd_step and
 * mhd_get_state, bit for bit, except that the context's clock (t, step
 * count) carries on instead of restarting at t = 0. */
MHD_API int mhd_step_host(mhd_ctx *ctx, void *u, void *b, int nsteps, double cfl, int variant);
MHD_API int mhd_set_time(mhd_ctx *ctx, double t, double tf);
MHD_API int mhd_get_time(mhd_ctx *ctx, double *t, double *dt, long long *steps);
/* Capture each step variant into a CUDA graph on first use (default on). */
MHD_API int mhd_use_graphs(mhd_ctx *ctx, int enable);
/* Synchronises and returns MHD_OK or the first device-side error recorded. */
MHD_API int mhd_check(mhd_ctx *ctx);
/* Clears the device-side error word (synchronous). */
MHD_API int mhd_clear_errors(mhd_ctx *ctx);
/* Self-test of the bounded device waits: queues a one-warp kernel that waits
 * on a barrier nothing completes and gives up after `seconds` (0 < s <= 2),
 * so that the next mhd_check returns MHD_ERR_TIMEOUT; the context stays
 * usable (mhd_clear_errors, then step as usual).  No reference counterpart:
 * the reference's CUDA path exits on any error (Cuda/cuda_function.h:4-12). */
MHD_API int mhd_selftest_wait(mhd_ctx *ctx, double seconds);

/* Per-kernel timing with CUDA events on the context stream (off by default;
 * while on, steps run as direct launches).  Kernel ids: */
#define MHD_K_CALCFL 0
#define MHD_K_FLUIDX 1
#define MHD_K_ADVECT 2
#define MHD_K_TRANSPOSE12 3
#define MHD_K_TRANSPOSE13 4
#define MHD_K_COPY 5
#define MHD_K_FINALIZE 6
#define MHD_K_SWEEP 7
#define MHD_K_COUNT 8
MHD_API int mhd_profile(mhd_ctx *ctx, int enable);
MHD_API int mhd_profile_read(mhd_ctx *ctx, int kernel, double *total_ms, long long *launches);
MHD_API int mhd_profile_reset(mhd_ctx *ctx);
/* Kernel launches made since the context was created (all kernels). */
MHD_API long long mhd_launch_count(mhd_ctx *ctx);

/* Launch-shape knobs consulted by the kernel planners, for the autotuner
 * (heterogeneous_mhd_gb300/autotune.py).  Keys: "fluidx.threads" (threads
 * per CTA of the register-resident fluidx: 64, 128 or 256), "advect.cells"
 * (cells per thread of the marching advectbyzx: 4 or 8), "advect.slots"
 * (plane-slab ring depth: 2 or 3; chunk buffers of the x-walking kernel),
 * "advect.J" (pencils per CTA), "advect.K" (planes per CTA), "fluidx.cells"
 * (4, or 8: one warp per pencil), "advect.kernel" (3: the marching
 * advectbyzx, 4: the x-walking one), "advect.xk" (planes per CTA of the
 * x-walking kernel: 2, 4 or 8), and for the fused step's sweeps along y and z
 * "sweep.kernel" (5: the sweep-walking advectbyzx, 3: the marching one),
 * "sweep.k" (its planes per CTA: 2, 4 or 8) and "sweep.slots" (its chunk
 * buffers: 2 or 3).  0 restores the planner's own choice; a value that does
 * not fit the grid is ignored.  Captured step graphs are rebuilt on the next
 * mhd_step.  mhd_tune_get returns the current value (-1 for an unknown key). */
MHD_API int mhd_tune_set(const char *key, int value);
MHD_API int mhd_tune_get(const char *key);

/* Run diagnostics of the current state, reduced on the device in FP64
 * (synchronous): out[MHD_DIAG_COUNT] in the order below.  B_c is the
 * cell-centred field (mean of the two faces of the cell), p = (5/3 - 1) *
 * (E - |m|^2/(2 rho) - |B_c|^2/2).  A NaN density or pressure propagates into
 * the minima.  No reference counterpart (the reference prints two sample
 * values per step, C/mhd.c:66). */
#define MHD_DIAG_MIN_RHO 0
#define MHD_DIAG_MIN_P 1
#define MHD_DIAG_MAX_DIVB 2
#define MHD_DIAG_MASS 3
#define MHD_DIAG_KINETIC 4
#define MHD_DIAG_MAGNETIC 5
#define MHD_DIAG_ENERGY 6
#define MHD_DIAG_MAX_SPEED 7
#define MHD_DIAG_COUNT 8
MHD_API int mhd_diagnostics(mhd_ctx *ctx, double *out);

/* max |div B| of the current state, computed on the device (synchronous). */
MHD_API int mhd_divb_max(mhd_ctx *ctx, double *out);

/* 1/max_c of calcfl without any device allocation.  No counterpart in the
 * reference: it is for callers that cannot let a library allocate device
 * memory (inside a CUDA-graph stream capture, under a host framework that owns
 * all device memory, or in a loop that must not enter the allocator).  Its
 * scratch is a fixed file-scope device array (768 KB per device, held until the
 * process exits).  u, b and inv_cmax are device pointers; the two kernels are
 * queued on `stream` (a cudaStream_t, NULL for the default stream) and
 * *inv_cmax is written when the stream reaches them.  It always computes with
 * the FAST arithmetic (FP32 with contraction), whatever MHD_GB300_MODE or a
 * context's flags say.  Grids of more than 134,217,728 cells (512^3) return
 * MHD_ERR_UNSUPPORTED.  The first call on a device looks up the array's
 * address and should come before any stream capture; the address is kept for
 * the life of the process, so calling it after cudaDeviceReset is not
 * supported.  All calls share the array: calls that overlap on the GPU race. */
MHD_API int mhd_calcfl_noalloc(const float *u, const float *b, int nx, int ny, int nz, float *inv_cmax,
                               void *stream);

/* ------------------------------------------------------------ batched boxes */

/* Many independent periodic cubes advanced together, each with its own dt.
 * No counterpart in the reference, whose driver runs one box per process
 * (C/mhd.c:18-128); each box takes exactly the steps mhd_step takes on it.
 * Boxes of equal edge share a size class whose states are contiguous, so each
 * operator of the step is one launch per class; a whole step of every class is
 * one CUDA graph.  sizes[i] is the edge of box i (1..512); flags as mhd_create.
 * Every box must be loaded with mhd_batch_set_box (which also resets its clock
 * to t = 0) before mhd_batch_step.  Boxes are never clamped to a final time. */
typedef struct mhd_batch mhd_batch;
MHD_API int mhd_batch_create(mhd_batch **out, int nboxes, const int *sizes, int flags);
MHD_API int mhd_batch_destroy(mhd_batch *batch);
MHD_API int mhd_batch_set_box(mhd_batch *batch, int box, const void *u, const void *b, int where);
MHD_API int mhd_batch_get_box(mhd_batch *batch, int box, void *u, void *b, int where);
MHD_API int mhd_batch_step(mhd_batch *batch, int nsteps, double cfl);
MHD_API int mhd_batch_sync(mhd_batch *batch);  /* also reports device-side errors */
MHD_API int mhd_batch_time(mhd_batch *batch, int box, double *t, double *dt);
MHD_API void *mhd_batch_stream(mhd_batch *batch);
MHD_API long long mhd_batch_launch_count(mhd_batch *batch);
MHD_API int mhd_batch_classes(mhd_batch *batch);
/* Launch-shape knob (the names of mhd_tune_set) for the launches of the boxes
 * of one edge only; -1 returns that knob to the global setting.  No
 * counterpart in the reference (see mhd_batch_create). */
MHD_API int mhd_batch_tune_edge(mhd_batch *batch, int edge, const char *key, int value);
/* Work-list launches (on by default): the FP32 classes of edge 32, 48, 64, 96
 * and 128 (up to eight classes, the largest by cells when there are more) step
 * together, each operator of the step one launch that walks the (class, box,
 * tile) list of all of them: 17 launches per step for the whole group instead
 * of 17 per class.  A class given its own launch shapes by
 * mhd_batch_tune_edge keeps its own launches.  Off: one launch per class and
 * operator.  The results are the same bit for bit either way.
 * mhd_batch_worklist_classes returns how many classes the work list holds.
 * No counterpart in the reference, whose driver runs one box per process
 * (C/mhd.c:18-128). */
MHD_API int mhd_batch_set_worklist(mhd_batch *batch, int on);
MHD_API int mhd_batch_worklist_classes(mhd_batch *batch);

/* ------------------------------------------------- initial conditions (host) */

/* Orszag-Tang-like vortex: rho = rho0, p = p0,
 * v = vscale (-sin 2pi y, sin 2pi x, 0.1 sin 2pi z) + noise N(0,1) per component,
 * B = bscale (-sin 2pi y, sin 4pi x, 0)/sqrt(4pi) on faces (div B = 0). */
MHD_API int mhd_init_vortex(void *u, void *b, int nx, int ny, int nz, int fp64,
                            unsigned long long seed, double rho0, double p0, double vscale,
                            double noise, double bscale);
/* Decaying-turbulence cube of side n: Gaussian random velocity with shell
 * spectrum k^-2 on kmin <= |k| <= kmax scaled to rms Mach `mach`, and
 * B = bx0 x + curl A with A of spectrum k^-3, scaled to rms |dB| = dbrms,
 * evaluated as a discrete curl on the staggered grid (div B at round-off). */
MHD_API int mhd_init_turbulence(void *u, void *b, int n, int fp64, unsigned long long seed,
                                double rho0, double p0, double mach, double bx0, double dbrms,
                                int kmin, int kmax);
MHD_API double mhd_host_divb_max(const void *b, int nx, int ny, int nz, int fp64);

#ifdef __cplusplus
}
#endif
#endif /* MHD_GB300_H */

/*
 * stencil_dispatch.h -- C ABI of libstencil_gb300.so, the GB300 (sm_103a)
 * iterative star-stencil sweep library.
 *
 * Plain C: no C++ or CUDA types cross the boundary.  A stream is passed as
 * stencil_stream_t, which is ABI-identical to cudaStream_t (NULL = the legacy
 * default stream).  Every entry point returns STENCIL_OK (0) or a negative
 * STENCIL_E* status; none of them exits the process.
 *
 * Grid layout (same as the reference, src/stencil_kernel_base.cu:14): FP32,
 * x fastest, idx = i + j*nx + k*nx*ny.  A sweep updates exactly the cells whose
 * every coordinate lies in [R, N-R) (src/stencil_border_check.cu:6-44) and
 * never writes any other cell ("the border band").
 */
#ifndef STENCIL_DISPATCH_H
#define STENCIL_DISPATCH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define STENCIL_ABI_VERSION 1

typedef struct CUstream_st *stencil_stream_t;

#if defined(__GNUC__)
#define STENCIL_API __attribute__((visibility("default")))
#else
#define STENCIL_API
#endif

/* Status codes. */
enum {
    STENCIL_OK = 0,
    STENCIL_EINVAL = -1,       /* bad parameter, shape or pointer alignment */
    STENCIL_ENOMEM = -2,       /* device or pinned-host allocation failed */
    STENCIL_ECUDA = -3,        /* a CUDA runtime call failed (see stencil_last_error) */
    STENCIL_ETIMEOUT = -4,     /* a bounded device-side wait gave up */
    STENCIL_EUNSUPPORTED = -5, /* valid request that this build cannot serve */
    STENCIL_ENODEVICE = -6     /* no CUDA device of compute capability 10.3 */
};

/* Update rule. */
enum {
    /* u' = (sum of the 2*D*R axis neighbours)/(float)(2*D*R) - u: the reference
     * formula (src/stencils.cu:18).  The border band of each buffer is whatever
     * the caller put there (the reference leaves its second buffer as allocated). */
    STENCIL_MODE_LEGACY = 0,
    /* u' = (sum of the 2*D*R axis neighbours)/(float)(2*D*R): Jacobi for the
     * Laplace-type steady state with fixed Dirichlet borders.  The caller keeps
     * the border band equal in both buffers (stencil_copy_border). */
    STENCIL_MODE_JACOBI = 1
};

/* Kernel family.  The first five name the reference's variants
 * (src/stencil_dispatch.cu:14-42); all of them produce bit-identical results
 * because every kernel keeps the reference's per-cell summation order. */
enum {
    STENCIL_VARIANT_AUTO = 0,          /* library picks (tuning database, then heuristic) */
    STENCIL_VARIANT_BASE = 1,          /* one sweep per launch, 128-bit vector loads */
    STENCIL_VARIANT_SMEM = 2,          /* TMA-staged shared-memory tile with halo */
    STENCIL_VARIANT_SMEM_PADDED = 3,   /* same kernel as SMEM */
    STENCIL_VARIANT_SMEM_REGISTER = 4, /* 2.5D stream along the slowest axis */
    STENCIL_VARIANT_COOP = 5,          /* all sweeps in one cooperative launch; 3-D: one
                                          sweep per HBM pass (temporal 0 or 1; block_z
                                          1..6 = a stream-kernel shape with a
                                          persistent form) or `temporal` (>= 2, JACOBI,
                                          R <= 2) per pass;
                                          2-D grids of at most one tile per SM: every SM,
                                          `temporal` sweeps per halo exchange, tile
                                          block_x * coarsen_x by block_y cells (0: chosen);
                                          larger 2-D grids: a grid barrier per sweep
                                          (nx % 4 == 0, R <= 4); 3-D grids that fit
                                          one cluster's shared memory go to CLUSTER */
    STENCIL_VARIANT_CLUSTER = 6        /* all sweeps on one thread-block cluster: the grid
                                          resident in its shared memory when it fits, else
                                          swept from L2/HBM (nx % 4 == 0, R <= 4; other
                                          shapes fall back to COOP) */
};

/* Runtime description of one sweep loop.  Zero in a tuning field means "choose". */
typedef struct stencil_params {
    int dims;        /* 2 or 3 */
    int nx, ny, nz;  /* extents; nz is ignored for dims == 2 */
    int radius;      /* R >= 1, 2R < every extent */
    int iterations;  /* sweeps, >= 0 */
    int mode;        /* STENCIL_MODE_* */
    int variant;     /* STENCIL_VARIANT_* */
    int block_x, block_y, block_z; /* thread-block shape hint */
    int coarsen_x;   /* cells per thread along x (vector kernels use multiples of 4) */
    int temporal;    /* sweeps per pass (3-D) or per exchange (2-D) for STENCIL_VARIANT_COOP */
    int reserved[4]; /* must be zero */
} stencil_params;

/* Fills *p with the reference's compile-time defaults
 * (3-D, 256^3, R=1, 64 sweeps, LEGACY, AUTO). */
STENCIL_API int stencil_params_init(stencil_params *p);

/* Validates *p without touching the device. */
STENCIL_API int stencil_params_check(const stencil_params *p);

/* The sweep loop.  Replaces dispatch_kernels(float*, float*)
 * (src/stencil_dispatch.cu:138-158) and the never-launched cooperative
 * dispatch (src/stencil_dispatch.cu:160-177).
 *   d_u1  device buffer holding the initial state (read, and overwritten as
 *         ping-pong scratch)
 *   d_u2  device buffer of the same size (ping-pong scratch; its border band
 *         is read, never written)
 * Runs asynchronously on `stream` and writes to *d_result (if non-NULL) which
 * of d_u1 / d_u2 holds the state after the last sweep.  Allocates nothing,
 * except that the 2-D temporally blocked engine (COOP or AUTO on small 2-D
 * grids) keeps a per-device exchange buffer, grown on first use (outside a
 * CUDA graph capture: run such a dispatch once before capturing it) and freed
 * by stencil_release().
 * Both buffers must be 16-byte aligned (cudaMalloc gives 256). */
STENCIL_API int stencil_dispatch_ex(const stencil_params *p, float *d_u1, float *d_u2,
                        stencil_stream_t stream, float **d_result);

/* End to end through host memory, the flow of src/main.cu:33-89: copies h_in
 * into device buffer 1, fills buffer 2 (LEGACY: zero, like the reference's
 * fresh cudaMalloc; JACOBI: a copy of h_in, so the border band is equal), runs
 * the sweeps, copies the final state into h_out and synchronises.  Device
 * buffers come from a per-device workspace that is kept for later calls and
 * freed by stencil_release().  *ms (if non-NULL) receives the time between
 * the start of the upload and the end of the download. */
STENCIL_API int stencil_run_host(const stencil_params *p, const float *h_in, float *h_out, float *ms);

/* stencil_run_host with two clocks: *ms_total (if non-NULL) as above, and
 * *ms_sweeps (if non-NULL) the time of the sweeps alone -- the interval the
 * reference's binary prints as its last stdout line (events around
 * dispatch_kernels, src/main.cu:58-72 and :89). */
STENCIL_API int stencil_run_host_timed(const stencil_params *p, const float *h_in, float *h_out,
                                       float *ms_total, float *ms_sweeps);

/* Device-side initial states (same generators as the CPU oracle). */
/* include/stencil_initializer.h:6-52: outermost layer 1.0f, everything else 0. */
STENCIL_API int stencil_init_reference(const stencil_params *p, float *d_u, stencil_stream_t stream);
/* count cells i.i.d. uniform [0,1): value(i) = (mix64(mix64(seed) + G*(i+1)) >> 40) * 2^-24,
 * mix64 = the SplitMix64 finaliser, G = 0x9E3779B97F4A7C15. */
STENCIL_API int stencil_init_uniform(float *d_u, size_t count, uint64_t seed, stencil_stream_t stream);
/* Border band: sum of `modes` (<= 16) smooth modes A cos(2 pi (a x/nx + b y/ny
 * + c z/nz) + phi), a, b, c in {0..3}, A ~ N(0,1), phi ~ U[0, 2 pi); interior:
 * uniform [0,1) as stencil_init_uniform(seed).  Parameters are drawn from
 * `seed` on the host; values evaluated in double and rounded to float. */
STENCIL_API int stencil_init_fourier(const stencil_params *p, float *d_u, uint64_t seed, int modes,
                                     stencil_stream_t stream);
/* 2-D Laplace borders: per edge, the linear interpolation of its two corner
 * values (N(0,1)) plus sum_{k=1..K} A_k sin(pi k t), K ~ U{1..16}, A_k ~ N(0,1),
 * t in [0,1] along the edge (continuous at the corners).  Interior zero. */
STENCIL_API int stencil_init_laplace2d(const stencil_params *p, float *d_u, uint64_t seed,
                                       stencil_stream_t stream);
/* Copies the border band of src into dst (JACOBI set-up). */
STENCIL_API int stencil_copy_border(const stencil_params *p, const float *d_src, float *d_dst,
                        stencil_stream_t stream);

/* ---- Batched persistent sweeps: many grids of uneven sizes and sweep counts
 * in ONE launch over a device work queue (no counterpart in the reference,
 * which runs one grid per process).  Each job is one grid with its own two
 * buffers; after the launch its result is in d_u1 for an even sweep count and
 * in d_u2 for an odd one, as the ping-pong loop leaves it (the other buffer
 * holds an earlier state).  Jobs need radius <= 4; a job whose nx is not a
 * multiple of 4 (rows not 16-byte aligned) is swept in a copy with the row
 * pitch rounded up to 4 cells, held in the workspace and copied in and out by
 * stencil_batch_launch. */
typedef struct stencil_batch_job {
    float *d_u1, *d_u2;
    int dims, nx, ny, nz;
    int radius, iterations, mode;
    /* Tuning hints (0 = the library's choice), as an autotuner sets them:
     * temporal: sweeps between halo exchanges -- for a job kept in a
     * cluster's shared memory the most it may use (the largest of 8, 4, 2, 1
     * at most this that fits), for a 2-D job with a whole-GPU launch the
     * temporally blocked engine's depth, and for a 3-D one with a whole-GPU
     * launch >= 2 selects the temporally blocked kernel with that depth (R
     * <= 2, JACOBI; else the one-sweep-per-pass stream kernel);
     * tile_x, tile_y: the 2-D whole-GPU engine's tile in cells.
     * These three are used by the phased engine.  team: the CTAs the
     * one-launch engine gives this grid (rounded down to one of its team
     * sizes, the device's CTA count halved repeatedly; 0 = from the grid's
     * cells), ignored by the phased engine. */
    int temporal, tile_x, tile_y;
    int team;
    int reserved[2]; /* must be zero */
} stencil_batch_job;

/* Device workspace bytes for njobs jobs whose nx are multiples of 4 (a job
 * table and the queue counter). */
STENCIL_API int stencil_batch_workspace_bytes(int njobs, size_t *bytes);
/* Device workspace bytes for these jobs: the job table and the pitched copies
 * of the jobs whose nx is not a multiple of 4. */
STENCIL_API int stencil_batch_workspace_bytes_for(const stencil_batch_job *jobs, int njobs,
                                                  size_t *bytes);
/* Validates the jobs, orders them largest first and writes the job table into
 * d_workspace (256-byte aligned, caller-owned).  cluster_size: CTAs per
 * cluster (1, 2, 4, 8 or 16; 0 = the largest the device schedules; 1 suits
 * many small grids, each then swept by one CTA).  Synchronises
 * `stream`. */
STENCIL_API int stencil_batch_prepare(const stencil_batch_job *jobs, int njobs, int cluster_size,
                                      void *d_workspace, size_t workspace_bytes,
                                      stencil_stream_t stream);
/* Runs the prepared jobs with the engine chosen at prepare time (see the
 * engines below).  The one-launch engine: a memset node (its queues and
 * counters) and one cooperative kernel.  The phased engine: the copies of
 * ragged jobs in (one kernel), one
 * persistent cluster launch over a device work queue (every cluster the
 * device can hold) for the jobs that a cluster sweeps, then, for each job too
 * large for a cluster's shared memory, one persistent launch of its own, and
 * the copies out.  Those launches run on the whole GPU, except that 2-D jobs and
 * mid-size 3-D jobs (below 2^25 cells) of one radius and mode run in lanes
 * side by side, each lane a queue of jobs on its share of the CTAs the device
 * holds (jobs assigned largest first to the lane with the least work; 2-D
 * ones on the rows kernel), all lanes but the first on streams that prepare
 * creates for the workspace (forked from and joined back into `stream` by
 * events).  Environment variables read by prepare override the defaults:
 * STENCIL_BATCH_LANES and STENCIL_BATCH_LANES_2D (4; 1 = no lanes),
 * STENCIL_BATCH_LANE_MAX_CELLS (2^25) and STENCIL_BATCH_LANE_MAX_CELLS_2D
 * (2^30; 0 = no lanes), and STENCIL_BATCH_STREAM_MIN_CELLS_3D (1.2 M: 3-D jobs below it that do not fit
 * a cluster's shared memory are swept by a cluster from L2).  Resets the queue
 * counter first.  Asynchronous; allocates nothing; can be captured into a
 * CUDA graph (the queue reset is a memset node, so every replay runs the
 * whole batch again; lanes become parallel branches). */
STENCIL_API int stencil_batch_launch(const void *d_workspace, stencil_stream_t stream);
/* Batch engines.  PHASED: what stencil_batch_launch describes above (a
 * cluster launch, whole-GPU launches and lanes, the copy kernels; it applies
 * the jobs' tuning hints).
 * ONE_LAUNCH: every job in ONE persistent cooperative launch (one CTA per SM)
 * -- the CTAs form teams, each team sweeps one grid at a time with all its
 * sweeps (3-D grids with the stream kernel's TMA-ring code, 2-D grids with
 * the rows kernel's register-queue code, a bounded barrier over the team
 * between sweeps) and then takes the next grid from a device queue; grids
 * are placed in tiers by the team size their cells keep busy (about
 * STENCIL_BATCH1_CELLS_PER_CTA_2D = 50000 / _3D = 50000 update cells per
 * CTA, at most STENCIL_BATCH1_MAX_TEAM = a quarter of the CTAs; environment
 * variables of these names override them at prepare time), every team
 * starts in the largest tier and splits into the next tier's teams when its
 * queue is empty; ragged grids are copied in and out by their team inside the
 * launch.  It uses the jobs' team fields, not temporal / tile_x / tile_y.  AUTO:
 * the environment variable STENCIL_BATCH_ENGINE ("phased" or "one_launch")
 * at prepare time, else PHASED when some job carries tuning hints, else
 * ONE_LAUNCH. */
#define STENCIL_BATCH_ENGINE_AUTO 0
#define STENCIL_BATCH_ENGINE_PHASED 1
#define STENCIL_BATCH_ENGINE_ONE_LAUNCH 2
/* stencil_batch_prepare with a choice of engine (stencil_batch_prepare is
 * this with STENCIL_BATCH_ENGINE_AUTO).  Re-preparing a workspace replaces
 * its plan.  The workspace sizes above suffice for either engine. */
STENCIL_API int stencil_batch_prepare_engine(const stencil_batch_job *jobs, int njobs, int engine,
                                             int cluster_size, void *d_workspace,
                                             size_t workspace_bytes, stencil_stream_t stream);
/* How stencil_batch_launch runs a prepared workspace: *cluster_jobs jobs in
 * the cluster launch (none: no cluster launch), *whole_gpu_jobs jobs with a
 * launch of their own (both 0 for the one-launch engine). */
STENCIL_API int stencil_batch_plan(const void *d_workspace, int *cluster_jobs, int *whole_gpu_jobs);
/* Kernel launches of one stencil_batch_launch of a prepared workspace (1 for
 * the one-launch engine, 0 when it has no job). */
STENCIL_API int stencil_batch_launches(const void *d_workspace, int *kernel_launches);
/* The one-launch engine's tiers: *tiers of them (0 for a phased workspace),
 * the nominal team size and the job count of each of the first max_tiers in
 * team_sizes / tier_jobs (either may be NULL). */
STENCIL_API int stencil_batch_teams(const void *d_workspace, int *tiers, int *team_sizes,
                                    int *tier_jobs, int max_tiers);
/* *groups = how many sets of lanes run side by side (one per radius and
 * mode), *jobs = the jobs in them. */
STENCIL_API int stencil_batch_side_by_side(const void *d_workspace, int *groups, int *jobs);
/* Drops the host-side record of a prepared workspace and its streams (call
 * before freeing it). */
STENCIL_API int stencil_batch_forget(const void *d_workspace);

/* ---- Mixed-precision iterative refinement (no counterpart in the reference).
 * Solves the JACOBI steady state in outer steps of inner_sweeps sweeps: the
 * residual r = (M u + c) - u is recomputed in FP32 from the FP32 master grid
 * d_u, the correction e of (I - M) e = r is swept in BF16 or FP16 storage
 * with FP32 accumulation, and u += e.  In exact arithmetic the result after
 * p->iterations sweeps is that of p->iterations plain sweeps.  With tol > 0
 * the solve stops once the relative residual (stencil_residual, computed on
 * the GPU every check_every outer steps) drops below tol.  Needs p->mode == JACOBI and
 * nx % 8 == 0; d_u's border band is never written.  Allocates nothing: the
 * caller passes a 256-byte aligned workspace of stencil_ir_workspace_bytes.
 * Engines: 2-D grids of at most one tile per SM (R = 1, 2, 4) run each outer
 * step as one cooperative launch with every correction sweep in shared
 * memory (PERSISTENT_2D); other grids launch each correction sweep
 * (LAUNCHES).  Both give bit-identical results.  3-D correction sweeps at
 * R = 4 form their x- and y-neighbour sums on the tensor cores (products with
 * banded matrices, FP32 accumulation: the same result up to FP32 roundings);
 * the environment variable STENCIL_LP_MMA=0, read once per process, selects
 * per-term adds instead. */
enum { STENCIL_STORAGE_FP32 = 0, STENCIL_STORAGE_BF16 = 1, STENCIL_STORAGE_FP16 = 2 };
enum {
    STENCIL_IR_ENGINE_AUTO = 0,          /* PERSISTENT_2D where it applies, else LAUNCHES */
    STENCIL_IR_ENGINE_LAUNCHES = 1,      /* residual, sweeps and update as separate launches */
    STENCIL_IR_ENGINE_PERSISTENT_2D = 2  /* one cooperative launch per outer step (2-D only) */
};

typedef struct stencil_ir_params {
    int storage;       /* STENCIL_STORAGE_BF16 or STENCIL_STORAGE_FP16 */
    int inner_sweeps;  /* correction sweeps per outer step (0 = 50) */
    int check_every;   /* outer steps between residual checks when tol > 0 */
    int engine;        /* STENCIL_IR_ENGINE_* */
    int temporal;      /* PERSISTENT_2D: sweeps per halo exchange (0 = chosen) */
    int tile_x, tile_y; /* PERSISTENT_2D: owned tile in cells (0 = chosen; tile_x % 8 == 0) */
    int reserved;      /* must be zero */
    double tol;        /* stop at this relative residual (0 = run all sweeps) */
} stencil_ir_params;

typedef struct stencil_ir_result {
    int sweeps;          /* sweeps performed */
    int outer_steps;     /* refinement steps performed */
    double rel_residual; /* relative residual of the final u (stencil_residual) */
    int engine;          /* STENCIL_IR_ENGINE_LAUNCHES or _PERSISTENT_2D: the one that ran */
    int kernel_launches; /* kernels launched (residual checks included) */
    int temporal, tile_x, tile_y; /* PERSISTENT_2D: the plan that ran (else 0) */
} stencil_ir_result;

STENCIL_API int stencil_ir_workspace_bytes(const stencil_params *p, const stencil_ir_params *ir,
                                           size_t *bytes);
/* Synchronises `stream` at each residual check and at the end. */
STENCIL_API int stencil_ir_solve(const stencil_params *p, const stencil_ir_params *ir, float *d_u,
                                 void *d_workspace, size_t workspace_bytes,
                                 stencil_stream_t stream, stencil_ir_result *result);

/* Relative residual ||b - A u||_2 / ||b||_2 of the steady state that JACOBI
 * iterates to, (A u)(x) = u(x) - mean of the 2*D*R axis neighbours over the
 * update region, b = the border contributions.  Each cell's residual is
 * evaluated in FP32 as the sum of its (neighbour - centre) differences
 * (exact wherever neighbour and centre are within a factor of two, so it
 * stays accurate relative to itself as it shrinks); FP64 is used for the
 * sums of squares only.  Agrees with an all-FP64 evaluation to about 1e-7
 * relative.  d_u must be 16-byte aligned (STENCIL_EINVAL otherwise; cudaMalloc
 * gives 256).  Synchronises `stream`. */
STENCIL_API int stencil_residual(const stencil_params *p, const float *d_u, double *rel_residual,
                     stencil_stream_t stream);

/* The plain sweep loop run to a tolerance (no counterpart in the reference,
 * whose loop runs a fixed ITERATIONS, src/stencil_dispatch.cu:153-157): from
 * d_u1, chunks of check_every sweeps of p (JACOBI) on the engine
 * stencil_dispatch_ex picks, the relative residual (stencil_residual) before
 * the first chunk and after each one, until it is below tol or p->iterations
 * sweeps are done.  Both buffers keep the JACOBI contract (equal border
 * bands); result->d_result is the one holding the final state.  Synchronises
 * `stream` at every check. */
typedef struct stencil_solve_result {
    int sweeps;          /* sweeps performed */
    int checks;          /* residual evaluations */
    double rel_residual; /* relative residual of the final state */
    float *d_result;     /* d_u1 or d_u2 */
} stencil_solve_result;

STENCIL_API int stencil_solve(const stencil_params *p, float *d_u1, float *d_u2, double tol,
                              int check_every, stencil_stream_t stream,
                              stencil_solve_result *result);

/* Same result as stencil_residual, for callers that must not allocate device
 * memory -- e.g. a process whose own pool allocator already owns all free
 * device memory, or a latency-critical loop where cudaMalloc/cudaFree and
 * their device-wide synchronisation are not allowed.  No counterpart in the
 * reference.  Allocates nothing: its scratch is a fixed 262,160-byte device
 * array inside the library (kept on every GPU that loads it until exit), so
 * grids with more than 2^30 update cells are rejected with STENCIL_EINVAL.
 * The array is reserved when the CUDA runtime loads the library's module on a
 * device (its first kernel launch or symbol lookup under the default lazy
 * loading; context creation with CUDA_MODULE_LOADING=EAGER), never by this
 * call; each call looks up its address on the current device.  Calls share
 * the array: calls that can overlap on one GPU (two streams, two host
 * threads) race and must be serialised.  d_u must be 16-byte aligned
 * (STENCIL_EINVAL otherwise).  Synchronises `stream`, so it cannot be
 * captured into a CUDA graph. */
STENCIL_API int stencil_residual_noalloc(const stencil_params *p, const float *d_u,
                                         double *rel_residual, stencil_stream_t stream);

/* Error reporting. */
STENCIL_API const char *stencil_strerror(int status);
/* Text of the last failure on the calling thread (empty if none). */
STENCIL_API const char *stencil_last_error(void);
/* What this thread's last stencil_dispatch_ex (or stencil_run_host*) ran:
 * the engine ("stream3d", "stream3d-persistent", "rows3d", "tb3d", "cluster",
 * "base", "tile"; the first one when a dispatch uses two) and how many kernel
 * launches it made (iterations for one launch per sweep, 1 for the
 * persistent engines).  For diagnostics and launch accounting. */
STENCIL_API int stencil_last_dispatch(const char **engine, long long *kernel_launches);
/* Reads and clears the device-side status word that bounded waits set when
 * they give up (0 = no fault).  Synchronises the device. */
STENCIL_API int stencil_device_status(int *status);

/* Diagnostics (no counterpart in the reference).
 * stencil_selftest_div: runs the kernels' division-by-coefficient path against
 * IEEE division for all 2^32 float bit patterns; *mismatches receives the
 * count (0 expected), *first_mismatch (optional) the smallest failing pattern.
 * coeff is one of the coefficients 2*D*R the kernels use: 4, 6, 8, 12, 16, 18,
 * 24, 32, 36, 48, 64, 96.
 * stencil_selftest_wait: launches one bounded mbarrier wait that nothing
 * completes, with a limit of limit_ms (1..2000); *completed receives 0 when the
 * wait gave up and *status the device status word it set (then cleared). */
STENCIL_API int stencil_selftest_div(int coeff, unsigned long long *mismatches,
                                     unsigned *first_mismatch);
STENCIL_API int stencil_selftest_wait(int limit_ms, int *completed, int *status);

/* ---- Tuning table consulted by STENCIL_VARIANT_AUTO (filled by the
 * project's autotuner, thesis_gb300/autotune.py; no counterpart in the
 * reference, whose tuner rebuilt the binary per configuration).  An entry
 * maps (dims, radius, the smallest power of two >= the largest extent) to a
 * variant and its tuning fields (block_*, coarsen_x, temporal) taken from
 * `choice`; setting an existing key replaces it.  At most 256 entries. */
STENCIL_API int stencil_tuning_set(const stencil_params *key, const stencil_params *choice);
/* Looks up the entry for key; returns STENCIL_EINVAL if there is none. */
STENCIL_API int stencil_tuning_get(const stencil_params *key, stencil_params *choice);
STENCIL_API int stencil_tuning_clear(void);

/* Frees every workspace this library holds on the current device.  Call it
 * before cudaDeviceReset(): the library keeps device pointers to its
 * workspaces between calls, and a reset leaves them dangling. */
STENCIL_API int stencil_release(void);

/* Library version and the compute capability it was built for (103). */
/* The reference's HEURISTIC block shape (set_max_occupancy_block_dimensions,
 * src/stencil_dispatch.cu:89-101) for a block of `threads` threads (the
 * reference takes it from cudaOccupancyMaxPotentialBlockSizeVariableSMem,
 * :143): 3-D: b0 = BLOCK_X (p->block_x), halved while a padded smem block of
 * b0*R*R cells exceeds the threads; b1 = min(max(2, R), 8); b2 =
 * threads/(b0*b1); the three sorted in descending order.  2-D: (BLOCK_X,
 * threads/BLOCK_X, 1).  A pure function: with block = 0 the library uses its
 * own per-kernel default (or the tuning table) instead; callers that want the
 * reference's shape pass this result as p->block_*. */
STENCIL_API int stencil_heuristic_block(const stencil_params *p, int threads, int *bx, int *by,
                                        int *bz);
/* The reference's HEURISTIC geometry (src/stencil_dispatch.cu:138-146): the
 * thread count that cudaOccupancyMaxPotentialBlockSizeVariableSMem returns for
 * the kernel this library runs in p->variant's role (BASE: the vector or
 * scalar base kernel; SMEM, SMEM_PADDED, SMEM_REGISTER: the TMA tile kernel),
 * with the dynamic shared memory of each candidate block given by the
 * reference's set_smem (src/stencil_dispatch.cu:46-66) on the block that
 * stencil_heuristic_block shapes from it (p->block_x = BLOCK_X, default 32;
 * p->coarsen_x = COARSEN_X); then that shape.  With HEURISTIC == 2 the
 * constants.h drop-in launches the one-sweep roles with this block (the 3-D
 * SMEM_REGISTER role, whose stream kernel has fixed thread shapes, takes its
 * x and y as the tile: 4 * bx by by cells). */
STENCIL_API int stencil_heuristic_geometry(const stencil_params *p, int *threads, int *bx, int *by,
                                           int *bz);

STENCIL_API int stencil_version(int *abi_version, int *sm);

#ifdef __cplusplus
} /* extern "C" */
#endif

/* Drop-in for the reference's compile-time configured dispatch: shape, radius,
 * variant and sweep count come from constants.h exactly as they do for
 * dispatch_kernels (src/stencil_dispatch.cu:138).  Include constants.h (or pass
 * the -D macros) before this header. */
#ifdef STENCIL_CONSTANTS_H
static inline int stencil_params_from_constants(stencil_params *p)
{
    int rc = stencil_params_init(p);
    if (rc) return rc;
    p->dims = DIMENSIONS;
    p->nx = NX; p->ny = NY; p->nz = DIMENSIONS == 3 ? NZ : 1;
    p->radius = RADIUS;
    p->iterations = ITERATIONS;
    p->mode = STENCIL_MODE;
    p->block_x = HEURISTIC ? 0 : BLOCK_X;
    p->block_y = HEURISTIC ? 0 : BLOCK_Y;
    p->block_z = HEURISTIC ? 0 : BLOCK_Z;
    p->coarsen_x = COARSEN_X;
    p->temporal = TEMPORAL_T;
    if (COOP) p->variant = STENCIL_VARIANT_COOP;
    else if (SMEM && REGISTER) p->variant = STENCIL_VARIANT_SMEM_REGISTER;
    else if (SMEM && PADDED) p->variant = STENCIL_VARIANT_SMEM_PADDED;
    else if (SMEM) p->variant = STENCIL_VARIANT_SMEM;
    else p->variant = STENCIL_VARIANT_BASE;
    if (HEURISTIC == 2 && !COOP) {
        /* the reference's occupancy-based block (src/stencil_dispatch.cu:143) */
        int t = 0, bx = 0, by = 0, bz = 0;
        p->block_x = BLOCK_X;
        rc = stencil_heuristic_geometry(p, &t, &bx, &by, &bz);
        if (rc) return rc;
        p->block_x = bx; p->block_y = by;
        p->block_z = (p->variant == STENCIL_VARIANT_SMEM_REGISTER && p->dims == 3) ? 0 : bz;
    }
    return STENCIL_OK;
}

/* Same role as dispatch_kernels(d_u1, d_u2) (src/stencil_dispatch.cu:138), plus
 * a stream, a status and the location of the result. */
static inline int stencil_dispatch(float *d_u1, float *d_u2, stencil_stream_t stream,
                                   float **d_result)
{
    stencil_params p;
    int rc = stencil_params_from_constants(&p);
    if (rc) return rc;
    return stencil_dispatch_ex(&p, d_u1, d_u2, stream, d_result);
}
#endif /* STENCIL_CONSTANTS_H */

#endif /* STENCIL_DISPATCH_H */

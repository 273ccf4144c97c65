// host.hpp -- host-side internals shared by the translation units of
// libstencil_gb300 (not part of the C ABI).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <string>

#include "../../include/stencil_dispatch.h"
#include "common.cuh"

namespace st {

// Records a failure for stencil_last_error() and returns `code`.
int fail(int code, const char *fmt, ...);
// Maps a CUDA runtime error to STENCIL_ECUDA (recording the message) or OK.
int cuda_fail(cudaError_t e, const char *what);
#define ST_CUDA(call)                                             \
    do {                                                          \
        cudaError_t st_e_ = (call);                               \
        if (st_e_ != cudaSuccess) return ::st::cuda_fail(st_e_, #call); \
    } while (0)

Geom make_geom(const stencil_params &p);
long long cell_count(const stencil_params &p);
int num_sms();
int current_device();

// Builds a tiled TMA descriptor for an FP32 grid (rank 2 or 3); pitch: the
// row pitch in elements when it exceeds dims[0] (0 = dims[0]).  Box cells
// outside the grid read as zeros, or as NaN with nan_fill.
int make_tensor_map(CUtensorMap *map, const float *base, int rank, const long long *dims,
                    const int *box, long long pitch = 0, bool nan_fill = false);
// Any rank (1..5), element type, byte strides of dims 1.. and swizzle.
int make_tensor_map_general(CUtensorMap *map, CUtensorMapDataType dtype, int rank, const void *base,
                            const unsigned long long *dims, const unsigned long long *strides,
                            const unsigned *box, CUtensorMapSwizzle swizzle);
// The same for another element type (e.g. BF16/FP16 grids, 2 bytes).
int make_tensor_map_typed(CUtensorMap *map, const void *base, int rank, const long long *dims,
                          const int *box, CUtensorMapDataType dtype, int elem_bytes,
                          long long pitch = 0, bool nan_fill = false);

// One sweep per launch kernels (src -> dst).  Each returns a status.
int launch_base_sweep(const Geom &g, int dims, const float *src, float *dst, int bx, int by,
                      int bz, int cf, cudaStream_t s);
int launch_tile_sweep(const Geom &g, int dims, const float *src, float *dst, int bx, int by,
                      int bz, cudaStream_t s);

// Multi-sweep drivers: run `iters` sweeps ping-ponging between a and b
// starting from a; *res receives the buffer holding the final state.
// shape_hint (block_z of the parameters): 0 = by tile fields, 1..3 = a shape.
// Records kernel launches of the current dispatch (stencil_last_dispatch).
void note_launches(const char *engine, long long n);
bool stream3d_supported(const Geom &g);
// persistent: all sweeps in one cooperative launch with a grid barrier
// between sweeps (default shape of each radius) instead of one launch each.
// max_ctas > 0 caps the CTAs of the launch (the persistent form then keeps
// its grid barrier over those CTAs only).
int run_stream3d(const Geom &g, float *a, float *b, int iters, int tile_x, int tile_y,
                 cudaStream_t s, float **res, int shape_hint = 0, bool persistent = false,
                 int max_ctas = 0);
// CTAs of the device that the persistent stream kernel for g can hold at once.
int stream3d_capacity(const Geom &g, int *ctas);
// Work items of a stream sweep of g with tx x ty tiles on `resident` CTAs:
// tiles along x and y, planes per z-chunk, (tile, z-chunk) items.
void stream3d_plan(const Geom &g, int tx, int ty, int resident, int *tiles_x, int *tiles_y,
                   int *zchunk, int *items);
int run_tb3d(const Geom &g, float *a, float *b, int iters, int temporal, cudaStream_t s,
             float **res);
// A zeroed grid-barrier counter for one persistent launch on stream s
// (round-robin over a fixed device array; k_stream.cu).
int grid_bar_slot(cudaStream_t s, unsigned **slot);
// Small 2-D grids: all sweeps in one cooperative launch, one tile per CTA,
// `temporal` sweeps per exchange through global memory (k_tb2d.cu).
// tile_x/tile_y/temporal 0 = chosen by the library.  tb2d_release frees the
// current device's exchange buffers.
bool tb2d_supported(const Geom &g, int dims);
int run_tb2d(const Geom &g, float *a, float *b, int iters, int temporal, int tile_x, int tile_y,
             cudaStream_t s, float **res);
void tb2d_release();
// Larger 2-D grids: all sweeps in one cooperative launch, a grid-wide barrier
// between sweeps, register-queue columns (k_rows2d.cu).
// max_ctas > 0 caps the CTAs of the launch; rows2d_capacity = the CTAs of the
// device that the kernel for g's radius can hold at once.
bool rows2d_supported(const Geom &g, int dims);
int rows2d_capacity(const Geom &g);
// Row blocks of a rows sweep of g on `threads` threads: *hb rows per block,
// *nblk blocks.
void rows2d_plan(const Geom &g, long long threads, int *hb, int *nblk);
int run_rows2d(const Geom &g, float *a, float *b, int iters, cudaStream_t s, float **res,
               int max_ctas = 0);
// All sweeps of one grid on one thread-block cluster (k_cluster.cu).
int run_cluster(const Geom &g, int dims, float *a, float *b, int iters, cudaStream_t s,
                float **res);
// The grid fits the cluster's shared memory (resident mode).
bool cluster_resident(const Geom &g, int dims);
// The cluster engine takes the shape (nx % 4 == 0, R <= 4, 3-D planes of
// fewer than 2^31 float4 chunks).
bool cluster_shape_ok(int dims, int px, int ny, int radius);

// Batches (k_cluster.cu, k_batch1.cu).  check_batch_job: the checks every
// batch job passes, *out its parameters.  batch1_*: the one-launch engine
// (prepare writes the job table, tensor maps and tiers into the workspace and
// remembers the plan; launch = a memset node and one cooperative kernel).
int check_batch_job(const stencil_batch_job &b, int i, stencil_params *out);
size_t batch1_bytes_for(const stencil_batch_job *jobs, int njobs);
int batch1_prepare(const stencil_batch_job *jobs, int njobs, void *d_workspace,
                   size_t workspace_bytes, cudaStream_t s);
bool batch1_known(const void *d_workspace);
int batch1_launch(const void *d_workspace, cudaStream_t s);
int batch1_launches(const void *d_workspace);  // kernels per launch: 1, or 0 without jobs
int batch1_teams(const void *d_workspace, int *ntiers, int *team_sizes, int *tier_jobs, int max_tiers);
void batch1_forget(const void *d_workspace);

// Mixed-precision refinement, persistent 2-D form of an outer step
// (k_ir2d.cu): one CTA per tile, T correction sweeps per halo exchange.
struct Ir2Plan {
    int tx, ty;          // owned tile (cells); tx % 8 == 0
    int t;               // sweeps per exchange
    int hx, hy;          // halo: x in whole 8-cell chunks, y = t * R
    int pw, ph;          // grown tile (pw % 8 == 0)
    int tiles_x, tiles_y;
};
// Exchange-buffer bytes any plan of the grid needs.
size_t ir2_xch_bytes(const Geom &g);
// A plan for outer steps of m sweeps (temporal / tile_* 0 = chosen); false
// if the grid does not fit one tile per SM.  E = __nv_bfloat16 or __half.
template <typename E>
bool ir2_plan(const Geom &g, int m, int temporal, int tile_x, int tile_y, Ir2Plan *p);
// One outer step of m sweeps on u.  The counters (bar, the two max_bits
// words) and the exchange buffer are zeroed once per solve; step counts the
// launches since then and tag0 grows by m + 1 per launch.
template <typename E>
int ir2_launch(const Geom &g, const Ir2Plan &p, float *u, unsigned long long *xch, unsigned *bar,
               unsigned *max_bits, float *scale, int step, unsigned tag0, int m, cudaStream_t s);

// Plain whole-grid helpers.
int launch_copy_border(const Geom &g, int dims, const float *src, float *dst, cudaStream_t s);
// Copies bytes (a multiple of 16, both addresses 16-byte aligned) with a
// streaming kernel over every SM (k_util.cu).
int launch_copy16(void *dst, const void *src, size_t bytes, cudaStream_t s);
int launch_init_reference(const Geom &g, int dims, float *u, cudaStream_t s);

}  // namespace st

// api.cu -- the C ABI of libstencil_gb300 (include/stencil_dispatch.h):
// parameter validation, variant selection, the sweep loop driver, the
// host-buffer end-to-end entry point, workspaces and error reporting.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include <cstdlib>
#include <string>
#include "host.hpp"

namespace st {

// Declared in the kernel translation units.
int launch_init_uniform(float *u, size_t count, uint64_t seed, cudaStream_t s);
size_t residual_scratch_bytes();
int launch_residual(const Geom &g, int dims, const float *u, double *scratch, cudaStream_t s);
bool stream3d_supported(const Geom &g);
bool tile_supported(const Geom &g, int dims);
bool tb3d_supported(const Geom &g);
bool rows3d_supported(const Geom &g);
int run_rows3d(const Geom &g, float *a, float *b, int iters, int shape, cudaStream_t s,
               float **res);
const void *base_kernel_ptr(const Geom &g, int dims);
const void *tile_kernel_ptr(int dims, int r);

static thread_local char t_err[512];
static thread_local long long t_launches = 0;
static thread_local const char *t_engine = "none";

int fail(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_err, sizeof t_err, fmt, ap);
    va_end(ap);
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return STENCIL_OK;
    const int code = e == cudaErrorMemoryAllocation ? STENCIL_ENOMEM
                     : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
                         ? STENCIL_ENODEVICE
                         : STENCIL_ECUDA;
    return fail(code, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

Geom make_geom(const stencil_params &p) {
    Geom g;
    g.nx = p.nx;
    g.ny = p.ny;
    g.nz = p.dims == 3 ? p.nz : 1;
    g.radius = p.radius;
    g.legacy = p.mode == STENCIL_MODE_LEGACY;
    g.sy = p.nx;
    g.sz = (long long)p.nx * p.ny;
    return g;
}

long long cell_count(const stencil_params &p) {
    return (long long)p.nx * p.ny * (p.dims == 3 ? p.nz : 1);
}

int current_device() {
    int d = 0;
    cudaGetDevice(&d);
    return d;
}

int num_sms() {
    static int cache[64] = {0};
    const int d = current_device();
    if (d >= 0 && d < 64 && cache[d]) return cache[d];
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, d) != cudaSuccess || n <= 0)
        n = 152;
    if (d >= 0 && d < 64) cache[d] = n;
    return n;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point, so the
// library does not link libcuda directly.
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion,
                                  CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

int make_tensor_map_typed(CUtensorMap *map, const void *base, int rank, const long long *dims,
                          const int *box, CUtensorMapDataType dtype, int elem_bytes,
                          long long pitch, bool nan_fill) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return fail(STENCIL_ECUDA, "cuTensorMapEncodeTiled is unavailable");
    cuuint64_t gdim[3], gstride[2];
    cuuint32_t bdim[3], estride[3] = {1, 1, 1};
    for (int i = 0; i < rank; ++i) {
        gdim[i] = (cuuint64_t)dims[i];
        bdim[i] = (cuuint32_t)box[i];
    }
    const long long row = pitch > 0 ? pitch : dims[0];  // row pitch in elements
    gstride[0] = (cuuint64_t)row * elem_bytes;
    if (rank == 3) gstride[1] = (cuuint64_t)row * dims[1] * elem_bytes;
    CUresult r = fn(map, dtype, (cuuint32_t)rank, const_cast<void *>(base), gdim, gstride, bdim,
                    estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    nan_fill ? CU_TENSOR_MAP_FLOAT_OOB_FILL_NAN_REQUEST_ZERO_FMA
                             : CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(STENCIL_EINVAL, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return STENCIL_OK;
}

int make_tensor_map_general(CUtensorMap *map, CUtensorMapDataType dtype, int rank, const void *base,
                            const unsigned long long *dims, const unsigned long long *strides,
                            const unsigned *box, CUtensorMapSwizzle swizzle) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return fail(STENCIL_ECUDA, "cuTensorMapEncodeTiled is unavailable");
    if (rank < 1 || rank > 5) return fail(STENCIL_EINVAL, "tensor map rank %d", rank);
    cuuint64_t gdim[5], gstride[4];
    cuuint32_t bdim[5], estride[5] = {1, 1, 1, 1, 1};
    for (int i = 0; i < rank; ++i) {
        gdim[i] = (cuuint64_t)dims[i];
        bdim[i] = (cuuint32_t)box[i];
        if (i + 1 < rank) gstride[i] = (cuuint64_t)strides[i];
    }
    CUresult r = fn(map, dtype, (cuuint32_t)rank, const_cast<void *>(base), gdim, gstride, bdim, estride,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(STENCIL_EINVAL, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return STENCIL_OK;
}

int make_tensor_map(CUtensorMap *map, const float *base, int rank, const long long *dims,
                    const int *box, long long pitch, bool nan_fill) {
    return make_tensor_map_typed(map, base, rank, dims, box, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
                                 pitch, nan_fill);
}

// Per-device scratch kept between calls (host-buffer entry, residual).
struct DeviceWorkspace {
    float *u[2] = {nullptr, nullptr};
    size_t grid_bytes = 0;
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
};

static std::mutex g_ws_mu;
static std::vector<DeviceWorkspace> g_ws(64);

static int ws_grids(int dev, size_t bytes, DeviceWorkspace **out) {
    DeviceWorkspace &w = g_ws[dev];
    if (!w.stream) {
        ST_CUDA(cudaStreamCreateWithFlags(&w.stream, cudaStreamNonBlocking));
        for (auto &e : w.ev) ST_CUDA(cudaEventCreate(&e));
    }
    if (w.grid_bytes < bytes) {
        cudaStreamSynchronize(w.stream);
        cudaFree(w.u[0]);
        cudaFree(w.u[1]);
        w.u[0] = w.u[1] = nullptr;
        w.grid_bytes = 0;
        ST_CUDA(cudaMalloc(&w.u[0], bytes));
        ST_CUDA(cudaMalloc(&w.u[1], bytes));
        w.grid_bytes = bytes;
    }
    *out = &w;
    return STENCIL_OK;
}

static int ws_scratch(int dev, size_t bytes, void **out) {
    DeviceWorkspace &w = g_ws[dev];
    if (w.scratch_bytes < bytes) {
        cudaDeviceSynchronize();
        cudaFree(w.scratch);
        w.scratch = nullptr;
        w.scratch_bytes = 0;
        ST_CUDA(cudaMalloc(&w.scratch, bytes));
        w.scratch_bytes = bytes;
    }
    *out = w.scratch;
    return STENCIL_OK;
}

// Tuning table (stencil_tuning_set): (dims, radius, size bucket) -> choice.
struct TuneEntry {
    int dims, radius, bucket;
    stencil_params choice;
};
static std::mutex g_tune_mu;
static std::vector<TuneEntry> g_tune;

static int size_bucket(const stencil_params &p) {
    int m = std::max(p.nx, std::max(p.ny, p.dims == 3 ? p.nz : 1));
    int b = 1;
    while (b < m) b <<= 1;
    return b;
}

static bool tuned_choice(const stencil_params &p, stencil_params *out) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    const int b = size_bucket(p);
    for (const TuneEntry &e : g_tune)
        if (e.dims == p.dims && e.radius == p.radius && e.bucket == b) {
            *out = e.choice;
            return true;
        }
    return false;
}

// Variant choice when the caller leaves it to the library: 2-D grids small
// enough for one tile per SM run the temporally blocked cooperative engine;
// other grids that fit a cluster's shared memory run all sweeps in one
// cluster launch (launch- and sync-bound otherwise); large 3-D grids stream;
// the rest use the base kernel.
void note_launches(const char *engine, long long n) {
    if (!t_launches) t_engine = engine;
    t_launches += n;
}

static int choose_variant(const stencil_params &p) {
    const Geom g = make_geom(p);
    // 2-D: small grids every SM, temporally blocked (2-5x the one-cluster
    // engine); larger ones every sweep in one persistent launch
    if (p.dims == 2 && p.iterations >= 8 && (tb2d_supported(g, 2) || rows2d_supported(g, 2)))
        return STENCIL_VARIANT_COOP;
    if (p.iterations >= 8 && cluster_resident(g, p.dims)) return STENCIL_VARIANT_CLUSTER;
    if (p.dims == 3 && stream3d_supported(g)) return STENCIL_VARIANT_SMEM_REGISTER;
    return STENCIL_VARIANT_BASE;
}

}  // namespace st

using namespace st;

extern "C" {

int stencil_params_init(stencil_params *p) {
    if (!p) return fail(STENCIL_EINVAL, "null params");
    memset(p, 0, sizeof *p);
    p->dims = 3;
    p->nx = p->ny = p->nz = 256;
    p->radius = 1;
    p->iterations = 64;
    p->mode = STENCIL_MODE_LEGACY;
    p->variant = STENCIL_VARIANT_AUTO;
    return STENCIL_OK;
}

int stencil_params_check(const stencil_params *p) {
    if (!p) return fail(STENCIL_EINVAL, "null params");
    if (p->dims != 2 && p->dims != 3) return fail(STENCIL_EINVAL, "dims must be 2 or 3 (got %d)", p->dims);
    if (p->radius < 1) return fail(STENCIL_EINVAL, "radius must be >= 1");
    const int nz = p->dims == 3 ? p->nz : 1;
    if (p->nx < 1 || p->ny < 1 || nz < 1) return fail(STENCIL_EINVAL, "extents must be positive");
    if (2 * p->radius >= p->nx || 2 * p->radius >= p->ny || (p->dims == 3 && 2 * p->radius >= p->nz))
        return fail(STENCIL_EINVAL, "every extent must exceed 2*radius");
    if ((long long)p->nx * p->ny * nz >= (1LL << 40)) return fail(STENCIL_EINVAL, "grid too large");
    if (p->iterations < 0) return fail(STENCIL_EINVAL, "iterations must be >= 0");
    if (p->mode != STENCIL_MODE_LEGACY && p->mode != STENCIL_MODE_JACOBI)
        return fail(STENCIL_EINVAL, "unknown mode %d", p->mode);
    if (p->variant < STENCIL_VARIANT_AUTO || p->variant > STENCIL_VARIANT_CLUSTER)
        return fail(STENCIL_EINVAL, "unknown variant %d", p->variant);
    if (p->block_x < 0 || p->block_y < 0 || p->block_z < 0 || p->coarsen_x < 0 || p->temporal < 0)
        return fail(STENCIL_EINVAL, "tuning fields must be >= 0");
    if ((long long)std::max(p->block_x, 1) * std::max(p->block_y, 1) * std::max(p->block_z, 1) > 1024)
        return fail(STENCIL_EINVAL, "block shape exceeds 1024 threads");
    for (int r : p->reserved)
        if (r) return fail(STENCIL_EINVAL, "reserved fields must be zero");
    return STENCIL_OK;
}

int stencil_dispatch_ex(const stencil_params *p, float *d_u1, float *d_u2,
                        stencil_stream_t stream, float **d_result) {
    int rc = stencil_params_check(p);
    if (rc) return rc;
    if (!d_u1 || !d_u2 || d_u1 == d_u2) return fail(STENCIL_EINVAL, "two distinct device buffers are required");
    if ((reinterpret_cast<uintptr_t>(d_u1) | reinterpret_cast<uintptr_t>(d_u2)) & 15)
        return fail(STENCIL_EINVAL, "device buffers must be 16-byte aligned");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const Geom g = make_geom(*p);
    float *cur = d_u1, *nxt = d_u2;
    t_launches = 0;
    t_engine = "none";
    if (d_result) *d_result = cur;
    if (p->iterations == 0) return STENCIL_OK;
    int variant = p->variant;
    stencil_params tuned;
    if (variant == STENCIL_VARIANT_AUTO && tuned_choice(*p, &tuned)) {
        // The tuned variant and tuning fields replace the caller's zeros.
        stencil_params q = *p;
        q.variant = tuned.variant;
        if (!q.block_x) q.block_x = tuned.block_x;
        if (!q.block_y) q.block_y = tuned.block_y;
        if (!q.block_z) q.block_z = tuned.block_z;
        if (!q.coarsen_x) q.coarsen_x = tuned.coarsen_x;
        if (!q.temporal) q.temporal = tuned.temporal;
        if (q.variant != STENCIL_VARIANT_AUTO) return stencil_dispatch_ex(&q, d_u1, d_u2, stream, d_result);
    }
    const bool auto_pick = variant == STENCIL_VARIANT_AUTO;
    if (auto_pick) variant = choose_variant(*p);
    if (variant == STENCIL_VARIANT_SMEM_REGISTER && !(p->dims == 3 && stream3d_supported(g)))
        variant = STENCIL_VARIANT_SMEM_PADDED;
    if ((variant == STENCIL_VARIANT_SMEM || variant == STENCIL_VARIANT_SMEM_PADDED) &&
        !tile_supported(g, p->dims))
        variant = STENCIL_VARIANT_BASE;
    if (variant == STENCIL_VARIANT_COOP && p->dims == 2 && tb2d_supported(g, 2)) {
        // Whole GPU, one tile per SM, `temporal` sweeps per exchange; the
        // tile is block_x * coarsen_x by block_y cells when given.
        float *res = nullptr;
        rc = run_tb2d(g, cur, nxt, p->iterations, p->temporal,
                      p->block_x * std::max(p->coarsen_x, 1), p->block_y, s, &res);
        if (rc) return rc;
        if (d_result) *d_result = res;
        return STENCIL_OK;
    }
    if (variant == STENCIL_VARIANT_COOP && p->dims == 2 && rows2d_supported(g, 2)) {
        float *res = nullptr;
        rc = run_rows2d(g, cur, nxt, p->iterations, s, &res);
        if (rc) return rc;
        if (d_result) *d_result = res;
        return STENCIL_OK;
    }
    if (variant == STENCIL_VARIANT_COOP && cluster_resident(g, p->dims))
        variant = STENCIL_VARIANT_CLUSTER;
    if (variant == STENCIL_VARIANT_CLUSTER) {
        if (cluster_shape_ok(p->dims, (int)g.sy, g.ny, g.radius)) {
            float *res = nullptr;
            rc = run_cluster(g, p->dims, cur, nxt, p->iterations, s, &res);
            if (rc) return rc;
            if (d_result) *d_result = res;
            return STENCIL_OK;
        }
        variant = STENCIL_VARIANT_COOP;
    }
    // 3-D: several sweeps per HBM pass only when asked for (temporal >= 2);
    // left to the library (0) or 1, one sweep per pass in one persistent
    // launch, which is faster on GB300 (512^3 R=1: 708 vs 367 GCell/s)
    if (variant == STENCIL_VARIANT_COOP && p->dims == 3 && tb3d_supported(g) &&
        p->temporal >= 2) {
        float *res = nullptr;
        rc = run_tb3d(g, cur, nxt, p->iterations, p->temporal, s, &res);
        if (rc) return rc;
        if (d_result) *d_result = res;
        return STENCIL_OK;
    }
    if (variant == STENCIL_VARIANT_COOP && p->dims == 3 && stream3d_supported(g)) {
        // One sweep per HBM pass, all sweeps in one persistent cooperative
        // launch with a grid-wide barrier between them (block_z 1..6 picks
        // the stream kernel's shape where its persistent form exists).
        float *res = nullptr;
        rc = run_stream3d(g, cur, nxt, p->iterations, 0, 0, s, &res,
                          (p->block_z >= 1 && p->block_z <= 6) ? p->block_z : 0, true);
        if (rc) return rc;
        if (d_result) *d_result = res;
        return STENCIL_OK;
    }
    if (variant == STENCIL_VARIANT_COOP) variant = STENCIL_VARIANT_BASE;
    if (variant == STENCIL_VARIANT_SMEM_REGISTER && p->block_x == 0 && p->block_y == 8 &&
        rows3d_supported(g)) {
        float *res = nullptr;
        rc = run_rows3d(g, cur, nxt, p->iterations, p->block_z, s, &res);
        if (rc) return rc;
        if (d_result) *d_result = res;
        return STENCIL_OK;
    }
    if (variant == STENCIL_VARIANT_SMEM_REGISTER) {
        // Left to the library (no tile shape given): all sweeps in one
        // persistent launch, at least as fast as a launch per sweep (512^3:
        // equal at R = 1, +4 % at R = 4; 256^3: +8 %).
        const bool persistent = auto_pick && !p->block_x && !p->block_y && !p->block_z;
        float *res = nullptr;
        rc = run_stream3d(g, cur, nxt, p->iterations, p->block_x ? 4 * p->block_x : 0,
                          p->block_y, s, &res, p->block_z, persistent);
        if (rc) return rc;
        if (d_result) *d_result = res;
        return STENCIL_OK;
    }
    note_launches(variant == STENCIL_VARIANT_BASE ? "base" : "tile", p->iterations);
    for (int it = 0; it < p->iterations; ++it) {
        if (variant == STENCIL_VARIANT_BASE)
            rc = launch_base_sweep(g, p->dims, cur, nxt, p->block_x, p->block_y, p->block_z,
                                   p->coarsen_x, s);
        else
            rc = launch_tile_sweep(g, p->dims, cur, nxt, p->block_x, p->block_y, p->block_z, s);
        if (rc) return rc;
        std::swap(cur, nxt);
    }
    if (d_result) *d_result = cur;
    return STENCIL_OK;
}

namespace st {
namespace {
// The device-side address of a pinned (page-locked, mapped) host buffer of at
// least `bytes` bytes, 16-byte aligned, or null: such a buffer is copied by
// a kernel running on every SM over the host link (GB300, 512 MiB each way:
// see the bench's e2e), any other by cudaMemcpyAsync.
// STENCIL_HOST_COPY=engine keeps every transfer on the copy engines.
const void *mapped_host(const void *h, size_t bytes) {
    const char *e = std::getenv("STENCIL_HOST_COPY");
    if (e && std::string(e) == "engine") return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
    if (((reinterpret_cast<uintptr_t>(a.devicePointer) | bytes) & 15) != 0) return nullptr;
    return a.devicePointer;
}
}  // namespace
}  // namespace st

int stencil_run_host_timed(const stencil_params *p, const float *h_in, float *h_out,
                           float *ms_total, float *ms_sweeps) {
    int rc = stencil_params_check(p);
    if (rc) return rc;
    if (!h_in || !h_out) return fail(STENCIL_EINVAL, "null host buffer");
    const size_t bytes = (size_t)cell_count(*p) * sizeof(float);
    std::lock_guard<std::mutex> lock(g_ws_mu);
    const int dev = current_device();
    if (dev < 0 || dev >= 64) return fail(STENCIL_ENODEVICE, "device index out of range");
    DeviceWorkspace *w = nullptr;
    rc = ws_grids(dev, bytes, &w);
    if (rc) return rc;
    const void *d_in = mapped_host(h_in, bytes);
    void *d_out = const_cast<void *>(mapped_host(h_out, bytes));
    ST_CUDA(cudaEventRecord(w->ev[0], w->stream));
    if (d_in) {
        rc = launch_copy16(w->u[0], d_in, bytes, w->stream);
        if (rc) return rc;
    } else {
        ST_CUDA(cudaMemcpyAsync(w->u[0], h_in, bytes, cudaMemcpyHostToDevice, w->stream));
    }
    if (p->mode == STENCIL_MODE_JACOBI)
        ST_CUDA(cudaMemcpyAsync(w->u[1], w->u[0], bytes, cudaMemcpyDeviceToDevice, w->stream));
    else
        ST_CUDA(cudaMemsetAsync(w->u[1], 0, bytes, w->stream));
    float *res = nullptr;
    ST_CUDA(cudaEventRecord(w->ev[2], w->stream));
    rc = stencil_dispatch_ex(p, w->u[0], w->u[1], reinterpret_cast<stencil_stream_t>(w->stream),
                             &res);
    if (rc) {
        cudaStreamSynchronize(w->stream);
        return rc;
    }
    ST_CUDA(cudaEventRecord(w->ev[3], w->stream));
    if (d_out) {
        rc = launch_copy16(d_out, res, bytes, w->stream);
        if (rc) {
            cudaStreamSynchronize(w->stream);
            return rc;
        }
    } else {
        ST_CUDA(cudaMemcpyAsync(h_out, res, bytes, cudaMemcpyDeviceToHost, w->stream));
    }
    ST_CUDA(cudaEventRecord(w->ev[1], w->stream));
    ST_CUDA(cudaStreamSynchronize(w->stream));
    if (ms_total) ST_CUDA(cudaEventElapsedTime(ms_total, w->ev[0], w->ev[1]));
    if (ms_sweeps) ST_CUDA(cudaEventElapsedTime(ms_sweeps, w->ev[2], w->ev[3]));
    return STENCIL_OK;
}

int stencil_run_host(const stencil_params *p, const float *h_in, float *h_out, float *ms) {
    return stencil_run_host_timed(p, h_in, h_out, ms, nullptr);
}

int stencil_init_reference(const stencil_params *p, float *d_u, stencil_stream_t stream) {
    int rc = stencil_params_check(p);
    if (rc) return rc;
    if (!d_u) return fail(STENCIL_EINVAL, "null buffer");
    return launch_init_reference(make_geom(*p), p->dims, d_u, reinterpret_cast<cudaStream_t>(stream));
}

int stencil_init_uniform(float *d_u, size_t count, uint64_t seed, stencil_stream_t stream) {
    if (!d_u && count) return fail(STENCIL_EINVAL, "null buffer");
    return launch_init_uniform(d_u, count, seed, reinterpret_cast<cudaStream_t>(stream));
}

int stencil_copy_border(const stencil_params *p, const float *d_src, float *d_dst,
                        stencil_stream_t stream) {
    int rc = stencil_params_check(p);
    if (rc) return rc;
    if (!d_src || !d_dst) return fail(STENCIL_EINVAL, "null buffer");
    return launch_copy_border(make_geom(*p), p->dims, d_src, d_dst,
                              reinterpret_cast<cudaStream_t>(stream));
}

int stencil_residual(const stencil_params *p, const float *d_u, double *rel_residual,
                     stencil_stream_t stream) {
    int rc = stencil_params_check(p);
    if (rc) return rc;
    if (!d_u || !rel_residual) return fail(STENCIL_EINVAL, "null pointer");
    if (reinterpret_cast<uintptr_t>(d_u) & 15)
        return fail(STENCIL_EINVAL, "d_u must be 16-byte aligned (the kernels read 16-byte vectors)");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    void *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_ws_mu);
        const int dev = current_device();
        rc = ws_scratch(dev, residual_scratch_bytes(), &scratch);
        if (rc) return rc;
        rc = launch_residual(make_geom(*p), p->dims, d_u, static_cast<double *>(scratch), s);
        if (rc) return rc;
        double sums[2];
        const size_t off = residual_scratch_bytes() / sizeof(double) - 2;
        ST_CUDA(cudaMemcpyAsync(sums, static_cast<double *>(scratch) + off, sizeof sums,
                                cudaMemcpyDeviceToHost, s));
        ST_CUDA(cudaStreamSynchronize(s));
        *rel_residual = sums[1] > 0.0 ? sqrt(sums[0]) / sqrt(sums[1]) : sqrt(sums[0]);
    }
    return STENCIL_OK;
}

int stencil_solve(const stencil_params *p, float *d_u1, float *d_u2, double tol, int check_every,
                  stencil_stream_t stream, stencil_solve_result *result) {
    int rc = stencil_params_check(p);
    if (rc) return rc;
    if (!result) return fail(STENCIL_EINVAL, "null result");
    if (p->mode != STENCIL_MODE_JACOBI) return fail(STENCIL_EINVAL, "a tolerance needs JACOBI sweeps");
    if (check_every < 1 || !(tol >= 0.0)) return fail(STENCIL_EINVAL, "check_every >= 1 and tol >= 0");
    float *cur = d_u1, *nxt = d_u2;
    stencil_params q = *p;
    double rel = 0.0;
    int done = 0, checks = 0;
    rc = stencil_residual(p, cur, &rel, stream);
    if (rc) return rc;
    ++checks;
    long long launches = 0;
    while (rel >= tol && done < p->iterations) {
        q.iterations = std::min(check_every, p->iterations - done);
        float *res = nullptr;
        rc = stencil_dispatch_ex(&q, cur, nxt, stream, &res);
        if (rc) return rc;
        launches += t_launches;
        if (res != cur) std::swap(cur, nxt);
        done += q.iterations;
        rc = stencil_residual(p, cur, &rel, stream);
        if (rc) return rc;
        ++checks;
    }
    t_launches = launches + 2LL * checks;
    result->sweeps = done;
    result->checks = checks;
    result->rel_residual = rel;
    result->d_result = cur;
    return STENCIL_OK;
}

int stencil_tuning_set(const stencil_params *key, const stencil_params *choice) {
    int rc = stencil_params_check(key);
    if (rc) return rc;
    if (!choice) return fail(STENCIL_EINVAL, "null choice");
    stencil_params c = *choice;
    c.dims = key->dims; c.nx = key->nx; c.ny = key->ny; c.nz = key->nz;
    c.radius = key->radius; c.iterations = key->iterations; c.mode = key->mode;
    rc = stencil_params_check(&c);
    if (rc) return rc;
    std::lock_guard<std::mutex> lock(g_tune_mu);
    const int b = size_bucket(*key);
    for (TuneEntry &e : g_tune)
        if (e.dims == key->dims && e.radius == key->radius && e.bucket == b) {
            e.choice = c;
            return STENCIL_OK;
        }
    if (g_tune.size() >= 256) return fail(STENCIL_EINVAL, "tuning table full (256 entries)");
    g_tune.push_back({key->dims, key->radius, b, c});
    return STENCIL_OK;
}

int stencil_tuning_get(const stencil_params *key, stencil_params *choice) {
    int rc = stencil_params_check(key);
    if (rc) return rc;
    if (!choice) return fail(STENCIL_EINVAL, "null choice");
    if (!tuned_choice(*key, choice)) return fail(STENCIL_EINVAL, "no tuning entry for this key");
    return STENCIL_OK;
}

int stencil_tuning_clear(void) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune.clear();
    return STENCIL_OK;
}

const char *stencil_strerror(int status) {
    switch (status) {
        case STENCIL_OK: return "success";
        case STENCIL_EINVAL: return "invalid argument";
        case STENCIL_ENOMEM: return "out of memory";
        case STENCIL_ECUDA: return "CUDA runtime error";
        case STENCIL_ETIMEOUT: return "device-side wait timed out";
        case STENCIL_EUNSUPPORTED: return "unsupported configuration";
        case STENCIL_ENODEVICE: return "no suitable CUDA device";
        default: return "unknown status";
    }
}

const char *stencil_last_error(void) { return t_err; }

int stencil_last_dispatch(const char **engine, long long *kernel_launches) {
    if (engine) *engine = t_engine;
    if (kernel_launches) *kernel_launches = t_launches;
    return STENCIL_OK;
}

int stencil_device_status(int *status) {
    if (!status) return fail(STENCIL_EINVAL, "null pointer");
    ST_CUDA(cudaDeviceSynchronize());
    unsigned v = 0, zero = 0;
    ST_CUDA(cudaMemcpyFromSymbol(&v, g_device_status, sizeof v));
    ST_CUDA(cudaMemcpyToSymbol(g_device_status, &zero, sizeof zero));
    *status = (int)v;
    return STENCIL_OK;
}

int stencil_release(void) {
    tb2d_release();
    std::lock_guard<std::mutex> lock(g_ws_mu);
    const int dev = current_device();
    if (dev < 0 || dev >= 64) return STENCIL_OK;
    DeviceWorkspace &w = g_ws[dev];
    if (w.stream) cudaStreamSynchronize(w.stream);
    cudaFree(w.u[0]);
    cudaFree(w.u[1]);
    cudaFree(w.scratch);
    if (w.ev[0]) cudaEventDestroy(w.ev[0]);
    if (w.ev[1]) cudaEventDestroy(w.ev[1]);
    if (w.stream) cudaStreamDestroy(w.stream);
    w = DeviceWorkspace();
    return STENCIL_OK;
}

int stencil_heuristic_block(const stencil_params *p, int threads, int *bx, int *by, int *bz) {
    if (!p || !bx || !by || !bz) return fail(STENCIL_EINVAL, "null argument");
    if (p->block_x < 1 || threads < 1 || threads > 1024 || p->radius < 1 ||
        (p->dims != 2 && p->dims != 3))
        return fail(STENCIL_EINVAL, "heuristic needs dims 2/3, radius >= 1, block_x >= 1, 1..1024 threads");
    if (p->dims == 3) {
        int b0 = p->block_x;
        const bool padded = p->variant == STENCIL_VARIANT_SMEM_PADDED;
        while (padded && threads / (b0 * p->radius * p->radius) == 0 && b0 > 1) b0 /= 2;
        int b1 = std::min(std::max(2, p->radius), 8);
        int b2 = threads / (b0 * b1);
        // descending order of the three extents
        if (b0 < b2) std::swap(b0, b2);
        if (b0 < b1) std::swap(b0, b1);
        if (b1 < b2) std::swap(b1, b2);
        *bx = b0, *by = b1, *bz = b2;
    } else {
        *bx = p->block_x, *by = threads / p->block_x, *bz = 1;
    }
    return STENCIL_OK;
}

// The reference's set_smem (src/stencil_dispatch.cu:46-66): dynamic shared
// memory of a block of the role's kernel, COARSEN_X cells per thread in x.
static long long ref_role_smem(const stencil_params &p, int bx, int by, int bz) {
    if (p.variant == STENCIL_VARIANT_BASE) return 0;
    const long long R = p.radius, cf = std::max(p.coarsen_x, 1);
    const long long sx = (long long)bx * cf, px = sx + 2 * R, py = by + 2 * R, pz = bz + 2 * R;
    if (p.dims == 3) {
        if (p.variant == STENCIL_VARIANT_SMEM_PADDED) return px * py * pz * 4;
        if (p.variant == STENCIL_VARIANT_SMEM_REGISTER) return px * py * bz * 4;
        return sx * by * bz * 4;
    }
    if (p.variant == STENCIL_VARIANT_SMEM_PADDED) return px * py * 4;
    if (p.variant == STENCIL_VARIANT_SMEM_REGISTER) return px * by * 4;
    return sx * by * 4;
}

// calculate_smem (src/stencil_dispatch.cu:103-112): threads -> the shaped
// block's shared memory.
struct RefRoleSmem {
    stencil_params p;
    size_t operator()(int threads) const {
        int bx = 0, by = 0, bz = 0;
        if (stencil_heuristic_block(&p, threads, &bx, &by, &bz)) return 0;
        return (size_t)ref_role_smem(p, bx, by, bz);
    }
};

int stencil_heuristic_geometry(const stencil_params *p, int *threads, int *bx, int *by, int *bz) {
    int rc = stencil_params_check(p);
    if (rc) return rc;
    if (!threads || !bx || !by || !bz) return fail(STENCIL_EINVAL, "null argument");
    stencil_params q = *p;
    if (q.block_x < 1) q.block_x = 32;  // BLOCK_X's default (include/constants.h)
    if (q.variant == STENCIL_VARIANT_AUTO || q.variant == STENCIL_VARIANT_COOP ||
        q.variant == STENCIL_VARIANT_CLUSTER)
        return fail(STENCIL_EINVAL, "the heuristic shapes the one-sweep roles (BASE, SMEM, "
                                    "SMEM_PADDED, SMEM_REGISTER)");
    const Geom g = make_geom(q);
    const void *fn = q.variant == STENCIL_VARIANT_BASE ? base_kernel_ptr(g, q.dims)
                                                       : tile_kernel_ptr(q.dims, q.radius);
    if (!fn) return fail(STENCIL_EUNSUPPORTED, "no kernel for this role at radius %d", q.radius);
    // cudaOccupancyMaxPotentialBlockSizeVariableSMem, as the reference calls it
    // (src/stencil_dispatch.cu:143), on the kernel this library runs for the role
    int min_grid = 0, t = 0;
    RefRoleSmem smem{q};
    ST_CUDA(cudaOccupancyMaxPotentialBlockSizeVariableSMem(&min_grid, &t, fn, smem));
    rc = stencil_heuristic_block(&q, t, bx, by, bz);
    if (rc) return rc;
    *threads = t;
    return STENCIL_OK;
}

int stencil_version(int *abi_version, int *sm) {
    if (abi_version) *abi_version = STENCIL_ABI_VERSION;
    if (sm) *sm = 103;
    return STENCIL_OK;
}

}  // extern "C"

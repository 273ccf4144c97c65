// noalloc.cu -- stencil_residual_noalloc(): the relative-residual reduction of
// stencil_residual() for callers that must not allocate device memory.
//
// Some callers cannot let a library allocate: a serving or solver process that
// has already handed all free device memory to its own pool allocator, or code
// on a latency-critical path where cudaMalloc / cudaFree (cudaFree
// synchronises the whole device) are not allowed.  stencil_residual() keeps a
// lazily grown workspace for its per-block partial sums; this entry point uses
// a fixed, file-scope device array instead and calls no allocating routine.
//
// The array holds kNoAllocMaxParts (sum r^2, sum b^2) pairs plus the final
// pair: 16384 * 16 + 16 = 262,160 bytes, which every GPU that loads this
// library keeps until the process exits.  One partial pair covers 65,536
// update cells, so grids with more than 16384 * 65536 = 2^30 update cells are
// rejected with STENCIL_EINVAL.
//
// All calls share the array and it keeps the previous call's contents.  No
// slot needs clearing: every pair the final stage reads was written earlier by
// the same call.  Calls whose kernels can overlap on one GPU (calls on two
// streams, or from two host threads) race on the array: serialise them.
//
// Every call looks up the array's device address (cudaGetSymbolAddress, which
// allocates nothing) with the caller's device current, so the address stays
// right after a cudaDeviceReset reloads the library's module.  The array is
// reserved when the CUDA runtime loads this library's module on a device: at
// the first kernel launch or symbol lookup under lazy module loading (the
// default), at context creation with CUDA_MODULE_LOADING=EAGER.  The call
// synchronises its stream, so it cannot be captured into a CUDA graph.
#include <stdint.h>

#include "host.hpp"

namespace st {

// The two stages of the regular residual path (k_util.cu; 256-thread blocks).
int launch_residual_partial(const Geom &g, int dims, const float *u, double *part, int blocks,
                            cudaStream_t s);
int launch_residual_final(const Geom &g, int dims, const double *part, int nparts, double *out,
                          cudaStream_t s);

constexpr int kNoAllocMaxParts = 16384;
constexpr long long kNoAllocCellsPerPart = 65536;

static __device__ __align__(256) double g_noalloc_scratch[2 * kNoAllocMaxParts + 2];

// Device address of g_noalloc_scratch on the current device.  In host code
// the array's name is only a host-side stand-in, never a device address.
static int noalloc_scratch(double **out) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    *out = static_cast<double *>(p);
    return STENCIL_OK;
}

}  // namespace st

using namespace st;

extern "C" int stencil_residual_noalloc(const stencil_params *p, const float *d_u,
                                        double *rel_residual, stencil_stream_t stream) {
    int rc = stencil_params_check(p);
    if (rc) return rc;
    if (!d_u || !rel_residual) return fail(STENCIL_EINVAL, "null pointer");
    if (reinterpret_cast<uintptr_t>(d_u) & 15)
        return fail(STENCIL_EINVAL, "d_u must be 16-byte aligned (the kernels read 16-byte vectors)");
    const Geom g = make_geom(*p);
    const long long inner = (long long)(g.nx - 2 * g.radius) * (g.ny - 2 * g.radius) *
                            (p->dims == 3 ? g.nz - 2 * g.radius : 1);
    const long long parts = (inner + kNoAllocCellsPerPart - 1) / kNoAllocCellsPerPart;
    if (parts > kNoAllocMaxParts)
        return fail(STENCIL_EINVAL,
                    "grid has %lld update cells; stencil_residual_noalloc handles at most "
                    "%lld (its fixed scratch holds %d partial sums of %lld cells each); use "
                    "stencil_residual for larger grids",
                    inner, (long long)kNoAllocMaxParts * kNoAllocCellsPerPart, kNoAllocMaxParts,
                    kNoAllocCellsPerPart);
    double *scratch = nullptr;
    rc = noalloc_scratch(&scratch);
    if (rc) return rc;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const int nparts = parts > 0 ? (int)parts : 1;
    rc = launch_residual_partial(g, p->dims, d_u, scratch, nparts, s);
    if (!rc) rc = launch_residual_final(g, p->dims, scratch, nparts, scratch + 2 * kNoAllocMaxParts, s);
    if (rc) return rc;
    double sums[2];
    ST_CUDA(cudaMemcpyAsync(sums, scratch + 2 * kNoAllocMaxParts, sizeof sums,
                            cudaMemcpyDeviceToHost, s));
    ST_CUDA(cudaStreamSynchronize(s));
    *rel_residual = sums[1] > 0.0 ? sqrt(sums[0]) / sqrt(sums[1]) : sqrt(sums[0]);
    return STENCIL_OK;
}

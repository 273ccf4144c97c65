// k_rows2d.cu -- 2-D grids too large for one tile per SM: every sweep in one
// cooperative launch over the whole GPU ("coop" role,
// src/stencil_kernel_coop.cu:5-49), with a bounded grid-wide barrier between
// sweeps instead of a launch per sweep.
//
// A thread owns one float4 chunk column of a block of HB rows: it keeps the
// column's rows j-R .. j+R in a register queue (one new 16-byte load per
// row, the smem_register idea of src/stencils.cu:71-83 on registers) and
// loads the chunks left and right of its own for the x-neighbours, so a
// 4-cell update costs three 16-byte loads at any R <= 4 (the base kernel:
// 3 + 2R).  Items (chunk column, row block) are spread over the resident CTAs
// with a grid stride; consecutive threads take consecutive chunk columns, so
// a warp's loads and stores are contiguous 512-byte segments.
//
// Loads are plain (L1-cached): a buffer is rewritten every other sweep
// inside the launch, and every read of another CTA's writes follows the grid
// barrier's acquire at GPU scope and a CTA barrier, after which weak loads
// observe those writes (PTX memory model).  Every cell keeps the reference's summation order (axis i
// offsets -R..-1, +1..+R, then axis j, from +0) and division, so results are
// bit-identical to single sweeps; cells outside the update region are never
// written.
#include <algorithm>
#include <cstdlib>
#include <mutex>
#include <vector>

#include "host.hpp"
#include "rows_body.cuh"

namespace st {
namespace {

constexpr int kRowsThreads = 512;

template <int R, bool L1>
__global__ void __launch_bounds__(kRowsThreads, R <= 2 ? 2 : 1)
    k_rows2d(float *a, float *b, Geom g, int hb, int nblk, int iters, unsigned *bar) {
    __shared__ int s_ok;
    for (int sw = 0; sw < iters; ++sw) {
        const float *src = (sw & 1) ? b : a;
        float *dst = (sw & 1) ? a : b;
        rows2d_sweep<R, kRowsThreads, L1>(src, dst, g, hb, nblk, blockIdx.x, gridDim.x);
        if (sw + 1 < iters) {
            // every CTA's writes of this sweep before any CTA's next reads
            __syncthreads();
            if (threadIdx.x == 0) {
                grid_arrive(bar);
                s_ok = grid_wait_bounded(bar, (unsigned)(sw + 1) * gridDim.x) ? 1 : 0;
            }
            __syncthreads();
            if (!s_ok) return;
        }
    }
}

using RowsFn = void (*)(float *, float *, Geom, int, int, int, unsigned *);

// Loads: plain, L1-cached (the x-neighbour chunks are other threads' centre
// chunks of the same row), legal because every read of another CTA's writes
// follows the grid barrier's acquire and a CTA barrier; STENCIL_ROWS_L1=0
// (read at each launch) selects ld.global.cg.  GB300, R = 1, bit-identical:
// 1024^2 309.5 -> 327.0, 1500^2 438.7 -> 493.0, 2048^2 575.1 -> 640.4,
// 4096^2 626.1 -> 634.4, 8192^2 592.8 -> 596.1 GCell/s; R = 4 2048^2
// 426.0 -> 445.0.
RowsFn rows_fn(int r, bool l1 = false) {
    switch (r * 2 + (l1 ? 1 : 0)) {
        case 2: return k_rows2d<1, false>;
        case 3: return k_rows2d<1, true>;
        case 4: return k_rows2d<2, false>;
        case 5: return k_rows2d<2, true>;
        case 6: return k_rows2d<3, false>;
        case 7: return k_rows2d<3, true>;
        case 8: return k_rows2d<4, false>;
        case 9: return k_rows2d<4, true>;
        default: return nullptr;
    }
}

bool rows_l1() {
    const char *e = std::getenv("STENCIL_ROWS_L1");
    return !(e && e[0] == '0');
}

// Resident CTAs of the radius-r kernel (once per radius and device).
int rows_ctas(int r) {
    static std::mutex mu;
    static std::vector<std::pair<int, int>> cache;  // (device * 8 + r, ctas)
    const int dev = current_device();
    std::lock_guard<std::mutex> lock(mu);
    for (auto &c : cache)
        if (c.first == dev * 8 + r) return c.second;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, reinterpret_cast<const void *>(rows_fn(r)),
                                                      kRowsThreads, 0) != cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    const int ctas = n * num_sms();
    cache.push_back({dev * 8 + r, ctas});
    return ctas;
}

}  // namespace

bool rows2d_supported(const Geom &g, int dims) {
    return dims == 2 && g.sy % 4 == 0 && g.radius >= 1 && g.radius <= 4 &&
           (long long)(g.sy / 4) * (g.ny - 2 * g.radius) < (1LL << 31) && rows_ctas(g.radius) > 0;
}

int rows2d_capacity(const Geom &g) { return rows_ctas(g.radius); }

// Row blocks of a rows sweep of g on `threads` threads: as tall as keeps
// about four items per thread (a taller block re-reads fewer halo rows), at
// most 64 rows and at least 4 (R = 1) or 8 rows (measured on 1024^2 to
// 32768^2 grids).
void rows2d_plan(const Geom &g, long long threads, int *hb, int *nblk) {
    const int nch = (int)(g.sy / 4), rows = g.ny - 2 * g.radius;
    const long long hb_min = g.radius == 1 ? 4 : 8;
    int h = (int)std::min<long long>(64, std::max<long long>(hb_min, (long long)nch * rows / (4 * std::max(1LL, threads))));
    h = std::max(1, std::min(h, rows));
    *hb = h;
    *nblk = (rows + h - 1) / h;
}

int run_rows2d(const Geom &g, float *a, float *b, int iters, cudaStream_t s, float **res,
               int max_ctas) {
    if (!rows2d_supported(g, 2))
        return fail(STENCIL_EUNSUPPORTED, "persistent 2-D rows kernel: row pitch %% 4 == 0, R <= 4");
    if (res) *res = (iters & 1) ? b : a;
    if (iters <= 0) return STENCIL_OK;
    const int ctas = max_ctas > 0 ? std::min(max_ctas, rows_ctas(g.radius)) : rows_ctas(g.radius);
    const int nch = (int)(g.sy / 4);
    int hb = 0, nblk = 0;
    rows2d_plan(g, (long long)ctas * kRowsThreads, &hb, &nblk);
    const int items = nch * nblk;
    const int grid = (int)std::max<long long>(1, std::min<long long>(ctas, (items + kRowsThreads - 1) / kRowsThreads));
    unsigned *bar = nullptr;
    int rc = grid_bar_slot(s, &bar);
    if (rc) return rc;
    Geom gg = g;
    int hb_ = hb, nb_ = nblk, n = iters;
    void *args[] = {&a, &b, &gg, &hb_, &nb_, &n, &bar};
    ST_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(rows_fn(g.radius, rows_l1())), dim3(grid),
                                        dim3(kRowsThreads), args, 0, s));
    note_launches("rows2d-persistent", 1);
    return STENCIL_OK;
}

}  // namespace st

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
// Loads use ld.global.cg (L2, not L1): a buffer is rewritten every other
// sweep inside the launch, so a line kept in an SM's L1 from two sweeps back
// would be stale.  Every cell keeps the reference's summation order (axis i
// offsets -R..-1, +1..+R, then axis j, from +0) and division, so results are
// bit-identical to single sweeps; cells outside the update region are never
// written.
#include <algorithm>
#include <mutex>
#include <vector>

#include "host.hpp"

namespace st {
namespace {

constexpr int kRowsThreads = 512;

__device__ __forceinline__ float4 rows_ld4(const float *p) {
    return __ldcg(reinterpret_cast<const float4 *>(p));
}

template <int R>
__global__ void __launch_bounds__(kRowsThreads, R <= 2 ? 2 : 1)
    k_rows2d(float *a, float *b, Geom g, int hb, int nblk, int iters, unsigned *bar) {
    constexpr int C = 4 * R;
    constexpr int RA = (R + 3) & ~3;  // x halo in whole chunks (R <= 4: one chunk)
    static_assert(RA == 4, "one neighbour chunk per side");
    __shared__ int s_ok;
    // nx: the width (update region x < nx - R); px: the row pitch (a
    // multiple of 4, the chunk columns cover it)
    const int nx = g.nx, ny = g.ny, px = (int)g.sy, nch = px >> 2;
    const int items = nch * nblk;
    for (int sw = 0; sw < iters; ++sw) {
        const float *src = (sw & 1) ? b : a;
        float *dst = (sw & 1) ? a : b;
        for (int it = blockIdx.x * kRowsThreads + threadIdx.x; it < items;
             it += gridDim.x * kRowsThreads) {
            const int c = it % nch, rb = it / nch;
            const int x0 = 4 * c;
            if (x0 + 3 < R || x0 >= nx - R) continue;
            const int j0 = R + rb * hb, j1 = min(j0 + hb, ny - R);
            const bool full = x0 >= R && x0 + 3 < nx - R;
            const float *col = src + x0;
            float *dcol = dst + x0;
            float4 q[2 * R + 1];  // rows j-R .. j+R of this chunk column
#pragma unroll
            for (int k = 0; k < 2 * R; ++k) q[k] = rows_ld4(col + (long long)(j0 - R + k) * px);
            // the loads of row j+1 are issued before row j is computed (one
            // row of software pipelining: two rows of loads in flight)
            const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
            float4 nq = rows_ld4(col + (long long)(j0 + R) * px);
            float4 nl = c > 0 ? rows_ld4(col + (long long)j0 * px - 4) : z4;
            float4 nr = c + 1 < nch ? rows_ld4(col + (long long)j0 * px + 4) : z4;
            for (int j = j0; j < j1; ++j) {
                q[2 * R] = nq;
                const float4 l4 = nl, r4 = nr;
                if (j + 1 < j1) {
                    const float *nrow = col + (long long)(j + 1) * px;
                    nq = rows_ld4(col + (long long)(j + 1 + R) * px);
                    if (c > 0) nl = rows_ld4(nrow - 4);
                    if (c + 1 < nch) nr = rows_ld4(nrow + 4);
                }
                const float4 m4 = q[R];
                const float w[12] = {l4.x, l4.y, l4.z, l4.w, m4.x, m4.y,
                                     m4.z, m4.w, r4.x, r4.y, r4.z, r4.w};
                float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
                for (int o = -R; o <= R; ++o) {
                    if (!o) continue;
#pragma unroll
                    for (int e = 0; e < 4; ++e) acc[e] += w[4 + e + o];
                }
#pragma unroll
                for (int o = -R; o <= R; ++o) {
                    if (!o) continue;
                    const float4 v = q[R + o];
                    acc[0] += v.x; acc[1] += v.y; acc[2] += v.z; acc[3] += v.w;
                }
                float out[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    out[e] = div_coeff<C>(acc[e]);
                    if (g.legacy) out[e] -= w[4 + e];
                }
                float *d = dcol + (long long)j * px;
                if (full) {
                    *reinterpret_cast<float4 *>(d) = make_float4(out[0], out[1], out[2], out[3]);
                } else {
#pragma unroll
                    for (int e = 0; e < 4; ++e)
                        if (in_range(x0 + e, nx, R)) d[e] = out[e];
                }
#pragma unroll
                for (int k = 0; k < 2 * R; ++k) q[k] = q[k + 1];
            }
        }
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

RowsFn rows_fn(int r) {
    switch (r) {
        case 1: return k_rows2d<1>;
        case 2: return k_rows2d<2>;
        case 3: return k_rows2d<3>;
        case 4: return k_rows2d<4>;
        default: return nullptr;
    }
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

int run_rows2d(const Geom &g, float *a, float *b, int iters, cudaStream_t s, float **res,
               int max_ctas) {
    if (!rows2d_supported(g, 2))
        return fail(STENCIL_EUNSUPPORTED, "persistent 2-D rows kernel: row pitch %% 4 == 0, R <= 4");
    if (res) *res = (iters & 1) ? b : a;
    if (iters <= 0) return STENCIL_OK;
    const int ctas = max_ctas > 0 ? std::min(max_ctas, rows_ctas(g.radius)) : rows_ctas(g.radius);
    const int nch = (int)(g.sy / 4), rows = g.ny - 2 * g.radius;
    // Row blocks as tall as keeps about four items per resident thread (a
    // taller block re-reads fewer halo rows), at most 64 rows and at least 4
    // (R = 1) or 8 rows (measured on 1024^2 to 32768^2 grids).
    const long long threads = (long long)ctas * kRowsThreads;
    const long long hb_min = g.radius == 1 ? 4 : 8;
    int hb = (int)std::min<long long>(64, std::max<long long>(hb_min, (long long)nch * rows / (4 * threads)));
    hb = std::min(hb, rows);
    const int nblk = (rows + hb - 1) / hb;
    const int items = nch * nblk;
    const int grid = (int)std::max<long long>(1, std::min<long long>(ctas, (items + kRowsThreads - 1) / kRowsThreads));
    unsigned *bar = nullptr;
    int rc = grid_bar_slot(s, &bar);
    if (rc) return rc;
    Geom gg = g;
    int hb_ = hb, nb_ = nblk, n = iters;
    void *args[] = {&a, &b, &gg, &hb_, &nb_, &n, &bar};
    ST_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(rows_fn(g.radius)), dim3(grid),
                                        dim3(kRowsThreads), args, 0, s));
    note_launches("rows2d-persistent", 1);
    return STENCIL_OK;
}

}  // namespace st

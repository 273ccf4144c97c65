// k_rows.cu -- 2.5D streaming sweep over full-width row slabs (3-D grids with
// nx a multiple of 128 and nx <= 512; "smem_register" role).
//
// Same pipeline as k_stream.cu (one producer warp, consumer warps with a
// register z-queue, full/empty mbarriers, bounded waits), but a CTA owns all
// nx columns of TY rows.  The rows y0-R .. y0+TY+R-1 of a plane are one
// contiguous range of global memory, so each plane arrives with ONE
// cp.async.bulk copy of (TY + 2R) * nx * 4 bytes: DRAM sees long sequential
// reads instead of many short box rows, and no x halo is needed (the
// x-neighbours of the first/last chunk are border cells' neighbours only).
#include <algorithm>
#include <cmath>

#include "host.hpp"

namespace st {

template <int R, int TY, int RY, int NS>
struct RowsShape {
    static constexpr int ROWS = TY + 2 * R;
    static constexpr int CONSUMER_ROWS = TY / RY;
    static_assert(TY % RY == 0 && (NS & (NS - 1)) == 0 && NS >= R + 2, "bad shape");
    __host__ __device__ static int slot_floats(int nx) { return ((ROWS * nx * 4 + 127) & ~127) / 4; }
    static int smem_bytes(int nx) { return NS * slot_floats(nx) * 4 + 128 + 2 * NS * 8; }
    static int threads(int nx) { return (nx / 4) * CONSUMER_ROWS + 32; }
};

__device__ __forceinline__ float4 rl4(const float *p) { return *reinterpret_cast<const float4 *>(p); }

// Up to nx = 512 columns: 128 chunks x 4 consumer rows + the producer warp.
constexpr int kRowsMaxThreads = 544;

template <int R, int TY, int RY, int NS>
__global__ void __launch_bounds__(128 * (TY / RY) + 32, 1)
    k_rows3d(const float *__restrict__ src, float *__restrict__ dst, Geom g, int zchunk,
             int items) {
    using S = RowsShape<R, TY, RY, NS>;
    constexpr int C = 6 * R;
    const int nx = g.nx, CW = nx >> 2;
    const int consumers = CW * S::CONSUMER_ROWS;
    const int slotf = S::slot_floats(nx);
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float *ring = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) &
                                            ~static_cast<uintptr_t>(127));
    uint64_t *full = reinterpret_cast<uint64_t *>(ring + NS * slotf);
    uint64_t *empty = full + NS;
    const int tid = threadIdx.x, lane = tid & 31;
    const int cwarps = consumers >> 5;
    if (tid == 0) {
        for (int s = 0; s < NS; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], cwarps);
        }
        fence_mbar_init();
    }
    __syncthreads();
    const int slabs = (g.ny + TY - 1) / TY;

    if (tid >= consumers) {
        // ---------------- producer ----------------
        if (tid != consumers) return;
        uint32_t q = 0;
        for (int item = blockIdx.x; item < items; item += gridDim.x) {
            const int sl = item % slabs, ch = item / slabs;
            const int y0 = sl * TY;
            const int z0 = R + ch * zchunk, z1 = min(z0 + zchunk, g.nz - R);
            const int np = (z1 - z0) + 2 * R;
            const int ra = max(0, y0 - R), rb = min(g.ny, y0 + TY + R);
            const uint32_t bytes = (uint32_t)((rb - ra) * nx * 4);
            for (int p = 0; p < np; ++p, ++q) {
                const int s = q & (NS - 1);
                const uint32_t use = q / NS;
                if (use > 0 && !mbar_wait_bounded(&empty[s], (use - 1) & 1)) return;
                fence_proxy_async();  // the consumers' reads of the slot before the bulk copy
                mbar_arrive_expect_tx(&full[s], bytes);
                const long long z = z0 - R + p;
                bulk_load(ring + s * slotf + (ra - (y0 - R)) * nx,
                          src + z * g.sz + (long long)ra * nx, bytes, &full[s]);
            }
        }
        return;
    }

    // ---------------- consumers ----------------
    const int cx = tid % CW, cy = tid / CW;
    auto release = [&](int s) {
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);
    };
    constexpr int QN = 2 * R + 1;
    float4 qz[RY][QN];
    uint32_t qb = 0;
    const int x = 4 * cx;
    const bool xin = x >= R && x + 3 < nx - R;
    const int lft = cx > 0 ? -4 : 0, rgt = cx < CW - 1 ? 4 : 0;  // clamped chunk steps
    for (int item = blockIdx.x; item < items; item += gridDim.x) {
        const int sl = item % slabs, ch = item / slabs;
        const int y0 = sl * TY;
        const int z0 = R + ch * zchunk, z1 = min(z0 + zchunk, g.nz - R);
        const int np = (z1 - z0) + 2 * R;
        const int ybase = y0 + cy * RY;
        const int own = (cy * RY + R) * nx + x;
        unsigned live = 0;
#pragma unroll
        for (int r = 0; r < RY; ++r)
            if (in_range(ybase + r, g.ny, R)) live |= 1u << r;
#pragma unroll
        for (int p = 0; p < 2 * R; ++p) {
            const uint32_t q = qb + p;
            const int s = q & (NS - 1);
            if (!mbar_wait_bounded(&full[s], (q / NS) & 1)) return;
            const float *sp = ring + s * slotf + own;
#pragma unroll
            for (int r = 0; r < RY; ++r) qz[r][p] = rl4(sp + r * nx);
            if (p < R || p >= np - R) release(s);
        }
        float *drow = dst + (long long)z0 * g.sz + (long long)ybase * g.sy + x;
        for (int zb = z0; zb < z1; zb += QN) {
#pragma unroll
            for (int ph = 0; ph < QN; ++ph) {
                const int z = zb + ph;
                if (z >= z1) break;
                const int step = z - z0;
                const int sc = (qb + step + R) & (NS - 1);
                const float *cb = ring + sc * slotf + own;
                // rows -R .. RY-1+R; at R >= 2 the own rows are the centre
                // plane's entries of the z queue, so only the 2R halo rows
                // are loaded (as in the stream kernel)
                float4 col[RY + 2 * R];
#pragma unroll
                for (int k = 0; k < RY + 2 * R; ++k)
                    col[k] = (R >= 2 && k >= R && k < R + RY) ? qz[k - R][(ph + R) % QN] : rl4(cb + (k - R) * nx);
                float acc[RY][4];
#pragma unroll
                for (int r = 0; r < RY; ++r) {
                    const float4 a = rl4(cb + r * nx + lft), b = rl4(cb + r * nx + rgt);
                    const float4 c = col[r + R];
                    const float w[12] = {a.x, a.y, a.z, a.w, c.x, c.y, c.z, c.w, b.x, b.y, b.z, b.w};
#pragma unroll
                    for (int e = 0; e < 4; ++e) acc[r][e] = 0.0f;
#pragma unroll
                    for (int o = -R; o <= R; ++o) {
                        if (o == 0) continue;
#pragma unroll
                        for (int e = 0; e < 4; ++e) acc[r][e] += w[4 + e + o];
                    }
#pragma unroll
                    for (int o = -R; o <= R; ++o) {
                        if (o == 0) continue;
                        const float4 v = col[r + R + o];
                        acc[r][0] += v.x; acc[r][1] += v.y; acc[r][2] += v.z; acc[r][3] += v.w;
                    }
#pragma unroll
                    for (int o = -R; o <= -1; ++o) {
                        const float4 v = qz[r][(ph + R + o + QN) % QN];
                        acc[r][0] += v.x; acc[r][1] += v.y; acc[r][2] += v.z; acc[r][3] += v.w;
                    }
                }
                release(sc);
                {
                    const int pn = step + 2 * R;
                    const uint32_t q = qb + pn;
                    const int s = q & (NS - 1);
                    if (!mbar_wait_bounded(&full[s], (q / NS) & 1)) return;
                    const float *sp = ring + s * slotf + own;
#pragma unroll
                    for (int r = 0; r < RY; ++r) qz[r][(ph + 2 * R) % QN] = rl4(sp + r * nx);
                    if (pn >= np - R) release(s);
                }
#pragma unroll
                for (int r = 0; r < RY; ++r)
#pragma unroll
                    for (int o = 1; o <= R; ++o) {
                        const float4 v = qz[r][(ph + R + o) % QN];
                        acc[r][0] += v.x; acc[r][1] += v.y; acc[r][2] += v.z; acc[r][3] += v.w;
                    }
                float lo = 0x1p-100f, hi = 0x1p+120f;
#pragma unroll
                for (int r = 0; r < RY; ++r)
                    if (live & (1u << r))
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            lo = fminf(lo, fabsf(acc[r][e]));
                            hi = fmaxf(hi, fabsf(acc[r][e]));
                        }
                if (__all_sync(0xffffffffu, lo >= 0x1p-100f && hi <= 0x1p+120f)) {
#pragma unroll
                    for (int r = 0; r < RY; ++r)
#pragma unroll
                        for (int e = 0; e < 4; ++e) acc[r][e] = div_fast<C>(acc[r][e]);
                } else {
#pragma unroll
                    for (int r = 0; r < RY; ++r)
#pragma unroll
                        for (int e = 0; e < 4; ++e) acc[r][e] = acc[r][e] / (float)C;
                }
                if (g.legacy) {
#pragma unroll
                    for (int r = 0; r < RY; ++r) {
                        const float4 c = col[r + R];
                        acc[r][0] -= c.x; acc[r][1] -= c.y; acc[r][2] -= c.z; acc[r][3] -= c.w;
                    }
                }
                if (xin) {
#pragma unroll
                    for (int r = 0; r < RY; ++r)
                        if (live & (1u << r))
                            stg4(drow + r * g.sy, acc[r][0], acc[r][1], acc[r][2], acc[r][3]);
                } else {
#pragma unroll
                    for (int r = 0; r < RY; ++r)
                        if (live & (1u << r))
#pragma unroll
                            for (int e = 0; e < 4; ++e)
                                if (in_range(x + e, nx, R)) drow[r * g.sy + e] = acc[r][e];
                }
                drow += g.sz;
            }
        }
        qb += np;
    }
}

namespace {

struct RowsKernel {
    const void *fn;
    int ty, smem, threads;
};

template <int R, int TY, int RY, int NS>
RowsKernel rk(int nx) {
    using S = RowsShape<R, TY, RY, NS>;
    return {reinterpret_cast<const void *>(k_rows3d<R, TY, RY, NS>), TY, S::smem_bytes(nx),
            S::threads(nx)};
}

// Slab shapes (rows per CTA, rows per thread, ring slots).  shape 0 is the
// default per radius (fastest measured at 512^3); 1 and 2 are alternatives
// for the tuner.  Deep rings (many planes in flight) matter most.
RowsKernel pick_rows(int r, int nx, int shape = 0) {
    switch (r) {
        case 1:
            if (shape == 1) return rk<1, 8, 2, 8>(nx);
            if (shape == 2) return rk<1, 16, 4, 4>(nx);
            return rk<1, 4, 1, 16>(nx);
        case 2:
            if (shape == 1) return rk<2, 8, 2, 8>(nx);
            if (shape == 2) return rk<2, 2, 1, 16>(nx);
            return rk<2, 4, 1, 8>(nx);
        case 4:
            if (shape == 1) return rk<4, 4, 1, 8>(nx);
            return rk<4, 2, 1, 8>(nx);
        default:
            return {nullptr, 0, 0, 0};
    }
}

}  // namespace

bool rows3d_supported(const Geom &g) {
    if (g.nx % 128 || g.radius < 1 || g.radius > 4) return false;
    RowsKernel k = pick_rows(g.radius, g.nx);
    return k.fn && k.smem <= 227 * 1024 && k.threads <= kRowsMaxThreads;
}

int run_rows3d(const Geom &g, float *a, float *b, int iters, int shape, cudaStream_t s,
               float **res) {
    if (!rows3d_supported(g)) return fail(STENCIL_EUNSUPPORTED, "row-slab kernel: nx %% 128 == 0, nx <= 512, R in {1, 2, 4}");
    const int R = g.radius;
    RowsKernel k = pick_rows(R, g.nx, shape);
    if (k.smem > 227 * 1024 || k.threads > kRowsMaxThreads)
        return fail(STENCIL_EUNSUPPORTED, "row-slab shape %d does not fit nx %d", shape, g.nx);
    ST_CUDA(cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, k.smem));
    int per_sm = 0;
    ST_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k.fn, k.threads, k.smem));
    if (per_sm < 1) return fail(STENCIL_EUNSUPPORTED, "row-slab kernel does not fit on an SM");
    const int resident = per_sm * num_sms();
    const int slabs = (g.ny + k.ty - 1) / k.ty;
    const int zin = g.nz - 2 * R;
    int nchunks = 1;
    double best = 1e30;
    for (int n = 1; n <= std::max(1, zin / 8); ++n) {
        const int zc = (zin + n - 1) / n;
        const long long it = (long long)slabs * ((zin + zc - 1) / zc);
        const double waves = std::ceil((double)it / resident);
        const double fill = (double)it / (waves * resident);
        const double halo = 1.0 + 0.5 * (2.0 * R) / zc;  // chunk-edge planes are re-read
        const double cost = halo / fill + 0.002 * waves;
        if (cost < best - 1e-9) { best = cost; nchunks = n; }
    }
    int zchunk = (zin + nchunks - 1) / nchunks;
    nchunks = (zin + zchunk - 1) / zchunk;
    int items = slabs * nchunks;
    const int grid = std::min(items, resident);
    float *cur = a, *nxt = b;
    Geom gg = g;
    note_launches("rows3d", iters);
    for (int it = 0; it < iters; ++it) {
        const float *src = cur;
        void *args[] = {&src, &nxt, &gg, &zchunk, &items};
        ST_CUDA(cudaLaunchKernel(k.fn, dim3(grid), dim3(k.threads), args, k.smem, s));
        std::swap(cur, nxt);
    }
    if (res) *res = cur;
    return STENCIL_OK;
}

}  // namespace st

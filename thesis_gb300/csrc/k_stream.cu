// k_stream.cu -- 2.5D streaming sweep for 3-D grids ("smem_register" role,
// src/stencil_kernel_smem_register.cu:8-62, and "coop" single-sweep role).
//
// A CTA owns an x-y tile of TX x TY cells and a chunk of z-planes, and marches
// along z.  Plane tiles including their halo ((TX + 2*RA) x (TY + 2*R) cells,
// RA = R rounded up to 4 so that every TMA x coordinate is 16-byte aligned)
// are fetched by TMA (cp.async.bulk.tensor.3d, completion on an mbarrier) into
// a ring of NS = 2R + 1 + LOOK slots: the 2R+1 planes of the current window
// plus LOOK planes in flight.  Cells outside the grid arrive as zeros (TMA
// out-of-bounds fill); they are never used by an updated cell.  Each thread
// computes four consecutive cells of one row: x-neighbours from 16-byte shared
// loads of its row, y-neighbours from the rows above and below, z-neighbours
// from the other planes of the window.  Every input cell is read from HBM
// once per sweep; halos of neighbouring tiles and chunks come from L2.
//
// The work list is (tile, z-chunk) items, chunk-major so that co-resident CTAs
// work on neighbouring tiles of the same z range (their halo reads hit L2).
// CTAs loop over items (grid <= resident CTAs) with a monotone plane sequence
// number that fixes each plane's ring slot and mbarrier parity.
#include <algorithm>

#include "host.hpp"

namespace st {

template <int R, int TX, int TY>
struct StreamShape {
    static constexpr int RA = (R + 3) & ~3;
    static constexpr int PW = TX + 2 * RA;     // plane tile width (cells)
    static constexpr int PH = TY + 2 * R;      // plane tile height (rows)
    static constexpr int PLANE_BYTES = PW * PH * 4;
    static constexpr int SLOT_BYTES = (PLANE_BYTES + 127) & ~127;
    static constexpr int LOOK = R >= 4 ? 2 : 3;
    static constexpr int NS = 2 * R + 1 + LOOK;
    static constexpr int THREADS = (TX / 4) * TY;
    // ring + alignment slack + one mbarrier per slot
    static constexpr int SMEM_BYTES = NS * SLOT_BYTES + 128 + NS * 8;
    static_assert(PW <= 256 && PH <= 256, "TMA box dimensions are limited to 256");
    static_assert(TX % 4 == 0, "TX must be a multiple of 4");
};

template <int R, int TX, int TY>
__global__ void __launch_bounds__(StreamShape<R, TX, TY>::THREADS)
    k_stream3d(const __grid_constant__ CUtensorMap src_map, float *__restrict__ dst, Geom g,
               int tiles_x, int tiles_y, int zchunk, int items) {
    using S = StreamShape<R, TX, TY>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float *ring = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) &
                                            ~static_cast<uintptr_t>(127));
    uint64_t *full = reinterpret_cast<uint64_t *>(ring + S::NS * (S::SLOT_BYTES / 4));
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = tx + ty * (TX / 4);
    if (tid == 0) {
        prefetch_tensormap(&src_map);
        for (int s = 0; s < S::NS; ++s) mbar_init(&full[s], 1);
        fence_mbar_init();
    }
    __syncthreads();

    uint32_t qbase = 0;  // sequence number of the first plane of the current item
    const int ntiles = tiles_x * tiles_y;
    for (int item = blockIdx.x; item < items; item += gridDim.x) {
        const int t = item % ntiles, ch = item / ntiles;
        const int x0 = (t % tiles_x) * TX, y0 = (t / tiles_x) * TY;
        const int z0 = R + ch * zchunk;
        const int z1 = min(z0 + zchunk, g.nz - R);
        const int np = (z1 - z0) + 2 * R;  // planes z0-R .. z1+R-1
        if (tid == 0) {
            const int pro = min(np, S::NS);
            for (int p = 0; p < pro; ++p) {
                const uint32_t q = qbase + p;
                const int s = q % S::NS;
                mbar_arrive_expect_tx(&full[s], S::PLANE_BYTES);
                tma_load_3d(ring + s * (S::SLOT_BYTES / 4), &src_map, &full[s], x0 - S::RA,
                            y0 - R, z0 - R + p);
            }
        }
        const int x = x0 + 4 * tx, y = y0 + ty;
        const bool row_live = x < g.nx && in_range(y, g.ny, R);
        for (int z = z0; z < z1; ++z) {
            const uint32_t qlo = qbase + (z - z0);  // plane z-R
            bool ok = true;
            // Wait for the planes of the window that have not been waited on.
            for (int p = (z == z0 ? 0 : 2 * R); p <= 2 * R && ok; ++p) {
                const uint32_t q = qlo + p;
                ok = mbar_wait_bounded(&full[q % S::NS], (q / S::NS) & 1);
            }
            if (ok && row_live) {
                const float *pl[2 * R + 1];
#pragma unroll
                for (int p = 0; p <= 2 * R; ++p)
                    pl[p] = ring + ((qlo + p) % S::NS) * (S::SLOT_BYTES / 4);
                const float *c_row = pl[R] + (ty + R) * S::PW + 4 * tx;  // starts RA left of x
                float w[4 + 2 * S::RA];
#pragma unroll
                for (int q = 0; q < (4 + 2 * S::RA) / 4; ++q) {
                    const float4 v = *reinterpret_cast<const float4 *>(c_row + 4 * q);
                    w[4 * q] = v.x; w[4 * q + 1] = v.y; w[4 * q + 2] = v.z; w[4 * q + 3] = v.w;
                }
                float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
                for (int o = -R; o <= R; ++o) {
                    if (o == 0) continue;
#pragma unroll
                    for (int e = 0; e < 4; ++e) acc[e] += w[S::RA + e + o];
                }
#pragma unroll
                for (int o = -R; o <= R; ++o) {
                    if (o == 0) continue;
                    const float4 v =
                        *reinterpret_cast<const float4 *>(c_row + o * S::PW + S::RA);
                    acc[0] += v.x; acc[1] += v.y; acc[2] += v.z; acc[3] += v.w;
                }
#pragma unroll
                for (int o = -R; o <= R; ++o) {
                    if (o == 0) continue;
                    const float4 v = *reinterpret_cast<const float4 *>(
                        pl[R + o] + (ty + R) * S::PW + 4 * tx + S::RA);
                    acc[0] += v.x; acc[1] += v.y; acc[2] += v.z; acc[3] += v.w;
                }
                float out[4];
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    out[e] = star_finish<3, R>(acc[e], w[S::RA + e], g.legacy);
                float *drow = dst + (long long)z * g.sz + (long long)y * g.sy;
                if (x >= R && x + 3 < g.nx - R) {
                    *reinterpret_cast<float4 *>(drow + x) =
                        make_float4(out[0], out[1], out[2], out[3]);
                } else {
#pragma unroll
                    for (int e = 0; e < 4; ++e)
                        if (in_range(x + e, g.nx, R)) drow[x + e] = out[e];
                }
            }
            // Every thread has finished reading plane z-R: its slot may be refilled.
            if (!__syncthreads_and(ok)) return;
            if (tid == 0) {
                const int p = (z - z0) + S::NS;  // next plane of this item
                if (p < np) {
                    const uint32_t q = qbase + p;
                    const int s = q % S::NS;
                    mbar_arrive_expect_tx(&full[s], S::PLANE_BYTES);
                    tma_load_3d(ring + s * (S::SLOT_BYTES / 4), &src_map, &full[s],
                                x0 - S::RA, y0 - R, z0 - R + p);
                }
            }
        }
        // Consume the completions of planes loaded but not waited on (the last
        // 2R planes are waited inside the loop; nothing else is outstanding).
        qbase += np;
    }
}

namespace {

struct StreamKernel {
    const void *fn;
    int tx, ty, threads, smem;
};

template <int R, int TX, int TY>
StreamKernel sk() {
    using S = StreamShape<R, TX, TY>;
    return {reinterpret_cast<const void *>(k_stream3d<R, TX, TY>), TX, TY, S::THREADS,
            S::SMEM_BYTES};
}

StreamKernel pick(int r, int tile_x, int tile_y) {
    const bool wide = tile_x >= 128;
    const bool tall = tile_y >= 16;
    switch (r) {
        case 1: return wide ? (tall ? sk<1, 128, 16>() : sk<1, 128, 8>()) : (tall ? sk<1, 64, 16>() : sk<1, 64, 8>());
        case 2: return wide ? (tall ? sk<2, 128, 16>() : sk<2, 128, 8>()) : (tall ? sk<2, 64, 16>() : sk<2, 64, 8>());
        case 3: return wide ? sk<3, 128, 8>() : sk<3, 64, 8>();
        case 4: return wide ? (tall ? sk<4, 128, 16>() : sk<4, 128, 8>()) : (tall ? sk<4, 64, 16>() : sk<4, 64, 8>());
        default: return {nullptr, 0, 0, 0, 0};
    }
}

}  // namespace

bool stream3d_supported(const Geom &g) {
    return g.nx % 4 == 0 && (g.radius >= 1 && g.radius <= 4);
}

int run_stream3d(const Geom &g, float *a, float *b, int iters, int tile_x, int tile_y,
                 cudaStream_t s, float **res) {
    const int R = g.radius;
    StreamKernel k = pick(R, tile_x ? tile_x : 128, tile_y ? tile_y : 16);
    if (!k.fn) return fail(STENCIL_EUNSUPPORTED, "stream kernel has no radius-%d instance", R);
    if (g.nx % 4) return fail(STENCIL_EUNSUPPORTED, "stream kernel needs nx %% 4 == 0");
    ST_CUDA(cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, k.smem));
    int per_sm = 0;
    ST_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k.fn, k.threads, k.smem));
    if (per_sm < 1) return fail(STENCIL_EUNSUPPORTED, "stream kernel does not fit on an SM");
    const int resident = per_sm * num_sms();
    const int tiles_x = (g.nx + k.tx - 1) / k.tx, tiles_y = (g.ny + k.ty - 1) / k.ty;
    const int tiles = tiles_x * tiles_y;
    const int zin = g.nz - 2 * R;
    // About four waves of items so the tail is short, chunks of >= 8 planes.
    int nchunks = std::max(1, (4 * resident + tiles - 1) / tiles);
    int zchunk = std::max(8, (zin + nchunks - 1) / nchunks);
    zchunk = std::min(zchunk, zin);
    nchunks = (zin + zchunk - 1) / zchunk;
    const int items = tiles * nchunks;
    const int grid = std::min(items, resident);

    CUtensorMap maps[2];
    const long long dims[3] = {g.nx, g.ny, g.nz};
    const int box[3] = {k.tx + 2 * ((R + 3) & ~3), k.ty + 2 * R, 1};
    int rc = make_tensor_map(&maps[0], a, 3, dims, box);
    if (!rc) rc = make_tensor_map(&maps[1], b, 3, dims, box);
    if (rc) return rc;
    float *cur = a, *nxt = b;
    int ci = 0;
    dim3 block(k.tx / 4, k.ty);
    for (int it = 0; it < iters; ++it) {
        void *args[] = {&maps[ci], &nxt, const_cast<Geom *>(&g), const_cast<int *>(&tiles_x),
                        const_cast<int *>(&tiles_y), &zchunk, const_cast<int *>(&items)};
        ST_CUDA(cudaLaunchKernel(k.fn, dim3(grid), block, args, k.smem, s));
        std::swap(cur, nxt);
        ci ^= 1;
    }
    if (res) *res = cur;
    return STENCIL_OK;
}

}  // namespace st

// k_stream.cu -- 2.5D streaming sweep for 3-D grids ("smem_register" role,
// src/stencil_kernel_smem_register.cu:8-62; it is also the single-sweep engine
// behind the other 3-D variants).
//
// A CTA owns an x-y tile of TX x TY cells and a chunk of z-planes and marches
// along z.  Warp-specialised:
//   * one producer warp (one elected lane) streams plane tiles including their
//     halo -- (TX + 2*RA) x (TY + 2*R) cells, RA = R rounded up to 4 so every
//     TMA x coordinate is 16-byte aligned -- into a ring of NS shared-memory
//     slots with cp.async.bulk.tensor.3d, completion on a per-slot "full"
//     mbarrier, and refills a slot once every consumer warp has arrived on its
//     "empty" mbarrier;
//   * consumer warps compute.  A consumer thread owns 4 consecutive cells of RY
//     rows.  The z-neighbours of its cells live in a register queue of 2R+1
//     planes (each plane's own cells are read from shared memory once, when
//     the plane arrives; the z loop is unrolled 2R+1 times so the queue
//     rotates without register moves); x- and y-neighbours come from the centre plane's
//     slot with 16-byte shared loads.  So a slot is needed only while its
//     plane is the newest or the centre: the ring holds R+1 planes plus the
//     planes in flight.
// Out-of-grid box cells arrive as NaN (TMA out-of-bounds fill) and are never
// used by an updated cell.  Each input cell is read from HBM once per sweep;
// halos of neighbouring tiles and chunks are re-read from L2.
//
// Work items are (tile, z-chunk) pairs, chunk-major so that co-resident CTAs
// work on neighbouring tiles of one z range.  CTAs loop over items; the
// producer and the consumers walk the same item sequence, and a monotone plane
// sequence number fixes each plane's slot and mbarrier phase.  No CTA-wide
// barrier is used after set-up, and every mbarrier wait is bounded.
#include <algorithm>
#include <atomic>
#include <mutex>
#include <vector>
#include <cmath>

#include "host.hpp"
#include "stream_body.cuh"

namespace st {

// MULTI: one cooperative launch runs `sweeps` sweeps, ping-ponging between
// (map0 -> dst0) and (map1 -> dst1), with a grid-wide barrier on *grid_bar
// between sweeps; otherwise one sweep map0 -> dst0.
// XS: the x-neighbour chunks come from the neighbouring lanes' centre chunks
// by warp shuffles (only the lanes at the tile's x edges read the halo chunk
// from shared memory) instead of two 16-byte shared loads per row.
template <int R, int TX, int TY, int RY, int NS, bool MULTI, bool XS = false>
__global__ void __launch_bounds__(StreamShape<R, TX, TY, RY, NS>::THREADS, StreamShape<R, TX, TY, RY, NS>::MIN_BLOCKS)
    k_stream3d(const __grid_constant__ CUtensorMap map0, const __grid_constant__ CUtensorMap map1,
               float *dst0, float *dst1, Geom g, int tiles_x, int tiles_y, int zchunk, int items,
               int sweeps, unsigned *grid_bar) {
    using S = StreamShape<R, TX, TY, RY, NS>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float *ring = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) &
                                            ~static_cast<uintptr_t>(127));
    uint64_t *full = reinterpret_cast<uint64_t *>(ring + NS * S::SLOT_FLOATS);
    uint64_t *empty = full + NS;
    uint64_t *swept = empty + NS;  // MULTI, R = 1: every consumer warp has stored its part of a sweep
    if (threadIdx.x == 0) {
        prefetch_tensormap(&map0);
        if (MULTI) prefetch_tensormap(&map1);
        for (int s = 0; s < NS; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], S::CWARPS);
        }
        mbar_init(swept, S::CWARPS);
        fence_mbar_init();
    }
    __syncthreads();
    stream3d_sweeps<R, TX, TY, RY, NS, MULTI, XS>(ring, full, empty, swept, &map0, &map1, dst0, dst1,
                                                  g, tiles_x, tiles_y, zchunk, items, sweeps,
                                                  grid_bar, 0u, blockIdx.x, gridDim.x, false);
}

namespace {

struct StreamKernel {
    const void *fn;     // one sweep per launch
    const void *multi;  // persistent: all sweeps in one cooperative launch (default shapes only)
    int tx, ty, threads, smem;
};

template <int R, int TX, int TY, int RY, int NS, bool WITH_MULTI = false, bool XS = false>
StreamKernel sk() {
    using S = StreamShape<R, TX, TY, RY, NS>;
    const void *multi = nullptr;
    if constexpr (WITH_MULTI) multi = reinterpret_cast<const void *>(k_stream3d<R, TX, TY, RY, NS, true, XS>);
    return {reinterpret_cast<const void *>(k_stream3d<R, TX, TY, RY, NS, false, XS>), multi, TX, TY,
            S::THREADS, S::SMEM_BYTES};
}

// shape: 0 = 128 x 16, 2 rows per thread; 1 = tall (64 x 32); 2 = one row
// per thread (more warps, fewer registers each); 3 = a 16-slot ring (more
// planes in flight, one CTA per SM); 4 (R >= 3) = 128 x 16, one row per
// thread, 16 consumer warps in one CTA; 5 (R <= 2) = 128 x 32, two rows per
// thread (half the y-halo rows per output row).  The persistent form exists
// for the shape it uses (R = 1: 3, R = 2: 5, R >= 3: 4).
StreamKernel pick(int r, int shape) {
    // shape 6: the persistent-form shape of the radius with x neighbours by
    // warp shuffles (A/B against the shared-memory reads)
    if (shape == 6) {
        switch (r) {
            case 1: return sk<1, 128, 16, 1, 16, false, true>();
            case 2: return sk<2, 128, 32, 2, 8, true, true>();
            case 3: return sk<3, 128, 16, 1, 8, false, true>();
            case 4: return sk<4, 128, 16, 1, 8, false, true>();
            default: return {nullptr, nullptr, 0, 0, 0, 0};
        }
    }
    switch (r) {
        case 1: return shape == 5 ? sk<1, 128, 32, 2, 8>() : shape == 3 ? sk<1, 128, 16, 1, 16, true>() : shape == 2 ? sk<1, 128, 16, 1, 8>() : shape == 1 ? sk<1, 64, 32, 2, 8>() : sk<1, 128, 16, 2, 8>();
        case 2: return shape == 5 ? sk<2, 128, 32, 2, 8, true>() : shape == 3 ? sk<2, 128, 16, 1, 16>() : shape == 2 ? sk<2, 128, 16, 1, 8>() : shape == 1 ? sk<2, 64, 32, 2, 8>() : sk<2, 128, 16, 2, 8>();
        case 3: return shape == 4 ? sk<3, 128, 16, 1, 8, true>() : shape == 2 ? sk<3, 128, 8, 1, 8>() : shape == 1 ? sk<3, 64, 32, 2, 8>() : sk<3, 128, 16, 2, 8>();
        case 4: return shape == 4 ? sk<4, 128, 16, 1, 8, true>() : shape == 3 ? sk<4, 128, 16, 2, 16>() : shape == 2 ? sk<4, 128, 8, 1, 8>() : shape == 1 ? sk<4, 64, 32, 2, 8>() : sk<4, 128, 16, 2, 8>();
        default: return {nullptr, nullptr, 0, 0, 0, 0};
    }
}

}  // namespace

// Grid-barrier counters of the persistent launches: a fixed device array (no
// allocation, so a launch can be captured in a CUDA graph), one slot per
// launch taken round-robin and zeroed on the launch's stream just before it.
constexpr int kGridBarSlots = 256;
__device__ unsigned g_grid_bar[kGridBarSlots];

int grid_bar_slot(cudaStream_t s, unsigned **slot) {
    static std::atomic<unsigned> next{0};
    unsigned *base = nullptr;
    ST_CUDA(cudaGetSymbolAddress(reinterpret_cast<void **>(&base), g_grid_bar));
    *slot = base + (next.fetch_add(1) % kGridBarSlots);
    ST_CUDA(cudaMemsetAsync(*slot, 0, sizeof(unsigned), s));
    return STENCIL_OK;
}

namespace {

// Sets the kernel's shared-memory limit and returns its resident CTAs per SM,
// once per kernel and device (later calls, e.g. inside a CUDA graph capture,
// only read the cache).
int kernel_residency(const void *fn, int threads, int smem, int *per_sm) {
    static std::mutex mu;
    static std::vector<std::pair<std::pair<const void *, int>, int>> cache;
    int dev = 0;
    ST_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    for (auto &c : cache)
        if (c.first.first == fn && c.first.second == dev) { *per_sm = c.second; return STENCIL_OK; }
    ST_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    int n = 0;
    ST_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, threads, smem));
    cache.push_back({{fn, dev}, n});
    *per_sm = n;
    return STENCIL_OK;
}

}  // namespace

bool stream3d_supported(const Geom &g) {
    return g.sy % 4 == 0 && (g.radius >= 1 && g.radius <= 4);
}

namespace {

// The shape run_stream3d sweeps with (see there).
int stream_shape(const Geom &g, int tile_x, int tile_y, int shape_hint, bool persistent) {
    const int R = g.radius;
    // Defaults measured fastest at 512^3 on GB300 (a launch per sweep,
    // GCell/s): R <= 2 one row per thread with the 16-slot ring (R = 1: 701
    // vs 634 with 8 slots and 613 with two rows per thread; R = 2: 692 vs
    // 674 with 8 slots, 616 with 128 x 32 tiles and 581 with two rows), R >= 3
    // one row per thread in 16 warps (R = 3: 574 vs 533 with two rows per
    // thread; R = 4: 542 vs 531 with 8 warps and 491 with two rows).  In the
    // persistent form R = 2 uses 128 x 32 tiles: 709 GCell/s at 512^3 with
    // either shape, and neither wins across 96^3 to 384^3 (within 10 %
    // either way).
    int shape = (!tile_x && !tile_y) ? (R <= 2 ? 3 : 4)
                                     : (tile_y == 1 ? 2 : ((tile_x && tile_x < 128) || tile_y > 16 ? 1 : 0));
    if (shape_hint >= 1 && shape_hint <= 6) shape = shape_hint;
    // Persistent default per radius; at R = 2 on large grids (2^25 cells and
    // up) the same shape with x neighbours by warp shuffles (GB300, same box:
    // 512^3 694 vs 631 GCell/s, 384^3 653 vs 636; on 256^3 and smaller the
    // shared-memory reads win: 525 vs 605 at 256^3, 258 vs 301 at 128^3).
    const bool big = (long long)g.nx * g.ny * g.nz >= (1LL << 25);
    if (persistent && !(shape_hint >= 1 && shape_hint <= 6))
        shape = R == 1 ? 3 : (R == 2 ? (big ? 6 : 5) : 4);
    return shape;
}

}  // namespace

// Work items of a stream sweep of g with TX x TY tiles on `resident` CTAs:
// (tile, z-chunk) pairs taken chunk-major, so CTAs running at the same time
// work on neighbouring tiles of one z range and their halo re-reads hit L2.
// The chunk count is chosen so the items fill whole waves of resident CTAs (a
// partly filled last wave idles SMs) while chunks stay long (each re-reads 2R
// halo planes and re-primes the queue).  Chunks may be as short as 2 planes:
// on small grids a long chunk is a long chain of dependent plane steps on few
// CTAs (96^3 R=2: 11 us per sweep with 9-plane chunks on 33 CTAs).
void stream3d_plan(const Geom &g, int tx, int ty, int resident, int *tiles_x, int *tiles_y,
                   int *zchunk, int *items) {
    const int R = g.radius;
    *tiles_x = (g.nx + tx - 1) / tx;
    *tiles_y = (g.ny + ty - 1) / ty;
    const int tiles = *tiles_x * *tiles_y;
    const int zin = g.nz - 2 * R;
    resident = std::max(1, resident);
    int nchunks = 1;
    double best = 1e30;
    for (int n = 1; n <= std::max(1, zin / 2); ++n) {
        const int zc = (zin + n - 1) / n;
        const long long it = (long long)tiles * ((zin + zc - 1) / zc);
        const double waves = std::ceil((double)it / resident);
        const double fill = (double)it / (waves * resident);  // <= 1
        const double halo = 1.0 + 0.25 * (2.0 * R) / zc;      // halo planes mostly hit L2
        const double cost = halo / fill + 0.002 * waves;       // small per-item overhead
        if (cost < best - 1e-9) { best = cost; nchunks = n; }
    }
    *zchunk = (zin + nchunks - 1) / nchunks;
    nchunks = (zin + *zchunk - 1) / *zchunk;
    *items = tiles * nchunks;
}

int stream3d_capacity(const Geom &g, int *ctas) {
    *ctas = 0;
    StreamKernel k = pick(g.radius, stream_shape(g, 0, 0, 0, true));
    if (!k.multi) return fail(STENCIL_EUNSUPPORTED, "no persistent stream kernel for radius %d", g.radius);
    int per_sm = 0;
    int rc = kernel_residency(k.multi, k.threads, k.smem, &per_sm);
    if (rc) return rc;
    *ctas = per_sm * num_sms();
    return STENCIL_OK;
}

int run_stream3d(const Geom &g, float *a, float *b, int iters, int tile_x, int tile_y,
                 cudaStream_t s, float **res, int shape_hint, bool persistent, int max_ctas) {
    const int R = g.radius;
    const int shape = stream_shape(g, tile_x, tile_y, shape_hint, persistent);
    StreamKernel k = pick(R, shape);
    if (!k.fn) return fail(STENCIL_EUNSUPPORTED, "stream kernel has no radius-%d instance", R);
    if (persistent && !k.multi)
        return fail(STENCIL_EUNSUPPORTED, "the persistent stream kernel exists for the default shapes only");
    if (g.sy % 4) return fail(STENCIL_EUNSUPPORTED, "stream kernel needs a row pitch %% 4 == 0");
    const void *fn = persistent ? k.multi : k.fn;
    int per_sm = 0;
    int rc = kernel_residency(fn, k.threads, k.smem, &per_sm);
    if (rc) return rc;
    if (per_sm < 1) return fail(STENCIL_EUNSUPPORTED, "stream kernel does not fit on an SM");
    // at most max_ctas CTAs when given (a batch runs two mid-size grids side by
    // side, each on part of the GPU)
    const int resident = max_ctas > 0 ? std::min(per_sm * num_sms(), max_ctas) : per_sm * num_sms();
    int tiles_x = 0, tiles_y = 0, zchunk = 0, items = 0;
    stream3d_plan(g, k.tx, k.ty, resident, &tiles_x, &tiles_y, &zchunk, &items);
    const int grid = std::min(items, resident);

    CUtensorMap maps[2];
    const long long dims[3] = {g.nx, g.ny, g.nz};
    const int box[3] = {k.tx + 2 * ((R + 3) & ~3), k.ty + 2 * R, 1};
    // Box cells outside the grid arrive as NaN: no stored cell reads them,
    // and the epilogue's range test (fminf / fmaxf) ignores the NaN sums of
    // the unstored cells past the last column of a width that is not a
    // multiple of 4 -- zero sums there sent whole warps to the slow division
    // (160^2 x 161 R = 2: 25.0 us per sweep against 10.8 at 160^3).
    rc = make_tensor_map(&maps[0], a, 3, dims, box, g.sy, true);
    if (!rc) rc = make_tensor_map(&maps[1], b, 3, dims, box, g.sy, true);
    if (rc) return rc;
    Geom gg = g;
    int tx_ = tiles_x, ty_ = tiles_y, it_ = items;
    if (persistent) {
        // One cooperative launch (every CTA resident, as the grid barrier
        // needs): sweep k reads maps[k & 1] and writes the other buffer.
        if (iters > 0) {
            unsigned *bar = nullptr;
            rc = grid_bar_slot(s, &bar);
            if (rc) return rc;
            float *d0 = b, *d1 = a;
            int sw = iters;
            void *args[] = {&maps[0], &maps[1], &d0, &d1, &gg, &tx_, &ty_, &zchunk, &it_, &sw, &bar};
            ST_CUDA(cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(k.threads), args, k.smem, s));
            note_launches("stream3d-persistent", 1);
        }
        if (res) *res = (iters & 1) ? b : a;
        return STENCIL_OK;
    }
    note_launches("stream3d", iters);
    float *cur = a, *nxt = b;
    int ci = 0;
    int one = 1;
    unsigned *no_bar = nullptr;
    for (int it = 0; it < iters; ++it) {
        void *args[] = {&maps[ci], &maps[ci], &nxt, &nxt, &gg, &tx_, &ty_, &zchunk, &it_, &one, &no_bar};
        ST_CUDA(cudaLaunchKernel(fn, dim3(grid), dim3(k.threads), args, k.smem, s));
        std::swap(cur, nxt);
        ci ^= 1;
    }
    if (res) *res = cur;
    return STENCIL_OK;
}

}  // namespace st

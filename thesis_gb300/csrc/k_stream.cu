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

namespace st {

template <int R, int TX, int TY, int RY, int NS>
struct StreamShape {
    static constexpr int RA = (R + 3) & ~3;
    static constexpr int PW = TX + 2 * RA;  // plane tile width (cells)
    static constexpr int PH = TY + 2 * R;   // plane tile height (rows)
    static constexpr int PLANE_BYTES = PW * PH * 4;
    static constexpr int SLOT_FLOATS = ((PLANE_BYTES + 127) & ~127) / 4;
    static constexpr int CW = TX / 4;       // consumer threads along x
    static constexpr int CONSUMERS = CW * (TY / RY);
    static constexpr int CWARPS = CONSUMERS / 32;
    static constexpr int THREADS = CONSUMERS + 32;
    static constexpr int SMEM_BYTES = NS * SLOT_FLOATS * 4 + 128 + (2 * NS + 1) * 8;
    // Two resident CTAs where the registers allow: the 8-slot R = 1 shapes
    // of 9 warps, or of 17 one-row warps (56 registers), and the
    // one-row-per-thread 9-warp shapes at larger radii (their budget, 96 to
    // 112 registers, holds the 2R+1-plane queue of one row).
    static constexpr int MIN_BLOCKS =
        ((R <= 1 && NS <= 8 && (THREADS <= 320 || RY == 1)) || (RY == 1 && THREADS <= 320)) ? 2 : 1;
    static_assert(PW <= 256 && PH <= 256, "TMA box dimensions are limited to 256");
    static_assert(TX % 4 == 0 && TY % RY == 0 && CONSUMERS % 32 == 0, "bad tile");
    static_assert((NS & (NS - 1)) == 0 && NS >= R + 2, "ring must be a power of two > R+1");
};

__device__ __forceinline__ float4 lds4(const float *p) { return *reinterpret_cast<const float4 *>(p); }

// Sums of two cells at a time: packed f32x2 instructions where the kernel is
// issue-bound (R >= 3: 467 vs 412 GCell/s at 512^3, R = 4), scalar ones where
// it is bandwidth-bound (R = 1: 691 scalar vs 627 packed) -- the same
// roundings either way.
template <bool PK>
__device__ __forceinline__ float2 add_pair(float2 a, float2 b) {
    if constexpr (PK) return fadd2(a, b);
    else return make_float2(a.x + b.x, a.y + b.y);
}
template <bool PK, int C>
__device__ __forceinline__ float2 div_pair(float2 a) {
    if constexpr (PK) return div_fast2<C>(a);
    else return make_float2(div_fast<C>(a.x), div_fast<C>(a.y));
}

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
    constexpr int C = 6 * R;  // 2*D*R with D = 3
    constexpr bool PK = R >= 3;
    // How a consumer warp leaves after a bounded wait gave up: R = 1 returns
    // at once; R >= 2 clears `ok` and leaves its loops, and the warps agree at
    // a named barrier.  Same behaviour, but the code generated for each form
    // differs in speed (same-box A/B at 512^3: R = 1 713 vs 628 GCell/s with
    // early returns; R = 4 541 vs 467 with the flag).
    constexpr bool FLAG_EXIT = R >= 2;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float *ring = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) &
                                            ~static_cast<uintptr_t>(127));
    uint64_t *full = reinterpret_cast<uint64_t *>(ring + NS * S::SLOT_FLOATS);
    uint64_t *empty = full + NS;
    uint64_t *swept = empty + NS;  // MULTI, R = 1: every consumer warp has stored its part of a sweep
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (!MULTI) sweeps = 1;
    if (tid == 0) {
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
    const int ntiles = tiles_x * tiles_y;

    if (warp == S::CWARPS) {
        // ---------------- producer ----------------
        if (lane != 0) return;
        uint32_t q = 0;
        for (int sw = 0; sw < sweeps; ++sw) {
            // Sweep sw reads what every CTA wrote in sweep sw-1.
            if (MULTI && sw > 0 && !grid_wait_bounded(grid_bar, (unsigned)sw * gridDim.x)) return;
            const CUtensorMap *src_map = (sw & 1) ? &map1 : &map0;
            for (int item = blockIdx.x; item < items; item += gridDim.x) {
                const int t = item % ntiles, ch = item / ntiles;
                const int x0 = (t % tiles_x) * TX, y0 = (t / tiles_x) * TY;
                const int z0 = R + ch * zchunk, z1 = min(z0 + zchunk, g.nz - R);
                const int np = (z1 - z0) + 2 * R;
                for (int p = 0; p < np; ++p, ++q) {
                    const int s = q & (NS - 1);
                    const uint32_t use = q / NS;
                    if (use > 0 && !mbar_wait_bounded(&empty[s], (use - 1) & 1)) return;
                    fence_proxy_async();  // the consumers' reads of the slot before the TMA write
                    mbar_arrive_expect_tx(&full[s], S::PLANE_BYTES);
                    tma_load_3d(ring + s * S::SLOT_FLOATS, src_map, &full[s], x0 - S::RA, y0 - R,
                                z0 - R + p);
                }
            }
        }
        return;
    }

    // ---------------- consumers ----------------
    const int cx = tid % S::CW, cy = tid / S::CW;
    // R = 1: the sweep's output marked evict-first in L2 (+1.5 % at 512^3;
    // at R >= 2 it costs registers and measured 1.5-2 % slower)
    const uint64_t wpol = R == 1 ? l2_evict_first_policy() : 0;
    auto release = [&](int s) {
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);
    };
    constexpr int QN = 2 * R + 1;
    float4 qz[RY][QN];  // z register queue, rotated by unrolling: plane z+k-R sits at index (z-z0+k) % QN
    uint32_t qb = 0;    // sequence number of plane 0 of the current item
    bool ok = true;     // false once a bounded wait gave up
    for (int sw = 0; sw < sweeps && ok; ++sw) {
    float *dst = (sw & 1) ? dst1 : dst0;
    for (int item = blockIdx.x; item < items && ok; item += gridDim.x) {
        const int t = item % ntiles, ch = item / ntiles;
        const int x0 = (t % tiles_x) * TX, y0 = (t / tiles_x) * TY;
        const int z0 = R + ch * zchunk, z1 = min(z0 + zchunk, g.nz - R);
        const int np = (z1 - z0) + 2 * R;
        const int x = x0 + 4 * cx, ybase = y0 + cy * RY;
        const int own = (cy * RY + R) * S::PW + 4 * cx + S::RA;  // slot offset of row 0, cell 0
        // Which of this thread's rows are stored, and whether its 4 cells are
        // all inside the update region along x (16-byte store) or not.
        unsigned live = 0;
#pragma unroll
        for (int r = 0; r < RY; ++r)
            if (x < g.nx && in_range(ybase + r, g.ny, R)) live |= 1u << r;
        const bool xin = x >= R && x + 3 < g.nx - R;
        // Prime the queue with planes z0-R .. z0+R-1 (queue indices 0 .. 2R-1).
#pragma unroll
        for (int p = 0; p < 2 * R; ++p) {
            const uint32_t q = qb + p;
            const int s = q & (NS - 1);
            if (!mbar_wait_bounded(&full[s], (q / NS) & 1)) {
                if constexpr (FLAG_EXIT) { ok = false; break; } else { return; }
            }
            const float *sl = ring + s * S::SLOT_FLOATS + own;
#pragma unroll
            for (int r = 0; r < RY; ++r) qz[r][p] = lds4(sl + r * S::PW);
            if (p < R || p >= np - R) release(s);
        }
        if (!ok) break;
        float *drow = dst + (long long)z0 * g.sz + (long long)ybase * g.sy + x;
        const float *ring_own = ring + own;
        for (int zb = z0; zb < z1 && ok; zb += QN) {
#pragma unroll
            for (int ph = 0; ph < QN; ++ph) {
                const int z = zb + ph;
                if (z >= z1) break;
                const int step = z - z0;
                // Centre plane z (already waited on as the newest, R steps ago).
                const int sc = (qb + step + R) & (NS - 1);
                const float *cb = ring_own + sc * S::SLOT_FLOATS;
                // The thread's 4 columns, rows -R .. RY-1+R.  At R >= 2 its own
                // rows are taken from the centre plane's entries of the z
                // queue (the same words of the same slot), so only the 2R halo
                // rows are loaded (512^3: R = 2 +2 %, R = 3 +5 %, R = 4 +3 %,
                // 96^3-300^3 R = 2 +7-9 %; R = 1 measured 1-4 % slower).
                float4 col[RY + 2 * R];
#pragma unroll
                for (int k = 0; k < RY + 2 * R; ++k)
                    col[k] = (R >= 2 && k >= R && k < R + RY) ? qz[k - R][(ph + R) % QN] : lds4(cb + (k - R) * S::PW);
                // Sums of cells (0, 1) and (2, 3) of each row as pairs (add_pair),
                // started from the first term (div_slow_from_first).
                float2 acc[RY][2];
#pragma unroll
                for (int r = 0; r < RY; ++r) {
                    float w[4 + 2 * S::RA];
                    if constexpr (XS) {
                        static_assert(S::RA == 4 && (S::CW == 16 || S::CW == 32), "shuffle form: R <= 4, 16 or 32 lanes per row");
                        const float4 cc = col[r + R];
                        float4 a, b;
                        a.x = __shfl_up_sync(0xffffffffu, cc.x, 1, S::CW);
                        a.y = __shfl_up_sync(0xffffffffu, cc.y, 1, S::CW);
                        a.z = __shfl_up_sync(0xffffffffu, cc.z, 1, S::CW);
                        a.w = __shfl_up_sync(0xffffffffu, cc.w, 1, S::CW);
                        b.x = __shfl_down_sync(0xffffffffu, cc.x, 1, S::CW);
                        b.y = __shfl_down_sync(0xffffffffu, cc.y, 1, S::CW);
                        b.z = __shfl_down_sync(0xffffffffu, cc.z, 1, S::CW);
                        b.w = __shfl_down_sync(0xffffffffu, cc.w, 1, S::CW);
                        if (cx == 0) a = lds4(cb + r * S::PW - 4);
                        if (cx == S::CW - 1) b = lds4(cb + r * S::PW + 4);
                        w[0] = a.x; w[1] = a.y; w[2] = a.z; w[3] = a.w;
                        w[8] = b.x; w[9] = b.y; w[10] = b.z; w[11] = b.w;
                    } else {
#pragma unroll
                        for (int h = 0; h < S::RA / 4; ++h) {
                            const float4 a = lds4(cb + r * S::PW - S::RA + 4 * h);
                            const float4 b = lds4(cb + r * S::PW + 4 + 4 * h);
                            w[4 * h] = a.x; w[4 * h + 1] = a.y; w[4 * h + 2] = a.z; w[4 * h + 3] = a.w;
                            w[S::RA + 4 + 4 * h] = b.x; w[S::RA + 5 + 4 * h] = b.y;
                            w[S::RA + 6 + 4 * h] = b.z; w[S::RA + 7 + 4 * h] = b.w;
                        }
                    }
                    const float4 c = col[r + R];
                    w[S::RA] = c.x; w[S::RA + 1] = c.y; w[S::RA + 2] = c.z; w[S::RA + 3] = c.w;
                    // axis i: an even offset reads aligned pairs of the
                    // loaded vectors (pair adds), an odd one straddles them
                    // (scalar adds)
                    acc[r][0] = make_float2(w[S::RA - R], w[S::RA - R + 1]);
                    acc[r][1] = make_float2(w[S::RA - R + 2], w[S::RA - R + 3]);
#pragma unroll
                    for (int o = -R + 1; o <= R; ++o) {
                        if (o == 0) continue;
                        const int off = S::RA + o;
                        if ((off & 1) == 0) {
                            acc[r][0] = add_pair<PK>(acc[r][0], make_float2(w[off], w[off + 1]));
                            acc[r][1] = add_pair<PK>(acc[r][1], make_float2(w[off + 2], w[off + 3]));
                        } else {
                            acc[r][0].x += w[off]; acc[r][0].y += w[off + 1];
                            acc[r][1].x += w[off + 2]; acc[r][1].y += w[off + 3];
                        }
                    }
                    // axis j
#pragma unroll
                    for (int o = -R; o <= R; ++o) {
                        if (o == 0) continue;
                        const float4 v = col[r + R + o];
                        acc[r][0] = add_pair<PK>(acc[r][0], make_float2(v.x, v.y));
                        acc[r][1] = add_pair<PK>(acc[r][1], make_float2(v.z, v.w));
                    }
                    // axis k, previous planes z-R .. z-1 (queue indices (ph + R + o) % QN)
#pragma unroll
                    for (int o = -R; o <= -1; ++o) {
                        const float4 v = qz[r][(ph + R + o + QN) % QN];
                        acc[r][0] = add_pair<PK>(acc[r][0], make_float2(v.x, v.y));
                        acc[r][1] = add_pair<PK>(acc[r][1], make_float2(v.z, v.w));
                    }
                }
                // The centre slot is no longer read by this warp.
                release(sc);
                // Newest plane z+R enters the queue at index (ph + 2R) % QN;
                // waiting for it overlaps the work above.
                {
                    const int pn = step + 2 * R;
                    const uint32_t q = qb + pn;
                    const int s = q & (NS - 1);
                    if (!mbar_wait_bounded(&full[s], (q / NS) & 1)) {
                        if constexpr (FLAG_EXIT) { ok = false; break; } else { return; }
                    }
                    const float *sl = ring_own + s * S::SLOT_FLOATS;
#pragma unroll
                    for (int r = 0; r < RY; ++r) qz[r][(ph + 2 * R) % QN] = lds4(sl + r * S::PW);
                    if (pn >= np - R) release(s);
                }
                // axis k, next planes z+1 .. z+R
#pragma unroll
                for (int r = 0; r < RY; ++r)
#pragma unroll
                    for (int o = 1; o <= R; ++o) {
                        const float4 v = qz[r][(ph + R + o) % QN];
                        acc[r][0] = add_pair<PK>(acc[r][0], make_float2(v.x, v.y));
                        acc[r][1] = add_pair<PK>(acc[r][1], make_float2(v.z, v.w));
                    }
                // Epilogue: correctly rounded division by 6R.  The fast path
                // applies when every stored sum lies in [2^-100, 2^120] (NaN
                // sums pass through it as NaN); otherwise the warp divides.
                float lo = 0x1p-100f, hi = 0x1p+120f;
#pragma unroll
                for (int r = 0; r < RY; ++r)
                    if (live & (1u << r))
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            lo = fminf(lo, fminf(fabsf(acc[r][h].x), fabsf(acc[r][h].y)));
                            hi = fmaxf(hi, fmaxf(fabsf(acc[r][h].x), fabsf(acc[r][h].y)));
                        }
                if (__all_sync(0xffffffffu, lo >= 0x1p-100f && hi <= 0x1p+120f)) {
#pragma unroll
                    for (int r = 0; r < RY; ++r)
#pragma unroll
                        for (int h = 0; h < 2; ++h) acc[r][h] = div_pair<PK, C>(acc[r][h]);
                } else {
#pragma unroll
                    for (int r = 0; r < RY; ++r)
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            acc[r][h].x = div_slow_from_first<C>(acc[r][h].x);
                            acc[r][h].y = div_slow_from_first<C>(acc[r][h].y);
                        }
                }
                if (g.legacy) {
#pragma unroll
                    for (int r = 0; r < RY; ++r) {
                        const float4 c = col[r + R];
                        acc[r][0].x -= c.x; acc[r][0].y -= c.y; acc[r][1].x -= c.z; acc[r][1].y -= c.w;
                    }
                }
                if (xin) {
#pragma unroll
                    for (int r = 0; r < RY; ++r)
                        if (live & (1u << r))
                            if constexpr (R == 1)
                                stg4_hint(drow + r * g.sy, acc[r][0].x, acc[r][0].y, acc[r][1].x,
                                          acc[r][1].y, wpol);
                            else
                                stg4(drow + r * g.sy, acc[r][0].x, acc[r][0].y, acc[r][1].x, acc[r][1].y);
                } else {
#pragma unroll
                    for (int r = 0; r < RY; ++r)
                        if (live & (1u << r)) {
                            const float v[4] = {acc[r][0].x, acc[r][0].y, acc[r][1].x, acc[r][1].y};
#pragma unroll
                            for (int e = 0; e < 4; ++e)
                                if (in_range(x + e, g.nx, R)) drow[r * g.sy + e] = v[e];
                        }
                }
                drow += g.sz;
            }
        }
        qb += np;
    }
    if (MULTI && sw + 1 < sweeps) {
        // Once every consumer warp of this CTA has stored its part of sweep
        // sw (or given up), one thread arrives at the grid barrier.
        if constexpr (FLAG_EXIT) {
            ok = named_barrier_and(1, S::CONSUMERS, ok);
        } else {
            // a warp that gave up has returned; the others give up here
            __syncwarp();
            if (lane == 0) mbar_arrive(swept);
            if (!mbar_wait_bounded(swept, sw & 1)) return;
        }
        if (ok && tid == 0) grid_arrive(grid_bar);
    }
    }
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
    const int tiles_x = (g.nx + k.tx - 1) / k.tx, tiles_y = (g.ny + k.ty - 1) / k.ty;
    const int tiles = tiles_x * tiles_y;
    const int zin = g.nz - 2 * R;
    // Items are (tile, z-chunk) pairs taken chunk-major, so CTAs running at
    // the same time work on neighbouring tiles of one z range and their halo
    // re-reads hit L2.  The chunk count is chosen so the items fill whole
    // waves of resident CTAs (a partly filled last wave idles SMs) while
    // chunks stay long (each re-reads 2R halo planes and re-primes the queue).
    // Chunks may be as short as 2 planes: on small grids a long chunk is a
    // long chain of dependent plane steps on few CTAs (96^3 R=2: 11 us per
    // sweep with 9-plane chunks on 33 CTAs).
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
    int zchunk = (zin + nchunks - 1) / nchunks;
    nchunks = (zin + zchunk - 1) / zchunk;
    const int items = tiles * nchunks;
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

// stream_body.cuh -- the per-CTA part of the 2.5D streaming sweep for 3-D
// grids (k_stream3d in k_stream.cu, "smem_register" role of
// src/stencil_kernel_smem_register.cu:8-62), shared by the kernels that run
// it: k_stream3d (one grid on the whole GPU or on part of it) and the
// one-launch batch kernel (k_batch1.cu, one grid per team of CTAs).
//
// A CTA owns an x-y tile of TX x TY cells and a chunk of z-planes and marches
// along z.  Warp-specialised: one producer warp (one elected lane) streams
// plane tiles with their halo -- (TX + 2*RA) x (TY + 2*R) cells, RA = R
// rounded up to 4 so every TMA x coordinate is 16-byte aligned -- into a ring
// of NS shared-memory slots (full/empty mbarriers); consumer threads own 4
// cells of RY rows each, keep the z-neighbours in a register queue of 2R+1
// planes and read x/y neighbours from the centre plane's slot.  Work items
// are (tile, z-chunk) pairs, chunk-major, spread over the `nctas` CTAs that
// share the grid (this CTA is number `cta` of them).
#pragma once

#include "common.cuh"

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

// fence.proxy.async for global memory: orders this thread's view of global
// data (generic-proxy writes it has synchronised with) before its later TMA
// (async-proxy) reads.
__device__ __forceinline__ void fence_proxy_async_global() {
    asm volatile("fence.proxy.async.global;" ::: "memory");
}

// The sweeps of one grid by one CTA of the `nctas` CTAs that share it; ring,
// full, empty and swept are the shared-memory ring and its mbarriers
// (initialised by the caller: full[s] count 1, empty[s] and swept count
// CWARPS).  MULTI: `sweeps` sweeps, ping-ponging between (map0 -> dst0) and
// (map1 -> dst1), with a barrier over the nctas CTAs on *grid_bar between
// sweeps (before sweep sw the counter must reach bar_base + sw * nctas);
// otherwise one sweep map0 -> dst0.  entry_fence: the producer fences the
// async proxy before its first load (the grid was written inside the same
// launch).  XS: the x-neighbour chunks come from the neighbouring lanes'
// centre chunks by warp shuffles (only the lanes at the tile's x edges read
// the halo chunk from shared memory) instead of two 16-byte shared loads per
// row.  Returns early after a bounded wait gave up (the device status word
// says so).
template <int R, int TX, int TY, int RY, int NS, bool MULTI, bool XS>
__device__ __forceinline__ void stream3d_sweeps(float *ring, uint64_t *full, uint64_t *empty,
                                                uint64_t *swept, const CUtensorMap *map0,
                                                const CUtensorMap *map1, float *dst0, float *dst1,
                                                const Geom g, int tiles_x, int tiles_y, int zchunk,
                                                int items, int sweeps, unsigned *grid_bar,
                                                unsigned bar_base, unsigned cta, unsigned nctas,
                                                bool entry_fence) {
    using S = StreamShape<R, TX, TY, RY, NS>;
    constexpr int C = 6 * R;  // 2*D*R with D = 3
    constexpr bool PK = R >= 3;
    // How a consumer warp leaves after a bounded wait gave up: R = 1 returns
    // at once; R >= 2 clears `ok` and leaves its loops, and the warps agree at
    // a named barrier.  Same behaviour, but the code generated for each form
    // differs in speed (same-box A/B at 512^3: R = 1 713 vs 628 GCell/s with
    // early returns; R = 4 541 vs 467 with the flag).
    constexpr bool FLAG_EXIT = R >= 2;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (!MULTI) sweeps = 1;
    const int ntiles = tiles_x * tiles_y;

    if (warp == S::CWARPS) {
        // ---------------- producer ----------------
        if (lane != 0) return;
        uint32_t q = 0;
        for (int sw = 0; sw < sweeps; ++sw) {
            // Sweep sw reads what every CTA wrote in sweep sw-1.
            if (MULTI && sw > 0 && !grid_wait_bounded(grid_bar, bar_base + (unsigned)sw * nctas)) return;
            if (sw == 0 && entry_fence) fence_proxy_async_global();
            const CUtensorMap *src_map = (sw & 1) ? map1 : map0;
            for (int item = cta; item < items; item += nctas) {
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
    for (int item = cta; item < items && ok; item += nctas) {
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

}  // namespace st

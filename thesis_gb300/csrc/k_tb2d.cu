// k_tb2d.cu -- small 2-D grids (the whole grid lives in L2): every sweep in
// one cooperative launch over the whole GPU ("coop" role,
// src/stencil_kernel_coop.cu:5-49, whose launch the reference left commented
// out at src/stencil_dispatch.cu:160-177), with temporal blocking.
//
// Each CTA owns one TX x TY tile of the grid and keeps its tile plus a halo
// of T*R cells per side (x halo in whole float4 chunks) in shared memory.  A
// block of T sweeps updates, at sweep k, the tile grown by (T-k)*R cells per
// side (overlapped, or "trapezoidal", tiling: the halo cells are recomputed
// by every CTA that needs them, with arithmetic identical to their owner's),
// so after T sweeps the owned tile is exact without any exchange in between.
//
// Exchange between blocks: no grid-wide barrier and no flag.  Each CTA
// publishes its owned tile to an exchange buffer as 8-byte (value, block
// number) words, written and read as single-copy-atomic 8-byte units, and
// reads the halo ring of its next block from the neighbours' tiles (the halo
// never reaches past an adjacent tile: T*R <= tile sides), spinning (bounded)
// until every word carries the block number it waits for -- one L2 round
// trip after the neighbour's store, without fences.  Exchange slots alternate
// by block parity: a CTA can only get two blocks ahead of a neighbour's read
// after reading that neighbour's next block, which comes after the read.
// Before each launch the buffer is zeroed (no stale block numbers).
//
// The caller's buffers are read at the start (the first whole, the second
// only in its border band, which no sweep writes and which LEGACY reads on
// alternate sweeps) and written at the end: the last sweep to the result
// buffer and the sweep before to the other one, as the ping-pong loop leaves
// them (a launch with two or more sweeps has at least two blocks, so every
// neighbour has finished its initial reads before those writes).  Every cell
// keeps the reference's summation order (axis i offsets -R..-1, +1..+R, then
// axis j; the sum starts from +0), so results are bit-identical to single
// sweeps.
//
// The per-sweep cost of a small grid is latency -- a few dependent
// shared-memory loads and adds plus a CTA barrier -- so spreading the grid
// over every SM and exchanging once per T sweeps is what makes it fast (one
// cluster of 16 SMs is issue-bound on the same grid).
#include <algorithm>
#include <atomic>
#include <mutex>
#include <vector>

#include "host.hpp"

namespace st {
namespace {

constexpr int kTb2Threads = 512;
constexpr int kTb2MaxItems = 4;  // float4 chunks of the extended tile per thread
constexpr int kTb2MaxT = 32;       // sweeps per exchange (and s_region entries)
constexpr int kTb2SmemMax = 160 * 1024;
constexpr int kTb2MaxTiles = 256;

struct Tb2Plan {
    int tx, ty;          // owned tile (cells); tx % 4 == 0
    int t;               // sweeps per exchange
    int hx, hy;          // halo: x in whole chunks, y = t * R
    int pw, ph;          // extended tile (pw % 4 == 0)
    int tiles_x, tiles_y;
};

__device__ __forceinline__ float4 tb2_ld4(const float *p) { return *reinterpret_cast<const float4 *>(p); }

// 8-byte exchange word: value bits (low) and block number (high).
__device__ __forceinline__ unsigned long long tb2_word(float v, unsigned blk) {
    return (unsigned long long)__float_as_uint(v) | ((unsigned long long)blk << 32);
}

// One chunk of 4 cells: the reference order sum (axis i -R..-1, +1..+R, then
// axis j) divided by C = 4R, minus the centre in LEGACY.  For C a power of
// two the sum starts from its first term and the division is fma(s, 1/C,
// +0): the reference's leading +0 only matters when every term is -0 (its
// sum is +0, this one -0), and the fma's +0 addend maps exactly that -0 to
// +0 while leaving every other value as the exact product (one rounding, as
// the reference's division).  Other C divide the reference sum exactly.
template <int R, bool LEGACY>
__device__ __forceinline__ float4 tb2_chunk(const float *c, int pw) {
    constexpr int C = 4 * R;
    constexpr bool POW2 = (C & (C - 1)) == 0;
    const float4 l4 = tb2_ld4(c - 4), m4 = tb2_ld4(c), r4 = tb2_ld4(c + 4);
    const float w[12] = {l4.x, l4.y, l4.z, l4.w, m4.x, m4.y, m4.z, m4.w, r4.x, r4.y, r4.z, r4.w};
    float acc[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) acc[e] = POW2 ? w[4 + e - R] : 0.0f + w[4 + e - R];
#pragma unroll
    for (int o = -R + 1; o <= R; ++o) {
        if (!o) continue;
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[e] += w[4 + e + o];
    }
#pragma unroll
    for (int o = -R; o <= R; ++o) {
        if (!o) continue;
        const float4 v = tb2_ld4(c + o * pw);
        acc[0] += v.x; acc[1] += v.y; acc[2] += v.z; acc[3] += v.w;
    }
    float out[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        out[e] = POW2 ? fmaf(acc[e], 1.0f / C, 0.0f) : div_coeff<C>(acc[e]);
        if (LEGACY) out[e] -= w[4 + e];
    }
    return make_float4(out[0], out[1], out[2], out[3]);
}

// NI: chunks of the extended tile per thread (1, 2 or 4: the smallest that
// covers it; every unused slot costs latency in each sweep).
template <int R, bool LEGACY, int NI>
__global__ void __launch_bounds__(kTb2Threads, 1)
    k_tb2d(float *g0, float *g1, Geom g, Tb2Plan p, int iters, unsigned long long *xch) {
    extern __shared__ __align__(16) float tb2_smem[];
    // nx: the grid's width (update region x < nx - R); px: its row pitch (a
    // multiple of 4; cells nx .. px-1 of a row are padding that no update
    // reads and no sweep writes)
    const int nx = g.nx, ny = g.ny, px = (int)g.sy, pw = p.pw;
    float *const S0 = tb2_smem, *const S1 = tb2_smem + pw * p.ph;
    const int tile = blockIdx.x, ntiles = p.tiles_x * p.tiles_y;
    const int x0 = (tile % p.tiles_x) * p.tx, y0 = (tile / p.tiles_x) * p.ty;
    const int ox = x0 - p.hx, oy = y0 - p.hy;  // grid coordinates of local (0, 0)
    const int x1 = min(x0 + p.tx, px), y1 = min(y0 + p.ty, ny);  // owned tile end
    const size_t tile_words = (size_t)p.tx * p.ty;
    // two sweeps or more: at least two blocks (see the header)
    const int T = iters >= 2 ? min(p.t, iters - 1) : 1;
    // The extended tile clipped to the grid.
    const int exa = max(ox, 0), exb = min(ox + pw, px);
    const int eya = max(oy, 0), eyb = min(oy + p.ph, ny);

    // This thread's float4 chunks of the extended tile, fixed for the launch
    // (chunk column, row, shared-memory offset; -1: none), so a sweep costs
    // no index arithmetic: only a compare with the sweep's region.
    const int nc = pw >> 2;
    int icol[NI], irow[NI], ioff[NI];
#pragma unroll
    for (int i = 0; i < NI; ++i) {
        const int u = threadIdx.x + i * kTb2Threads;
        icol[i] = irow[i] = -1;
        if (u < nc * p.ph) {
            icol[i] = u % nc;
            irow[i] = u / nc;
        }
        ioff[i] = irow[i] * pw + 4 * icol[i];
    }
    // Region of each sweep of a block in local chunk columns [x, y) and rows
    // [z, w): the owned tile grown by (kk - k) * R, inside the update region;
    // a chunk's cells outside it are computed from whatever the tile holds
    // there and never read before being recomputed; border cells are never
    // written.  Written by threads 0..kk-1 while the previous block ends.
    __shared__ int4 s_region[kTb2MaxT];
    auto plan_block = [&](int kk) {
        if (threadIdx.x < kk) {
            const int ext = (kk - 1 - threadIdx.x) * R;
            const int rxa = max(x0 - ext, R), rxb = min(x1 + ext, nx - R);
            const int rya = max(y0 - ext, R), ryb = min(y1 + ext, ny - R);
            int4 b = make_int4(0, 0, 0, 0);
            if (rxa < rxb && rya < ryb)
                b = make_int4((rxa - ox) >> 2, (rxb - ox + 3) >> 2, rya - oy, ryb - oy);
            s_region[threadIdx.x] = b;
        }
    };
    // This thread's exchange pairs, fixed for the launch (the extended tile
    // holds at most 2 * NI * kTb2Threads pairs of cells): own pairs to publish
    // (shared-memory offset, word offset in the exchange slot; -1: none) and
    // halo pairs to read (word offset in the slot, shared-memory offset).
    constexpr int NP = 2 * NI;
    int pub_s[NP], pub_w[NP], ring_w[NP], ring_s[NP];
    {
        const int ocw = (x1 - x0) >> 1, on = ocw * (y1 - y0);
        const int ecw = (exb - exa) >> 1, en = ecw * (eyb - eya);
#pragma unroll
        for (int i = 0; i < NP; ++i) {
            const int u = threadIdx.x + i * kTb2Threads;
            pub_s[i] = pub_w[i] = ring_w[i] = ring_s[i] = -1;
            if (u < on) {
                const int y = y0 + u / ocw, x = x0 + 2 * (u % ocw);
                pub_s[i] = (y - oy) * pw + (x - ox);
                pub_w[i] = (int)(tile * tile_words) + (y - y0) * p.tx + (x - x0);
            }
            if (u < en) {
                const int y = eya + u / ecw, x = exa + 2 * (u % ecw);
                if (!(x >= x0 && x < x1 && y >= y0 && y < y1)) {  // not an own cell
                    const int ocx = x / p.tx, ocy = y / p.ty;
                    ring_w[i] = (int)((ocy * p.tiles_x + ocx) * tile_words) + (y - ocy * p.ty) * p.tx +
                                (x - ocx * p.tx);
                    ring_s[i] = (y - oy) * pw + (x - ox);
                }
            }
        }
    }

    // Initial state: the first buffer's extended tile, the second buffer's
    // border band (its interior is rewritten by the first sweep before any read).
    {
        const int cw = (exb - exa) >> 2;
        const int n = cw * (eyb - eya);
        for (int u = threadIdx.x; u < n; u += kTb2Threads) {
            const int y = eya + u / cw, x = exa + 4 * (u % cw);
            const long long gi = (long long)y * px + x;
            const int si = (y - oy) * pw + (x - ox);
            *reinterpret_cast<float4 *>(S0 + si) = __ldcg(reinterpret_cast<const float4 *>(g0 + gi));
            if (y < R || y >= ny - R) {
                *reinterpret_cast<float4 *>(S1 + si) = __ldcg(reinterpret_cast<const float4 *>(g1 + gi));
            } else if (x < R || x + 3 >= nx - R) {
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (x + e < R || x + e >= nx - R) S1[si + e] = __ldcg(g1 + gi + e);
            }
        }
    }
    int kk = min(T, iters);
    plan_block(kk);
    __syncthreads();

    int cur = 0;  // shared buffer holding the newest state
    unsigned blk = 0;
    for (int done = 0; done < iters;) {
        int4 rg_next = s_region[0];
        for (int k = 1; k <= kk; ++k) {
            const float *src = cur ? S1 : S0;
            float *dst = cur ? S0 : S1;
            // this sweep's region, read before the previous sweep's barrier
            const int4 rg = rg_next;
            if (k < kk) rg_next = s_region[k];
#pragma unroll
            for (int i = 0; i < NI; ++i) {
                if (icol[i] < rg.x || icol[i] >= rg.y || irow[i] < rg.z || irow[i] >= rg.w) continue;
                const float4 v = tb2_chunk<R, LEGACY>(src + ioff[i], pw);
                float *q = dst + ioff[i];
                const int gx = ox + 4 * icol[i];
                if (gx >= R && gx + 3 < nx - R) {
                    *reinterpret_cast<float4 *>(q) = v;
                } else {
                    if (gx >= R && gx < nx - R) q[0] = v.x;
                    if (gx + 1 >= R && gx + 1 < nx - R) q[1] = v.y;
                    if (gx + 2 >= R && gx + 2 < nx - R) q[2] = v.z;
                    if (gx + 3 >= R && gx + 3 < nx - R) q[3] = v.w;
                }
            }
            __syncthreads();
            cur ^= 1;
        }
        done += kk;
        ++blk;
        if (done >= iters) break;
        const float *S = cur ? S1 : S0;
        float *Sw = cur ? S1 : S0;
        unsigned long long *slot = xch + (size_t)(blk & 1) * ntiles * tile_words;
        // Publish the owned tile (pairs of cells; tx and x0 are multiples of 4).
#pragma unroll
        for (int i = 0; i < NP; ++i) {
            if (pub_s[i] < 0) continue;
            const float2 v = *reinterpret_cast<const float2 *>(S + pub_s[i]);
            asm volatile("st.volatile.global.v2.u64 [%0], {%1, %2};" ::"l"(slot + pub_w[i]),
                         "l"(tb2_word(v.x, blk)), "l"(tb2_word(v.y, blk))
                         : "memory");
        }
        kk = min(T, iters - done);
        plan_block(kk);
        // Read the halo ring from the neighbours' tiles, waiting for block
        // blk: every pair of a thread is requested before any is checked, so
        // the common case costs one L2 round trip.
        bool ok = true;
        {
            unsigned long long a[NP], b[NP];
#pragma unroll
            for (int i = 0; i < NP; ++i) {
                a[i] = b[i] = 0;
                if (ring_w[i] >= 0)
                    asm volatile("ld.volatile.global.v2.u64 {%0, %1}, [%2];"
                                 : "=l"(a[i]), "=l"(b[i])
                                 : "l"(slot + ring_w[i])
                                 : "memory");
            }
#pragma unroll
            for (int i = 0; i < NP; ++i) {
                if (ring_w[i] < 0) continue;
                uint64_t t0 = 0;
                while (ok && ((unsigned)(a[i] >> 32) != blk || (unsigned)(b[i] >> 32) != blk)) {
                    const uint64_t t = globaltimer_ns();
                    if (!t0) t0 = t;
                    else if (t - t0 > kWaitLimitNs) {
                        report_status(kStatusTimeout);
                        ok = false;
                    }
                    asm volatile("ld.volatile.global.v2.u64 {%0, %1}, [%2];"
                                 : "=l"(a[i]), "=l"(b[i])
                                 : "l"(slot + ring_w[i])
                                 : "memory");
                }
                *reinterpret_cast<float2 *>(Sw + ring_s[i]) =
                    make_float2(__uint_as_float((unsigned)a[i]), __uint_as_float((unsigned)b[i]));
            }
        }
        if (!__syncthreads_and(ok)) return;
    }
    // Owned cells of the update region back to the caller's buffers: the last
    // sweep to the result buffer, the one before (exact on the owned tile) to
    // the other; with one sweep the other buffer already holds the input.
    {
        const int ya = max(y0, R), yb = min(y1, ny - R);
        const int cw = (x1 - x0) >> 2;
        const int n = cw * max(yb - ya, 0);
        const float *Sn = cur ? S1 : S0, *Sp = cur ? S0 : S1;
        float *Gn = (iters & 1) ? g1 : g0, *Gp = (iters & 1) ? g0 : g1;
        for (int u = threadIdx.x; u < n; u += kTb2Threads) {
            const int y = ya + u / cw, x = x0 + 4 * (u % cw);
            const int si = (y - oy) * pw + (x - ox);
            const long long gi = (long long)y * px + x;
            const float4 vn = tb2_ld4(Sn + si), vp = tb2_ld4(Sp + si);
            if (x >= R && x + 3 < nx - R) {
                __stcg(reinterpret_cast<float4 *>(Gn + gi), vn);
                if (iters >= 2) __stcg(reinterpret_cast<float4 *>(Gp + gi), vp);
            } else {
                const float an[4] = {vn.x, vn.y, vn.z, vn.w}, ap[4] = {vp.x, vp.y, vp.z, vp.w};
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (x + e >= R && x + e < nx - R) {
                        Gn[gi + e] = an[e];
                        if (iters >= 2) Gp[gi + e] = ap[e];
                    }
            }
        }
    }
}

using Tb2Fn = void (*)(float *, float *, Geom, Tb2Plan, int, unsigned long long *);

template <int R, bool LEGACY>
Tb2Fn tb2_fn_ni(int ni) {
    return ni <= 1 ? k_tb2d<R, LEGACY, 1> : ni <= 2 ? k_tb2d<R, LEGACY, 2> : k_tb2d<R, LEGACY, 4>;
}

// The kernel for radius r, mode and chunks per thread (1, 2 or 4).
Tb2Fn tb2_fn(int r, bool legacy, int ni) {
    switch (r) {
        case 1: return legacy ? tb2_fn_ni<1, true>(ni) : tb2_fn_ni<1, false>(ni);
        case 2: return legacy ? tb2_fn_ni<2, true>(ni) : tb2_fn_ni<2, false>(ni);
        case 3: return legacy ? tb2_fn_ni<3, true>(ni) : tb2_fn_ni<3, false>(ni);
        case 4: return legacy ? tb2_fn_ni<4, true>(ni) : tb2_fn_ni<4, false>(ni);
        default: return nullptr;
    }
}

// Chunks per thread a plan needs.
int plan_items(const Tb2Plan &p) {
    const int n = (p.pw / 4) * p.ph;
    return n <= kTb2Threads ? 1 : n <= 2 * kTb2Threads ? 2 : 4;
}

int roundup4(int v) { return (v + 3) & ~3; }

// Fills the geometry of a (tile, T) choice; false if it does not fit the
// engine's limits (one CTA per SM, items per thread, shared memory).
bool make_plan(const Geom &g, int t, int tx, int ty, int max_ctas, Tb2Plan *p) {
    if (t < 1 || tx < 4 || tx % 4 || ty < 1) return false;
    const int R = g.radius;
    Tb2Plan q;
    q.tx = tx;
    q.ty = ty;
    q.t = t;
    q.hx = roundup4((t - 1) * R) + 4;
    q.hy = t * R;
    q.pw = tx + 2 * q.hx;
    q.ph = ty + 2 * q.hy;
    q.tiles_x = ((int)g.sy + tx - 1) / tx;  // tiles cover the row pitch
    q.tiles_y = (g.ny + ty - 1) / ty;
    if ((long long)q.tiles_x * q.tiles_y > max_ctas) return false;
    // the halo reaches the adjacent tiles only
    if ((q.tiles_x > 1 && q.hx > tx) || (q.tiles_y > 1 && q.hy > ty)) return false;
    if ((long long)(q.pw / 4) * q.ph > (long long)kTb2MaxItems * kTb2Threads) return false;
    if (2LL * q.pw * q.ph * 4 > kTb2SmemMax) return false;
    *p = q;
    return true;
}

// Modelled time per sweep, in SM cycles, fitted to clock64 timings of the
// kernel's phases on a GB300 (64^2 to 512^2, R = 1): a block costs its
// exchange (about 1800 cycles of L2 latency, 1.35 per halo pair read and 400
// per further pair slot of a thread) and each sweep about 350 cycles of
// latency (shared-memory loads, the CTA barrier), 90 per further chunk slot
// of a thread, and the shared-memory traffic of its region (3 + 2R loads and
// one store of 16 bytes per chunk).
double plan_cost(const Geom &g, const Tb2Plan &p) {
    const int R = g.radius, ni = plan_items(p);
    const long long ring = ((long long)p.pw * p.ph - (long long)p.tx * p.ty) / 2;
    double c = 1800.0 + 1.35 * ring + 400.0 * (ni - 1);
    for (int k = 1; k <= p.t; ++k) {
        const int ext = (p.t - k) * R;
        const int chunks = (p.tx + 2 * roundup4(ext)) / 4, rows = p.ty + 2 * ext;
        c += 350.0 + 90.0 * (ni - 1) + (0.4 + 0.15 * R) * chunks * rows;
    }
    return c / p.t;
}

// The cheapest plan by the model among T <= min(iters - 1, 31) (the
// caller's T when given) and the candidate tiles (the caller's tile when
// given).
bool choose_plan(const Geom &g, int iters, int temporal, int tile_x, int tile_y, int max_ctas,
                 Tb2Plan *p) {
    struct Key {
        int nx, ny, r, tmax, temporal, tile_x, tile_y, max_ctas;
        bool operator==(const Key &o) const {
            return nx == o.nx && ny == o.ny && r == o.r && tmax == o.tmax && temporal == o.temporal &&
                   tile_x == o.tile_x && tile_y == o.tile_y && max_ctas == o.max_ctas;
        }
    };
    static std::mutex mu;
    static std::vector<std::pair<Key, std::pair<bool, Tb2Plan>>> cache;
    // two sweeps or more take at least two blocks (see the kernel)
    const int tmax = iters >= 2 ? std::min(iters - 1, 31) : 1;
    if (temporal > 0) temporal = std::min(temporal, tmax);
    const Key key = {(int)g.sy, g.ny, g.radius, tmax, temporal, tile_x, tile_y, max_ctas};
    std::lock_guard<std::mutex> lock(mu);
    for (auto &c : cache)
        if (c.first == key) {
            if (c.second.first) *p = c.second.second;
            return c.second.first;
        }
    bool found = false;
    double best = 1e30;
    Tb2Plan bestp = {};
    for (int t = 1; t <= tmax; ++t) {
        if (temporal > 0 && t != temporal) continue;
        for (int tx : {16, 24, 32, 40, 48, 64, 96, 128, 256}) {
            if (tile_x > 0 && tx != tile_x) continue;
            for (int ty : {4, 8, 12, 16, 20, 24, 32, 48, 64, 128}) {
                if (tile_y > 0 && ty != tile_y) continue;
                Tb2Plan q;
                if (!make_plan(g, t, tx, ty, max_ctas, &q)) continue;
                const double c = plan_cost(g, q);
                if (c < best - 1e-9) {
                    best = c;
                    bestp = q;
                    found = true;
                }
            }
        }
    }
    // a caller tile outside the candidate list
    if (!found && tile_x > 0 && tile_y > 0 &&
        make_plan(g, temporal > 0 ? temporal : 1, tile_x, tile_y, max_ctas, &bestp))
        found = true;
    if (cache.size() > 256) cache.clear();
    cache.push_back({key, {found, bestp}});
    if (found) *p = bestp;
    return found;
}

// Exchange buffers: per device a few slots taken round-robin (so launches on
// different streams do not share one), all grown together outside any graph
// capture and zeroed on the launch's stream just before each launch.
constexpr int kTb2XchSlots = 4;
struct XchPool {
    unsigned long long *buf[kTb2XchSlots] = {};
    size_t bytes = 0;
    unsigned next = 0;
};
std::mutex g_xch_mu;
XchPool g_xch[64];

int xch_slot(cudaStream_t s, size_t bytes, unsigned long long **out) {
    const int dev = current_device();
    if (dev < 0 || dev >= 64) return fail(STENCIL_ECUDA, "no current device");
    std::lock_guard<std::mutex> lock(g_xch_mu);
    XchPool &pool = g_xch[dev];
    if (pool.bytes < bytes) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        ST_CUDA(cudaStreamIsCapturing(s, &cs));
        if (cs != cudaStreamCaptureStatusNone)
            return fail(STENCIL_EUNSUPPORTED,
                        "2-D temporal blocking: run the dispatch once outside the graph capture "
                        "(its exchange buffer is allocated then)");
        for (auto &b : pool.buf) {
            cudaFree(b);  // waits for the device
            b = nullptr;
        }
        pool.bytes = 0;
        for (auto &b : pool.buf) ST_CUDA(cudaMalloc(reinterpret_cast<void **>(&b), bytes));
        pool.bytes = bytes;
    }
    *out = pool.buf[pool.next++ % kTb2XchSlots];
    ST_CUDA(cudaMemsetAsync(*out, 0, bytes, s));
    return STENCIL_OK;
}

// CTAs of the launch that can be resident at once (one per SM), checked once
// per radius and device with the largest shared-memory size the plans use
// (which is also set as each kernel's dynamic shared-memory limit).
int tb2_max_ctas(int r) {
    static std::mutex mu;
    static std::vector<std::pair<int, int>> cache;  // (device * 8 + r, ctas)
    const int dev = current_device();
    std::lock_guard<std::mutex> lock(mu);
    for (auto &c : cache)
        if (c.first == dev * 8 + r) return c.second;
    int n = 1 << 30;
    for (bool legacy : {false, true})
        for (int ni : {1, 2, 4}) {
            const void *fn = reinterpret_cast<const void *>(tb2_fn(r, legacy, ni));
            int m = 0;
            if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, kTb2SmemMax) !=
                    cudaSuccess ||
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&m, fn, kTb2Threads, kTb2SmemMax) !=
                    cudaSuccess) {
                cudaGetLastError();
                m = 0;
            }
            n = std::min(n, m);
        }
    const int ctas = n >= 1 ? std::min(num_sms(), kTb2MaxTiles) : 0;
    cache.push_back({dev * 8 + r, ctas});
    return ctas;
}

}  // namespace

void tb2d_release() {
    const int dev = current_device();
    if (dev < 0 || dev >= 64) return;
    std::lock_guard<std::mutex> lock(g_xch_mu);
    for (auto &b : g_xch[dev].buf) {
        cudaFree(b);
        b = nullptr;
    }
    g_xch[dev].bytes = 0;
}

bool tb2d_supported(const Geom &g, int dims) {
    if (dims != 2 || g.sy % 4 || g.radius < 1 || g.radius > 4) return false;
    const int ctas = tb2_max_ctas(g.radius);
    Tb2Plan p;
    return ctas > 0 && choose_plan(g, 1, 1, 0, 0, ctas, &p);
}

int run_tb2d(const Geom &g, float *a, float *b, int iters, int temporal, int tile_x, int tile_y,
             cudaStream_t s, float **res) {
    if (g.sy % 4 || g.radius < 1 || g.radius > 4)
        return fail(STENCIL_EUNSUPPORTED, "2-D temporal blocking needs a row pitch %% 4 == 0 and R <= 4");
    const int ctas = tb2_max_ctas(g.radius);
    Tb2Plan p;
    // a caller tile (then a caller depth) that does not fit falls back to the
    // library's choice
    if (ctas <= 0 || (!choose_plan(g, iters, temporal, tile_x, tile_y, ctas, &p) &&
                      !choose_plan(g, iters, temporal, 0, 0, ctas, &p) &&
                      !choose_plan(g, iters, 0, 0, 0, ctas, &p)))
        return fail(STENCIL_EUNSUPPORTED, "grid too large for one tile per SM");
    if (res) *res = (iters & 1) ? b : a;
    if (iters <= 0) return STENCIL_OK;
    const void *fn = reinterpret_cast<const void *>(tb2_fn(g.radius, g.legacy != 0, plan_items(p)));
    const int grid = p.tiles_x * p.tiles_y;
    const size_t smem = 2ull * p.pw * p.ph * sizeof(float);
    unsigned long long *xch = nullptr;
    int rc = xch_slot(s, 2ull * grid * p.tx * p.ty * sizeof(unsigned long long), &xch);
    if (rc) return rc;
    Geom gg = g;
    int n = iters;
    void *args[] = {&a, &b, &gg, &p, &n, &xch};
    ST_CUDA(cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(kTb2Threads), args, smem, s));
    note_launches("tb2d-persistent", 1);
    return STENCIL_OK;
}

}  // namespace st

// k_ir2d.cu -- one outer step of the mixed-precision refinement (k_ir.cu) on
// a small 2-D grid in ONE cooperative launch over every SM.
//
// The per-launch form of an outer step costs two residual passes, a copy,
// m - 1 correction-sweep launches and an update launch; on a grid that lives
// in L2 (512^2 is 1 MiB) each of them is a few microseconds of launch and
// tail latency for well under a microsecond of work.  Here a CTA owns one
// tile of the grid for the whole step and keeps, in shared memory, the tile
// grown by a halo of T*R cells of the correction e (two 16-bit buffers) and
// of the scaled residual rhs (one 16-bit buffer):
//   1. prologue: the FP32 master u on the grown tile (read through L2) gives
//      r = (M u + c) - u in FP32 -- the same arithmetic, order and rounding as
//      k_ir_resid -- on the tile grown by (T-1)*R; the CTAs meet once at a
//      bounded grid barrier to agree on max |r| (the scale s = 2^ceil(log2
//      max |r|), as k_ir_resid), and rhs = e_1 = E(r / s) (16-bit);
//   2. the remaining m - 1 correction sweeps e <- E(M e + rhs), FP32 sums in
//      the order of k_lp_sweep (axis i offsets -R..-1, +1..+R, then axis j;
//      the sum starts from its first term), T sweeps per exchange on the
//      shrinking trapezoid of the grown tile;
//   3. between blocks of T sweeps each CTA publishes its owned e cells as
//      8-byte words (two 16-bit values and a 32-bit block tag; each word is
//      single-copy atomic, a quad of 4 cells is one 16-byte pair of words
//      that both carry the tag) and reads its halo ring
//      from the <= 8 adjacent tiles, spinning (bounded) until every word
//      carries the awaited tag; tags grow monotonically across the launches
//      of a solve, so the exchange buffer is zeroed once per solve, and the
//      two exchange slots alternate with the tag's parity;
//   4. epilogue: u += s * e_m (one FMA per cell, as k_ir_update) on the owned
//      tile.  Every CTA finished reading u before the grid barrier, so no
//      CTA can overwrite a cell that another one still has to read.
// Given the same u, the step is bit-identical to the per-launch form (r, s,
// every correction sweep and the update round exactly as there), so the two
// engines of stencil_ir_solve agree bit for bit.  Traffic per step: one read
// of u, one read-modify-write of the owned tile, and 8 bytes per halo-ring
// quad of 4 cells per exchange; every correction sweep stays on chip.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "host.hpp"

namespace st {

namespace {

constexpr int kIr2Threads = 512;
constexpr int kIr2MaxT = 32;
constexpr int kIr2SmemMax = 160 * 1024;
constexpr int kIr2MaxTiles = 256;

// 16-bit storage formats: exact widening of two packed values, and rounding
// of two floats to nearest even.
template <typename E>
struct Ir2Cvt;
template <>
struct Ir2Cvt<__nv_bfloat16> {
    __device__ static float2 two(uint32_t w) {
        return make_float2(__uint_as_float(w << 16), __uint_as_float(w & 0xffff0000u));
    }
    __device__ static uint32_t pack(float a, float b) {
        __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
        return *reinterpret_cast<uint32_t *>(&h);
    }
};
template <>
struct Ir2Cvt<__half> {
    __device__ static float2 two(uint32_t w) {
        return __half22float2(*reinterpret_cast<const __half2 *>(&w));
    }
    __device__ static uint32_t pack(float a, float b) {
        __half2 h = __floats2half2_rn(a, b);
        return *reinterpret_cast<uint32_t *>(&h);
    }
};

template <typename E>
__device__ __forceinline__ void ir2_unpack8(const uint4 &q, float *f) {
    const float2 a = Ir2Cvt<E>::two(q.x), b = Ir2Cvt<E>::two(q.y), c = Ir2Cvt<E>::two(q.z),
                 d = Ir2Cvt<E>::two(q.w);
    f[0] = a.x; f[1] = a.y; f[2] = b.x; f[3] = b.y; f[4] = c.x; f[5] = c.y; f[6] = d.x; f[7] = d.y;
}

__device__ __forceinline__ uint4 ir2_lds(const uint16_t *p) { return *reinterpret_cast<const uint4 *>(p); }

// 8-byte exchange word: two 16-bit values (low) and the block tag (high).
__device__ __forceinline__ unsigned long long ir2_word(uint32_t vals, unsigned tag) {
    return (unsigned long long)vals | ((unsigned long long)tag << 32);
}

// One correction sweep of an 8-cell chunk at shared offset c (a multiple of
// 8): E(sum / C + rhs), the sum in the order of k_lp_sweep.
template <typename E, int R>
__device__ __forceinline__ uint4 ir2_chunk(const uint16_t *c, const uint16_t *rh, int pw) {
    constexpr int C = 4 * R;
    float w[24];
    ir2_unpack8<E>(ir2_lds(c - 8), w);
    ir2_unpack8<E>(ir2_lds(c), w + 8);
    ir2_unpack8<E>(ir2_lds(c + 8), w + 16);
    float acc[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) acc[e] = w[8 + e - R];
#pragma unroll
    for (int o = -R + 1; o <= R; ++o) {
        if (!o) continue;
#pragma unroll
        for (int e = 0; e < 8; ++e) acc[e] += w[8 + e + o];
    }
#pragma unroll
    for (int o = -R; o <= R; ++o) {
        if (!o) continue;
        float f[8];
        ir2_unpack8<E>(ir2_lds(c + o * pw), f);
#pragma unroll
        for (int e = 0; e < 8; ++e) acc[e] += f[e];
    }
    float rf[8];
    ir2_unpack8<E>(ir2_lds(rh), rf);
    float out[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) out[e] = div_coeff<C>(acc[e]) + rf[e];
    uint4 q;
    q.x = Ir2Cvt<E>::pack(out[0], out[1]);
    q.y = Ir2Cvt<E>::pack(out[2], out[3]);
    q.z = Ir2Cvt<E>::pack(out[4], out[5]);
    q.w = Ir2Cvt<E>::pack(out[6], out[7]);
    return q;
}

// Launch arguments of one outer step.
struct Ir2Args {
    float *u;                 // FP32 master grid (read, owned tiles updated)
    unsigned long long *xch;  // two exchange slots, zeroed once per solve
    unsigned *bar;            // grid-barrier counter, zeroed once per solve
    unsigned *max_bits;       // two max |r| words (this step's: step & 1), zeroed per solve
    float *scale;             // s of this step (diagnostics)
    unsigned bar_target;      // counter value once every CTA of this step arrived
    unsigned tag0;            // tags of this step: tag0 + 1 ..
    int step;                 // outer steps before this one in the solve
    int m;                    // correction sweeps of the step (>= 1)
};

// NI: 8-cell chunks of the grown tile per thread (1, 2 or 4).
template <typename E, int R, int NI>
__global__ void __launch_bounds__(kIr2Threads, 1) k_ir2d(Geom g, Ir2Plan p, Ir2Args a) {
    extern __shared__ __align__(16) uint16_t ir2_smem[];
    constexpr int C = 4 * R;
    const int nx = g.nx, ny = g.ny, pw = p.pw, ph = p.ph;
    uint16_t *const S0 = ir2_smem, *const S1 = ir2_smem + pw * ph, *const RH = ir2_smem + 2 * pw * ph;
    float *const W = reinterpret_cast<float *>(ir2_smem);  // prologue only: u on the grown tile (aliases S0, S1)
    const int tile = blockIdx.x, ntiles = p.tiles_x * p.tiles_y;
    const int x0 = (tile % p.tiles_x) * p.tx, y0 = (tile / p.tiles_x) * p.ty;
    const int ox = x0 - p.hx, oy = y0 - p.hy;                      // grid coordinates of local (0, 0)
    const int x1 = min(x0 + p.tx, nx), y1 = min(y0 + p.ty, ny);    // owned tile end
    const int exa = max(ox, 0), exb = min(ox + pw, nx);            // grown tile clipped to the grid
    const int eya = max(oy, 0), eyb = min(oy + ph, ny);
    const size_t quads_per_tile = (size_t)(p.tx / 4) * p.ty;
    const int T = p.t;

    // This thread's 8-cell chunks of the grown tile (column, row, offset).
    const int nc = pw >> 3;
    int icol[NI], irow[NI], ioff[NI];
#pragma unroll
    for (int i = 0; i < NI; ++i) {
        const int q = threadIdx.x + i * kIr2Threads;
        icol[i] = irow[i] = -1;
        if (q < nc * ph) {
            icol[i] = q % nc;
            irow[i] = q / nc;
        }
        ioff[i] = irow[i] * pw + 8 * icol[i];
    }
    // Region of sweep k of a block of kk sweeps: the owned tile grown by
    // (kk - k) * R, inside the update region, in local chunk columns [x, y)
    // and rows [z, w).
    __shared__ int4 s_region[kIr2MaxT];
    __shared__ float s_red[kIr2Threads / 32];
    __shared__ float s_scale;
    auto region = [&](int ext) {
        const int rxa = max(x0 - ext, R), rxb = min(x1 + ext, nx - R);
        const int rya = max(y0 - ext, R), ryb = min(y1 + ext, ny - R);
        int4 b = make_int4(0, 0, 0, 0);
        if (rxa < rxb && rya < ryb) b = make_int4((rxa - ox) >> 3, (rxb - ox + 7) >> 3, rya - oy, ryb - oy);
        return b;
    };
    auto plan_block = [&](int kk) {
        if (threadIdx.x < kk) s_region[threadIdx.x] = region((kk - 1 - threadIdx.x) * R);
    };
    // Exchange quads (4 cells, 16 bytes of two words) of this thread: own
    // quads to publish (shared offset, quad index in the slot) and halo
    // quads to read (quad index in the slot, shared offset).
    constexpr int NP = 2 * NI;
    int pub_s[NP], pub_w[NP], ring_w[NP], ring_s[NP];
    {
        const int ocw = (x1 - x0) >> 2, on = ocw * (y1 - y0);
        const int ecw = (exb - exa) >> 2, en = ecw * (eyb - eya);
#pragma unroll
        for (int i = 0; i < NP; ++i) {
            const int q = threadIdx.x + i * kIr2Threads;
            pub_s[i] = pub_w[i] = ring_w[i] = ring_s[i] = -1;
            if (q < on) {
                const int y = y0 + q / ocw, x = x0 + 4 * (q % ocw);
                pub_s[i] = (y - oy) * pw + (x - ox);
                pub_w[i] = (int)(tile * quads_per_tile) + (y - y0) * (p.tx / 4) + (x - x0) / 4;
            }
            if (q < en) {
                const int y = eya + q / ecw, x = exa + 4 * (q % ecw);
                if (!(x >= x0 && x < x1 && y >= y0 && y < y1)) {
                    const int ocx = x / p.tx, ocy = y / p.ty;
                    ring_w[i] = (int)((ocy * p.tiles_x + ocx) * quads_per_tile) +
                                (y - ocy * p.ty) * (p.tx / 4) + (x - ocx * p.tx) / 4;
                    ring_s[i] = (y - oy) * pw + (x - ox);
                }
            }
        }
    }

    // ---- 1. prologue: u on the grown tile, r, the scale, rhs = e_1 -------
    {
        const int cw = (exb - exa) >> 2;
        const int n = cw * (eyb - eya);
        for (int q = threadIdx.x; q < n; q += kIr2Threads) {
            const int y = eya + q / cw, x = exa + 4 * (q % cw);
            *reinterpret_cast<float4 *>(W + (y - oy) * pw + (x - ox)) =
                __ldcg(reinterpret_cast<const float4 *>(a.u + (long long)y * nx + x));
        }
    }
    __syncthreads();
    const int4 rq = region((T - 1) * R);
    float r[NI][8];
    float local = 0.0f;
#pragma unroll
    for (int i = 0; i < NI; ++i) {
#pragma unroll
        for (int e = 0; e < 8; ++e) r[i][e] = 0.0f;
        if (icol[i] < rq.x || icol[i] >= rq.y || irow[i] < rq.z || irow[i] >= rq.w) continue;
        const float *c = W + ioff[i];
        // k_ir_resid's arithmetic: a sum from +0 over axis i then axis j,
        // the correctly rounded division, minus the centre
        float acc[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) acc[e] = 0.0f;
#pragma unroll
        for (int o = -R; o <= R; ++o) {
            if (!o) continue;
#pragma unroll
            for (int e = 0; e < 8; ++e) acc[e] += c[e + o];
        }
#pragma unroll
        for (int o = -R; o <= R; ++o) {
            if (!o) continue;
#pragma unroll
            for (int e = 0; e < 8; ++e) acc[e] += c[o * pw + e];
        }
        const int gx = ox + 8 * icol[i], gy = oy + irow[i];
        const bool own_row = gy >= y0 && gy < y1;
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            r[i][e] = div_coeff<C>(acc[e]) - c[e];
            if (own_row && gx + e >= x0 && gx + e < x1 && in_range(gx + e, nx, R))
                local = fmaxf(local, fabsf(r[i][e]));
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) local = fmaxf(local, __shfl_xor_sync(0xffffffffu, local, o));
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = local;
    __syncthreads();  // also: every read of W is done
    bool ok = true;
    if (threadIdx.x == 0) {
        float m = 0.0f;
        for (int w = 0; w < kIr2Threads / 32; ++w) m = fmaxf(m, s_red[w]);
        // non-negative floats order as their bit patterns
        atomicMax(a.max_bits + (a.step & 1), __float_as_uint(m));
        grid_arrive(a.bar);
        ok = grid_wait_bounded(a.bar, a.bar_target);
        unsigned mb;
        asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(mb) : "l"(a.max_bits + (a.step & 1)) : "memory");
        const float mx = __uint_as_float(mb);
        int ex = 0;
        if (mx > 0.0f) frexpf(mx, &ex);  // mx = f * 2^ex, f in [0.5, 1)
        s_scale = ldexpf(1.0f, ex);
        if (blockIdx.x == 0) {
            *a.scale = s_scale;
            a.max_bits[(a.step + 1) & 1] = 0u;  // the next step's word (unused by this one)
        }
    }
    // zero both correction buffers (their border bands stay zero), then e_1 = rhs
    for (int q = threadIdx.x; q < (2 * pw * ph) / 8; q += kIr2Threads)
        reinterpret_cast<uint4 *>(ir2_smem)[q] = make_uint4(0, 0, 0, 0);
    if (!__syncthreads_and(ok)) return;
    const float s = s_scale, inv = 1.0f / s;
#pragma unroll
    for (int i = 0; i < NI; ++i) {
        if (icol[i] < rq.x || icol[i] >= rq.y || irow[i] < rq.z || irow[i] >= rq.w) continue;
        const int gx = ox + 8 * icol[i];
        float v[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) v[e] = in_range(gx + e, nx, R) ? r[i][e] * inv : 0.0f;
        uint4 q;
        q.x = Ir2Cvt<E>::pack(v[0], v[1]);
        q.y = Ir2Cvt<E>::pack(v[2], v[3]);
        q.z = Ir2Cvt<E>::pack(v[4], v[5]);
        q.w = Ir2Cvt<E>::pack(v[6], v[7]);
        *reinterpret_cast<uint4 *>(S0 + ioff[i]) = q;
        *reinterpret_cast<uint4 *>(RH + ioff[i]) = q;
    }
    int kk = min(T, a.m);
    plan_block(kk);
    __syncthreads();

    // ---- 2./3. correction sweeps in blocks of T, exchanges between -----
    int cur = 0;  // buffer holding the newest e
    unsigned tag = a.tag0;
    int k0 = 2;   // the first block's first sweep was e_1 = rhs
    for (int done = 0; done < a.m;) {
        int4 rg_next = s_region[k0 - 1];
        for (int k = k0; k <= kk; ++k) {
            const uint16_t *src = cur ? S1 : S0;
            uint16_t *dst = cur ? S0 : S1;
            const int4 rg = rg_next;
            if (k < kk) rg_next = s_region[k];
#pragma unroll
            for (int i = 0; i < NI; ++i) {
                if (icol[i] < rg.x || icol[i] >= rg.y || irow[i] < rg.z || irow[i] >= rg.w) continue;
                const uint4 v = ir2_chunk<E, R>(src + ioff[i], RH + ioff[i], pw);
                uint16_t *q = dst + ioff[i];
                const int gx = ox + 8 * icol[i];
                if (gx >= R && gx + 7 < nx - R) {
                    *reinterpret_cast<uint4 *>(q) = v;
                } else {
                    const uint32_t wv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                    for (int e = 0; e < 8; ++e)
                        if (in_range(gx + e, nx, R)) q[e] = (uint16_t)(wv[e >> 1] >> (16 * (e & 1)));
                }
            }
            __syncthreads();
            cur ^= 1;
        }
        done += kk;
        k0 = 1;
        if (done >= a.m) break;
        ++tag;
        const uint16_t *Sc = cur ? S1 : S0;
        uint16_t *Sw = cur ? S1 : S0;
        unsigned long long *slot = a.xch + (size_t)(tag & 1) * ntiles * quads_per_tile * 2;
#pragma unroll
        for (int i = 0; i < NP; ++i) {
            if (pub_s[i] < 0) continue;
            const uint2 v = *reinterpret_cast<const uint2 *>(Sc + pub_s[i]);
            asm volatile("st.volatile.global.v2.u64 [%0], {%1, %2};" ::"l"(slot + 2 * (size_t)pub_w[i]),
                         "l"(ir2_word(v.x, tag)), "l"(ir2_word(v.y, tag))
                         : "memory");
        }
        kk = min(T, a.m - done);
        plan_block(kk);
        {
            unsigned long long lo[NP], hi[NP];
#pragma unroll
            for (int i = 0; i < NP; ++i) {
                lo[i] = hi[i] = 0;
                if (ring_w[i] >= 0)
                    asm volatile("ld.volatile.global.v2.u64 {%0, %1}, [%2];"
                                 : "=l"(lo[i]), "=l"(hi[i])
                                 : "l"(slot + 2 * (size_t)ring_w[i])
                                 : "memory");
            }
#pragma unroll
            for (int i = 0; i < NP; ++i) {
                if (ring_w[i] < 0) continue;
                uint64_t t0 = 0;
                while (ok && ((unsigned)(lo[i] >> 32) != tag || (unsigned)(hi[i] >> 32) != tag)) {
                    const uint64_t t = globaltimer_ns();
                    if (!t0) t0 = t;
                    else if (t - t0 > kWaitLimitNs) {
                        report_status(kStatusTimeout);
                        ok = false;
                    }
                    asm volatile("ld.volatile.global.v2.u64 {%0, %1}, [%2];"
                                 : "=l"(lo[i]), "=l"(hi[i])
                                 : "l"(slot + 2 * (size_t)ring_w[i])
                                 : "memory");
                }
                *reinterpret_cast<uint2 *>(Sw + ring_s[i]) = make_uint2((unsigned)lo[i], (unsigned)hi[i]);
            }
        }
        if (!__syncthreads_and(ok)) return;
    }

    // ---- 4. epilogue: u += s * e_m on the owned tile ---------------------
    {
        const uint16_t *Se = cur ? S1 : S0;
        const int ya = max(y0, R), yb = min(y1, ny - R);
        const int cw = (x1 - x0) >> 2;
        const int n = cw * max(yb - ya, 0);
        for (int q = threadIdx.x; q < n; q += kIr2Threads) {
            const int y = ya + q / cw, x = x0 + 4 * (q % cw);
            float *up = a.u + (long long)y * nx + x;
            const float4 v = __ldcg(reinterpret_cast<const float4 *>(up));
            const uint2 ew = *reinterpret_cast<const uint2 *>(Se + (y - oy) * pw + (x - ox));
            const float2 e01 = Ir2Cvt<E>::two(ew.x), e23 = Ir2Cvt<E>::two(ew.y);
            const float o4[4] = {fmaf(s, e01.x, v.x), fmaf(s, e01.y, v.y), fmaf(s, e23.x, v.z),
                                 fmaf(s, e23.y, v.w)};
            if (x >= R && x + 3 < nx - R) {
                __stcg(reinterpret_cast<float4 *>(up), make_float4(o4[0], o4[1], o4[2], o4[3]));
            } else {
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (in_range(x + e, nx, R)) up[e] = o4[e];
            }
        }
    }
}

using Ir2Fn = void (*)(Geom, Ir2Plan, Ir2Args);

template <typename E, int R>
Ir2Fn ir2_fn_ni(int ni) {
    return ni <= 1 ? k_ir2d<E, R, 1> : ni <= 2 ? k_ir2d<E, R, 2> : k_ir2d<E, R, 4>;
}

template <typename E>
Ir2Fn ir2_fn(int r, int ni) {
    switch (r) {
        case 1: return ir2_fn_ni<E, 1>(ni);
        case 2: return ir2_fn_ni<E, 2>(ni);
        case 4: return ir2_fn_ni<E, 4>(ni);
        default: return nullptr;
    }
}

int ir2_items(const Ir2Plan &p) {
    const int n = (p.pw / 8) * p.ph;
    return n <= kIr2Threads ? 1 : n <= 2 * kIr2Threads ? 2 : 4;
}

int roundup8(int v) { return (v + 7) & ~7; }

bool ir2_make_plan(const Geom &g, int t, int tx, int ty, int max_ctas, Ir2Plan *p) {
    if (t < 1 || t > kIr2MaxT || tx < 8 || tx % 8 || ty < 1) return false;
    const int R = g.radius;
    Ir2Plan q;
    q.tx = tx;
    q.ty = ty;
    q.t = t;
    q.hx = roundup8((t - 1) * R) + 8;
    q.hy = t * R;
    q.pw = tx + 2 * q.hx;
    q.ph = ty + 2 * q.hy;
    q.tiles_x = (g.nx + tx - 1) / tx;
    q.tiles_y = (g.ny + ty - 1) / ty;
    if ((long long)q.tiles_x * q.tiles_y > max_ctas) return false;
    if ((q.tiles_x > 1 && q.hx > tx) || (q.tiles_y > 1 && q.hy > ty)) return false;
    if ((long long)(q.pw / 8) * q.ph > 4LL * kIr2Threads) return false;
    if (6LL * q.pw * q.ph > kIr2SmemMax) return false;
    *p = q;
    return true;
}

// Modelled SM cycles per sweep, fitted to event timings of this kernel on a
// GB300 (512^2, R = 1, FP16; 120 plans with T = 2..31 and tiles 32x64 ..
// 128x64: mean error 3.5 %, the modelled best within 3 % of the measured
// best): an exchange costs 1060 cycles plus 4.16 per halo quad, a sweep 278
// cycles plus 1.33 per 8-cell chunk of its region and 136 per further chunk
// slot of a thread.
double ir2_cost(const Geom &g, const Ir2Plan &p) {
    const int R = g.radius, ni = ir2_items(p);
    const long long ring = ((long long)p.pw * p.ph - (long long)p.tx * p.ty) / 4;
    double c = 1060.0 + 4.16 * ring;
    for (int k = 1; k <= p.t; ++k) {
        const int ext = (p.t - k) * R;
        const int chunks = (p.tx + 2 * roundup8(ext)) / 8, rows = p.ty + 2 * ext;
        c += 278.0 + 136.0 * (ni - 1) + 1.33 * chunks * rows;
    }
    return c / p.t;
}

bool ir2_choose(const Geom &g, int m, int temporal, int tile_x, int tile_y, int max_ctas,
                Ir2Plan *out) {
    const int tmax = std::max(1, std::min(m, kIr2MaxT - 1));
    bool found = false;
    double best = 1e30;
    for (int t = 1; t <= tmax; ++t) {
        if (temporal > 0 && t != std::min(temporal, tmax)) continue;
        for (int tx : {16, 24, 32, 40, 48, 64, 96, 128, 256}) {
            if (tile_x > 0 && tx != tile_x) continue;
            for (int ty : {4, 8, 12, 16, 20, 24, 32, 48, 64, 128}) {
                if (tile_y > 0 && ty != tile_y) continue;
                Ir2Plan q;
                if (!ir2_make_plan(g, t, tx, ty, max_ctas, &q)) continue;
                const double c = ir2_cost(g, q);
                if (c < best - 1e-9) {
                    best = c;
                    *out = q;
                    found = true;
                }
            }
        }
    }
    if (!found && tile_x > 0 && tile_y > 0)
        found = ir2_make_plan(g, temporal > 0 ? std::min(temporal, tmax) : 1, tile_x, tile_y,
                              max_ctas, out);
    return found;
}

// CTAs that can be resident at once (one per SM), per storage type and radius.
template <typename E>
int ir2_max_ctas(int r) {
    static std::mutex mu;
    static std::vector<std::pair<int, int>> cache;  // (device * 8 + r, ctas)
    const int dev = current_device();
    std::lock_guard<std::mutex> lock(mu);
    for (auto &c : cache)
        if (c.first == dev * 8 + r) return c.second;
    int n = 1 << 30;
    for (int ni : {1, 2, 4}) {
        const void *fn = reinterpret_cast<const void *>(ir2_fn<E>(r, ni));
        int k = 0;
        if (!fn ||
            cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, kIr2SmemMax) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k, fn, kIr2Threads, kIr2SmemMax) != cudaSuccess) {
            cudaGetLastError();
            k = 0;
        }
        n = std::min(n, k);
    }
    const int ctas = n >= 1 ? std::min(num_sms(), kIr2MaxTiles) : 0;
    cache.push_back({dev * 8 + r, ctas});
    return ctas;
}

}  // namespace

// Two slots of 16 bytes per quad of the tiles covering the grid (tiles are
// at most 256 x 128 cells, so they overhang the grid by less than one tile
// per axis).
size_t ir2_xch_bytes(const Geom &g) {
    return 2ull * ((size_t)g.nx + 256) * ((size_t)g.ny + 128) * 4;
}

template <typename E>
bool ir2_plan(const Geom &g, int m, int temporal, int tile_x, int tile_y, Ir2Plan *p) {
    if (g.nx % 8 || (g.radius != 1 && g.radius != 2 && g.radius != 4)) return false;
    const int ctas = ir2_max_ctas<E>(g.radius);
    if (ctas <= 0) return false;
    return ir2_choose(g, m, temporal, tile_x, tile_y, ctas, p) ||
           ((temporal || tile_x || tile_y) && ir2_choose(g, m, 0, 0, 0, ctas, p));
}

template <typename E>
int ir2_launch(const Geom &g, const Ir2Plan &p, float *u, unsigned long long *xch, unsigned *bar,
               unsigned *max_bits, float *scale, int step, unsigned tag0, int m, cudaStream_t s) {
    Ir2Fn fn = ir2_fn<E>(g.radius, ir2_items(p));
    if (!fn) return fail(STENCIL_EUNSUPPORTED, "no 2-D refinement engine for R=%d", g.radius);
    const int grid = p.tiles_x * p.tiles_y;
    Ir2Args a;
    a.u = u;
    a.xch = xch;
    a.bar = bar;
    a.max_bits = max_bits;
    a.scale = scale;
    a.bar_target = (unsigned)(step + 1) * (unsigned)grid;
    a.tag0 = tag0;
    a.step = step;
    a.m = m;
    Geom gg = g;
    Ir2Plan pp = p;
    void *args[] = {&gg, &pp, &a};
    const size_t smem = 6ull * p.pw * p.ph;
    ST_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(fn), dim3(grid),
                                        dim3(kIr2Threads), args, smem, s));
    return STENCIL_OK;
}

template bool ir2_plan<__nv_bfloat16>(const Geom &, int, int, int, int, Ir2Plan *);
template bool ir2_plan<__half>(const Geom &, int, int, int, int, Ir2Plan *);
template int ir2_launch<__nv_bfloat16>(const Geom &, const Ir2Plan &, float *, unsigned long long *,
                                       unsigned *, unsigned *, float *, int, unsigned, int, cudaStream_t);
template int ir2_launch<__half>(const Geom &, const Ir2Plan &, float *, unsigned long long *,
                                unsigned *, unsigned *, float *, int, unsigned, int, cudaStream_t);

}  // namespace st

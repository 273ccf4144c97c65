// k_tb.cu -- temporally blocked 3-D sweeps ("coop" role, src/stencil_kernel_coop.cu:5-49):
// one launch performs T sweeps (src -> dst) with one HBM round trip.
//
// A CTA owns an output tile of TX x TY cells and marches along z over a
// contiguous share of the (tile, plane) steps.  Level 0 plane tiles -- the
// output tile plus a halo of T*R cells (x halo rounded up to 4 for TMA
// alignment) -- stream in by TMA (cp.async.bulk.tensor.3d, mbarrier
// completion) from a warp-specialised producer into a ring of NS slots.
// Levels 1..T-1 live in shared-memory rings of 2R+1 plane tiles each.  When
// level-0 plane p arrives, level t computes its plane p - t*R from level t-1's
// planes p - (t+1)R .. p - (t-1)R; level T writes its plane p - T*R to global
// memory.  Each level's valid region shrinks by R per side (overlapped, or
// "trapezoidal", tiling with redundant halo compute), so no CTA waits for
// another: the only synchronisation is a named barrier among the consumer
// warps between levels.  Every cell keeps the reference's summation order, so
// results are bit-identical to T single sweeps.
//
// JACOBI only (the border band is equal in both buffers, so a border cell
// keeps its value at every level); LEGACY falls back to single sweeps.
#include <algorithm>

#include "host.hpp"

namespace st {

template <int R, int T, int TX, int TY>
struct TbShape {
    static constexpr int HX = ((T * R + 3) / 4) * 4;  // x halo, whole float4 chunks
    static constexpr int HY = T * R;
    static constexpr int PW = TX + 2 * HX;
    static constexpr int PH = TY + 2 * HY;
    static constexpr int NC = PW / 4;  // float4 chunks per row
    static constexpr int PLANE_FLOATS = PW * PH;
    static constexpr int SLOT_FLOATS = (PLANE_FLOATS + 31) & ~31;
    static constexpr int PLANE_BYTES = PLANE_FLOATS * 4;
    static constexpr int NR = 2 * R + 1;      // ring of levels 1..T-1
    static constexpr int NS = 2 * R + 1 + 3;  // level-0 ring: window + 3 in flight
    static constexpr int CONSUMERS = 512;
    static constexpr int THREADS = CONSUMERS + 32;
    static constexpr int SMEM_BYTES =
        (NS + (T - 1) * NR) * SLOT_FLOATS * 4 + 128 + 2 * NS * 8;
    static_assert(PW <= 256 && PH <= 256, "TMA box dimensions are limited to 256");
    static_assert(SMEM_BYTES <= 227 * 1024, "shared memory");
};

__device__ __forceinline__ float4 tb_ld4(const float *p) {
    return *reinterpret_cast<const float4 *>(p);
}

__device__ __forceinline__ void consumer_barrier() {
    asm volatile("bar.sync 1, 512;" ::: "memory");
}

}  // namespace st

namespace st {

// Named barrier over the consumer warps that also ANDs a predicate, so that
// a failed bounded wait ends every consumer together.
__device__ __forceinline__ bool consumer_barrier_and(bool ok) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.and.pred p, 1, 512, p;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)ok)
        : "memory");
    return r != 0;
}

// One unit: 4 cells (one float4 chunk c of one row) of a level's plane.
// xmask: bit e set if cell e of the chunk lies in the update range along x.
template <int R, int T, int TX, int TY, bool LAST>
__device__ __forceinline__ void tb_unit(const float *cp, const float *const *zp, float *outp,
                                        float *drow, int row, int c, unsigned xmask, bool yin,
                                        bool xin4) {
    using S = TbShape<R, T, TX, TY>;
    constexpr int C = 6 * R;
    const int off = row * S::PW + 4 * c;
    const float4 left = tb_ld4(cp + off - (c > 0 ? 4 : 0));
    const float4 mid = tb_ld4(cp + off);
    const float4 right = tb_ld4(cp + off + (c < S::NC - 1 ? 4 : 0));
    const float w[12] = {left.x, left.y, left.z, left.w, mid.x, mid.y, mid.z,
                         mid.w, right.x, right.y, right.z, right.w};
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
        const float4 v = tb_ld4(cp + off + o * S::PW);
        acc[0] += v.x; acc[1] += v.y; acc[2] += v.z; acc[3] += v.w;
    }
#pragma unroll
    for (int o = -R; o <= R; ++o) {
        if (!o) continue;
        const float4 v = tb_ld4(zp[o + R] + off);
        acc[0] += v.x; acc[1] += v.y; acc[2] += v.z; acc[3] += v.w;
    }
    // +0 sums are exact on the fast path (a sum never yields -0)
    float a4[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) a4[e] = acc[e] == 0.0f ? 1.0f : fabsf(acc[e]);
    const float lo4 = fminf(fminf(a4[0], a4[1]), fminf(a4[2], a4[3]));
    const float hi4 = fmaxf(fmaxf(a4[0], a4[1]), fmaxf(a4[2], a4[3]));
    if (__all_sync(__activemask(), lo4 >= 0x1p-100f && hi4 <= 0x1p+120f)) {
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[e] = div_fast<C>(acc[e]);
    } else {
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[e] = acc[e] / (float)C;
    }
    if (!LAST) {
        float o4[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) o4[e] = (yin && ((xmask >> e) & 1)) ? acc[e] : w[4 + e];
        *reinterpret_cast<float4 *>(outp + off) = make_float4(o4[0], o4[1], o4[2], o4[3]);
    } else if (yin) {
        if (xin4) {
            stg4(drow, acc[0], acc[1], acc[2], acc[3]);
        } else {
#pragma unroll
            for (int e = 0; e < 4; ++e)
                if ((xmask >> e) & 1) drow[e] = acc[e];
        }
    }
}

// One level's plane.  Warp w owns rows r0 + w, r0 + w + 16, ...; lane l owns
// chunk 1 + l (the 32 chunks of the output tile's columns).  Levels below T
// also need the two edge chunks of each row (their halo cells); those units
// go to the last warps, which own fewer rows.  Border cells (outside the
// update region) keep the centre value; the whole-plane border case copies.
template <int R, int T, int TX, int TY, bool LAST>
__device__ __forceinline__ void tb_level(const float *cp, const float *const *zp, float *outp,
                                         float *__restrict__ dst, const Geom &g, int x0, int y0,
                                         int gz, int r0, int r1, bool border_plane,
                                         unsigned lane_xmask, unsigned edge_xmask0,
                                         unsigned edge_xmask1) {
    using S = TbShape<R, T, TX, TY>;
    static_assert(S::NC == TX / 4 + 2 && S::HX == 4, "one edge chunk per side");
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int c = 1 + lane;
    if (border_plane) {  // whole plane outside the update region: copy (levels < T only)
        for (int u = tid; u < (r1 - r0) * S::NC; u += S::CONSUMERS) {
            const int off = (r0 + u / S::NC) * S::PW + 4 * (u % S::NC);
            *reinterpret_cast<float4 *>(outp + off) = tb_ld4(cp + off);
        }
        return;
    }
    const int gx0 = x0 - S::HX + 4 * c;
    const bool xin4 = lane_xmask == 0xFu;
    for (int row = r0 + warp; row < r1; row += S::CONSUMERS / 32) {
        const int gy = y0 - S::HY + row;
        const bool yin = in_range(gy, g.ny, R);
        float *drow = LAST ? dst + (long long)gz * g.sz + (long long)gy * g.sy + gx0 : nullptr;
        tb_unit<R, T, TX, TY, LAST>(cp, zp, outp, drow, row, c, lane_xmask, yin, xin4);
    }
    if (!LAST) {
        const int et = S::CONSUMERS - 1 - tid;  // edge units on the last threads
        if (et < 2 * (r1 - r0)) {
            const int row = r0 + (et >> 1), side = et & 1;
            const int gy = y0 - S::HY + row;
            tb_unit<R, T, TX, TY, false>(cp, zp, outp, nullptr, row, side ? S::NC - 1 : 0,
                                         side ? edge_xmask1 : edge_xmask0, in_range(gy, g.ny, R),
                                         false);
        }
    }
}

template <int R, int T, int TX, int TY>
__global__ void __launch_bounds__(TbShape<R, T, TX, TY>::THREADS, 1)
    k_tb3d(const __grid_constant__ CUtensorMap src_map, float *__restrict__ dst, Geom g,
           int tiles_x, long long total) {
    using S = TbShape<R, T, TX, TY>;
    constexpr int C = 6 * R;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float *ring0 = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) &
                                             ~static_cast<uintptr_t>(127));
    float *lring = ring0 + S::NS * S::SLOT_FLOATS;  // level t (1..T-1) at (t-1)*NR slots
    uint64_t *full = reinterpret_cast<uint64_t *>(lring + (T - 1) * S::NR * S::SLOT_FLOATS);
    uint64_t *empty = full + S::NS;
    const int tid = threadIdx.x;
    if (tid == 0) {
        prefetch_tensormap(&src_map);
        for (int s = 0; s < S::NS; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        fence_mbar_init();
    }
    __syncthreads();
    const int zin = g.nz - 2 * R;
    const long long lo = total * blockIdx.x / gridDim.x;
    const long long hi = total * (blockIdx.x + 1) / gridDim.x;

    if (tid >= S::CONSUMERS) {
        // ---------------- producer (one lane) ----------------
        if (tid != S::CONSUMERS) return;
        uint32_t seq = 0;
        for (long long i = lo; i < hi;) {
            const int t = (int)(i / zin);
            const int za = R + (int)(i - (long long)t * zin);
            const long long rem = hi - (long long)t * zin;
            const int zb = R + (int)(rem < zin ? rem : (long long)zin);
            i = (long long)t * zin + (zb - R);
            const int x0 = (t % tiles_x) * TX, y0 = (t / tiles_x) * TY;
            const int p0 = max(0, za - T * R), h0 = min(g.nz, zb + T * R);
            for (int p = p0; p < h0; ++p, ++seq) {
                const int s = seq % S::NS;
                const uint32_t use = seq / S::NS;
                if (use > 0 && !mbar_wait_bounded(&empty[s], (use - 1) & 1)) return;
                fence_proxy_async();  // the consumers' reads of the slot before the TMA write
                mbar_arrive_expect_tx(&full[s], S::PLANE_BYTES);
                tma_load_3d(ring0 + s * S::SLOT_FLOATS, &src_map, &full[s], x0 - S::HX,
                            y0 - S::HY, p);
            }
        }
        return;
    }

    // ---------------- consumers ----------------
    uint32_t qb = 0;  // sequence number of this segment's first level-0 plane
    for (long long i = lo; i < hi;) {
        const int t = (int)(i / zin);
        const int za = R + (int)(i - (long long)t * zin);
        const long long rem = hi - (long long)t * zin;
        const int zb = R + (int)(rem < zin ? rem : (long long)zin);
        i = (long long)t * zin + (zb - R);
        const int x0 = (t % tiles_x) * TX, y0 = (t / tiles_x) * TY;
        const int p0 = max(0, za - T * R), h0 = min(g.nz, zb + T * R);
        auto xmask_of = [&](int chunk) {
            unsigned m = 0;
            const int gx = x0 - S::HX + 4 * chunk;
#pragma unroll
            for (int e = 0; e < 4; ++e)
                if (in_range(gx + e, g.nx, R)) m |= 1u << e;
            return m;
        };
        const unsigned lane_xmask = xmask_of(1 + (tid & 31));
        const unsigned edge_xmask0 = xmask_of(0), edge_xmask1 = xmask_of(S::NC - 1);
        auto plane0 = [&](int z) -> float * {
            return ring0 + ((qb + (uint32_t)(z - p0)) % S::NS) * S::SLOT_FLOATS;
        };
        auto planeL = [&](int lvl, int z) -> float * {  // level lvl >= 1
            return lring + ((lvl - 1) * S::NR + z % S::NR) * S::SLOT_FLOATS;
        };
        for (int p = p0; p < h0 + T * R; ++p) {
            bool ok = true;
            if (p < h0) {
                const uint32_t q = qb + (uint32_t)(p - p0);
                ok = mbar_wait_bounded(&full[q % S::NS], (q / S::NS) & 1);
            }
            if (!consumer_barrier_and(ok)) return;
#pragma unroll 1
            for (int lvl = 1; lvl <= T; ++lvl) {
                const int q = p - lvl * R;
                const int lo_t = max(0, za - (T - lvl) * R), hi_t = min(g.nz, zb + (T - lvl) * R);
                if (q >= lo_t && q < hi_t) {
                    auto prev = [&](int z) -> const float * {
                        return lvl == 1 ? plane0(z) : planeL(lvl - 1, z);
                    };
                    const int r0 = lvl * R, r1 = S::PH - lvl * R;
                    const bool border_plane = q < R || q >= g.nz - R;
                    const float *cp = prev(q);
                    float *outp = lvl < T ? planeL(lvl, q) : nullptr;
                    const float *zp[2 * R + 1];
#pragma unroll
                    for (int o = -R; o <= R; ++o) zp[o + R] = (o && !border_plane) ? prev(q + o) : cp;
                    if (lvl < T)
                        tb_level<R, T, TX, TY, false>(cp, zp, outp, dst, g, x0, y0, q, r0, r1,
                                                      border_plane, lane_xmask, edge_xmask0,
                                                      edge_xmask1);
                    else if (!border_plane)
                        tb_level<R, T, TX, TY, true>(cp, zp, outp, dst, g, x0, y0, q, r0, r1,
                                                     false, lane_xmask, edge_xmask0, edge_xmask1);
                }
                consumer_barrier();
                // Level 1 no longer needs level-0 plane p - 2R: hand its slot back.
                if (lvl == 1 && tid == 0) {
                    const int z = p - 2 * R;
                    if (z >= p0 && z < h0) mbar_arrive(&empty[(qb + (uint32_t)(z - p0)) % S::NS]);
                }
            }
        }
        qb += (uint32_t)(h0 - p0);
    }
}

}  // namespace st

namespace st {
namespace {

struct TbKernel {
    const void *fn;
    int tx, ty, threads, smem, T, hx, hy;
};

template <int R, int T, int TX, int TY>
TbKernel tbk() {
    using S = TbShape<R, T, TX, TY>;
    return {reinterpret_cast<const void *>(k_tb3d<R, T, TX, TY>), TX, TY, S::THREADS,
            S::SMEM_BYTES, T, S::HX, S::HY};
}

TbKernel pick_tb(int r, int t) {
    if (r == 1) {
        if (t >= 4) return tbk<1, 4, 128, 16>();
        if (t == 3) return tbk<1, 3, 128, 16>();
        return tbk<1, 2, 128, 16>();
    }
    if (r == 2) return tbk<2, 2, 128, 16>();
    return {nullptr, 0, 0, 0, 0, 0, 0, 0};
}

}  // namespace

bool tb3d_supported(const Geom &g) {
    return !g.legacy && g.nx % 4 == 0 && (g.radius == 1 || g.radius == 2);
}

int default_temporal(int radius) { return radius == 1 ? 4 : 2; }

// iters sweeps a -> ... with passes of T sweeps each; remainder by single sweeps.
int run_tb3d(const Geom &g, float *a, float *b, int iters, int temporal, cudaStream_t s,
             float **res) {
    if (!tb3d_supported(g)) return fail(STENCIL_EUNSUPPORTED, "temporal blocking needs JACOBI, nx %% 4 == 0, R <= 2");
    TbKernel k = pick_tb(g.radius, temporal > 0 ? temporal : default_temporal(g.radius));
    if (!k.fn) return fail(STENCIL_EUNSUPPORTED, "no temporal-blocking instance for R=%d", g.radius);
    ST_CUDA(cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, k.smem));
    int per_sm = 0;
    ST_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k.fn, k.threads, k.smem));
    if (per_sm < 1) return fail(STENCIL_EUNSUPPORTED, "temporal-blocking kernel does not fit");
    const int tiles_x = (g.nx + k.tx - 1) / k.tx, tiles_y = (g.ny + k.ty - 1) / k.ty;
    const long long total = (long long)tiles_x * tiles_y * (g.nz - 2 * g.radius);
    const int grid = (int)std::min<long long>((long long)per_sm * num_sms(), total);
    const long long dims[3] = {g.nx, g.ny, g.nz};
    const int box[3] = {k.tx + 2 * k.hx, k.ty + 2 * k.hy, 1};
    CUtensorMap maps[2];
    int rc = make_tensor_map(&maps[0], a, 3, dims, box);
    if (!rc) rc = make_tensor_map(&maps[1], b, 3, dims, box);
    if (rc) return rc;
    float *cur = a, *nxt = b;
    int ci = 0;
    Geom gg = g;
    int tx_ = tiles_x;
    long long tot_ = total;
    const int passes = iters / k.T;
    note_launches("tb3d", passes);
    for (int it = 0; it < passes; ++it) {
        void *args[] = {&maps[ci], &nxt, &gg, &tx_, &tot_};
        ST_CUDA(cudaLaunchKernel(k.fn, dim3(grid), dim3(k.threads), args, k.smem, s));
        std::swap(cur, nxt);
        ci ^= 1;
    }
    const int remainder = iters - passes * k.T;
    if (remainder) {
        float *out = nullptr;
        rc = run_stream3d(g, cur, nxt, remainder, 0, 0, s, &out);
        if (rc) return rc;
        cur = out;
    }
    if (res) *res = cur;
    return STENCIL_OK;
}

}  // namespace st

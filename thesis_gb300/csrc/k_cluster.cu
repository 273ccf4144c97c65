// k_cluster.cu -- the cluster engine: one thread-block cluster runs every sweep
// of one grid in a single persistent launch ("coop" role,
// src/stencil_kernel_coop.cu:5-49, whose launch the reference left commented
// out at src/stencil_dispatch.cu:160-177), and a batch of grids of uneven
// sizes and sweep counts runs as one launch over a device work queue.
//
// The slowest axis (rows in 2-D, planes in 3-D) is split into slabs, one per
// CTA of the cluster.  Per sweep every CTA updates its slab, then the cluster
// synchronises with the hardware cluster barrier (release/acquire at cluster
// scope) -- the grid-wide sync of the reference's coop kernel, restricted to
// the CTAs that share the grid.  Two storage modes:
//   * resident: both ping-pong buffers of the slab plus R halo slices on each
//     side live in shared memory; after a sweep each CTA pushes its first and
//     last R slices into its neighbours' halos through distributed shared
//     memory (st.shared::cluster), so HBM is touched only to load and store
//     the grid once per launch;
//   * global: the slabs are swept from global memory (L2-resident for the
//     batch sizes) with the same per-cell code.
// Per-cell code: 3-D slabs by columns of float4 chunks marched along z with
// a register queue (sweep_cols3d), 2-D slabs by chunk columns of row blocks
// with a register queue along y (sweep_rows2d, rows of at most 4 * blockDim.x
// cells), other 2-D rows by the generic sweep (sweep_slab).
// Cells outside the update region are never written, and both buffers are
// loaded from the caller's two buffers, so LEGACY (second-buffer border) and
// JACOBI semantics are exactly those of the ping-pong loop; at the end both
// global buffers hold what the ping-pong loop leaves (last sweep in the result
// buffer, the sweep before in the other).
//
// Work queue: CTA rank 0 of each cluster takes the next job index with an
// atomic on a device counter and shares it through distributed shared memory.
// Jobs are ordered by the host (largest first).  Every wait is a hardware
// cluster barrier: no spin loops.
#include <algorithm>
#include <cstdlib>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "host.hpp"

namespace st {

bool tb3d_supported(const Geom &g);

struct ClusterJob {
    float *a, *b;       // the grid's two buffers (a = initial state)
    int dims, nx, ny, nz;
    int radius, iters, legacy, resident;
    int tblock;         // resident mode: sweeps between halo exchanges (>= 1)
    int px;             // row pitch in cells (a multiple of 4, >= nx)
};

constexpr int kClusterThreads = 512;

__device__ __forceinline__ float4 ld4(const float *p) { return *reinterpret_cast<const float4 *>(p); }

// One sweep of the cells of slices [s_begin, s_end) (global slice indices).
// src/dst address slice s at (s - base) * slice_len; the slice stride is
// slice_len; within a slice the row pitch is px (a multiple of 4; cells nx ..
// px-1 of a row are padding, read only for cells outside the update region).
// Rows of the update region only; float4 chunks.  Generic form (any D); used
// for 2-D rows wider than 4 * blockDim.x cells.
template <int D, int R>
__device__ __forceinline__ void sweep_slab(const float *src, float *dst, long long base,
                                           int s_begin, int s_end, const ClusterJob &j) {
    constexpr int C = 2 * D * R;
    const int nx = j.nx, ny = j.ny, px = j.px;
    const long long slice_len = D == 3 ? (long long)px * ny : px;
    const int chunks = px >> 2;
    const int rows = D == 3 ? ny - 2 * R : 1;  // update rows per slice
    const int S = D == 3 ? j.nz : ny;
    const int sb = max(s_begin, R), se = min(s_end, S - R);
    if (sb >= se) return;
    const long long units = (long long)(se - sb) * rows * chunks;
    for (long long u = threadIdx.x; u < units; u += blockDim.x) {
        const int c = (int)(u % chunks);
        const long long rs = u / chunks;
        const int row = D == 3 ? R + (int)(rs % rows) : 0;
        const int s = sb + (int)(rs / rows);
        const int x0 = c * 4;
        if (x0 + 3 < R || x0 >= nx - R) continue;
        const long long off = (long long)(s - base) * slice_len + (long long)row * px + x0;
        const float *p = src + off;
        float w[4 + 2 * ((R + 3) & ~3)];
        constexpr int RA = (R + 3) & ~3;
#pragma unroll
        for (int h = 0; h < (4 + 2 * RA) / 4; ++h) {
            const int cc = c - RA / 4 + h;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (cc >= 0 && cc < chunks) v = ld4(p - RA + 4 * h);
            w[4 * h] = v.x; w[4 * h + 1] = v.y; w[4 * h + 2] = v.z; w[4 * h + 3] = v.w;
        }
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int o = -R; o <= R; ++o) {
            if (!o) continue;
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[e] += w[RA + e + o];
        }
        // axis j: the next row (3-D) or the next slice (2-D)
        const long long sj = D == 3 ? px : slice_len;
#pragma unroll
        for (int o = -R; o <= R; ++o) {
            if (!o) continue;
            const float4 v = ld4(p + o * sj);
            acc[0] += v.x; acc[1] += v.y; acc[2] += v.z; acc[3] += v.w;
        }
        if (D == 3) {
#pragma unroll
            for (int o = -R; o <= R; ++o) {
                if (!o) continue;
                const float4 v = ld4(p + o * slice_len);
                acc[0] += v.x; acc[1] += v.y; acc[2] += v.z; acc[3] += v.w;
            }
        }
        float out[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            out[e] = div_coeff<C>(acc[e]);
            if (j.legacy) out[e] -= w[RA + e];
        }
        float *q = dst + off;
        if (x0 >= R && x0 + 3 < nx - R) {
            *reinterpret_cast<float4 *>(q) = make_float4(out[0], out[1], out[2], out[3]);
        } else {
#pragma unroll
            for (int e = 0; e < 4; ++e)
                if (x0 + e >= R && x0 + e < nx - R) q[e] = out[e];
        }
    }
}

// 2-D slab sweep with a fixed thread -> (chunk, row block) map: lane group
// g of the CTA owns a contiguous block of rows, thread c of the group owns
// float4 chunk c of every row in it.  The chunk's column of the rows j-R ..
// j+R rides in a register queue down the block (one new 16-byte load per
// row); only the x-neighbour chunks are loaded per row.  No index division in
// the loop.  Requires px / 4 <= blockDim.x.
template <int R>
__device__ __forceinline__ void sweep_rows2d(const float *src, float *dst, long long base,
                                             int s_begin, int s_end, const ClusterJob &j) {
    constexpr int C = 4 * R;
    constexpr int RA = (R + 3) & ~3;
    const int nx = j.nx, ny = j.ny, px = j.px, chunks = px >> 2;
    const int G = blockDim.x / chunks;
    const int c = threadIdx.x % chunks, grp = threadIdx.x / chunks;
    const int rb = max(s_begin, R), re = min(s_end, ny - R);
    if (grp >= G || rb >= re) return;
    const int per = (re - rb + G - 1) / G;
    const int j0 = rb + grp * per, j1 = min(re, j0 + per);
    if (j0 >= j1) return;
    const int x0 = 4 * c;
    unsigned mask = 0;
#pragma unroll
    for (int e = 0; e < 4; ++e)
        if (x0 + e >= R && x0 + e < nx - R) mask |= 1u << e;
    if (!mask) return;
    const float *col = src + (long long)(-base) * px + x0;  // row j of this chunk at col + j*px
    float *dcol = dst + (long long)(-base) * px + x0;
    float4 q[2 * R + 1];  // rows j-R .. j+R of this chunk
#pragma unroll
    for (int k = 0; k < 2 * R; ++k) q[k] = ld4(col + (long long)(j0 - R + k) * px);
#pragma unroll 2
    for (int jj = j0; jj < j1; ++jj) {
        q[2 * R] = ld4(col + (long long)(jj + R) * px);
        const float *row = col + (long long)jj * px;
        float w[4 + 2 * RA];
#pragma unroll
        for (int h = 0; h < RA / 4; ++h) {
            float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
            if (c - RA / 4 + h >= 0) a = ld4(row - RA + 4 * h);
            if (c + 1 + h < chunks) b = ld4(row + 4 + 4 * h);
            w[4 * h] = a.x; w[4 * h + 1] = a.y; w[4 * h + 2] = a.z; w[4 * h + 3] = a.w;
            w[RA + 4 + 4 * h] = b.x; w[RA + 5 + 4 * h] = b.y;
            w[RA + 6 + 4 * h] = b.z; w[RA + 7 + 4 * h] = b.w;
        }
        const float4 m = q[R];
        w[RA] = m.x; w[RA + 1] = m.y; w[RA + 2] = m.z; w[RA + 3] = m.w;
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int o = -R; o <= R; ++o) {
            if (!o) continue;
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[e] += w[RA + e + o];
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
            if (j.legacy) out[e] -= w[RA + e];
        }
        float *d = dcol + (long long)jj * px;
        if (mask == 0xFu) {
            *reinterpret_cast<float4 *>(d) = make_float4(out[0], out[1], out[2], out[3]);
        } else {
#pragma unroll
            for (int e = 0; e < 4; ++e)
                if ((mask >> e) & 1) d[e] = out[e];
        }
#pragma unroll
        for (int k = 0; k < 2 * R; ++k) q[k] = q[k + 1];
    }
}

// 3-D slab sweep with a fixed thread -> column map: thread u owns float4
// chunk u % chunks of update row R + u / chunks (one 32-bit division per
// column, none per cell) and marches it through the slab's slices, keeping the
// column's slices s-R .. s+R in a register queue (one new 16-byte load per
// slice).  Per 4 cells: 1 + 2 (x-neighbour chunks) + 2R (y rows) loads, where
// the generic slab sweep re-derives (slice, row, chunk) with 64-bit divisions
// and issues 3 + 4R loads.  Same per-cell summation order and division.
// PIPE: the loads of slice s+1 are issued before slice s is computed, for the
// global mode, which is bound by L2 latency (18 grids of 56^3 .. 104^3, R = 2,
// in one batch: 193.8 GCell/s with the generic sweep, 232.6 with the column
// sweep, 260.8 with PIPE; R = 1: 220.4 / 259.0 / 325.8); from shared memory
// the extra registers cost more than the early loads gain (36 grids of
// 24^3 .. 48^3, R = 2: 102.3 without, 94.5 with).
template <int R, bool PIPE>
__device__ __forceinline__ void sweep_cols3d(const float *src, float *dst, long long base,
                                             int s_begin, int s_end, const ClusterJob &j) {
    constexpr int C = 6 * R;
    constexpr int RA = (R + 3) & ~3;
    static_assert(RA == 4, "one neighbour chunk per side");
    const int nx = j.nx, ny = j.ny, px = j.px, chunks = px >> 2;
    const long long sl = (long long)px * ny;
    const int rows = ny - 2 * R;
    const int sb = max(s_begin, R), se = min(s_end, j.nz - R);
    if (sb >= se || rows <= 0) return;
    const int cols = rows * chunks;
    for (int u = threadIdx.x; u < cols; u += blockDim.x) {
        const int c = u % chunks, row = R + u / chunks;
        const int x0 = 4 * c;
        unsigned mask = 0;
#pragma unroll
        for (int e = 0; e < 4; ++e)
            if (x0 + e >= R && x0 + e < nx - R) mask |= 1u << e;
        if (!mask) continue;
        const long long off = (long long)(sb - base) * sl + (long long)row * px + x0;
        const float *col = src + off;  // slice sb of this column
        float *dcol = dst + off;
        const bool has_l = c > 0, has_r = c + 1 < chunks;
        const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
        float4 q[2 * R + 1];  // slices s-R .. s+R of this column
#pragma unroll
        for (int k = 0; k < 2 * R; ++k) q[k] = ld4(col + (k - R) * sl);
        float4 nq = z4, nl = z4, nr = z4, nyv[2 * R];
        if constexpr (PIPE) {
            nq = ld4(col + R * sl);
            if (has_l) nl = ld4(col - 4);
            if (has_r) nr = ld4(col + 4);
#pragma unroll
            for (int o = -R; o <= R; ++o)
                if (o) nyv[o < 0 ? o + R : o + R - 1] = ld4(col + o * px);
        }
#pragma unroll 2
        for (int s = sb; s < se; ++s) {
            float4 l4, r4, yv[2 * R];
            if constexpr (PIPE) {
                q[2 * R] = nq;
                l4 = nl;
                r4 = nr;
#pragma unroll
                for (int k = 0; k < 2 * R; ++k) yv[k] = nyv[k];
                if (s + 1 < se) {
                    const float *nc = col + sl;
                    nq = ld4(nc + R * sl);
                    if (has_l) nl = ld4(nc - 4);
                    if (has_r) nr = ld4(nc + 4);
#pragma unroll
                    for (int o = -R; o <= R; ++o)
                        if (o) nyv[o < 0 ? o + R : o + R - 1] = ld4(nc + o * px);
                }
            } else {
                q[2 * R] = ld4(col + R * sl);
                l4 = has_l ? ld4(col - 4) : z4;
                r4 = has_r ? ld4(col + 4) : z4;
#pragma unroll
                for (int o = -R; o <= R; ++o)
                    if (o) yv[o < 0 ? o + R : o + R - 1] = ld4(col + o * px);
            }
            const float4 m4 = q[R];
            const float w[12] = {l4.x, l4.y, l4.z, l4.w, m4.x, m4.y, m4.z, m4.w, r4.x, r4.y, r4.z, r4.w};
            float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int o = -R; o <= R; ++o) {
                if (!o) continue;
#pragma unroll
                for (int e = 0; e < 4; ++e) acc[e] += w[4 + e + o];
            }
#pragma unroll
            for (int k = 0; k < 2 * R; ++k) {
                acc[0] += yv[k].x; acc[1] += yv[k].y; acc[2] += yv[k].z; acc[3] += yv[k].w;
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
                if (j.legacy) out[e] -= w[4 + e];
            }
            if (mask == 0xFu) {
                *reinterpret_cast<float4 *>(dcol) = make_float4(out[0], out[1], out[2], out[3]);
            } else {
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if ((mask >> e) & 1) dcol[e] = out[e];
            }
#pragma unroll
            for (int k = 0; k < 2 * R; ++k) q[k] = q[k + 1];
            col += sl;
            dcol += sl;
        }
    }
}

// Copies slices [s_begin, s_end) between a global grid and a local slab.
__device__ __forceinline__ void copy_slices(float *to, const float *from, long long count4) {
    for (long long i = threadIdx.x; i < count4; i += blockDim.x)
        reinterpret_cast<float4 *>(to)[i] = reinterpret_cast<const float4 *>(from)[i];
}

template <int D, int R>
__device__ void run_job(const ClusterJob &j, float *smem, uint32_t rank, uint32_t csize) {
    const int S = D == 3 ? j.nz : j.ny;
    const long long slice_len = D == 3 ? (long long)j.px * j.ny : j.px;
    const int H = (S + csize - 1) / csize;
    const int s0 = min((int)rank * H, S), s1 = min(s0 + H, S);
    if (j.resident) {
        // Slab with a halo of HT = tblock * R slices per side: local slice k
        // <-> global slice s0 - HT + k.  Between halo exchanges the CTA runs
        // tblock sweeps; sweep k of a block also updates the (tblock - k) * R
        // halo slices next to its own slab (a trapezoid), with arithmetic
        // identical to the owner's, so one exchange serves tblock sweeps.
        const int TB = j.tblock, HT = TB * R;
        const long long slab = (long long)(H + 2 * HT) * slice_len;
        float *buf[2] = {smem, smem + slab};
        const int l0 = max(s0 - HT, 0), l1 = min(s1 + HT, S);
        if (l0 < l1) {
            const long long off = (long long)(l0 - (s0 - HT)) * slice_len;
            copy_slices(buf[0] + off, j.a + (long long)l0 * slice_len, (l1 - l0) * slice_len / 4);
            copy_slices(buf[1] + off, j.b + (long long)l0 * slice_len, (l1 - l0) * slice_len / 4);
        }
        cluster_sync();
        const uint32_t my0 = smem_u32(buf[0]);
        int cur = 0;
        for (int it = 0; it < j.iters;) {
            const int kk = min(TB, j.iters - it);
            for (int k = 1; k <= kk; ++k) {
                const int ext = (kk - k) * R;
                const int a = max(s0 - ext, 0), b = min(s1 + ext, S);
                if (s1 > s0) {
                    if constexpr (D == 3)
                        sweep_cols3d<R, false>(buf[cur], buf[cur ^ 1], s0 - HT, a, b, j);
                    else if ((j.px >> 2) <= (int)blockDim.x)
                        sweep_rows2d<R>(buf[cur], buf[cur ^ 1], s0 - HT, a, b, j);
                    else
                        sweep_slab<D, R>(buf[cur], buf[cur ^ 1], s0 - HT, a, b, j);
                }
                __syncthreads();
                cur ^= 1;
            }
            it += kk;
            if (it >= j.iters) break;
            // Every CTA has finished reading its halo; refresh the halos of
            // buf[cur] with the neighbours' newest own slices.
            if (TB > 1) cluster_sync();
            const long long n4 = (long long)HT * slice_len / 4;
            const uint32_t dst_base = my0 + (uint32_t)(cur * slab * 4);
            if (rank > 0 && s1 > s0) {
                // my slices s0 .. s0+HT-1 -> rank-1's local slices H+HT .. H+2HT-1
                const float4 *from = reinterpret_cast<const float4 *>(buf[cur] + (long long)HT * slice_len);
                const uint32_t to = mapa_shared(dst_base + (uint32_t)((long long)(H + HT) * slice_len * 4), rank - 1);
                for (long long i = threadIdx.x; i < n4; i += blockDim.x) st_cluster_v4(to + (uint32_t)(i * 16), from[i]);
            }
            if (rank + 1 < csize && s1 > s0 && s1 < S) {
                // my slices s1-HT .. s1-1 -> rank+1's local slices 0 .. HT-1
                const float4 *from = reinterpret_cast<const float4 *>(buf[cur] + (long long)(s1 - s0) * slice_len);
                const uint32_t to = mapa_shared(dst_base, rank + 1);
                for (long long i = threadIdx.x; i < n4; i += blockDim.x) st_cluster_v4(to + (uint32_t)(i * 16), from[i]);
            }
            cluster_sync();
        }
        // Both buffers back to the caller's buffers (owned slices only).
        if (s1 > s0) {
            const long long off = (long long)HT * slice_len;
            float *ga = (j.iters & 1) ? j.b : j.a;  // holds buf[cur]
            float *gb = (j.iters & 1) ? j.a : j.b;
            copy_slices(ga + (long long)s0 * slice_len, buf[cur] + off, (s1 - s0) * slice_len / 4);
            copy_slices(gb + (long long)s0 * slice_len, buf[cur ^ 1] + off, (s1 - s0) * slice_len / 4);
        }
        cluster_sync();  // the slab is reused by the next job
    } else {
        const float *src = j.a;
        float *dst = j.b;
        for (int it = 0; it < j.iters; ++it) {
            if constexpr (D == 3)
                sweep_cols3d<R, (R <= 2)>(src, dst, 0, s0, s1, j);  // R >= 3: no register room
            else if ((j.px >> 2) <= (int)blockDim.x)
                sweep_rows2d<R>(src, dst, 0, s0, s1, j);
            else
                sweep_slab<D, R>(src, dst, 0, s0, s1, j);
            cluster_sync();
            const float *t = src;
            src = dst;
            dst = const_cast<float *>(t);
        }
    }
}

// queue == nullptr: the single job `one` (one cluster).  Otherwise clusters
// take job indices from *queue until it passes njobs.
__global__ void __launch_bounds__(kClusterThreads)
    k_cluster(ClusterJob one, const ClusterJob *__restrict__ jobs, int njobs, unsigned *queue) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ int s_job;
    __shared__ int s_jid;
    float *smem = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) &
                                            ~static_cast<uintptr_t>(127));
    const uint32_t rank = cluster_ctarank(), csize = cluster_nctarank();
    const uint32_t job_addr = mapa_shared(smem_u32(&s_job), 0);
    for (int round = 0;; ++round) {
        int jid;
        if (queue) {
            if (rank == 0 && threadIdx.x == 0) s_job = (int)atomicAdd(queue, 1u);
            cluster_sync();
            if (threadIdx.x == 0) {
                int v;
                asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(job_addr) : "memory");
                s_jid = v;
            }
            __syncthreads();
            jid = s_jid;
            cluster_sync();  // rank 0 overwrites s_job only after everyone read it
        } else {
            jid = round;
            njobs = 1;
        }
        if (jid >= njobs) break;
        const ClusterJob j = queue ? jobs[jid] : one;
        if (j.dims == 3) {
            switch (j.radius) {
                case 1: run_job<3, 1>(j, smem, rank, csize); break;
                case 2: run_job<3, 2>(j, smem, rank, csize); break;
                case 3: run_job<3, 3>(j, smem, rank, csize); break;
                case 4: run_job<3, 4>(j, smem, rank, csize); break;
            }
        } else {
            switch (j.radius) {
                case 1: run_job<2, 1>(j, smem, rank, csize); break;
                case 2: run_job<2, 2>(j, smem, rank, csize); break;
                case 3: run_job<2, 3>(j, smem, rank, csize); break;
                case 4: run_job<2, 4>(j, smem, rank, csize); break;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
constexpr int kClusterSmemMax = 200 * 1024;

static long long slab_bytes(const ClusterJob &j, int csize, int tblock) {
    const int S = j.dims == 3 ? j.nz : j.ny;
    const long long slice_len = j.dims == 3 ? (long long)j.px * j.ny : j.px;
    const int H = (S + csize - 1) / csize;
    return 2LL * (H + 2 * tblock * j.radius) * slice_len * 4;
}

// The cluster sweeps read float4 chunks of rows with pitch px and number a
// plane's chunk columns with 32-bit integers.
bool cluster_shape_ok(int dims, int px, int ny, int radius) {
    return px % 4 == 0 && radius >= 1 && radius <= 4 &&
           (dims == 2 || (long long)(px / 4) * ny < (1LL << 31));
}

bool cluster_job_ok(int dims, int nx, int ny, int nz, int radius) {
    (void)nz;
    return cluster_shape_ok(dims, nx, ny, radius);
}

// Resident when the slab fits and every CTA that owns slices owns at least R
// (so each halo comes from one neighbour).
// The sweeps between halo exchanges: the largest of 4, 2, 1 (or of 8, 4,
// 2, 1 at most tmax when a tuning hint gives one) whose deeper halo still
// fits and is owned by a single neighbour.
static void plan_job(ClusterJob &j, int csize, int tmax = 0) {
    const int S = j.dims == 3 ? j.nz : j.ny;
    const int H = (S + csize - 1) / csize;
    const int last = S - ((S + H - 1) / H - 1) * H;
    j.resident = 0;
    j.tblock = 1;
    for (int tb : {8, 4, 2, 1}) {
        if (tmax > 0 ? tb > tmax : tb > 4) continue;
        const int ht = tb * j.radius;
        if (slab_bytes(j, csize, tb) + 128 <= kClusterSmemMax && H >= ht && last >= ht) {
            j.resident = 1;
            j.tblock = (csize == 1) ? 1 : tb;
            break;
        }
    }
}

// Function attributes of k_cluster (once per device, outside any capture).
static int ensure_cluster_attrs() {
    static bool done[64] = {false};
    const int d = current_device();
    if (d >= 0 && d < 64 && done[d]) return STENCIL_OK;
    ST_CUDA(cudaFuncSetAttribute(reinterpret_cast<const void *>(k_cluster),
                                 cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    ST_CUDA(cudaFuncSetAttribute(reinterpret_cast<const void *>(k_cluster),
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, kClusterSmemMax + 128));
    if (d >= 0 && d < 64) done[d] = true;
    return STENCIL_OK;
}

int cluster_size_for_device() {
    static int cached = 0;
    if (cached) return cached;
    int v = 0;
    ensure_cluster_attrs();
    for (int c : {16, 8}) {
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = c;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3(c);
        cfg.blockDim = dim3(kClusterThreads);
        cfg.dynamicSmemBytes = kClusterSmemMax + 128;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        if (cudaOccupancyMaxActiveClusters(&v, reinterpret_cast<const void *>(k_cluster), &cfg) ==
                cudaSuccess && v > 0) {
            cached = c;
            return c;
        }
        cudaGetLastError();
    }
    cached = 8;
    return cached;
}

// Launches `clusters` clusters over the jobs (already in device memory).
int launch_cluster_jobs(const ClusterJob *d_jobs, int njobs, unsigned *d_queue, int clusters,
                        int csize, cudaStream_t s) {
    ST_CUDA(cudaMemsetAsync(d_queue, 0, sizeof(unsigned), s));
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = csize;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(clusters * csize);
    cfg.blockDim = dim3(kClusterThreads);
    cfg.dynamicSmemBytes = kClusterSmemMax + 128;
    cfg.stream = s;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    ClusterJob none = {};
    ST_CUDA(cudaLaunchKernelEx(&cfg, k_cluster, none, d_jobs, njobs, d_queue));
    return STENCIL_OK;
}

int max_active_clusters(int csize) {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = csize;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(csize);
    cfg.blockDim = dim3(kClusterThreads);
    cfg.dynamicSmemBytes = kClusterSmemMax + 128;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int v = 0;
    if (cudaOccupancyMaxActiveClusters(&v, reinterpret_cast<const void *>(k_cluster), &cfg) !=
        cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return std::max(1, v);
}

ClusterJob make_job(const Geom &g, int dims, float *a, float *b, int iters, int csize,
                    int tmax = 0) {
    ClusterJob j;
    j.a = a;
    j.b = b;
    j.dims = dims;
    j.nx = g.nx;
    j.ny = g.ny;
    j.nz = dims == 3 ? g.nz : 1;
    j.radius = g.radius;
    j.iters = iters;
    j.legacy = g.legacy;
    j.px = (int)g.sy;
    plan_job(j, csize, tmax);
    return j;
}

size_t cluster_job_size() { return sizeof(ClusterJob); }

// Single grid on one cluster, all sweeps in one launch (queue-less mode).
int run_cluster(const Geom &g, int dims, float *a, float *b, int iters, cudaStream_t s,
                float **res) {
    if (!cluster_shape_ok(dims, (int)g.sy, g.ny, g.radius))
        return fail(STENCIL_EUNSUPPORTED,
                    "cluster engine needs nx %% 4 == 0, R <= 4 and (3-D) nx/4 * ny < 2^31");
    const int csize = cluster_size_for_device();
    ClusterJob j = make_job(g, dims, a, b, iters, csize);
    int rc = ensure_cluster_attrs();
    if (rc) return rc;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = csize;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(csize);
    cfg.blockDim = dim3(kClusterThreads);
    cfg.dynamicSmemBytes = kClusterSmemMax + 128;
    cfg.stream = s;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    const ClusterJob *none = nullptr;
    unsigned *noq = nullptr;
    ST_CUDA(cudaLaunchKernelEx(&cfg, k_cluster, j, none, 1, noq));
    note_launches("cluster", 1);
    if (res) *res = (iters & 1) ? b : a;
    return STENCIL_OK;
}

// Whether a single grid is better served by one cluster than by the
// full-GPU kernels: it fits in the cluster's shared memory.
bool cluster_resident(const Geom &g, int dims) {
    if (!cluster_shape_ok(dims, (int)g.sy, g.ny, g.radius)) return false;
    ClusterJob j = make_job(g, dims, nullptr, nullptr, 0, cluster_size_for_device());
    return j.resident != 0;
}



// ---------------------------------------------------------------------------
// Batch C ABI: a device job table + queue counter in a caller-provided
// workspace, one persistent launch (capturable in a CUDA graph).
// ---------------------------------------------------------------------------
namespace {

struct BatchHeader {
    unsigned queue;
    int njobs;
    int cluster_size;
    int clusters;
};

// A job too large for a cluster's shared memory: swept by the whole GPU
// after the cluster jobs (one cooperative launch per job: the persistent
// stream kernel for 3-D; for 2-D the temporally blocked engine where the grid
// fits one tile per SM, else the persistent rows kernel) instead of by one
// 16-SM cluster from L2/HBM (about twice the throughput on the 128-grid 3-D
// part of the benchmark batch).
struct StreamedJob {
    Geom g;
    float *a, *b;
    int iters;
    int dims;
    int temporal, tile_x, tile_y;  // tuning hints (0 = the library's choice)
};

// A job whose width is not a multiple of 4 (its rows are not 16-byte
// aligned): swept in a copy with the row pitch rounded up to 4 cells, in the
// caller's workspace, copied in before the batch's kernels and back after by
// k_stage (the table of these entries is in the workspace too).
struct StagedJob {
    float *ua, *ub;  // the caller's buffers
    float *sa, *sb;  // the pitched copies
    int nx, px;      // width and pitch in cells
    long long rows;  // rows of the grid (ny * nz)
    long long row0;  // rows of the entries before this one
};

// Copies every staged job's two buffers between the caller's rows (pitch nx)
// and the pitched copies (pitch px): to the copies when `in`, back otherwise.
// A warp owns a run of consecutive rows of the concatenated jobs (one search
// of the table per run) and copies a row with coalesced 4-byte accesses,
// four per lane in flight.  One launch for all jobs: a 2-D memcpy per buffer
// pays a fixed cost per row, about 1.2 s per batch for the 3-D grids of the
// 512-grid benchmark batch.
constexpr int kStageThreads = 256;
__global__ void __launch_bounds__(kStageThreads)
    k_stage(const StagedJob *__restrict__ t, int n, long long total_rows, int rows_per_warp, bool in) {
    const int lane = threadIdx.x & 31;
    const long long warp = ((long long)blockIdx.x * kStageThreads + threadIdx.x) >> 5;
    long long r = warp * rows_per_warp;
    const long long r_end = min(r + rows_per_warp, total_rows);
    if (r >= r_end) return;
    int lo = 0, hi = n - 1;  // the last entry with row0 <= r
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (t[mid].row0 <= r) lo = mid; else hi = mid - 1;
    }
    int j = lo;
    while (r < r_end) {
        const StagedJob e = t[j];
        const long long stop = min(r_end, e.row0 + e.rows);
        for (; r < stop; ++r) {
            const long long lr = r - e.row0;
            for (int h = 0; h < 2; ++h) {
                const float *src = in ? (h ? e.ub : e.ua) + lr * e.nx : (h ? e.sb : e.sa) + lr * e.px;
                float *dst = in ? (h ? e.sb : e.sa) + lr * e.px : (h ? e.ub : e.ua) + lr * e.nx;
                for (int x = lane; x < e.nx; x += 128) {
                    float v[4];
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if (x + 32 * k < e.nx) v[k] = __ldcs(src + x + 32 * k);
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if (x + 32 * k < e.nx) dst[x + 32 * k] = v[k];
                }
            }
        }
        ++j;
    }
}

// Up to kLanes - 1 extra streams with their fork and join events, owned by
// one prepared workspace: mid-size 3-D jobs run side by side, one lane on
// the caller's stream and the others here, each lane a queue of jobs on its
// share of the CTAs the device holds (a whole-GPU launch of one of them is
// latency-bound).
constexpr int kLanes = 8;
struct Lanes {
    cudaStream_t s[kLanes - 1] = {};
    cudaEvent_t fork = nullptr, join[kLanes - 1] = {};
    ~Lanes() {
        for (auto &e : join)
            if (e) cudaEventDestroy(e);
        if (fork) cudaEventDestroy(fork);
        for (auto &x : s)
            if (x) cudaStreamDestroy(x);
    }
};

struct BatchPlan {
    BatchHeader h;                    // the cluster part (njobs = cluster jobs)
    std::vector<StreamedJob> streamed;
    int nstaged = 0;                  // staged jobs (their table is in the workspace)
    long long staged_rows = 0;
    size_t stage_table = 0;           // workspace offset of the table
    // the whole-GPU jobs in phases, one after the other: a phase of one lane
    // runs its jobs in order on the whole GPU; a phase of n > 1 lanes runs
    // n queues side by side, each job with at most `ctas` CTAs
    struct Phase { int ctas; std::vector<std::vector<int>> queue; };
    std::vector<Phase> phases;
    std::shared_ptr<Lanes> lanes;     // set when some phase has two lanes or more
};

// Launch plan of each prepared workspace (set by prepare, read by launch).
std::mutex g_batch_mu;
std::vector<std::pair<const void *, BatchPlan>> g_batch;

void remember(const void *ws, const BatchPlan &h) {
    std::lock_guard<std::mutex> lock(g_batch_mu);
    for (auto &c : g_batch)
        if (c.first == ws) { c.second = h; return; }
    g_batch.emplace_back(ws, h);
}

bool recall(const void *ws, BatchPlan *h) {
    std::lock_guard<std::mutex> lock(g_batch_mu);
    for (auto &c : g_batch)
        if (c.first == ws) { *h = c.second; return true; }
    return false;
}

// 3-D jobs below this many cells (about 106^3) that do not fit a cluster's
// shared memory are swept by a cluster from L2, several jobs at a time: on
// the 512-grid batch 3.79 s, against 4.12 s with every such job on the whole
// GPU (thresholds 0.3 M / 0.7 M / 2.5 M cells: 4.04 / 3.85 / 3.81 s).  The
// environment variable STENCIL_BATCH_STREAM_MIN_CELLS_3D overrides it at
// prepare time.
#ifndef STENCIL_STREAM_MIN_CELLS_3D
#define STENCIL_STREAM_MIN_CELLS_3D 1200000
#endif
constexpr long long kStreamMinCells3d = STENCIL_STREAM_MIN_CELLS_3D;

// 3-D whole-GPU jobs below STENCIL_BATCH_LANE_MAX_CELLS cells (2^25, about
// 320^3) run side by side in STENCIL_BATCH_LANES lanes, each on that share of
// the device's CTAs, and 2-D ones below STENCIL_BATCH_LANE_MAX_CELLS_2D (2^30)
// in STENCIL_BATCH_LANES_2D lanes on the rows kernel; environment variables of
// the same names override them at prepare time (lanes 1 or cells 0 = never).
// GB300, the 512-grid benchmark batch: its 56 3-D whole-GPU jobs (R = 2,
// 106-256^3) 1.93 s alone, 1.64 s in 4 or 8 lanes; its 122 2-D ones
// (640-2048^2, R = 1) 1.14 s alone (the temporally blocked engine where the
// grid fits one tile per SM, else the rows kernel), 0.89 / 0.70 / 0.71 s in
// 2 / 4 / 8 lanes of the rows kernel (8 equal 1000^2 grids: 296 GCell/s alone,
// 559 in 4 lanes; 2048^2: 577 alone, 630 in 4 lanes, 711 in 2).
#ifndef STENCIL_BATCH_LANE_MAX_CELLS
#define STENCIL_BATCH_LANE_MAX_CELLS 33554432
#endif
#ifndef STENCIL_BATCH_LANES
#define STENCIL_BATCH_LANES 4
#endif
#ifndef STENCIL_BATCH_LANE_MAX_CELLS_2D
#define STENCIL_BATCH_LANE_MAX_CELLS_2D 1073741824
#endif
#ifndef STENCIL_BATCH_LANES_2D
#define STENCIL_BATCH_LANES_2D 4
#endif

long long env_cells(const char *name, long long dflt) {
    const char *e = std::getenv(name);
    if (e && *e) {
        char *end = nullptr;
        const long long v = std::strtoll(e, &end, 10);
        if (end && *end == 0 && v >= 0) return v;
    }
    return dflt;
}

// 3-D jobs swept by the stream kernel (not the temporally blocked one).
bool stream_job(const StreamedJob &j) {
    return j.dims == 3 && !(j.temporal >= 2 && !j.g.legacy && j.g.sy == j.g.nx && tb3d_supported(j.g));
}

long long job_cells(const StreamedJob &j) { return (long long)j.g.nx * j.g.ny * j.g.nz; }

// Orders the whole-GPU jobs into phases.  First every job that runs alone,
// in the given order; then, per kernel (radius, arithmetic, shape class: the
// grids' CTAs are then interchangeable on an SM, so all lanes' CTAs fit on
// the device at once), the mid-size 3-D stream jobs in lanes, each job to the
// lane with the least work so far, largest first (longest-processing-time
// scheduling; work = cells x sweeps).
int plan_phases(BatchPlan *plan) {
    auto lanes_env = [](const char *name, long long dflt) {
        return (int)std::min<long long>(kLanes, std::max<long long>(1, env_cells(name, dflt)));
    };
    const long long cap = env_cells("STENCIL_BATCH_LANE_MAX_CELLS", STENCIL_BATCH_LANE_MAX_CELLS);
    const long long cap2 = env_cells("STENCIL_BATCH_LANE_MAX_CELLS_2D", STENCIL_BATCH_LANE_MAX_CELLS_2D);
    const int lanes = lanes_env("STENCIL_BATCH_LANES", STENCIL_BATCH_LANES);
    const int lanes2 = lanes_env("STENCIL_BATCH_LANES_2D", STENCIL_BATCH_LANES_2D);
    const int n = (int)plan->streamed.size();
    auto work = [&](int i) { return (double)job_cells(plan->streamed[i]) * plan->streamed[i].iters; };
    auto laned = [&](int i) {
        const StreamedJob &j = plan->streamed[i];
        // a 2-D job with tuning hints runs alone on the engine they tune
        if (j.dims == 2)
            return lanes2 > 1 && job_cells(j) < cap2 && !j.temporal && !j.tile_x && !j.tile_y;
        return lanes > 1 && stream_job(j) && job_cells(j) < cap;
    };
    // kernel class of a laned job: 3-D by radius, arithmetic and shape
    // class, 2-D (the rows kernel) by radius
    auto kclass = [&](int i) {
        const StreamedJob &j = plan->streamed[i];
        if (j.dims == 2) return 20 + j.g.radius;
        return j.g.radius * 4 + (j.g.legacy ? 2 : 0) + (job_cells(j) >= (1LL << 25) ? 1 : 0);
    };
    plan->phases.clear();
    BatchPlan::Phase alone{0, {{}}};
    std::vector<std::vector<int>> byclass(25);
    for (int i = 0; i < n; ++i) {
        if (laned(i)) byclass[kclass(i)].push_back(i);
        else alone.queue[0].push_back(i);
    }
    for (auto &c : byclass)
        if (c.size() == 1) {  // nothing to run beside it
            alone.queue[0].push_back(c[0]);
            c.clear();
        }
    if (!alone.queue[0].empty()) plan->phases.push_back(alone);
    // A phase's launches take consecutive grid-barrier counters (a ring of
    // 256): at most 128 jobs per phase keeps the counters of lanes running at
    // once distinct.
    constexpr size_t kPhaseJobs = 128;
    std::vector<std::vector<int>> parts;
    for (auto &c : byclass) {
        if (c.empty()) continue;
        std::stable_sort(c.begin(), c.end(), [&](int x, int y) { return work(x) > work(y); });
        for (size_t k = 0; k < c.size(); k += kPhaseJobs)
            parts.emplace_back(c.begin() + k, c.begin() + std::min(c.size(), k + kPhaseJobs));
    }
    bool shared = false;
    for (auto &c : parts) {
        const StreamedJob &j0 = plan->streamed[c[0]];
        const int nl = std::min<int>(j0.dims == 2 ? lanes2 : lanes, (int)c.size());
        int ctas = 0;
        if (j0.dims == 2) {
            ctas = rows2d_capacity(j0.g);
        } else {
            int rc = stream3d_capacity(j0.g, &ctas);
            if (rc) return rc;
        }
        if (ctas < nl) {
            plan->phases.push_back({0, {c}});
            continue;
        }
        BatchPlan::Phase ph{ctas / nl, std::vector<std::vector<int>>(nl)};
        std::vector<double> load(nl, 0.0);
        for (int i : c) {
            const int l = (int)(std::min_element(load.begin(), load.end()) - load.begin());
            ph.queue[l].push_back(i);
            load[l] += work(i);
        }
        plan->phases.push_back(ph);
        shared = true;
    }
    if (shared) {
        auto ln = std::make_shared<Lanes>();
        ST_CUDA(cudaEventCreateWithFlags(&ln->fork, cudaEventDisableTiming));
        for (int k = 0; k < kLanes - 1; ++k) {
            ST_CUDA(cudaStreamCreateWithFlags(&ln->s[k], cudaStreamNonBlocking));
            ST_CUDA(cudaEventCreateWithFlags(&ln->join[k], cudaEventDisableTiming));
        }
        plan->lanes = ln;
    }
    return STENCIL_OK;
}

// One whole-GPU job on stream s.
int run_alone(const StreamedJob &j, cudaStream_t s) {
    if (!stream_job(j) && j.dims == 3) {
        // temporally blocked passes leave the result where the pass count
        // puts it; the batch keeps the ping-pong loop's place (d_u1 for an
        // even sweep count, d_u2 for an odd one)
        float *out = nullptr;
        int rc = run_tb3d(j.g, j.a, j.b, j.iters, j.temporal, s, &out);
        float *want = (j.iters & 1) ? j.b : j.a;
        if (!rc && out != want)
            ST_CUDA(cudaMemcpyAsync(want, out, (size_t)j.g.sz * j.g.nz * sizeof(float),
                                    cudaMemcpyDeviceToDevice, s));
        return rc;
    }
    if (j.dims == 3) return run_stream3d(j.g, j.a, j.b, j.iters, 0, 0, s, nullptr, 0, true);
    return tb2d_supported(j.g, 2)
               ? run_tb2d(j.g, j.a, j.b, j.iters, j.temporal, j.tile_x, j.tile_y, s, nullptr)
               : run_rows2d(j.g, j.a, j.b, j.iters, s, nullptr);
}

// The staged jobs' copies in (before the batch's kernels) or out (after).
int launch_stage(const BatchPlan &plan, const void *ws, bool in, cudaStream_t s) {
    const StagedJob *t = reinterpret_cast<const StagedJob *>(static_cast<const char *>(ws) + plan.stage_table);
    const long long rows = plan.staged_rows;
    const int warps_per_block = kStageThreads / 32;
    const long long max_warps = (long long)num_sms() * 8 * warps_per_block;
    const int per_warp = (int)std::max<long long>(1, (rows + max_warps - 1) / max_warps);
    const long long warps = (rows + per_warp - 1) / per_warp;
    const int blocks = (int)((warps + warps_per_block - 1) / warps_per_block);
    k_stage<<<blocks, kStageThreads, 0, s>>>(t, plan.nstaged, rows, per_warp, in);
    ST_CUDA(cudaGetLastError());
    return STENCIL_OK;
}

size_t batch_bytes(int njobs) {
    return ((sizeof(BatchHeader) + 255) & ~(size_t)255) + (size_t)njobs * sizeof(ClusterJob);
}

// Bytes of one staged buffer of a job (0 when its rows are 16-byte aligned).
size_t staged_bytes(const stencil_batch_job &b) {
    if (b.nx % 4 == 0 || b.nx <= 0 || b.ny <= 0) return 0;
    const size_t px = ((size_t)b.nx + 3) & ~(size_t)3;
    const size_t rows = (size_t)b.ny * (b.dims == 3 && b.nz > 0 ? (size_t)b.nz : 1);
    return (px * rows * sizeof(float) + 255) & ~(size_t)255;
}

// The job table, the table of staged jobs, then their copies (two per
// ragged job).
size_t batch_bytes_for(const stencil_batch_job *jobs, int njobs) {
    size_t n = (batch_bytes(njobs) + 255) & ~(size_t)255;
    size_t ragged = 0;
    for (int i = 0; i < njobs; ++i) ragged += staged_bytes(jobs[i]) > 0;
    n += (ragged * sizeof(StagedJob) + 255) & ~(size_t)255;
    for (int i = 0; i < njobs; ++i) n += 2 * staged_bytes(jobs[i]);
    return n;
}

}  // namespace

// The checks every batch job passes (either engine): valid parameters, two
// distinct 16-byte aligned buffers, radius <= 4, tuning fields in range.
int check_batch_job(const stencil_batch_job &b, int i, stencil_params *out) {
    stencil_params p;
    stencil_params_init(&p);
    p.dims = b.dims; p.nx = b.nx; p.ny = b.ny; p.nz = b.dims == 3 ? b.nz : 1;
    p.radius = b.radius; p.iterations = b.iterations; p.mode = b.mode;
    int rc = stencil_params_check(&p);
    if (rc) return fail(rc, "job %d: %s", i, stencil_last_error());
    if (!b.d_u1 || !b.d_u2 || b.d_u1 == b.d_u2 ||
        ((reinterpret_cast<uintptr_t>(b.d_u1) | reinterpret_cast<uintptr_t>(b.d_u2)) & 15))
        return fail(STENCIL_EINVAL, "job %d: two distinct 16-byte aligned buffers required", i);
    const int px = (b.nx + 3) & ~3;
    if (!cluster_job_ok(b.dims, px, b.ny, b.nz, b.radius))
        return fail(STENCIL_EUNSUPPORTED, "job %d: batch jobs need radius <= 4", i);
    if (b.temporal < 0 || b.tile_x < 0 || b.tile_y < 0 || (b.tile_x % 4) || b.team < 0 ||
        b.reserved[0] || b.reserved[1])
        return fail(STENCIL_EINVAL,
                    "job %d: temporal, tile_x, tile_y, team >= 0, tile_x %% 4 == 0, reserved zero", i);
    *out = p;
    return STENCIL_OK;
}

}  // namespace st

using namespace st;

extern "C" int stencil_batch_workspace_bytes(int njobs, size_t *bytes) {
    if (njobs < 0 || !bytes) return fail(STENCIL_EINVAL, "bad arguments");
    // enough for either engine: the one-launch engine's table with every job
    // 3-D (two tensor maps each)
    std::vector<stencil_batch_job> any(njobs);
    for (auto &j : any) { j = stencil_batch_job{}; j.dims = 3; j.nx = 4; j.ny = 1; }
    *bytes = std::max(batch_bytes(njobs), batch1_bytes_for(any.data(), njobs));
    return STENCIL_OK;
}

extern "C" int stencil_batch_workspace_bytes_for(const stencil_batch_job *jobs, int njobs,
                                                 size_t *bytes) {
    if (njobs < 0 || (njobs && !jobs) || !bytes) return fail(STENCIL_EINVAL, "bad arguments");
    *bytes = std::max(batch_bytes_for(jobs, njobs), batch1_bytes_for(jobs, njobs));
    return STENCIL_OK;
}

namespace st {
namespace {
// The engine STENCIL_BATCH_ENGINE_AUTO stands for: the environment variable
// STENCIL_BATCH_ENGINE ("phased" or "one_launch") read at prepare time, else
// the phased engine when some job carries tuning hints (only it uses them),
// else the one-launch engine (GB300, the 512-grid benchmark batch: 2.63 s in
// one launch against 2.68 s phased).
int batch_engine_auto(const stencil_batch_job *jobs, int njobs) {
    const char *e = std::getenv("STENCIL_BATCH_ENGINE");
    if (e && std::string(e) == "one_launch") return STENCIL_BATCH_ENGINE_ONE_LAUNCH;
    if (e && std::string(e) == "phased") return STENCIL_BATCH_ENGINE_PHASED;
    for (int i = 0; i < njobs; ++i)
        if (jobs[i].temporal || jobs[i].tile_x || jobs[i].tile_y) return STENCIL_BATCH_ENGINE_PHASED;
    return STENCIL_BATCH_ENGINE_ONE_LAUNCH;
}
}  // namespace
}  // namespace st

extern "C" int stencil_batch_prepare(const stencil_batch_job *jobs, int njobs, int cluster_size,
                                     void *d_workspace, size_t workspace_bytes,
                                     stencil_stream_t stream) {
    return stencil_batch_prepare_engine(jobs, njobs, STENCIL_BATCH_ENGINE_AUTO, cluster_size,
                                        d_workspace, workspace_bytes, stream);
}

extern "C" int stencil_batch_prepare_engine(const stencil_batch_job *jobs, int njobs, int engine,
                                            int cluster_size, void *d_workspace,
                                            size_t workspace_bytes, stencil_stream_t stream) {
    if (njobs < 0 || (njobs && !jobs) || !d_workspace)
        return fail(STENCIL_EINVAL, "bad arguments");
    if (engine < STENCIL_BATCH_ENGINE_AUTO || engine > STENCIL_BATCH_ENGINE_ONE_LAUNCH)
        return fail(STENCIL_EINVAL, "unknown batch engine %d", engine);
    if (engine == STENCIL_BATCH_ENGINE_AUTO) engine = batch_engine_auto(jobs, njobs);
    if (engine == STENCIL_BATCH_ENGINE_ONE_LAUNCH) {
        if (reinterpret_cast<uintptr_t>(d_workspace) & 255)
            return fail(STENCIL_EINVAL, "workspace must be 256-byte aligned");
        stencil_batch_forget(d_workspace);
        return batch1_prepare(jobs, njobs, d_workspace, workspace_bytes,
                              reinterpret_cast<cudaStream_t>(stream));
    }
    batch1_forget(d_workspace);
    if (workspace_bytes < batch_bytes_for(jobs, njobs))
        return fail(STENCIL_EINVAL,
                    "workspace too small: %zu < %zu bytes (stencil_batch_workspace_bytes_for "
                    "counts the copies of jobs whose nx is not a multiple of 4)",
                    workspace_bytes, batch_bytes_for(jobs, njobs));
    if (reinterpret_cast<uintptr_t>(d_workspace) & 255)
        return fail(STENCIL_EINVAL, "workspace must be 256-byte aligned");
    if (cluster_size < 0 || cluster_size > 16 || (cluster_size & (cluster_size - 1)))
        return fail(STENCIL_EINVAL, "cluster_size must be 0 or a power of two <= 16");
    int rc0 = ensure_cluster_attrs();
    if (rc0) return rc0;
    const int csize = cluster_size ? cluster_size : cluster_size_for_device();
    std::vector<ClusterJob> table;
    std::vector<double> work;
    BatchPlan plan;
    std::vector<StagedJob> staged;
    int ragged = 0;
    for (int i = 0; i < njobs; ++i) ragged += staged_bytes(jobs[i]) > 0;
    plan.stage_table = (batch_bytes(njobs) + 255) & ~(size_t)255;
    size_t stage_off = plan.stage_table + (((size_t)ragged * sizeof(StagedJob) + 255) & ~(size_t)255);
    table.reserve(njobs);
    const long long stream_min3d = env_cells("STENCIL_BATCH_STREAM_MIN_CELLS_3D", kStreamMinCells3d);
    for (int i = 0; i < njobs; ++i) {
        const stencil_batch_job &b = jobs[i];
        stencil_params p;
        int rc = check_batch_job(b, i, &p);
        if (rc) return rc;
        const int px = (b.nx + 3) & ~3;
        Geom g = make_geom(p);
        float *ga = b.d_u1, *gb = b.d_u2;
        if (px != b.nx) {
            // swept in pitched copies in the workspace
            const size_t sb = staged_bytes(b);
            StagedJob st;
            st.ua = b.d_u1;
            st.ub = b.d_u2;
            st.sa = reinterpret_cast<float *>(static_cast<char *>(d_workspace) + stage_off);
            st.sb = reinterpret_cast<float *>(static_cast<char *>(d_workspace) + stage_off + sb);
            st.nx = b.nx;
            st.px = px;
            st.rows = (long long)b.ny * (b.dims == 3 ? b.nz : 1);
            st.row0 = plan.staged_rows;
            plan.staged_rows += st.rows;
            stage_off += 2 * sb;
            staged.push_back(st);
            ga = st.sa;
            gb = st.sb;
            g.sy = px;
            g.sz = (long long)px * b.ny;
        }
        ClusterJob j = make_job(g, p.dims, ga, gb, b.iterations, csize, b.temporal);
        // small non-resident 3-D grids stay on clusters, many at a time: a
        // whole-GPU launch of one of them is latency-bound
        const bool big3d = (long long)cell_count(p) >= stream_min3d;
        if (!j.resident && ((p.dims == 3 && big3d && stream3d_supported(g)) ||
                            (p.dims == 2 && rows2d_supported(g, 2)))) {
            plan.streamed.push_back({g, ga, gb, b.iterations, p.dims, b.temporal, b.tile_x,
                                     b.tile_y});
            continue;
        }
        table.push_back(j);
        work.push_back((double)cell_count(p) * b.iterations);
    }
    plan.nstaged = (int)staged.size();
    int rcg = plan_phases(&plan);
    if (rcg) return rcg;
    const int nc = (int)table.size();
    // Largest job first: the queue hands them out in this order.
    std::vector<int> order(nc);
    for (int i = 0; i < nc; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return work[x] > work[y]; });
    std::vector<ClusterJob> sorted(nc);
    for (int i = 0; i < nc; ++i) sorted[i] = table[order[i]];
    BatchHeader &h = plan.h;
    h.queue = 0;
    h.njobs = nc;
    h.cluster_size = csize;
    h.clusters = max_active_clusters(csize);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const size_t hb = (sizeof(BatchHeader) + 255) & ~(size_t)255;
    char *ws = static_cast<char *>(d_workspace);
    ST_CUDA(cudaMemcpyAsync(ws, &h, sizeof h, cudaMemcpyHostToDevice, s));
    if (nc)
        ST_CUDA(cudaMemcpyAsync(ws + hb, sorted.data(), nc * sizeof(ClusterJob),
                                cudaMemcpyHostToDevice, s));
    if (!staged.empty())
        ST_CUDA(cudaMemcpyAsync(ws + plan.stage_table, staged.data(),
                                staged.size() * sizeof(StagedJob), cudaMemcpyHostToDevice, s));
    ST_CUDA(cudaStreamSynchronize(s));
    remember(d_workspace, plan);
    return STENCIL_OK;
}

extern "C" int stencil_batch_launch(const void *d_workspace, stencil_stream_t stream) {
    if (!d_workspace) return fail(STENCIL_EINVAL, "null workspace");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (batch1_known(d_workspace)) return batch1_launch(d_workspace, s);
    BatchPlan plan;
    if (!recall(d_workspace, &plan))
        return fail(STENCIL_EINVAL, "workspace was not prepared by stencil_batch_prepare");
    const BatchHeader &h = plan.h;
    if (plan.nstaged) {
        int rc = launch_stage(plan, d_workspace, true, s);
        if (rc) return rc;
    }
    if (h.njobs) {
        const size_t hb = (sizeof(BatchHeader) + 255) & ~(size_t)255;
        const ClusterJob *table = reinterpret_cast<const ClusterJob *>(static_cast<const char *>(d_workspace) + hb);
        unsigned *queue = reinterpret_cast<unsigned *>(const_cast<void *>(d_workspace));
        int rc = launch_cluster_jobs(table, h.njobs, queue, std::min(h.clusters, h.njobs), h.cluster_size, s);
        if (rc) return rc;
    }
    for (const BatchPlan::Phase &ph : plan.phases) {
        if (ph.queue.size() == 1) {
            for (int i : ph.queue[0]) {
                int rc = run_alone(plan.streamed[i], s);
                if (rc) return rc;
            }
            continue;
        }
        // lanes side by side: the first on the caller's stream, the others
        // on the workspace's streams, forked from and joined back into it
        const Lanes &ln = *plan.lanes;
        const int nl = (int)ph.queue.size();
        ST_CUDA(cudaEventRecord(ln.fork, s));
        int rc = STENCIL_OK;
        for (int l = 0; l < nl; ++l) {
            cudaStream_t sl = l ? ln.s[l - 1] : s;
            if (l) ST_CUDA(cudaStreamWaitEvent(sl, ln.fork, 0));
            for (int i : ph.queue[l]) {
                const StreamedJob &x = plan.streamed[i];
                if (!rc)
                    rc = x.dims == 2 ? run_rows2d(x.g, x.a, x.b, x.iters, sl, nullptr, ph.ctas)
                                     : run_stream3d(x.g, x.a, x.b, x.iters, 0, 0, sl, nullptr, 0, true, ph.ctas);
            }
        }
        // joined even after a failure, so that a capture stays well formed
        for (int l = 1; l < nl; ++l) {
            ST_CUDA(cudaEventRecord(ln.join[l - 1], ln.s[l - 1]));
            ST_CUDA(cudaStreamWaitEvent(s, ln.join[l - 1], 0));
        }
        if (rc) return rc;
    }
    if (plan.nstaged) {
        int rc = launch_stage(plan, d_workspace, false, s);
        if (rc) return rc;
    }
    return STENCIL_OK;
}

extern "C" int stencil_batch_plan(const void *d_workspace, int *cluster_jobs, int *whole_gpu_jobs) {
    if (!d_workspace || !cluster_jobs || !whole_gpu_jobs) return fail(STENCIL_EINVAL, "null argument");
    if (batch1_known(d_workspace)) {
        *cluster_jobs = *whole_gpu_jobs = 0;
        return STENCIL_OK;
    }
    BatchPlan plan;
    if (!recall(d_workspace, &plan))
        return fail(STENCIL_EINVAL, "workspace was not prepared by stencil_batch_prepare");
    *cluster_jobs = plan.h.njobs;
    *whole_gpu_jobs = (int)plan.streamed.size();
    return STENCIL_OK;
}

extern "C" int stencil_batch_side_by_side(const void *d_workspace, int *groups, int *jobs) {
    if (!d_workspace || !groups || !jobs) return fail(STENCIL_EINVAL, "null argument");
    *groups = *jobs = 0;
    if (batch1_known(d_workspace)) return STENCIL_OK;
    BatchPlan plan;
    if (!recall(d_workspace, &plan))
        return fail(STENCIL_EINVAL, "workspace was not prepared by stencil_batch_prepare");
    for (const BatchPlan::Phase &ph : plan.phases)
        if (ph.queue.size() > 1) {
            ++*groups;
            for (const auto &q : ph.queue) *jobs += (int)q.size();
        }
    return STENCIL_OK;
}

extern "C" int stencil_batch_launches(const void *d_workspace, int *kernel_launches) {
    if (!d_workspace || !kernel_launches) return fail(STENCIL_EINVAL, "null argument");
    if (batch1_known(d_workspace)) {
        *kernel_launches = batch1_launches(d_workspace);
        return STENCIL_OK;
    }
    BatchPlan plan;
    if (!recall(d_workspace, &plan))
        return fail(STENCIL_EINVAL, "workspace was not prepared by stencil_batch_prepare");
    *kernel_launches = (plan.h.njobs ? 1 : 0) + (int)plan.streamed.size() + (plan.nstaged ? 2 : 0);
    return STENCIL_OK;
}

extern "C" int stencil_batch_teams(const void *d_workspace, int *tiers, int *team_sizes,
                                   int *tier_jobs, int max_tiers) {
    if (!d_workspace || !tiers) return fail(STENCIL_EINVAL, "null argument");
    if (!batch1_known(d_workspace)) {
        *tiers = 0;
        return STENCIL_OK;
    }
    return batch1_teams(d_workspace, tiers, team_sizes, tier_jobs, max_tiers);
}

extern "C" int stencil_batch_forget(const void *d_workspace) {
    batch1_forget(d_workspace);
    std::lock_guard<std::mutex> lock(g_batch_mu);
    for (size_t i = 0; i < g_batch.size(); ++i)
        if (g_batch[i].first == d_workspace) {
            g_batch.erase(g_batch.begin() + i);
            break;
        }
    return STENCIL_OK;
}

// rows_body.cuh -- one sweep of a 2-D grid by register-queue chunk columns,
// the per-CTA part of the persistent 2-D rows kernel (k_rows2d.cu) and of the
// one-launch batch kernel (k_batch1.cu).
//
// A thread owns one float4 chunk column of a block of hb rows: it keeps the
// column's rows j-R .. j+R in a register queue (one new 16-byte load per
// row, the smem_register idea of src/stencils.cu:71-83 on registers) and
// loads the chunks left and right of its own for the x-neighbours, so a
// 4-cell update costs three 16-byte loads at any R <= 4.  Items (chunk
// column, row block) are spread over the nctas CTAs that share the grid with
// a grid stride; consecutive threads take consecutive chunk columns, so a
// warp's loads and stores are contiguous 512-byte segments.  Loads are
// ld.global.cg (L2) or, with L1, plain L1-cached loads: a buffer is rewritten
// every other sweep inside one launch, and the plain form relies on every
// read of another CTA's writes following an acquire at GPU scope and a CTA
// barrier (then weak loads observe those writes).  Every cell keeps the
// reference's summation order (axis i offsets -R..-1, +1..+R, then axis j,
// from +0) and division; cells outside the update region are never written.
#pragma once

#include "common.cuh"

namespace st {

// One sweep src -> dst of a 2-D grid (g.sy: the row pitch, a multiple of 4;
// the chunk columns cover it) by CTA `cta` of the nctas CTAs of NT threads
// that share it; hb rows per block, nblk blocks.
template <int R, int NT, bool L1 = false>
__device__ __forceinline__ void rows2d_sweep(const float *src, float *dst, const Geom g, int hb,
                                             int nblk, unsigned cta, unsigned nctas) {
    // L1: plain (L1-cached) loads instead of ld.global.cg (see rows2d_sweep_d)
    auto rows_ld4 = [](const float *p) {
        if constexpr (L1) return *reinterpret_cast<const float4 *>(p);
        else return __ldcg(reinterpret_cast<const float4 *>(p));
    };
    constexpr int C = 4 * R;
    constexpr int RA = (R + 3) & ~3;  // x halo in whole chunks (R <= 4: one chunk)
    static_assert(RA == 4, "one neighbour chunk per side");
    // nx: the width (update region x < nx - R); px: the row pitch
    const int nx = g.nx, ny = g.ny, px = (int)g.sy, nch = px >> 2;
    const int items = nch * nblk;
    for (int it = (int)(cta * NT + threadIdx.x); it < items; it += (int)(nctas * NT)) {
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
}

// The same sweep with the loads of the next D rows in flight (D = 1 is
// rows2d_sweep), for kernels with fewer resident warps per SM than the rows
// kernel's two 16-warp CTAs.  Same cells, same arithmetic.
template <int R, int NT, int D, bool L1 = false>
__device__ __forceinline__ void rows2d_sweep_d(const float *src, float *dst, const Geom g, int hb,
                                               int nblk, unsigned cta, unsigned nctas) {
    // L1: plain loads (cached in L1) instead of ld.global.cg.  Correct where
    // every read of data written by other CTAs in this launch follows an
    // acquire at GPU scope and a CTA barrier (weak loads that follow them
    // observe those writes in the PTX memory model).
    auto rows_ld4 = [](const float *p) {
        if constexpr (L1) return *reinterpret_cast<const float4 *>(p);
        else return __ldcg(reinterpret_cast<const float4 *>(p));
    };
    constexpr int C = 4 * R;
    const int nx = g.nx, ny = g.ny, px = (int)g.sy, nch = px >> 2;
    const int items = nch * nblk;
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int it = (int)(cta * NT + threadIdx.x); it < items; it += (int)(nctas * NT)) {
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
        // row j0+d's new queue entry (row j0+d+R) and x-neighbour chunks
        float4 pq[D], pl[D], pr[D];
#pragma unroll
        for (int d = 0; d < D; ++d) {
            pq[d] = pl[d] = pr[d] = z4;
            if (j0 + d < j1) {
                const float *row = col + (long long)(j0 + d) * px;
                pq[d] = rows_ld4(col + (long long)(j0 + d + R) * px);
                if (c > 0) pl[d] = rows_ld4(row - 4);
                if (c + 1 < nch) pr[d] = rows_ld4(row + 4);
            }
        }
        for (int j = j0; j < j1; ++j) {
            q[2 * R] = pq[0];
            const float4 l4 = pl[0], r4 = pr[0];
#pragma unroll
            for (int d = 0; d + 1 < D; ++d) {
                pq[d] = pq[d + 1];
                pl[d] = pl[d + 1];
                pr[d] = pr[d + 1];
            }
            if (j + D < j1) {
                const float *row = col + (long long)(j + D) * px;
                pq[D - 1] = rows_ld4(col + (long long)(j + D + R) * px);
                if (c > 0) pl[D - 1] = rows_ld4(row - 4);
                if (c + 1 < nch) pr[D - 1] = rows_ld4(row + 4);
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
}

}  // namespace st

// k_base.cu -- one sweep per launch, neighbours through L1/L2 ("base" role,
// src/stencil_kernel_base.cu:5-65).
//
// k_base_vec: each thread owns `cf` float4 chunks (4 consecutive cells) of one
// row, strided by blockDim.x chunks so that a warp's loads and stores are
// contiguous 512-byte segments.  The x-neighbours come from the float4 chunks
// left and right of the thread's own (16-byte aligned loads), the y/z
// neighbours from aligned float4 loads of the rows/planes at +-d.  Requires
// nx % 4 == 0 and 16-byte aligned buffers.
//
// k_base_any: one thread per cell, runtime radius; serves every shape the
// vector kernel does not (nx % 4 != 0, radii without an instantiation).
#include "host.hpp"

namespace st {

template <int D, int R>
__global__ void __launch_bounds__(1024)
    k_base_vec(const float *__restrict__ src, float *__restrict__ dst, Geom g, int cf) {
    constexpr int RA = (R + 3) & ~3;  // x halo rounded up to whole float4 chunks
    constexpr int W = 4 + 2 * RA;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = (D == 3) ? (int)(blockIdx.z * blockDim.z + threadIdx.z) : 0;
    if (!in_range(j, g.ny, R)) return;
    if (D == 3 && !in_range(k, g.nz, R)) return;
    const int nchunk = g.nx >> 2;
    const long long row = (long long)j * g.sy + (long long)k * g.sz;
    const float4 *srow = reinterpret_cast<const float4 *>(src + row);
    const int c0 = blockIdx.x * blockDim.x * cf + threadIdx.x;
    for (int u = 0; u < cf; ++u) {
        const int c = c0 + u * blockDim.x;
        if (c >= nchunk) break;
        const int x0 = c * 4;
        if (x0 + 3 < R || x0 >= g.nx - R) continue;
        float w[W];
#pragma unroll
        for (int q = 0; q < W / 4; ++q) {
            const int cc = c - RA / 4 + q;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (cc >= 0 && cc < nchunk) v = __ldg(srow + cc);
            w[4 * q + 0] = v.x; w[4 * q + 1] = v.y; w[4 * q + 2] = v.z; w[4 * q + 3] = v.w;
        }
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        // axis i
#pragma unroll
        for (int o = -R; o <= R; ++o) {
            if (o == 0) continue;
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[e] += w[RA + e + o];
        }
        // axis j
#pragma unroll
        for (int o = -R; o <= R; ++o) {
            if (o == 0) continue;
            const float4 v = __ldg(reinterpret_cast<const float4 *>(src + row + o * g.sy) + c);
            acc[0] += v.x; acc[1] += v.y; acc[2] += v.z; acc[3] += v.w;
        }
        // axis k
        if (D == 3) {
#pragma unroll
            for (int o = -R; o <= R; ++o) {
                if (o == 0) continue;
                const float4 v =
                    __ldg(reinterpret_cast<const float4 *>(src + row + o * g.sz) + c);
                acc[0] += v.x; acc[1] += v.y; acc[2] += v.z; acc[3] += v.w;
            }
        }
        float out[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) out[e] = star_finish<D, R>(acc[e], w[RA + e], g.legacy);
        float *drow = dst + row;
        if (x0 >= R && x0 + 3 < g.nx - R) {
            *reinterpret_cast<float4 *>(drow + x0) = make_float4(out[0], out[1], out[2], out[3]);
        } else {
#pragma unroll
            for (int e = 0; e < 4; ++e)
                if (in_range(x0 + e, g.nx, R)) drow[x0 + e] = out[e];
        }
    }
}

template <int D>
__global__ void __launch_bounds__(1024)
    k_base_any(const float *__restrict__ src, float *__restrict__ dst, Geom g) {
    const int R = g.radius;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = (D == 3) ? (int)(blockIdx.z * blockDim.z + threadIdx.z) : 0;
    if (!in_range(i, g.nx, R) || !in_range(j, g.ny, R)) return;
    if (D == 3 && !in_range(k, g.nz, R)) return;
    const long long idx = i + (long long)j * g.sy + (long long)k * g.sz;
    float acc = 0.0f;
    for (int o = -R; o <= R; ++o)
        if (o) acc += src[idx + o];
    for (int o = -R; o <= R; ++o)
        if (o) acc += src[idx + o * g.sy];
    if (D == 3)
        for (int o = -R; o <= R; ++o)
            if (o) acc += src[idx + o * g.sz];
    dst[idx] = star_finish_rt(acc, (float)(2 * D * R), src[idx], g.legacy);
}

namespace {

using VecFn = void (*)(const float *, float *, Geom, int);

template <int D>
VecFn vec_kernel(int r) {
    switch (r) {
        case 1: return k_base_vec<D, 1>;
        case 2: return k_base_vec<D, 2>;
        case 3: return k_base_vec<D, 3>;
        case 4: return k_base_vec<D, 4>;
        case 6: return k_base_vec<D, 6>;
        case 8: return k_base_vec<D, 8>;
        case 16: return k_base_vec<D, 16>;
        default: return nullptr;
    }
}

bool grid_ok(dim3 grid) { return grid.y <= 65535u && grid.z <= 65535u && grid.x > 0; }

}  // namespace

// The kernel launch_base_sweep runs for this grid on 16-byte aligned buffers.
const void *base_kernel_ptr(const Geom &g, int dims) {
    VecFn fn = g.nx % 4 == 0 ? (dims == 3 ? vec_kernel<3>(g.radius) : vec_kernel<2>(g.radius)) : nullptr;
    if (fn) return reinterpret_cast<const void *>(fn);
    return dims == 3 ? reinterpret_cast<const void *>(k_base_any<3>)
                     : reinterpret_cast<const void *>(k_base_any<2>);
}

int launch_base_sweep(const Geom &g, int dims, const float *src, float *dst, int bx, int by,
                      int bz, int cf, cudaStream_t s) {
    if (bx <= 0) bx = 32;
    if (by <= 0) by = dims == 3 ? 4 : 8;
    if (bz <= 0 || dims == 2) bz = 1;
    if ((long long)bx * by * bz > 1024) return fail(STENCIL_EINVAL, "block %dx%dx%d exceeds 1024 threads", bx, by, bz);
    const bool aligned = ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15) == 0;
    VecFn fn = (g.nx % 4 == 0 && aligned)
                   ? (dims == 3 ? vec_kernel<3>(g.radius) : vec_kernel<2>(g.radius))
                   : nullptr;
    if (fn) {
        const int chunks = g.nx / 4;
        cf = cf < 4 ? 1 : cf / 4;  // cells per thread -> float4 chunks per thread
        dim3 block(bx, by, bz);
        dim3 grid((chunks + bx * cf - 1) / (bx * cf), (g.ny + by - 1) / by,
                  dims == 3 ? (g.nz + bz - 1) / bz : 1);
        if (!grid_ok(grid)) return fail(STENCIL_EINVAL, "grid too large for block shape");
        fn<<<grid, block, 0, s>>>(src, dst, g, cf);
    } else {
        dim3 block(bx * 4 > 1024 / (by * bz) ? bx : bx * 4, by, bz);
        if ((long long)block.x * by * bz > 1024) block.x = bx;
        dim3 grid((g.nx + block.x - 1) / block.x, (g.ny + by - 1) / by,
                  dims == 3 ? (g.nz + bz - 1) / bz : 1);
        if (!grid_ok(grid)) return fail(STENCIL_EINVAL, "grid too large for block shape");
        if (dims == 3) k_base_any<3><<<grid, block, 0, s>>>(src, dst, g);
        else k_base_any<2><<<grid, block, 0, s>>>(src, dst, g);
    }
    return cuda_fail(cudaGetLastError(), "base sweep launch");
}

}  // namespace st

// k_util.cu -- whole-grid helper kernels: seeded initial states, border copy,
// and the residual norm (FP64 sums).
#include <algorithm>

#include "host.hpp"

namespace st {

__device__ unsigned g_device_status = 0;

__global__ void k_init_uniform(float *__restrict__ u, size_t count, uint64_t seed) {
    const uint64_t base = mix64(seed);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count;
         i += (size_t)gridDim.x * blockDim.x) {
        const uint64_t z = mix64(base + 0x9E3779B97F4A7C15ull * (i + 1));
        u[i] = (float)(z >> 40) * (1.0f / 16777216.0f);
    }
}

// include/stencil_initializer.h:6-52: outermost layer 1, else 0.
__global__ void k_init_reference(float *__restrict__ u, Geom g, int dims) {
    const size_t n = (size_t)g.nx * g.ny * (dims == 3 ? g.nz : 1);
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(idx % g.nx);
        const int j = (int)((idx / g.nx) % g.ny);
        const int k = (int)(idx / ((size_t)g.nx * g.ny));
        const bool edge = i == 0 || i == g.nx - 1 || j == 0 || j == g.ny - 1 ||
                          (dims == 3 && (k == 0 || k == g.nz - 1));
        u[idx] = edge ? 1.0f : 0.0f;
    }
}

// Copies cells outside the update region.  One thread per (row, plane) walks
// the row's border cells; rows outside the update region are copied whole.
__global__ void k_copy_border(const float *__restrict__ src, float *__restrict__ dst, Geom g,
                              int dims) {
    const int R = g.radius;
    const long long rows = (long long)g.ny * (dims == 3 ? g.nz : 1);
    for (long long r = blockIdx.x; r < rows; r += gridDim.x) {
        const int j = (int)(r % g.ny), k = (int)(r / g.ny);
        const long long base = (long long)j * g.sy + (long long)k * g.sz;
        const bool whole = !in_range(j, g.ny, R) || (dims == 3 && !in_range(k, g.nz, R));
        if (whole) {
            for (int i = threadIdx.x; i < g.nx; i += blockDim.x) dst[base + i] = src[base + i];
        } else {
            for (int i = threadIdx.x; i < 2 * R; i += blockDim.x) {
                const int x = i < R ? i : g.nx - 2 * R + i;
                dst[base + x] = src[base + x];
            }
        }
    }
}

// Residual of the JACOBI steady state.  Per update-region cell, in FP32:
// d = sum over the 2DR axis neighbours of (neighbour - centre) (= 2DR r, with
// r = (sum of neighbours)/(2DR) - u; the differences are exact wherever
// neighbour and centre are within a factor of two, so r keeps its relative
// accuracy as it shrinks, unlike sum/(2DR) - u), and bsum = sum of the border
// neighbours.  FP64 only for the reduction: stage 1 writes one (sum d^2,
// sum bsum^2) pair per block, stage 2 adds the pairs in a fixed order (the
// result does not depend on scheduling) and divides by (2DR)^2.  One warp per
// row of the update region (rows handed out round-robin), lanes along x.
constexpr int kResidBlocks = 1024;
constexpr int kResidThreads = 256;

__device__ __forceinline__ void block_sum2(double &a, double &b, double *sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { sh[2 * w] = a; sh[2 * w + 1] = b; }
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        a = l < nw ? sh[2 * l] : 0.0;
        b = l < nw ? sh[2 * l + 1] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_down_sync(0xffffffffu, a, o);
            b += __shfl_down_sync(0xffffffffu, b, o);
        }
    }
}

// Adds d^2 to the unevaluated FP32 pair (s + cs): the exact error of the
// square (fma) and of the addition (TwoSum, Knuth) go into cs, so the pair
// carries the sum to about FP32^2 precision without FP64 arithmetic per cell
// (GB300's FP64 rate would bind the kernel).  Explicit roundings: nothing is
// contracted into fused operations.
__device__ __forceinline__ void acc_square(float d, float &s, float &cs) {
    const float p = __fmul_rn(d, d);
    const float pe = fmaf(d, d, -p);
    const float t = __fadd_rn(s, p);
    const float z = __fsub_rn(t, s);
    cs = __fadd_rn(cs, __fadd_rn(__fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z)), pe));
    s = t;
}

// Any radius and nx: one lane per cell of a row.
__global__ void __launch_bounds__(kResidThreads)
    k_residual_partial_any(const float *__restrict__ u, Geom g, int dims, double *__restrict__ part) {
    __shared__ double sh[2 * (kResidThreads / 32)];
    const int R = g.radius;
    const int ry = g.ny - 2 * R, nrows = ry * (dims == 3 ? g.nz - 2 * R : 1);
    const int wpb = blockDim.x >> 5, lane = threadIdx.x & 31;
    double bb = 0.0;
    float s = 0.0f, cs = 0.0f;
    for (int q = blockIdx.x * wpb + (threadIdx.x >> 5); q < nrows; q += gridDim.x * wpb) {
        const int j = R + q % ry, k = dims == 3 ? R + q / ry : 0;
        const long long base = (long long)j * g.sy + (long long)k * g.sz;
        // rows whose y or z neighbours reach the border band
        const bool near_yz = j < 2 * R || j >= g.ny - 2 * R ||
                             (dims == 3 && (k < 2 * R || k >= g.nz - 2 * R));
        for (int i = R + lane; i < g.nx - R; i += 32) {
            const long long idx = base + i;
            const float c = u[idx];
            float d = 0.0f, bs = 0.0f;
            for (int o = -R; o <= R; ++o) {
                if (!o) continue;
                const float v = u[idx + o];
                d += v - c;
                if (!in_range(i + o, g.nx, R)) bs += v;
            }
            for (int o = -R; o <= R; ++o) {
                if (!o) continue;
                const float v = u[idx + o * g.sy];
                d += v - c;
                if (near_yz && !in_range(j + o, g.ny, R)) bs += v;
            }
            if (dims == 3)
                for (int o = -R; o <= R; ++o) {
                    if (!o) continue;
                    const float v = u[idx + o * g.sz];
                    d += v - c;
                    if (near_yz && !in_range(k + o, g.nz, R)) bs += v;
                }
            acc_square(d, s, cs);
            if (bs != 0.0f) bb = fma((double)bs, (double)bs, bb);
        }
    }
    double rr = (double)s + (double)cs;
    block_sum2(rr, bb, sh);
    if (threadIdx.x == 0) { part[2 * blockIdx.x] = rr; part[2 * blockIdx.x + 1] = bb; }
}

// nx % 4 == 0 and R <= 4: a lane owns 4-cell chunks of its row and issues
// every neighbour load of a chunk (3 + 2R or 3 + 4R float4) before using any.
template <int D, int R>
__global__ void __launch_bounds__(kResidThreads)
    k_residual_partial_vec(const float *__restrict__ u, Geom g, double *__restrict__ part) {
    __shared__ double sh[2 * (kResidThreads / 32)];
    const int ry = g.ny - 2 * R, nrows = ry * (D == 3 ? g.nz - 2 * R : 1);
    const int nch = g.nx >> 2;
    const int wpb = blockDim.x >> 5, lane = threadIdx.x & 31;
    double bb = 0.0;
    float s = 0.0f, cs = 0.0f;
    for (int q = blockIdx.x * wpb + (threadIdx.x >> 5); q < nrows; q += gridDim.x * wpb) {
        const int j = R + q % ry, k = D == 3 ? R + q / ry : 0;
        const float *row = u + (long long)j * g.sy + (long long)k * g.sz;
        const bool near_yz = j < 2 * R || j >= g.ny - 2 * R ||
                             (D == 3 && (k < 2 * R || k >= g.nz - 2 * R));
        for (int cc = lane; cc < nch; cc += 32) {
            const int x0 = 4 * cc;
            if (x0 + 3 < R || x0 >= g.nx - R) continue;
            const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
            const float4 l4 = cc > 0 ? *reinterpret_cast<const float4 *>(row + x0 - 4) : z4;
            const float4 m4 = *reinterpret_cast<const float4 *>(row + x0);
            const float4 r4 = cc + 1 < nch ? *reinterpret_cast<const float4 *>(row + x0 + 4) : z4;
            float4 yz[(D == 3 ? 4 : 2) * R];
#pragma unroll
            for (int o = 1; o <= R; ++o) {
                yz[2 * (o - 1)] = *reinterpret_cast<const float4 *>(row + x0 - o * g.sy);
                yz[2 * (o - 1) + 1] = *reinterpret_cast<const float4 *>(row + x0 + o * g.sy);
                if (D == 3) {
                    yz[2 * R + 2 * (o - 1)] = *reinterpret_cast<const float4 *>(row + x0 - o * g.sz);
                    yz[2 * R + 2 * (o - 1) + 1] = *reinterpret_cast<const float4 *>(row + x0 + o * g.sz);
                }
            }
            const float w[12] = {l4.x, l4.y, l4.z, l4.w, m4.x, m4.y, m4.z, m4.w, r4.x, r4.y, r4.z, r4.w};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int i = x0 + e;
                if (!in_range(i, g.nx, R)) continue;
                const float c = w[4 + e];
                float d = 0.0f, bs = 0.0f;
#pragma unroll
                for (int o = -R; o <= R; ++o) {
                    if (!o) continue;
                    const float v = w[4 + e + o];
                    d += v - c;
                    if (!in_range(i + o, g.nx, R)) bs += v;
                }
#pragma unroll
                for (int o = 1; o <= R; ++o) {
                    const float vm = (&yz[2 * (o - 1)].x)[e], vp = (&yz[2 * (o - 1) + 1].x)[e];
                    d += vm - c;
                    d += vp - c;
                    if (near_yz) {
                        if (!in_range(j - o, g.ny, R)) bs += vm;
                        if (!in_range(j + o, g.ny, R)) bs += vp;
                    }
                }
                if (D == 3) {
#pragma unroll
                    for (int o = 1; o <= R; ++o) {
                        const float vm = (&yz[2 * R + 2 * (o - 1)].x)[e], vp = (&yz[2 * R + 2 * (o - 1) + 1].x)[e];
                        d += vm - c;
                        d += vp - c;
                        if (near_yz) {
                            if (!in_range(k - o, g.nz, R)) bs += vm;
                            if (!in_range(k + o, g.nz, R)) bs += vp;
                        }
                    }
                }
                acc_square(d, s, cs);
                if (bs != 0.0f) bb = fma((double)bs, (double)bs, bb);
            }
        }
    }
    double rr = (double)s + (double)cs;
    block_sum2(rr, bb, sh);
    if (threadIdx.x == 0) { part[2 * blockIdx.x] = rr; part[2 * blockIdx.x + 1] = bb; }
}

// inv_c2 = 1 / (2DR)^2 turns the sums of d^2 and bsum^2 into sums of r^2 and b^2.
__global__ void __launch_bounds__(kResidThreads)
    k_residual_final(const double *__restrict__ part, int nparts, double *__restrict__ out,
                     double inv_c2) {
    __shared__ double sh[2 * (kResidThreads / 32)];
    double rr = 0.0, bb = 0.0;
    for (int p = threadIdx.x; p < nparts; p += blockDim.x) {
        rr += part[2 * p];
        bb += part[2 * p + 1];
    }
    block_sum2(rr, bb, sh);
    if (threadIdx.x == 0) { out[0] = rr * inv_c2; out[1] = bb * inv_c2; }
}

int launch_init_reference(const Geom &g, int dims, float *u, cudaStream_t s) {
    k_init_reference<<<4 * num_sms(), 256, 0, s>>>(u, g, dims);
    return cuda_fail(cudaGetLastError(), "init_reference launch");
}

int launch_copy_border(const Geom &g, int dims, const float *src, float *dst, cudaStream_t s) {
    k_copy_border<<<8 * num_sms(), 128, 0, s>>>(src, dst, g, dims);
    return cuda_fail(cudaGetLastError(), "copy_border launch");
}

int launch_init_uniform(float *u, size_t count, uint64_t seed, cudaStream_t s) {
    if (!count) return STENCIL_OK;
    const int blocks = (int)std::min<size_t>((count + 255) / 256, 8 * (size_t)num_sms());
    k_init_uniform<<<blocks, 256, 0, s>>>(u, count, seed);
    return cuda_fail(cudaGetLastError(), "init_uniform launch");
}

// scratch: >= residual_scratch_bytes() of device memory, 8-byte aligned.
size_t residual_scratch_bytes() { return (2 * kResidBlocks + 2) * sizeof(double); }

// Stage 1 over `blocks` blocks (any count: rows are handed out round-robin).
int launch_residual_partial(const Geom &g, int dims, const float *u, double *part, int blocks,
                            cudaStream_t s) {
    const bool vec = g.nx % 4 == 0 && g.radius <= 4;
    if (!vec) {
        k_residual_partial_any<<<blocks, kResidThreads, 0, s>>>(u, g, dims, part);
    } else {
        const int key = dims * 10 + g.radius;
        switch (key) {
            case 21: k_residual_partial_vec<2, 1><<<blocks, kResidThreads, 0, s>>>(u, g, part); break;
            case 22: k_residual_partial_vec<2, 2><<<blocks, kResidThreads, 0, s>>>(u, g, part); break;
            case 23: k_residual_partial_vec<2, 3><<<blocks, kResidThreads, 0, s>>>(u, g, part); break;
            case 24: k_residual_partial_vec<2, 4><<<blocks, kResidThreads, 0, s>>>(u, g, part); break;
            case 31: k_residual_partial_vec<3, 1><<<blocks, kResidThreads, 0, s>>>(u, g, part); break;
            case 32: k_residual_partial_vec<3, 2><<<blocks, kResidThreads, 0, s>>>(u, g, part); break;
            case 33: k_residual_partial_vec<3, 3><<<blocks, kResidThreads, 0, s>>>(u, g, part); break;
            default: k_residual_partial_vec<3, 4><<<blocks, kResidThreads, 0, s>>>(u, g, part); break;
        }
    }
    return cuda_fail(cudaGetLastError(), "residual launch");
}

int launch_residual_final(const Geom &g, int dims, const double *part, int nparts, double *out,
                          cudaStream_t s) {
    const double c = 2.0 * dims * g.radius;
    k_residual_final<<<1, kResidThreads, 0, s>>>(part, nparts, out, 1.0 / (c * c));
    return cuda_fail(cudaGetLastError(), "residual launch");
}

int launch_residual(const Geom &g, int dims, const float *u, double *scratch, cudaStream_t s) {
    int rc = launch_residual_partial(g, dims, u, scratch, kResidBlocks, s);
    if (rc) return rc;
    return launch_residual_final(g, dims, scratch, kResidBlocks, scratch + 2 * kResidBlocks, s);
}


// Streaming copy of n16 16-byte words, for host<->device transfers through
// the device-side address of pinned (mapped) host memory: every SM pulls
// (or pushes) over the C2C link instead of one copy engine.  Four loads per
// thread in flight; loads and stores marked streaming (no L1 allocation).
constexpr int kCopyThreads = 512;
__global__ void __launch_bounds__(kCopyThreads)
    k_copy16(float4 *__restrict__ dst, const float4 *__restrict__ src, size_t n16) {
    const size_t stride = (size_t)gridDim.x * kCopyThreads;
    size_t i = (size_t)blockIdx.x * kCopyThreads + threadIdx.x;
    for (; i + 3 * stride < n16; i += 4 * stride) {
        float4 v[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) v[k] = __ldcs(src + i + k * stride);
#pragma unroll
        for (int k = 0; k < 4; ++k) __stcs(dst + i + k * stride, v[k]);
    }
    for (; i < n16; i += stride) __stcs(dst + i, __ldcs(src + i));
}

int launch_copy16(void *dst, const void *src, size_t bytes, cudaStream_t s) {
    if (((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src) | bytes) & 15) != 0)
        return fail(STENCIL_EINVAL, "copy kernel: 16-byte aligned addresses and size required");
    if (!bytes) return STENCIL_OK;
    const size_t n16 = bytes / 16;
    const int blocks = (int)std::min<size_t>((size_t)num_sms() * 4, (n16 + kCopyThreads - 1) / kCopyThreads);
    k_copy16<<<blocks, kCopyThreads, 0, s>>>(static_cast<float4 *>(dst), static_cast<const float4 *>(src), n16);
    ST_CUDA(cudaGetLastError());
    return STENCIL_OK;
}

}  // namespace st

// k_tile.cu -- one sweep per launch from a TMA-staged shared-memory tile with
// halo ("smem" / "smem_padded" roles, src/stencil_kernel_smem.cu:8-106 and
// src/stencil_kernel_smem_padded.cu:8-119).
//
// The CTA's tile of (4*bx) x by x bz cells plus its halo -- x halo RA = R
// rounded up to 4 so the TMA x coordinate is 16-byte aligned, y/z halo R -- is
// fetched by one TMA box load (cp.async.bulk.tensor, out-of-bounds cells
// arrive as zeros) completing on an mbarrier; every neighbour is then read
// from shared memory.  This replaces the reference's edge-thread halo
// prefetch (src/prefetch_smem.cu:112-149) with a single asynchronous copy.
#include <algorithm>

#include "host.hpp"

namespace st {

template <int D, int R>
__global__ void __launch_bounds__(1024)
    k_tile(const __grid_constant__ CUtensorMap map, float *__restrict__ dst, Geom g) {
    constexpr int RA = (R + 3) & ~3;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float *tile = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) &
                                            ~static_cast<uintptr_t>(127));
    const int TX = 4 * blockDim.x, TY = blockDim.y, TZ = blockDim.z;
    const int PW = TX + 2 * RA, PH = TY + 2 * R, PD = D == 3 ? TZ + 2 * R : 1;
    uint64_t &bar = *reinterpret_cast<uint64_t *>(tile + ((PW * PH * PD + 31) & ~31));
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * TZ;
    if (tid == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
        mbar_arrive_expect_tx(&bar, (uint32_t)(PW * PH * PD * 4));
        if (D == 3) tma_load_3d(tile, &map, &bar, x0 - RA, y0 - R, z0 - R);
        else tma_load_2d(tile, &map, &bar, x0 - RA, y0 - R);
    }
    __syncthreads();
    const bool ok = mbar_wait_bounded(&bar, 0);
    if (!ok) return;
    const int tx = threadIdx.x, ty = threadIdx.y, tz = threadIdx.z;
    const int x = x0 + 4 * tx, y = y0 + ty, z = D == 3 ? z0 + tz : 0;
    if (x >= g.nx || !in_range(y, g.ny, R)) return;
    if (D == 3 && !in_range(z, g.nz, R)) return;
    const int plane = PW * PH;
    const float *c_row = tile + (D == 3 ? (tz + R) * plane : 0) + (ty + R) * PW + 4 * tx;
    float w[4 + 2 * RA];
#pragma unroll
    for (int q = 0; q < (4 + 2 * RA) / 4; ++q) {
        const float4 v = *reinterpret_cast<const float4 *>(c_row + 4 * q);
        w[4 * q] = v.x; w[4 * q + 1] = v.y; w[4 * q + 2] = v.z; w[4 * q + 3] = v.w;
    }
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int o = -R; o <= R; ++o) {
        if (o == 0) continue;
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[e] += w[RA + e + o];
    }
#pragma unroll
    for (int o = -R; o <= R; ++o) {
        if (o == 0) continue;
        const float4 v = *reinterpret_cast<const float4 *>(c_row + o * PW + RA);
        acc[0] += v.x; acc[1] += v.y; acc[2] += v.z; acc[3] += v.w;
    }
    if (D == 3) {
#pragma unroll
        for (int o = -R; o <= R; ++o) {
            if (o == 0) continue;
            const float4 v = *reinterpret_cast<const float4 *>(c_row + o * plane + RA);
            acc[0] += v.x; acc[1] += v.y; acc[2] += v.z; acc[3] += v.w;
        }
    }
    float out[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) out[e] = star_finish<D, R>(acc[e], w[RA + e], g.legacy);
    float *drow = dst + (long long)z * g.sz + (long long)y * g.sy;
    if (x >= R && x + 3 < g.nx - R) {
        *reinterpret_cast<float4 *>(drow + x) = make_float4(out[0], out[1], out[2], out[3]);
    } else {
#pragma unroll
        for (int e = 0; e < 4; ++e)
            if (in_range(x + e, g.nx, R)) drow[x + e] = out[e];
    }
}

namespace {

template <int D>
const void *tile_kernel(int r) {
    switch (r) {
        case 1: return reinterpret_cast<const void *>(k_tile<D, 1>);
        case 2: return reinterpret_cast<const void *>(k_tile<D, 2>);
        case 3: return reinterpret_cast<const void *>(k_tile<D, 3>);
        case 4: return reinterpret_cast<const void *>(k_tile<D, 4>);
        case 8: return reinterpret_cast<const void *>(k_tile<D, 8>);
        default: return nullptr;
    }
}

}  // namespace

// The kernel launch_tile_sweep runs (null if none), with its dynamic
// shared-memory limit raised to the largest box the launcher allows.
const void *tile_kernel_ptr(int dims, int r) {
    const void *fn = dims == 3 ? tile_kernel<3>(r) : tile_kernel<2>(r);
    if (fn && cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024 + 256) !=
                  cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return fn;
}

bool tile_supported(const Geom &g, int dims) {
    (void)dims;
    return g.nx % 4 == 0 && (g.radius <= 4 || g.radius == 8);
}

// One sweep src -> dst.  bx threads along x (4 cells each), by, bz.
int launch_tile_sweep(const Geom &g, int dims, const float *src, float *dst, int bx, int by,
                      int bz, cudaStream_t s) {
    const int R = g.radius, RA = (R + 3) & ~3;
    if (bx <= 0) bx = dims == 3 ? 8 : 32;
    if (by <= 0) by = 8;
    if (bz <= 0 || dims == 2) bz = dims == 3 ? 4 : 1;
    const void *fn = dims == 3 ? tile_kernel<3>(R) : tile_kernel<2>(R);
    if (!fn || g.nx % 4) return fail(STENCIL_EUNSUPPORTED, "tile kernel: radius %d / nx %d", R, g.nx);
    // Shrink the block until the halo box fits TMA (<= 256 per dimension) and
    // shared memory (<= 200 KB).
    auto box_bytes = [&]() {
        return 4LL * (4 * bx + 2 * RA) * (by + 2 * R) * (dims == 3 ? bz + 2 * R : 1);
    };
    while ((4 * bx + 2 * RA > 256 || box_bytes() > 200 * 1024) && bx > 1) bx /= 2;
    while ((by + 2 * R > 256 || box_bytes() > 200 * 1024) && by > 1) by /= 2;
    while ((bz + 2 * R > 256 || box_bytes() > 200 * 1024) && bz > 1) bz /= 2;
    if ((long long)bx * by * bz > 1024) return fail(STENCIL_EINVAL, "block exceeds 1024 threads");
    // box (rounded to 128 B) + alignment slack + the mbarrier
    const int smem = (int)((box_bytes() + 127) & ~127LL) + 128 + 16;
    if (smem > 200 * 1024) return fail(STENCIL_EUNSUPPORTED, "tile halo box too large");
    CUtensorMap map;
    const long long dimv[3] = {g.nx, g.ny, g.nz};
    const int box[3] = {4 * bx + 2 * RA, by + 2 * R, bz + 2 * R};
    int rc = make_tensor_map(&map, src, dims, dimv, box);
    if (rc) return rc;
    ST_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    dim3 block(bx, by, bz);
    dim3 grid((g.nx + 4 * bx - 1) / (4 * bx), (g.ny + by - 1) / by,
              dims == 3 ? (g.nz + bz - 1) / bz : 1);
    if (grid.y > 65535u || grid.z > 65535u) return fail(STENCIL_EINVAL, "grid too large");
    Geom gg = g;
    void *args[] = {&map, &dst, &gg};
    ST_CUDA(cudaLaunchKernel(fn, grid, block, args, smem, s));
    return STENCIL_OK;
}

}  // namespace st

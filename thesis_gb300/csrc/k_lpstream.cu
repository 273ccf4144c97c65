// k_lpstream.cu -- the correction sweep of the mixed-precision refinement
// (e_out = M e + rhs, e and rhs stored in BF16 or FP16, every sum in FP32) on
// 3-D grids, built like the FP32 stream kernel (k_stream.cu):
//   * one producer warp streams (TX + 2*RA) x (TY + 2*R) plane tiles of e --
//     RA = 8 cells, so that every TMA x coordinate of the 2-byte grid is
//     16-byte aligned -- into a ring of NS shared-memory slots (full/empty
//     mbarriers, bounded waits);
//   * a consumer thread owns 4 consecutive cells of one row: it converts the
//     z-neighbours once, when their plane arrives, into an FP32 register queue
//     of 2R+1 planes; x- and y-neighbours come from the centre slot as 8-byte
//     loads and enter the FP32 sums through mixed-precision adds
//     (add.rn.f32.bf16 / .f16: the 16-bit operand is converted exactly, one
//     rounding, no separate conversion); its rhs values come from global
//     memory one plane ahead;
//   * the sum runs in the order of the FP32 sweep (axis i, j, k; offsets -R..-1,
//     +1..+R) and starts from its first term; sum / C + rhs is one fused
//     multiply-add by RN(1/C) (within an FP32 ulp of the division, far below
//     the 16-bit storage rounding).
// Per cell update it reads 4 bytes (e and rhs) and writes 2, against 8 for an
// FP32 sweep; the border band of e_out is never written.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>

#include "host.hpp"

namespace st {
namespace {

template <typename E>
struct Cvt;
template <>
struct Cvt<__nv_bfloat16> {
    // two BF16 in one word -> two floats (exact)
    __device__ static float2 two(uint32_t w) {
        return make_float2(__uint_as_float(w << 16), __uint_as_float(w & 0xffff0000u));
    }
    __device__ static uint32_t pack(float a, float b) {
        __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
        return *reinterpret_cast<uint32_t *>(&h);
    }
    // acc + (half H of w), one rounding: the mixed-precision add converts the
    // BF16 operand exactly, so this equals acc + (float)value
    template <int H>
    __device__ static float add(uint32_t w, float acc) {
        float d;
        if constexpr (H == 0)
            asm("{.reg .b16 l, h; mov.b32 {l, h}, %1; add.rn.f32.bf16 %0, l, %2;}" : "=f"(d) : "r"(w), "f"(acc));
        else
            asm("{.reg .b16 l, h; mov.b32 {l, h}, %1; add.rn.f32.bf16 %0, h, %2;}" : "=f"(d) : "r"(w), "f"(acc));
        return d;
    }
    static constexpr CUtensorMapDataType kTma = CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
};
template <>
struct Cvt<__half> {
    __device__ static float2 two(uint32_t w) {
        return __half22float2(*reinterpret_cast<const __half2 *>(&w));
    }
    __device__ static uint32_t pack(float a, float b) {
        __half2 h = __floats2half2_rn(a, b);
        return *reinterpret_cast<uint32_t *>(&h);
    }
    template <int H>
    __device__ static float add(uint32_t w, float acc) {
        float d;
        if constexpr (H == 0)
            asm("{.reg .b16 l, h; mov.b32 {l, h}, %1; add.rn.f32.f16 %0, l, %2;}" : "=f"(d) : "r"(w), "f"(acc));
        else
            asm("{.reg .b16 l, h; mov.b32 {l, h}, %1; add.rn.f32.f16 %0, h, %2;}" : "=f"(d) : "r"(w), "f"(acc));
        return d;
    }
    static constexpr CUtensorMapDataType kTma = CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
};

// acc + value of cell c (0 .. 11) of the 6 words holding cells x-4 .. x+7
template <typename E, int CELL>
__device__ __forceinline__ float add_cell(const uint32_t (&wd)[6], float acc) {
    return Cvt<E>::template add<CELL & 1>(wd[CELL >> 1], acc);
}

// the four cells of one 8-byte row segment added to four sums
template <typename E>
__device__ __forceinline__ void add_row(uint2 v, float (&acc)[4]) {
    acc[0] = Cvt<E>::template add<0>(v.x, acc[0]);
    acc[1] = Cvt<E>::template add<1>(v.x, acc[1]);
    acc[2] = Cvt<E>::template add<0>(v.y, acc[2]);
    acc[3] = Cvt<E>::template add<1>(v.y, acc[3]);
}

template <int E0, int O, int R, typename E>
__device__ __forceinline__ void add_x(const uint32_t (&wd)[6], float (&acc)[4]) {
    acc[E0] = add_cell<E, 4 + E0 + O>(wd, acc[E0]);
}

template <typename E>
__device__ __forceinline__ float4 to4(uint2 v) {
    const float2 a = Cvt<E>::two(v.x), b = Cvt<E>::two(v.y);
    return make_float4(a.x, a.y, b.x, b.y);
}

// axis-i sum of the four cells in the reference order (offsets -R..-1, +1..+R)
template <typename E, int R, int O = -R>
__device__ __forceinline__ void xsum(const uint32_t (&wd)[6], float (&acc)[4]) {
    if constexpr (O == -R) {
        acc[0] = add_cell<E, 4 + 0 + O>(wd, -0.0f);
        acc[1] = add_cell<E, 4 + 1 + O>(wd, -0.0f);
        acc[2] = add_cell<E, 4 + 2 + O>(wd, -0.0f);
        acc[3] = add_cell<E, 4 + 3 + O>(wd, -0.0f);
    } else if constexpr (O != 0) {
        acc[0] = add_cell<E, 4 + 0 + O>(wd, acc[0]);
        acc[1] = add_cell<E, 4 + 1 + O>(wd, acc[1]);
        acc[2] = add_cell<E, 4 + 2 + O>(wd, acc[2]);
        acc[3] = add_cell<E, 4 + 3 + O>(wd, acc[3]);
    }
    if constexpr (O < R) xsum<E, R, O + 1>(wd, acc);
}

// four FP32 queue values added to four sums (as pairs where the kernel is
// issue-bound, R >= 3; the same roundings either way)
template <bool PK>
__device__ __forceinline__ void add_q(float4 v, float (&acc)[4]) {
    if constexpr (PK) {
        const float2 a = fadd2(make_float2(acc[0], acc[1]), make_float2(v.x, v.y));
        const float2 b = fadd2(make_float2(acc[2], acc[3]), make_float2(v.z, v.w));
        acc[0] = a.x; acc[1] = a.y; acc[2] = b.x; acc[3] = b.y;
    } else {
        acc[0] += v.x; acc[1] += v.y; acc[2] += v.z; acc[3] += v.w;
    }
}


constexpr int kTX = 128, kTY = 16, kNS = 16, kRA = 8;

template <int R>
struct LpShape {
    static constexpr int PW = kTX + 2 * kRA;  // elements
    static constexpr int PH = kTY + 2 * R;
    static constexpr int PLANE_BYTES = PW * PH * 2;
    static constexpr int SLOT_BYTES = (PLANE_BYTES + 127) & ~127;
    static constexpr int CWARPS = kTY;  // one warp per row, 4 cells per lane
    static constexpr int THREADS = 32 * CWARPS + 32;
    static constexpr int SMEM_BYTES = kNS * SLOT_BYTES + 128 + 2 * kNS * 8;
    // two CTAs per SM where the registers allow it (R <= 2: 34 warps per SM)
    static constexpr int MIN_BLOCKS = R <= 2 ? 2 : 1;
};

template <typename E, int R>
__global__ void __launch_bounds__(LpShape<R>::THREADS, LpShape<R>::MIN_BLOCKS)
    k_lp_stream(const __grid_constant__ CUtensorMap e_map, E *__restrict__ eo,
                const E *__restrict__ rhs, Geom g, int tiles_x, int tiles_y, int zchunk,
                int items) {
    using S = LpShape<R>;
    constexpr int C = 6 * R;
    constexpr int QN = 2 * R + 1;
    constexpr int PF = R == 4 ? 3 : QN;  // rhs prefetch distance (registers at R = 4)
    static_assert(QN % PF == 0, "the rhs ring must divide the plane queue");
    constexpr bool PK = R >= 3;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char *ring = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~static_cast<uintptr_t>(127));
    uint64_t *full = reinterpret_cast<uint64_t *>(ring + kNS * S::SLOT_BYTES);
    uint64_t *empty = full + kNS;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        prefetch_tensormap(&e_map);
        for (int s = 0; s < kNS; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], S::CWARPS);
        }
        fence_mbar_init();
    }
    __syncthreads();
    const int ntiles = tiles_x * tiles_y;

    if (warp == S::CWARPS) {
        if (lane != 0) return;
        uint32_t q = 0;
        for (int item = blockIdx.x; item < items; item += gridDim.x) {
            const int t = item % ntiles, ch = item / ntiles;
            const int x0 = (t % tiles_x) * kTX, y0 = (t / tiles_x) * kTY;
            const int z0 = R + ch * zchunk, z1 = min(z0 + zchunk, g.nz - R);
            const int np = (z1 - z0) + 2 * R;
            for (int p = 0; p < np; ++p, ++q) {
                const int s = q & (kNS - 1);
                const uint32_t use = q / kNS;
                if (use > 0 && !mbar_wait_bounded(&empty[s], (use - 1) & 1)) return;
                mbar_arrive_expect_tx(&full[s], S::PLANE_BYTES);
                tma_load_3d(ring + s * S::SLOT_BYTES, &e_map, &full[s], x0 - kRA, y0 - R,
                            z0 - R + p);
            }
        }
        return;
    }

    const int cx = lane, cy = warp;
    auto release = [&](int s) {
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);
    };
    // byte offset of this thread's 4 cells in a slot (row cy + R, cell RA + 4 cx)
    const int own = ((cy + R) * S::PW + kRA + 4 * cx) * 2;
    constexpr int ROW = S::PW * 2;
    float4 qz[QN];
    uint32_t qb = 0;
    for (int item = blockIdx.x; item < items; item += gridDim.x) {
        const int t = item % ntiles, ch = item / ntiles;
        const int x0 = (t % tiles_x) * kTX, y0 = (t / tiles_x) * kTY;
        const int z0 = R + ch * zchunk, z1 = min(z0 + zchunk, g.nz - R);
        const int np = (z1 - z0) + 2 * R;
        const int x = x0 + 4 * cx, y = y0 + cy;
        const bool live = x < g.nx && in_range(y, g.ny, R);
        const bool xin = x >= R && x + 3 < g.nx - R;
        const long long rowoff = (long long)y * g.sy + x;
#pragma unroll
        for (int p = 0; p < 2 * R; ++p) {
            const uint32_t q = qb + p;
            const int s = q & (kNS - 1);
            if (!mbar_wait_bounded(&full[s], (q / kNS) & 1)) return;
            qz[p] = to4<E>(*reinterpret_cast<const uint2 *>(ring + s * S::SLOT_BYTES + own));
            if (p < R || p >= np - R) release(s);
        }
        // rhs of planes z .. z+PF-1 in a register ring, each fetched PF plane
        // steps before its use (one step is shorter than a DRAM round trip);
        // PF divides QN so the ring position is known at compile time
        uint2 rq[PF];
#pragma unroll
        for (int p = 0; p < PF; ++p) {
            rq[p] = make_uint2(0, 0);
            if (live && z0 + p < z1)
                rq[p] = __ldg(reinterpret_cast<const uint2 *>(rhs + (long long)(z0 + p) * g.sz + rowoff));
        }
        for (int zb = z0; zb < z1; zb += QN) {
#pragma unroll
            for (int ph = 0; ph < QN; ++ph) {
                const int z = zb + ph;
                if (z >= z1) break;
                const int step = z - z0;
                const uint2 rc = rq[ph % PF];
                if (live && z + PF < z1)
                    rq[ph % PF] = __ldg(reinterpret_cast<const uint2 *>(rhs + (long long)(z + PF) * g.sz + rowoff));
                const int sc = (qb + step + R) & (kNS - 1);
                const unsigned char *cb = ring + sc * S::SLOT_BYTES + own;
                // cells x-4 .. x+7 of row y as six 2-cell words; x- and y-neighbours
                // are added straight from the 16-bit values (mixed-precision adds)
                uint32_t wd[6];
                {
                    const uint2 a = *reinterpret_cast<const uint2 *>(cb - 8);
                    const uint2 c = *reinterpret_cast<const uint2 *>(cb);
                    const uint2 b = *reinterpret_cast<const uint2 *>(cb + 8);
                    wd[0] = a.x; wd[1] = a.y; wd[2] = c.x; wd[3] = c.y; wd[4] = b.x; wd[5] = b.y;
                }
                float acc[4];
                // axis i; the first term starts the sum (x + -0 = x exactly)
                xsum<E, R>(wd, acc);
                // axis j
#pragma unroll
                for (int o = -R; o <= R; ++o) {
                    if (!o) continue;
                    add_row<E>(*reinterpret_cast<const uint2 *>(cb + o * ROW), acc);
                }
                // axis k, planes z-R .. z-1
#pragma unroll
                for (int o = -R; o <= -1; ++o) add_q<PK>(qz[(ph + R + o + QN) % QN], acc);
                release(sc);
                {
                    const int pn = step + 2 * R;
                    const uint32_t q = qb + pn;
                    const int s = q & (kNS - 1);
                    if (!mbar_wait_bounded(&full[s], (q / kNS) & 1)) return;
                    qz[(ph + 2 * R) % QN] =
                        to4<E>(*reinterpret_cast<const uint2 *>(ring + s * S::SLOT_BYTES + own));
                    if (pn >= np - R) release(s);
                }
#pragma unroll
                for (int o = 1; o <= R; ++o) add_q<PK>(qz[(ph + R + o) % QN], acc);
                if (live) {
                    // sum / C + rhs as one fused multiply-add by RN(1/C): the
                    // correction is stored in 16 bits, so the division's last
                    // FP32 bit is immaterial
                    float out[4];
                    constexpr float kInv = 1.0f / (float)C;
                    const float2 r01 = Cvt<E>::two(rc.x), r23 = Cvt<E>::two(rc.y);
                    if constexpr (PK) {
                        const float2 a = ffma2(make_float2(acc[0], acc[1]), make_float2(kInv, kInv), r01);
                        const float2 b = ffma2(make_float2(acc[2], acc[3]), make_float2(kInv, kInv), r23);
                        out[0] = a.x; out[1] = a.y; out[2] = b.x; out[3] = b.y;
                    } else {
                        out[0] = fmaf(acc[0], kInv, r01.x);
                        out[1] = fmaf(acc[1], kInv, r01.y);
                        out[2] = fmaf(acc[2], kInv, r23.x);
                        out[3] = fmaf(acc[3], kInv, r23.y);
                    }
                    E *dst = eo + (long long)z * g.sz + rowoff;
                    if (xin) {
                        uint2 o2;
                        o2.x = Cvt<E>::pack(out[0], out[1]);
                        o2.y = Cvt<E>::pack(out[2], out[3]);
                        *reinterpret_cast<uint2 *>(dst) = o2;
                    } else {
#pragma unroll
                        for (int e = 0; e < 4; ++e)
                            if (in_range(x + e, g.nx, R)) {
                                const uint32_t h = Cvt<E>::pack(out[e], 0.0f);
                                *reinterpret_cast<unsigned short *>(dst + e) = (unsigned short)(h & 0xffffu);
                            }
                    }
                }
            }
        }
        qb += np;
    }
}

template <typename E, int R>
int run_lp(const Geom &g, const E *e, E *eo, const E *rhs, cudaStream_t s) {
    using S = LpShape<R>;
    const void *fn = reinterpret_cast<const void *>(k_lp_stream<E, R>);
    static int per_sm_cached[64] = {0};
    const int dev = current_device();
    int per_sm = (dev >= 0 && dev < 64) ? per_sm_cached[dev] : 0;
    if (!per_sm) {
        ST_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, S::SMEM_BYTES));
        ST_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     cudaSharedmemCarveoutMaxShared));
        ST_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, S::THREADS, S::SMEM_BYTES));
        if (per_sm < 1) return fail(STENCIL_EUNSUPPORTED, "low-precision stream kernel does not fit");
        if (dev >= 0 && dev < 64) per_sm_cached[dev] = per_sm;
    }
    const int resident = per_sm * num_sms();
    const int tiles_x = (g.nx + kTX - 1) / kTX, tiles_y = (g.ny + kTY - 1) / kTY;
    const int tiles = tiles_x * tiles_y;
    const int zin = g.nz - 2 * R;
    // (tile, z-chunk) items, chunk count filling whole waves (as k_stream.cu)
    int nchunks = 1;
    double best = 1e30;
    for (int n = 1; n <= std::max(1, zin / 8); ++n) {
        const int zc = (zin + n - 1) / n;
        const long long it = (long long)tiles * ((zin + zc - 1) / zc);
        const double waves = std::ceil((double)it / resident);
        const double fill = (double)it / (waves * resident);
        const double cost = (1.0 + 0.25 * (2.0 * R) / zc) / fill + 0.002 * waves;
        if (cost < best - 1e-9) { best = cost; nchunks = n; }
    }
    int zchunk = (zin + nchunks - 1) / nchunks;
    nchunks = (zin + zchunk - 1) / zchunk;
    int items = tiles * nchunks;
    const int grid = std::min(items, resident);
    CUtensorMap map;
    const long long dims[3] = {g.nx, g.ny, g.nz};
    const int box[3] = {S::PW, S::PH, 1};
    int rc = make_tensor_map_typed(&map, e, 3, dims, box, Cvt<E>::kTma, 2);
    if (rc) return rc;
    Geom gg = g;
    int tx_ = tiles_x, ty_ = tiles_y;
    void *args[] = {&map, &eo, &rhs, &gg, &tx_, &ty_, &zchunk, &items};
    ST_CUDA(cudaLaunchKernel(fn, dim3(grid), dim3(S::THREADS), args, S::SMEM_BYTES, s));
    return STENCIL_OK;
}

}  // namespace

bool lp_stream_supported(const Geom &g, int dims) {
    return dims == 3 && g.nx % 8 == 0 && (g.radius == 1 || g.radius == 2 || g.radius == 4);
}

template <typename E>
int launch_lp_stream(const Geom &g, const E *e, E *eo, const E *rhs, cudaStream_t s) {
    switch (g.radius) {
        case 1: return run_lp<E, 1>(g, e, eo, rhs, s);
        case 2: return run_lp<E, 2>(g, e, eo, rhs, s);
        case 4: return run_lp<E, 4>(g, e, eo, rhs, s);
        default: return fail(STENCIL_EUNSUPPORTED, "low-precision stream kernel: R=%d", g.radius);
    }
}

template int launch_lp_stream<__nv_bfloat16>(const Geom &, const __nv_bfloat16 *, __nv_bfloat16 *,
                                             const __nv_bfloat16 *, cudaStream_t);
template int launch_lp_stream<__half>(const Geom &, const __half *, __half *, const __half *,
                                      cudaStream_t);

}  // namespace st

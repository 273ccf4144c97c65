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
#include <cstdlib>

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
                fence_proxy_async();  // the consumers' reads of the slot before the TMA write
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

// ---- R = 4 on the tensor cores --------------------------------------------
//
// The x- and y-neighbour sums of a plane are products with constant banded
// matrices: for a 16 x 16 block of cells (rows y0..y0+15, columns j0..j0+15)
//   X = P[rows][j0-8 .. j0+23] . Bx   (two 16-column windows, coefficient 1
//       at 1 <= |dx| <= 4 and -1 at dx = 0),
//   Y = Ay . P[y0-4 .. y0+19][cols]   (k = 16 + 8 rows, coefficient 1 at
//       1 <= |dy| <= 4),
// computed by mma.sync (BF16 / FP16 operands as stored, FP32 accumulation:
// the products are exact, the sums FP32) with the block's operands loaded by
// ldmatrix from the TMA-filled plane slot.  The z sum is a running FP32 sum W
// of the 2R+1 planes z-R .. z+R (one plane added, one subtracted per step)
// that also holds the centre, which the -1 of Bx cancels; W is the
// accumulator the products are added to.  A warp owns one 16 x 16 block of
// the CTA's 128 x 32 tile (16 consumer warps, two 16-row blocks sharing one
// halo), so a cell costs about 0.3 warp instructions against about 1.4 for
// the per-term mixed-precision adds.  The result differs from the in-order
// FP32 sum by FP32 roundings only (the correction equation is not bound to
// the reference's order).
//
// Measured on GB300 (504^3 R = 4, one sweep): per-term adds 240 us; this
// structure with 128 x 16 tiles and per-thread rhs loads / stores 248 us (9
// warps per SM: latency-bound); 128 x 32 tiles 195 us (the L1/TEX pipe 90 %
// busy: per-thread global accesses in the mma fragment layout touch 8
// half-used sectors per warp instruction); rhs and output by TMA as below:
// 768^3 refinement 1.24x the FP32 loop.  The producer issues
// fence.proxy.async after acquiring a slot and before its TMA write into it,
// ordering the consumers' generic-proxy reads (released to it through the
// empty mbarrier) before the async-proxy write; repeated runs are
// bit-identical.  (An earlier form that read rhs and stored its output with
// per-thread global accesses showed rare differing cells between repeated
// runs without such a fence.)
constexpr int kTcTX = 128;
constexpr int kTcPW = 152;  // slot row: 76 words, so ldmatrix rows hit distinct banks

template <typename E>
struct Bits;
template <>
struct Bits<__nv_bfloat16> {
    static constexpr uint32_t kOne = 0x3f80u, kMinusOne = 0xbf80u;
};
template <>
struct Bits<__half> {
    static constexpr uint32_t kOne = 0x3c00u, kMinusOne = 0xbc00u;
};

template <typename E>
__device__ __forceinline__ uint32_t coef_bits(int c) {
    return c > 0 ? Bits<E>::kOne : (c < 0 ? Bits<E>::kMinusOne : 0u);
}

// x coefficient of input column offset d from the output column
__device__ __forceinline__ int xcoef(int d) { return d == 0 ? -1 : ((d >= -4 && d <= 4) ? 1 : 0); }
// y coefficient of k rows from the block's first input row (output row - 4)
// for output row m
__device__ __forceinline__ int ycoef(int k, int m) {
    const int d = k - 4 - m;
    return (d != 0 && d >= -4 && d <= 4) ? 1 : 0;
}

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], uint32_t addr) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(addr));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], uint32_t addr) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(addr));
}
__device__ __forceinline__ void ldsm_x2_t(uint32_t (&r)[2], uint32_t addr) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0, %1}, [%2];"
                 : "=r"(r[0]), "=r"(r[1])
                 : "r"(addr));
}

// D = A B + C (m16n8k16 / m16n8k8, FP32 accumulation)
template <typename E>
struct Mma;
template <>
struct Mma<__nv_bfloat16> {
    __device__ static void k16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1,
                               const float (&c)[4]) {
        asm volatile(
            "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, "
            "{%8, %9}, {%10, %11, %12, %13};"
            : "=f"(d[0]), "=f"(d[1]), "=f"(d[2]), "=f"(d[3])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1), "f"(c[0]), "f"(c[1]),
              "f"(c[2]), "f"(c[3]));
    }
    __device__ static void k8(float (&d)[4], const uint32_t (&a)[2], uint32_t b0, const float (&c)[4]) {
        asm volatile(
            "mma.sync.aligned.m16n8k8.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5}, {%6}, "
            "{%7, %8, %9, %10};"
            : "=f"(d[0]), "=f"(d[1]), "=f"(d[2]), "=f"(d[3])
            : "r"(a[0]), "r"(a[1]), "r"(b0), "f"(c[0]), "f"(c[1]), "f"(c[2]), "f"(c[3]));
    }
};
template <>
struct Mma<__half> {
    __device__ static void k16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1,
                               const float (&c)[4]) {
        asm volatile(
            "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, "
            "{%8, %9}, {%10, %11, %12, %13};"
            : "=f"(d[0]), "=f"(d[1]), "=f"(d[2]), "=f"(d[3])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1), "f"(c[0]), "f"(c[1]),
              "f"(c[2]), "f"(c[3]));
    }
    __device__ static void k8(float (&d)[4], const uint32_t (&a)[2], uint32_t b0, const float (&c)[4]) {
        asm volatile(
            "mma.sync.aligned.m16n8k8.row.col.f32.f16.f16.f32 {%0, %1, %2, %3}, {%4, %5}, {%6}, "
            "{%7, %8, %9, %10};"
            : "=f"(d[0]), "=f"(d[1]), "=f"(d[2]), "=f"(d[3])
            : "r"(a[0]), "r"(a[1]), "r"(b0), "f"(c[0]), "f"(c[1]), "f"(c[2]), "f"(c[3]));
    }
};

// A bounded mbarrier wait that every lane of the warp leaves the same way
// (the warp-wide ldmatrix / mma after it need all lanes).
__device__ __forceinline__ bool warp_wait(uint64_t *bar, uint32_t parity) {
    return __all_sync(0xffffffffu, mbar_wait_bounded(bar, parity));
}

// Data movement: the e plane tiles (152 x 40) by TMA into a ring of NE slots;
//   * the producer also streams each step's rhs tile (136 x 32: 68-word rows,
//     conflict-free fragment reads) into a ring of 4 slots, issued with the
//     e plane that the same step first needs;
//   * a consumer warp writes its 16 x 16 output block into one of two staging
//     buffers and one lane stores it with cp.async.bulk.tensor (the box is
//     clipped at the grid's end; cells of the border band are written as 0,
//     the value they hold for the whole refinement).
template <int NE>
struct LpTc3Shape {
    static constexpr int R = 4, RB = 2, TY = 32;
    static constexpr int PH = TY + 2 * R;
    static constexpr int E_BYTES = kTcPW * PH * 2;            // 12160
    static constexpr int E_SLOT = (E_BYTES + 127) & ~127;
    static constexpr int RW = 136;                             // rhs tile row
    static constexpr int R_BYTES = RW * TY * 2;                // 8704
    static constexpr int R_SLOT = (R_BYTES + 127) & ~127;
    static constexpr int NR = 4;
    static constexpr int CWARPS = 16;
    static constexpr int THREADS = 32 * CWARPS + 32;
    static constexpr int STAGE = 16 * 16 * 2;                  // one output block
    static constexpr int OFF_R = NE * E_SLOT;
    static constexpr int OFF_O = OFF_R + NR * R_SLOT;
    static constexpr int OFF_BAR = OFF_O + CWARPS * 2 * STAGE;
    static constexpr int SMEM_BYTES = OFF_BAR + 2 * (NE + NR) * 8 + 128;
    static_assert(NE >= 2 * R + 2, "ring too short for the running z sum");
};

__device__ __forceinline__ void tma_store_3d(const CUtensorMap *map, const void *src, int x, int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%2, %3, %4}], [%1];" ::"l"(
            reinterpret_cast<uint64_t>(map)),
        "r"(smem_u32(src)), "r"(x), "r"(y), "r"(z)
        : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void bulk_wait_read() {
    asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

template <typename E, int NE>
__global__ void __launch_bounds__(LpTc3Shape<NE>::THREADS, 1)
    k_lp_stream_tc3(const __grid_constant__ CUtensorMap e_map, const __grid_constant__ CUtensorMap r_map,
                    const __grid_constant__ CUtensorMap o_map, Geom g, int tiles_x, int tiles_y,
                    int zchunk, int items) {
    using S = LpTc3Shape<NE>;
    constexpr int R = S::R;
    constexpr int C = 6 * R;
    constexpr int NR = S::NR;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char *sm = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~static_cast<uintptr_t>(127));
    unsigned char *ering = sm, *rring = sm + S::OFF_R, *ostage = sm + S::OFF_O;
    uint64_t *full = reinterpret_cast<uint64_t *>(sm + S::OFF_BAR);
    uint64_t *empty = full + NE;
    uint64_t *rfull = empty + NE;
    uint64_t *rempty = rfull + NR;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        prefetch_tensormap(&e_map);
        prefetch_tensormap(&r_map);
        prefetch_tensormap(&o_map);
        for (int s = 0; s < NE; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], S::CWARPS);
        }
        for (int s = 0; s < NR; ++s) {
            mbar_init(&rfull[s], 1);
            mbar_init(&rempty[s], S::CWARPS);
        }
        fence_mbar_init();
    }
    __syncthreads();
    const int ntiles = tiles_x * tiles_y;

    if (warp == S::CWARPS) {
        if (lane != 0) return;
        uint32_t q = 0, qr = 0;
        for (int item = blockIdx.x; item < items; item += gridDim.x) {
            const int t = item % ntiles, ch = item / ntiles;
            const int x0 = (t % tiles_x) * kTcTX, y0 = (t / tiles_x) * S::TY;
            const int z0 = R + ch * zchunk, z1 = min(z0 + zchunk, g.nz - R);
            const int np = (z1 - z0) + 2 * R;
            for (int p = 0; p < np; ++p, ++q) {
                const int s = (int)(q % NE);
                const uint32_t use = q / NE;
                if (use > 0 && !mbar_wait_bounded(&empty[s], (use - 1) & 1)) return;
                // the consumers' reads of the slot (they arrived after them)
                // before this TMA write into it
                fence_proxy_async();
                mbar_arrive_expect_tx(&full[s], S::E_BYTES);
                tma_load_3d(ering + s * S::E_SLOT, &e_map, &full[s], x0 - 8, y0 - R, z0 - R + p);
                if (p >= 2 * R) {
                    // the rhs of step p - 2R (plane z0 + p - 2R), first needed with e plane p
                    const int rs = (int)(qr % NR);
                    const uint32_t ruse = qr / NR;
                    if (ruse > 0 && !mbar_wait_bounded(&rempty[rs], (ruse - 1) & 1)) return;
                    fence_proxy_async();
                    mbar_arrive_expect_tx(&rfull[rs], S::R_BYTES);
                    tma_load_3d(rring + rs * S::R_SLOT, &r_map, &rfull[rs], x0, y0, z0 + p - 2 * R);
                    ++qr;
                }
            }
        }
        return;
    }

    const int gq = lane >> 2, tq = lane & 3;
    uint32_t bx[2][2][2];
#pragma unroll
    for (int w = 0; w < 2; ++w)
#pragma unroll
        for (int nb = 0; nb < 2; ++nb)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int k = 2 * tq + 8 * h, n = gq + 8 * nb;
                const int d0 = (w == 0 ? k - 8 : k + 8) - n;
                bx[w][nb][h] = coef_bits<E>(xcoef(d0)) | (coef_bits<E>(xcoef(d0 + 1)) << 16);
            }
    uint32_t ay16[4], ay8[2];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int m = gq + 8 * (i & 1), k = 2 * tq + 8 * (i >> 1);
        ay16[i] = coef_bits<E>(ycoef(k, m)) | (coef_bits<E>(ycoef(k + 1, m)) << 16);
    }
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const int m = gq + 8 * i, k = 16 + 2 * tq;
        ay8[i] = coef_bits<E>(ycoef(k, m)) | (coef_bits<E>(ycoef(k + 1, m)) << 16);
    }
    const int rb = warp >> 3, cw = 16 * (warp & 7), ry = 16 * rb;
    const int mi = lane >> 3, rr = lane & 7;
    const uint32_t off_a = ((R + ry + rr + (mi & 1) * 8) * kTcPW + cw + (mi >> 1) * 8) * 2;
    const uint32_t off_b16 = ((ry + rr + (mi & 1) * 8) * kTcPW + cw + 8 + (mi >> 1) * 8) * 2;
    const uint32_t off_b8 = ((ry + 16 + rr) * kTcPW + cw + 8 + (mi & 1) * 8) * 2;
    const uint32_t off_w = ((R + ry + gq) * kTcPW + cw + 8 + 2 * tq) * 2;
    const uint32_t off_r = ((ry + gq) * S::RW + cw + 2 * tq) * 2;  // rhs words; +16: n block 1; +8 rows
    const uint32_t off_o = (gq * 16 + 2 * tq) * 2;                 // staging words; +16; +8 rows
    constexpr uint32_t HALF = 8 * kTcPW * 2, RHALF = 8 * S::RW * 2, OHALF = 8 * 16 * 2;
    const uint32_t ering_s = smem_u32(ering);
    unsigned char *stage0 = ostage + warp * 2 * S::STAGE;
    // a slot's reads are done: one arrival per warp
    auto release = [&](uint64_t *bar) {
        __syncwarp();
        if (lane == 0) mbar_arrive(bar);
    };
    auto bail = [&]() {
        if (lane == 0) bulk_wait_all();
    };
    auto words = [&](int s, uint32_t (&wv)[2][2]) {
        const unsigned char *b = ering + s * S::E_SLOT + off_w;
        wv[0][0] = *reinterpret_cast<const uint32_t *>(b);
        wv[0][1] = *reinterpret_cast<const uint32_t *>(b + 16);
        wv[1][0] = *reinterpret_cast<const uint32_t *>(b + HALF);
        wv[1][1] = *reinterpret_cast<const uint32_t *>(b + HALF + 16);
    };
    uint32_t qb = 0, qr = 0, sb = 0;  // e plane, rhs and staging sequence numbers
    for (int item = blockIdx.x; item < items; item += gridDim.x) {
        const int t = item % ntiles, ch = item / ntiles;
        const int x0 = (t % tiles_x) * kTcTX, y0 = (t / tiles_x) * S::TY;
        const int z0 = R + ch * zchunk, z1 = min(z0 + zchunk, g.nz - R);
        const int np = (z1 - z0) + 2 * R;
        const int xa = x0 + cw + 2 * tq, ya = y0 + ry + gq;
        const bool r0 = in_range(ya, g.ny, R), r1 = in_range(ya + 8, g.ny, R);
        const bool c0 = xa >= R && xa + 1 < g.nx - R, c1 = xa + 8 >= R && xa + 9 < g.nx - R;
        const bool ok[2][2] = {{r0 && c0, r0 && c1}, {r1 && c0, r1 && c1}};
        float2 wsum[2][2];
#pragma unroll
        for (int p = 0; p <= 2 * R; ++p) {
            const uint32_t q = qb + p;
            if (!warp_wait(&full[q % NE], (q / NE) & 1)) { bail(); return; }
            uint32_t wv[2][2];
            words((int)(q % NE), wv);
#pragma unroll
            for (int h = 0; h < 2; ++h)
#pragma unroll
                for (int nb = 0; nb < 2; ++nb) {
                    const float2 v = Cvt<E>::two(wv[h][nb]);
                    wsum[h][nb] = p == 0 ? v : fadd2(wsum[h][nb], v);
                }
        }
        for (int z = z0; z < z1; ++z) {
            const int step = z - z0;
            int old_slot = -1;
            if (step > 0) {
                const uint32_t qn = qb + step + 2 * R, qo = qb + step - 1;
                if (!warp_wait(&full[qn % NE], (qn / NE) & 1)) { bail(); return; }
                uint32_t wn[2][2], wo[2][2];
                words((int)(qn % NE), wn);
                words((int)(qo % NE), wo);
#pragma unroll
                for (int h = 0; h < 2; ++h)
#pragma unroll
                    for (int nb = 0; nb < 2; ++nb) {
                        const float2 d = ffma2(Cvt<E>::two(wo[h][nb]), make_float2(-1.0f, -1.0f),
                                               Cvt<E>::two(wn[h][nb]));
                        wsum[h][nb] = fadd2(wsum[h][nb], d);
                    }
                old_slot = (int)(qo % NE);
            }
            float wc[2][4];
#pragma unroll
            for (int nb = 0; nb < 2; ++nb) {
                wc[nb][0] = wsum[0][nb].x; wc[nb][1] = wsum[0][nb].y;
                wc[nb][2] = wsum[1][nb].x; wc[nb][3] = wsum[1][nb].y;
            }
            const uint32_t cs = ering_s + ((qb + step + R) % NE) * S::E_SLOT;
            uint32_t a1[4], a2[4], b16[4], b8[2];
            ldsm_x4(a1, cs + off_a);
            ldsm_x4(a2, cs + off_a + 32);
            ldsm_x4_t(b16, cs + off_b16);
            ldsm_x2_t(b8, cs + off_b8);
            float acc[2][4];
#pragma unroll
            for (int nb = 0; nb < 2; ++nb) {
                float t1[4], t2[4], t3[4];
                Mma<E>::k16(t1, a1, bx[0][nb][0], bx[0][nb][1], wc[nb]);
                Mma<E>::k16(t2, a2, bx[1][nb][0], bx[1][nb][1], t1);
                Mma<E>::k16(t3, ay16, b16[2 * nb], b16[2 * nb + 1], t2);
                Mma<E>::k8(acc[nb], ay8, b8[nb], t3);
            }
            // rhs of this step
            const int rs = (int)(qr % NR);
            if (!warp_wait(&rfull[rs], (qr / NR) & 1)) { bail(); return; }
            uint32_t rw[2][2];
            {
                const unsigned char *b = rring + rs * S::R_SLOT + off_r;
                rw[0][0] = *reinterpret_cast<const uint32_t *>(b);
                rw[0][1] = *reinterpret_cast<const uint32_t *>(b + 16);
                rw[1][0] = *reinterpret_cast<const uint32_t *>(b + RHALF);
                rw[1][1] = *reinterpret_cast<const uint32_t *>(b + RHALF + 16);
            }
            // the staging buffer of this step: free once the store issued two
            // steps ago has read it
            unsigned char *st = stage0 + (sb & 1) * S::STAGE;
            if (lane == 0) bulk_wait_read<1>();
            __syncwarp();
            constexpr float kInv = 1.0f / (float)C;
#pragma unroll
            for (int h = 0; h < 2; ++h)
#pragma unroll
                for (int nb = 0; nb < 2; ++nb) {
                    const float2 r = Cvt<E>::two(rw[h][nb]);
                    const float2 o = ffma2(make_float2(acc[nb][2 * h], acc[nb][2 * h + 1]),
                                           make_float2(kInv, kInv), r);
                    *reinterpret_cast<uint32_t *>(st + off_o + h * OHALF + nb * 16) =
                        ok[h][nb] ? Cvt<E>::pack(o.x, o.y) : 0u;
                }
            // the staged block becomes visible to the bulk copy, then one lane
            // stores it
            fence_proxy_async();
            __syncwarp();
            if (lane == 0) {
                tma_store_3d(&o_map, st, x0 + cw, y0 + ry, z);
                bulk_commit();
            }
            ++sb;
            release(&rempty[rs]);
            ++qr;
            if (old_slot >= 0) release(&empty[old_slot]);
        }
        const int last = (z1 - z0) - 1;
        for (int p = last; p < np; ++p) release(&empty[(qb + p) % NE]);
        qb += np;
    }
    if (lane == 0) bulk_wait_all();
}

template <typename E, int NE>
int run_lp_tc3(const Geom &g, const E *e, E *eo, const E *rhs, cudaStream_t s) {
    using S = LpTc3Shape<NE>;
    const void *fn = reinterpret_cast<const void *>(k_lp_stream_tc3<E, NE>);
    static int per_sm_cached[64] = {0};
    const int dev = current_device();
    int per_sm = (dev >= 0 && dev < 64) ? per_sm_cached[dev] : 0;
    if (!per_sm) {
        ST_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, S::SMEM_BYTES));
        ST_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     cudaSharedmemCarveoutMaxShared));
        ST_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, S::THREADS, S::SMEM_BYTES));
        if (per_sm < 1) return fail(STENCIL_EUNSUPPORTED, "tensor-core correction sweep does not fit");
        if (dev >= 0 && dev < 64) per_sm_cached[dev] = per_sm;
    }
    const int resident = per_sm * num_sms();
    const int tiles_x = (g.nx + kTcTX - 1) / kTcTX, tiles_y = (g.ny + S::TY - 1) / S::TY;
    const int tiles = tiles_x * tiles_y;
    const int zin = g.nz - 2 * S::R;
    int nchunks = 1;
    double best = 1e30;
    for (int n = 1; n <= std::max(1, zin / 8); ++n) {
        const int zc = (zin + n - 1) / n;
        const long long it = (long long)tiles * ((zin + zc - 1) / zc);
        const double waves = std::ceil((double)it / resident);
        const double fill = (double)it / (waves * resident);
        const double cost = (1.0 + 0.25 * (2.0 * S::R + 1) / zc) / fill + 0.002 * waves;
        if (cost < best - 1e-9) { best = cost; nchunks = n; }
    }
    int zchunk = (zin + nchunks - 1) / nchunks;
    nchunks = (zin + zchunk - 1) / zchunk;
    int items = tiles * nchunks;
    const int grid = std::min(items, resident);
    CUtensorMap emap, rmap, omap;
    const long long dims[3] = {g.nx, g.ny, g.nz};
    const int ebox[3] = {kTcPW, S::PH, 1}, rbox[3] = {S::RW, S::TY, 1}, obox[3] = {16, 16, 1};
    int rc = make_tensor_map_typed(&emap, e, 3, dims, ebox, Cvt<E>::kTma, 2);
    if (!rc) rc = make_tensor_map_typed(&rmap, rhs, 3, dims, rbox, Cvt<E>::kTma, 2);
    if (!rc) rc = make_tensor_map_typed(&omap, eo, 3, dims, obox, Cvt<E>::kTma, 2);
    if (rc) return rc;
    Geom gg = g;
    int tx_ = tiles_x, ty_ = tiles_y;
    void *args[] = {&emap, &rmap, &omap, &gg, &tx_, &ty_, &zchunk, &items};
    ST_CUDA(cudaLaunchKernel(fn, dim3(grid), dim3(S::THREADS), args, S::SMEM_BYTES, s));
    return STENCIL_OK;
}

// The R = 4 correction sweep on the tensor cores unless the environment
// variable STENCIL_LP_MMA is 0 (then with the per-term mixed-precision adds).
bool lp_mma_enabled() {
    static const bool on = [] {
        const char *v = std::getenv("STENCIL_LP_MMA");
        return !(v && v[0] == '0' && v[1] == 0);
    }();
    return on;
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
        case 4: return lp_mma_enabled() ? run_lp_tc3<E, 13>(g, e, eo, rhs, s) : run_lp<E, 4>(g, e, eo, rhs, s);
        default: return fail(STENCIL_EUNSUPPORTED, "low-precision stream kernel: R=%d", g.radius);
    }
}

template int launch_lp_stream<__nv_bfloat16>(const Geom &, const __nv_bfloat16 *, __nv_bfloat16 *,
                                             const __nv_bfloat16 *, cudaStream_t);
template int launch_lp_stream<__half>(const Geom &, const __half *, __half *, const __half *,
                                      cudaStream_t);

}  // namespace st

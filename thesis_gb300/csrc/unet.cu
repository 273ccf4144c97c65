// unet.cu -- kernels of the learned-warm-start U-Net (include/unet.h).
//
// Convolutions are implicit GEMMs on the BF16 tensor cores with FP32
// accumulation (warp-level mma.sync.m16n8k16; operands staged in shared
// memory by cp.async, fragments loaded with ldmatrix):
//   forward / data gradient:  M = pixels, N = output channels, K = 9 x input
//     channels (taps outer, 32-channel chunks inner), zero padding by
//     cp.async zero-fill;
//   weight gradient:          M = output channels, N = input channels, K =
//     pixels (split across blocks, FP32 atomics), one tap per grid slice.
// Everything else (pooling, upsampling, ReLU gradient, head, loss, Adam,
// features) is bandwidth-bound element-wise work on 16-byte vectors.
#include <cuda_bf16.h>

#include "../../include/unet.h"
#include "host.hpp"

namespace st {
namespace {

typedef __nv_bfloat16 bf16;

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, bool valid) {
    const uint32_t s = smem_u32(smem);
    const int n = valid ? 16 : 0;  // zero-fill when the source is outside the tensor
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(s), "l"(gmem), "r"(n)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t &r0, uint32_t &r1, uint32_t &r2,
                                        uint32_t &r3) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(addr));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t addr, uint32_t &r0, uint32_t &r1, uint32_t &r2,
                                          uint32_t &r3) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(addr));
}
__device__ __forceinline__ void mma16816(float *d, const uint32_t *a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, "
        "{%8, %9}, {%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

struct Act {
    bf16 *p;
    int n, h, w, cs, co, c;
};

Act to_act(const unet_act &a) { return {static_cast<bf16 *>(a.ptr), a.n, a.h, a.w, a.c_stride, a.c_off, a.c}; }

// ---------------------------------------------------------------------------
// 3x3 convolution, forward (also the data gradient with flipped weights).
// Block: 128 threads = 2 x 2 warps; tile BM = 128 pixels x BN output channels,
// K chunk BK = 32 input channels of one tap; two cp.async stages.
// ---------------------------------------------------------------------------
constexpr int BM = 128, BK = 32, PITCH = BK + 8;  // 80-byte rows: conflict-free ldmatrix

template <int BN>
__global__ void __launch_bounds__(128)
    k_conv3x3(Act x, const bf16 *__restrict__ w, const float *__restrict__ bias, Act y, int relu,
              int dil) {
    __shared__ __align__(128) bf16 As[2][BM][PITCH];
    __shared__ __align__(128) bf16 Bs[2][BN][PITCH];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int wm = warp & 1, wn = warp >> 1;
    const long long P = (long long)x.n * x.h * x.w;
    const long long m0 = (long long)blockIdx.x * BM;
    const int n0 = blockIdx.y * BN;
    const int cin = x.c, cout = y.c;
    const int nc = cin / BK, KB = 9 * nc;
    // Rows this thread loads for A: idx = tid + 128*i, row = idx / 4, part = idx % 4.
    int a_n[4], a_y[4], a_x[4];
    bool a_ok[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int row = (tid + 128 * i) >> 2;
        const long long p = m0 + row;
        a_ok[i] = p < P;
        const long long pp = a_ok[i] ? p : 0;
        a_x[i] = (int)(pp % x.w);
        a_y[i] = (int)((pp / x.w) % x.h);
        a_n[i] = (int)(pp / ((long long)x.w * x.h));
    }
    auto load = [&](int kb, int st) {
        const int tap = kb / nc, c0 = (kb % nc) * BK;
        const int dy = (tap / 3 - 1) * dil, dx = (tap % 3 - 1) * dil;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int idx = tid + 128 * i, row = idx >> 2, part = idx & 3;
            const int yy = a_y[i] + dy, xx = a_x[i] + dx;
            const bool v = a_ok[i] && yy >= 0 && yy < x.h && xx >= 0 && xx < x.w;
            const bf16 *src = x.p + (((long long)a_n[i] * x.h + (v ? yy : 0)) * x.w + (v ? xx : 0)) * x.cs +
                              x.co + c0 + part * 8;
            cp_async16(&As[st][row][part * 8], src, v);
        }
#pragma unroll
        for (int i = 0; i < (BN * 4) / 128; ++i) {
            const int idx = tid + 128 * i, row = idx >> 2, part = idx & 3;
            const int co = n0 + row;
            const bool v = co < cout;
            const bf16 *src = w + ((long long)(v ? co : 0) * 9 + tap) * cin + c0 + part * 8;
            cp_async16(&Bs[st][row][part * 8], src, v);
        }
        cp_async_commit();
    };
    constexpr int NT = BN / 16;  // n8 tiles per warp (warp covers BN/2 channels)
    float acc[4][NT][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < NT; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.f;
    load(0, 0);
    for (int kb = 0; kb < KB; ++kb) {
        const int st = kb & 1;
        cp_async_wait_all();
        __syncthreads();
        if (kb + 1 < KB) load(kb + 1, st ^ 1);
#pragma unroll
        for (int ks = 0; ks < BK; ks += 16) {
            uint32_t af[4][4];
#pragma unroll
            for (int mi = 0; mi < 4; ++mi) {
                const int row = wm * 64 + mi * 16 + (lane & 7) + 8 * ((lane >> 3) & 1);
                const int col = ks + 8 * (lane >> 4);
                ldsm_x4(smem_u32(&As[st][row][col]), af[mi][0], af[mi][1], af[mi][2], af[mi][3]);
            }
#pragma unroll
            for (int nj = 0; nj < NT / 2; ++nj) {
                const int nrow = wn * (BN / 2) + nj * 16 + (lane & 7) + 8 * (lane >> 4);
                const int col = ks + 8 * ((lane >> 3) & 1);
                uint32_t b0, b1, b2, b3;
                ldsm_x4(smem_u32(&Bs[st][nrow][col]), b0, b1, b2, b3);
#pragma unroll
                for (int mi = 0; mi < 4; ++mi) {
                    mma16816(acc[mi][2 * nj], af[mi], b0, b1);
                    mma16816(acc[mi][2 * nj + 1], af[mi], b2, b3);
                }
            }
        }
        __syncthreads();
    }
    // Epilogue: bias, ReLU, BF16 pairs.
#pragma unroll
    for (int mi = 0; mi < 4; ++mi)
#pragma unroll
        for (int nj = 0; nj < NT; ++nj)
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
                const long long p = m0 + wm * 64 + mi * 16 + (lane >> 2) + 8 * hh;
                const int co = n0 + wn * (BN / 2) + nj * 8 + (lane & 3) * 2;
                if (p >= P || co >= cout) continue;
                float v0 = acc[mi][nj][2 * hh], v1 = acc[mi][nj][2 * hh + 1];
                if (bias) { v0 += bias[co]; v1 += bias[co + 1]; }
                if (relu) { v0 = fmaxf(v0, 0.f); v1 = fmaxf(v1, 0.f); }
                *reinterpret_cast<__nv_bfloat162 *>(y.p + p * y.cs + y.co + co) =
                    __floats2bfloat162_rn(v0, v1);
            }
}

// ---------------------------------------------------------------------------
// 3x3 convolution, forward / data gradient, on the 5th-generation tensor
// cores: tcgen05.mma (kind::f16, BF16 operands, FP32 accumulator in tensor
// memory), issued by one thread, completion tracked by tcgen05.commit on an
// mbarrier per shared-memory stage.
//   D[128 pixels x BN channels] (TMEM, BN columns) += A[128 x 16] B[BN x 16]^T
// per instruction; K runs over (tap, 32-channel chunk), two instructions per
// chunk.  A (the shifted input pixels, zero outside the image) and B (the
// weights of one tap and chunk) are staged by cp.async into a ring of
// TC_STAGES buffers in the canonical K-major layout without swizzle: 8-row x
// 16-byte core matrices, 128 bytes apart along K (leading byte offset) and
// 512 bytes apart along M/N (stride byte offset).  The epilogue reads the
// accumulator with tcgen05.ld (warp w owns TMEM lanes 32w..32w+31 = pixels),
// adds the bias, applies ReLU and stores BF16.  Every mbarrier wait is
// bounded; a CTA that gives up waits (bounded) for its issued MMAs and frees
// its TMEM.
// ---------------------------------------------------------------------------
// shared-memory stages: more for wide tiles, fewer (more resident CTAs) for narrow ones
template <int BN>
__host__ __device__ constexpr int tc_stages() { return BN >= 128 ? 6 : (BN >= 64 ? 4 : 3); }
constexpr int TC_A_BYTES = BM * BK * 2;  // 8 KiB per stage

__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr) {
    // start address, leading byte offset 128 (K), stride byte offset 512
    // (M/N), descriptor version 1, no swizzle
    return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)(128 >> 4) << 16) |
           ((uint64_t)(512 >> 4) << 32) | (1ull << 46);
}

template <int BN>
__device__ __forceinline__ constexpr uint32_t umma_idesc() {
    // D FP32, A and B BF16, both K-major, N = BN, M = 128
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

template <int BN>
__global__ void __launch_bounds__(160)
    k_conv3x3_tc(Act x, const bf16 *__restrict__ w, const float *__restrict__ bias, Act y, int relu,
                 int dil) {
    // warps 0-3: cp.async producers, then the epilogue (TMEM lanes 32w..32w+31);
    // warp 4: one thread issues the MMAs
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    constexpr int B_BYTES = BN * BK * 2;
    constexpr int TC_STAGES = tc_stages<BN>();
    constexpr int LAG = TC_STAGES - 2;  // chunks in flight per producer before it signals
    unsigned char *base = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(tc_smem) + 1023) & ~static_cast<uintptr_t>(1023));
    unsigned char *As = base;
    unsigned char *Bs = base + TC_STAGES * TC_A_BYTES;
    uint64_t *full = reinterpret_cast<uint64_t *>(Bs + TC_STAGES * B_BYTES);
    uint64_t *done = full + TC_STAGES;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(done + TC_STAGES);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long long P = (long long)x.n * x.h * x.w;
    const long long m0 = (long long)blockIdx.x * BM;
    const int n0 = blockIdx.y * BN;
    const int cin = x.c, cout = y.c;
    const int nc = cin / BK, KB = 9 * nc;

    if (tid == 0) {
        for (int s = 0; s < TC_STAGES; ++s) {
            mbar_init(&full[s], 128);
            mbar_init(&done[s], 1);
        }
        fence_mbar_init();
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"(BN) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    bool ok = true;

    if (warp < 4) {
        // ---------------- producers ----------------
        int a_n[4], a_y[4], a_x[4];
        bool a_ok[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int row = (tid + 128 * i) >> 2;
            const long long p = m0 + row;
            a_ok[i] = p < P;
            const long long pp = a_ok[i] ? p : 0;
            a_x[i] = (int)(pp % x.w);
            a_y[i] = (int)((pp / x.w) % x.h);
            a_n[i] = (int)(pp / ((long long)x.w * x.h));
        }
        int signalled = 0;  // chunks whose copies this thread has reported complete
        for (int k = 0; k < KB; ++k) {
            const int st = k % TC_STAGES;
            // the MMAs of chunk k - TC_STAGES read this stage last
            if (k >= TC_STAGES && !mbar_wait_bounded(&done[st], ((k - TC_STAGES) / TC_STAGES) & 1)) {
                ok = false;
                break;
            }
            const int tap = k / nc, c0 = (k % nc) * BK;
            const int dy = (tap / 3 - 1) * dil, dx = (tap % 3 - 1) * dil;
            unsigned char *a = As + st * TC_A_BYTES;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int idx = tid + 128 * i, row = idx >> 2, part = idx & 3;
                const int yy = a_y[i] + dy, xx = a_x[i] + dx;
                const bool v = a_ok[i] && yy >= 0 && yy < x.h && xx >= 0 && xx < x.w;
                const bf16 *src = x.p + (((long long)a_n[i] * x.h + (v ? yy : 0)) * x.w + (v ? xx : 0)) * x.cs +
                                  x.co + c0 + part * 8;
                cp_async16(a + (row >> 3) * 512 + part * 128 + (row & 7) * 16, src, v);
            }
            unsigned char *b = Bs + st * B_BYTES;
#pragma unroll
            for (int i = 0; i < (BN * 4) / 128; ++i) {
                const int idx = tid + 128 * i, row = idx >> 2, part = idx & 3;
                const int co = n0 + row;
                const bool v = co < cout;
                const bf16 *src = w + ((long long)(v ? co : 0) * 9 + tap) * cin + c0 + part * 8;
                cp_async16(b + (row >> 3) * 512 + part * 128 + (row & 7) * 16, src, v);
            }
            cp_async_commit();
            if (k >= LAG) {
                // chunk k - LAG has landed: make it visible to the async proxy, report it
                asm volatile("cp.async.wait_group %0;" ::"n"(LAG) : "memory");
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_arrive(&full[(k - LAG) % TC_STAGES]);
                signalled = k - LAG + 1;
            }
        }
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        if (ok)
            for (int k = signalled; k < KB; ++k) mbar_arrive(&full[k % TC_STAGES]);
    } else if (lane == 0) {
        // ---------------- MMA issuer ----------------
        constexpr uint32_t IDESC = umma_idesc<BN>();
        int issued = 0;
        for (int k = 0; k < KB; ++k) {
            const int st = k % TC_STAGES;
            if (!mbar_wait_bounded(&full[st], (k / TC_STAGES) & 1)) { ok = false; break; }
            tc_fence_after();
            const uint32_t a = smem_u32(As + st * TC_A_BYTES), b = smem_u32(Bs + st * B_BYTES);
#pragma unroll
            for (int j = 0; j < BK / 16; ++j) {
                const uint64_t ad = umma_desc(a + j * 256), bd = umma_desc(b + j * 256);
                const uint32_t acc = (k > 0 || j > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(IDESC), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&done[st]))
                         : "memory");
            issued = k + 1;
        }
        // every issued MMA has completed once the last commit has arrived
        if (issued > 0 &&
            !mbar_wait_bounded(&done[(issued - 1) % TC_STAGES], ((issued - 1) / TC_STAGES) & 1))
            ok = false;
        if (issued < KB) ok = false;
    }
    tc_fence_before();
    ok = __syncthreads_and(ok);
    tc_fence_after();
    if (ok && warp < 4) {
        const long long p = m0 + warp * 32 + lane;
#pragma unroll
        for (int c = 0; c < BN; c += 8) {
            uint32_t r[8];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                  "=r"(r[7])
                : "r"(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            const int co = n0 + c;
            if (p < P && co < cout) {
                float v[8];
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    v[e] = __uint_as_float(r[e]) + (bias ? bias[co + e] : 0.f);
                    if (relu) v[e] = fmaxf(v[e], 0.f);
                }
                uint4 q;
                __nv_bfloat162 h0 = __floats2bfloat162_rn(v[0], v[1]), h1 = __floats2bfloat162_rn(v[2], v[3]);
                __nv_bfloat162 h2 = __floats2bfloat162_rn(v[4], v[5]), h3 = __floats2bfloat162_rn(v[6], v[7]);
                q.x = *reinterpret_cast<uint32_t *>(&h0);
                q.y = *reinterpret_cast<uint32_t *>(&h1);
                q.z = *reinterpret_cast<uint32_t *>(&h2);
                q.w = *reinterpret_cast<uint32_t *>(&h3);
                *reinterpret_cast<uint4 *>(y.p + p * y.cs + y.co + co) = q;
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN) : "memory");
    }
}

// ---------------------------------------------------------------------------
// The same convolution with TMA-fed operands (grids whose 128-pixel tiles are
// whole image rows or 128-pixel runs of one row: W a power of two, or a
// multiple of 128).  One thread streams each K chunk as two tensor-map loads
// -- a 4-D box of 32 channels x the tile's pixels shifted by the tap (its
// out-of-bounds cells arrive as zeros, which is the convolution's padding)
// and a 3-D box of the weights -- with 64-byte swizzle, which is the layout
// the UMMA descriptors below describe; one thread issues the MMAs; 4 warps
// run the epilogue.  Warps: 0-3 epilogue, 4 TMA producer, 5 MMA issuer.
// ---------------------------------------------------------------------------
constexpr int TMA_STAGES = 6;

__device__ __forceinline__ uint64_t umma_desc_sw64(uint32_t saddr) {
    // K-major, 64-byte swizzle: 8-row groups 512 bytes apart, version 1
    return (uint64_t)((saddr >> 4) & 0x3FFF) | (1ull << 16) | ((uint64_t)(512 >> 4) << 32) |
           (1ull << 46) | (4ull << 61);
}

__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, uint64_t *bar, int c0,
                                            int c1, int c2, int c3) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%3, %4, %5, %6}], [%2];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2), "r"(c3)
        : "memory");
}

template <int BN>
__global__ void __launch_bounds__(192)
    k_conv3x3_tma(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap wmap,
                  const float *__restrict__ bias, Act y, int cin, int H, int W, int tile_w, int relu,
                  int dil) {
    extern __shared__ __align__(1024) unsigned char tm_smem[];
    constexpr int B_BYTES = BN * BK * 2;
    constexpr int STAGE = TC_A_BYTES + B_BYTES;
    unsigned char *base = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(tm_smem) + 1023) & ~static_cast<uintptr_t>(1023));
    uint64_t *full = reinterpret_cast<uint64_t *>(base + TMA_STAGES * STAGE);
    uint64_t *empty = full + TMA_STAGES;
    uint64_t *accd = empty + TMA_STAGES;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(accd + 1);
    int *bad = reinterpret_cast<int *>(tslot + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long long m0 = (long long)blockIdx.x * BM;
    const int n0 = blockIdx.y * BN;
    const int nc = cin / BK, KB = 9 * nc;
    // tile origin: image n, row h0, column w0 (tile = 128 / tile_w rows of tile_w pixels)
    const int n = (int)(m0 / ((long long)H * W));
    const int h0 = (int)((m0 / W) % H), w0 = (int)(m0 % W);

    if (tid == 0) {
        prefetch_tensormap(&xmap);
        prefetch_tensormap(&wmap);
        for (int s = 0; s < TMA_STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(accd, 1);
        *bad = 0;
        fence_mbar_init();
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"(BN) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    if (warp == 4) {
        if (lane == 0) {
            for (int k = 0; k < KB; ++k) {
                const int st = k % TMA_STAGES;
                if (k >= TMA_STAGES && !mbar_wait_bounded(&empty[st], ((k / TMA_STAGES) - 1) & 1)) {
                    *bad = 1;
                    break;
                }
                const int tap = k / nc, c0 = (k % nc) * BK;
                const int dy = (tap / 3 - 1) * dil, dx = (tap % 3 - 1) * dil;
                unsigned char *a = base + st * STAGE;
                mbar_arrive_expect_tx(&full[st], STAGE);
                tma_load_4d(a, &xmap, &full[st], c0, w0 + dx, h0 + dy, n);
                tma_load_3d(a + TC_A_BYTES, &wmap, &full[st], c0, tap, n0);
            }
        }
    } else if (warp == 5) {
        if (lane == 0) {
            constexpr uint32_t IDESC = umma_idesc<BN>();
            for (int k = 0; k < KB; ++k) {
                const int st = k % TMA_STAGES;
                if (!mbar_wait_bounded(&full[st], (k / TMA_STAGES) & 1)) {
                    *bad = 1;
                    break;
                }
                tc_fence_after();
                const uint32_t a = smem_u32(base + st * STAGE), b = a + TC_A_BYTES;
#pragma unroll
                for (int j = 0; j < BK / 16; ++j) {
                    const uint64_t ad = umma_desc_sw64(a + j * 32), bd = umma_desc_sw64(b + j * 32);
                    const uint32_t acc = (k > 0 || j > 0) ? 1u : 0u;
                    asm volatile(
                        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                        "l"(ad), "l"(bd), "r"(IDESC), "r"(acc)
                        : "memory");
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 smem_u32(&empty[st]))
                             : "memory");
            }
            // arrives once every MMA issued above has completed
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(accd))
                         : "memory");
        }
    } else {
        // epilogue warps 0-3: TMEM lanes 32w .. 32w+31 = pixels m0 + 32w + lane
        const bool done = mbar_wait_bounded(accd, 0);
        tc_fence_after();
        if (done && !*reinterpret_cast<volatile int *>(bad)) {
            const long long p = m0 + warp * 32 + lane;
#pragma unroll
            for (int c = 0; c < BN; c += 8) {
                uint32_t r[8];
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                      "=r"(r[7])
                    : "r"(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                const int co = n0 + c;
                float v[8];
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    v[e] = __uint_as_float(r[e]) + (bias ? bias[co + e] : 0.f);
                    if (relu) v[e] = fmaxf(v[e], 0.f);
                }
                uint4 q;
                __nv_bfloat162 h0v = __floats2bfloat162_rn(v[0], v[1]), h1v = __floats2bfloat162_rn(v[2], v[3]);
                __nv_bfloat162 h2v = __floats2bfloat162_rn(v[4], v[5]), h3v = __floats2bfloat162_rn(v[6], v[7]);
                q.x = *reinterpret_cast<uint32_t *>(&h0v);
                q.y = *reinterpret_cast<uint32_t *>(&h1v);
                q.z = *reinterpret_cast<uint32_t *>(&h2v);
                q.w = *reinterpret_cast<uint32_t *>(&h3v);
                *reinterpret_cast<uint4 *>(y.p + p * y.cs + y.co + co) = q;
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN) : "memory");
    }
}

template <int BN>
constexpr int tma_smem_bytes() {
    return TMA_STAGES * (TC_A_BYTES + BN * BK * 2) + (2 * TMA_STAGES + 1) * 8 + 16 + 1024;
}

// ---------------------------------------------------------------------------
// Weight gradient on tcgen05:
//   dW[co][tap][ci] += sum_p dy[p][co] x[p + tap][ci]
// as per-tap GEMMs D[co][ci] (M = 128 output channels, N = BN input
// channels) with K = pixels in 32-pixel chunks (a run of one image row),
// accumulated in TMEM over the CTA's slice of the pixels and added to dW
// with FP32 atomics.  Both operands must be K-major (pixels contiguous), so
// dy and x are first transposed into channel-major copies (k_to_cmajor) in
// the caller's workspace; a chunk is then one 4-D tensor-map box per operand
// (the x box shifted by the tap, out-of-bounds zeros = the padding), 64-byte
// swizzle, the same UMMA descriptors as the forward kernel.  Warps: 0-3
// epilogue, 4 TMA producer, 5 MMA issuer.
// ---------------------------------------------------------------------------
// out[c][p] = view[p shifted by dx columns][c], zero where the shifted
// column leaves the image (32 x 32 tiles through shared memory; W % 32 == 0,
// so a 32-pixel tile lies in one image row).  The shift is applied here, not
// by the tensor map, because a TMA box may only start at a 16-byte aligned
// innermost coordinate and the pixels are the innermost dimension.
__global__ void __launch_bounds__(256) k_to_cmajor(Act a, bf16 *__restrict__ out, long long P, int W, int dx) {
    // tile: 64 pixels x 32 channels; 16-byte loads (8 channels of a pixel)
    // and 16-byte stores (8 pixels of a channel)
    __shared__ __align__(16) bf16 t[32][64 + 8];
    const long long p0 = (long long)blockIdx.x * 64;
    const int c0 = blockIdx.y * 32;
    const int tid = threadIdx.x;
    {
        const int r = tid >> 2, q = tid & 3;
        const long long p = p0 + r;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (p < P) {
            const int ws = (int)(p % W) + dx;
            if (ws >= 0 && ws < W)
                v = *reinterpret_cast<const uint4 *>(a.p + (p + dx) * a.cs + a.co + c0 + 8 * q);
        }
        const bf16 *e = reinterpret_cast<const bf16 *>(&v);
#pragma unroll
        for (int k = 0; k < 8; ++k) t[8 * q + k][r] = e[k];
    }
    __syncthreads();
    {
        const int c = tid >> 3, q = tid & 7;
        const long long p = p0 + 8 * q;
        if (p + 8 <= P) {
            *reinterpret_cast<uint4 *>(out + (long long)(c0 + c) * P + p) =
                *reinterpret_cast<const uint4 *>(&t[c][8 * q]);
        } else {
            for (int k = 0; k < 8 && p + k < P; ++k) out[(long long)(c0 + c) * P + p + k] = t[c][8 * q + k];
        }
    }
}

__device__ __forceinline__ void tma_load_5d(void *dst, const CUtensorMap *map, uint64_t *bar, int c0,
                                            int c1, int c2, int c3, int c4) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%3, %4, %5, %6, %7}], [%2];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2), "r"(c3),
        "r"(c4)
        : "memory");
}

template <int BN>
__global__ void __launch_bounds__(192)
    k_wgrad_tma(const __grid_constant__ CUtensorMap gmap, const __grid_constant__ CUtensorMap xmap,
                float *__restrict__ dw, int cin, int cout, int H, int W, int dil, int chunks_per_cta,
                long long nchunks) {
    extern __shared__ __align__(1024) unsigned char wg_smem[];
    constexpr int A_BYTES = BM * BK * 2;
    constexpr int B_BYTES = BN * BK * 2;
    constexpr int STAGE = A_BYTES + B_BYTES;
    unsigned char *base = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(wg_smem) + 1023) & ~static_cast<uintptr_t>(1023));
    uint64_t *full = reinterpret_cast<uint64_t *>(base + TMA_STAGES * STAGE);
    uint64_t *empty = full + TMA_STAGES;
    uint64_t *accd = empty + TMA_STAGES;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(accd + 1);
    int *bad = reinterpret_cast<int *>(tslot + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int co0 = blockIdx.x * BM, ci0 = blockIdx.y * BN;
    const int tap = blockIdx.z % 9;
    const long long k0 = (long long)(blockIdx.z / 9) * chunks_per_cta;
    const int KB = (int)min((long long)chunks_per_cta, nchunks - k0);
    const int dy = (tap / 3 - 1) * dil;
    const int rowchunks = W / BK;  // 32-pixel chunks per image row

    if (tid == 0) {
        prefetch_tensormap(&gmap);
        prefetch_tensormap(&xmap);
        for (int s = 0; s < TMA_STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(accd, 1);
        *bad = 0;
        fence_mbar_init();
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"(BN) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    if (warp == 4) {
        if (lane == 0) {
            for (int k = 0; k < KB; ++k) {
                const int st = k % TMA_STAGES;
                if (k >= TMA_STAGES && !mbar_wait_bounded(&empty[st], ((k / TMA_STAGES) - 1) & 1)) {
                    *bad = 1;
                    break;
                }
                const long long ch = k0 + k;  // chunk = (n, h, 32-pixel run of the row)
                const int wc = (int)(ch % rowchunks);
                const long long r = ch / rowchunks;
                const int h = (int)(r % H), n = (int)(r / H);
                unsigned char *a = base + st * STAGE;
                mbar_arrive_expect_tx(&full[st], STAGE);
                tma_load_4d(a, &gmap, &full[st], wc * BK, h, n, co0);
                // x copy shifted by this tap's column offset (index tap % 3), row shift by coordinate
                tma_load_5d(a + A_BYTES, &xmap, &full[st], wc * BK, h + dy, n, ci0, tap % 3);
            }
        }
    } else if (warp == 5) {
        if (lane == 0) {
            constexpr uint32_t IDESC = umma_idesc<BN>();
            for (int k = 0; k < KB; ++k) {
                const int st = k % TMA_STAGES;
                if (!mbar_wait_bounded(&full[st], (k / TMA_STAGES) & 1)) {
                    *bad = 1;
                    break;
                }
                tc_fence_after();
                const uint32_t a = smem_u32(base + st * STAGE), b = a + A_BYTES;
#pragma unroll
                for (int j = 0; j < BK / 16; ++j) {
                    const uint64_t ad = umma_desc_sw64(a + j * 32), bd = umma_desc_sw64(b + j * 32);
                    const uint32_t acc = (k > 0 || j > 0) ? 1u : 0u;
                    asm volatile(
                        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                        "l"(ad), "l"(bd), "r"(IDESC), "r"(acc)
                        : "memory");
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 smem_u32(&empty[st]))
                             : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(accd))
                         : "memory");
        }
    } else {
        const bool done = mbar_wait_bounded(accd, 0);
        tc_fence_after();
        if (done && KB > 0 && !*reinterpret_cast<volatile int *>(bad)) {
            const int co = co0 + warp * 32 + lane;
#pragma unroll
            for (int c = 0; c < BN; c += 8) {
                uint32_t r[8];
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                      "=r"(r[7])
                    : "r"(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (co < cout) {
                    float *d = dw + ((long long)co * 9 + tap) * cin + ci0 + c;
#pragma unroll
                    for (int e = 0; e < 8; ++e) atomicAdd(d + e, __uint_as_float(r[e]));
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN) : "memory");
    }
}

template <int BN>
constexpr int tc_smem_bytes() {
    return tc_stages<BN>() * (TC_A_BYTES + BN * BK * 2) + 2 * tc_stages<BN>() * 8 + 16 + 1024;
}

// ---------------------------------------------------------------------------
// Weight gradient: dW[co][tap][ci] += sum_p dy[p][co] x[p + tap][ci].
// Block: 128 threads = 2 x 2 warps, tile 64 (co) x 64 (ci), K = pixels in
// chunks of 32 from this block's pixel range; grid.z = tap.
// ---------------------------------------------------------------------------
constexpr int WK = 32, WPITCH = 64 + 8;

__global__ void __launch_bounds__(128)
    k_wgrad(Act x, Act dy, float *__restrict__ dw, long long pix_per_block, int dil) {
    __shared__ __align__(128) bf16 As[2][WK][WPITCH];  // [p][co]
    __shared__ __align__(128) bf16 Bs[2][WK][WPITCH];  // [p][ci]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int wm = warp & 1, wn = warp >> 1;
    const int co0 = blockIdx.x * 64, ci0 = blockIdx.y * 64;
    const int tap = blockIdx.z % 9, split = blockIdx.z / 9;
    const int ddy = (tap / 3 - 1) * dil, ddx = (tap % 3 - 1) * dil;
    const long long P = (long long)x.n * x.h * x.w;
    const long long pb = split * pix_per_block, pe = min(P, pb + pix_per_block);
    if (pb >= pe) return;
    const int KB = (int)((pe - pb + WK - 1) / WK);
    auto load = [&](int kb, int st) {
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const int idx = tid + 128 * i, row = idx >> 3, part = idx & 7;
            const long long p = pb + (long long)kb * WK + row;
            const bool pv = p < pe;
            const long long pp = pv ? p : 0;
            // dy row
            const int co = co0 + part * 8;
            const bool av = pv && co < dy.c;
            cp_async16(&As[st][row][part * 8], dy.p + pp * dy.cs + dy.co + (av ? co : 0), av);
            // shifted x row
            const int xx = (int)(pp % x.w) + ddx;
            const int yy = (int)((pp / x.w) % x.h) + ddy;
            const int nn = (int)(pp / ((long long)x.w * x.h));
            const int ci = ci0 + part * 8;
            const bool bv = pv && ci < x.c && xx >= 0 && xx < x.w && yy >= 0 && yy < x.h;
            const bf16 *src = x.p + (((long long)nn * x.h + (bv ? yy : 0)) * x.w + (bv ? xx : 0)) * x.cs +
                              x.co + (bv ? ci : 0);
            cp_async16(&Bs[st][row][part * 8], src, bv);
        }
        cp_async_commit();
    };
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.f;
    load(0, 0);
    for (int kb = 0; kb < KB; ++kb) {
        const int st = kb & 1;
        cp_async_wait_all();
        __syncthreads();
        if (kb + 1 < KB) load(kb + 1, st ^ 1);
#pragma unroll
        for (int ks = 0; ks < WK; ks += 16) {
            uint32_t af[2][4];
#pragma unroll
            for (int mi = 0; mi < 2; ++mi) {
                const int q = lane >> 3, r = lane & 7;
                const int krow = ks + r + 8 * (q >> 1);
                const int mcol = wm * 32 + mi * 16 + 8 * (q & 1);
                ldsm_x4_t(smem_u32(&As[st][krow][mcol]), af[mi][0], af[mi][1], af[mi][2], af[mi][3]);
            }
#pragma unroll
            for (int nj = 0; nj < 2; ++nj) {
                const int q = lane >> 3, r = lane & 7;
                const int krow = ks + r + 8 * (q & 1);
                const int ncol = wn * 32 + nj * 16 + 8 * (q >> 1);
                uint32_t b0, b1, b2, b3;
                ldsm_x4_t(smem_u32(&Bs[st][krow][ncol]), b0, b1, b2, b3);
#pragma unroll
                for (int mi = 0; mi < 2; ++mi) {
                    mma16816(acc[mi][2 * nj], af[mi], b0, b1);
                    mma16816(acc[mi][2 * nj + 1], af[mi], b2, b3);
                }
            }
        }
        __syncthreads();
    }
    const int cin = x.c;
#pragma unroll
    for (int mi = 0; mi < 2; ++mi)
#pragma unroll
        for (int nj = 0; nj < 4; ++nj)
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
                const int co = co0 + wm * 32 + mi * 16 + (lane >> 2) + 8 * hh;
                const int ci = ci0 + wn * 32 + nj * 8 + (lane & 3) * 2;
                if (co >= dy.c || ci >= cin) continue;
                float *d = dw + ((long long)co * 9 + tap) * cin + ci;
                atomicAdd(d, acc[mi][nj][2 * hh]);
                atomicAdd(d + 1, acc[mi][nj][2 * hh + 1]);
            }
}

// Bias gradient: db[c] += sum_p dy[p][c]; one block per 32-channel group.
__global__ void k_bias_grad(Act dy, float *db) {
    __shared__ float sh[8][33];
    const int c = blockIdx.y * 32 + (threadIdx.x & 31);
    const int r = threadIdx.x >> 5;  // 8 warps
    const long long P = (long long)dy.n * dy.h * dy.w;
    float s = 0.f;
    if (c < dy.c)
        for (long long p = blockIdx.x * 8 + r; p < P; p += (long long)gridDim.x * 8)
            s += __bfloat162float(dy.p[p * dy.cs + dy.co + c]);
    sh[r][threadIdx.x & 31] = s;
    __syncthreads();
    if (r == 0 && c < dy.c) {
        float t = 0.f;
        for (int k = 0; k < 8; ++k) t += sh[k][threadIdx.x];
        atomicAdd(&db[c], t);
    }
}

__global__ void k_flip(const bf16 *__restrict__ w, bf16 *__restrict__ wt, int cout, int cin) {
    const long long n = (long long)cout * 9 * cin;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int ci = (int)(i % cin);
        const int tap = (int)((i / cin) % 9);
        const int co = (int)(i / ((long long)cin * 9));
        // wt[ci][tap'][co] with tap' = 8 - tap (ky -> 2-ky, kx -> 2-kx)
        wt[((long long)ci * 9 + (8 - tap)) * cout + co] = w[i];
    }
}

// Element-wise kernels over 8-channel vectors of a view.
__device__ __forceinline__ long long vec_count(const Act &a) {
    return (long long)a.n * a.h * a.w * (a.c / 8);
}
__device__ __forceinline__ uint4 *vec_at(const Act &a, long long v) {
    const long long p = v / (a.c / 8);
    const int c8 = (int)(v % (a.c / 8));
    return reinterpret_cast<uint4 *>(a.p + p * a.cs + a.co + c8 * 8);
}

__global__ void k_relu_bwd(Act g, Act y) {
    const long long n = vec_count(g);
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n;
         v += (long long)gridDim.x * blockDim.x) {
        uint4 gv = *vec_at(g, v);
        const uint4 yv = *vec_at(y, v);
        __nv_bfloat162 *gp = reinterpret_cast<__nv_bfloat162 *>(&gv);
        const __nv_bfloat162 *yp = reinterpret_cast<const __nv_bfloat162 *>(&yv);
        const __nv_bfloat162 zero = __floats2bfloat162_rn(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float2 yf = __bfloat1622float2(yp[k]);
            float2 gf = __bfloat1622float2(gp[k]);
            gf.x = yf.x > 0.f ? gf.x : 0.f;
            gf.y = yf.y > 0.f ? gf.y : 0.f;
            gp[k] = __float22bfloat162_rn(gf);
        }
        (void)zero;
        *vec_at(g, v) = gv;
    }
}

__global__ void k_add(Act a, Act b) {
    const long long n = vec_count(a);
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n;
         v += (long long)gridDim.x * blockDim.x) {
        uint4 av = *vec_at(a, v);
        const uint4 bv = *vec_at(b, v);
        __nv_bfloat162 *ap = reinterpret_cast<__nv_bfloat162 *>(&av);
        const __nv_bfloat162 *bp = reinterpret_cast<const __nv_bfloat162 *>(&bv);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float2 x = __bfloat1622float2(ap[k]), y = __bfloat1622float2(bp[k]);
            ap[k] = __floats2bfloat162_rn(x.x + y.x, x.y + y.y);
        }
        *vec_at(a, v) = av;
    }
}

// y (h/2 x w/2) = max over 2x2 blocks of x.
__global__ void k_pool_fwd(Act x, Act y) {
    const long long n = vec_count(y);
    const int c8n = y.c / 8;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n;
         v += (long long)gridDim.x * blockDim.x) {
        const int c8 = (int)(v % c8n);
        const long long p = v / c8n;
        const int ox = (int)(p % y.w), oy = (int)((p / y.w) % y.h), nn = (int)(p / ((long long)y.w * y.h));
        float m[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) m[k] = -3.0e38f;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const long long ip = ((long long)nn * x.h + 2 * oy + (q >> 1)) * x.w + 2 * ox + (q & 1);
            const uint4 xv = *reinterpret_cast<const uint4 *>(x.p + ip * x.cs + x.co + c8 * 8);
            const __nv_bfloat162 *xp = reinterpret_cast<const __nv_bfloat162 *>(&xv);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float2 f = __bfloat1622float2(xp[k]);
                m[2 * k] = fmaxf(m[2 * k], f.x);
                m[2 * k + 1] = fmaxf(m[2 * k + 1], f.y);
            }
        }
        uint4 ov;
        __nv_bfloat162 *op = reinterpret_cast<__nv_bfloat162 *>(&ov);
#pragma unroll
        for (int k = 0; k < 4; ++k) op[k] = __floats2bfloat162_rn(m[2 * k], m[2 * k + 1]);
        *reinterpret_cast<uint4 *>(y.p + p * y.cs + y.co + c8 * 8) = ov;
    }
}

// dx = dy routed to the first input of each 2x2 block equal to the max (y).
__global__ void k_pool_bwd(Act x, Act y, Act dy, Act dx) {
    const long long n = vec_count(y);
    const int c8n = y.c / 8;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n;
         v += (long long)gridDim.x * blockDim.x) {
        const int c8 = (int)(v % c8n);
        const long long p = v / c8n;
        const int ox = (int)(p % y.w), oy = (int)((p / y.w) % y.h), nn = (int)(p / ((long long)y.w * y.h));
        const uint4 yv = *reinterpret_cast<const uint4 *>(y.p + p * y.cs + y.co + c8 * 8);
        const uint4 gv = *reinterpret_cast<const uint4 *>(dy.p + p * dy.cs + dy.co + c8 * 8);
        const bf16 *yb = reinterpret_cast<const bf16 *>(&yv);
        const bf16 *gb = reinterpret_cast<const bf16 *>(&gv);
        bool taken[8] = {false, false, false, false, false, false, false, false};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const long long ip = ((long long)nn * x.h + 2 * oy + (q >> 1)) * x.w + 2 * ox + (q & 1);
            const uint4 xv = *reinterpret_cast<const uint4 *>(x.p + ip * x.cs + x.co + c8 * 8);
            const bf16 *xb = reinterpret_cast<const bf16 *>(&xv);
            uint4 ov;
            bf16 *ob = reinterpret_cast<bf16 *>(&ov);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const bool hit = !taken[k] && __bfloat162float(xb[k]) == __bfloat162float(yb[k]);
                taken[k] = taken[k] || hit;
                ob[k] = hit ? gb[k] : __float2bfloat16_rn(0.f);
            }
            *reinterpret_cast<uint4 *>(dx.p + ip * dx.cs + dx.co + c8 * 8) = ov;
        }
    }
}

__global__ void k_up_fwd(Act x, Act y) {
    const long long n = vec_count(y);
    const int c8n = y.c / 8;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n;
         v += (long long)gridDim.x * blockDim.x) {
        const int c8 = (int)(v % c8n);
        const long long p = v / c8n;
        const int ox = (int)(p % y.w), oy = (int)((p / y.w) % y.h), nn = (int)(p / ((long long)y.w * y.h));
        const long long ip = ((long long)nn * x.h + oy / 2) * x.w + ox / 2;
        *reinterpret_cast<uint4 *>(y.p + p * y.cs + y.co + c8 * 8) =
            *reinterpret_cast<const uint4 *>(x.p + ip * x.cs + x.co + c8 * 8);
    }
}

__global__ void k_up_bwd(Act dy, Act dx) {
    const long long n = vec_count(dx);
    const int c8n = dx.c / 8;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n;
         v += (long long)gridDim.x * blockDim.x) {
        const int c8 = (int)(v % c8n);
        const long long p = v / c8n;
        const int ox = (int)(p % dx.w), oy = (int)((p / dx.w) % dx.h), nn = (int)(p / ((long long)dx.w * dx.h));
        float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const long long ip = ((long long)nn * dy.h + 2 * oy + (q >> 1)) * dy.w + 2 * ox + (q & 1);
            const uint4 gv = *reinterpret_cast<const uint4 *>(dy.p + ip * dy.cs + dy.co + c8 * 8);
            const __nv_bfloat162 *gp = reinterpret_cast<const __nv_bfloat162 *>(&gv);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float2 f = __bfloat1622float2(gp[k]);
                s[2 * k] += f.x;
                s[2 * k + 1] += f.y;
            }
        }
        uint4 ov;
        __nv_bfloat162 *op = reinterpret_cast<__nv_bfloat162 *>(&ov);
#pragma unroll
        for (int k = 0; k < 4; ++k) op[k] = __floats2bfloat162_rn(s[2 * k], s[2 * k + 1]);
        *reinterpret_cast<uint4 *>(dx.p + p * dx.cs + dx.co + c8 * 8) = ov;
    }
}

// Head: one warp per pixel group; channel count <= 256 (multiple of 8).
__global__ void k_head_fwd(Act x, const float *__restrict__ w, const float *__restrict__ b,
                           float *__restrict__ y) {
    const long long P = (long long)x.n * x.h * x.w;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < P;
         p += (long long)gridDim.x * blockDim.x) {
        float s = b[0];
        for (int c = 0; c < x.c; c += 8) {
            const uint4 xv = *reinterpret_cast<const uint4 *>(x.p + p * x.cs + x.co + c);
            const __nv_bfloat162 *xp = reinterpret_cast<const __nv_bfloat162 *>(&xv);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float2 f = __bfloat1622float2(xp[k]);
                s = fmaf(f.x, w[c + 2 * k], s);
                s = fmaf(f.y, w[c + 2 * k + 1], s);
            }
        }
        y[p] = s;
    }
}

__global__ void k_head_bwd(Act x, const float *__restrict__ w, const float *__restrict__ dy, Act dx,
                           float *__restrict__ dw, float *__restrict__ db) {
    // block: 256 threads; thread t owns channel t % x.c partial sums for dw.
    __shared__ float sdw[256];
    __shared__ float sdb;
    if (threadIdx.x < 256) sdw[threadIdx.x] = 0.f;
    if (threadIdx.x == 0) sdb = 0.f;
    __syncthreads();
    const long long P = (long long)x.n * x.h * x.w;
    float mydb = 0.f;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < P;
         p += (long long)gridDim.x * blockDim.x) {
        const float g = dy[p];
        mydb += g;
        for (int c = 0; c < x.c; c += 8) {
            const uint4 xv = *reinterpret_cast<const uint4 *>(x.p + p * x.cs + x.co + c);
            const __nv_bfloat162 *xp = reinterpret_cast<const __nv_bfloat162 *>(&xv);
            uint4 ov;
            __nv_bfloat162 *op = reinterpret_cast<__nv_bfloat162 *>(&ov);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float2 f = __bfloat1622float2(xp[k]);
                atomicAdd(&sdw[c + 2 * k], g * f.x);
                atomicAdd(&sdw[c + 2 * k + 1], g * f.y);
                op[k] = __floats2bfloat162_rn(g * w[c + 2 * k], g * w[c + 2 * k + 1]);
            }
            *reinterpret_cast<uint4 *>(dx.p + p * dx.cs + dx.co + c) = ov;
        }
    }
    atomicAdd(&sdb, mydb);
    __syncthreads();
    if (threadIdx.x < x.c) atomicAdd(&dw[threadIdx.x], sdw[threadIdx.x]);
    if (threadIdx.x == 0) atomicAdd(db, sdb);
}

// Features: ch0 border field, ch1 mask, ch2 Coons patch, other channels 0.
__global__ void k_features(const float *__restrict__ f, int n, int h, int w, Act x,
                           float *__restrict__ coons) {
    const long long P = (long long)n * h * w;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < P;
         p += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(p % w), j = (int)((p / w) % h), nn = (int)(p / ((long long)w * h));
        const float *g = f + (long long)nn * h * w;
        const bool bnd = i == 0 || j == 0 || i == w - 1 || j == h - 1;
        const float s = (float)i / (w - 1), t = (float)j / (h - 1);
        const float B = g[i], T = g[(long long)(h - 1) * w + i];
        const float L = g[(long long)j * w], Rr = g[(long long)j * w + w - 1];
        const float c00 = g[0], c10 = g[w - 1], c01 = g[(long long)(h - 1) * w], c11 = g[(long long)h * w - 1];
        float cp = (1 - t) * B + t * T + (1 - s) * L + s * Rr -
                   ((1 - s) * (1 - t) * c00 + s * (1 - t) * c10 + (1 - s) * t * c01 + s * t * c11);
        if (bnd) cp = g[(long long)j * w + i];
        if (coons) coons[p] = cp;
        bf16 *o = x.p + p * x.cs + x.co;
        for (int c = 0; c < x.c; c += 8) {
            uint4 v = make_uint4(0, 0, 0, 0);
            if (c == 0) {
                __nv_bfloat162 *vp = reinterpret_cast<__nv_bfloat162 *>(&v);
                vp[0] = __floats2bfloat162_rn(bnd ? g[(long long)j * w + i] : 0.f, bnd ? 1.f : 0.f);
                vp[1] = __floats2bfloat162_rn(cp, 0.f);
            }
            *reinterpret_cast<uint4 *>(o + c) = v;
        }
    }
}

__global__ void k_mse(const float *__restrict__ out, const float *__restrict__ coons,
                      const float *__restrict__ target, int n, int h, int w, float scale,
                      float *loss, float *__restrict__ dout) {
    const long long P = (long long)n * h * w;
    float s = 0.f;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < P;
         p += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(p % w), j = (int)((p / w) % h);
        const bool bnd = i == 0 || j == 0 || i == w - 1 || j == h - 1;
        float g = 0.f;
        if (!bnd) {
            const float d = coons[p] + out[p] - target[p];
            s += d * d;
            g = 2.f * d * scale;
        }
        dout[p] = g;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, s);
}

__global__ void k_adam(float *p, const float *g, float *m, float *v, bf16 *pb, long long n, float lr,
                       float b1, float b2, float eps, float c1, float c2) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        p[i] = pi;
        if (pb) pb[i] = __float2bfloat16_rn(pi);
    }
}

__global__ void k_assemble(const float *f, const float *coons, const float *out, int n, int h, int w,
                           float *u) {
    const long long P = (long long)n * h * w;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < P;
         p += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(p % w), j = (int)((p / w) % h);
        const bool bnd = i == 0 || j == 0 || i == w - 1 || j == h - 1;
        u[p] = bnd ? f[p] : coons[p] + out[p];
    }
}

// Transfinite (Coons) interpolation of each field's border on its interior,
// the border band copied (the formula of k_features' channel 2).
__global__ void k_coons_fill(const float *__restrict__ f, int n, int h, int w, float *__restrict__ u) {
    const long long P = (long long)n * h * w;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < P;
         p += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(p % w), j = (int)((p / w) % h), nn = (int)(p / ((long long)w * h));
        const float *g = f + (long long)nn * h * w;
        const bool bnd = i == 0 || j == 0 || i == w - 1 || j == h - 1;
        const float s = (float)i / (w - 1), t = (float)j / (h - 1);
        const float B = g[i], T = g[(long long)(h - 1) * w + i];
        const float L = g[(long long)j * w], Rr = g[(long long)j * w + w - 1];
        const float c00 = g[0], c10 = g[w - 1], c01 = g[(long long)(h - 1) * w], c11 = g[(long long)h * w - 1];
        const float cp = (1 - t) * B + t * T + (1 - s) * L + s * Rr -
                         ((1 - s) * (1 - t) * c00 + s * (1 - t) * c10 + (1 - s) * t * c01 + s * t * c11);
        u[p] = bnd ? g[(long long)j * w + i] : cp;
    }
}

// Nearest source index of coarse index k when k = 0..m-1 spans 0..M-1:
// round(k (M-1) / (m-1)), ties up.
__device__ __forceinline__ int nearest_index(int k, int m, int M) {
    return m > 1 ? (int)((2LL * k * (M - 1) + (m - 1)) / (2LL * (m - 1))) : 0;
}

// Coarse h x w problems from fine H x W borders: each coarse border cell
// takes the fine border value at the nearest position; interior zero.
__global__ void k_resample_border(const float *__restrict__ f, int n, int H, int W, int h, int w,
                                  float *__restrict__ c) {
    const long long P = (long long)n * h * w;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < P;
         p += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(p % w), j = (int)((p / w) % h), nn = (int)(p / ((long long)w * h));
        const bool bnd = i == 0 || j == 0 || i == w - 1 || j == h - 1;
        float v = 0.0f;
        if (bnd)
            v = f[(long long)nn * H * W + (long long)nearest_index(j, h, H) * W + nearest_index(i, w, W)];
        c[p] = v;
    }
}

// Fine H x W fields from coarse h x w ones: bilinear interpolation with the
// corner cells aligned (fine index I maps to I (w-1)/(W-1)) on the interior;
// the fine border band is copied from f.
__global__ void k_upsample_bilinear(const float *__restrict__ c, int n, int h, int w,
                                    const float *__restrict__ f, int H, int W, float *__restrict__ u) {
    const long long P = (long long)n * H * W;
    const float sx = W > 1 ? (float)(w - 1) / (float)(W - 1) : 0.0f;
    const float sy = H > 1 ? (float)(h - 1) / (float)(H - 1) : 0.0f;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < P;
         p += (long long)gridDim.x * blockDim.x) {
        const int I = (int)(p % W), J = (int)((p / W) % H), nn = (int)(p / ((long long)W * H));
        if (I == 0 || J == 0 || I == W - 1 || J == H - 1) {
            u[p] = f[p];
            continue;
        }
        const float x = I * sx, y = J * sy;
        const int x0 = min((int)x, w - 2), y0 = min((int)y, h - 2);
        const float ax = x - x0, ay = y - y0;
        const float *g = c + (long long)nn * h * w + (long long)y0 * w + x0;
        const float top = (1.0f - ax) * g[0] + ax * g[1];
        const float bot = (1.0f - ax) * g[w] + ax * g[w + 1];
        u[p] = (1.0f - ay) * top + ay * bot;
    }
}

__global__ void k_to_bf16(const float *s, bf16 *d, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        d[i] = __float2bfloat16_rn(s[i]);
}

int check_act(const unet_act *a, const char *what) {
    if (!a || !a->ptr) return fail(STENCIL_EINVAL, "%s: null view", what);
    if (a->n < 1 || a->h < 1 || a->w < 1 || a->c < 8 || a->c % 8 || a->c_stride % 8 ||
        a->c_off % 8 || a->c_off + a->c > a->c_stride)
        return fail(STENCIL_EINVAL, "%s: bad view (c %d, stride %d, off %d)", what, a->c, a->c_stride, a->c_off);
    if (reinterpret_cast<uintptr_t>(a->ptr) & 15) return fail(STENCIL_EINVAL, "%s: 16-byte alignment", what);
    return STENCIL_OK;
}

int grid_for(long long n) {
    long long b = (n + 255) / 256;
    const long long cap = 16LL * num_sms();
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace
}  // namespace st

using namespace st;

#define CHECK_VIEW(v) \
    do { int rc_ = check_act(v, #v); if (rc_) return rc_; } while (0)
#define STREAM(s) reinterpret_cast<cudaStream_t>(s)

template <int BN>
int launch_conv_tc(const Act &xa, const bf16 *wb, const float *b, const Act &ya, int relu, int dil,
                   long long P, cudaStream_t s) {
    static bool attr[64] = {false};
    const int dev = current_device();
    if (dev >= 0 && dev < 64 && !attr[dev]) {
        ST_CUDA(cudaFuncSetAttribute(k_conv3x3_tc<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     tc_smem_bytes<BN>()));
        attr[dev] = true;
    }
    dim3 grid((unsigned)((P + BM - 1) / BM), ya.c / BN);
    k_conv3x3_tc<BN><<<grid, 160, tc_smem_bytes<BN>(), s>>>(xa, wb, b, ya, relu, dil);
    return cuda_fail(cudaGetLastError(), "conv3x3 (tcgen05) launch");
}

// Tile shape for the TMA engine: 128 pixels = whole rows (W < 128, a power of
// two dividing 128, H a multiple of 128 / W) or a 128-pixel run of one row
// (W a multiple of 128); 0 if neither.
int tma_tile_w(int H, int W) {
    if (W >= 128) return W % 128 == 0 ? 128 : 0;
    if (128 % W == 0 && H % (128 / W) == 0) return W;
    return 0;
}

template <int BN>
int launch_conv_tma(const unet_act *x, const bf16 *wb, const float *b, const Act &ya, int relu, int dil,
                    int tile_w, cudaStream_t s) {
    static bool attr[64] = {false};
    const int dev = current_device();
    if (dev >= 0 && dev < 64 && !attr[dev]) {
        ST_CUDA(cudaFuncSetAttribute(k_conv3x3_tma<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     tma_smem_bytes<BN>()));
        attr[dev] = true;
    }
    const int cin = x->c, cout = ya.c;
    CUtensorMap xm, wm;
    const unsigned long long cs2 = (unsigned long long)x->c_stride * 2;
    const unsigned long long xd[4] = {(unsigned long long)cin, (unsigned long long)x->w,
                                      (unsigned long long)x->h, (unsigned long long)x->n};
    const unsigned long long xs[3] = {cs2, cs2 * x->w, cs2 * x->w * x->h};
    const unsigned xb[4] = {(unsigned)BK, (unsigned)tile_w, (unsigned)(BM / tile_w), 1u};
    const bf16 *xbase = static_cast<const bf16 *>(x->ptr) + x->c_off;
    int rc = make_tensor_map_general(&xm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, xbase, xd, xs, xb,
                                     CU_TENSOR_MAP_SWIZZLE_64B);
    if (rc) return rc;
    const unsigned long long wd[3] = {(unsigned long long)cin, 9ull, (unsigned long long)cout};
    const unsigned long long ws[2] = {(unsigned long long)cin * 2, 9ull * cin * 2};
    const unsigned wbx[3] = {(unsigned)BK, 1u, (unsigned)BN};
    rc = make_tensor_map_general(&wm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, wb, wd, ws, wbx,
                                 CU_TENSOR_MAP_SWIZZLE_64B);
    if (rc) return rc;
    const long long P = (long long)x->n * x->h * x->w;
    dim3 grid((unsigned)(P / BM), cout / BN);
    k_conv3x3_tma<BN><<<grid, 192, tma_smem_bytes<BN>(), s>>>(xm, wm, b, ya, cin, x->h, x->w, tile_w,
                                                              relu, dil);
    return cuda_fail(cudaGetLastError(), "conv3x3 (tcgen05, TMA) launch");
}

extern "C" int unet_conv3x3_fwd_engine(const unet_act *x, const void *w, const float *b,
                                       const unet_act *y, int relu, int dilation, int engine,
                                       stencil_stream_t s) {
    CHECK_VIEW(x);
    CHECK_VIEW(y);
    if (!w) return fail(STENCIL_EINVAL, "null weights");
    if (dilation < 1) return fail(STENCIL_EINVAL, "dilation must be >= 1");
    if (engine < 0 || engine > 2) return fail(STENCIL_EINVAL, "engine must be 0, 1 or 2");
    if (x->c % 32 || y->c % 32) return fail(STENCIL_EINVAL, "channels must be multiples of 32");
    if (x->n != y->n || x->h != y->h || x->w != y->w) return fail(STENCIL_EINVAL, "shape mismatch");
    const long long P = (long long)x->n * x->h * x->w;
    const Act xa = to_act(*x), ya = to_act(*y);
    const bf16 *wb = static_cast<const bf16 *>(w);
    // default: tcgen05 with TMA-fed operands wherever the tiles allow it
    // (measured 1.5-3.4x the mma.sync engine on every U-Net layer: 199 vs 129
    // TFLOP/s at 128^2 x 32 -> 32, 759 vs 222 at 32^2 x 384 -> 128); the
    // cp.async-fed tcgen05 form is slower than mma.sync (operand staging
    // bound), so other shapes use mma.sync
    if (engine == 0) engine = (tma_tile_w(x->h, x->w) && P % BM == 0) ? 1 : 2;
    if (engine == 1) {
        const int tw = tma_tile_w(x->h, x->w);
        if (tw && P % BM == 0) {
            if (y->c % 128 == 0) return launch_conv_tma<128>(x, wb, b, ya, relu, dilation, tw, STREAM(s));
            if (y->c % 64 == 0) return launch_conv_tma<64>(x, wb, b, ya, relu, dilation, tw, STREAM(s));
            return launch_conv_tma<32>(x, wb, b, ya, relu, dilation, tw, STREAM(s));
        }
        if (y->c % 128 == 0) return launch_conv_tc<128>(xa, wb, b, ya, relu, dilation, P, STREAM(s));
        if (y->c % 64 == 0) return launch_conv_tc<64>(xa, wb, b, ya, relu, dilation, P, STREAM(s));
        return launch_conv_tc<32>(xa, wb, b, ya, relu, dilation, P, STREAM(s));
    }
    if (y->c % 64 == 0) {
        dim3 grid((unsigned)((P + BM - 1) / BM), y->c / 64);
        k_conv3x3<64><<<grid, 128, 0, STREAM(s)>>>(xa, wb, b, ya, relu, dilation);
    } else {
        dim3 grid((unsigned)((P + BM - 1) / BM), y->c / 32);
        k_conv3x3<32><<<grid, 128, 0, STREAM(s)>>>(xa, wb, b, ya, relu, dilation);
    }
    return cuda_fail(cudaGetLastError(), "conv3x3 launch");
}

extern "C" int unet_conv3x3_fwd_dil(const unet_act *x, const void *w, const float *b,
                                    const unet_act *y, int relu, int dilation, stencil_stream_t s) {
    return unet_conv3x3_fwd_engine(x, w, b, y, relu, dilation, 0, s);
}

extern "C" int unet_conv3x3_fwd(const unet_act *x, const void *w, const float *b, const unet_act *y,
                                int relu, stencil_stream_t s) {
    return unet_conv3x3_fwd_dil(x, w, b, y, relu, 1, s);
}

extern "C" int unet_flip_weights(const void *w, void *wt, int cout, int cin, stencil_stream_t s) {
    if (!w || !wt || cout < 1 || cin < 1) return fail(STENCIL_EINVAL, "bad arguments");
    k_flip<<<grid_for((long long)cout * 9 * cin), 256, 0, STREAM(s)>>>(
        static_cast<const bf16 *>(w), static_cast<bf16 *>(wt), cout, cin);
    return cuda_fail(cudaGetLastError(), "flip launch");
}

template <int BN>
int launch_wgrad_tma(const unet_act *x, const unet_act *dy, float *dw, int dil, void *ws, cudaStream_t s) {
    static bool attr[64] = {false};
    constexpr int SMEM = TMA_STAGES * (BM * BK * 2 + BN * BK * 2) + (2 * TMA_STAGES + 1) * 8 + 16 + 1024;
    const int dev = current_device();
    if (dev >= 0 && dev < 64 && !attr[dev]) {
        ST_CUDA(cudaFuncSetAttribute(k_wgrad_tma<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM));
        attr[dev] = true;
    }
    const int cin = x->c, cout = dy->c, H = x->h, W = x->w, N = x->n;
    const long long P = (long long)N * H * W;
    // workspace: x as three channel-major copies shifted by -dil, 0, +dil
    // columns, then dy channel-major
    bf16 *xT = static_cast<bf16 *>(ws);
    bf16 *gT = xT + 3LL * cin * P;
    for (int k = 0; k < 3; ++k)
        k_to_cmajor<<<dim3((unsigned)((P + 63) / 64), cin / 32), 256, 0, s>>>(
            to_act(*x), xT + (long long)k * cin * P, P, W, (k - 1) * dil);
    k_to_cmajor<<<dim3((unsigned)((P + 63) / 64), cout / 32), 256, 0, s>>>(to_act(*dy), gT, P, W, 0);
    ST_CUDA(cudaGetLastError());
    CUtensorMap gm, xm;
    const unsigned long long p2 = (unsigned long long)P * 2;
    const unsigned long long gd[4] = {(unsigned long long)W, (unsigned long long)H, (unsigned long long)N,
                                      (unsigned long long)cout};
    const unsigned long long st[4] = {(unsigned long long)W * 2, (unsigned long long)W * H * 2, p2,
                                      p2 * (unsigned long long)cin};
    const unsigned gb[4] = {(unsigned)BK, 1u, 1u, (unsigned)BM};
    int rc = make_tensor_map_general(&gm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, gT, gd, st, gb,
                                     CU_TENSOR_MAP_SWIZZLE_64B);
    if (rc) return rc;
    const unsigned long long xd[5] = {(unsigned long long)W, (unsigned long long)H, (unsigned long long)N,
                                      (unsigned long long)cin, 3ull};
    const unsigned xb[5] = {(unsigned)BK, 1u, 1u, (unsigned)BN, 1u};
    rc = make_tensor_map_general(&xm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, xT, xd, st, xb,
                                 CU_TENSOR_MAP_SWIZZLE_64B);
    if (rc) return rc;
    const long long nchunks = P / BK;
    const int tiles = ((cout + BM - 1) / BM) * (cin / BN) * 9;
    long long splits = (2LL * num_sms() + tiles - 1) / tiles;
    long long per = (nchunks + splits - 1) / splits;
    if (per < 16) per = 16;
    splits = (nchunks + per - 1) / per;
    dim3 grid((unsigned)((cout + BM - 1) / BM), (unsigned)(cin / BN), (unsigned)(9 * splits));
    k_wgrad_tma<BN><<<grid, 192, SMEM, s>>>(gm, xm, dw, cin, cout, H, W, dil, (int)per, nchunks);
    return cuda_fail(cudaGetLastError(), "wgrad (tcgen05) launch");
}

extern "C" int unet_wgrad_workspace_bytes(const unet_act *x, const unet_act *dy, size_t *bytes) {
    CHECK_VIEW(x);
    CHECK_VIEW(dy);
    if (!bytes) return fail(STENCIL_EINVAL, "null bytes");
    *bytes = (size_t)(3 * x->c + dy->c) * (size_t)x->n * x->h * x->w * 2;
    return STENCIL_OK;
}

extern "C" int unet_conv3x3_wgrad_engine(const unet_act *x, const unet_act *dy, float *dw, float *db,
                                         int dilation, int engine, void *workspace,
                                         size_t workspace_bytes, stencil_stream_t s) {
    CHECK_VIEW(x);
    CHECK_VIEW(dy);
    if (!dw) return fail(STENCIL_EINVAL, "null dw");
    if (dilation < 1) return fail(STENCIL_EINVAL, "dilation must be >= 1");
    if (engine < 0 || engine > 2) return fail(STENCIL_EINVAL, "engine must be 0, 1 or 2");
    if (x->n != dy->n || x->h != dy->h || x->w != dy->w) return fail(STENCIL_EINVAL, "shape mismatch");
    const size_t need = (size_t)(3 * x->c + dy->c) * (size_t)x->n * x->h * x->w * 2;
    const bool fits = x->w % 32 == 0 && x->c % 32 == 0 && dy->c % 32 == 0 && workspace &&
                      workspace_bytes >= need && (reinterpret_cast<uintptr_t>(workspace) & 255) == 0;
    if (engine == 1 && !fits)
        return fail(STENCIL_EINVAL, "tcgen05 weight gradient needs W %% 32 == 0 and a %zu-byte workspace", need);
    if (engine == 0) engine = fits ? 1 : 2;
    if (engine == 1) {
        const int cin = x->c;
        int rc = cin % 128 == 0 ? launch_wgrad_tma<128>(x, dy, dw, dilation, workspace, STREAM(s))
                 : cin % 64 == 0 ? launch_wgrad_tma<64>(x, dy, dw, dilation, workspace, STREAM(s))
                                 : launch_wgrad_tma<32>(x, dy, dw, dilation, workspace, STREAM(s));
        if (rc || !db) return rc;
        const long long P = (long long)x->n * x->h * x->w;
        dim3 g2((unsigned)std::min<long long>(1024, (P + 255) / 256), (dy->c + 31) / 32);
        k_bias_grad<<<g2, 256, 0, STREAM(s)>>>(to_act(*dy), db);
        return cuda_fail(cudaGetLastError(), "bias grad launch");
    }
    return unet_conv3x3_wgrad_dil(x, dy, dw, db, dilation, s);
}

extern "C" int unet_conv3x3_wgrad_dil(const unet_act *x, const unet_act *dy, float *dw, float *db,
                                      int dilation, stencil_stream_t s) {
    CHECK_VIEW(x);
    CHECK_VIEW(dy);
    if (!dw) return fail(STENCIL_EINVAL, "null dw");
    if (dilation < 1) return fail(STENCIL_EINVAL, "dilation must be >= 1");
    if (x->n != dy->n || x->h != dy->h || x->w != dy->w) return fail(STENCIL_EINVAL, "shape mismatch");
    const long long P = (long long)x->n * x->h * x->w;
    const int mt = (dy->c + 63) / 64, nt = (x->c + 63) / 64;
    // Split the pixels so that about 4 blocks per SM run.
    long long splits = (4LL * num_sms() + 9LL * mt * nt - 1) / (9LL * mt * nt);
    if (splits < 1) splits = 1;
    long long per = (P + splits - 1) / splits;
    per = ((per + WK - 1) / WK) * WK;
    splits = (P + per - 1) / per;
    dim3 grid(mt, nt, (unsigned)(9 * splits));
    k_wgrad<<<grid, 128, 0, STREAM(s)>>>(to_act(*x), to_act(*dy), dw, per, dilation);
    int rc = cuda_fail(cudaGetLastError(), "wgrad launch");
    if (rc || !db) return rc;
    dim3 g2((unsigned)std::min<long long>(1024, (P + 255) / 256), (dy->c + 31) / 32);
    k_bias_grad<<<g2, 256, 0, STREAM(s)>>>(to_act(*dy), db);
    return cuda_fail(cudaGetLastError(), "bias grad launch");
}

extern "C" int unet_conv3x3_wgrad(const unet_act *x, const unet_act *dy, float *dw, float *db,
                                  stencil_stream_t s) {
    return unet_conv3x3_wgrad_dil(x, dy, dw, db, 1, s);
}

extern "C" int unet_relu_bwd(const unet_act *g, const unet_act *y, stencil_stream_t s) {
    CHECK_VIEW(g);
    CHECK_VIEW(y);
    const Act ga = to_act(*g);
    k_relu_bwd<<<grid_for((long long)g->n * g->h * g->w * (g->c / 8)), 256, 0, STREAM(s)>>>(ga, to_act(*y));
    return cuda_fail(cudaGetLastError(), "relu_bwd launch");
}

extern "C" int unet_maxpool2_fwd(const unet_act *x, const unet_act *y, stencil_stream_t s) {
    CHECK_VIEW(x);
    CHECK_VIEW(y);
    if (x->h != 2 * y->h || x->w != 2 * y->w || x->c != y->c) return fail(STENCIL_EINVAL, "pool shapes");
    k_pool_fwd<<<grid_for((long long)y->n * y->h * y->w * (y->c / 8)), 256, 0, STREAM(s)>>>(to_act(*x), to_act(*y));
    return cuda_fail(cudaGetLastError(), "pool launch");
}

extern "C" int unet_maxpool2_bwd(const unet_act *x, const unet_act *y, const unet_act *dy,
                                 const unet_act *dx, stencil_stream_t s) {
    CHECK_VIEW(x);
    CHECK_VIEW(y);
    CHECK_VIEW(dy);
    CHECK_VIEW(dx);
    k_pool_bwd<<<grid_for((long long)y->n * y->h * y->w * (y->c / 8)), 256, 0, STREAM(s)>>>(
        to_act(*x), to_act(*y), to_act(*dy), to_act(*dx));
    return cuda_fail(cudaGetLastError(), "pool bwd launch");
}

extern "C" int unet_upsample2_fwd(const unet_act *x, const unet_act *y, stencil_stream_t s) {
    CHECK_VIEW(x);
    CHECK_VIEW(y);
    if (y->h != 2 * x->h || y->w != 2 * x->w || x->c != y->c) return fail(STENCIL_EINVAL, "upsample shapes");
    k_up_fwd<<<grid_for((long long)y->n * y->h * y->w * (y->c / 8)), 256, 0, STREAM(s)>>>(to_act(*x), to_act(*y));
    return cuda_fail(cudaGetLastError(), "upsample launch");
}

extern "C" int unet_upsample2_bwd(const unet_act *dy, const unet_act *dx, stencil_stream_t s) {
    CHECK_VIEW(dy);
    CHECK_VIEW(dx);
    k_up_bwd<<<grid_for((long long)dx->n * dx->h * dx->w * (dx->c / 8)), 256, 0, STREAM(s)>>>(to_act(*dy), to_act(*dx));
    return cuda_fail(cudaGetLastError(), "upsample bwd launch");
}

extern "C" int unet_add(const unet_act *a, const unet_act *b, stencil_stream_t s) {
    CHECK_VIEW(a);
    CHECK_VIEW(b);
    k_add<<<grid_for((long long)a->n * a->h * a->w * (a->c / 8)), 256, 0, STREAM(s)>>>(to_act(*a), to_act(*b));
    return cuda_fail(cudaGetLastError(), "add launch");
}

extern "C" int unet_head_fwd(const unet_act *x, const float *w, const float *b, float *y,
                             stencil_stream_t s) {
    CHECK_VIEW(x);
    if (!w || !b || !y) return fail(STENCIL_EINVAL, "null pointer");
    k_head_fwd<<<grid_for((long long)x->n * x->h * x->w), 256, 0, STREAM(s)>>>(to_act(*x), w, b, y);
    return cuda_fail(cudaGetLastError(), "head launch");
}

extern "C" int unet_head_bwd(const unet_act *x, const float *w, const float *dy, const unet_act *dx,
                             float *dw, float *db, stencil_stream_t s) {
    CHECK_VIEW(x);
    CHECK_VIEW(dx);
    if (!w || !dy || !dw || !db || x->c > 256) return fail(STENCIL_EINVAL, "bad head arguments");
    k_head_bwd<<<grid_for((long long)x->n * x->h * x->w), 256, 0, STREAM(s)>>>(to_act(*x), w, dy, to_act(*dx), dw, db);
    return cuda_fail(cudaGetLastError(), "head bwd launch");
}

extern "C" int unet_features(const float *fields, int n, int h, int w, const unet_act *x, float *coons,
                             stencil_stream_t s) {
    CHECK_VIEW(x);
    if (!fields || x->n != n || x->h != h || x->w != w || h < 3 || w < 3)
        return fail(STENCIL_EINVAL, "feature shapes");
    k_features<<<grid_for((long long)n * h * w), 256, 0, STREAM(s)>>>(fields, n, h, w, to_act(*x), coons);
    return cuda_fail(cudaGetLastError(), "features launch");
}

extern "C" int unet_mse(const float *out, const float *coons, const float *target, int n, int h, int w,
                        float scale, float *loss_sum, float *dout, stencil_stream_t s) {
    if (!out || !coons || !target || !loss_sum || !dout) return fail(STENCIL_EINVAL, "null pointer");
    k_mse<<<grid_for((long long)n * h * w), 256, 0, STREAM(s)>>>(out, coons, target, n, h, w, scale, loss_sum, dout);
    return cuda_fail(cudaGetLastError(), "mse launch");
}

extern "C" int unet_adam(float *p, const float *g, float *m, float *v, void *p_bf16, long long count,
                         float lr, float beta1, float beta2, float eps, int step, stencil_stream_t s) {
    if (!p || !g || !m || !v || count < 0 || step < 1) return fail(STENCIL_EINVAL, "bad adam arguments");
    const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
    k_adam<<<grid_for(count), 256, 0, STREAM(s)>>>(p, g, m, v, static_cast<bf16 *>(p_bf16), count, lr, beta1,
                                                    beta2, eps, c1, c2);
    return cuda_fail(cudaGetLastError(), "adam launch");
}

extern "C" int unet_assemble(const float *fields, const float *coons, const float *out, int n, int h, int w,
                             float *u, stencil_stream_t s) {
    if (!fields || !coons || !out || !u) return fail(STENCIL_EINVAL, "null pointer");
    k_assemble<<<grid_for((long long)n * h * w), 256, 0, STREAM(s)>>>(fields, coons, out, n, h, w, u);
    return cuda_fail(cudaGetLastError(), "assemble launch");
}

extern "C" int unet_coons_fill(const float *fields, int n, int h, int w, float *u, stencil_stream_t s) {
    if (!fields || !u || n < 0 || h < 2 || w < 2) return fail(STENCIL_EINVAL, "bad arguments");
    k_coons_fill<<<grid_for((long long)n * h * w), 256, 0, STREAM(s)>>>(fields, n, h, w, u);
    return cuda_fail(cudaGetLastError(), "coons_fill launch");
}

extern "C" int unet_resample_border(const float *fields, int n, int H, int W, int h, int w,
                                    float *coarse, stencil_stream_t s) {
    if (!fields || !coarse || n < 0 || H < 2 || W < 2 || h < 2 || w < 2)
        return fail(STENCIL_EINVAL, "bad arguments");
    k_resample_border<<<grid_for((long long)n * h * w), 256, 0, STREAM(s)>>>(fields, n, H, W, h, w, coarse);
    return cuda_fail(cudaGetLastError(), "resample_border launch");
}

extern "C" int unet_upsample_bilinear(const float *coarse, int n, int h, int w, const float *fields,
                                      int H, int W, float *u, stencil_stream_t s) {
    if (!coarse || !fields || !u || n < 0 || H < 2 || W < 2 || h < 2 || w < 2)
        return fail(STENCIL_EINVAL, "bad arguments");
    k_upsample_bilinear<<<grid_for((long long)n * H * W), 256, 0, STREAM(s)>>>(coarse, n, h, w, fields, H,
                                                                             W, u);
    return cuda_fail(cudaGetLastError(), "upsample_bilinear launch");
}

extern "C" int unet_to_bf16(const float *src, void *dst, long long count, stencil_stream_t s) {
    if (!src || !dst || count < 0) return fail(STENCIL_EINVAL, "bad arguments");
    k_to_bf16<<<grid_for(count), 256, 0, STREAM(s)>>>(src, static_cast<bf16 *>(dst), count);
    return cuda_fail(cudaGetLastError(), "to_bf16 launch");
}

// common.cuh -- shared device helpers of libstencil_gb300: the per-cell star
// update in the reference's summation order, PTX wrappers for mbarrier / TMA /
// clusters, and bounded waits that report through a device status word instead
// of hanging.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/stencil_dispatch.h"

namespace st {

// ---------------------------------------------------------------------------
// Geometry of one grid as the kernels see it.
// ---------------------------------------------------------------------------
struct Geom {
    int nx, ny, nz;      // nz == 1 for 2-D
    int radius;
    int legacy;          // 1: subtract the centre (STENCIL_MODE_LEGACY)
    long long sy, sz;    // strides of y and z in cells
};

// Device status word: bounded waits that give up OR in a code and return.
// Read and cleared by stencil_device_status().
enum : unsigned { kStatusTimeout = 1u, kStatusBadLaunch = 2u };
extern __device__ unsigned g_device_status;

__device__ __forceinline__ void report_status(unsigned code) { atomicOr(&g_device_status, code); }

// SplitMix64 finaliser (Steele, Lea & Flood 2014); identical to the oracle's.
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// ---------------------------------------------------------------------------
// The per-cell update.  Order follows src/stencils.cu:8-19 with
// src/stencil_accumulators.cu:6-16: axes i, j, k; on each axis the offsets
// -R..-1 ("prev", distance R down to 1) and then +1..+R ("next").  One float
// accumulator starting at 0.0f; then the correctly rounded acc / (float)(2*D*R)
// (IEEE semantics: this library is never built with fast-math; see div_coeff)
// and, in LEGACY mode, minus the centre value.  Every kernel calls this with its own value source, so all
// variants are bit-identical to the reference.
// ---------------------------------------------------------------------------
template <int D, int R, class Get>
__device__ __forceinline__ float star_sum(Get get) {
    float acc = 0.0f;
#pragma unroll
    for (int a = 0; a < D; ++a) {
#pragma unroll
        for (int o = -R; o <= R; ++o)
            if (o != 0) acc += get(a, o);
    }
    return acc;
}

// ---------------------------------------------------------------------------
// Correctly rounded division by the stencil coefficient c = 2*D*R, without
// the general IEEE division sequence.  Method: Markstein, "Computation of
// elementary functions on the IBM RISC System/6000 processor", IBM J. Res.
// Dev. 34(1), 1990: with rc = RN(1/c), q0 = RN(x*rc) is within one ulp of x/c,
// the remainder r = x - q0*c is exact in one FMA, and RN(q0 + r*rc) is the
// correctly rounded quotient.  The steps assume no underflow/overflow, so the
// method is used for +0 and |x| in [2^-100, 2^120] and the plain division
// otherwise (-0, tiny, huge and non-finite values).  Powers of two divide exactly by a
// multiplication.  stencil_selftest_div() checks every float bit pattern
// against the compiler's IEEE division for each coefficient.
// ---------------------------------------------------------------------------
template <int C>
__device__ __forceinline__ bool div_fast_ok(float x) {
    const float a = fabsf(x);
    // +0 is exact on the fast path too (the sums never produce -0: they start
    // from +0.0f, and +0 + -0 = +0).
    return (C & (C - 1)) == 0 || __float_as_uint(x) == 0u || (a >= 0x1p-100f && a <= 0x1p+120f);
}

template <int C>
__device__ __forceinline__ float div_fast(float x) {
    constexpr float rc = 1.0f / (float)C;
    if ((C & (C - 1)) == 0) return x * rc;
    const float q0 = x * rc;
    const float r = fmaf(-q0, (float)C, x);
    return fmaf(r, rc, q0);
}

// Per-value form: the fast path where it applies, else IEEE division.
template <int C>
__device__ __forceinline__ float div_coeff(float x) {
    return div_fast_ok<C>(x) ? div_fast<C>(x) : x / (float)C;
}

// ---------------------------------------------------------------------------
// Packed FP32 pairs (sm_100 family: add/mul/fma.rn.f32x2).  Each element is
// rounded exactly as the scalar instruction would round it (IEEE round to
// nearest, subnormals kept), so a sum built from pairs is bit-identical to
// the scalar sum in the same order; one instruction does two cells' work.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 fadd2(float2 a, float2 b) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "add.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}

__device__ __forceinline__ float2 fmul2(float2 a, float2 b) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "mul.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}

__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "mov.b64 rc, {%6, %7};\n\tfma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
}

// div_fast on a pair (the same three roundings per element; -q0*c + x is
// formed as q0*(-c) + x, the negation being exact).
template <int C>
__device__ __forceinline__ float2 div_fast2(float2 x) {
    constexpr float rc = 1.0f / (float)C;
    if ((C & (C - 1)) == 0) return fmul2(x, make_float2(rc, rc));
    const float2 q0 = fmul2(x, make_float2(rc, rc));
    const float2 r = ffma2(q0, make_float2(-(float)C, -(float)C), x);
    return ffma2(r, make_float2(rc, rc), q0);
}

// Division of a sum that was started from its first term instead of +0.0f:
// the two differ only for an all-(-0) sum (-0 here, +0 in the reference), and
// x + 0.0f maps exactly that case to +0 and leaves every other value as is.
template <int C>
__device__ __forceinline__ float div_slow_from_first(float x) {
    return (x + 0.0f) / (float)C;
}

template <int D, int R>
__device__ __forceinline__ float star_finish(float acc, float centre, int legacy) {
    const float v = div_coeff<2 * D * R>(acc);
    return legacy ? v - centre : v;
}

// Runtime-radius forms for the generic kernels.
__device__ __forceinline__ float star_finish_rt(float acc, float coeff, float centre,
                                                int legacy) {
    float v = acc / coeff;
    return legacy ? v - centre : v;
}

// ---------------------------------------------------------------------------
// PTX wrappers.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Default limit of one bounded wait: 2 s.  A healthy wait in these kernels
// ends in microseconds.
constexpr uint64_t kWaitLimitNs = 2000000000ull;

// Waits for the phase with the given parity of an mbarrier.  Returns false
// (after setting the device status word) if the limit passes first.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity,
                                                  uint64_t limit_ns = kWaitLimitNs) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    while (!mbar_try_wait(bar, parity)) {
        if (globaltimer_ns() - t0 > limit_ns) {
            report_status(kStatusTimeout);
            return false;
        }
    }
    return true;
}

// Named barrier `id` over `count` threads (a multiple of 32) that also ANDs a
// predicate, so that a failed bounded wait in one warp ends all of them
// together.
__device__ __forceinline__ bool named_barrier_and(int id, int count, bool ok) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.and.pred p, %2, %3, p;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)ok), "r"(id), "r"(count)
        : "memory");
    return r != 0;
}

// Grid-wide barrier of a cooperative launch (all CTAs co-resident), on a
// counter that the host zeroes before the launch.  A CTA arrives once its
// threads have passed a CTA-level barrier after their last stores: a fence,
// then a release add at GPU scope.  A waiter spins with acquire loads until
// the counter reaches the target (a bounded wait), then orders what it
// acquired before its own later TMA (async-proxy) reads.
__device__ __forceinline__ void grid_arrive(unsigned *ctr) {
    __threadfence();
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(ctr) : "memory");
}

__device__ __forceinline__ bool grid_wait_bounded(const unsigned *ctr, unsigned target,
                                                  uint64_t limit_ns = kWaitLimitNs) {
    unsigned v;
    uint64_t t0 = 0;
    for (;;) {
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(ctr) : "memory");
        if (v >= target) break;
        const uint64_t t = globaltimer_ns();
        if (!t0) t0 = t;
        else if (t - t0 > limit_ns) {
            report_status(kStatusTimeout);
            return false;
        }
    }
    asm volatile("fence.proxy.async.global;" ::: "memory");
    return true;
}

// TMA tiled loads into this CTA's shared memory, completion on an mbarrier.
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar,
                                            int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%3, %4}], [%2];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, uint64_t *bar,
                                            int x, int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(z)
        : "memory");
}

// Bulk (non-tensor) copy of `bytes` contiguous bytes (16-byte aligned, a
// multiple of 16) into this CTA's shared memory, completion on an mbarrier.
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void prefetch_tensormap(const CUtensorMap *map) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// Thread-block cluster helpers.
__device__ __forceinline__ uint32_t cluster_ctarank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

__device__ __forceinline__ uint32_t cluster_nctarank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}

__device__ __forceinline__ void cluster_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
                 "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Address of the same shared-memory variable in CTA `rank` of this cluster.
__device__ __forceinline__ uint32_t mapa_shared(uint32_t addr, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
    return r;
}

__device__ __forceinline__ void st_cluster_f32(uint32_t addr, float v) {
    asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(addr), "f"(v) : "memory");
}

__device__ __forceinline__ void st_cluster_v4(uint32_t addr, float4 v) {
    asm volatile("st.shared::cluster.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "f"(v.x),
                 "f"(v.y), "f"(v.z), "f"(v.w)
                 : "memory");
}

__device__ __forceinline__ float4 ld_cluster_v4(uint32_t addr) {
    float4 v;
    asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "r"(addr)
                 : "memory");
    return v;
}

__device__ __forceinline__ float ld_cluster_f32(uint32_t addr) {
    float v;
    asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(addr) : "memory");
    return v;
}

// 16-byte global store that the compiler cannot split into scalar stores.
__device__ __forceinline__ void stg4(float *p, float a, float b, float c, float d) {
    asm volatile("st.global.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(a), "f"(b), "f"(c),
                 "f"(d)
                 : "memory");
}

// L2 policy for data written once and not read again soon (a sweep's
// output): evict first, so it does not displace the rows other CTAs are
// about to re-read as halos.
__device__ __forceinline__ uint64_t l2_evict_first_policy() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

__device__ __forceinline__ void stg4_hint(float *p, float a, float b, float c, float d, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(p), "f"(a),
                 "f"(b), "f"(c), "f"(d), "l"(pol)
                 : "memory");
}

__device__ __forceinline__ float f4get(const float4 &v, int c) {
    return c == 0 ? v.x : (c == 1 ? v.y : (c == 2 ? v.z : v.w));
}

// Whether cell coordinate q lies in [R, n-R).
__device__ __forceinline__ bool in_range(int q, int n, int r) { return q >= r && q < n - r; }

}  // namespace st

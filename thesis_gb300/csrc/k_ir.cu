// k_ir.cu -- mixed-precision iterative refinement for the JACOBI steady state.
//
// The Jacobi sweep u' = M u + c (M = mean of the 2*D*R axis neighbours over
// the update region, c = the border contributions) is split into outer steps
// of m sweeps.  Each outer step:
//   1. r = (M u + c) - u from the FP32 master u (FP32 arithmetic), scaled by a
//      power of two s so that |r/s| <= 1, stored in BF16 or FP16;
//   2. e_1 = r/s (the first correction sweep from e_0 = 0), then m-1 sweeps
//      e_{j+1} = M e_j + r/s with e stored in BF16/FP16 and every sum
//      accumulated in FP32 (the border band of e and r is zero);
//   3. u += s * e_m in FP32.
// In exact arithmetic u + s*e_m is exactly m Jacobi sweeps from u, so the
// total sweep count means the same as for the FP32 loop; only rounding
// differs.  The relative residual (k_util.cu; FP64 sums) decides convergence when a
// tolerance is given.  Correction sweeps move 6 bytes per cell update (read e
// and r, write e) instead of 8; on 3-D grids they run on the TMA-fed stream
// form (k_lpstream.cu), elsewhere on k_lp_sweep below (the same arithmetic).
// 2-D grids of at most one tile per SM run each outer step as one
// cooperative launch instead (k_ir2d.cu: every correction sweep on chip,
// bit-identical to the launches here).
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>

#include "host.hpp"

namespace st {

size_t residual_scratch_bytes();
int launch_residual(const Geom &g, int dims, const float *u, double *scratch, cudaStream_t s);
// The TMA-fed correction sweep for 3-D grids (k_lpstream.cu): eo = M e + rhs
// over the update region.  eo's border band must hold zeros (at R = 4 the
// sweep's block stores write them there again); e and rhs are read only.
bool lp_stream_supported(const Geom &g, int dims);
template <typename E>
int launch_lp_stream(const Geom &g, const E *e, E *eo, const E *rhs, cudaStream_t s);

template <typename E>
struct LowP;
template <>
struct LowP<__nv_bfloat16> {
    __device__ static float2 to2(uint32_t w) {
        return __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&w));
    }
    __device__ static uint32_t from2(float a, float b) {
        __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
        return *reinterpret_cast<uint32_t *>(&h);
    }
    __device__ static float to(const __nv_bfloat16 v) { return __bfloat162float(v); }
    __device__ static __nv_bfloat16 from(float v) { return __float2bfloat16_rn(v); }
};
template <>
struct LowP<__half> {
    __device__ static float2 to2(uint32_t w) {
        return __half22float2(*reinterpret_cast<const __half2 *>(&w));
    }
    __device__ static uint32_t from2(float a, float b) {
        __half2 h = __floats2half2_rn(a, b);
        return *reinterpret_cast<uint32_t *>(&h);
    }
    __device__ static float to(const __half v) { return __half2float(v); }
    __device__ static __half from(float v) { return __float2half_rn(v); }
};

template <typename E>
__device__ __forceinline__ void unpack8(const uint4 &q, float *f) {
    const float2 a = LowP<E>::to2(q.x), b = LowP<E>::to2(q.y), c = LowP<E>::to2(q.z),
                 d = LowP<E>::to2(q.w);
    f[0] = a.x; f[1] = a.y; f[2] = b.x; f[3] = b.y; f[4] = c.x; f[5] = c.y; f[6] = d.x; f[7] = d.y;
}

// One correction sweep e_out = M e + rhs on 8-cell vectors (nx % 8 == 0).
template <typename E, int D, int R>
__global__ void __launch_bounds__(256)
    k_lp_sweep(const E *__restrict__ e, E *__restrict__ eo, const E *__restrict__ rhs, Geom g) {
    constexpr int C = 2 * D * R;
    const int nv = g.nx >> 3;
    const long long nrows = (long long)(g.ny - 2 * R) * (D == 3 ? g.nz - 2 * R : 1);
    const long long total = nrows * nv;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int v = (int)(t % nv);
        const long long rr = t / nv;
        const int j = R + (int)(rr % (g.ny - 2 * R));
        const int k = D == 3 ? R + (int)(rr / (g.ny - 2 * R)) : 0;
        const int x0 = v * 8;
        if (x0 + 7 < R || x0 >= g.nx - R) continue;
        const long long row = (long long)j * g.sy + (long long)k * g.sz;
        const uint4 *src = reinterpret_cast<const uint4 *>(e + row);
        float w[24];
        {
            const uint4 z4 = make_uint4(0, 0, 0, 0);
            unpack8<E>(v > 0 ? __ldg(src + v - 1) : z4, w);
            unpack8<E>(__ldg(src + v), w + 8);
            unpack8<E>(v + 1 < nv ? __ldg(src + v + 1) : z4, w + 16);
        }
        // the sum starts from its first term, as in the persistent 2-D form
        // (k_ir2d.cu) and the 3-D stream form (a sum started from +0 differs
        // only when every term is -0: +0 there, -0 here)
        float acc[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) acc[c] = w[8 + c - R];
#pragma unroll
        for (int o = -R + 1; o <= R; ++o) {
            if (!o) continue;
#pragma unroll
            for (int c = 0; c < 8; ++c) acc[c] += w[8 + c + o];
        }
#pragma unroll
        for (int o = -R; o <= R; ++o) {
            if (!o) continue;
            float f[8];
            unpack8<E>(__ldg(reinterpret_cast<const uint4 *>(e + row + o * g.sy) + v), f);
#pragma unroll
            for (int c = 0; c < 8; ++c) acc[c] += f[c];
        }
        if (D == 3) {
#pragma unroll
            for (int o = -R; o <= R; ++o) {
                if (!o) continue;
                float f[8];
                unpack8<E>(__ldg(reinterpret_cast<const uint4 *>(e + row + o * g.sz) + v), f);
#pragma unroll
                for (int c = 0; c < 8; ++c) acc[c] += f[c];
            }
        }
        float rf[8];
        unpack8<E>(__ldg(reinterpret_cast<const uint4 *>(rhs + row) + v), rf);
        float out[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) out[c] = div_coeff<C>(acc[c]) + rf[c];
        E *dst = eo + row + x0;
        if (x0 >= R && x0 + 7 < g.nx - R) {
            uint4 q;
            q.x = LowP<E>::from2(out[0], out[1]);
            q.y = LowP<E>::from2(out[2], out[3]);
            q.z = LowP<E>::from2(out[4], out[5]);
            q.w = LowP<E>::from2(out[6], out[7]);
            *reinterpret_cast<uint4 *>(dst) = q;
        } else {
#pragma unroll
            for (int c = 0; c < 8; ++c)
                if (in_range(x0 + c, g.nx, R)) dst[c] = LowP<E>::from(out[c]);
        }
    }
}

// Rows of the update region are handed to warps round-robin (no 64-bit
// index division); a lane owns 4-cell chunks of its row (nx % 8 == 0).
struct IrRows {
    int R, ry, nrows, nch;
    __device__ IrRows(const Geom &g, int D, int r) : R(r), ry(g.ny - 2 * r) {
        nrows = ry * (D == 3 ? g.nz - 2 * r : 1);
        nch = g.nx >> 2;
    }
    __device__ long long base(const Geom &g, int q) const {
        return (long long)(R + q % ry) * g.sy + (long long)(q / ry + (g.nz > 1 ? R : 0)) * g.sz;
    }
};

__device__ __forceinline__ float4 ir_ld4(const float *p) { return *reinterpret_cast<const float4 *>(p); }

// r = (M u + c) - u over the update region (FP32, the sweep's summation
// order).  pass 0: max |r| into *max_bits.  pass 1: stores r * 2^-ceil(log2
// max) in E and the scale in *scale.
template <typename E, int D, int R>
__global__ void __launch_bounds__(256)
    k_ir_resid(const float *__restrict__ u, E *__restrict__ r, Geom g, unsigned *max_bits,
               float *scale, int pass) {
    constexpr int C = 2 * D * R;
    constexpr int RA = (R + 3) & ~3;
    float inv = 1.0f;
    if (pass == 1) {
        const float m = __uint_as_float(*max_bits);
        int ex = 0;
        if (m > 0.0f) frexpf(m, &ex);  // m = f * 2^ex, f in [0.5, 1)
        const float s = ldexpf(1.0f, ex);
        inv = 1.0f / s;
        if (blockIdx.x == 0 && threadIdx.x == 0) *scale = s;
    }
    const IrRows rows(g, D, R);
    const int wpb = blockDim.x >> 5, lane = threadIdx.x & 31;
    float local = 0.0f;
    for (int q = blockIdx.x * wpb + (threadIdx.x >> 5); q < rows.nrows; q += gridDim.x * wpb) {
        const long long base = rows.base(g, q);
        const float *row = u + base;
        for (int c = lane; c < rows.nch; c += 32) {
            const int x0 = 4 * c;
            if (x0 + 3 < R || x0 >= g.nx - R) continue;
            float w[4 + 2 * RA];
#pragma unroll
            for (int h = 0; h < (4 + 2 * RA) / 4; ++h) {
                const int cc = c - RA / 4 + h;
                float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                if (cc >= 0 && cc < rows.nch) v = ir_ld4(row + 4 * cc);
                w[4 * h] = v.x; w[4 * h + 1] = v.y; w[4 * h + 2] = v.z; w[4 * h + 3] = v.w;
            }
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
                const float4 v = ir_ld4(row + x0 + o * g.sy);
                acc[0] += v.x; acc[1] += v.y; acc[2] += v.z; acc[3] += v.w;
            }
            if (D == 3) {
#pragma unroll
                for (int o = -R; o <= R; ++o) {
                    if (!o) continue;
                    const float4 v = ir_ld4(row + x0 + o * g.sz);
                    acc[0] += v.x; acc[1] += v.y; acc[2] += v.z; acc[3] += v.w;
                }
            }
            float res[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) res[e] = div_coeff<C>(acc[e]) - w[RA + e];
            const bool full = x0 >= R && x0 + 3 < g.nx - R;
            if (pass == 0) {
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (full || in_range(x0 + e, g.nx, R)) local = fmaxf(local, fabsf(res[e]));
            } else if (full) {
                uint2 q2;
                q2.x = LowP<E>::from2(res[0] * inv, res[1] * inv);
                q2.y = LowP<E>::from2(res[2] * inv, res[3] * inv);
                *reinterpret_cast<uint2 *>(r + base + x0) = q2;
            } else {
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (in_range(x0 + e, g.nx, R)) r[base + x0 + e] = LowP<E>::from(res[e] * inv);
            }
        }
    }
    if (pass == 0) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) local = fmaxf(local, __shfl_xor_sync(0xffffffffu, local, o));
        if ((threadIdx.x & 31) == 0) atomicMax(max_bits, __float_as_uint(local));
    }
}

// u += s * e over the update region.
template <typename E, int D, int R>
__global__ void __launch_bounds__(256)
    k_ir_update(float *__restrict__ u, const E *__restrict__ e, Geom g, const float *scale) {
    const float s = *scale;
    const IrRows rows(g, D, R);
    const int wpb = blockDim.x >> 5, lane = threadIdx.x & 31;
    for (int q = blockIdx.x * wpb + (threadIdx.x >> 5); q < rows.nrows; q += gridDim.x * wpb) {
        const long long base = rows.base(g, q);
        for (int c = lane; c < rows.nch; c += 32) {
            const int x0 = 4 * c;
            if (x0 + 3 < R || x0 >= g.nx - R) continue;
            float *up = u + base + x0;
            const float4 v = ir_ld4(up);
            const uint2 ew = *reinterpret_cast<const uint2 *>(e + base + x0);
            const float2 e01 = LowP<E>::to2(ew.x), e23 = LowP<E>::to2(ew.y);
            const float out[4] = {fmaf(s, e01.x, v.x), fmaf(s, e01.y, v.y), fmaf(s, e23.x, v.z),
                                  fmaf(s, e23.y, v.w)};
            if (x0 >= R && x0 + 3 < g.nx - R) {
                *reinterpret_cast<float4 *>(up) = make_float4(out[0], out[1], out[2], out[3]);
            } else {
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if (in_range(x0 + k, g.nx, R)) up[k] = out[k];
            }
        }
    }
}

namespace {

// Workspace layout: r, e_a, e_b (16-bit grids), a 256-byte block of
// counters, the residual scratch, and for 2-D grids the exchange buffer of
// the persistent form.
struct IrLayout {
    size_t lp, ctl, resid, xch, total;
};

IrLayout ir_layout(const stencil_params &p, int storage) {
    const size_t n = (size_t)cell_count(p);
    const size_t esz = storage == STENCIL_STORAGE_FP32 ? 4 : 2;
    IrLayout l;
    l.lp = (n * esz + 255) & ~(size_t)255;
    l.ctl = 3 * l.lp;
    l.resid = l.ctl + 256;
    l.xch = (l.resid + residual_scratch_bytes() + 255) & ~(size_t)255;
    l.total = l.xch + (p.dims == 2 ? ir2_xch_bytes(make_geom(p)) : 0);
    return l;
}

// Relative residual of u into *rel (synchronises s).
int ir_check(const Geom &g, int dims, const float *u, double *resid, cudaStream_t s, double *rel) {
    int rc = launch_residual(g, dims, u, resid, s);
    if (rc) return rc;
    double sums[2];
    const size_t off = residual_scratch_bytes() / sizeof(double) - 2;
    ST_CUDA(cudaMemcpyAsync(sums, resid + off, sizeof sums, cudaMemcpyDeviceToHost, s));
    ST_CUDA(cudaStreamSynchronize(s));
    *rel = sums[1] > 0.0 ? sqrt(sums[0]) / sqrt(sums[1]) : sqrt(sums[0]);
    return STENCIL_OK;
}

template <typename E, int D, int R>
int ir_loop(const stencil_params &p, const stencil_ir_params &ir, float *u, char *ws,
            cudaStream_t s, stencil_ir_result *out) {
    const Geom g = make_geom(p);
    const size_t n = (size_t)cell_count(p);
    const IrLayout L = ir_layout(p, ir.storage);
    E *r = reinterpret_cast<E *>(ws);
    E *ea = reinterpret_cast<E *>(ws + L.lp);
    E *eb = reinterpret_cast<E *>(ws + 2 * L.lp);
    unsigned *max_bits = reinterpret_cast<unsigned *>(ws + L.ctl);
    float *scale = reinterpret_cast<float *>(ws + L.ctl + 4);
    unsigned *max2 = reinterpret_cast<unsigned *>(ws + L.ctl + 16);  // two words
    unsigned *bar2 = reinterpret_cast<unsigned *>(ws + L.ctl + 32);
    double *resid = reinterpret_cast<double *>(ws + L.resid);
    unsigned long long *xch = reinterpret_cast<unsigned long long *>(ws + L.xch);
    const int m_inner = ir.inner_sweeps > 0 ? ir.inner_sweeps : 50;
    Ir2Plan plan = {};
    const bool persistent = D == 2 && ir.engine != STENCIL_IR_ENGINE_LAUNCHES &&
                            ir2_plan<E>(g, m_inner, ir.temporal, ir.tile_x, ir.tile_y, &plan);
    if (ir.engine == STENCIL_IR_ENGINE_PERSISTENT_2D && !persistent)
        return fail(STENCIL_EUNSUPPORTED,
                    "the persistent refinement engine takes 2-D grids of at most one tile per SM "
                    "with R = 1, 2 or 4");
    if (persistent) {
        ST_CUDA(cudaMemsetAsync(ws + L.ctl, 0, 256, s));
        ST_CUDA(cudaMemsetAsync(xch, 0, ir2_xch_bytes(g), s));
    } else {
        // Border bands of r and e stay zero for the whole solve.
        ST_CUDA(cudaMemsetAsync(ws, 0, 3 * L.lp, s));
    }
    const int blocks = 4 * num_sms();
    int done = 0, outer = 0, step = 0;
    unsigned tag0 = 0;
    long long launches = 0;
    double rel = -1.0;
    while (done < p.iterations) {
        const int m = std::min(m_inner, p.iterations - done);
        if (persistent) {
            // counters grow monotonically within a solve; restart them before
            // they could wrap
            const unsigned grid = (unsigned)(plan.tiles_x * plan.tiles_y);
            if ((unsigned long long)(step + 2) * grid >= 0xffffffffull ||
                (unsigned long long)tag0 + (unsigned)m + 2 >= 0xffffffffull) {
                ST_CUDA(cudaMemsetAsync(ws + L.ctl, 0, 256, s));
                ST_CUDA(cudaMemsetAsync(xch, 0, ir2_xch_bytes(g), s));
                step = 0;
                tag0 = 0;
            }
            int rc = ir2_launch<E>(g, plan, u, xch, bar2, max2, scale, step, tag0, m, s);
            if (rc) return rc;
            ++step;
            tag0 += (unsigned)m + 1;
            ++launches;
        } else {
            ST_CUDA(cudaMemsetAsync(max_bits, 0, sizeof(unsigned), s));
            k_ir_resid<E, D, R><<<blocks, 256, 0, s>>>(u, r, g, max_bits, scale, 0);
            k_ir_resid<E, D, R><<<blocks, 256, 0, s>>>(u, r, g, max_bits, scale, 1);
            ST_CUDA(cudaGetLastError());
            ST_CUDA(cudaMemcpyAsync(ea, r, n * sizeof(E), cudaMemcpyDeviceToDevice, s));
            E *cur = ea, *nxt = eb;
            const bool streamed = lp_stream_supported(g, D);
            for (int it = 1; it < m; ++it) {
                if (streamed) {
                    int rc = launch_lp_stream<E>(g, cur, nxt, r, s);
                    if (rc) return rc;
                } else {
                    k_lp_sweep<E, D, R><<<8 * num_sms(), 256, 0, s>>>(cur, nxt, r, g);
                }
                std::swap(cur, nxt);
            }
            ST_CUDA(cudaGetLastError());
            k_ir_update<E, D, R><<<blocks, 256, 0, s>>>(u, cur, g, scale);
            ST_CUDA(cudaGetLastError());
            launches += 3 + (m - 1);
        }
        done += m;
        ++outer;
        const bool last = done >= p.iterations;
        if ((ir.tol > 0.0 && (ir.check_every <= 1 || outer % ir.check_every == 0)) || last) {
            int rc = ir_check(g, p.dims, u, resid, s, &rel);
            if (rc) return rc;
            launches += 2;
            if (ir.tol > 0.0 && rel < ir.tol) break;
        }
    }
    if (out) {
        out->sweeps = done;
        out->outer_steps = outer;
        out->rel_residual = rel;
        out->engine = persistent ? STENCIL_IR_ENGINE_PERSISTENT_2D : STENCIL_IR_ENGINE_LAUNCHES;
        out->kernel_launches = (int)std::min<long long>(launches, 0x7fffffff);
        out->temporal = persistent ? plan.t : 0;
        out->tile_x = persistent ? plan.tx : 0;
        out->tile_y = persistent ? plan.ty : 0;
    }
    return STENCIL_OK;
}

template <typename E>
int ir_dispatch(const stencil_params &p, const stencil_ir_params &ir, float *u, char *ws,
                cudaStream_t s, stencil_ir_result *out) {
    const int key = p.dims * 10 + p.radius;
    switch (key) {
        case 21: return ir_loop<E, 2, 1>(p, ir, u, ws, s, out);
        case 22: return ir_loop<E, 2, 2>(p, ir, u, ws, s, out);
        case 24: return ir_loop<E, 2, 4>(p, ir, u, ws, s, out);
        case 31: return ir_loop<E, 3, 1>(p, ir, u, ws, s, out);
        case 32: return ir_loop<E, 3, 2>(p, ir, u, ws, s, out);
        case 34: return ir_loop<E, 3, 4>(p, ir, u, ws, s, out);
        default: return fail(STENCIL_EUNSUPPORTED, "IR has no D=%d R=%d instance", p.dims, p.radius);
    }
}

size_t ir_bytes(const stencil_params &p, int storage) { return ir_layout(p, storage).total; }

}  // namespace
}  // namespace st

using namespace st;

extern "C" int stencil_ir_workspace_bytes(const stencil_params *p, const stencil_ir_params *ir,
                                          size_t *bytes) {
    int rc = stencil_params_check(p);
    if (rc) return rc;
    if (!ir || !bytes) return fail(STENCIL_EINVAL, "null pointer");
    *bytes = ir_bytes(*p, ir->storage);
    return STENCIL_OK;
}

extern "C" int stencil_ir_solve(const stencil_params *p, const stencil_ir_params *ir, float *d_u,
                                void *d_workspace, size_t workspace_bytes,
                                stencil_stream_t stream, stencil_ir_result *result) {
    int rc = stencil_params_check(p);
    if (rc) return rc;
    if (!ir || !d_u || !d_workspace) return fail(STENCIL_EINVAL, "null pointer");
    if (p->mode != STENCIL_MODE_JACOBI)
        return fail(STENCIL_EINVAL, "iterative refinement solves the JACOBI steady state");
    if (ir->storage != STENCIL_STORAGE_BF16 && ir->storage != STENCIL_STORAGE_FP16)
        return fail(STENCIL_EINVAL, "storage must be STENCIL_STORAGE_BF16 or STENCIL_STORAGE_FP16");
    if (ir->inner_sweeps < 0 || ir->check_every < 0 || ir->tol < 0.0 || ir->temporal < 0 ||
        ir->tile_x < 0 || ir->tile_y < 0)
        return fail(STENCIL_EINVAL,
                    "inner_sweeps, check_every, temporal, tile_x, tile_y and tol must be >= 0");
    if (ir->engine < STENCIL_IR_ENGINE_AUTO || ir->engine > STENCIL_IR_ENGINE_PERSISTENT_2D)
        return fail(STENCIL_EINVAL, "engine must be a STENCIL_IR_ENGINE_* value");
    if (ir->reserved) return fail(STENCIL_EINVAL, "reserved fields must be zero");
    if (p->nx % 8) return fail(STENCIL_EUNSUPPORTED, "IR needs nx %% 8 == 0");
    if (workspace_bytes < ir_bytes(*p, ir->storage))
        return fail(STENCIL_EINVAL, "workspace too small (%zu < %zu bytes)", workspace_bytes,
                    ir_bytes(*p, ir->storage));
    if ((reinterpret_cast<uintptr_t>(d_workspace) & 255) || (reinterpret_cast<uintptr_t>(d_u) & 15))
        return fail(STENCIL_EINVAL, "workspace must be 256-byte and u 16-byte aligned");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    char *ws = static_cast<char *>(d_workspace);
    if (ir->storage == STENCIL_STORAGE_BF16)
        return ir_dispatch<__nv_bfloat16>(*p, *ir, d_u, ws, s, result);
    return ir_dispatch<__half>(*p, *ir, d_u, ws, s, result);
}

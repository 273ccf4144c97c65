// k_border.cu -- seeded smooth Dirichlet borders for the precision and
// learned-warm-start workloads (no counterpart in the reference, whose only
// initial state is include/stencil_initializer.h:6-52).
//
// Mode parameters are drawn on the host from a SplitMix64 stream (Steele, Lea
// & Flood 2014) with Box-Muller normals, so the same seed gives the same
// border everywhere; values are evaluated on the device in double precision
// and rounded to float.
#include <math.h>

#include "host.hpp"

namespace st {

namespace {

struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(mix64(seed ^ 0x6A09E667F3BCC909ull)) {}
    double uniform() {  // [0, 1)
        s += 0x9E3779B97F4A7C15ull;
        return (double)(mix64(s) >> 11) * (1.0 / 9007199254740992.0);
    }
    double normal() {
        double u1 = uniform(), u2 = uniform();
        if (u1 < 1e-300) u1 = 1e-300;
        return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
    }
    int below(int n) { return (int)(uniform() * n); }
};

constexpr int kMaxModes = 16;

struct Modes3 {
    int n;
    float amp[kMaxModes], phase[kMaxModes];
    int kx[kMaxModes], ky[kMaxModes], kz[kMaxModes];
};

struct Edges2 {
    float corner[4];  // (0,0), (nx-1,0), (0,ny-1), (nx-1,ny-1)
    int count[4];     // bottom, top, left, right
    float amp[4][kMaxModes];
};

}  // namespace

__device__ __forceinline__ bool band(int i, int j, int k, const Geom &g, int dims) {
    const int R = g.radius;
    return !(in_range(i, g.nx, R) && in_range(j, g.ny, R) && (dims == 2 || in_range(k, g.nz, R)));
}

// Border band: sum of smooth periodic modes of the cell position; interior:
// uniform [0,1) from the same generator as stencil_init_uniform (seed).
__global__ void k_init_fourier(float *__restrict__ u, Geom g, int dims, Modes3 m, uint64_t seed) {
    const size_t n = (size_t)g.nx * g.ny * (dims == 3 ? g.nz : 1);
    const uint64_t base = mix64(seed);
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(idx % g.nx);
        const int j = (int)((idx / g.nx) % g.ny);
        const int k = (int)(idx / ((size_t)g.nx * g.ny));
        if (band(i, j, k, g, dims)) {
            double v = 0.0;
            for (int q = 0; q < m.n; ++q) {
                const double ph = 6.283185307179586 *
                                      ((double)m.kx[q] * i / g.nx + (double)m.ky[q] * j / g.ny +
                                       (double)m.kz[q] * k / (dims == 3 ? g.nz : 1)) +
                                  m.phase[q];
                v += (double)m.amp[q] * cos(ph);
            }
            u[idx] = (float)v;
        } else {
            const uint64_t z = mix64(base + 0x9E3779B97F4A7C15ull * (idx + 1));
            u[idx] = (float)(z >> 40) * (1.0f / 16777216.0f);
        }
    }
}

// 2-D Laplace borders: on each edge the linear interpolation of its two
// corner values plus sum_k amp_k sin(pi k t), t in [0, 1] along the edge, so
// the border is continuous at the corners.  Interior zero.
__global__ void k_init_laplace2d(float *__restrict__ u, Geom g, Edges2 e) {
    const size_t n = (size_t)g.nx * g.ny;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(idx % g.nx), j = (int)(idx / g.nx);
        const int R = g.radius;
        float val = 0.0f;
        if (!(in_range(i, g.nx, R) && in_range(j, g.ny, R))) {
            int edge;
            double t;
            if (j < R) { edge = 0; t = (double)i / (g.nx - 1); }
            else if (j >= g.ny - R) { edge = 1; t = (double)i / (g.nx - 1); }
            else if (i < R) { edge = 2; t = (double)j / (g.ny - 1); }
            else { edge = 3; t = (double)j / (g.ny - 1); }
            const double c0 = edge == 0 ? e.corner[0] : edge == 1 ? e.corner[2] : edge == 2 ? e.corner[0] : e.corner[1];
            const double c1 = edge == 0 ? e.corner[1] : edge == 1 ? e.corner[3] : edge == 2 ? e.corner[2] : e.corner[3];
            double v = c0 + (c1 - c0) * t;
            if (t > 0.0 && t < 1.0)
                for (int q = 0; q < e.count[edge]; ++q) v += (double)e.amp[edge][q] * sin(3.141592653589793 * (q + 1) * t);
            val = (float)v;
        }
        u[idx] = val;
    }
}

}  // namespace st

using namespace st;

extern "C" int stencil_init_fourier(const stencil_params *p, float *d_u, uint64_t seed, int modes,
                                    stencil_stream_t stream) {
    int rc = stencil_params_check(p);
    if (rc) return rc;
    if (!d_u || modes < 0 || modes > kMaxModes) return fail(STENCIL_EINVAL, "modes must be in [0, 16]");
    Modes3 m = {};
    Rng rng(seed);
    m.n = modes;
    for (int q = 0; q < modes; ++q) {
        m.kx[q] = rng.below(4);
        m.ky[q] = rng.below(4);
        m.kz[q] = p->dims == 3 ? rng.below(4) : 0;
        m.amp[q] = (float)rng.normal();
        m.phase[q] = (float)(6.283185307179586 * rng.uniform());
    }
    const Geom g = make_geom(*p);
    k_init_fourier<<<8 * num_sms(), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
        d_u, g, p->dims, m, seed);
    return cuda_fail(cudaGetLastError(), "init_fourier launch");
}

extern "C" int stencil_init_laplace2d(const stencil_params *p, float *d_u, uint64_t seed,
                                      stencil_stream_t stream) {
    int rc = stencil_params_check(p);
    if (rc) return rc;
    if (!d_u || p->dims != 2) return fail(STENCIL_EINVAL, "2-D grid required");
    Edges2 e = {};
    Rng rng(seed);
    for (int c = 0; c < 4; ++c) e.corner[c] = (float)rng.normal();
    for (int ed = 0; ed < 4; ++ed) {
        e.count[ed] = 1 + rng.below(kMaxModes);
        for (int q = 0; q < e.count[ed]; ++q) e.amp[ed][q] = (float)rng.normal();
    }
    const Geom g = make_geom(*p);
    k_init_laplace2d<<<8 * num_sms(), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(d_u, g, e);
    return cuda_fail(cudaGetLastError(), "init_laplace2d launch");
}

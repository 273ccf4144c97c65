/*
 * stencil_oracle.c -- CPU restatement of the reference star-stencil sweep loop.
 *
 * TEST INFRASTRUCTURE ONLY (the checker): used by tests/, by smoke() and by the
 * CPU-baseline leg of bench.py; never linked into the CUDA library.  See
 * stencil_oracle.h for the reference lines each function follows.
 *
 * Build: gcc -O2 -fPIC -shared -fopenmp -ffp-contract=off (oracle/build.py).
 * The sweep contains no multiplications that could be contracted, but the
 * flag documents that none may be.
 */
#include "stencil_oracle.h"

#include <math.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---------------------------------------------------------------------------
 * FP32 sweep.  The cell loop body follows src/stencils.cu:8-19 with the
 * accumulators of src/stencil_accumulators.cu:6-16/:46-74: for each axis in the
 * order i (stride 1), j (stride nx), k (stride nx*ny) add the R "previous"
 * neighbours from distance R down to 1, then the R "next" neighbours from
 * distance 1 up to R, into one float accumulator; divide by (float)(2*D*R).
 * The j-axis "next" stride in the reference is NY (stencil_accumulators.cu:63),
 * equal to NX for the reference's square grids; the restatement uses nx, the
 * row pitch, which is what the reference means.
 * ------------------------------------------------------------------------- */
static inline float cell_f32(const float *u, size_t idx, int dims, size_t sy, size_t sz,
                             int radius, float coeff, int mode)
{
    float acc = 0.0f;
    int d;
    for (d = radius; d >= 1; d--) acc += u[idx - (size_t)d];
    for (d = 1; d <= radius; d++) acc += u[idx + (size_t)d];
    for (d = radius; d >= 1; d--) acc += u[idx - (size_t)d * sy];
    for (d = 1; d <= radius; d++) acc += u[idx + (size_t)d * sy];
    if (dims > 2) {
        for (d = radius; d >= 1; d--) acc += u[idx - (size_t)d * sz];
        for (d = 1; d <= radius; d++) acc += u[idx + (size_t)d * sz];
    }
    if (mode == STENCIL_ORACLE_LEGACY) return acc / coeff - u[idx];
    return acc / coeff;
}

static inline double cell_f64(const double *u, size_t idx, int dims, size_t sy, size_t sz,
                              int radius, double coeff, int mode)
{
    double acc = 0.0;
    int d;
    for (d = radius; d >= 1; d--) acc += u[idx - (size_t)d];
    for (d = 1; d <= radius; d++) acc += u[idx + (size_t)d];
    for (d = radius; d >= 1; d--) acc += u[idx - (size_t)d * sy];
    for (d = 1; d <= radius; d++) acc += u[idx + (size_t)d * sy];
    if (dims > 2) {
        for (d = radius; d >= 1; d--) acc += u[idx - (size_t)d * sz];
        for (d = 1; d <= radius; d++) acc += u[idx + (size_t)d * sz];
    }
    if (mode == STENCIL_ORACLE_LEGACY) return acc / coeff - u[idx];
    return acc / coeff;
}

void oracle_sweep_f32(const float *src, float *dst, int dims, int nx, int ny, int nz,
                      int radius, int mode, int threads)
{
    const size_t sy = (size_t)nx, sz = (size_t)nx * (size_t)ny;
    const float coeff = (float)2 * dims * radius; /* include/constants.h:43 */
    const long kz0 = dims > 2 ? radius : 0, kz1 = dims > 2 ? nz - radius : 1;
    long k;
    if (threads < 1) threads = 1;
#pragma omp parallel for schedule(static) num_threads(threads) if (threads > 1)
    for (k = kz0; k < kz1; k++) {
        long j, i;
        for (j = radius; j < ny - radius; j++)
            for (i = radius; i < nx - radius; i++) {
                size_t idx = (size_t)i + (size_t)j * sy + (size_t)k * sz;
                dst[idx] = cell_f32(src, idx, dims, sy, sz, radius, coeff, mode);
            }
    }
}

void oracle_sweep_f64(const double *src, double *dst, int dims, int nx, int ny, int nz,
                      int radius, int mode, int threads)
{
    const size_t sy = (size_t)nx, sz = (size_t)nx * (size_t)ny;
    const double coeff = 2.0 * dims * radius;
    const long kz0 = dims > 2 ? radius : 0, kz1 = dims > 2 ? nz - radius : 1;
    long k;
    if (threads < 1) threads = 1;
#pragma omp parallel for schedule(static) num_threads(threads) if (threads > 1)
    for (k = kz0; k < kz1; k++) {
        long j, i;
        for (j = radius; j < ny - radius; j++)
            for (i = radius; i < nx - radius; i++) {
                size_t idx = (size_t)i + (size_t)j * sy + (size_t)k * sz;
                dst[idx] = cell_f64(src, idx, dims, sy, sz, radius, coeff, mode);
            }
    }
}

/* Ping-pong driver after src/stencil_cpu.cu:32-35. */
int oracle_run_f32(float *a, float *b, int dims, int nx, int ny, int nz, int radius,
                   int mode, int iterations, int threads)
{
    float *cur = a, *nxt = b, *t;
    int it;
    for (it = 0; it < iterations; it++) {
        oracle_sweep_f32(cur, nxt, dims, nx, ny, nz, radius, mode, threads);
        t = cur; cur = nxt; nxt = t;
    }
    return cur == a ? 0 : 1;
}

int oracle_run_f64(double *a, double *b, int dims, int nx, int ny, int nz, int radius,
                   int mode, int iterations, int threads)
{
    double *cur = a, *nxt = b, *t;
    int it;
    for (it = 0; it < iterations; it++) {
        oracle_sweep_f64(cur, nxt, dims, nx, ny, nz, radius, mode, threads);
        t = cur; cur = nxt; nxt = t;
    }
    return cur == a ? 0 : 1;
}

/* include/stencil_initializer.h:6-52: outer layer 1.0f, else 0.0f. */
void oracle_init_reference(float *u, int dims, int nx, int ny, int nz)
{
    long i, j, k;
    const long kn = dims > 2 ? nz : 1;
    for (k = 0; k < kn; k++)
        for (j = 0; j < ny; j++)
            for (i = 0; i < nx; i++) {
                int edge = i == 0 || i == nx - 1 || j == 0 || j == ny - 1 ||
                           (dims > 2 && (k == 0 || k == nz - 1));
                u[(size_t)i + (size_t)j * nx + (size_t)k * nx * ny] = edge ? 1.0f : 0.0f;
            }
}

/* SplitMix64 finaliser (Steele, Lea & Flood 2014). */
static inline uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

float oracle_uniform01(uint64_t seed, uint64_t idx)
{
    uint64_t z = mix64(mix64(seed) + 0x9E3779B97F4A7C15ULL * (idx + 1));
    return (float)(z >> 40) * (1.0f / 16777216.0f);
}

void oracle_init_uniform(float *u, size_t count, uint64_t seed)
{
    size_t i;
    for (i = 0; i < count; i++) u[i] = oracle_uniform01(seed, i);
}

static inline int in_update(long i, long j, long k, int dims, int nx, int ny, int nz, int r)
{
    if (i < r || i >= nx - r || j < r || j >= ny - r) return 0;
    if (dims > 2 && (k < r || k >= nz - r)) return 0;
    return 1;
}

void oracle_copy_border(const float *src, float *dst, int dims, int nx, int ny, int nz,
                        int radius)
{
    long i, j, k;
    const long kn = dims > 2 ? nz : 1;
    for (k = 0; k < kn; k++)
        for (j = 0; j < ny; j++)
            for (i = 0; i < nx; i++)
                if (!in_update(i, j, k, dims, nx, ny, nz, radius)) {
                    size_t idx = (size_t)i + (size_t)j * nx + (size_t)k * nx * ny;
                    dst[idx] = src[idx];
                }
}

/* include/stencil_error_checker.h:6-54 accumulates (a-b)^2 in double. */
double oracle_sq_err(const float *a, const float *b, size_t count)
{
    double err = 0.0;
    size_t i;
    for (i = 0; i < count; i++) {
        double d = (double)a[i] - (double)b[i];
        err += d * d;
    }
    return err;
}

double oracle_max_rel_err(const float *a, const float *b, size_t count, double floor_,
                          size_t *nonfinite)
{
    double m = 0.0;
    size_t i, bad = 0;
    for (i = 0; i < count; i++) {
        double x = a[i], y = b[i], den, e;
        if (!isfinite(x) || !isfinite(y)) { bad++; continue; }
        den = fabs(y) > floor_ ? fabs(y) : floor_;
        e = fabs(x - y) / den;
        if (e > m) m = e;
    }
    if (nonfinite) *nonfinite = bad;
    return m;
}

double oracle_max_rel_err_f64(const float *a, const double *b, size_t count,
                              double floor_, size_t *nonfinite)
{
    double m = 0.0;
    size_t i, bad = 0;
    for (i = 0; i < count; i++) {
        double x = a[i], y = b[i], den, e;
        if (!isfinite(x) || !isfinite(y)) { bad++; continue; }
        den = fabs(y) > floor_ ? fabs(y) : floor_;
        e = fabs(x - y) / den;
        if (e > m) m = e;
    }
    if (nonfinite) *nonfinite = bad;
    return m;
}

double oracle_rel_residual(const float *u, int dims, int nx, int ny, int nz, int radius,
                           int threads)
{
    const size_t sy = (size_t)nx, sz = (size_t)nx * (size_t)ny;
    const double coeff = 2.0 * dims * radius;
    const long kz0 = dims > 2 ? radius : 0, kz1 = dims > 2 ? nz - radius : 1;
    double rr = 0.0, bb = 0.0;
    long k;
    if (threads < 1) threads = 1;
#pragma omp parallel for schedule(static) num_threads(threads) reduction(+:rr,bb) if (threads > 1)
    for (k = kz0; k < kz1; k++) {
        long j, i;
        for (j = radius; j < ny - radius; j++)
            for (i = radius; i < nx - radius; i++) {
                size_t idx = (size_t)i + (size_t)j * sy + (size_t)k * sz;
                double all = 0.0, bnd = 0.0, r;
                int d, ax;
                for (ax = 0; ax < dims; ax++) {
                    size_t s = ax == 0 ? 1 : (ax == 1 ? sy : sz);
                    for (d = -radius; d <= radius; d++) {
                        long ii = i, jj = j, kk = k;
                        double v;
                        if (d == 0) continue;
                        if (ax == 0) ii += d; else if (ax == 1) jj += d; else kk += d;
                        v = (double)u[(size_t)((long)idx + (long)d * (long)s)];
                        all += v;
                        if (!in_update(ii, jj, kk, dims, nx, ny, nz, radius)) bnd += v;
                    }
                }
                r = all / coeff - (double)u[idx];
                bnd /= coeff;
                rr += r * r;
                bb += bnd * bnd;
            }
    }
    return bb > 0.0 ? sqrt(rr) / sqrt(bb) : sqrt(rr);
}

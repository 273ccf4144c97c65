/*
 * stencil_oracle.h -- CPU restatement of the reference star-stencil sweep loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This header and stencil_oracle.c are the checker
 * for the CUDA library in thesis_gb300/: the parity tests, smoke() and the
 * CPU-baseline leg of bench.py call it.  No product code path links it.
 *
 * What it restates (reference paths are relative to the mrfarstad/thesis root):
 *   - per-cell update           src/stencils.cu:8-19 (stencil())
 *   - accumulation order        src/stencil_accumulators.cu:6-16 (prev d=R..1,
 *                               next d=1..R), :46-74 (i, then j, then k axis)
 *   - sweep loops               src/stencil_cpu_kernel.cu:4-25 (cells with every
 *                               coordinate in [R, N-R), k outer, i inner)
 *   - ping-pong driver          src/stencil_cpu.cu:20-43 (swap after each sweep)
 *   - reference initial state   include/stencil_initializer.h:6-52 (outer cell
 *                               layer 1.0f, everything else 0.0f)
 *   - error check               include/stencil_error_checker.h:6-54 (sum of
 *                               squared differences, RMS)
 *
 * Two update modes share one loop nest:
 *   STENCIL_ORACLE_LEGACY : u' = (sum of the 2*D*R axis neighbours)/(float)(2*D*R) - u
 *                           (the reference's formula, bit-exact with its stencil_cpu)
 *   STENCIL_ORACLE_JACOBI : u' = (sum of the 2*D*R axis neighbours)/(float)(2*D*R)
 *
 * Parity pin: in LEGACY mode with the reference initial state and an all-zero
 * second buffer the FP32 sweep is bit-identical to the reference's own
 * stencil_cpu, compiled from its sources by oracle/build_ref.sh; the golden
 * fixtures in tests/golden/ were produced that way.  JACOBI mode differs only
 * in the epilogue (no centre subtraction) and is pinned by the same loop.
 */
#ifndef STENCIL_ORACLE_H
#define STENCIL_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { STENCIL_ORACLE_LEGACY = 0, STENCIL_ORACLE_JACOBI = 1 };

/* One sweep, FP32, reference summation order.  Writes only cells whose every
 * coordinate lies in [R, N-R); every other cell of dst is left untouched.
 * nz is ignored when dims == 2.  threads <= 1 runs the single-threaded loop
 * nest of the reference; threads > 1 splits the outermost axis across OpenMP
 * threads (each cell's arithmetic is unchanged, so results are identical). */
void oracle_sweep_f32(const float *src, float *dst, int dims, int nx, int ny, int nz,
                      int radius, int mode, int threads);

/* The same sweep in FP64 (inputs and coefficient promoted to double). */
void oracle_sweep_f64(const double *src, double *dst, int dims, int nx, int ny, int nz,
                      int radius, int mode, int threads);

/* `iterations` ping-pong sweeps between a and b starting from a.  Returns 0 if
 * the final state is in a, 1 if it is in b (src/stencil_cpu.cu:32-35 swaps
 * after every sweep, so the result is in a for even counts). */
int oracle_run_f32(float *a, float *b, int dims, int nx, int ny, int nz, int radius,
                   int mode, int iterations, int threads);
int oracle_run_f64(double *a, double *b, int dims, int nx, int ny, int nz, int radius,
                   int mode, int iterations, int threads);

/* Reference initial state: 1.0f on the outermost cell layer, 0.0f elsewhere
 * (include/stencil_initializer.h:6-52). */
void oracle_init_reference(float *u, int dims, int nx, int ny, int nz);

/* Seeded i.i.d. uniform [0,1) fill: value(idx) = top 24 bits of
 * mix64(mix64(seed) + GAMMA*(idx+1)) times 2^-24, where mix64 is the
 * SplitMix64 finaliser (Steele, Lea & Flood, OOPSLA 2014) and GAMMA =
 * 0x9E3779B97F4A7C15.  Integer-only, so host and device agree bit for bit. */
float oracle_uniform01(uint64_t seed, uint64_t idx);
void oracle_init_uniform(float *u, size_t count, uint64_t seed);

/* Copies the border band (cells with any coordinate outside [R, N-R)) of src
 * into dst. */
void oracle_copy_border(const float *src, float *dst, int dims, int nx, int ny, int nz,
                        int radius);

/* Sum of squared differences and max relative error |a-b|/max(|b|, floor). The
 * non-finite count is returned through *nonfinite (cells where a or b is NaN
 * or Inf). */
double oracle_sq_err(const float *a, const float *b, size_t count);
double oracle_max_rel_err(const float *a, const float *b, size_t count, double floor_,
                          size_t *nonfinite);
double oracle_max_rel_err_f64(const float *a, const double *b, size_t count,
                              double floor_, size_t *nonfinite);

/* Relative residual of the steady-state problem that JACOBI mode iterates to:
 * A u = b with (A u)(x) = u(x) - mean of the 2*D*R axis neighbours inside the
 * update region and b the border contributions.  Returns ||b - A u||_2 / ||b||_2
 * accumulated in FP64. */
double oracle_rel_residual(const float *u, int dims, int nx, int ny, int nz, int radius,
                           int threads);

#ifdef __cplusplus
}
#endif
#endif

/*
 * constants.h -- compile-time configuration of the drop-in stencil_dispatch()
 * entry point (include/stencil_dispatch.h).
 *
 * Same macro names, meanings and defaults as the reference's include/constants.h
 * (mrfarstad/thesis include/constants.h:1-110), so a build line such as
 *     nvcc ... -D DIMENSIONS=3 -D DIM=512 -D RADIUS=4 -D ITERATIONS=1000 -D SMEM=true -D REGISTER=true
 * selects the same configuration here as there.  Kept names: HEURISTIC, ARCH,
 * BLOCK_X/Y/Z, NGPUS, ITERATIONS, DIM, DIMENSIONS, RADIUS, SMEM_PAD,
 * STENCIL_COEFF, COARSEN_X, PADDED, REGISTER, SMEM, COOP, DEBUG, NX/NY/NZ, SIZE,
 * BYTES, MAX, MIN.  Dropped: the multi-GPU slab sizes (OFFSET, BYTES_PER_GPU,
 * GHOST_ZONE*, INTERNAL_*), since this library runs on one GPU; NGPUS is kept
 * but must be 1.
 *
 * Added:
 *   STENCIL_MODE  STENCIL_MODE_LEGACY (default): the reference update
 *                 u' = sum/(2*D*R) - u with whatever border the caller's second
 *                 buffer holds; STENCIL_MODE_JACOBI: u' = sum/(2*D*R) with the
 *                 border band equal in both buffers.
 *   TEMPORAL_T    sweeps fused per HBM round trip by the COOP variant
 *                 (0 = the library chooses).
 * HEURISTIC keeps its name with two settings: true (1) leaves the block shape
 * to this library (its per-kernel default or tuning table); 2 takes the
 * reference's occupancy-based shape (stencil_heuristic_geometry).
 */
#ifndef STENCIL_CONSTANTS_H
#define STENCIL_CONSTANTS_H

/* true/false as in the reference, which is compiled as C++; C callers get them
 * from stdbool.h. */
#if !defined(__cplusplus)
#include <stdbool.h>
#endif

#ifndef HEURISTIC
#define HEURISTIC false
#endif
#ifndef ARCH
#define ARCH sm_103a
#endif

#ifndef BLOCK_X
#define BLOCK_X 32
#endif
#ifndef BLOCK_Y
#define BLOCK_Y 2
#endif
#ifndef BLOCK_Z
#define BLOCK_Z 2
#endif

#ifndef NGPUS
#define NGPUS 1
#endif
#if NGPUS != 1
#error "this library runs on one GPU: NGPUS must be 1 (the multi-GPU halo exchange is not built)"
#endif

#ifndef ITERATIONS
#define ITERATIONS 64
#endif
#ifndef DIM
#define DIM 256
#endif
#ifndef DIMENSIONS
#define DIMENSIONS 3
#endif
#ifndef RADIUS
#define RADIUS 1
#endif
#ifndef SMEM_PAD
#define SMEM_PAD 0
#endif

#define STENCIL_COEFF ((float)2 * DIMENSIONS * RADIUS)

#ifndef COARSEN_X
#define COARSEN_X 4
#endif
#ifndef PADDED
#define PADDED false
#endif
#ifndef REGISTER
#define REGISTER false
#endif
#ifndef SMEM
#define SMEM false
#endif
#ifndef COOP
#define COOP false
#endif
#ifndef DEBUG
#define DEBUG false
#endif

#ifndef STENCIL_MODE
#define STENCIL_MODE STENCIL_MODE_LEGACY
#endif
#ifndef TEMPORAL_T
#define TEMPORAL_T 0
#endif

#define NX (DIM)
#define NY (DIM)
#define NZ (DIM)
#if DIMENSIONS == 3
#define SIZE (NX * NY * (unsigned long)NZ)
#elif DIMENSIONS == 2
#define SIZE (NX * (unsigned long)NY)
#else
#define SIZE ((unsigned long)NX)
#endif
#define BYTES (SIZE * sizeof(float))

#define MAX(x, y) (((x) > (y)) ? (x) : (y))
#define MIN(x, y) (((x) < (y)) ? (x) : (y))

#endif /* STENCIL_CONSTANTS_H */

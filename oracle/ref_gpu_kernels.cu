/*
 * Wrapper translation unit that compiles the reference's own one-sweep GPU
 * kernels (src/stencil_kernel_{base,smem,smem_padded,smem_register}.cu,
 * mrfarstad/thesis) unchanged, from where their sources lie, for sm_103a.
 * TEST INFRASTRUCTURE ONLY: oracle/build.py builds it into one cubin per
 * compile-time configuration under oracle/_ref/ (the kernels take DIM,
 * RADIUS, BLOCK_X/Y/Z and COARSEN_X as macros); oracle/ref_gpu.py launches
 * them with the reference's dispatch geometry.  The coop kernel is left out:
 * the reference never launches it (src/stencil_dispatch.cu:160-177).
 */
#include "src/stencil_kernel_base.cu"
#include "src/stencil_kernel_smem.cu"
#include "src/stencil_kernel_smem_padded.cu"
#include "src/stencil_kernel_smem_register.cu"

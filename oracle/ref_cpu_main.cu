/*
 * Wrapper translation unit that compiles the reference's own CPU sweep loop,
 * src/stencil_cpu.cu (mrfarstad/thesis), unchanged, from where its sources lie.
 * TEST INFRASTRUCTURE ONLY: oracle/build.py builds it into oracle/_ref/ with the
 * reference's -D DIMENSIONS/DIM/RADIUS/ITERATIONS macros.  Running the binary
 * writes solutions/solution_<DIM>_<ITERATIONS>_<RADIUS>_<DIMENSIONS>d (raw
 * float32, include/stencil_utils.h:16-44) into its working directory and prints
 * the sweep-loop time (in seconds, src/stencil_cpu.cu:36-37).
 */
#include "src/stencil_cpu.cu"

int main() { stencil_cpu(); return 0; }

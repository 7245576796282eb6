// kdgrid_fast.cu — the MDAS kernels in the reference's arithmetic.
// Compiled with --use_fast_math, as SDK/CMakeLists.txt:163-180 compiles
// SDK/lib/mdas/kdgrid.cu, so divisions, square roots, powf and FMA contraction
// lower to the same instructions as in the reference build.
#define MDAS_NS mdas_fast
#define MDAS_REFERENCE_ARITH 1
#include "kdgrid_kernels.cuh"
#include "batch_kernels.cuh"

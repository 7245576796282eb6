// kdgrid_ieee.cu — the MDAS kernels in strict IEEE-754 binary32 arithmetic.
// Compiled with -fmad=false -prec-div=true -prec-sqrt=true -ftz=false and the
// reproducible pow of ieee_math.h, so that a CPU restatement compiled with
// -ffp-contract=off reproduces every bit of every pass.
#define MDAS_NS mdas_ieee
#include "kdgrid_kernels.cuh"
#include "batch_kernels.cuh"

// lu_exact.cu -- the LU-MZ kernels without FMA contraction (-fmad=false):
// the reference's rounding, bit-for-bit the oracle.  The default.
#define LU_NS lu_exact
#include "lu_kernels.cuh"

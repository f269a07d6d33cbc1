// lu_fast.cu -- the LU-MZ kernels with FMA contraction (-fmad=true), used
// for the hot kernels of an NPBMZ_LU_FMA handle.
#define LU_NS lu_fast
#include "lu_kernels.cuh"

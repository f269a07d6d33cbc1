// step_fast.cu -- time-step kernels with FMA contraction (compiled with
// -fmad=true), FP64 and the FP32 line-solve instantiations.
#define NPBMZ_NS fast
#define NPBMZ_HAS_FP32 1
#include "step_launch.h"
#include "step_kernels.cuh"

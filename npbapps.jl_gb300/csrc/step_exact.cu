// step_exact.cu -- time-step kernels, FP64 without FMA contraction
// (compiled with -fmad=false): the reference's arithmetic bit for bit.
#define NPBMZ_NS exact
#define NPBMZ_HAS_FP32 0
#include "step_launch.h"
#include "step_kernels.cuh"

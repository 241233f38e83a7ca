// FP32 population kernels (FP32 collision arithmetic with FMA contraction;
// force, momentum and tracer reductions stay in FP64).
#define SLBC_T float
#define SLBC_SUFFIX f32
#define SLBC_EXACT false
#include "slbc_launch.cuh"

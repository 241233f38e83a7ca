// FP64 population kernels.  This translation unit is compiled with
// -fmad=false: no multiply-add contraction, so every FP64 operation rounds
// exactly as the reference's double-precision C code does and the FP64 path
// reproduces its populations bit for bit.
#define SLBC_T double
#define SLBC_SUFFIX f64
#define SLBC_EXACT true
#include "slbc_launch.cuh"

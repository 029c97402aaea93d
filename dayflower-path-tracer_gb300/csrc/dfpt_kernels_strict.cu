// dfpt_kernels_strict.cu - the kernel set compiled with -fmad=false: one rounding per float
// operation, the arithmetic of the reference kernel, for bit-exact ray-cast parity; sin, cos, asin,
// atan2 and pow in double rounded once to float, as java.lang.Math's results cast to float.
#define DFPT_NS dfpt_strict
#define DFPT_STRICT_MATH
#include "dfpt_kernels.cuh"

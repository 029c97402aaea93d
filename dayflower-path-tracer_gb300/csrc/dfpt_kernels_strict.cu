// dfpt_kernels_strict.cu - the kernel set compiled with -fmad=false: one rounding per float
// operation, the arithmetic of the reference kernel, for bit-exact ray-cast parity.
#define DFPT_NS dfpt_strict
#include "dfpt_kernels.cuh"

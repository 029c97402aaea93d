// dfpt_kernels_fast.cu - the kernel set with FMA contraction (the path tracer's fast path).
#define DFPT_NS dfpt_fast
#include "dfpt_kernels.cuh"

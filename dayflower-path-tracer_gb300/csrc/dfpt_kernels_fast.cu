// dfpt_kernels_fast.cu - the kernel set with FMA contraction (the path tracer's fast path), with
// the batch stages and the path-replay adjoint.
#define DFPT_NS dfpt_fast
#define DFPT_EXTENDED_KERNELS
#define DFPT_FMA_SLABS
#include "dfpt_kernels.cuh"

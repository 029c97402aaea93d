// dfpt_kernels_wide.cu - the batch stages compiled for one scene (a handle's waves of passes): the
// scene record is the kernel parameter (constant bank) instead of a per-ray record in global
// memory, with the fast set's arithmetic. Only the batch stages and their adjoint are built here.
#define DFPT_NS dfpt_wide
#define DFPT_EXTENDED_KERNELS
#define DFPT_FMA_SLABS
#define DFPT_ONE_SCENE
#include "dfpt_kernels.cuh"

// Assembly kernels for throughput: multiply-adds contracted, and the
// closed-form linear-tet stiffness.
#define SG_ASM_NS fast
#define SG_ASM_EXACT false
#include "sg_assemble_impl.cuh"

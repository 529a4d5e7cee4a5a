// Assembly kernels in the reference operation order, compiled with
// --fmad=false (see simit_gb300/build.py) so that FP64 results match the
// reference's unfused arithmetic.
#define SG_ASM_NS exact
#define SG_ASM_EXACT true
#include "sg_assemble_impl.cuh"

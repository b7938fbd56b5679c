// Instantiations of the propagation kernel for one precision / value type
// (separate translation units so the build compiles them in parallel).
#define SPX_INST_F64 false
#define SPX_INST_CPLX false
#define SPX_INST_FN spx_kernel_f32r
#include "kern_inst.inc"

// Instantiations of the propagation kernel for one precision, value type and
// coil layout (separate translation units so the build compiles them in parallel).
#define SPX_INST_F64 false
#define SPX_INST_CPLX true
#define SPX_INST_SC true
#define SPX_INST_FN spx_kernel_f32c_sc
#define SPX_INST_WIDE
#include "kern_inst.inc"

// Instantiations of the propagation kernel with trajectory outputs (the state
// at every step) for one precision, value type and coil layout.
#define SPX_INST_F64 false
#define SPX_INST_CPLX false
#define SPX_INST_SC true
#define SPX_INST_TRJ true
#define SPX_INST_FN spx_kernel_f32r_sc_t
#include "kern_inst.inc"

// Instantiations of the propagation kernel with trajectory outputs (the state
// at every step) for one precision, value type and coil layout.
#define SPX_INST_F64 true
#define SPX_INST_CPLX true
#define SPX_INST_SC false
#define SPX_INST_TRJ true
#define SPX_INST_FN spx_kernel_f64c_dc_t
#include "kern_inst.inc"

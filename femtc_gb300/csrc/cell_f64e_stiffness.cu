// CUDA-core stiffness cell kernels, FP64 storage, double-float (FP32-pair)
// arithmetic: FP64-accurate results on the FP32 pipes.  Degrees 1..4, exact
// semantics.
#include "cell_inst.cuh"
FEMTC_CELL_UNIT_EXACT_UPTO(register_cell_f64e_stiffness, df64, 4, OP_STIFFNESS, 1, 5)

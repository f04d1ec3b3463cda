// CUDA-core stiffness cell kernels, float arithmetic and storage.
#include "cell_inst.cuh"
FEMTC_CELL_UNIT(register_cell_f32_stiffness, float, 1, OP_STIFFNESS)

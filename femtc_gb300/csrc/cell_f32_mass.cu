// CUDA-core mass cell kernels, float arithmetic and storage.
#include "cell_inst.cuh"
FEMTC_CELL_UNIT(register_cell_f32_mass, float, 1, OP_MASS)

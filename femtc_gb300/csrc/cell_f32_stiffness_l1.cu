// CUDA-core stiffness cell kernels, float arithmetic and storage, 1 lane(s) per slab.
#include "cell_inst.cuh"
FEMTC_CELL_UNIT(register_cell_f32_stiffness_l1, float, 1, OP_STIFFNESS, 1)

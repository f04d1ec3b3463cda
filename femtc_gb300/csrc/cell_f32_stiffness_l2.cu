// CUDA-core stiffness cell kernels, float arithmetic and storage, 2 lane(s) per slab.
#include "cell_inst.cuh"
FEMTC_CELL_UNIT(register_cell_f32_stiffness_l2, float, 1, OP_STIFFNESS, 2)

// CUDA-core mass cell kernels, float arithmetic and storage, 2 lane(s) per slab.
#include "cell_inst.cuh"
FEMTC_CELL_UNIT(register_cell_f32_mass_l2, float, 1, OP_MASS, 2)

// CUDA-core stiffness cell kernels, double arithmetic and storage, one lane per slab.
#include "cell_inst.cuh"
FEMTC_CELL_UNIT(register_cell_f64_stiffness, double, 0, OP_STIFFNESS, 1)

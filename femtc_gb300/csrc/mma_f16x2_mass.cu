// Tensor-core mass kernels, FP16 hi/lo split, FP32 accumulate.
#include "mma_inst.cuh"
FEMTC_MMA_UNIT(register_mma_f16x2_mass, SPLIT_F16X2, 2, OP_MASS)

// Tensor-core stiffness kernels, FP16 hi/lo split, FP32 accumulate.
#include "mma_inst.cuh"
FEMTC_MMA_UNIT(register_mma_f16x2_stiffness, SPLIT_F16X2, 2, OP_STIFFNESS)

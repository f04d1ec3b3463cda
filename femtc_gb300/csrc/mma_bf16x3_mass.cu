// Tensor-core mass kernels, BF16 three-term split, FP32 accumulate.
#include "mma_inst.cuh"
FEMTC_MMA_UNIT(register_mma_bf16x3_mass, SPLIT_BF16X3, 3, OP_MASS)

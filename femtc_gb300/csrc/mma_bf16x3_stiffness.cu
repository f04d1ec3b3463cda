// Tensor-core stiffness kernels, BF16 three-term split, FP32 accumulate.
#include "mma_inst.cuh"
FEMTC_MMA_UNIT(register_mma_bf16x3_stiffness, SPLIT_BF16X3, 3, OP_STIFFNESS)

// CUDA-core mass cell kernels, FP64 storage, double-float arithmetic, two
// lanes per slab (the autotuner picks one or two lanes).  Degrees 1..4,
// exact semantics.
#include "cell_inst.cuh"
FEMTC_CELL_UNIT_EXACT_UPTO(register_cell_f64e_mass_l2, df64, 4, OP_MASS, 2, 5)

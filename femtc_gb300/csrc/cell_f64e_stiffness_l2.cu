// CUDA-core stiffness cell kernels, FP64 storage, double-float arithmetic,
// two lanes per slab (the slab passes of a tile keep twice as many threads
// busy; the autotuner picks one or two lanes).  Degrees 1..4, exact
// semantics.
#include "cell_inst.cuh"
FEMTC_CELL_UNIT_EXACT_UPTO(register_cell_f64e_stiffness_l2, df64, 4, OP_STIFFNESS, 2, 5)

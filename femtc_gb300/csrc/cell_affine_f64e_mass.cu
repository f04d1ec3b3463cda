// CUDA-core mass cell kernels of the affine form (one geometry set per
// cell), FP64 storage, double-float arithmetic, exact semantics, one lane per
// slab, plain and even-odd, N = 2..5 (the double-float form's register
// footprint is twice FP32's; degrees above 4 spill).
#include "cell_inst.cuh"

namespace femtc
{
void register_cell_affine_f64e_mass(std::vector<CellVariant>& v, std::vector<FaultReader>& f)
{
  add_affine<df64, OP_MASS_AFFINE, 2, 5, 5>(v, 4); // FEMTC_F64E
  f.push_back(&read_clear_fault_word);
}
} // namespace femtc

// CUDA-core stiffness cell kernels of the affine form (one geometry set per
// cell), float arithmetic and storage, exact semantics, one lane per slab:
// plain N = 2..8 and even-odd N = 2..8.
#include "cell_inst.cuh"

namespace femtc
{
void register_cell_affine_f32_stiffness(std::vector<CellVariant>& v, std::vector<FaultReader>& f)
{
  add_affine<float, OP_STIFFNESS_AFFINE, 2, 8>(v, 1); // FEMTC_F32
  f.push_back(&read_clear_fault_word);
}
} // namespace femtc

// CUDA-core stiffness cell kernels, float arithmetic and storage, even-odd
// contractions (tables with the GLL-to-Gauss symmetry), exact semantics.
#include "cell_inst.cuh"

namespace femtc
{
void register_cell_f32eo_stiffness(std::vector<CellVariant>& v, std::vector<FaultReader>& f)
{
  add_even_odd<float, OP_STIFFNESS, 2, 8>(v, 1); // FEMTC_F32
  f.push_back(&read_clear_fault_word);
}
} // namespace femtc

// CUDA-core stiffness cell kernels, FP64 storage, double-float arithmetic,
// even-odd contractions (tables with the GLL-to-Gauss symmetry), exact
// semantics, degrees 1..4.
#include "cell_inst.cuh"

namespace femtc
{
void register_cell_f64eeo_stiffness(std::vector<CellVariant>& v, std::vector<FaultReader>& f)
{
  add_even_odd<df64, OP_STIFFNESS, 2, 5>(v, 4); // FEMTC_F64E
  f.push_back(&read_clear_fault_word);
}
} // namespace femtc

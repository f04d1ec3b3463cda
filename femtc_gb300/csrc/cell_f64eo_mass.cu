// CUDA-core mass cell kernels, double arithmetic and storage, even-odd
// contractions (tables with the GLL-to-Gauss symmetry), exact semantics.
#include "cell_inst.cuh"

namespace femtc
{
void register_cell_f64eo_mass(std::vector<CellVariant>& v, std::vector<FaultReader>& f)
{
  add_even_odd<double, OP_MASS, 2, 8>(v, 0); // FEMTC_F64
  f.push_back(&read_clear_fault_word);
}
} // namespace femtc

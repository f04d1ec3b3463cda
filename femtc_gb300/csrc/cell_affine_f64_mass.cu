// CUDA-core mass cell kernels of the affine form (one geometry set per
// cell), double arithmetic and storage, exact semantics, one lane per slab:
// plain N = 2..8 and even-odd N = 2..7.
#include "cell_inst.cuh"

namespace femtc
{
void register_cell_affine_f64_mass(std::vector<CellVariant>& v, std::vector<FaultReader>& f)
{
  add_affine<double, OP_MASS_AFFINE, 2, 7>(v, 0); // FEMTC_F64
  f.push_back(&read_clear_fault_word);
}
} // namespace femtc

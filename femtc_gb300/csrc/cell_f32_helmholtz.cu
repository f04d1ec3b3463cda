// CUDA-core Helmholtz cell kernels (alpha M + beta K in one pass), float
// arithmetic and storage, exact semantics.
#include "cell_inst.cuh"

namespace femtc
{
void register_cell_f32_helmholtz(std::vector<CellVariant>& v, std::vector<FaultReader>& f)
{
  add_helmholtz<float, 2>(v, 1); // FEMTC_F32
  f.push_back(&read_clear_fault_word);
}
} // namespace femtc

// CUDA-core Helmholtz cell kernels (alpha M + beta K in one pass), float
// arithmetic and storage, exact semantics; plain and even-odd contractions.
#include "cell_inst.cuh"

namespace femtc
{
void register_cell_f32_helmholtz(std::vector<CellVariant>& v, std::vector<FaultReader>& f)
{
  add_helmholtz<float, 2>(v, 1); // FEMTC_F32
  add_even_odd<float, OP_HELMHOLTZ, 2, 8>(v, 1);
  f.push_back(&read_clear_fault_word);
}
} // namespace femtc

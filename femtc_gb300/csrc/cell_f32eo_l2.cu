// CUDA-core mass and stiffness cell kernels, float arithmetic and storage,
// even-odd contractions with two lanes per slab (tables with the
// GLL-to-Gauss symmetry), exact semantics, degrees 1..4: the twins of the
// two-lane FP32 kernels, which the two-lane choice runs when the tables
// allow it.
#include "cell_inst.cuh"

namespace femtc
{
void register_cell_f32eo_l2(std::vector<CellVariant>& v, std::vector<FaultReader>& f)
{
  add_even_odd<float, OP_MASS, 2, 5, 2>(v, 1);      // FEMTC_F32
  add_even_odd<float, OP_STIFFNESS, 2, 5, 2>(v, 1); // FEMTC_F32
  f.push_back(&read_clear_fault_word);
}
} // namespace femtc

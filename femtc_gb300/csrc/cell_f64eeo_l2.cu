// CUDA-core mass and stiffness cell kernels, FP64 storage, double-float
// arithmetic, even-odd contractions with two lanes per slab (tables with the
// GLL-to-Gauss symmetry), exact semantics, degrees 1..4: the twins of the
// two-lane double-float kernels, which the two-lane choice runs when the
// tables allow it.
#include "cell_inst.cuh"

namespace femtc
{
void register_cell_f64eeo_l2(std::vector<CellVariant>& v, std::vector<FaultReader>& f)
{
  add_even_odd<df64, OP_MASS, 2, 5, 2>(v, 4);      // FEMTC_F64E
  add_even_odd<df64, OP_STIFFNESS, 2, 5, 2>(v, 4); // FEMTC_F64E
  f.push_back(&read_clear_fault_word);
}
} // namespace femtc

// CUDA-core stiffness cell kernels, FP64 storage, double-float arithmetic,
// exact semantics, degree 6 with Q = 8 (the P + 2 Gauss rule), two lanes per
// slab: the even-odd kernel, which runs for tables with the GLL-to-Gauss
// symmetry, and its plain twin, which holds the tile shape (it spills, so
// the launch path runs the general-degree kernel for tables without the
// symmetry).
#include "cell_inst.cuh"

namespace femtc
{
void register_cell_f64e_p6(std::vector<CellVariant>& v, std::vector<FaultReader>& f)
{
  add_variant<df64, 7, 8, OP_STIFFNESS, SEM_EXACT, 2>(v, 4);       // FEMTC_F64E
  add_variant<df64, 7, 8, OP_STIFFNESS, SEM_EXACT, 2, true>(v, 4); // FEMTC_F64E
  f.push_back(&read_clear_fault_word);
}
} // namespace femtc

// Host-side registry of the compiled kernel variants.  Each translation unit
// that instantiates kernels appends its variants (and the reader of its
// device fault word) at library load.
#pragma once

#include <cuda_runtime.h>
#include <vector>

namespace femtc
{

struct CellVariant
{
  int dtype;   // femtc_dtype
  int op;      // femtc_op
  int sem;     // femtc_semantics
  int n, q;    // DOFs and quadrature points per axis
  const void* fn;
  // dynamic shared memory (bytes) of a tile of cb cells
  unsigned (*smem)(int cb, int staged, int sq, int sbc);
  int slab;    // 1: slab-merged CUDA-core kernel (uses sq, sbc)
  int esize;   // bytes per stored value
  int lanes;   // slab kernels: lanes sharing one slab
  int eo = 0;  // 1: even-odd contractions (tables with the GLL-to-Gauss symmetry)
};

using FaultReader = unsigned (*)(); // returns and clears the unit's fault word

void register_cell_f64_mass(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_cell_f64_stiffness(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_cell_f32_mass_l1(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_cell_f32_mass_l2(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_cell_f32_stiffness_l1(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_cell_f32_stiffness_l2(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_cell_f32_helmholtz(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_cell_f64eo_mass(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_cell_f64eo_stiffness(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_cell_f32eo_mass(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_cell_f32eo_stiffness(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_cell_f64eeo_mass(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_cell_f64eeo_stiffness(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_cell_f64eeo_l2(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_cell_f64e_p6(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_cell_f64e_mass(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_cell_f64e_stiffness(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_cell_f64e_mass_l2(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_cell_f64e_stiffness_l2(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_cell_affine_f64_mass(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_cell_affine_f64_stiffness(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_cell_affine_f32_mass(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_cell_affine_f32_stiffness(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_cell_affine_f64e_mass(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_cell_affine_f64e_stiffness(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_mma_f16x2_mass(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_mma_f16x2_stiffness(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_mma_bf16x3_mass(std::vector<CellVariant>&, std::vector<FaultReader>&);
void register_mma_bf16x3_stiffness(std::vector<CellVariant>&, std::vector<FaultReader>&);
// General-degree kernels (cell_general.cu): runtime N and Q, mass and
// stiffness, FP64 and FP32, for the (N, Q) the slab kernels do not cover.
bool general_supported(int op, int dtype, int sem, int n, int q);
int launch_general(int op, int dtype, int sem, int n, int q, const void* tables, const void* u,
                   void* y, const void* geo, size_t ncells, cudaStream_t st);
// fault words of the batch kernel families and of the diagnostic unit
void register_batch_faults(std::vector<FaultReader>&);
void register_diag(std::vector<CellVariant>&, std::vector<FaultReader>&);

} // namespace femtc

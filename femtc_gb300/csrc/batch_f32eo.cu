// Batched persistent kernel, f32 family with even-odd contractions (see
// batch_kernel.cuh): used when every mesh's tables have the GLL-to-Gauss
// symmetry.
#include "batch_kernel.cuh"

namespace femtc
{
BatchKernelInfo batch_kernel_f32eo()
{
  return BatchKernelInfo{reinterpret_cast<const void*>(&batch_kernel<float, kFamilySlabEO>),
                         kFamilySlabEO, 1, &batch_bytes<float, kFamilySlabEO>,
                         &read_clear_fault_word};
}
} // namespace femtc

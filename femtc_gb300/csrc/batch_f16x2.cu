// Batched persistent kernel, f16x2 family (see batch_kernel.cuh).
#include "batch_kernel.cuh"

namespace femtc
{
BatchKernelInfo batch_kernel_f16x2()
{
  return BatchKernelInfo{reinterpret_cast<const void*>(&batch_kernel<float, kFamilyF16X2>),
                         kFamilyF16X2, 2, &batch_bytes<float, kFamilyF16X2>,
                         &read_clear_fault_word};
}
} // namespace femtc

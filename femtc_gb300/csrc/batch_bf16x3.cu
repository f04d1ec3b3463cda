// Batched persistent kernel, bf16x3 family (see batch_kernel.cuh).
#include "batch_kernel.cuh"

namespace femtc
{
BatchKernelInfo batch_kernel_bf16x3()
{
  return BatchKernelInfo{reinterpret_cast<const void*>(&batch_kernel<float, kFamilyBF16X3>),
                         kFamilyBF16X3, 3, &batch_bytes<float, kFamilyBF16X3>,
                         &read_clear_fault_word};
}
} // namespace femtc

// Batched persistent kernel, f32 family (see batch_kernel.cuh).
#include "batch_kernel.cuh"

namespace femtc
{
BatchKernelInfo batch_kernel_f32()
{
  return BatchKernelInfo{reinterpret_cast<const void*>(&batch_kernel<float, kFamilySlab>),
                         kFamilySlab, 1, &batch_bytes<float, kFamilySlab>,
                         &read_clear_fault_word};
}
} // namespace femtc

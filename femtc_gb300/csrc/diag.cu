// Diagnostic entry point: femtc_bounded_wait_check.
//
// Every mbarrier wait of the library's kernels is bounded (mbar_wait in
// common.cuh): a copy that never completes ends the kernel with a fault bit
// in its unit's fault word, read back by femtc_device_status, instead of a
// hang.  This unit launches one CTA whose wait can only run out -- thread 0
// arms an mbarrier for 16 transaction bytes that no copy will deliver -- so
// that path can be exercised on a GPU without any fault: no copy is issued,
// nothing is read or written out of bounds, and the kernel returns after
// `polls` polls.
#include "femtc_gpu.h"

#include "common.cuh"
#include "registry.hpp"

namespace femtc
{
int aux_fail(int code, const char* msg); // femtc_abi.cu

namespace
{
__global__ void bounded_wait_probe(int polls)
{
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0)
  {
    mbar_init(&bar, 1);
    fence_mbar_init();
    // the arrival is counted; the 16 transaction bytes never come, so the
    // phase cannot complete
    mbar_arrive_expect_tx(&bar, 16);
    if (!mbar_wait(&bar, 0, polls))
      record_fault(FAULT_MBAR_TIMEOUT);
  }
}
} // namespace

void register_diag(std::vector<CellVariant>&, std::vector<FaultReader>& f)
{
  f.push_back(&read_clear_fault_word);
}
} // namespace femtc

extern "C" int femtc_bounded_wait_check(int polls, void* stream)
{
  using namespace femtc;
  if (polls < 1 || polls > kMbarSpinLimit)
    return aux_fail(FEMTC_ERR_INVALID, "bounded_wait_check: polls in [1, 2^22]");
  bounded_wait_probe<<<1, 32, 0, static_cast<cudaStream_t>(stream)>>>(polls);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FEMTC_OK : aux_fail(FEMTC_ERR_CUDA, cudaGetErrorString(e));
}

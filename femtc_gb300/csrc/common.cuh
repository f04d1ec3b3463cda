// Shared device helpers for the femtc GB300 kernels: bulk-copy (TMA) and
// mbarrier wrappers in inline PTX, the bounded wait, and the device fault
// word that a timed-out wait sets instead of hanging.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace femtc
{

// Fault bits recorded by kernels (read back by femtc_device_status()).
enum : unsigned
{
  FAULT_MBAR_TIMEOUT = 1u,   // a TMA load never completed within the limit
  FAULT_BAD_DESCRIPTOR = 2u, // a batched work item named an unknown variant
};

// One word per device and translation unit; bounded waits set bits here and
// the host reads (and clears) it through the unit's registration hook.
static __device__ unsigned g_fault_word;

// Host: returns and clears this translation unit's fault word.  Internal
// linkage, so that every unit that includes this header reads its own word
// (an external inline function would be merged into one copy by the linker,
// reading one unit's word for all of them).
static inline unsigned read_clear_fault_word()
{
  unsigned w = 0, z = 0;
  if (cudaMemcpyFromSymbol(&w, g_fault_word, sizeof(w)) != cudaSuccess)
    return 0;
  if (w)
    cudaMemcpyToSymbol(g_fault_word, &z, sizeof(z));
  return w;
}

// Iteration limit of every mbarrier spin in this library.  try_wait suspends
// for a bounded, hardware-chosen time per call, so the limit is a bound on
// wall time of the order of a second, never an infinite loop.
constexpr int kMbarSpinLimit = 1 << 22;

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_mbar_init()
{
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem()
{
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar,
                                                      uint32_t bytes)
{
  asm volatile(
      "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
          smem_addr(bar)),
      "r"(bytes)
      : "memory");
}

// One arrival (no transaction bytes) on an mbarrier.
__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// Returns false when the phase did not complete within `limit` polls
// (kMbarSpinLimit for every kernel of the library; femtc_bounded_wait_check
// passes a short one).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity,
                                          int limit = kMbarSpinLimit)
{
  const uint32_t a = smem_addr(bar);
  for (int i = 0; i < limit; ++i)
  {
    uint32_t done;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(done)
                 : "r"(a), "r"(parity)
                 : "memory");
    if (done)
      return true;
  }
  return false;
}

// 1D bulk copy global -> shared (TMA engine), completion on `bar`.
// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src,
                                         uint32_t bytes, uint64_t* bar)
{
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::"
               "bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

// 1D bulk copy shared -> global (TMA store), tracked by bulk groups.
__device__ __forceinline__ void bulk_s2g(void* dst, const void* src,
                                         uint32_t bytes)
{
  asm volatile(
      "cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst),
      "r"(smem_addr(src)), "r"(bytes)
      : "memory");
}

// 2D tiled tensor copy global -> shared of the box at (x, y) of the tensor
// map `map` (a __grid_constant__ parameter), completion on `bar`; dst
// 128-byte aligned, x * element size a multiple of 16 bytes.  Box elements
// outside the tensor are written as zeros.
__device__ __forceinline__ void tma_load_2d(void* dst, const void* map, int x, int y,
                                            uint64_t* bar)
{
  asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
               " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_addr(dst)),
               "l"(map), "r"(x), "r"(y), "r"(smem_addr(bar))
               : "memory");
}

// 2D tiled tensor copy shared -> global of the box at (x, y), tracked by
// bulk groups; box elements outside the tensor are not written.
__device__ __forceinline__ void tma_store_2d(const void* map, int x, int y, const void* src)
{
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::
                   "l"(map), "r"(x), "r"(y), "r"(smem_addr(src))
               : "memory");
}

__device__ __forceinline__ void bulk_commit()
{
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

// Wait until the smem sources of all committed bulk stores may be reused.
__device__ __forceinline__ void bulk_wait_read0()
{
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

// Wait until all committed bulk stores are complete (visible in global).
__device__ __forceinline__ void bulk_wait0()
{
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

// Hint: fetch the line holding p into L2 (no result, no register; p must
// lie inside an allocation).
__device__ __forceinline__ void prefetch_l2(const void* p)
{
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// Hint: fetch the 128-byte lines of [p, p + bytes) into L2; worker `id` of
// `n` takes lines id, id + n, ...  Every address asked for lies inside the
// range (the first line is asked for at p itself).
__device__ __forceinline__ void prefetch_range_l2(const void* p, size_t bytes, int id, int n)
{
  const uintptr_t b = reinterpret_cast<uintptr_t>(p), e = b + bytes;
  const uintptr_t a = b & ~uintptr_t(127);
  for (uintptr_t k = (uintptr_t)id;; k += (uintptr_t)n)
  {
    const uintptr_t l = k == 0 ? b : a + k * 128u;
    if (l >= e)
      break;
    prefetch_l2(reinterpret_cast<const void*>(l));
  }
}

__device__ __forceinline__ void record_fault(unsigned bits)
{
  atomicOr(&g_fault_word, bits);
}

} // namespace femtc

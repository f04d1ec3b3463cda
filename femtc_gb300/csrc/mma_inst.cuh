// Instantiates the tensor-core split kernels of one split form for every
// supported (N, Q), exact semantics: N = 2..8, Q = N, N+1, N+2 (Q <= 10).
#pragma once

#include "mma_kernel.cuh"
#include "registry.hpp"

namespace femtc
{
template <int SPLIT, int N, int Q, int OP>
unsigned mma_smem_bytes(int cb, int staged, int, int)
{
  CellParams<float> p{};
  p.cb = cb;
  p.geo_staged = staged;
  return tile_layout<float, MmaTile<SPLIT, N, Q, OP>, N, Q,
                     geo_nc(OP)>(p)
      .total;
}

template <int SPLIT, int N, int Q, int OP>
void add_mma_variant(std::vector<CellVariant>& v, int dtype)
{
  v.push_back(CellVariant{dtype, OP, SEM_EXACT, N, Q,
                          reinterpret_cast<const void*>(&mma_kernel<SPLIT, N, Q, OP>),
                          &mma_smem_bytes<SPLIT, N, Q, OP>, 0, 4, 1});
}

template <int SPLIT, int OP, int N>
void add_mma_degree(std::vector<CellVariant>& v, int dtype)
{
  add_mma_variant<SPLIT, N, N, OP>(v, dtype);
  add_mma_variant<SPLIT, N, N + 1, OP>(v, dtype);
  if constexpr (N + 2 <= kMaxQ)
    add_mma_variant<SPLIT, N, N + 2, OP>(v, dtype);
}

template <int SPLIT, int OP>
void add_mma_all(std::vector<CellVariant>& v, int dtype)
{
  add_mma_degree<SPLIT, OP, 2>(v, dtype);
  add_mma_degree<SPLIT, OP, 3>(v, dtype);
  add_mma_degree<SPLIT, OP, 4>(v, dtype);
  add_mma_degree<SPLIT, OP, 5>(v, dtype);
  add_mma_degree<SPLIT, OP, 6>(v, dtype);
  add_mma_degree<SPLIT, OP, 7>(v, dtype);
  add_mma_degree<SPLIT, OP, 8>(v, dtype);
}

} // namespace femtc

#define FEMTC_MMA_UNIT(NAME, SPLIT, DTYPE, OP)                                 \
  namespace femtc                                                              \
  {                                                                            \
  void NAME(std::vector<CellVariant>& v, std::vector<FaultReader>& f)          \
  {                                                                            \
    add_mma_all<SPLIT, OP>(v, DTYPE);                                          \
    f.push_back(&read_clear_fault_word);                                       \
  }                                                                            \
  }

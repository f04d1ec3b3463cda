// Instantiates the CUDA-core cell kernels of one (element type, operator)
// for every supported (N, Q, semantics) and registers them.
//   exact semantics     : N = 2..8 (degree 1..7), Q = N, N+1, N+2 (Q <= 10)
//   reference semantics : Q = N (the reference's only option)
#pragma once

#include "cell_kernel.cuh"
#include "registry.hpp"

namespace femtc
{
template <typename T, int N, int Q, int OP, int SEM, int L, bool EVOD = false>
unsigned cell_smem_bytes(int cb, int staged, int sq, int sbc)
{
  CellParams<T> p{};
  p.cb = cb;
  p.geo_staged = staged;
  p.sq = sq;
  p.sbc = sbc;
  return tile_layout<T, SlabTile<T, N, Q, OP, SEM, L, EVOD, true>, N, Q, geo_nc(OP)>(p)
      .total;
}

template <typename T, int N, int Q, int OP, int SEM, int L, bool EVOD = false>
void add_variant(std::vector<CellVariant>& v, int dtype)
{
  v.push_back(CellVariant{dtype, OP, SEM, N, Q,
                          reinterpret_cast<const void*>(
                              &cell_kernel<T, N, Q, OP, SEM, L, EVOD>),
                          &cell_smem_bytes<T, N, Q, OP, SEM, L, EVOD>, 1, (int)sizeof(T),
                          L, EVOD ? 1 : 0});
}

// Even-odd variants (exact semantics, L lanes per slab), N = N0..MAXN,
// Q = N..N+2.
template <typename T, int OP, int N, int MAXN, int L = 1>
void add_even_odd(std::vector<CellVariant>& v, int dtype)
{
  if constexpr (N <= MAXN)
  {
    add_variant<T, N, N, OP, SEM_EXACT, L, true>(v, dtype);
    add_variant<T, N, N + 1, OP, SEM_EXACT, L, true>(v, dtype);
    add_variant<T, N, N + 2, OP, SEM_EXACT, L, true>(v, dtype);
    add_even_odd<T, OP, N + 1, MAXN, L>(v, dtype);
  }
}

template <typename T, int OP, int N, int L>
void add_degree(std::vector<CellVariant>& v, int dtype)
{
  add_variant<T, N, N, OP, SEM_EXACT, L>(v, dtype);
  add_variant<T, N, N + 1, OP, SEM_EXACT, L>(v, dtype);
  if constexpr (N + 2 <= kMaxQ)
    add_variant<T, N, N + 2, OP, SEM_EXACT, L>(v, dtype);
  add_variant<T, N, N, OP, SEM_REFERENCE, L>(v, dtype);
}

// L = lanes sharing one slab (1 or 2; see SlabTile)
template <typename T, int OP, int L>
void add_all(std::vector<CellVariant>& v, int dtype)
{
  add_degree<T, OP, 2, L>(v, dtype);
  add_degree<T, OP, 3, L>(v, dtype);
  add_degree<T, OP, 4, L>(v, dtype);
  add_degree<T, OP, 5, L>(v, dtype);
  add_degree<T, OP, 6, L>(v, dtype);
  add_degree<T, OP, 7, L>(v, dtype);
  add_degree<T, OP, 8, L>(v, dtype);
}

// Exact semantics, N = 2..MAXN only (the double-float form: its register
// footprint is twice FP32's, and degrees above 4 spill).
template <typename T, int OP, int L, int N, int MAXN>
void add_exact_upto(std::vector<CellVariant>& v, int dtype)
{
  if constexpr (N <= MAXN)
  {
    add_variant<T, N, N, OP, SEM_EXACT, L>(v, dtype);
    add_variant<T, N, N + 1, OP, SEM_EXACT, L>(v, dtype);
    add_variant<T, N, N + 2, OP, SEM_EXACT, L>(v, dtype);
    add_exact_upto<T, OP, L, N + 1, MAXN>(v, dtype);
  }
}

// Helmholtz (exact semantics only), N = N0..8, Q = N..N+2; lanes per slab
// as the stiffness operator's default (two up to N = 5).
template <typename T, int N>
void add_helmholtz(std::vector<CellVariant>& v, int dtype)
{
  if constexpr (N <= 8)
  {
    constexpr int L = N <= 5 ? 2 : 1;
    add_variant<T, N, N, OP_HELMHOLTZ, SEM_EXACT, L>(v, dtype);
    add_variant<T, N, N + 1, OP_HELMHOLTZ, SEM_EXACT, L>(v, dtype);
    add_variant<T, N, N + 2, OP_HELMHOLTZ, SEM_EXACT, L>(v, dtype);
    add_helmholtz<T, N + 1>(v, dtype);
  }
}

// Affine forms (exact semantics, one lane per slab), N = N0..MAXN, Q =
// N..N+2: the plain kernels, and the even-odd ones up to N = MAXEO.
template <typename T, int OP, int N, int MAXEO, int MAXN = 8>
void add_affine(std::vector<CellVariant>& v, int dtype)
{
  if constexpr (N <= MAXN)
  {
    add_variant<T, N, N, OP, SEM_EXACT, 1>(v, dtype);
    add_variant<T, N, N + 1, OP, SEM_EXACT, 1>(v, dtype);
    add_variant<T, N, N + 2, OP, SEM_EXACT, 1>(v, dtype);
    if constexpr (N <= MAXEO)
    {
      add_variant<T, N, N, OP, SEM_EXACT, 1, true>(v, dtype);
      add_variant<T, N, N + 1, OP, SEM_EXACT, 1, true>(v, dtype);
      add_variant<T, N, N + 2, OP, SEM_EXACT, 1, true>(v, dtype);
    }
    add_affine<T, OP, N + 1, MAXEO, MAXN>(v, dtype);
  }
}

} // namespace femtc

#define FEMTC_CELL_UNIT(NAME, T, DTYPE, OP, L)                                 \
  namespace femtc                                                              \
  {                                                                            \
  void NAME(std::vector<CellVariant>& v, std::vector<FaultReader>& f)          \
  {                                                                            \
    add_all<T, OP, L>(v, DTYPE);                                               \
    f.push_back(&read_clear_fault_word);                                       \
  }                                                                            \
  }

#define FEMTC_CELL_UNIT_EXACT_UPTO(NAME, T, DTYPE, OP, L, MAXN)                 \
  namespace femtc                                                              \
  {                                                                            \
  void NAME(std::vector<CellVariant>& v, std::vector<FaultReader>& f)          \
  {                                                                            \
    add_exact_upto<T, OP, L, 2, MAXN>(v, DTYPE);                               \
    f.push_back(&read_clear_fault_word);                                       \
  }                                                                            \
  }

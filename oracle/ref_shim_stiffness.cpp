// Exposes the reference's own stiffness kernel template (IgorBaratta/femtc
// src/stiffness.hpp:34-99) through a C ABI so the oracle can be pinned
// against it.  Compiled from the reference sources where they lie (see
// oracle/Makefile); nothing of the reference is copied here.  Test
// infrastructure only.  Lives in its own shared object because
// src/linalg.hpp defines a non-inline function without an include guard.
#include <array>
#include <cstddef>
#include <iostream>
#include <span>

#include "stiffness.hpp"

namespace
{
template <typename T, int P>
void run(const T* tables, T* U, T* W, const T* G, std::size_t ncells)
{
  constexpr std::size_t n = P + 1, nd = n * n * n;
  // The kernel reads 2(P+1)^2 table values: Phi then its derivative
  // (src/stiffness.hpp:44-48).
  operators::stiffness_operator<T, P, linalg::Order::kij, 0, 0>(
      std::span<const T>(tables, 2 * n * n), std::span<T>(U, nd * ncells),
      std::span<T>(W, nd * ncells), std::span<const T>(G, 6 * nd * ncells),
      ncells);
}

template <typename T>
int dispatch(int P, const T* tables, T* U, T* W, const T* G,
             std::size_t ncells)
{
  switch (P)
  {
  case 1: run<T, 1>(tables, U, W, G, ncells); return 0;
  case 2: run<T, 2>(tables, U, W, G, ncells); return 0;
  case 3: run<T, 3>(tables, U, W, G, ncells); return 0;
  case 4: run<T, 4>(tables, U, W, G, ncells); return 0;
  case 5: run<T, 5>(tables, U, W, G, ncells); return 0;
  case 6: run<T, 6>(tables, U, W, G, ncells); return 0;
  case 7: run<T, 7>(tables, U, W, G, ncells); return 0;
  case 8: run<T, 8>(tables, U, W, G, ncells); return 0;
  default: return -1;
  }
}
} // namespace

extern "C" int ref_stiffness_f64(int P, const double* tables, double* U,
                                 double* W, const double* G,
                                 std::size_t ncells)
{
  return dispatch<double>(P, tables, U, W, G, ncells);
}

extern "C" int ref_stiffness_f32(int P, const float* tables, float* U,
                                 float* W, const float* G, std::size_t ncells)
{
  return dispatch<float>(P, tables, U, W, G, ncells);
}

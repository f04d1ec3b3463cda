// Exposes the reference's own mass kernel template (IgorBaratta/femtc
// src/mass.hpp:10-49) through a C ABI so the oracle can be pinned against it.
// Compiled from the reference sources where they lie (see oracle/Makefile);
// nothing of the reference is copied here.  Test infrastructure only.
#include <array>
#include <cstddef>
#include <iostream>
#include <span>

#include "mass.hpp"

namespace
{
template <typename T, int P>
void run(const T* phi, T* U, T* W, const T* detJ, std::size_t ncells)
{
  constexpr std::size_t n = P + 1, nd = n * n * n;
  operators::mass_operator<T, P, linalg::Order::kij, 0, 0>(
      std::span<const T>(phi, n * n), std::span<T>(U, nd * ncells),
      std::span<T>(W, nd * ncells), std::span<const T>(detJ, nd * ncells),
      ncells);
}

template <typename T>
int dispatch(int P, const T* phi, T* U, T* W, const T* detJ,
             std::size_t ncells)
{
  switch (P)
  {
  case 1: run<T, 1>(phi, U, W, detJ, ncells); return 0;
  case 2: run<T, 2>(phi, U, W, detJ, ncells); return 0;
  case 3: run<T, 3>(phi, U, W, detJ, ncells); return 0;
  case 4: run<T, 4>(phi, U, W, detJ, ncells); return 0;
  case 5: run<T, 5>(phi, U, W, detJ, ncells); return 0;
  case 6: run<T, 6>(phi, U, W, detJ, ncells); return 0;
  case 7: run<T, 7>(phi, U, W, detJ, ncells); return 0;
  case 8: run<T, 8>(phi, U, W, detJ, ncells); return 0;
  default: return -1;
  }
}
} // namespace

extern "C" int ref_mass_f64(int P, const double* phi, double* U, double* W,
                            const double* detJ, std::size_t ncells)
{
  return dispatch<double>(P, phi, U, W, detJ, ncells);
}

extern "C" int ref_mass_f32(int P, const float* phi, float* U, float* W,
                            const float* detJ, std::size_t ncells)
{
  return dispatch<float>(P, phi, U, W, detJ, ncells);
}

// linalg::gemm_blocked (src/linalg.hpp:101-182) at the two block settings the
// reference's own test uses (tests/test_gemm.cpp:41,52), for P = 1..8.
namespace
{
template <int P>
void gb(int blocked, const double* a, const double* b, double* c)
{
  constexpr int k = P + 1, m = P + 1, n = (P + 1) * (P + 1);
  if (blocked)
    linalg::gemm_blocked<double, k, m, n, linalg::Order::kij, 8, 16>(a, b, c);
  else
    linalg::gemm_blocked<double, k, m, n, linalg::Order::kij, 0, 0>(a, b, c);
}
} // namespace

extern "C" int ref_gemm_blocked_f64(int P, int blocked, const double* a,
                                    const double* b, double* c)
{
  switch (P)
  {
  case 1: gb<1>(blocked, a, b, c); return 0;
  case 2: gb<2>(blocked, a, b, c); return 0;
  case 3: gb<3>(blocked, a, b, c); return 0;
  case 4: gb<4>(blocked, a, b, c); return 0;
  case 5: gb<5>(blocked, a, b, c); return 0;
  case 6: gb<6>(blocked, a, b, c); return 0;
  case 7: gb<7>(blocked, a, b, c); return 0;
  case 8: gb<8>(blocked, a, b, c); return 0;
  default: return -1;
  }
}

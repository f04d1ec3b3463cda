// femtc_gpu/operators.hpp -- drop-in C++ front end of the GB300 operator
// library, keeping the reference's per-cell call signatures.
//
// A caller of IgorBaratta/femtc swaps
//     #include "mass.hpp"        (or "stiffness.hpp")
// for
//     #include "femtc_gpu/operators.hpp"
// links libfemtc_gpu.so, and its calls
//     operators::mass_operator<T, P, Order, Mb, Nb>(phi, U, W, detJ, num_cells)
//     operators::mass_operator<T>(phi, U, W, detJ, num_cells, degree, order, Mb, Nb)
// (src/mass.hpp:10-12, :196-199) and the stiffness twins
// (src/stiffness.hpp:34-36, :245-248) run on the GPU through the C ABI in
// femtc_gpu.h.  Host spans are copied to the device, the operator is
// applied, and W is written back before the call returns.
//
// Semantics.  By default the calls reproduce the reference's arithmetic
// exactly (Semantics::Reference, Q = P+1): mass applies Phi again where the
// transpose is meant (src/mass.hpp:21), stiffness keeps only its last
// backward chain (src/stiffness.hpp:85-97).  Semantics::Exact computes the
// true operators y = B^T D B u and y = sum_d D_d^T (G D u)_d, for any
// supported Q (extra template argument).
//
// Differences from the reference, on purpose:
//   * an unsupported degree, loop order or block size throws
//     std::runtime_error instead of printing and returning with W untouched
//     (src/mass.hpp:135,166,191,216);
//   * Order, Mb and Nb select CPU loop nests in the reference; on the GPU
//     they are validated (same accepted values) and otherwise ignored;
//   * stiffness reads 2(P+1)Q table values (Phi, then Gamma), which is what
//     the reference kernel reads too (src/stiffness.hpp:44-48).
#pragma once

#include <cstddef>
#include <span>
#include <stdexcept>
#include <string>
#include <type_traits>

#include "../femtc_gpu.h"

namespace linalg
{
// Loop-order tag of the reference (src/linalg.hpp:11-19).
enum class Order
{
  ijk,
  ikj,
  jik,
  jki,
  kij,
  kji
};

// Same strings and the same exception as src/linalg.hpp:21-37.
inline Order string2order(const std::string& s)
{
  if (s == "ikj")
    return Order::ikj;
  if (s == "ijk")
    return Order::ijk;
  if (s == "jik")
    return Order::jik;
  if (s == "jki")
    return Order::jki;
  if (s == "kij")
    return Order::kij;
  if (s == "kji")
    return Order::kji;
  throw std::runtime_error("Invalid loop order");
}
} // namespace linalg

namespace operators
{
enum class Semantics
{
  Exact,
  Reference
};

namespace detail
{
template <typename T>
constexpr int dtype()
{
  static_assert(std::is_same_v<T, double> || std::is_same_v<T, float>,
                "femtc_gpu operators are instantiated for float and double");
  return std::is_same_v<T, double> ? FEMTC_F64 : FEMTC_F32;
}

inline void check(int rc)
{
  if (rc != FEMTC_OK)
    throw std::runtime_error(std::string("femtc_gpu: ") + femtc_last_error());
}

inline void check_blocks(int Mb, int Nb)
{
  auto ok = [](int b) { return b == 0 || b == 4 || b == 8 || b == 16; };
  if (!ok(Mb) || !ok(Nb))
    throw std::runtime_error("Block size not supported");
}

inline int sem(Semantics s)
{
  return s == Semantics::Exact ? FEMTC_EXACT : FEMTC_REFERENCE;
}
} // namespace detail

// ---------------------------------------------------------------- mass --
// src/mass.hpp:10-12
template <typename T, int P, linalg::Order layout = linalg::Order::ijk,
          int Mb = 0, int Nb = 0, int Q = P + 1,
          Semantics S = Semantics::Reference>
void mass_operator(std::span<const T> phi, std::span<T> U, std::span<T> W,
                   std::span<const T> detJ, std::size_t num_cells)
{
  static_assert(P >= 1, "degree must be at least 1");
  detail::check_blocks(Mb, Nb);
  detail::check(femtc_mass_apply_host(detail::dtype<T>(), detail::sem(S), P,
                                      Q, phi.data(), U.data(), W.data(),
                                      detJ.data(), num_cells));
}

// Runtime dispatcher, src/mass.hpp:196-199 (degree, loop order, blocks).
template <typename T>
void mass_operator(std::span<T> phi, std::span<T> U, std::span<T> W,
                   std::span<T> detJ, std::size_t num_cells, int degree,
                   linalg::Order order, int Mb, int Nb,
                   Semantics s = Semantics::Reference, int nquad = 0)
{
  (void)order;
  detail::check_blocks(Mb, Nb);
  detail::check(femtc_mass_apply_host(
      detail::dtype<T>(), detail::sem(s), degree,
      nquad > 0 ? nquad : degree + 1, phi.data(), U.data(), W.data(),
      detJ.data(), num_cells));
}

// ----------------------------------------------------------- stiffness --
// src/stiffness.hpp:34-36
template <typename T, int P, linalg::Order order = linalg::Order::ijk,
          int Mb = 0, int Nb = 0, int Q = P + 1,
          Semantics S = Semantics::Reference>
void stiffness_operator(std::span<const T> phi, std::span<T> U,
                        std::span<T> W, std::span<const T> G,
                        std::size_t num_cells)
{
  static_assert(P >= 1, "degree must be at least 1");
  detail::check_blocks(Mb, Nb);
  detail::check(femtc_stiffness_apply_host(
      detail::dtype<T>(), detail::sem(S), P, Q, phi.data(), U.data(),
      W.data(), G.data(), num_cells));
}

// Runtime dispatcher, src/stiffness.hpp:245-248 (which takes int num_cells).
template <typename T>
void stiffness_operator(std::span<T> phi, std::span<T> U, std::span<T> W,
                        std::span<T> G, int num_cells, int degree,
                        linalg::Order order, int Mb, int Nb,
                        Semantics s = Semantics::Reference, int nquad = 0)
{
  (void)order;
  detail::check_blocks(Mb, Nb);
  if (num_cells < 0)
    throw std::runtime_error("Number of cells is negative");
  detail::check(femtc_stiffness_apply_host(
      detail::dtype<T>(), detail::sem(s), degree,
      nquad > 0 ? nquad : degree + 1, phi.data(), U.data(), W.data(),
      G.data(), (std::size_t)num_cells));
}

// ------------------------------------------------------- affine cells --
// No reference counterpart (the reference takes per-point detJ and G,
// src/mass.hpp:10-12, src/stiffness.hpp:34-36).  On affine cells the
// geometry is one set per cell: detJ (mass) or detJ J^-1 J^-T as
// [zz,yz,xz,yy,xy,xx] (stiffness).  tables: Phi (Q x N), Gamma (Q x N),
// then the Q 1D quadrature weights.  Host buffers, as the operators above.
template <typename T, int P, int Q = P + 2>
void affine_mass_operator(std::span<const T> tables, std::span<const T> U, std::span<T> W,
                          std::span<const T> detJ, std::size_t num_cells)
{
  static_assert(P >= 1, "degree must be at least 1");
  if (tables.size() < std::size_t(2 * Q * (P + 1) + Q) || detJ.size() < num_cells)
    throw std::runtime_error("femtc_gpu: affine tables hold Phi, Gamma and the weights; "
                             "one detJ per cell");
  detail::check(femtc_affine_apply_host(FEMTC_OP_MASS_AFFINE, detail::dtype<T>(), P, Q,
                                        tables.data(), U.data(), W.data(), detJ.data(),
                                        num_cells));
}

template <typename T, int P, int Q = P + 2>
void affine_stiffness_operator(std::span<const T> tables, std::span<const T> U,
                               std::span<T> W, std::span<const T> G, std::size_t num_cells)
{
  static_assert(P >= 1, "degree must be at least 1");
  if (tables.size() < std::size_t(2 * Q * (P + 1) + Q) || G.size() < 6 * num_cells)
    throw std::runtime_error("femtc_gpu: affine tables hold Phi, Gamma and the weights; "
                             "six G values per cell");
  detail::check(femtc_affine_apply_host(FEMTC_OP_STIFFNESS_AFFINE, detail::dtype<T>(), P, Q,
                                        tables.data(), U.data(), W.data(), G.data(),
                                        num_cells));
}
} // namespace operators

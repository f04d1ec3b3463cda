// Drop-in check: the call sequence of the reference's benchmark drivers
// (bench_mass.cpp:60-110, bench_stiffness.cpp:60-110), compiled against
// femtc_gpu/operators.hpp instead of the reference's mass.hpp /
// stiffness.hpp, with no other change to the calls.
//
// usage: drop_in_driver <mass|stiffness> <degree> <ncells> <float|double> <outdir>
// Writes phi.bin, U.bin, G.bin (or detJ.bin), W_dispatch.bin, W_template.bin
// (raw arrays of the element type) for the test to compare with the oracle.
// Ops affine_mass and affine_stiffness call the header's affine operators
// (Q = P+2, tabulated tables) and write tables.bin, U.bin, geo.bin and
// W_template.bin.
#include "femtc_gpu/operators.hpp"

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <random>
#include <string>
#include <vector>

template <typename T>
static void dump(const std::string& path, const std::vector<T>& v)
{
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char*>(v.data()), v.size() * sizeof(T));
}

template <typename T, int P>
static void run_template(bool mass, std::vector<T>& phi, std::vector<T>& U,
                         std::vector<T>& W, std::vector<T>& geo,
                         std::size_t num_cells)
{
  if (mass)
    operators::mass_operator<T, P, linalg::Order::kij, 0, 0>(phi, U, W, geo,
                                                             num_cells);
  else
    operators::stiffness_operator<T, P, linalg::Order::kij, 0, 0>(
        phi, U, W, geo, num_cells);
}

// The reference's runtime ladder covers degrees 1..25 (src/mass.hpp:57-137,
// src/stiffness.hpp:109-181): the templated signature at every one of them.
template <typename T, int P = 1>
static bool run_template_ladder(int degree, bool mass, std::vector<T>& phi, std::vector<T>& U,
                                std::vector<T>& W, std::vector<T>& geo, std::size_t num_cells)
{
  if constexpr (P <= 25)
  {
    if (degree == P)
    {
      run_template<T, P>(mass, phi, U, W, geo, num_cells);
      return true;
    }
    return run_template_ladder<T, P + 1>(degree, mass, phi, U, W, geo, num_cells);
  }
  else
    return false;
}

template <typename T>
static int run(bool mass, int degree, int num_cells, const std::string& out)
{
  const int p = degree, ndofs = (p + 1) * (p + 1) * (p + 1);
  std::mt19937_64 rng(12345 + degree);
  std::uniform_real_distribution<double> U01(0.0, 1.0);
  auto rnd = [&]() { return static_cast<T>(U01(rng)); };
  // the reference allocates (p+1)^2 table values for mass; stiffness reads
  // Phi and Gamma, 2(p+1)^2 values (src/stiffness.hpp:44-48)
  std::vector<T> phi((mass ? 1 : 2) * (p + 1) * (p + 1));
  for (auto& x : phi)
    x = rnd();
  std::vector<T> U(num_cells * ndofs), W(num_cells * ndofs, 0.0);
  for (auto& x : U)
    x = rnd();
  std::vector<T> geo(num_cells * ndofs * (mass ? 1 : 6));
  for (auto& x : geo)
    x = rnd();

  linalg::Order order = linalg::string2order("kij");
  if (mass)
    operators::mass_operator<T>(phi, U, W, geo, num_cells, degree, order, 0, 0);
  else
    operators::stiffness_operator<T>(phi, U, W, geo, num_cells, degree, order,
                                     0, 0);
  dump(out + "/W_dispatch.bin", W);

  std::vector<T> W2(num_cells * ndofs, 0.0);
  if (!run_template_ladder<T>(degree, mass, phi, U, W2, geo, num_cells))
  {
    std::cerr << "degree not in 1..25\n";
    return 2;
  }
  dump(out + "/W_template.bin", W2);
  dump(out + "/phi.bin", phi);
  dump(out + "/U.bin", U);
  dump(out + "/geo.bin", geo);

  // error behaviour: a bad loop order string throws like the reference
  // (src/linalg.hpp:36); unsupported blocks and degrees throw here where
  // the reference prints and returns
  int thrown = 0;
  try { linalg::string2order("xyz"); } catch (const std::runtime_error&) { ++thrown; }
  try {
    operators::mass_operator<T>(phi, U, W, geo, num_cells, degree, order, 3, 0);
  } catch (const std::runtime_error&) { ++thrown; }
  try {
    operators::mass_operator<T>(phi, U, W, geo, num_cells, 40, order, 0, 0);
  } catch (const std::runtime_error&) { ++thrown; }
  std::printf("thrown %d\n", thrown);
  return thrown == 3 ? 0 : 3;
}

template <typename T, int P>
static void run_affine_template(bool mass, const std::vector<T>& tab, const std::vector<T>& U,
                                std::vector<T>& W, const std::vector<T>& geo,
                                std::size_t num_cells)
{
  if (mass)
    operators::affine_mass_operator<T, P>(tab, U, W, geo, num_cells);
  else
    operators::affine_stiffness_operator<T, P>(tab, U, W, geo, num_cells);
}

template <typename T>
static int run_affine(bool mass, int degree, int num_cells, const std::string& out)
{
  const int n = degree + 1, q = degree + 2, ndofs = n * n * n;
  std::vector<double> t64(2 * q * n), pts(q), wts(q), nodes(n);
  if (femtc_tabulate(degree, q, t64.data(), pts.data(), wts.data(), nodes.data()) != FEMTC_OK)
    return 4;
  std::vector<T> tab(t64.begin(), t64.end());
  tab.insert(tab.end(), wts.begin(), wts.end());
  std::mt19937_64 rng(777 + degree);
  std::uniform_real_distribution<double> U01(0.5, 1.5);
  std::vector<T> U(num_cells * ndofs), W(num_cells * ndofs, 0.0);
  for (auto& x : U)
    x = static_cast<T>(U01(rng) - 1.0);
  std::vector<T> geo(num_cells * (mass ? 1 : 6));
  for (std::size_t c = 0; c < (std::size_t)num_cells; ++c)
  {
    if (mass)
      geo[c] = static_cast<T>(U01(rng));
    else
    {
      // a symmetric positive definite G: dominant diagonal zz, yy, xx
      T* g = &geo[6 * c];
      g[0] = static_cast<T>(U01(rng) + 1.0);
      g[3] = static_cast<T>(U01(rng) + 1.0);
      g[5] = static_cast<T>(U01(rng) + 1.0);
      g[1] = static_cast<T>(0.2 * (U01(rng) - 1.0));
      g[2] = static_cast<T>(0.2 * (U01(rng) - 1.0));
      g[4] = static_cast<T>(0.2 * (U01(rng) - 1.0));
    }
  }
  switch (degree)
  {
  case 1: run_affine_template<T, 1>(mass, tab, U, W, geo, num_cells); break;
  case 2: run_affine_template<T, 2>(mass, tab, U, W, geo, num_cells); break;
  case 3: run_affine_template<T, 3>(mass, tab, U, W, geo, num_cells); break;
  case 4: run_affine_template<T, 4>(mass, tab, U, W, geo, num_cells); break;
  case 5: run_affine_template<T, 5>(mass, tab, U, W, geo, num_cells); break;
  case 6: run_affine_template<T, 6>(mass, tab, U, W, geo, num_cells); break;
  case 7: run_affine_template<T, 7>(mass, tab, U, W, geo, num_cells); break;
  default: std::cerr << "degree not in 1..7\n"; return 2;
  }
  dump(out + "/W_template.bin", W);
  dump(out + "/tables.bin", tab);
  dump(out + "/U.bin", U);
  dump(out + "/geo.bin", geo);
  // a table span without the weights throws (degree 1 needs 2*3*2 + 3)
  int thrown = 0;
  try
  {
    const std::vector<T> short_tab(14, T(0));
    run_affine_template<T, 1>(mass, short_tab, U, W, geo, 0);
  }
  catch (const std::runtime_error&)
  {
    ++thrown;
  }
  return thrown == 1 ? 0 : 3;
}

int main(int argc, char** argv)
{
  if (argc < 6)
  {
    std::cerr << "usage: " << argv[0]
              << " <mass|stiffness> <degree> <ncells> <float|double> <outdir>\n";
    return 1;
  }
  const std::string op = argv[1];
  const int degree = std::atoi(argv[2]), ncells = std::atoi(argv[3]);
  if (op == "affine_mass" || op == "affine_stiffness")
  {
    const bool am = op == "affine_mass";
    if (std::string(argv[4]) == "float")
      return run_affine<float>(am, degree, ncells, argv[5]);
    return run_affine<double>(am, degree, ncells, argv[5]);
  }
  const bool mass = op == "mass";
  if (std::string(argv[4]) == "float")
    return run<float>(mass, degree, ncells, argv[5]);
  return run<double>(mass, degree, ncells, argv[5]);
}

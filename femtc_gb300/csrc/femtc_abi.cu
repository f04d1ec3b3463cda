// C ABI of the femtc GB300 operator library (declared in include/femtc_gpu.h):
// argument checking, variant lookup, tile configuration, launch, the
// host-buffer drop-in path and the host-side basis tabulation.
#include "femtc_gpu.h"

#include "cell_kernel.cuh"
#include "registry.hpp"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

namespace femtc
{
namespace
{

thread_local std::string t_last_error;

int fail(int code, const char* fmt, ...)
{
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  t_last_error = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what)
{
  return fail(FEMTC_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

struct Registry
{
  std::vector<CellVariant> cells;
  std::vector<FaultReader> faults;
};

Registry& registry()
{
  static Registry r;
  static std::once_flag once;
  std::call_once(once, [] {
    register_cell_f64_mass(r.cells, r.faults);
    register_cell_f64_stiffness(r.cells, r.faults);
    register_cell_f32_mass(r.cells, r.faults);
    register_cell_f32_stiffness(r.cells, r.faults);
    register_mma_f16x2_mass(r.cells, r.faults);
    register_mma_f16x2_stiffness(r.cells, r.faults);
    register_mma_bf16x3_mass(r.cells, r.faults);
    register_mma_bf16x3_stiffness(r.cells, r.faults);
  });
  return r;
}

const CellVariant* find_cell(int op, int dtype, int sem, int n, int q)
{
  for (const CellVariant& v : registry().cells)
    if (v.op == op && v.dtype == dtype && v.sem == sem && v.n == n &&
        v.q == q)
      return &v;
  return nullptr;
}

// ---------------------------------------------------------------- tiles --
using Key = std::tuple<int, int, int, int, int>; // op dtype sem n q
std::mutex g_cfg_mutex;
std::map<Key, std::pair<int, int>> g_tile_cfg; // -> (cb, staged)

constexpr unsigned kSmemPerSmTarget = 113 * 1024; // 2 CTAs per SM

// Lane efficiency of a tile of `cb` cells: useful pencil slots over issued
// slots across the five passes, each weighted by its FMAs per pencil.
double lane_efficiency(int n, int q, int cb)
{
  const double np[5] = {double(n * n), double(n * q), double(q * q),
                        double(n * q), double(n * n)};
  const double wk[5] = {double(n * q), double(n * q), double(2 * n * q),
                        double(n * q), double(n * q)};
  double useful = 0, issued = 0;
  for (int i = 0; i < 5; ++i)
  {
    const double p = np[i] * cb;
    const double slots = std::ceil(p / kCellThreads) * kCellThreads;
    useful += p * wk[i];
    issued += slots * wk[i];
  }
  return useful / issued;
}

std::pair<int, int> default_tile(const CellVariant& v)
{
  int best_cb = 4, best_staged = 0;
  double best = -1.0;
  for (int staged = 1; staged >= 0; --staged)
  {
    for (int cb = 4; cb <= 64; cb += 4)
    {
      if (v.smem(cb, staged) > kSmemPerSmTarget)
        break;
      // prefer filled lanes, then larger tiles (fewer tile boundaries)
      const double s = lane_efficiency(v.n, v.q, cb) + 1e-4 * cb;
      if (s > best)
      {
        best = s;
        best_cb = cb;
        best_staged = staged;
      }
    }
    if (best > 0)
      break; // staging fits: keep it
  }
  return {best_cb, best_staged};
}

std::pair<int, int> tile_config(const CellVariant& v)
{
  std::lock_guard<std::mutex> lk(g_cfg_mutex);
  auto it = g_tile_cfg.find(Key(v.op, v.dtype, v.sem, v.n, v.q));
  if (it != g_tile_cfg.end())
    return it->second;
  return default_tile(v);
}

// -------------------------------------------------------- launch helpers --
struct FnState
{
  int max_smem_set = 0;
  std::map<unsigned, int> blocks_per_sm; // by dynamic smem
};
std::mutex g_fn_mutex;
std::map<const void*, FnState> g_fn_state;

int sm_count()
{
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 1;
}

int prepare(const void* fn, unsigned smem, int* blocks)
{
  std::lock_guard<std::mutex> lk(g_fn_mutex);
  FnState& st = g_fn_state[fn];
  if ((int)smem > st.max_smem_set)
  {
    cudaError_t e = cudaFuncSetAttribute(
        fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
      return cuda_fail(e, "cudaFuncSetAttribute");
    st.max_smem_set = (int)smem;
  }
  auto it = st.blocks_per_sm.find(smem);
  if (it == st.blocks_per_sm.end())
  {
    int nb = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &nb, fn, kCellThreads, smem);
    if (e != cudaSuccess)
      return cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    if (nb < 1)
      return fail(FEMTC_ERR_UNSUPPORTED,
                  "kernel does not fit on an SM with %u B shared memory",
                  smem);
    it = st.blocks_per_sm.emplace(smem, nb).first;
  }
  *blocks = it->second;
  return FEMTC_OK;
}

bool aligned16(const void* p)
{
  return (reinterpret_cast<uintptr_t>(p) & 15u) == 0;
}

int check_common(int op, int dtype, int sem, int degree, int nquad,
                 const void* tables, const void* u, const void* y,
                 const void* geo, const CellVariant** out)
{
  if (dtype != FEMTC_F64 && dtype != FEMTC_F32 && dtype != FEMTC_F16X2 &&
      dtype != FEMTC_BF16X3)
    return fail(FEMTC_ERR_INVALID, "unknown dtype %d", dtype);
  if (sem != FEMTC_EXACT && sem != FEMTC_REFERENCE)
    return fail(FEMTC_ERR_INVALID, "unknown semantics %d", sem);
  if (degree < 1)
    return fail(FEMTC_ERR_INVALID, "degree must be at least 1 (got %d)",
                degree);
  if (nquad < 1)
    return fail(FEMTC_ERR_INVALID, "nquad must be at least 1 (got %d)",
                nquad);
  if (sem == FEMTC_REFERENCE && nquad != degree + 1)
    return fail(FEMTC_ERR_INVALID,
                "reference semantics needs nquad == degree+1 (got %d, %d)",
                degree, nquad);
  if (!tables || !u || !y || !geo)
    return fail(FEMTC_ERR_INVALID, "null pointer argument");
  const CellVariant* v = find_cell(op, dtype, sem, degree + 1, nquad);
  if (!v)
    return fail(FEMTC_ERR_UNSUPPORTED,
                "no %s kernel for dtype %d, semantics %d, degree %d, nquad %d",
                op == FEMTC_OP_MASS ? "mass" : "stiffness", dtype, sem, degree,
                nquad);
  *out = v;
  return FEMTC_OK;
}

template <typename T>
int launch_cell(const CellVariant& v, const T* tables, const void* u,
                void* y, const void* geo, size_t ncells, cudaStream_t stream)
{
  if (!aligned16(u) || !aligned16(y) || !aligned16(geo))
    return fail(FEMTC_ERR_INVALID,
                "u, y and the geometry must be 16-byte aligned device "
                "pointers (TMA bulk copies)");
  const auto cfg = tile_config(v);
  CellParams<T> p;
  std::memset(&p, 0, sizeof(p));
  p.u = static_cast<const T*>(u);
  p.y = static_cast<T*>(y);
  p.geo = static_cast<const T*>(geo);
  p.ncells = (long long)ncells;
  p.cb = cfg.first;
  p.geo_staged = cfg.second;
  const int ntab = (v.op == FEMTC_OP_STIFFNESS) ? 2 : 1;
  for (int t = 0; t < ntab; ++t)
    for (int i = 0; i < v.n * v.q; ++i)
      p.tab[t][i] = tables[t * v.n * v.q + i];
  const unsigned smem = v.smem(p.cb, p.geo_staged);
  int blocks = 0;
  int rc = prepare(v.fn, smem, &blocks);
  if (rc != FEMTC_OK)
    return rc;
  const long long ntiles = ((long long)ncells + p.cb - 1) / p.cb;
  const long long grid =
      std::min<long long>(ntiles, (long long)blocks * sm_count());
  void* args[] = {&p};
  cudaError_t e = cudaLaunchKernel(v.fn, dim3((unsigned)grid),
                                   dim3(kCellThreads), args, smem, stream);
  if (e != cudaSuccess)
    return cuda_fail(e, "cudaLaunchKernel");
  return FEMTC_OK;
}

int apply(int op, int dtype, int sem, int degree, int nquad,
          const void* tables, const void* u, void* y, const void* geo,
          size_t ncells, void* stream)
{
  const CellVariant* v = nullptr;
  int rc = check_common(op, dtype, sem, degree, nquad, tables, u, y, geo, &v);
  if (rc != FEMTC_OK)
    return rc;
  if (ncells == 0)
    return FEMTC_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == FEMTC_F64)
    return launch_cell<double>(*v, static_cast<const double*>(tables), u, y,
                               geo, ncells, st);
  return launch_cell<float>(*v, static_cast<const float*>(tables), u, y, geo,
                            ncells, st);
}

size_t elem_size(int dtype) { return dtype == FEMTC_F64 ? 8 : 4; }

// ------------------------------------------------------- host-buffer path --
struct HostPath
{
  std::mutex m;
  int device = -1;
  cudaStream_t stream = nullptr;
  void* buf[3] = {nullptr, nullptr, nullptr};
  size_t cap[3] = {0, 0, 0};
};
HostPath g_host;

int host_buffer(int i, size_t bytes)
{
  if (g_host.cap[i] >= bytes)
    return FEMTC_OK;
  if (g_host.buf[i])
    cudaFree(g_host.buf[i]);
  g_host.buf[i] = nullptr;
  g_host.cap[i] = 0;
  cudaError_t e = cudaMalloc(&g_host.buf[i], bytes);
  if (e != cudaSuccess)
    return fail(FEMTC_ERR_NOMEM, "cudaMalloc(%zu): %s", bytes,
                cudaGetErrorString(e));
  g_host.cap[i] = bytes;
  return FEMTC_OK;
}

int apply_host(int op, int dtype, int sem, int degree, int nquad,
               const void* tables, const void* u, void* y, const void* geo,
               size_t ncells)
{
  const CellVariant* v = nullptr;
  int rc = check_common(op, dtype, sem, degree, nquad, tables, u, y, geo, &v);
  if (rc != FEMTC_OK)
    return rc;
  if (ncells == 0)
    return FEMTC_OK;
  std::lock_guard<std::mutex> lk(g_host.m);
  int dev = 0;
  cudaGetDevice(&dev);
  if (g_host.device != dev)
  {
    // a different device: drop buffers of the old one (they stay valid on
    // it until freed; free them with that device current)
    g_host.stream = nullptr;
    for (int i = 0; i < 3; ++i)
    {
      g_host.buf[i] = nullptr;
      g_host.cap[i] = 0;
    }
    g_host.device = dev;
  }
  if (!g_host.stream)
  {
    cudaError_t e =
        cudaStreamCreateWithFlags(&g_host.stream, cudaStreamNonBlocking);
    if (e != cudaSuccess)
      return cuda_fail(e, "cudaStreamCreate");
  }
  const size_t es = elem_size(dtype);
  const size_t n3 = (size_t)v->n * v->n * v->n;
  const size_t q3 = (size_t)v->q * v->q * v->q * (op == FEMTC_OP_MASS ? 1 : 6);
  const size_t bu = ncells * n3 * es, bg = ncells * q3 * es;
  if ((rc = host_buffer(0, bu)) != FEMTC_OK ||
      (rc = host_buffer(1, bu)) != FEMTC_OK ||
      (rc = host_buffer(2, bg)) != FEMTC_OK)
    return rc;
  cudaStream_t st = g_host.stream;
  cudaError_t e = cudaMemcpyAsync(g_host.buf[0], u, bu,
                                  cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(g_host.buf[2], geo, bg, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess)
    return cuda_fail(e, "cudaMemcpyAsync (host to device)");
  rc = apply(op, dtype, sem, degree, nquad, tables, g_host.buf[0],
             g_host.buf[1], g_host.buf[2], ncells, st);
  if (rc != FEMTC_OK)
  {
    cudaStreamSynchronize(st);
    return rc;
  }
  e = cudaMemcpyAsync(y, g_host.buf[1], bu, cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess)
    return cuda_fail(e, "cudaMemcpyAsync (device to host)");
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess)
    return cuda_fail(e, "cudaStreamSynchronize");
  return FEMTC_OK;
}

// ------------------------------------------------------------ tabulation --
// Legendre polynomial L_n and its derivative at x in [-1,1] (three-term
// recurrence, Bonnet's formula).
void legendre(int n, double x, double* p, double* dp)
{
  double p0 = 1.0, p1 = x;
  if (n == 0)
  {
    *p = 1.0;
    *dp = 0.0;
    return;
  }
  for (int k = 2; k <= n; ++k)
  {
    const double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
    p0 = p1;
    p1 = p2;
  }
  *p = p1;
  // (1-x^2) L_n' = n (L_{n-1} - x L_n)
  *dp = n * (p0 - x * p1) / (1.0 - x * x);
}

// Gauss-Legendre points/weights on [0,1] by Newton's method on L_q.
void gauss_legendre(int q, double* x, double* w)
{
  for (int k = 0; k < q; ++k)
  {
    double t = std::cos(M_PI * (k + 0.75) / (q + 0.5));
    for (int it = 0; it < 100; ++it)
    {
      double p, dp;
      legendre(q, t, &p, &dp);
      const double dt = p / dp;
      t -= dt;
      if (std::fabs(dt) < 1e-16)
        break;
    }
    double p, dp;
    legendre(q, t, &p, &dp);
    // points descend in t; store ascending on [0,1]
    x[q - 1 - k] = 0.5 * (1.0 + t);
    w[q - 1 - k] = 1.0 / ((1.0 - t * t) * dp * dp); // (2/((1-t^2)L'^2))/2
  }
}

// Gauss-Lobatto-Legendre nodes on [0,1]: endpoints and the roots of L_p'.
void gll_nodes(int p, double* x)
{
  x[0] = 0.0;
  x[p] = 1.0;
  for (int k = 1; k < p; ++k)
  {
    double t = -std::cos(M_PI * k / p);
    for (int it = 0; it < 100; ++it)
    {
      double l, dl;
      legendre(p, t, &l, &dl);
      // (1-t^2) L'' = 2 t L' - p(p+1) L
      const double d2 = (2.0 * t * dl - p * (p + 1.0) * l) / (1.0 - t * t);
      const double dt = dl / d2;
      t -= dt;
      if (std::fabs(dt) < 1e-16)
        break;
    }
    x[k] = 0.5 * (1.0 + t);
  }
}

} // namespace
} // namespace femtc

using namespace femtc;

extern "C" {

int femtc_version(void) { return 100; }

const char* femtc_last_error(void) { return t_last_error.c_str(); }

int femtc_device_status(void)
{
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess)
    return cuda_fail(e, "cudaDeviceSynchronize");
  unsigned w = 0;
  for (FaultReader f : registry().faults)
    w |= f();
  return (int)(w & 0x7fffffffu);
}

int femtc_supported(int op, int dtype, int semantics, int degree, int nquad)
{
  return find_cell(op, dtype, semantics, degree + 1, nquad) ? 1 : 0;
}

int femtc_mass_apply(int dtype, int semantics, int degree, int nquad,
                     const void* tables, const void* u, void* y,
                     const void* dw, size_t ncells, void* stream)
{
  return apply(FEMTC_OP_MASS, dtype, semantics, degree, nquad, tables, u, y,
               dw, ncells, stream);
}

int femtc_stiffness_apply(int dtype, int semantics, int degree, int nquad,
                          const void* tables, const void* u, void* y,
                          const void* G, size_t ncells, void* stream)
{
  return apply(FEMTC_OP_STIFFNESS, dtype, semantics, degree, nquad, tables, u,
               y, G, ncells, stream);
}

int femtc_mass_apply_host(int dtype, int semantics, int degree, int nquad,
                          const void* tables, const void* u, void* y,
                          const void* dw, size_t ncells)
{
  return apply_host(FEMTC_OP_MASS, dtype, semantics, degree, nquad, tables, u,
                    y, dw, ncells);
}

int femtc_stiffness_apply_host(int dtype, int semantics, int degree,
                               int nquad, const void* tables, const void* u,
                               void* y, const void* G, size_t ncells)
{
  return apply_host(FEMTC_OP_STIFFNESS, dtype, semantics, degree, nquad,
                    tables, u, y, G, ncells);
}

int femtc_set_tile_config(int op, int dtype, int semantics, int degree,
                          int nquad, int cb, int geo_staged)
{
  const CellVariant* v = find_cell(op, dtype, semantics, degree + 1, nquad);
  if (!v)
    return fail(FEMTC_ERR_UNSUPPORTED, "no such kernel variant");
  std::lock_guard<std::mutex> lk(g_cfg_mutex);
  const Key k(op, dtype, semantics, degree + 1, nquad);
  if (cb <= 0)
  {
    g_tile_cfg.erase(k);
    return FEMTC_OK;
  }
  if (cb % 4 != 0 || cb > 256)
    return fail(FEMTC_ERR_INVALID, "cb must be a multiple of 4 in [4,256]");
  if (v->smem(cb, geo_staged ? 1 : 0) > 227u * 1024u)
    return fail(FEMTC_ERR_INVALID, "tile needs %u B of shared memory",
                v->smem(cb, geo_staged ? 1 : 0));
  g_tile_cfg[k] = {cb, geo_staged ? 1 : 0};
  return FEMTC_OK;
}

int femtc_get_tile_config(int op, int dtype, int semantics, int degree,
                          int nquad, int* cb, int* geo_staged)
{
  const CellVariant* v = find_cell(op, dtype, semantics, degree + 1, nquad);
  if (!v)
    return fail(FEMTC_ERR_UNSUPPORTED, "no such kernel variant");
  const auto c = tile_config(*v);
  if (cb)
    *cb = c.first;
  if (geo_staged)
    *geo_staged = c.second;
  return FEMTC_OK;
}

int femtc_tabulate(int degree, int nquad, double* tables, double* points,
                   double* weights, double* nodes)
{
  if (degree < 1 || degree > 32 || nquad < 1 || nquad > 64)
    return fail(FEMTC_ERR_INVALID, "degree in [1,32], nquad in [1,64]");
  if (!tables)
    return fail(FEMTC_ERR_INVALID, "tables is null");
  const int n = degree + 1, q = nquad;
  std::vector<double> x(q), w(q), z(n);
  gauss_legendre(q, x.data(), w.data());
  gll_nodes(degree, z.data());
  for (int i = 0; i < n; ++i)
  {
    for (int k = 0; k < q; ++k)
    {
      const double t = x[k];
      double l = 1.0;
      for (int j = 0; j < n; ++j)
        if (j != i)
          l *= (t - z[j]) / (z[i] - z[j]);
      // l_i'(t) = sum_m 1/(z_i - z_m) prod_{j != i,m} (t - z_j)/(z_i - z_j)
      double dl = 0.0;
      for (int m = 0; m < n; ++m)
      {
        if (m == i)
          continue;
        double prod = 1.0 / (z[i] - z[m]);
        for (int j = 0; j < n; ++j)
          if (j != i && j != m)
            prod *= (t - z[j]) / (z[i] - z[j]);
        dl += prod;
      }
      tables[k + i * q] = l;
      tables[q * n + k + i * q] = dl;
    }
  }
  if (points)
    std::copy(x.begin(), x.end(), points);
  if (weights)
    std::copy(w.begin(), w.end(), weights);
  if (nodes)
    std::copy(z.begin(), z.end(), nodes);
  return FEMTC_OK;
}

} // extern "C"

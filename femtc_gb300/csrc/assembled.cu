// Assembled (global-DOF) operator action: y = sum_c P_c^T A_c P_c x, where
// P_c gathers cell c's N^3 local DOFs from the global vector through a DOF
// map (dofmap[c][i] = global index of local DOF i).  No reference
// counterpart: the reference applies the cell-local operator only
// (src/mass.hpp:10-49, src/stiffness.hpp:34-99); this is the format step
// around it that a finite-element code's global vectors need.
//
// Three stream-ordered steps on caller-provided scratch:
//   1. gather    u[c][i] = x[dofmap[c][i]]            (coalesced map reads)
//   2. operator  y_loc = A u (the library's cell kernels, any dtype)
//   3. sum       y[g] = sum of y_loc over the (cell, i) that map to g, in
//                the fixed order of the transposed map (CSR: offsets,
//                entries) -- no atomics, so the result's bits do not depend
//                on scheduling.
// femtc_dofmap_transpose builds the transposed map on the host.
#include "femtc_gpu.h"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>
#include <vector>

namespace femtc
{
int aux_fail(int code, const char* msg); // femtc_abi.cu

namespace
{
constexpr int kThreads = 256;

// Indices outside their arrays (a map that does not match the vectors) are
// not dereferenced: they yield NaN, which the result then shows.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    gather_kernel(const T* __restrict__ x, long long ndofs, const int32_t* __restrict__ dofmap,
                  T* __restrict__ u, long long n)
{
  for (long long i = blockIdx.x * (long long)kThreads + threadIdx.x; i < n;
       i += (long long)gridDim.x * kThreads)
  {
    const int32_t g = dofmap[i];
    u[i] = (g >= 0 && g < ndofs) ? x[g] : T(NAN);
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
    sum_kernel(const T* __restrict__ yloc, long long nloc, const int32_t* __restrict__ offsets,
               const int32_t* __restrict__ entries, T* __restrict__ y, long long ndofs)
{
  for (long long g = blockIdx.x * (long long)kThreads + threadIdx.x; g < ndofs;
       g += (long long)gridDim.x * kThreads)
  {
    T s = T(0);
    const int k0 = offsets[g], k1 = offsets[g + 1];
    if (k0 < 0 || k1 < k0 || k1 > nloc)
      s = T(NAN);
    else
      for (int k = k0; k < k1; ++k)
      {
        const int32_t e = entries[k];
        s += (e >= 0 && e < nloc) ? yloc[e] : T(NAN);
      }
    y[g] = s;
  }
}

int grid_for(long long work)
{
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long g = (work + kThreads - 1) / kThreads;
  const long long cap = (long long)(sms > 0 ? sms : 1) * 16;
  return (int)(g < 1 ? 1 : (g < cap ? g : cap));
}

size_t elem_bytes(int dtype)
{
  return (dtype == FEMTC_F64 || dtype == FEMTC_F64E) ? 8 : 4;
}

size_t round256(size_t b) { return (b + 255) & ~size_t(255); }

template <typename T>
int run(int op, int dtype, int semantics, int degree, int nquad, const void* tables,
        const int32_t* dofmap, const int32_t* offsets, const int32_t* entries, size_t ndofs,
        const T* x, T* y, const void* geo, size_t ncells, void* work, cudaStream_t st)
{
  const long long n3 = (long long)(degree + 1) * (degree + 1) * (degree + 1);
  const long long nloc = (long long)ncells * n3;
  T* u = static_cast<T*>(work);
  T* yl = reinterpret_cast<T*>(static_cast<char*>(work) + round256((size_t)nloc * sizeof(T)));
  gather_kernel<T><<<grid_for(nloc), kThreads, 0, st>>>(x, (long long)ndofs, dofmap, u, nloc);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return aux_fail(FEMTC_ERR_CUDA, cudaGetErrorString(e));
  const int rc = op == FEMTC_OP_MASS
                     ? femtc_mass_apply(dtype, semantics, degree, nquad, tables, u, yl, geo,
                                        ncells, st)
                     : femtc_stiffness_apply(dtype, semantics, degree, nquad, tables, u, yl,
                                             geo, ncells, st);
  if (rc != FEMTC_OK)
    return rc;
  sum_kernel<T><<<grid_for((long long)ndofs), kThreads, 0, st>>>(yl, nloc, offsets, entries, y,
                                                                 (long long)ndofs);
  e = cudaGetLastError();
  return e == cudaSuccess ? FEMTC_OK : aux_fail(FEMTC_ERR_CUDA, cudaGetErrorString(e));
}
} // namespace
} // namespace femtc

using namespace femtc;

extern "C" {

int femtc_dofmap_transpose(const int32_t* dofmap, size_t ncells, int n3, size_t ndofs,
                           int32_t* offsets, int32_t* entries)
{
  if (!dofmap || !offsets || !entries || n3 < 1)
    return aux_fail(FEMTC_ERR_INVALID, "dofmap_transpose: null pointer or n3 < 1");
  const size_t nloc = ncells * (size_t)n3;
  if (nloc >= (size_t)INT32_MAX || ndofs >= (size_t)INT32_MAX)
    return aux_fail(FEMTC_ERR_INVALID, "dofmap_transpose: more than 2^31 entries");
  std::memset(offsets, 0, (ndofs + 1) * sizeof(int32_t));
  for (size_t k = 0; k < nloc; ++k)
  {
    const int32_t g = dofmap[k];
    if (g < 0 || (size_t)g >= ndofs)
      return aux_fail(FEMTC_ERR_INVALID, "dofmap_transpose: global index out of range");
    ++offsets[g + 1];
  }
  for (size_t g = 0; g < ndofs; ++g)
    offsets[g + 1] += offsets[g];
  std::vector<int32_t> pos(offsets, offsets + ndofs);
  for (size_t k = 0; k < nloc; ++k) // increasing (cell, local index): the sum order
    entries[pos[dofmap[k]]++] = (int32_t)k;
  return FEMTC_OK;
}

size_t femtc_assembled_work_bytes(int dtype, int degree, size_t ncells)
{
  const size_t n = (size_t)degree + 1;
  return 2 * round256(ncells * n * n * n * elem_bytes(dtype));
}

int femtc_assembled_apply(int op, int dtype, int semantics, int degree, int nquad,
                          const void* tables, const int32_t* dofmap, const int32_t* offsets,
                          const int32_t* entries, size_t ndofs, const void* x, void* y,
                          const void* geo, size_t ncells, void* work, void* stream)
{
  if (op != FEMTC_OP_MASS && op != FEMTC_OP_STIFFNESS)
    return aux_fail(FEMTC_ERR_INVALID, "assembled apply: op is FEMTC_OP_MASS or FEMTC_OP_STIFFNESS");
  if (dtype != FEMTC_F64 && dtype != FEMTC_F32 && dtype != FEMTC_F16X2 &&
      dtype != FEMTC_BF16X3 && dtype != FEMTC_F64E)
    return aux_fail(FEMTC_ERR_INVALID, "assembled apply: unknown dtype");
  if (!tables || !dofmap || !offsets || !entries || !x || !y || !geo || !work)
    return aux_fail(FEMTC_ERR_INVALID, "assembled apply: null pointer argument");
  if ((reinterpret_cast<uintptr_t>(work) & 255u) != 0)
    return aux_fail(FEMTC_ERR_INVALID, "assembled apply: work must be 256-byte aligned");
  if (degree < 1)
    return aux_fail(FEMTC_ERR_INVALID, "assembled apply: degree must be at least 1");
  if (!femtc_supported(op, dtype, semantics, degree, nquad))
    return aux_fail(FEMTC_ERR_UNSUPPORTED, "assembled apply: no such cell operator variant");
  const size_t n = (size_t)degree + 1;
  if (ncells * n * n * n >= (size_t)INT32_MAX || ndofs >= (size_t)INT32_MAX)
    return aux_fail(FEMTC_ERR_INVALID,
                    "assembled apply: more than 2^31 local or global DOFs (int32 maps)");
  if (ndofs == 0)
    return FEMTC_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (ncells == 0)
  {
    // no cells: every global DOF's sum is empty
    cudaError_t e = cudaMemsetAsync(y, 0, ndofs * elem_bytes(dtype), st);
    return e == cudaSuccess ? FEMTC_OK : aux_fail(FEMTC_ERR_CUDA, cudaGetErrorString(e));
  }
  if (elem_bytes(dtype) == 8)
    return run<double>(op, dtype, semantics, degree, nquad, tables, dofmap, offsets, entries,
                       ndofs, static_cast<const double*>(x), static_cast<double*>(y), geo,
                       ncells, work, st);
  return run<float>(op, dtype, semantics, degree, nquad, tables, dofmap, offsets, entries, ndofs,
                    static_cast<const float*>(x), static_cast<float*>(y), geo, ncells, work, st);
}

} // extern "C"

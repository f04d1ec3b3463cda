// General-degree cell kernels: the mass and stiffness action for any degree
// P = 1..25 (N = P+1 <= 26 DOFs per axis) and Q <= 28 quadrature points per
// axis, FP64 and FP32 (exact and reference semantics) and the FP64-accurate
// double-float form F64E (exact semantics), with runtime sizes.
//
// The reference dispatches degrees 1..25 (src/mass.hpp:57-137,
// src/stiffness.hpp:109-181).  The slab kernels (cell_kernel.cuh) hold a
// cell's slabs in registers with compile-time sizes and are built for
// N <= 8; every other (N, Q) of mass and stiffness runs here.
//
// One CTA applies the operator to one cell at a time (grid-stride over
// cells).  Each axis contraction is the reference's rotating product
// (src/linalg.hpp:101-182 as chained in src/mass.hpp:36-47): the input is
// K x L with the contracted axis slowest, the output L x M with the new
// axis fastest, so three contractions return a tensor to its axis order.
// All threads of the CTA share the L*M outputs of a contraction; a CTA
// barrier separates dependent contractions.  Stiffness shares partial
// contractions between the gradient components (forward 2 + 3 + 3,
// backward 3 + 2 + 1 with two-input contractions), the same tree as the
// oracle's restatement of src/stiffness.hpp:34-99.
//
// Each thread computes two outputs of a contraction that share their input
// column (one load of each input value feeds two accumulations: more
// independent work per thread, half the input loads).  The double-float
// form converts each cell's u from FP64 once into a work buffer (the
// contractions then read double-float pairs) and its outputs back to FP64;
// its multiply-adds run on the FP32 pipes, each sum renormalised once
// (df64.cuh).
//
// Work buffers (max(N,Q)^3 values each; 3 for mass, 6 for stiffness) live
// in shared memory when they fit next to the tables, else in a per-CTA
// slice of a stream-ordered device workspace (cudaMallocAsync /
// cudaFreeAsync on the caller's stream, so calls on different streams never
// share one).  These degrees are bound by the arithmetic pipes (FP64:
// about 4.5 flops per byte of HBM traffic at N = 9, rising with N); the
// work buffers' traffic stays in L1/L2.
#include "femtc_gpu.h"

#include "df64.cuh"
#include "registry.hpp"

#include <type_traits>

#include <algorithm>
#include <cstring>

namespace femtc
{
int aux_fail(int code, const char* msg); // femtc_abi.cu

namespace
{
constexpr int kGenMaxN = 26; // degree 25
constexpr int kGenMaxQ = 28;
constexpr int kGenThreads = 256;

// Storage type of an arithmetic type: double-float keeps FP64 storage.
template <typename T>
struct gen_storage
{
  using type = T;
};
template <>
struct gen_storage<df64>
{
  using type = double;
};

template <typename T, typename S>
__device__ __forceinline__ T load_as(S v)
{
  if constexpr (std::is_same<T, df64>::value && !std::is_same<S, df64>::value)
    return to_df64(v);
  else
    return v;
}

template <typename S, typename T>
__device__ __forceinline__ S store_as(T v)
{
  if constexpr (std::is_same<T, df64>::value && !std::is_same<S, df64>::value)
    return to_double(v);
  else
    return v;
}

template <typename T>
struct GenParams
{
  using ST = typename gen_storage<T>::type;
  const ST* u;     // [ncells][N^3]
  ST* y;           // [ncells][N^3]
  const ST* geo;   // mass [ncells][Q^3]; stiffness [ncells][Q^3][6]
  T* work;         // device workspace (null: the buffers are in shared memory)
  long long ncells;
  long long work_cta; // workspace elements per CTA
  int n, q, op, sem;
  int buf;         // elements per work buffer
  int tab_elems;   // shared-memory elements of the tables (padded)
  // Phi(q,i) = tab[q + i*Q], then Gamma (stiffness)
  T tab[2 * kGenMaxQ * kGenMaxN];
};

// out[j*M + m] = sum_p A(m,p) in[p*L + j], A(m,p) = A[m*sm + p*sk], over all
// threads of the CTA (no barrier inside); with a second table/input pair
// (B, in2) the sum also runs over B(m,p) in2[p*L + j].  A work item is an
// output column j and two rows m, m+1 that share the input loads.
template <typename T, typename O>
__device__ __forceinline__ void rot2(int K, int L, int M, const T* __restrict__ A,
                                     const T* __restrict__ B, int sm, int sk,
                                     const T* __restrict__ in1, const T* __restrict__ in2,
                                     O* __restrict__ out)
{
  const int mp = (M + 1) >> 1; // row pairs
  const int total = L * mp;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x)
  {
    const int j = idx / mp, m = 2 * (idx - j * mp);
    const bool two = m + 1 < M;
    const T* a = A + m * sm;
    const T* a1 = A + (two ? m + 1 : m) * sm;
    const T* x = in1 + j;
    // accumulators (double-float: renormalised once per sum, df64acc)
    acc_t<T> acc0 = acc_mul(a[0], x[0]), acc1 = acc_mul(a1[0], x[0]);
    for (int p = 1; p < K; ++p)
    {
      const T v = x[(long long)p * L];
      acc0 = acc_fma(a[p * sk], v, acc0);
      acc1 = acc_fma(a1[p * sk], v, acc1);
    }
    if (B)
    {
      const T* b = B + m * sm;
      const T* b1 = B + (two ? m + 1 : m) * sm;
      const T* z = in2 + j;
      for (int p = 0; p < K; ++p)
      {
        const T v = z[(long long)p * L];
        acc0 = acc_fma(b[p * sk], v, acc0);
        acc1 = acc_fma(b1[p * sk], v, acc1);
      }
    }
    out[j * M + m] = store_as<O>(acc_val(acc0));
    if (two)
      out[j * M + m + 1] = store_as<O>(acc_val(acc1));
  }
}

template <typename T, typename O>
__device__ __forceinline__ void rot(int K, int L, int M, const T* __restrict__ A, int sm, int sk,
                                    const T* __restrict__ in, O* __restrict__ out)
{
  rot2<T, O>(K, L, M, A, (const T*)nullptr, sm, sk, in, (const T*)nullptr, out);
}

template <typename T>
__global__ void __launch_bounds__(kGenThreads)
    general_cell_kernel(const __grid_constant__ GenParams<T> p)
{
  using ST = typename gen_storage<T>::type;
  constexpr bool kConvert = !std::is_same<T, ST>::value; // double-float: FP64 storage
  extern __shared__ __align__(16) unsigned char smem[];
  const int n = p.n, q = p.q, nq = n * q;
  const int n3 = n * n * n, q3 = q * q * q;
  const bool stiff = p.op == FEMTC_OP_STIFFNESS;
  T* tP = reinterpret_cast<T*>(smem);
  T* tD = tP + nq;
  for (int i = threadIdx.x; i < (stiff ? 2 : 1) * nq; i += blockDim.x)
    tP[i] = p.tab[i];
  T* base = p.work ? p.work + blockIdx.x * p.work_cta : tP + p.tab_elems;
  T* w0 = base;
  T* w1 = base + p.buf;
  T* w2 = base + 2 * p.buf;
  T* w3 = base + 3 * p.buf;
  T* w4 = base + 4 * p.buf;
  T* w5 = base + 5 * p.buf;
  // backward tables: exact A(i,q) = t[q + i*Q] (the transpose); reference
  // A(i,q) = t[i + q*Q] (the forward table reused, Q == N)
  const bool exact = p.sem == FEMTC_EXACT;
  const int bsm = exact ? q : 1, bsk = exact ? 1 : q;
  __syncthreads();
  for (long long c = blockIdx.x; c < p.ncells; c += gridDim.x)
  {
    const ST* ug = p.u + c * n3;
    ST* yc = p.y + c * n3;
    // the forward contractions' input: u itself, or (double-float) u
    // converted once into a work buffer that is free until it is read
    const T* uc;
    if constexpr (kConvert)
    {
      T* ub = stiff ? w5 : w2;
      for (int i = threadIdx.x; i < n3; i += blockDim.x)
        ub[i] = load_as<T>(ug[i]);
      __syncthreads();
      uc = ub;
    }
    else
      uc = ug;
    if (!stiff)
    {
      // src/mass.hpp:36-47
      rot(n, n * n, q, tP, 1, q, uc, w0);
      __syncthreads();
      rot(n, n * q, q, tP, 1, q, w0, w1);
      __syncthreads();
      rot(n, q * q, q, tP, 1, q, w1, w2);
      __syncthreads();
      const ST* dw = p.geo + c * q3;
      for (int i = threadIdx.x; i < q3; i += blockDim.x)
        w2[i] *= load_as<T>(dw[i]);
      __syncthreads();
      rot(q, q * q, n, tP, bsm, bsk, w2, w0);
      __syncthreads();
      rot(q, q * n, n, tP, bsm, bsk, w0, w1);
      __syncthreads();
      rot(q, n * n, n, tP, bsm, bsk, w1, yc);
      __syncthreads();
      continue;
    }
    // stiffness, src/stiffness.hpp:34-99: forward Phi_0 u and Gamma_0 u
    // shared by the three gradients
    rot(n, n * n, q, tP, 1, q, uc, w0); // Phi_0 u
    rot(n, n * n, q, tD, 1, q, uc, w1); // Gamma_0 u
    __syncthreads();
    rot(n, n * q, q, tP, 1, q, w1, w2); // x: Phi_1
    rot(n, n * q, q, tD, 1, q, w0, w3); // y: Gamma_1
    rot(n, n * q, q, tP, 1, q, w0, w4); // z: Phi_1
    __syncthreads();
    rot(n, q * q, q, tP, 1, q, w2, w0); // d/dx
    rot(n, q * q, q, tP, 1, q, w3, w1); // d/dy
    // d/dz: Gamma_2 (exact); the reference's W_z carries no derivative
    // (src/stiffness.hpp:76-77)
    rot(n, q * q, q, exact ? tD : tP, 1, q, w4, w5);
    __syncthreads();
    // G transform per point, [zz,yz,xz,yy,xy,xx] (src/stiffness.hpp:14-29)
    const ST* G = p.geo + c * q3 * 6;
    for (int i = threadIdx.x; i < q3; i += blockDim.x)
    {
      const ST* gs = G + 6 * i;
      const T g0 = load_as<T>(gs[0]), g1 = load_as<T>(gs[1]), g2 = load_as<T>(gs[2]);
      const T a0 = w0[i], a1 = w1[i], a2 = w5[i];
      if (exact)
      {
        const T g3 = load_as<T>(gs[3]), g4 = load_as<T>(gs[4]), g5 = load_as<T>(gs[5]);
        w0[i] = g5 * a0 + g4 * a1 + g2 * a2;
        w1[i] = g4 * a0 + g3 * a1 + g1 * a2;
      }
      w5[i] = g2 * a0 + g1 * a1 + g0 * a2;
    }
    __syncthreads();
    if (exact)
    {
      // backward: x, y and z chains; y and x meet before their common
      // axis-2 table Phi_2^T, z keeps Gamma_2^T
      rot(q, q * q, n, tD, bsm, bsk, w0, w2); // x: Gamma_0^T
      rot(q, q * q, n, tP, bsm, bsk, w1, w3); // y: Phi_0^T
      rot(q, q * q, n, tP, bsm, bsk, w5, w4); // z: Phi_0^T
      __syncthreads();
      rot2(q, q * n, n, tP, tD, bsm, bsk, w2, w3, w0); // x: Phi_1^T, y: Gamma_1^T
      rot(q, q * n, n, tP, bsm, bsk, w4, w1);          // z: Phi_1^T
      __syncthreads();
      rot2(q, n * n, n, tP, tD, bsm, bsk, w0, w1, yc); // Phi_2^T (x + y) + Gamma_2^T z
    }
    else
    {
      // only the last backward chain (Phi, Phi, Gamma) survives in the
      // reference (src/stiffness.hpp:85,91,97)
      rot(q, q * q, n, tP, bsm, bsk, w5, w2);
      __syncthreads();
      rot(q, q * n, n, tP, bsm, bsk, w2, w3);
      __syncthreads();
      rot(q, n * n, n, tD, bsm, bsk, w3, yc);
    }
    __syncthreads();
  }
}

int max_smem_optin()
{
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return v;
}

int sms()
{
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
  return v > 0 ? v : 1;
}

template <typename T>
int launch(int op, int sem, int n, int q, const typename gen_storage<T>::type* tables,
           const void* u, void* y, const void* geo, size_t ncells, cudaStream_t st)
{
  using ST = typename gen_storage<T>::type;
  GenParams<T> p;
  std::memset(&p, 0, sizeof(p));
  p.u = static_cast<const ST*>(u);
  p.y = static_cast<ST*>(y);
  p.geo = static_cast<const ST*>(geo);
  p.ncells = (long long)ncells;
  p.n = n;
  p.q = q;
  p.op = op;
  p.sem = sem;
  const bool stiff = op == FEMTC_OP_STIFFNESS;
  // mass reads Phi only (the reference's mass table holds (P+1)^2 values)
  const int ntab = stiff ? 2 : 1;
  for (int i = 0; i < ntab * n * q; ++i)
  {
    if constexpr (std::is_same<T, df64>::value)
      p.tab[i] = host_df64(tables[i]);
    else
      p.tab[i] = tables[i];
  }
  const int big = std::max(n, q);
  const int align = 16 / (int)sizeof(T);
  p.buf = (big * big * big + align - 1) / align * align;
  p.tab_elems = (2 * n * q + align - 1) / align * align;
  const int nbuf = stiff ? 6 : 3;
  const size_t tab_bytes = sizeof(T) * p.tab_elems;
  const size_t buf_bytes = sizeof(T) * (size_t)p.buf * nbuf;
  const void* fn = reinterpret_cast<const void*>(&general_cell_kernel<T>);
  const bool in_smem = tab_bytes + buf_bytes <= (size_t)max_smem_optin();
  const size_t smem = in_smem ? tab_bytes + buf_bytes : tab_bytes;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess)
    return aux_fail(FEMTC_ERR_CUDA, cudaGetErrorString(e));
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kGenThreads, smem);
  if (e != cudaSuccess || per_sm < 1)
    return aux_fail(FEMTC_ERR_UNSUPPORTED, "general cell kernel does not fit on an SM");
  // workspace mode: two CTAs per SM bound the workspace (they are FP64- or
  // FP32-pipe bound, not latency bound)
  if (!in_smem)
    per_sm = std::min(per_sm, 2);
  const long long grid = std::min<long long>((long long)ncells, (long long)per_sm * sms());
  void* work = nullptr;
  if (!in_smem)
  {
    p.work_cta = (long long)p.buf * nbuf;
    e = cudaMallocAsync(&work, sizeof(T) * (size_t)p.work_cta * grid, st);
    if (e != cudaSuccess)
      return aux_fail(FEMTC_ERR_NOMEM, cudaGetErrorString(e));
    p.work = static_cast<T*>(work);
  }
  void* args[] = {&p};
  e = cudaLaunchKernel(fn, dim3((unsigned)grid), dim3(kGenThreads), args, smem, st);
  if (work)
  {
    const cudaError_t f = cudaFreeAsync(work, st);
    if (e == cudaSuccess)
      e = f;
  }
  if (e != cudaSuccess)
    return aux_fail(FEMTC_ERR_CUDA, cudaGetErrorString(e));
  return FEMTC_OK;
}
} // namespace

bool general_supported(int op, int dtype, int sem, int n, int q)
{
  if (op != FEMTC_OP_MASS && op != FEMTC_OP_STIFFNESS)
    return false;
  if (dtype != FEMTC_F64 && dtype != FEMTC_F32 && dtype != FEMTC_F64E)
    return false;
  if (n < 2 || n > kGenMaxN || q < 1 || q > kGenMaxQ)
    return false;
  if (dtype == FEMTC_F64E)
    return sem == FEMTC_EXACT; // the double-float form: exact semantics
  return sem == FEMTC_EXACT || (sem == FEMTC_REFERENCE && q == n);
}

int launch_general(int op, int dtype, int sem, int n, int q, const void* tables, const void* u,
                   void* y, const void* geo, size_t ncells, cudaStream_t st)
{
  if (!general_supported(op, dtype, sem, n, q))
    return aux_fail(FEMTC_ERR_UNSUPPORTED, "general cell kernel: unsupported variant");
  if (ncells == 0)
    return FEMTC_OK;
  if (dtype == FEMTC_F64)
    return launch<double>(op, sem, n, q, static_cast<const double*>(tables), u, y, geo, ncells,
                          st);
  if (dtype == FEMTC_F64E)
    return launch<df64>(op, sem, n, q, static_cast<const double*>(tables), u, y, geo, ncells,
                        st);
  return launch<float>(op, sem, n, q, static_cast<const float*>(tables), u, y, geo, ncells, st);
}
} // namespace femtc

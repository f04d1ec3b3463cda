// Stand-alone contraction entry points and the FP64 geometry kernel.
//
//  femtc_gemm_micro          linalg::gemm_micro (src/linalg.hpp:45-94),
//                            batched: C_b += A_b B_b with A column-major
//                            (lda), B and C row-major (ldb, ldc).
//  femtc_gemm_blocked        linalg::gemm_blocked (src/linalg.hpp:101-182),
//                            batched over cells: C_c = A B_c with A column-
//                            major m x k, B_c row-major k x n, C_c column-
//                            major m x n (assigned, not accumulated).
//  femtc_apply_contractions  apply_contractions (src/tmm.hpp:91-126) batched
//                            over cells: A = (I0 x I1 x I2) B, tables
//                            row-major Na x Nb (tr != 0) or their stored
//                            transposes Nb x Na (tr == 0).
//  femtc_geometry            per-point quadrature factors from Jacobians, in
//                            FP64: detJ*w (mass) and G = detJ w J^-1 J^-T as
//                            [zz,yz,xz,yy,xy,xx] (stiffness), stored as FP64
//                            or cast to FP32.
// These run at setup or in tests, not on the operator's hot loop, so they use
// runtime sizes and plain shared-memory staging.
#include "femtc_gpu.h"

#include "common.cuh"

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>

namespace femtc
{
int aux_fail(int code, const char* msg); // defined in femtc_abi.cu

namespace
{
constexpr int kMaxContract = 32; // sizes k, m <= 32 (the reference tests 26)

template <typename T>
struct GemmParams
{
  const T* b;
  T* c;
  long long batch;
  int k, m, n;
  T a[kMaxContract * kMaxContract]; // column-major m x k
};

// One CTA per cell; thread t -> output (i, j) with i fastest (coalesced C).
template <typename T>
__global__ void __launch_bounds__(256)
    gemm_blocked_kernel(const __grid_constant__ GemmParams<T> p)
{
  const int mn = p.m * p.n;
  for (long long cell = blockIdx.x; cell < p.batch; cell += gridDim.x)
  {
    const T* b = p.b + cell * (long long)p.k * p.n;
    T* c = p.c + cell * (long long)mn;
    for (int t = threadIdx.x; t < mn; t += blockDim.x)
    {
      const int j = t / p.m, i = t - j * p.m;
      T acc = T(0);
      for (int q = 0; q < p.k; ++q)
        acc = fma(p.a[i + q * p.m], b[q * p.n + j], acc);
      c[i + j * p.m] = acc;
    }
  }
}

// One thread per output element (item, i, j), j fastest (coalesced rows of
// C and B): c(i,j) += sum_p a[i + p*lda] b[p*ldb + j], the products added
// into c in increasing p (gemm_micro's kij order, src/linalg.hpp:73-79).
template <typename T>
__global__ void __launch_bounds__(256)
    gemm_micro_kernel(const T* __restrict__ a, const T* __restrict__ b, T* __restrict__ c, int k,
                      int m, int nc, int lda, int ldb, int ldc, long long batch, long long sa,
                      long long sb, long long sc)
{
  const long long per = (long long)m * nc;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < batch * per;
       t += (long long)gridDim.x * blockDim.x)
  {
    const long long item = t / per;
    const int r = (int)(t - item * per);
    const int i = r / nc, j = r - i * nc;
    const T* ai = a + item * sa + i;
    const T* bj = b + item * sb + j;
    T* cij = c + item * sc + (long long)i * ldc + j;
    T acc = *cij;
    for (int p = 0; p < k; ++p)
      acc = fma(ai[(long long)p * lda], bj[(long long)p * ldb], acc);
    *cij = acc;
  }
}

template <typename T>
struct ContractParams
{
  const T* b;
  T* a;
  long long ncells;
  int na, nb, tr;
  T t[3][16 * 16]; // I0, I1, I2 as given
};

template <typename T>
__device__ __forceinline__ T table(const ContractParams<T>& p, int w, int a,
                                   int b)
{
  // src/tmm.hpp:65-85: Tr reads I[a*Nb + b], otherwise I[b*Na + a]
  return p.tr ? p.t[w][a * p.nb + b] : p.t[w][b * p.na + a];
}

// One CTA per cell, three contractions through shared memory.
template <typename T>
__global__ void __launch_bounds__(256)
    apply_contractions_kernel(const __grid_constant__ ContractParams<T> p)
{
  extern __shared__ __align__(16) unsigned char sm[];
  const int na = p.na, nb = p.nb;
  T* sb = reinterpret_cast<T*>(sm);       // nb^3
  T* s1 = sb + nb * nb * nb;              // na*nb*nb
  T* s2 = s1 + na * nb * nb;              // na*na*nb
  for (long long cell = blockIdx.x; cell < p.ncells; cell += gridDim.x)
  {
    const T* b = p.b + cell * (long long)nb * nb * nb;
    for (int i = threadIdx.x; i < nb * nb * nb; i += blockDim.x)
      sb[i] = b[i];
    __syncthreads();
    // [a0, b1, b2] = sum_b0 I0(a0,b0) B[b0, b1, b2]
    for (int i = threadIdx.x; i < na * nb * nb; i += blockDim.x)
    {
      const int a0 = i / (nb * nb), r = i - a0 * nb * nb;
      T acc = T(0);
      for (int k = 0; k < nb; ++k)
        acc = fma(table(p, 0, a0, k), sb[k * nb * nb + r], acc);
      s1[i] = acc;
    }
    __syncthreads();
    // [a0, a1, b2] = sum_b1 I1(a1,b1) s1[a0, b1, b2]
    for (int i = threadIdx.x; i < na * na * nb; i += blockDim.x)
    {
      const int a0 = i / (na * nb), r = i - a0 * na * nb;
      const int a1 = r / nb, b2 = r - a1 * nb;
      T acc = T(0);
      for (int k = 0; k < nb; ++k)
        acc = fma(table(p, 1, a1, k), s1[(a0 * nb + k) * nb + b2], acc);
      s2[i] = acc;
    }
    __syncthreads();
    // [a0, a1, a2] = sum_b2 I2(a2,b2) s2[a0, a1, b2]
    T* a = p.a + cell * (long long)na * na * na;
    for (int i = threadIdx.x; i < na * na * na; i += blockDim.x)
    {
      const int r = i / na, a2 = i - r * na;
      T acc = T(0);
      for (int k = 0; k < nb; ++k)
        acc = fma(table(p, 2, a2, k), s2[r * nb + k], acc);
      a[i] = acc;
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------- geometry --
struct GeoParams
{
  const double* J;   // [ncells][9] (affine) or [ncells][Q^3][9], row-major
  void* dw;          // [ncells][Q^3] or null
  void* G;           // [ncells][Q^3][6] or null
  long long ncells;
  int q3;
  int per_point;
  int out_f32;
  double w[1024];    // tensor quadrature weights w_q0 w_q1 w_q2 (Q <= 10)
};

// One thread per (cell, point): 3x3 inverse by cofactors in FP64,
// K = J^-1 J^-T, factors detJ*w and detJ*w*K.
__global__ void __launch_bounds__(256)
    geometry_kernel(const __grid_constant__ GeoParams p)
{
  const long long total = p.ncells * p.q3;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
       i < total; i += (long long)gridDim.x * blockDim.x)
  {
    const long long cell = i / p.q3;
    const int q = (int)(i - cell * p.q3);
    const double* j = p.J + (p.per_point ? i : cell) * 9;
    const double a = j[0], b = j[1], c = j[2], d = j[3], e = j[4], f = j[5],
                 g = j[6], h = j[7], k = j[8];
    const double c00 = e * k - f * h, c01 = c * h - b * k, c02 = b * f - c * e;
    const double c10 = f * g - d * k, c11 = a * k - c * g, c12 = c * d - a * f;
    const double c20 = d * h - e * g, c21 = b * g - a * h, c22 = a * e - b * d;
    const double det = a * c00 + b * c10 + c * c20;
    const double s = p.w[q] * det;
    if (p.dw)
    {
      if (p.out_f32)
        static_cast<float*>(p.dw)[i] = (float)s;
      else
        static_cast<double*>(p.dw)[i] = s;
    }
    if (p.G)
    {
      // J^-1 = adj(J)/det with adj(J)[r][c] = c_rc above; K = J^-1 J^-T,
      // so det*w*K = (w/det) adj adj^T
      const double r = p.w[q] / det;
      const double kxx = r * (c00 * c00 + c01 * c01 + c02 * c02);
      const double kxy = r * (c00 * c10 + c01 * c11 + c02 * c12);
      const double kxz = r * (c00 * c20 + c01 * c21 + c02 * c22);
      const double kyy = r * (c10 * c10 + c11 * c11 + c12 * c12);
      const double kyz = r * (c10 * c20 + c11 * c21 + c12 * c22);
      const double kzz = r * (c20 * c20 + c21 * c21 + c22 * c22);
      const double v[6] = {kzz, kyz, kxz, kyy, kxy, kxx};
      if (p.out_f32)
      {
        float* o = static_cast<float*>(p.G) + i * 6;
        for (int t = 0; t < 6; ++t)
          o[t] = (float)v[t];
      }
      else
      {
        double* o = static_cast<double*>(p.G) + i * 6;
        for (int t = 0; t < 6; ++t)
          o[t] = v[t];
      }
    }
  }
}

int grid_for(long long work, int threads)
{
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long long g = (work + threads - 1) / threads;
  const long long cap = (long long)(sms > 0 ? sms : 1) * 8;
  return (int)(g < cap ? (g < 1 ? 1 : g) : cap);
}

int launch_error(cudaError_t e)
{
  if (e == cudaSuccess)
    return FEMTC_OK;
  return aux_fail(FEMTC_ERR_CUDA, cudaGetErrorString(e));
}

template <typename T>
int gemm_blocked_t(int k, int m, int n, const void* a, const void* b, void* c,
                   size_t batch, cudaStream_t st)
{
  GemmParams<T> p;
  std::memset(&p, 0, sizeof(p));
  p.b = static_cast<const T*>(b);
  p.c = static_cast<T*>(c);
  p.batch = (long long)batch;
  p.k = k;
  p.m = m;
  p.n = n;
  std::memcpy(p.a, a, sizeof(T) * m * k);
  gemm_blocked_kernel<T><<<grid_for((long long)batch * 256, 256), 256, 0, st>>>(p);
  return launch_error(cudaGetLastError());
}

template <typename T>
int contractions_t(int na, int nb, int tr, const void* i0, const void* i1,
                   const void* i2, const void* b, void* a, size_t ncells,
                   cudaStream_t st)
{
  ContractParams<T> p;
  std::memset(&p, 0, sizeof(p));
  p.b = static_cast<const T*>(b);
  p.a = static_cast<T*>(a);
  p.ncells = (long long)ncells;
  p.na = na;
  p.nb = nb;
  p.tr = tr ? 1 : 0;
  const void* src[3] = {i0, i1, i2};
  for (int w = 0; w < 3; ++w)
    std::memcpy(p.t[w], src[w], sizeof(T) * na * nb);
  const size_t smem =
      sizeof(T) * ((size_t)nb * nb * nb + (size_t)na * nb * nb + (size_t)na * na * nb);
  if (smem > 48 * 1024)
  {
    cudaError_t e = cudaFuncSetAttribute(apply_contractions_kernel<T>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess)
      return launch_error(e);
  }
  apply_contractions_kernel<T>
      <<<grid_for((long long)ncells * 256, 256), 256, smem, st>>>(p);
  return launch_error(cudaGetLastError());
}
} // namespace
} // namespace femtc

using namespace femtc;

// geo8[p] = (beta G[p][0..5], alpha dw[p], 0) per quadrature point p: the
// interleaved geometry of the Helmholtz operator (two 16-byte stores).
__global__ void __launch_bounds__(256)
    helmholtz_geometry_kernel(const float* __restrict__ dw, const float* __restrict__ G,
                              float alpha, float beta, float4* __restrict__ geo8,
                              long long npts)
{
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npts;
       p += (long long)gridDim.x * blockDim.x)
  {
    const float* g = G + p * 6;
    geo8[2 * p] = make_float4(beta * g[0], beta * g[1], beta * g[2], beta * g[3]);
    geo8[2 * p + 1] = make_float4(beta * g[4], beta * g[5], alpha * dw[p], 0.0f);
  }
}

extern "C" {

int femtc_gemm_micro(int dtype, int k, int m, int nc, int lda, int ldb, int ldc, const void* a,
                     const void* b, void* c, size_t batch, size_t stride_a, size_t stride_b,
                     size_t stride_c, void* stream)
{
  if (dtype != FEMTC_F64 && dtype != FEMTC_F32)
    return aux_fail(FEMTC_ERR_INVALID, "gemm_micro: dtype must be F64 or F32");
  if (k < 1 || m < 1 || nc < 1 || lda < m || ldb < nc || ldc < nc)
    return aux_fail(FEMTC_ERR_INVALID,
                    "gemm_micro: need k, m, nc >= 1, lda >= m, ldb >= nc, ldc >= nc");
  if (!a || !b || !c)
    return aux_fail(FEMTC_ERR_INVALID, "gemm_micro: null pointer");
  if (batch > 1 && stride_c < (size_t)(m - 1) * ldc + nc)
    return aux_fail(FEMTC_ERR_INVALID,
                    "gemm_micro: items' C blocks overlap (stride_c below one block)");
  if (batch == 0)
    return FEMTC_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const long long work = (long long)batch * m * nc;
  if (dtype == FEMTC_F64)
    gemm_micro_kernel<double><<<grid_for(work, 256), 256, 0, st>>>(
        static_cast<const double*>(a), static_cast<const double*>(b), static_cast<double*>(c), k,
        m, nc, lda, ldb, ldc, (long long)batch, (long long)stride_a, (long long)stride_b,
        (long long)stride_c);
  else
    gemm_micro_kernel<float><<<grid_for(work, 256), 256, 0, st>>>(
        static_cast<const float*>(a), static_cast<const float*>(b), static_cast<float*>(c), k, m,
        nc, lda, ldb, ldc, (long long)batch, (long long)stride_a, (long long)stride_b,
        (long long)stride_c);
  return launch_error(cudaGetLastError());
}

int femtc_gemm_blocked(int dtype, int k, int m, int n, const void* a,
                       const void* b, void* c, size_t batch, void* stream)
{
  if (dtype != FEMTC_F64 && dtype != FEMTC_F32)
    return aux_fail(FEMTC_ERR_INVALID, "gemm_blocked: dtype must be F64 or F32");
  if (k < 1 || m < 1 || n < 1 || k > kMaxContract || m > kMaxContract)
    return aux_fail(FEMTC_ERR_INVALID, "gemm_blocked: need 1 <= k, m <= 32 and n >= 1");
  if (!a || !b || !c)
    return aux_fail(FEMTC_ERR_INVALID, "gemm_blocked: null pointer");
  if (batch == 0)
    return FEMTC_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  return dtype == FEMTC_F64 ? gemm_blocked_t<double>(k, m, n, a, b, c, batch, st)
                            : gemm_blocked_t<float>(k, m, n, a, b, c, batch, st);
}

int femtc_apply_contractions(int dtype, int na, int nb, int tr,
                             const void* i0, const void* i1, const void* i2,
                             const void* b, void* a, size_t ncells,
                             void* stream)
{
  if (dtype != FEMTC_F64 && dtype != FEMTC_F32)
    return aux_fail(FEMTC_ERR_INVALID, "apply_contractions: dtype must be F64 or F32");
  if (na < 1 || nb < 1 || na > 16 || nb > 16)
    return aux_fail(FEMTC_ERR_INVALID, "apply_contractions: need 1 <= Na, Nb <= 16");
  if (!i0 || !i1 || !i2 || !a || !b)
    return aux_fail(FEMTC_ERR_INVALID, "apply_contractions: null pointer");
  if (ncells == 0)
    return FEMTC_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  return dtype == FEMTC_F64
             ? contractions_t<double>(na, nb, tr, i0, i1, i2, b, a, ncells, st)
             : contractions_t<float>(na, nb, tr, i0, i1, i2, b, a, ncells, st);
}

int femtc_geometry(int out_dtype, int nquad, const double* weights,
                   const double* J, int per_point, void* dw, void* G,
                   size_t ncells, void* stream)
{
  if (out_dtype != FEMTC_F64 && out_dtype != FEMTC_F32)
    return aux_fail(FEMTC_ERR_INVALID, "geometry: out_dtype must be F64 or F32");
  if (nquad < 1 || nquad > 10)
    return aux_fail(FEMTC_ERR_INVALID, "geometry: nquad in [1,10]");
  if (!weights || !J || (!dw && !G))
    return aux_fail(FEMTC_ERR_INVALID, "geometry: null pointer");
  if (ncells == 0)
    return FEMTC_OK;
  GeoParams p;
  std::memset(&p, 0, sizeof(p));
  p.J = J;
  p.dw = dw;
  p.G = G;
  p.ncells = (long long)ncells;
  p.q3 = nquad * nquad * nquad;
  p.per_point = per_point ? 1 : 0;
  p.out_f32 = out_dtype == FEMTC_F32;
  for (int a = 0; a < nquad; ++a)
    for (int b = 0; b < nquad; ++b)
      for (int c = 0; c < nquad; ++c)
        p.w[(a * nquad + b) * nquad + c] = weights[a] * weights[b] * weights[c];
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  geometry_kernel<<<grid_for(p.ncells * p.q3, 256), 256, 0, st>>>(p);
  return launch_error(cudaGetLastError());
}

int femtc_helmholtz_geometry(int nquad, double alpha, const void* dw, double beta,
                             const void* G, void* geo8, size_t ncells, void* stream)
{
  if (nquad < 1 || nquad > 10)
    return aux_fail(FEMTC_ERR_INVALID, "helmholtz_geometry: nquad in [1,10]");
  if (!dw || !G || !geo8)
    return aux_fail(FEMTC_ERR_INVALID, "helmholtz_geometry: null pointer");
  if ((reinterpret_cast<uintptr_t>(geo8) & 15u) != 0)
    return aux_fail(FEMTC_ERR_INVALID, "helmholtz_geometry: geo8 must be 16-byte aligned");
  if (ncells == 0)
    return FEMTC_OK;
  const long long npts = (long long)ncells * nquad * nquad * nquad;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  helmholtz_geometry_kernel<<<grid_for(npts, 256), 256, 0, st>>>(
      static_cast<const float*>(dw), static_cast<const float*>(G), (float)alpha, (float)beta,
      static_cast<float4*>(geo8), npts);
  return launch_error(cudaGetLastError());
}

} // extern "C"

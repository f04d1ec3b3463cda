// Matrix-free solve of (alpha M + beta K) x = b on cell-local hexahedral
// meshes: Jacobi-preconditioned CG with the mixed-precision operator, inside
// FP64 iterative refinement (femtc_solve in femtc_gpu.h).  The reference has
// no solver; this is the caller of its operators that the benchmark
// configuration for serving needs.
//
//   outer (FP64):  r = b - A x with the FP64 operators, ||r|| in FP64;
//                  stop at ||r|| <= rtol ||b||;
//   inner (mixed): CG on A d = r/||r|| with the FP32 / tensor-core operator,
//                  FP32 vectors, FP64 dot products, to a loose tolerance;
//                  x += ||r|| d.
// The FP32 inner operator is one fused Helmholtz launch (alpha M + beta K,
// femtc_helmholtz_apply); the tensor-core forms sum the library's mass and
// stiffness actions.  The
// Jacobi diagonal comes from sum factorization (squared and product 1D tables
// applied to the per-point factors).  Inner iterations run as CUDA graphs of
// kItersPerGraph iterations; the host reads one residual scalar per graph.
// An inner iteration is four launches: the operator, <p,Ap> partial sums,
// the update (every block first sums the <p,Ap> partials itself for alpha)
// and the direction (every block sums the <r,z> partials for beta).  The CG
// scalars live in two slots used in turn, so that the block that writes the
// next iteration's <r,z> never overwrites the value the others still read.
// All device memory of a request is one stream-ordered allocation whose size
// femtc_solve_bytes() reports up front, so a server can admit by HBM budget.
// Reductions use a fixed grid and a fixed summation order, so a solve gives
// the same bits whether it runs alone or next to other solves.
#include "femtc_gpu.h"

#include "common.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

namespace femtc
{
int aux_fail(int code, const char* msg); // femtc_abi.cu

namespace
{
constexpr int kRedBlocks = 512; // partial sums per reduction (fixed: deterministic)
constexpr int kRedThreads = 256;
constexpr int kItersPerGraph = 8;
constexpr int kDiagTab = 10 * 9; // Q*N entries of a 1D table (Q <= 10, N <= 9)

// ---------------------------------------------------------------- diag --
struct DiagParams
{
  const float* dw;   // [ncells][Q^3] (point stride gs: 1, or 8 in geo8)
  const float* G;    // [ncells][Q^3][gs] ([zz,yz,xz,yy,xy,xx]; gs = 6, or 8)
  int ds, gs;        // point strides of dw and G
  float* invdiag;    // [ncells][N^3]: 1 / diag(alpha M + beta K)
  long long ncells;
  int n, q;
  float alpha, beta;
  float phi[kDiagTab], gam[kDiagTab]; // Phi(q,i) = phi[q + i*Q]
};

// One CTA per cell.  diag_i = sum_q sum_t c_t F_t(q) A0_t(q0,i0) A1_t(q1,i1)
// A2_t(q2,i2) over seven point fields: alpha*D with (Phi^2, Phi^2, Phi^2),
// beta*G_xx with (Gam^2, Phi^2, Phi^2), ..., 2 beta G_xy with
// (Phi Gam, Phi Gam, Phi^2), ...; each term is three axis contractions.
__global__ void __launch_bounds__(256) diag_kernel(const __grid_constant__ DiagParams p)
{
  extern __shared__ float sm[];
  const int n = p.n, q = p.q, q3 = q * q * q, n3 = n * n * n, qn = q * n;
  float* F = sm;              // q^3
  float* T1 = F + q3;         // [i0][q1][q2]
  float* T2 = T1 + n * q * q; // [i0][i1][q2]
  float* out = T2 + n * n * q;
  float* tb = out + n3; // PP, GG, PG tables (q*n each)
  for (int i = threadIdx.x; i < qn; i += blockDim.x)
  {
    const float a = p.phi[i], g = p.gam[i];
    tb[i] = a * a;
    tb[qn + i] = g * g;
    tb[2 * qn + i] = a * g;
  }
  // term: (field component or -1 for D, coefficient, tables of axes 0/1/2)
  // table ids: 0 = PP, 1 = GG, 2 = PG; G components [zz,yz,xz,yy,xy,xx]
  const int comp[7] = {-1, 5, 3, 0, 4, 2, 1};
  const float coef[7] = {p.alpha, p.beta, p.beta, p.beta, 2 * p.beta, 2 * p.beta, 2 * p.beta};
  const int t0[7] = {0, 1, 0, 0, 2, 2, 0};
  const int t1[7] = {0, 0, 1, 0, 2, 0, 2};
  const int t2[7] = {0, 0, 0, 1, 0, 2, 2};
  __syncthreads();
  for (long long cell = blockIdx.x; cell < p.ncells; cell += gridDim.x)
  {
    for (int i = threadIdx.x; i < n3; i += blockDim.x)
      out[i] = 0.f;
    for (int t = 0; t < 7; ++t)
    {
      if (coef[t] == 0.f)
        continue;
      const float c = coef[t];
      for (int i = threadIdx.x; i < q3; i += blockDim.x)
        F[i] = c * (comp[t] < 0 ? p.dw[(cell * q3 + i) * p.ds] : p.G[(cell * q3 + i) * p.gs + comp[t]]);
      __syncthreads();
      const float* A0 = tb + t0[t] * qn;
      const float* A1 = tb + t1[t] * qn;
      const float* A2 = tb + t2[t] * qn;
      for (int i = threadIdx.x; i < n * q * q; i += blockDim.x)
      {
        const int i0 = i / (q * q), r = i - i0 * q * q;
        float s = 0.f;
        for (int k = 0; k < q; ++k)
          s = fmaf(A0[k + i0 * q], F[k * q * q + r], s);
        T1[i] = s;
      }
      __syncthreads();
      for (int i = threadIdx.x; i < n * n * q; i += blockDim.x)
      {
        const int i0 = i / (n * q), r = i - i0 * n * q, i1 = r / q, q2 = r - i1 * q;
        float s = 0.f;
        for (int k = 0; k < q; ++k)
          s = fmaf(A1[k + i1 * q], T1[(i0 * q + k) * q + q2], s);
        T2[i] = s;
      }
      __syncthreads();
      for (int i = threadIdx.x; i < n3; i += blockDim.x)
      {
        const int r = i / n, i2 = i - r * n;
        float s = 0.f;
        for (int k = 0; k < q; ++k)
          s = fmaf(A2[k + i2 * q], T2[r * q + k], s);
        out[i] += s;
      }
      __syncthreads();
    }
    for (int i = threadIdx.x; i < n3; i += blockDim.x)
      p.invdiag[cell * n3 + i] = 1.f / out[i];
    __syncthreads();
  }
}

// ----------------------------------------------------------- reductions --
struct Scalars
{
  double rz, pap, alpha, beta, rr, spare[3];
};

__device__ __forceinline__ double block_sum(double v)
{
  __shared__ double ws[kRedThreads / 32];
  for (int o = 16; o > 0; o >>= 1)
    v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0)
    ws[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kRedThreads / 32; ++w)
      s += ws[w];
  __syncthreads();
  return s; // valid in thread 0
}

// Partial sums: part[0..kRedBlocks) <r,z>, part[kRedBlocks..) <r,r>,
// part[2 kRedBlocks..) <p,Ap>.
constexpr int kPartRZ = 0, kPartRR = kRedBlocks, kPartPAP = 2 * kRedBlocks;

// Ap = a t1 + b t2 ; partial <p, Ap> (part: the <p,Ap> region)
__global__ void __launch_bounds__(kRedThreads)
    ap_dot_kernel(const float* t1, const float* t2, float a, float b,
                  const float* pv, float* Ap, long long n, double* part)
{
  double s = 0.0;
  for (long long i = blockIdx.x * (long long)kRedThreads + threadIdx.x; i < n;
       i += (long long)gridDim.x * kRedThreads)
  {
    const float ap = a * t1[i] + b * t2[i];
    Ap[i] = ap;
    s += (double)pv[i] * (double)ap;
  }
  s = block_sum(s);
  if (threadIdx.x == 0)
    part[blockIdx.x] = s;
}

__device__ __forceinline__ double sum_parts(const double* part, int nb)
{
  double s = 0.0;
  for (int i = threadIdx.x; i < nb; i += kRedThreads)
    s += part[i];
  return block_sum(s);
}

// alpha = <r,z> / <p,Ap> (every block sums the <p,Ap> partials in the same
// order, so all get the same bits); d += alpha p ; r -= alpha Ap ;
// z = r / diag ; partial <r,z>, <r,r>.  sc: this iteration's slot.
__global__ void __launch_bounds__(kRedThreads)
    update_kernel(Scalars* sc, const float* pv, const float* Ap, float* d,
                  float* r, float* z, const float* invdiag, long long n,
                  double* part, int nb)
{
  __shared__ double s_alpha;
  const double pap = sum_parts(part + kPartPAP, nb);
  if (threadIdx.x == 0)
  {
    const double rz0 = sc->rz;
    s_alpha = (pap > 0.0 && rz0 > 0.0) ? rz0 / pap : 0.0;
    if (blockIdx.x == 0)
    {
      sc->pap = pap;
      sc->alpha = s_alpha;
    }
  }
  __syncthreads();
  const float alpha = (float)s_alpha;
  double rz = 0.0, rr = 0.0;
  for (long long i = blockIdx.x * (long long)kRedThreads + threadIdx.x; i < n;
       i += (long long)gridDim.x * kRedThreads)
  {
    d[i] = fmaf(alpha, pv[i], d[i]);
    const float ri = fmaf(-alpha, Ap[i], r[i]);
    r[i] = ri;
    const float zi = ri * invdiag[i];
    z[i] = zi;
    rz += (double)ri * (double)zi;
    rr += (double)ri * (double)ri;
  }
  rz = block_sum(rz);
  rr = block_sum(rr);
  if (threadIdx.x == 0)
  {
    part[kPartRZ + blockIdx.x] = rz;
    part[kPartRR + blockIdx.x] = rr;
  }
}

// <r,z>, <r,r> of a start (no previous direction): into slot sc
__global__ void __launch_bounds__(kRedThreads)
    reduce_start_kernel(const double* part, int nb, Scalars* sc)
{
  const double rz = sum_parts(part + kPartRZ, nb);
  const double rr = sum_parts(part + kPartRR, nb);
  if (threadIdx.x == 0)
  {
    sc->beta = 0.0;
    sc->rz = rz;
    sc->rr = rr;
  }
}

// beta = <r,z>_new / <r,z> (every block sums the partials in the same
// order); p = z + beta p.  sc: this iteration's slot (read), next: the other
// slot, where block 0 leaves <r,z>_new, <r,r> and beta.
__global__ void __launch_bounds__(kRedThreads)
    dir_kernel(const Scalars* sc, Scalars* next, const double* part, int nb, const float* z,
               float* p, long long n)
{
  __shared__ double s_beta;
  const double rz = sum_parts(part + kPartRZ, nb);
  const double rr = sum_parts(part + kPartRR, nb);
  if (threadIdx.x == 0)
  {
    const double rz0 = sc->rz;
    s_beta = rz0 > 0.0 ? rz / rz0 : 0.0;
    if (blockIdx.x == 0)
    {
      next->beta = s_beta;
      next->rz = rz;
      next->rr = rr;
    }
  }
  __syncthreads();
  const float beta = (float)s_beta;
  for (long long i = blockIdx.x * (long long)kRedThreads + threadIdx.x; i < n;
       i += (long long)gridDim.x * kRedThreads)
    p[i] = fmaf(beta, p[i], z[i]);
}

// inner start: r32 = r64 * inv, d = 0, z = r32/diag, p = z ; partial <r,z>, <r,r>
__global__ void __launch_bounds__(kRedThreads)
    inner_init_kernel(const double* r64, double inv, float* r, float* d,
                      float* z, float* p, const float* invdiag, long long n,
                      double* part)
{
  double rz = 0.0, rr = 0.0;
  for (long long i = blockIdx.x * (long long)kRedThreads + threadIdx.x; i < n;
       i += (long long)gridDim.x * kRedThreads)
  {
    const float ri = (float)(r64[i] * inv);
    r[i] = ri;
    d[i] = 0.f;
    const float zi = ri * invdiag[i];
    z[i] = zi;
    p[i] = zi;
    rz += (double)ri * (double)zi;
    rr += (double)ri * (double)ri;
  }
  rz = block_sum(rz);
  rr = block_sum(rr);
  if (threadIdx.x == 0)
  {
    part[kPartRZ + blockIdx.x] = rz;
    part[kPartRR + blockIdx.x] = rr;
  }
}

// x += s d (FP64)
__global__ void __launch_bounds__(kRedThreads)
    axpy_kernel(double* x, double s, const float* d, long long n)
{
  for (long long i = blockIdx.x * (long long)kRedThreads + threadIdx.x; i < n;
       i += (long long)gridDim.x * kRedThreads)
    x[i] += s * (double)d[i];
}

// r = b - (a t1 + c t2) in FP64 ; partial <r,r>
__global__ void __launch_bounds__(kRedThreads)
    resid_kernel(const double* b, const double* t1, const double* t2, double a,
                 double c, double* r, long long n, double* part)
{
  double rr = 0.0;
  for (long long i = blockIdx.x * (long long)kRedThreads + threadIdx.x; i < n;
       i += (long long)gridDim.x * kRedThreads)
  {
    const double ri = b[i] - (a * t1[i] + c * t2[i]);
    r[i] = ri;
    rr += ri * ri;
  }
  rr = block_sum(rr);
  if (threadIdx.x == 0)
  {
    part[kPartRZ + blockIdx.x] = 0.0;
    part[kPartRR + blockIdx.x] = rr;
  }
}

// f64 -> f32 copy of the per-point factors
__global__ void __launch_bounds__(kRedThreads)
    to_f32_kernel(const double* a, float* b, long long n)
{
  for (long long i = blockIdx.x * (long long)kRedThreads + threadIdx.x; i < n;
       i += (long long)gridDim.x * kRedThreads)
    b[i] = (float)a[i];
}

// geo8[p] = (beta G[p][0..5], alpha dw[p], 0) in FP32 from the FP64 factors:
// the interleaved geometry of the Helmholtz kernel
__global__ void __launch_bounds__(kRedThreads)
    pack_geo8_kernel(const double* dw, const double* G, double a, double c, float4* geo8,
                     long long npts)
{
  for (long long i = blockIdx.x * (long long)kRedThreads + threadIdx.x; i < npts;
       i += (long long)gridDim.x * kRedThreads)
  {
    const double* g = G + i * 6;
    geo8[2 * i] = make_float4((float)(c * g[0]), (float)(c * g[1]), (float)(c * g[2]),
                              (float)(c * g[3]));
    geo8[2 * i + 1] = make_float4((float)(c * g[4]), (float)(c * g[5]), (float)(a * dw[i]), 0.f);
  }
}

// s = <p, Ap> partial sums (the fused operator already wrote Ap); part:
// the <p,Ap> region
__global__ void __launch_bounds__(kRedThreads)
    dot_kernel(const float* pv, const float* Ap, long long n, double* part)
{
  double s = 0.0;
  for (long long i = blockIdx.x * (long long)kRedThreads + threadIdx.x; i < n;
       i += (long long)gridDim.x * kRedThreads)
    s += (double)pv[i] * (double)Ap[i];
  s = block_sum(s);
  if (threadIdx.x == 0)
    part[blockIdx.x] = s;
}

// --------------------------------------------------------------- buffers --
struct Bufs
{
  double *J, *dw64, *G64, *b, *x, *r, *t1d, *t2d, *part;
  float *dw32, *G32, *geo8, *r32, *z, *p, *Ap, *t1, *t2, *d, *invdiag;
  Scalars* sc;
};

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

size_t carve(void* base, int n, int q, size_t nc, Bufs* B)
{
  const size_t n3 = (size_t)n * n * n * nc, q3 = (size_t)q * q * q * nc;
  size_t off = 0;
  auto take = [&](size_t bytes) -> char* {
    char* ptr = base ? static_cast<char*>(base) + off : nullptr;
    off += align256(bytes);
    return ptr;
  };
  Bufs b{};
  b.J = (double*)take(9 * nc * 8);
  b.dw64 = (double*)take(q3 * 8);
  b.G64 = (double*)take(6 * q3 * 8);
  b.b = (double*)take(n3 * 8);
  b.x = (double*)take(n3 * 8);
  b.r = (double*)take(n3 * 8);
  b.t1d = (double*)take(n3 * 8);
  b.t2d = (double*)take(n3 * 8);
  b.part = (double*)take(3 * kRedBlocks * 8);
  // FP32 geometry: separate dw and G (mass and stiffness launches), or the
  // interleaved geo8 of the fused Helmholtz launch, in one region sized for
  // the larger (8 values per point)
  {
    char* g = take(8 * q3 * 4);
    b.dw32 = (float*)g;
    b.G32 = g ? (float*)(g + align256(q3 * 4)) : nullptr;
    b.geo8 = (float*)g;
  }
  b.r32 = (float*)take(n3 * 4);
  b.z = (float*)take(n3 * 4);
  b.p = (float*)take(n3 * 4);
  b.Ap = (float*)take(n3 * 4);
  b.t1 = (float*)take(n3 * 4);
  b.t2 = (float*)take(n3 * 4);
  b.d = (float*)take(n3 * 4);
  b.invdiag = (float*)take(n3 * 4);
  b.sc = (Scalars*)take(2 * sizeof(Scalars)); // two slots, used in turn
  if (B)
    *B = b;
  return off;
}

int cuda_err(cudaError_t e)
{
  return e == cudaSuccess ? FEMTC_OK : aux_fail(FEMTC_ERR_CUDA, cudaGetErrorString(e));
}

int grid_of(long long n)
{
  const long long g = (n + kRedThreads - 1) / kRedThreads;
  return (int)(g < kRedBlocks ? (g < 1 ? 1 : g) : kRedBlocks);
}

// The FP32 inner operator with a stiffness term runs as one Helmholtz
// launch (alpha and beta folded into its geometry).
bool fused_operator(const femtc_solve_request& rq)
{
  return rq.inner_dtype == FEMTC_F32 && rq.beta != 0.0;
}

// One inner CG iteration (4 or 5 launches) on stream st; it reads <r,z> from
// slot `slot` and leaves the next one in the other slot.
int inner_iteration(const femtc_solve_request& rq, const Bufs& B, const float* tab32,
                    size_t nd, cudaStream_t st, int slot)
{
  const int g = grid_of((long long)nd);
  if (fused_operator(rq))
  {
    int rc = femtc_helmholtz_apply(FEMTC_F32, rq.degree, rq.nquad, tab32, B.p, B.Ap, B.geo8,
                                   rq.ncells, st);
    if (rc != FEMTC_OK)
      return rc;
    dot_kernel<<<g, kRedThreads, 0, st>>>(B.p, B.Ap, (long long)nd, B.part + kPartPAP);
  }
  else
  {
    int rc = femtc_mass_apply(rq.inner_dtype, FEMTC_EXACT, rq.degree, rq.nquad, tab32, B.p,
                              B.t1, B.dw32, rq.ncells, st);
    if (rc == FEMTC_OK && rq.beta != 0.0)
      rc = femtc_stiffness_apply(rq.inner_dtype, FEMTC_EXACT, rq.degree, rq.nquad, tab32, B.p,
                                 B.t2, B.G32, rq.ncells, st);
    if (rc != FEMTC_OK)
      return rc;
    ap_dot_kernel<<<g, kRedThreads, 0, st>>>(B.t1, rq.beta != 0.0 ? B.t2 : B.t1,
                                             (float)rq.alpha,
                                             rq.beta != 0.0 ? (float)rq.beta : 0.f, B.p, B.Ap,
                                             (long long)nd, B.part + kPartPAP);
  }
  update_kernel<<<g, kRedThreads, 0, st>>>(B.sc + slot, B.p, B.Ap, B.d, B.r32, B.z, B.invdiag,
                                           (long long)nd, B.part, g);
  dir_kernel<<<g, kRedThreads, 0, st>>>(B.sc + slot, B.sc + (slot ^ 1), B.part, g, B.z, B.p,
                                        (long long)nd);
  return cuda_err(cudaGetLastError());
}

// FP64 residual r = b - A x and rr = <r,r> (read back: synchronises st)
int residual64(const femtc_solve_request& rq, const Bufs& B, const double* tab64, size_t nd,
               cudaStream_t st, double* rr)
{
  int rc = femtc_mass_apply(FEMTC_F64, FEMTC_EXACT, rq.degree, rq.nquad, tab64, B.x, B.t1d,
                            B.dw64, rq.ncells, st);
  if (rc == FEMTC_OK && rq.beta != 0.0)
    rc = femtc_stiffness_apply(FEMTC_F64, FEMTC_EXACT, rq.degree, rq.nquad, tab64, B.x, B.t2d,
                               B.G64, rq.ncells, st);
  if (rc != FEMTC_OK)
    return rc;
  const int g = grid_of((long long)nd);
  resid_kernel<<<g, kRedThreads, 0, st>>>(B.b, B.t1d, rq.beta != 0.0 ? B.t2d : B.t1d, rq.alpha,
                                          rq.beta != 0.0 ? rq.beta : 0.0, B.r, (long long)nd,
                                          B.part);
  reduce_start_kernel<<<1, kRedThreads, 0, st>>>(B.part, g, B.sc);
  Scalars s;
  cudaMemcpyAsync(&s, B.sc, sizeof(s), cudaMemcpyDeviceToHost, st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess)
    return cuda_err(e);
  *rr = s.rr;
  return FEMTC_OK;
}
} // namespace

int solve_on_stream(const femtc_solve_request* rq, femtc_solve_result* res, cudaStream_t st)
{
  using clk = std::chrono::steady_clock;
  const auto t0 = clk::now();
  std::memset(res, 0, sizeof(*res));
  const int n = rq->degree + 1, q = rq->nquad;
  const size_t nc = rq->ncells, nd = (size_t)n * n * n * nc, q3 = (size_t)q * q * q * nc;
  // tables
  std::vector<double> tab64(2 * q * n);
  int rc = femtc_tabulate(rq->degree, q, tab64.data(), nullptr, nullptr, nullptr);
  if (rc != FEMTC_OK)
    return rc;
  std::vector<float> tab32(tab64.begin(), tab64.end());
  std::vector<double> wts(q);
  femtc_tabulate(rq->degree, q, tab64.data(), nullptr, wts.data(), nullptr);
  // memory: one stream-ordered allocation
  const size_t bytes = carve(nullptr, n, q, nc, nullptr);
  void* base = nullptr;
  cudaError_t e = cudaMallocAsync(&base, bytes, st);
  if (e != cudaSuccess)
    return aux_fail(FEMTC_ERR_NOMEM, "solve: device allocation failed");
  Bufs B;
  carve(base, n, q, nc, &B);
  auto finish = [&](int code) {
    cudaFreeAsync(base, st);
    cudaStreamSynchronize(st);
    res->status = code;
    res->ms_total = std::chrono::duration<double, std::milli>(clk::now() - t0).count();
    return code;
  };
  // inputs, geometry (FP64, then FP32 copies), diagonal
  cudaMemcpyAsync(B.J, rq->J, 9 * nc * 8, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(B.b, rq->b, nd * 8, cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(B.x, 0, nd * 8, st);
  rc = femtc_geometry(FEMTC_F64, q, wts.data(), B.J, 0, B.dw64, B.G64, nc, st);
  if (rc != FEMTC_OK)
    return finish(rc);
  const bool fused = fused_operator(*rq);
  if (fused)
    pack_geo8_kernel<<<grid_of((long long)q3), kRedThreads, 0, st>>>(
        B.dw64, B.G64, rq->alpha, rq->beta, reinterpret_cast<float4*>(B.geo8), (long long)q3);
  else
  {
    to_f32_kernel<<<grid_of((long long)q3), kRedThreads, 0, st>>>(B.dw64, B.dw32,
                                                                  (long long)q3);
    to_f32_kernel<<<grid_of((long long)(6 * q3)), kRedThreads, 0, st>>>(B.G64, B.G32,
                                                                        (long long)(6 * q3));
  }
  {
    DiagParams dp;
    std::memset(&dp, 0, sizeof(dp));
    // the fused geometry already carries alpha and beta
    dp.dw = fused ? B.geo8 + 6 : B.dw32;
    dp.G = fused ? B.geo8 : B.G32;
    dp.ds = fused ? 8 : 1;
    dp.gs = fused ? 8 : 6;
    dp.invdiag = B.invdiag;
    dp.ncells = (long long)nc;
    dp.n = n;
    dp.q = q;
    dp.alpha = fused ? 1.0f : (float)rq->alpha;
    dp.beta = fused ? 1.0f : (float)rq->beta;
    for (int i = 0; i < q * n; ++i)
    {
      dp.phi[i] = (float)tab64[i];
      dp.gam[i] = (float)tab64[q * n + i];
    }
    const size_t sm = sizeof(float) * ((size_t)q * q * q + (size_t)n * q * q +
                                       (size_t)n * n * q + (size_t)n * n * n + 3 * q * n);
    const int g = (int)std::min<size_t>(nc, 4096);
    diag_kernel<<<g, 256, sm, st>>>(dp);
  }
  if ((rc = cuda_err(cudaGetLastError())) != FEMTC_OK)
    return finish(rc);
  // r = b, ||b||
  double rr = 0.0;
  rc = residual64(*rq, B, tab64.data(), nd, st, &rr);
  if (rc != FEMTC_OK)
    return finish(rc);
  const double bnorm = std::sqrt(rr);
  res->bnorm = bnorm;
  if (bnorm == 0.0)
  {
    cudaMemcpyAsync(rq->x, B.x, nd * 8, cudaMemcpyDeviceToHost, st);
    res->relres = 0.0;
    return finish(FEMTC_OK);
  }
  // one eager inner iteration caches kernel attributes before capture
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  const double inner_tol = rq->inner_rtol > 0 ? rq->inner_rtol : 1e-4;
  const int max_outer = rq->max_outer > 0 ? rq->max_outer : 20;
  const int max_inner = rq->max_inner > 0 ? rq->max_inner : 2000;
  double relres = 1.0;
  int outer = 0, inner_total = 0;
  for (; outer < max_outer; ++outer)
  {
    relres = std::sqrt(rr) / bnorm;
    if (relres <= rq->rtol)
      break;
    const int g = grid_of((long long)nd);
    inner_init_kernel<<<g, kRedThreads, 0, st>>>(B.r, 1.0 / std::sqrt(rr), B.r32, B.d, B.z,
                                                 B.p, B.invdiag, (long long)nd, B.part);
    // slots: the first (eager) iteration of a solve reads slot 0 and leaves
    // its result in slot 1; the graph's iterations read slots 1, 0, 1, ...
    // (an even count), so every graph starts and ends on slot 1
    reduce_start_kernel<<<1, kRedThreads, 0, st>>>(B.part, g, B.sc + (exec ? 1 : 0));
    int it = 0;
    while (it < max_inner)
    {
      if (!exec)
      {
        // first use: one eager iteration, then capture a graph of k of them
        rc = inner_iteration(*rq, B, tab32.data(), nd, st, 0);
        if (rc != FEMTC_OK)
          return finish(rc);
        ++it;
        e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess)
          return finish(cuda_err(e));
        static_assert(kItersPerGraph % 2 == 0, "graphs start and end on slot 1");
        for (int k = 0; k < kItersPerGraph && rc == FEMTC_OK; ++k)
          rc = inner_iteration(*rq, B, tab32.data(), nd, st, (k & 1) ^ 1);
        e = cudaStreamEndCapture(st, &graph);
        if (rc != FEMTC_OK)
          return finish(rc);
        if (e != cudaSuccess || cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess)
          return finish(aux_fail(FEMTC_ERR_CUDA, "solve: graph capture failed"));
      }
      else
      {
        e = cudaGraphLaunch(exec, st);
        if (e != cudaSuccess)
          return finish(cuda_err(e));
        it += kItersPerGraph;
      }
      Scalars s; // the latest <r,z>, <r,r>: slot 1 after the eager iteration or a graph
      cudaMemcpyAsync(&s, B.sc + 1, sizeof(s), cudaMemcpyDeviceToHost, st);
      e = cudaStreamSynchronize(st);
      if (e != cudaSuccess)
        return finish(cuda_err(e));
      if (!(std::sqrt(s.rr) > inner_tol)) // converged (or NaN: stop)
        break;
    }
    inner_total += it;
    const int g2 = grid_of((long long)nd);
    axpy_kernel<<<g2, kRedThreads, 0, st>>>(B.x, std::sqrt(rr), B.d, (long long)nd);
    rc = residual64(*rq, B, tab64.data(), nd, st, &rr);
    if (rc != FEMTC_OK)
      return finish(rc);
  }
  relres = std::sqrt(rr) / bnorm;
  if (exec)
    cudaGraphExecDestroy(exec);
  if (graph)
    cudaGraphDestroy(graph);
  cudaMemcpyAsync(rq->x, B.x, nd * 8, cudaMemcpyDeviceToHost, st);
  res->outer_iters = outer;
  res->inner_iters = inner_total;
  res->relres = relres;
  return finish(relres <= rq->rtol ? FEMTC_OK : FEMTC_ERR_NOT_CONVERGED);
}

size_t solve_bytes(int degree, int nquad, size_t ncells)
{
  return carve(nullptr, degree + 1, nquad, ncells, nullptr);
}
} // namespace femtc

using namespace femtc;

extern "C" {

size_t femtc_solve_bytes(int degree, int nquad, size_t ncells)
{
  return solve_bytes(degree, nquad, ncells);
}

int femtc_solve(const femtc_solve_request* rq, femtc_solve_result* res, void* stream)
{
  if (!rq || !res)
    return aux_fail(FEMTC_ERR_INVALID, "solve: null argument");
  if (rq->degree < 1 || rq->degree > 7 || rq->nquad < rq->degree + 1 || rq->nquad > rq->degree + 3)
    return aux_fail(FEMTC_ERR_UNSUPPORTED, "solve: degree 1..7, nquad in degree+1..degree+3");
  if (!rq->J || !rq->b || !rq->x || rq->ncells == 0)
    return aux_fail(FEMTC_ERR_INVALID, "solve: missing inputs");
  if (rq->inner_dtype != FEMTC_F32 && rq->inner_dtype != FEMTC_F16X2 &&
      rq->inner_dtype != FEMTC_BF16X3)
    return aux_fail(FEMTC_ERR_INVALID,
                    "solve: inner dtype must be FEMTC_F32, FEMTC_F16X2 or FEMTC_BF16X3");
  if (!(rq->alpha > 0.0) || rq->beta < 0.0)
    return aux_fail(FEMTC_ERR_INVALID, "solve: need alpha > 0 and beta >= 0 (SPD operator)");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  bool own = false;
  if (!st)
  {
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
      return aux_fail(FEMTC_ERR_CUDA, "solve: stream creation failed");
    own = true;
  }
  const int rc = solve_on_stream(rq, res, st);
  if (own)
    cudaStreamDestroy(st);
  return rc;
}

} // extern "C"

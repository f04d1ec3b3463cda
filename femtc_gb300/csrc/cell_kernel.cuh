// Sum-factorized cell kernels for the hexahedral mass and stiffness action
// on GB300 (sm_103a), CUDA-core arithmetic (T = double or float).
//
// What one launch computes (per cell c, N = P+1 DOFs and Q points per axis):
//   mass      : y_c = B^T D_c B u_c,                 B = Phi x Phi x Phi
//   stiffness : y_c = sum_d D_d^T (G_c D u_c)_d,     D_x = Gamma x Phi x Phi ...
// in the reference's layouts (IgorBaratta/femtc src/mass.hpp:25-29,
// src/stiffness.hpp:20-27,44-48), with either exact semantics or the
// reference's literal semantics (src/mass.hpp:21, src/stiffness.hpp:76-97).
//
// GB300 design:
//  * persistent CTAs walk tiles of `cb` consecutive cells; the DOF slab of the
//    next tile (and optionally its geometry slab) is fetched by the TMA engine
//    (cp.async.bulk, 1D, mbarrier completion) into the other of two shared
//    memory stages while the current tile is computed;
//  * the output slab is written back by a TMA bulk store from shared memory;
//  * the 1D tables live in the launch's parameter block (__grid_constant__),
//    so every FMA takes its table operand straight from the constant bank:
//    no registers, no shared-memory traffic for the tables;
//  * each contraction is a "pencil" pass: a thread loads one pencil of the
//    tensor (K values along the contracted axis) and writes M outputs; all
//    threads of the CTA share the pencils of the whole tile, so lanes stay
//    busy whatever P and Q are;
//  * axis order 2 -> 1 -> 0: the last forward contraction, the quadrature
//    point scaling / G transform and the first backward contraction are
//    fused in registers, and there the geometry is read with unit stride
//    across threads;
//  * stiffness shares partial contractions between the three gradient
//    components (2/3/3 contractions forward, mirrored backward).
#pragma once

#include "common.cuh"

namespace femtc
{

enum Op : int
{
  OP_MASS = 0,
  OP_STIFFNESS = 1
};
enum Sem : int
{
  SEM_EXACT = 0,
  SEM_REFERENCE = 1
};

constexpr int kMaxN = 9;
constexpr int kMaxQ = 10;
constexpr int kCellThreads = 256;

template <typename T>
struct CellParams
{
  const T* u;        // [ncells][N^3]
  T* y;              // [ncells][N^3]
  const T* geo;      // mass: [ncells][Q^3]; stiffness: [ncells][Q^3][6]
  long long ncells;
  int cb;            // cells per tile, a multiple of 4
  int geo_staged;    // 1: geometry slab staged by TMA, 0: read in the fused pass
  T tab[2][kMaxQ * kMaxN]; // Phi(q,i) = tab[0][q + i*Q], Gamma = tab[1]
};

template <int N, int Q, int OP, int SEM>
struct Shape
{
  static constexpr int N3 = N * N * N;
  static constexpr int Q3 = Q * Q * Q;
  static constexpr int NC = (OP == OP_MASS) ? 1 : 6;
  static constexpr int QP = Q | 1; // odd row length: conflict-free pencils
  static constexpr int SA = N * N * QP; // [i0][i1][q2] buffers
  static constexpr int SB = N * Q * Q;  // [i0][q1][q2] buffers
  static constexpr int nA = (OP == OP_STIFFNESS && SEM == SEM_EXACT) ? 2 : 1;
  static constexpr int nB =
      (OP == OP_MASS) ? 1 : ((SEM == SEM_EXACT) ? 3 : 2);
  static constexpr int work = nA * SA + nB * SB; // per cell, elements
};

// Byte offsets of the shared-memory regions (identical on host and device).
struct CellLayout
{
  unsigned u0, g0, u1, g1, y, w, total;
  __host__ __device__ CellLayout(int cb, int esize, int n3, int q3nc,
                                 int work, int staged)
  {
    const unsigned bu = (unsigned)cb * n3 * esize;
    const unsigned bg = staged ? (unsigned)cb * q3nc * esize : 0u;
    u0 = 128; // the two mbarriers live in the first 128 bytes
    g0 = u0 + bu;
    u1 = g0 + bg;
    g1 = u1 + bu;
    y = g1 + bg;
    w = y + bu;
    total = w + (unsigned)cb * work * esize;
  }
};

template <int N, int Q, int OP, int SEM, typename T>
__host__ __device__ inline CellLayout make_layout(int cb, int staged)
{
  using S = Shape<N, Q, OP, SEM>;
  return CellLayout(cb, (int)sizeof(T), S::N3, S::Q3 * S::NC, S::work, staged);
}

// y[m] = sum_k A(m,k) x[k] with A(m,k) = A[m*SM + k*SK] (compile-time
// indices: the table operand comes from the constant bank).
template <int M, int K, int SM, int SK, typename T>
__device__ __forceinline__ void mv(const T* __restrict__ A, const T (&x)[K],
                                   T (&y)[M])
{
#pragma unroll
  for (int m = 0; m < M; ++m)
  {
    T acc = A[m * SM] * x[0];
#pragma unroll
    for (int k = 1; k < K; ++k)
      acc = fma(A[m * SM + k * SK], x[k], acc);
    y[m] = acc;
  }
}

// y[m] += sum_k A(m,k) x[k]
template <int M, int K, int SM, int SK, typename T>
__device__ __forceinline__ void mv_acc(const T* __restrict__ A,
                                       const T (&x)[K], T (&y)[M])
{
#pragma unroll
  for (int m = 0; m < M; ++m)
  {
    T acc = y[m];
#pragma unroll
    for (int k = 0; k < K; ++k)
      acc = fma(A[m * SM + k * SK], x[k], acc);
    y[m] = acc;
  }
}

template <typename T, int N, int Q, int OP, int SEM>
struct CellTile
{
  using S = Shape<N, Q, OP, SEM>;
  // Forward tables: out q, contracted i: A(q,i) = tab[q + i*Q].
  static constexpr int FSM = 1, FSK = Q;
  // Backward tables: exact applies the transpose A(i,q) = tab[q + i*Q];
  // the reference reuses the forward table A(i,q) = tab[i + q*Q] (Q == N).
  static constexpr int BSM = (SEM == SEM_EXACT) ? Q : 1;
  static constexpr int BSK = (SEM == SEM_EXACT) ? 1 : Q;

  // Pass 1: contract axis 2 (i2 -> q2).  u[c][i0][i1][i2] -> A[c][i0][i1][q2]
  static __device__ __forceinline__ void pass1(const CellParams<T>& p,
                                               const T* __restrict__ su,
                                               T* __restrict__ w, int ncb)
  {
    T* A0 = w;
    T* A1 = w + ncb * S::SA;
    const int np = ncb * N * N;
    for (int t = threadIdx.x; t < np; t += blockDim.x)
    {
      const int c = t / (N * N), r = t - c * (N * N);
      T x[N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        x[k] = su[c * S::N3 + r * N + k];
      T o[Q];
      mv<Q, N, FSM, FSK>(p.tab[0], x, o);
      T* dst = A0 + c * S::SA + r * S::QP;
#pragma unroll
      for (int q = 0; q < Q; ++q)
        dst[q] = o[q];
      if constexpr (OP == OP_STIFFNESS && SEM == SEM_EXACT)
      {
        mv<Q, N, FSM, FSK>(p.tab[1], x, o);
        T* dst1 = A1 + c * S::SA + r * S::QP;
#pragma unroll
        for (int q = 0; q < Q; ++q)
          dst1[q] = o[q];
      }
    }
  }

  // Pass 2: contract axis 1 (i1 -> q1).  A[c][i0][i1][q2] -> B[c][i0][q1][q2]
  static __device__ __forceinline__ void pass2(const CellParams<T>& p,
                                               T* __restrict__ w, int ncb)
  {
    const T* A0 = w;
    const T* A1 = w + ncb * S::SA;
    T* B0 = w + ncb * S::nA * S::SA;
    T* B1 = B0 + ncb * S::SB;
    T* B2 = B1 + ncb * S::SB;
    const int np = ncb * N * Q;
    for (int t = threadIdx.x; t < np; t += blockDim.x)
    {
      const int c = t / (N * Q), r = t - c * (N * Q);
      const int i0 = r / Q, q2 = r - i0 * Q;
      const int ia = c * S::SA + i0 * N * S::QP + q2;
      const int ib = c * S::SB + i0 * Q * Q + q2;
      T x[N], o[Q];
#pragma unroll
      for (int k = 0; k < N; ++k)
        x[k] = A0[ia + k * S::QP];
      mv<Q, N, FSM, FSK>(p.tab[0], x, o);
#pragma unroll
      for (int q = 0; q < Q; ++q)
        B0[ib + q * Q] = o[q];
      if constexpr (OP == OP_STIFFNESS)
      {
        mv<Q, N, FSM, FSK>(p.tab[1], x, o);
#pragma unroll
        for (int q = 0; q < Q; ++q)
          B1[ib + q * Q] = o[q];
        if constexpr (SEM == SEM_EXACT)
        {
#pragma unroll
          for (int k = 0; k < N; ++k)
            x[k] = A1[ia + k * S::QP];
          mv<Q, N, FSM, FSK>(p.tab[0], x, o);
#pragma unroll
          for (int q = 0; q < Q; ++q)
            B2[ib + q * Q] = o[q];
        }
      }
    }
  }

  // Pass 3 (fused): contract axis 0 (i0 -> q0), scale by D or transform by
  // G per quadrature point, contract back (q0 -> i0), in place in B.
  static __device__ __forceinline__ void pass3(const CellParams<T>& p,
                                               T* __restrict__ w, int ncb,
                                               const T* __restrict__ geo,
                                               long long geo_cell0)
  {
    T* B0 = w + ncb * S::nA * S::SA;
    T* B1 = B0 + ncb * S::SB;
    T* B2 = B1 + ncb * S::SB;
    const int np = ncb * Q * Q;
    for (int t = threadIdx.x; t < np; t += blockDim.x)
    {
      const int c = t / (Q * Q), r = t - c * (Q * Q);
      const int ib = c * S::SB + r;
      // geometry of this pencil: point (q0, r) at (c*Q3 + q0*Q*Q + r)*NC
      const T* g = geo + ((long long)(geo_cell0 + c) * S::Q3 + r) * S::NC;
      if constexpr (OP == OP_MASS)
      {
        T x[N], v[Q], o[N];
#pragma unroll
        for (int k = 0; k < N; ++k)
          x[k] = B0[ib + k * Q * Q];
        mv<Q, N, FSM, FSK>(p.tab[0], x, v);
#pragma unroll
        for (int q = 0; q < Q; ++q)
          v[q] *= g[q * Q * Q];
        mv<N, Q, BSM, BSK>(p.tab[0], v, o);
#pragma unroll
        for (int k = 0; k < N; ++k)
          B0[ib + k * Q * Q] = o[k];
      }
      else
      {
        T xa[N], xg[N], fx[Q], fy[Q], fz[Q];
#pragma unroll
        for (int k = 0; k < N; ++k)
        {
          xa[k] = B0[ib + k * Q * Q];
          xg[k] = B1[ib + k * Q * Q];
        }
        mv<Q, N, FSM, FSK>(p.tab[1], xa, fx); // d/dx: Gamma on axis 0
        mv<Q, N, FSM, FSK>(p.tab[0], xg, fy); // d/dy: Gamma was on axis 1
        if constexpr (SEM == SEM_EXACT)
        {
          T xb[N];
#pragma unroll
          for (int k = 0; k < N; ++k)
            xb[k] = B2[ib + k * Q * Q];
          mv<Q, N, FSM, FSK>(p.tab[0], xb, fz); // d/dz: Gamma on axis 2
        }
        else
        {
          mv<Q, N, FSM, FSK>(p.tab[0], xa, fz); // reference: no derivative
        }
        // transform (src/stiffness.hpp:14-29): G = [zz,yz,xz,yy,xy,xx]
#pragma unroll
        for (int q = 0; q < Q; ++q)
        {
          const T* G = g + q * Q * Q * 6;
          const T w0 = fx[q], w1 = fy[q], w2 = fz[q];
          if constexpr (SEM == SEM_EXACT)
          {
            fx[q] = G[5] * w0 + G[4] * w1 + G[2] * w2;
            fy[q] = G[4] * w0 + G[3] * w1 + G[1] * w2;
          }
          fz[q] = G[2] * w0 + G[1] * w1 + G[0] * w2;
        }
        T o[N];
        if constexpr (SEM == SEM_EXACT)
        {
          mv<N, Q, BSM, BSK>(p.tab[1], fx, o);
#pragma unroll
          for (int k = 0; k < N; ++k)
            B0[ib + k * Q * Q] = o[k];
          mv<N, Q, BSM, BSK>(p.tab[0], fy, o);
#pragma unroll
          for (int k = 0; k < N; ++k)
            B1[ib + k * Q * Q] = o[k];
          mv<N, Q, BSM, BSK>(p.tab[0], fz, o);
#pragma unroll
          for (int k = 0; k < N; ++k)
            B2[ib + k * Q * Q] = o[k];
        }
        else
        {
          // only the last chain (Phi, Phi, Gamma) survives; axis 0 is Phi
          mv<N, Q, BSM, BSK>(p.tab[0], fz, o);
#pragma unroll
          for (int k = 0; k < N; ++k)
            B0[ib + k * Q * Q] = o[k];
        }
      }
    }
  }

  // Pass 4: backward axis 1 (q1 -> i1).  B[c][i0][q1][q2] -> A[c][i0][i1][q2]
  static __device__ __forceinline__ void pass4(const CellParams<T>& p,
                                               T* __restrict__ w, int ncb)
  {
    T* A0 = w;
    T* A1 = w + ncb * S::SA;
    const T* B0 = w + ncb * S::nA * S::SA;
    const T* B1 = B0 + ncb * S::SB;
    const T* B2 = B1 + ncb * S::SB;
    const int np = ncb * N * Q;
    for (int t = threadIdx.x; t < np; t += blockDim.x)
    {
      const int c = t / (N * Q), r = t - c * (N * Q);
      const int i0 = r / Q, q2 = r - i0 * Q;
      const int ia = c * S::SA + i0 * N * S::QP + q2;
      const int ib = c * S::SB + i0 * Q * Q + q2;
      T x[Q], o[N];
#pragma unroll
      for (int q = 0; q < Q; ++q)
        x[q] = B0[ib + q * Q];
      if constexpr (OP == OP_STIFFNESS && SEM == SEM_EXACT)
      {
        // U1 = Phi^T X + Gamma^T Y ; U2 = Phi^T Z
        mv<N, Q, BSM, BSK>(p.tab[0], x, o);
#pragma unroll
        for (int q = 0; q < Q; ++q)
          x[q] = B1[ib + q * Q];
        mv_acc<N, Q, BSM, BSK>(p.tab[1], x, o);
#pragma unroll
        for (int k = 0; k < N; ++k)
          A0[ia + k * S::QP] = o[k];
#pragma unroll
        for (int q = 0; q < Q; ++q)
          x[q] = B2[ib + q * Q];
        mv<N, Q, BSM, BSK>(p.tab[0], x, o);
#pragma unroll
        for (int k = 0; k < N; ++k)
          A1[ia + k * S::QP] = o[k];
      }
      else
      {
        mv<N, Q, BSM, BSK>(p.tab[0], x, o);
#pragma unroll
        for (int k = 0; k < N; ++k)
          A0[ia + k * S::QP] = o[k];
      }
    }
  }

  // Pass 5: backward axis 2 (q2 -> i2).  A[c][i0][i1][q2] -> y[c][i0][i1][i2]
  static __device__ __forceinline__ void pass5(const CellParams<T>& p,
                                               const T* __restrict__ w,
                                               T* __restrict__ sy, int ncb)
  {
    const T* A0 = w;
    const T* A1 = w + ncb * S::SA;
    const int np = ncb * N * N;
    for (int t = threadIdx.x; t < np; t += blockDim.x)
    {
      const int c = t / (N * N), r = t - c * (N * N);
      const int ia = c * S::SA + r * S::QP;
      T x[Q], o[N];
#pragma unroll
      for (int q = 0; q < Q; ++q)
        x[q] = A0[ia + q];
      if constexpr (OP == OP_MASS)
      {
        mv<N, Q, BSM, BSK>(p.tab[0], x, o);
      }
      else if constexpr (SEM == SEM_EXACT)
      {
        mv<N, Q, BSM, BSK>(p.tab[0], x, o);
#pragma unroll
        for (int q = 0; q < Q; ++q)
          x[q] = A1[ia + q];
        mv_acc<N, Q, BSM, BSK>(p.tab[1], x, o);
      }
      else
      {
        mv<N, Q, BSM, BSK>(p.tab[1], x, o); // reference: Gamma on axis 2
      }
      T* dst = sy + c * S::N3 + r * N;
#pragma unroll
      for (int k = 0; k < N; ++k)
        dst[k] = o[k];
    }
  }
};

// The streaming main loop shared by every kernel family: persistent CTAs,
// two TMA stages, five passes per tile, TMA bulk store of the result.
// `Tile` provides the Shape `S` and the static passes pass1..pass5.
template <typename T, typename Tile>
__device__ __forceinline__ void stream_tiles(const CellParams<T>& p)
{
  using S = typename Tile::S;
  extern __shared__ __align__(128) unsigned char smem[];
  const int cb = p.cb;
  const bool staged = p.geo_staged != 0;
  const long long ntiles = (p.ncells + cb - 1) / cb;
  const CellLayout L(cb, (int)sizeof(T), S::N3, S::Q3 * S::NC, S::work,
                     p.geo_staged);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
  // stage s buffers (selected arithmetically: no local-memory arrays)
  auto su = [&](int s) { return reinterpret_cast<T*>(smem + (s ? L.u1 : L.u0)); };
  auto sg = [&](int s) { return reinterpret_cast<T*>(smem + (s ? L.g1 : L.g0)); };
  T* sy = reinterpret_cast<T*>(smem + L.y);
  T* sw = reinterpret_cast<T*>(smem + L.w);
  const unsigned bu = (unsigned)cb * S::N3 * sizeof(T);
  const unsigned bg = staged ? (unsigned)cb * S::Q3 * S::NC * sizeof(T) : 0u;

  if (threadIdx.x == 0)
  {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();

  auto is_full = [&](long long t) { return (t + 1) * cb <= p.ncells; };
  auto issue = [&](long long t, int s) {
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(&bar[s], bu + bg);
    bulk_g2s(su(s), p.u + t * cb * S::N3, bu, &bar[s]);
    if (staged)
      bulk_g2s(sg(s), p.geo + t * cb * S::Q3 * S::NC, bg, &bar[s]);
  };

  long long tile = blockIdx.x;
  if (threadIdx.x == 0 && tile < ntiles && is_full(tile))
    issue(tile, 0);

  for (int it = 0; tile < ntiles; tile += gridDim.x, ++it)
  {
    const int s = it & 1;
    const long long next = tile + gridDim.x;
    if (threadIdx.x == 0 && next < ntiles && is_full(next))
      issue(next, s ^ 1);
    const bool full = is_full(tile);
    const int ncb = full ? cb : (int)(p.ncells - tile * cb);
    bool ok = true;
    if (full)
    {
      ok = mbar_wait(&bar[s], (unsigned)(it >> 1) & 1u);
    }
    else
    {
      // ragged last tile: plain coalesced loads into the same stage
      const long long u0 = tile * cb * S::N3;
      for (int i = threadIdx.x; i < ncb * S::N3; i += blockDim.x)
        su(s)[i] = p.u[u0 + i];
      if (staged)
      {
        const long long g0 = tile * cb * S::Q3 * S::NC;
        for (int i = threadIdx.x; i < ncb * S::Q3 * S::NC; i += blockDim.x)
          sg(s)[i] = p.geo[g0 + i];
      }
    }
    if (__syncthreads_or(!ok))
    {
      if (threadIdx.x == 0)
        record_fault(FAULT_MBAR_TIMEOUT);
      break;
    }
    Tile::pass1(p, su(s), sw, ncb);
    __syncthreads();
    Tile::pass2(p, sw, ncb);
    __syncthreads();
    if (staged)
      Tile::pass3(p, sw, ncb, sg(s), 0);
    else
      Tile::pass3(p, sw, ncb, p.geo, tile * cb);
    __syncthreads();
    Tile::pass4(p, sw, ncb);
    if (threadIdx.x == 0)
      bulk_wait_read0(); // previous tile's store has left sy
    __syncthreads();
    Tile::pass5(p, sw, sy, ncb);
    if (full)
    {
      fence_proxy_async_smem();
      __syncthreads();
      if (threadIdx.x == 0)
      {
        bulk_s2g(p.y + tile * cb * S::N3, sy, bu);
        bulk_commit();
      }
    }
    else
    {
      __syncthreads();
      const long long y0 = tile * cb * S::N3;
      for (int i = threadIdx.x; i < ncb * S::N3; i += blockDim.x)
        p.y[y0 + i] = sy[i];
    }
  }
  if (threadIdx.x == 0)
    bulk_wait0();
}

template <typename T, int N, int Q, int OP, int SEM>
__global__ void __launch_bounds__(kCellThreads)
    cell_kernel(const __grid_constant__ CellParams<T> p)
{
  stream_tiles<T, CellTile<T, N, Q, OP, SEM>>(p);
}

} // namespace femtc

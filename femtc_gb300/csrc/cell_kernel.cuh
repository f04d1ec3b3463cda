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
#include "df64.cuh"
#include "slab_strides.hpp"

#include <cuda.h> // CUtensorMap (the type only)

#include <type_traits>

namespace femtc
{

enum Op : int
{
  OP_MASS = 0,
  OP_STIFFNESS = 1,
  OP_HELMHOLTZ = 2, // alpha M + beta K in one pass (exact semantics)
  // Affine cells (exact semantics): detJ and J^-1 J^-T are constant over a
  // cell, so one set of factors per cell replaces the Q^3 per-point values.
  // The tensor-product quadrature weight w(q0) w(q1) w(q2) is folded into
  // the backward tables: every backward contraction along axis d scales
  // its table rows by w(q_d), and each point's value passes one backward
  // contraction per axis.
  OP_MASS_AFFINE = 3,
  OP_STIFFNESS_AFFINE = 4
};

// How a slab or tensor-core kernel reads the per-point geometry (the
// tile configuration's geo_staged value).
enum GeoMode : int
{
  GEO_PENCIL_L2 = 0, // read in the fused pass; each thread asks L2 for the
                     // lines of its next pencil while it computes this one
  GEO_STAGED = 1,    // staged through shared memory with the DOF slab (TMA)
  GEO_TILE_L2 = 2    // read in the fused pass; at the start of a tile each
                     // warp (CTA-wide loop: the CTA) asks L2 for the lines
                     // of its cells' geometry
};

__host__ __device__ constexpr bool op_affine(int op)
{
  return op == OP_MASS_AFFINE || op == OP_STIFFNESS_AFFINE;
}
// The operator an affine form computes (mass or stiffness).
__host__ __device__ constexpr int op_base(int op)
{
  return op_affine(op) ? op - OP_MASS_AFFINE : op;
}

// Geometry values per quadrature point: mass detJ*w; stiffness the six
// components of G; Helmholtz [zz,yz,xz,yy,xy,xx] of beta*G, then alpha*detJ*w
// and one zero (eight values: four 8-byte pairs per point); none for the
// affine forms.
__host__ __device__ constexpr int geo_nc(int op)
{
  return op == OP_MASS ? 1 : (op == OP_STIFFNESS ? 6 : (op == OP_HELMHOLTZ ? 8 : 0));
}
// Geometry values per cell of the affine forms: detJ (mass); the six
// components of detJ J^-1 J^-T as [zz,yz,xz,yy,xy,xx] (stiffness).
__host__ __device__ constexpr int cell_nc(int op)
{
  return op == OP_MASS_AFFINE ? 1 : (op == OP_STIFFNESS_AFFINE ? 6 : 0);
}
enum Sem : int
{
  SEM_EXACT = 0,
  SEM_REFERENCE = 1
};

constexpr int kMaxN = 9;
constexpr int kMaxQ = 10;
constexpr int kCellThreads = 256;

// Storage type of a compute type: values live in HBM and in the staging
// buffers as `type`; double-float arithmetic keeps FP64 storage.
template <typename T>
struct storage_of
{
  using type = T;
};
template <>
struct storage_of<df64>
{
  using type = double;
};
template <typename T>
using storage_t = typename storage_of<T>::type;

template <typename T>
__device__ __forceinline__ T from_storage(storage_t<T> v)
{
  if constexpr (std::is_same<T, df64>::value)
    return to_df64(v);
  else
    return v;
}

template <typename T>
__device__ __forceinline__ storage_t<T> to_storage(T v)
{
  if constexpr (std::is_same<T, df64>::value)
    return to_double(v);
  else
    return v;
}

template <typename T>
__device__ __forceinline__ T shfl_xor(T v, int lane_mask)
{
  return __shfl_xor_sync(0xffffffffu, v, lane_mask);
}

// Table slots in a launch's parameter block: FP32 kernels carry pair
// tables beside the 1D tables (SlabTileF2).
template <typename T>
constexpr int kTabSlots = std::is_same<T, float>::value ? 8 : 4;

template <typename T>
struct CellParams
{
  using ST = storage_t<T>;
  // Padded DOF/output slab slots (see slot_stride) move by 2D tensor copies
  // when tma_rows > 0: u and y as [ncells*N rows][N*N] with boxes of
  // [tma_rows rows][slot] (the slot's padding columns lie outside the
  // tensor: zeros in, not written out).  tma_rows == 0: one bulk copy per
  // slab.
  CUtensorMap tmu, tmy;
  int tma_rows;
  const ST* u;       // [ncells][N^3]
  ST* y;             // [ncells][N^3]
  const ST* geo;     // [ncells][Q^3][geo_nc(op)] (mass: [ncells][Q^3])
  long long ncells;
  int cb;            // cells per tile, a multiple of 4
  int geo_staged;    // geometry per point (GEO_*): 1 staged by TMA; 0 and 2
                     // read in the fused pass, 0 with each thread asking L2
                     // for its next pencil's geometry, 2 with the tile's
                     // geometry asked of L2 at the start of the tile
  int sq;            // slab kernels: stride of one i0 slab in the work buffers
  int sbc;           // slab kernels: stride of one cell in the work buffers
  int host_io;       // 1: u, geo, y are host memory read/written over the
                     // coherent host link with plain vector accesses (no TMA)
  // Phi(q,i) = tab[0][q + i*Q], Gamma = tab[1]; even-odd kernels: the
  // even-odd tables of Phi, Gamma (forward) and Phi^T, Gamma^T (backward)
  // in tab[0..3] (see mv_eo); the paired FP32 kernels: their pair tables
  // in tab[2..6] (see SlabTileF2)
  alignas(16) T tab[kTabSlots<T>][kMaxQ * kMaxN];
};

// What the tile passes read besides the data: the two 1D tables (pointers
// into a launch's parameter block, so table operands stay in the constant
// bank) and the work-buffer strides of the slab kernels.
template <typename T>
struct TabView
{
  const T* __restrict__ P; // Phi(q,i) = P[q + i*Q] (even-odd: forward table)
  const T* __restrict__ D; // Gamma(q,i) = D[q + i*Q] (even-odd: forward table)
  int sq, sbc;
  const T* __restrict__ PB = nullptr; // even-odd kernels: Phi^T table
  const T* __restrict__ DB = nullptr; // even-odd kernels: Gamma^T table
  const T* __restrict__ X = nullptr;  // slot 0 of the parameter block's
                                      // tables (pair tables: SlabTileF2)
};

template <int N, int Q, int OP, int SEM>
struct Shape
{
  static constexpr int N3 = N * N * N;
  static constexpr int Q3 = Q * Q * Q;
  static constexpr int NC = geo_nc(OP);
  static constexpr int QP = Q | 1; // odd row length: conflict-free pencils
  static constexpr int SA = N * N * QP; // [i0][i1][q2] buffers
  // [i0][q1][q2] buffers: odd q1 stride BQ and odd i0 stride QQP (fewer
  // shared-memory bank conflicts of the fragment gathers along q1 and i0)
  static constexpr int BQ = Q | 1;
  static constexpr int QQP = (Q * BQ) | 1;
  static constexpr int SB = N * QQP;
  static constexpr int nA = (op_base(OP) == OP_STIFFNESS && SEM == SEM_EXACT) ? 2 : 1;
  static constexpr int nB =
      (op_base(OP) == OP_MASS) ? 1 : ((SEM == SEM_EXACT) ? 3 : 2);
  static constexpr int work = nA * SA + nB * SB; // per cell, elements
};

// Byte offsets of the shared-memory regions (identical on host and device):
// two mbarriers, two (DOF slab, geometry slab) stages, the output slab, and
// the kernel family's work buffers.  The DOF, geometry and output regions
// start 128-byte aligned (tensor copies), the work buffers 16-byte aligned.
struct CellLayout
{
  unsigned u0, g0, u1, g1, y, w, total;
  unsigned stage; // bytes of one (DOF slab, geometry slab) stage
  // ns stages (2 for the CTA-wide loop, more for the warp-split one)
  __host__ __device__ CellLayout(unsigned bu, unsigned bg, unsigned bw, int ns = 2)
  {
    const unsigned au = (bu + 127u) & ~127u, ag = (bg + 127u) & ~127u;
    stage = au + ag;
    u0 = 128; // the mbarriers live in the first 128 bytes
    g0 = u0 + au;
    u1 = u0 + stage;
    g1 = u1 + au;
    y = u0 + (unsigned)ns * stage;
    w = y + au;
    total = w + ((bw + 15u) & ~15u);
  }
  __host__ __device__ unsigned u(int s) const { return u0 + (unsigned)s * stage; }
  __host__ __device__ unsigned g(int s) const { return g0 + (unsigned)s * stage; }
};

// Slot stride (elements) of one i0 slab in conflict-free form: packed for
// odd N (odd strides are conflict free), else the smallest slot whose byte
// size is an odd multiple of 16, read and written with 16-byte vector
// accesses (conflict free per quarter-warp phase).
template <typename T>
__host__ __device__ constexpr int slot_stride(int n)
{
  if (n % 2 == 1)
    return n * n;
  int units = (n * n * (int)sizeof(T) + 15) / 16;
  if (units % 2 == 0)
    ++units;
  return units * 16 / (int)sizeof(T);
}

// Worst bank conflict (ways) of one quarter-warp phase of 16-byte accesses
// by 8 lanes to 8 consecutive packed slabs of n*n values: lanes whose slab
// starts fall on the same 16-byte slot of a 128-byte bank row collide.
template <typename T>
__host__ __device__ constexpr int packed_slab_conflict(int n)
{
  const int s = n * n * (int)sizeof(T);
  int worst = 0;
  for (int a = 0; a < 8; ++a)
  {
    int c = 0;
    for (int b = 0; b < 8; ++b)
      c += ((a * s) % 128) == ((b * s) % 128) ? 1 : 0;
    worst = c > worst ? c : worst;
  }
  return worst;
}

// Ways of conflict accepted on the slab loads and stores in exchange for
// one bulk copy per tile: the slab accesses are a small part of a tile's
// shared-memory traffic, while a padded layout needs one TMA copy per slab
// (128 copies of 64 bytes per tile of 32 FP32 cells at N = 4).
constexpr int kMaxSlabConflict = 4;

// Shared-memory stride (elements) of one i0 slab (N*N values) of the DOF and
// output stages for tiles whose slabs move by 1D bulk copies.  Packed (N*N:
// the tile is one contiguous bulk copy) when N is odd or when the packed
// slabs' 16-byte accesses conflict at most kMaxSlabConflict ways; else
// every slab is its own bulk copy into its slot (slot_stride).  Tiles whose
// padded slots move by 2D tensor copies use slot_stride throughout.
template <typename T>
__host__ __device__ constexpr int slab_stride(int n)
{
  if (n % 2 == 1 || (n * n * (int)sizeof(T)) % 16 != 0 ||
      packed_slab_conflict<T>(n) <= kMaxSlabConflict)
    return n * n;
  return slot_stride<T>(n);
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
    acc_t<T> acc = acc_mul(A[m * SM], x[0]);
#pragma unroll
    for (int k = 1; k < K; ++k)
      acc = acc_fma(A[m * SM + k * SK], x[k], acc);
    y[m] = acc_val(acc);
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
    acc_t<T> acc = acc_from(y[m]);
#pragma unroll
    for (int k = 0; k < K; ++k)
      acc = acc_fma(A[m * SM + k * SK], x[k], acc);
    y[m] = acc_val(acc);
  }
}

// Even-odd form of y = A x for an M x K matrix with A(M-1-m, K-1-k) =
// SIG * A(m, k): the GLL-to-Gauss tables are such matrices (Phi symmetric,
// Gamma antisymmetric, both nodes and points symmetric about the centre).
// This is the even-odd decomposition of Solomonoff (1992) as described by
// Kopriva, "Implementing Spectral Methods for PDEs" (2009), sec. 3.5: with
// xe_k = x_k + x_{K-1-k} and xo_k = x_k - x_{K-1-k} (k < K/2), each pair of
// outputs m, M-1-m costs K/2 + K/2 products instead of 2K:
//   s = sum_k E(m,k) xe_k (+ C(m) x_mid for odd K),  d = sum_k O(m,k) xo_k,
//   y_m = s + d,  y_{M-1-m} = SIG (s - d),
// with E, O = (A(m,k) +- A(m,K-1-k)) / 2, C(m) = A(m, K/2).  The middle row
// of odd M takes xe (SIG > 0) or xo (SIG < 0) alone.  t is the host-built
// table: rows m <= M/2 of K entries [E (K/2) | C (odd K) | O (K/2)]; the
// middle row keeps A(M/2, k) in the E (and C) slots for SIG > 0, in the O
// slots for SIG < 0.
template <int M, int K>
struct EO
{
  static constexpr int M2 = M / 2, MM = M % 2, K2 = K / 2, KM = K % 2;
  static constexpr int E = 0, C = K2, O = K2 + KM; // column offsets in a row
};

template <int M, int K, int SIG, typename T>
__device__ __forceinline__ void mv_eo(const T* __restrict__ t, const T (&x)[K], T (&y)[M])
{
  using S = EO<M, K>;
  T xe[S::K2], xo[S::K2];
#pragma unroll
  for (int k = 0; k < S::K2; ++k)
  {
    xe[k] = x[k] + x[K - 1 - k];
    xo[k] = x[k] - x[K - 1 - k];
  }
#pragma unroll
  for (int m = 0; m < S::M2; ++m)
  {
    acc_t<T> sa = acc_mul(t[m * K + S::E], xe[0]);
#pragma unroll
    for (int k = 1; k < S::K2; ++k)
      sa = acc_fma(t[m * K + S::E + k], xe[k], sa);
    if constexpr (S::KM)
      sa = acc_fma(t[m * K + S::C], x[S::K2], sa);
    acc_t<T> da = acc_mul(t[m * K + S::O], xo[0]);
#pragma unroll
    for (int k = 1; k < S::K2; ++k)
      da = acc_fma(t[m * K + S::O + k], xo[k], da);
    const T s = acc_val(sa), d = acc_val(da);
    y[m] = s + d;
    y[M - 1 - m] = SIG > 0 ? s - d : d - s;
  }
  if constexpr (S::MM)
  {
    constexpr int m = S::M2;
    if constexpr (SIG > 0)
    {
      acc_t<T> sa = acc_mul(t[m * K + S::E], xe[0]);
#pragma unroll
      for (int k = 1; k < S::K2; ++k)
        sa = acc_fma(t[m * K + S::E + k], xe[k], sa);
      if constexpr (S::KM)
        sa = acc_fma(t[m * K + S::C], x[S::K2], sa);
      y[m] = acc_val(sa);
    }
    else
    {
      acc_t<T> da = acc_mul(t[m * K + S::O], xo[0]);
#pragma unroll
      for (int k = 1; k < S::K2; ++k)
        da = acc_fma(t[m * K + S::O + k], xo[k], da);
      y[m] = acc_val(da);
    }
  }
}

// mv_eo with the symmetry as a run-time flag (neg: SIG < 0), so that one
// copy of the code serves Phi and Gamma.  Same results bit for bit: the
// mirrored output is negated instead of subtracted the other way (IEEE
// subtraction under round-to-nearest is antisymmetric, and so are the
// double-float sums built from it); the middle row of odd M takes the even
// or the odd sum, as in mv_eo.
template <int M, int K, typename T>
__device__ __forceinline__ void mv_eo_rt(const T* __restrict__ t, const T (&x)[K], T (&y)[M],
                                         bool neg)
{
  using S = EO<M, K>;
  T xe[S::K2], xo[S::K2];
#pragma unroll
  for (int k = 0; k < S::K2; ++k)
  {
    xe[k] = x[k] + x[K - 1 - k];
    xo[k] = x[k] - x[K - 1 - k];
  }
#pragma unroll
  for (int m = 0; m < S::M2; ++m)
  {
    acc_t<T> sa = acc_mul(t[m * K + S::E], xe[0]);
#pragma unroll
    for (int k = 1; k < S::K2; ++k)
      sa = acc_fma(t[m * K + S::E + k], xe[k], sa);
    if constexpr (S::KM)
      sa = acc_fma(t[m * K + S::C], x[S::K2], sa);
    acc_t<T> da = acc_mul(t[m * K + S::O], xo[0]);
#pragma unroll
    for (int k = 1; k < S::K2; ++k)
      da = acc_fma(t[m * K + S::O + k], xo[k], da);
    const T s = acc_val(sa), d = acc_val(da);
    y[m] = s + d;
    const T r = s - d;
    y[M - 1 - m] = neg ? -r : r;
  }
  if constexpr (S::MM)
  {
    constexpr int m = S::M2;
    acc_t<T> a;
    if (!neg)
    {
      a = acc_mul(t[m * K + S::E], xe[0]);
#pragma unroll
      for (int k = 1; k < S::K2; ++k)
        a = acc_fma(t[m * K + S::E + k], xe[k], a);
      if constexpr (S::KM)
        a = acc_fma(t[m * K + S::C], x[S::K2], a);
    }
    else
    {
      a = acc_mul(t[m * K + S::O], xo[0]);
#pragma unroll
      for (int k = 1; k < S::K2; ++k)
        a = acc_fma(t[m * K + S::O + k], xo[k], a);
    }
    y[m] = acc_val(a);
  }
}

// Host: the even-odd table of an M x K matrix A(m,k) = a[m*sm + k*sk] (see
// mv_eo), in the arithmetic of S; entries past the used rows are left as
// they are.
template <typename T, typename S>
inline void host_eo_table(const S* a, int M, int K, int sm, int sk, int sig, T* t)
{
  const int M2 = M / 2, MM = M % 2, K2 = K / 2, KM = K % 2;
  auto A = [&](int m, int k) { return a[m * sm + k * sk]; };
  for (int m = 0; m < M2 + MM; ++m)
    for (int k = 0; k < K; ++k)
      t[m * K + k] = T(0);
  for (int m = 0; m < M2; ++m)
  {
    for (int k = 0; k < K2; ++k)
    {
      t[m * K + k] = T((A(m, k) + A(m, K - 1 - k)) / 2);
      t[m * K + K2 + KM + k] = T((A(m, k) - A(m, K - 1 - k)) / 2);
    }
    if (KM)
      t[m * K + K2] = T(A(m, K2));
  }
  if (MM)
  {
    for (int k = 0; k < K2; ++k)
      t[M2 * K + (sig > 0 ? k : K2 + KM + k)] = T(A(M2, k));
    if (KM && sig > 0)
      t[M2 * K + K2] = T(A(M2, K2));
  }
}

// ---------------------------------------------------------------------------
// The streaming main loop shared by every kernel family.  `Tile` provides:
//   kSlabCopies, US      staging of the DOF/output slabs (see slab_stride)
//   work_bytes(p)        bytes of its work buffers for a tile of p.cb cells
//   forward(p, su, sw, ncb)               DOF stage -> work buffers
//   fused(p, sw, ncb, geo, geo_cell0)     quadrature-point pass, in place
//   backward(p, sw, sy, ncb)              work buffers -> output stage
// ---------------------------------------------------------------------------
template <typename T, typename Tile, int N, int Q, int NC>
__host__ __device__ inline CellLayout tile_layout(const CellParams<T>& p)
{
  using ST = storage_t<T>;
  const unsigned bu = (unsigned)p.cb * N * Tile::US * sizeof(ST);
  const unsigned bg =
      (NC > 0 && p.geo_staged == GEO_STAGED) ? (unsigned)p.cb * Q * Q * Q * NC * sizeof(ST) : 0u;
  return CellLayout(bu, bg, Tile::work_bytes(p), Tile::kStages);
}

template <typename T, typename Tile, int N, int Q, int NC>
__device__ __forceinline__ void stream_tiles(const CellParams<T>& p)
{
  using ST = storage_t<T>; // staged values; T is the arithmetic type
  constexpr int N2 = N * N, N3 = N * N * N, Q3NC = Q * Q * Q * NC;
  constexpr int US = Tile::US;
  extern __shared__ __align__(128) unsigned char smem[];
  const int cb = p.cb;
  const bool staged = NC > 0 && p.geo_staged == GEO_STAGED; // affine forms: nothing to stage
  const bool tile_pf = NC > 0 && p.geo_staged == GEO_TILE_L2 && !p.host_io;
  const long long ntiles = (p.ncells + cb - 1) / cb;
  static_assert(Tile::kStages == 2, "the CTA-wide loop keeps two stages");
  const CellLayout L = tile_layout<T, Tile, N, Q, NC>(p);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
  // stage s buffers (selected arithmetically: no local-memory arrays)
  auto su = [&](int s) { return reinterpret_cast<ST*>(smem + (s ? L.u1 : L.u0)); };
  auto sg = [&](int s) { return reinterpret_cast<ST*>(smem + (s ? L.g1 : L.g0)); };
  ST* sy = reinterpret_cast<ST*>(smem + L.y);
  T* sw = reinterpret_cast<T*>(smem + L.w);
  const unsigned bslab = N2 * sizeof(ST);
  const unsigned bu = (unsigned)cb * N3 * sizeof(ST);
  const unsigned bg = staged ? (unsigned)cb * Q3NC * sizeof(ST) : 0u;
  // padded slots by tensor copies (whole boxes, padding included, land)
  const bool tma = Tile::kSlabCopies && p.tma_rows > 0 && (cb * N) % p.tma_rows == 0;
  const unsigned bx = tma ? (unsigned)cb * N * US * sizeof(ST) : bu;
  const int lane = threadIdx.x & 31;
  const bool warp0 = threadIdx.x < 32;
  const TabView<T> tv{p.tab[0], p.tab[1], p.sq, p.sbc, p.tab[2], p.tab[3], p.tab[0]};

  if (threadIdx.x == 0)
  {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();

  // TMA moves full tiles of device memory; host-resident operands and the
  // ragged last tile go through plain vector loads and stores
  auto is_full = [&](long long t) { return !p.host_io && (t + 1) * cb <= p.ncells; };
  // warp 0 only: TMA loads of tile t into stage s
  auto issue = [&](long long t, int s) {
    if (lane == 0)
    {
      fence_proxy_async_smem();
      mbar_arrive_expect_tx(&bar[s], bx + bg);
      if (staged)
        bulk_g2s(sg(s), p.geo + t * cb * Q3NC, bg, &bar[s]);
      if constexpr (!Tile::kSlabCopies)
        bulk_g2s(su(s), p.u + t * cb * N3, bu, &bar[s]);
      else if (tma)
        for (int r = 0; r < cb * N; r += p.tma_rows)
          tma_load_2d(su(s) + r * US, &p.tmu, 0, (int)(t * cb * N) + r, &bar[s]);
    }
    if constexpr (Tile::kSlabCopies)
    {
      if (!tma)
      {
        __syncwarp();
        const long long slab0 = t * cb * N;
        for (int k = lane; k < cb * N; k += 32)
          bulk_g2s(su(s) + k * US, p.u + (slab0 + k) * N2, bslab, &bar[s]);
      }
    }
  };

  long long tile = blockIdx.x;
  if (warp0 && tile < ntiles && is_full(tile))
    issue(tile, 0);

  for (int it = 0; tile < ntiles; tile += gridDim.x, ++it)
  {
    const int s = it & 1;
    const long long next = tile + gridDim.x;
    if (warp0 && next < ntiles && is_full(next))
      issue(next, s ^ 1);
    const bool full = is_full(tile); // loaded and stored by TMA
    // cells in this tile (never more than the stage holds)
    const int ncb = (int)((p.ncells - tile * cb) < cb ? (p.ncells - tile * cb) : cb);
    if (tile_pf) // the fused pass reads this tile's geometry from L2
      prefetch_range_l2(p.geo + tile * cb * Q3NC, (size_t)ncb * Q3NC * sizeof(ST),
                        threadIdx.x, blockDim.x);
    bool ok = true;
    if (full)
    {
      ok = mbar_wait(&bar[s], (unsigned)(it >> 1) & 1u);
    }
    else if (p.host_io && ncb == cb)
    {
      // host-resident full tile: 16-byte vector loads (tile starts and slab
      // lengths are multiples of 16 bytes: cb % 4 == 0 and N*N % 4 == 0
      // whenever slabs are padded)
      using V = uint4;
      constexpr int W = 16 / sizeof(ST);
      const V* gu = reinterpret_cast<const V*>(p.u + tile * cb * N3);
      const int nv = cb * N3 / W;
#pragma unroll 4
      for (int i = threadIdx.x; i < nv; i += blockDim.x)
      {
        const int e = i * W;
        *reinterpret_cast<V*>(su(s) + (e / N2) * US + (e % N2)) = gu[i];
      }
      if (staged)
      {
        const V* gg = reinterpret_cast<const V*>(p.geo + tile * cb * Q3NC);
        V* dg = reinterpret_cast<V*>(sg(s));
#pragma unroll 4
        for (int i = threadIdx.x; i < cb * Q3NC / W; i += blockDim.x)
          dg[i] = gg[i];
      }
    }
    else
    {
      // ragged last tile: plain coalesced loads into the same stage layout
      const long long u0 = tile * cb * N3;
      for (int i = threadIdx.x; i < ncb * N3; i += blockDim.x)
        su(s)[(i / N2) * US + (i % N2)] = p.u[u0 + i];
      if (staged)
      {
        const long long g0 = tile * cb * Q3NC;
        for (int i = threadIdx.x; i < ncb * Q3NC; i += blockDim.x)
          sg(s)[i] = p.geo[g0 + i];
      }
    }
    if (__syncthreads_or(!ok))
    {
      if (threadIdx.x == 0)
        record_fault(FAULT_MBAR_TIMEOUT);
      break;
    }
    Tile::forward(tv, su(s), sw, ncb);
    __syncthreads();
    if (staged)
      Tile::fused(tv, sw, ncb, sg(s), 0);
    else
      Tile::fused(tv, sw, ncb, p.geo, tile * cb, !p.host_io && !tile_pf);
    if (warp0)
      bulk_wait_read0(); // the previous tile's stores have left sy
    __syncthreads();
    Tile::backward(tv, sw, sy, ncb);
    if (full)
    {
      fence_proxy_async_smem();
      __syncthreads();
      if constexpr (!Tile::kSlabCopies)
      {
        if (threadIdx.x == 0)
        {
          bulk_s2g(p.y + tile * cb * N3, sy, bu);
          bulk_commit();
        }
      }
      else if (tma)
      {
        if (threadIdx.x == 0)
        {
          for (int r = 0; r < cb * N; r += p.tma_rows)
            tma_store_2d(&p.tmy, 0, (int)(tile * cb * N) + r, sy + r * US);
          bulk_commit();
        }
      }
      else if (warp0)
      {
        const long long slab0 = tile * cb * N;
        for (int k = lane; k < cb * N; k += 32)
          bulk_s2g(p.y + (slab0 + k) * N2, sy + k * US, bslab);
        bulk_commit();
      }
    }
    else if (p.host_io && ncb == cb)
    {
      __syncthreads();
      using V = uint4;
      constexpr int W = 16 / sizeof(ST);
      V* gy = reinterpret_cast<V*>(p.y + tile * cb * N3);
      const int nv = cb * N3 / W;
#pragma unroll 4
      for (int i = threadIdx.x; i < nv; i += blockDim.x)
      {
        const int e = i * W;
        gy[i] = *reinterpret_cast<const V*>(sy + (e / N2) * US + (e % N2));
      }
    }
    else
    {
      __syncthreads();
      const long long y0 = tile * cb * N3;
      for (int i = threadIdx.x; i < ncb * N3; i += blockDim.x)
        p.y[y0 + i] = sy[(i / N2) * US + (i % N2)];
    }
  }
  if (warp0)
    bulk_wait0();
}

// ---------------------------------------------------------------------------
// CUDA-core tile: slab-merged sum factorization.
//   forward  : one thread per (cell, i0) slab holds u[c][i0][:][:] in
//              registers and contracts axis 2 and axis 1 there, writing
//              B[c][i0][q1][q2] (one column q2 at a time, so the live set is
//              the slab plus two columns);
//   fused    : one thread per (cell, q1, q2) pencil contracts axis 0, applies
//              D or the G transform per point, contracts back;
//   backward : one thread per slab contracts axes 1 and 2 back in registers
//              and writes y[c][i0][:][:].
// Only the fused pass exchanges data across threads, through the B buffers,
// whose slab and cell strides (SQ, SBC, from slab_strides.hpp) keep both
// access patterns free of shared-memory bank conflicts.
// ---------------------------------------------------------------------------
// S lanes share one slab (consecutive lanes of a warp): lane s of the group
// takes the q2 columns s, s+S, ...; the slab loads are shared-memory
// broadcasts, and the backward partial sums are reduced with shuffles.
template <typename T>
__host__ __device__ constexpr int slab_lanes()
{
  return sizeof(T) == 4 ? 2 : 1; // FP32: more busy lanes; FP64: pipe-bound
}

// The share of one tile's work a thread takes in the tile passes: cells
// [c0, c1) of a tile, work item tid, tid + nthr, ...  The whole CTA
// ({ncb, 0, ncb, threadIdx.x, blockDim.x}) or one warp ({cb, its cells,
// lane, 32}).  ncb sets the spacing of the work buffers (ncb cells each):
// warps that run ahead of one another use the stage's capacity cb there, so
// that a warp's regions stay the same from tile to tile (a ragged tile's
// smaller spacing would move them onto cells another warp still reads).
struct Part
{
  int ncb, c0, c1, tid, nthr;
};

__device__ __forceinline__ Part cta_part(int ncb)
{
  return Part{ncb, 0, ncb, (int)threadIdx.x, (int)blockDim.x};
}

// EVOD: even-odd contractions (mv_eo) for tables with the GLL-to-Gauss
// symmetry; one lane per slab, exact semantics.
// SLOTS: the DOF/output slabs always sit in conflict-free slots
// (slot_stride), moved by 2D tensor copies when the launch has tensor maps
// (the single-mesh kernels); else slab_stride's rule (the batch kernels).
template <typename T, int N, int Q, int OP, int SEM, int LANES = slab_lanes<T>(),
          bool EVOD = false, bool SLOTS = false>
struct SlabTile
{
  using ST = storage_t<T>; // staged u, y and geometry; T is the arithmetic
  static constexpr int S = LANES;
  static constexpr int US = SLOTS ? slot_stride<ST>(N) : slab_stride<ST>(N);
  // padded slots: one tensor copy per tile (or one bulk copy per slab);
  // packed slabs: one bulk copy per tile
  static constexpr bool kSlabCopies = (US != N * N);
  // slabs of whole 16-byte vectors: vector loads and stores (16-byte
  // aligned slots, packed or padded)
  static constexpr bool kVecSlab = (N * N * sizeof(ST)) % 16 == 0;
  static constexpr int N2 = N * N, Q2 = Q * Q, Q3 = Q * Q * Q;
  // the gradient passes: stiffness and Helmholtz (the latter exact only)
  static constexpr bool kGrad = (op_base(OP) != OP_MASS);
  // affine forms: per-cell geometry, quadrature weights in the backward
  // tables (PB, DB), which then differ from the forward ones in every form
  static constexpr bool kAffine = op_affine(OP);
  static_assert(OP != OP_HELMHOLTZ || SEM == SEM_EXACT, "Helmholtz: exact semantics only");
  static_assert(!kAffine || SEM == SEM_EXACT, "affine forms: exact semantics only");
  static_assert(!EVOD || (SEM == SEM_EXACT && LANES <= 2), "even-odd: exact, one or two lanes per slab");
  // Streaming loop: work split by warps (stream_tiles_warp) where its extra
  // live state costs no occupancy -- FP32 and N <= 4; the register-heavy
  // FP64 and double-float tiles of higher degree keep the CTA-wide loop
  // (stream_tiles).  The host's tile model (lane_efficiency) follows the
  // same rule.
  static constexpr bool kWarpSplit = sizeof(T) == 4 || N <= 4;
  // double-float even-odd stiffness: the quadrature-point pass loops over
  // its three forward and three backward contractions with one copy of the
  // code (its unrolled double-float form overflows the instruction cache)
  static constexpr bool kCompactFused =
      std::is_same<T, df64>::value && EVOD && OP == OP_STIFFNESS && SEM == SEM_EXACT;
  // TMA stages.  The warp-split loop takes any count; a third stage (two
  // tiles in flight ahead of the one computed) measured slower than two:
  // its shared memory costs more occupancy than the deeper prefetch gains.
  // FP32 tiles from N = 6 keep one: their work buffers fill most of the
  // shared memory, and one stage leaves room for larger tiles and more L1
  // (P=6: 99.6 against 91.3 GDoF/s at the same tile).  The stage is
  // refilled as soon as every warp is done with it (after the
  // quadrature-point pass), behind the backward pass.
  static constexpr int kStages = (sizeof(T) == 4 && N >= 6) ? 1 : 2;
  static constexpr int NBUF =
      (op_base(OP) == OP_MASS) ? 1 : ((SEM == SEM_EXACT) ? 3 : 2);
  // work-buffer strides (slab_strides.hpp): compile-time, so every work
  // buffer access takes an immediate offset; the host sets the same values
  // in the launch parameters (p.sq, p.sbc) to size the tile
  static constexpr int SQ = slab_strides(N, Q, (int)sizeof(T), LANES).sq;
  static constexpr int SBC = slab_strides(N, Q, (int)sizeof(T), LANES).sbc;
  static_assert(SQ >= Q * Q && SBC >= N * SQ, "no stride table entry for this slab variant");
  // tables: forward A(q,i) = tab[q + i*Q]; backward exact A(i,q) = tab[q + i*Q],
  // reference A(i,q) = tab[i + q*Q] (the forward table reused, Q == N)
  static constexpr int BSM = (SEM == SEM_EXACT) ? Q : 1;
  static constexpr int BSK = (SEM == SEM_EXACT) ? 1 : Q;
  static constexpr int QS = (Q + S - 1) / S; // q2 columns per lane (max)
  // unroll the q2 loop only while the unrolled body stays small
  static constexpr int UNR = (N * N * QS * NBUF <= 1200) ? QS : 1;
  // lane-dependent axis-2 table columns preloaded into registers
  static constexpr bool PRE = (S > 1) && (UNR == QS);

  static __host__ __device__ unsigned work_bytes(const CellParams<T>& p)
  {
    return (unsigned)NBUF * p.cb * p.sbc * sizeof(T);
  }

  static __device__ __forceinline__ void load_slab(const ST* __restrict__ src,
                                                   T (&x)[N2])
  {
    if constexpr (kVecSlab)
    {
      using V = typename std::conditional<sizeof(ST) == 4, float4, double2>::type;
      constexpr int W = 16 / sizeof(ST);
#pragma unroll
      for (int k = 0; k < N2 / W; ++k)
      {
        const V v = reinterpret_cast<const V*>(src)[k];
        const ST* e = reinterpret_cast<const ST*>(&v);
#pragma unroll
        for (int j = 0; j < W; ++j)
          x[k * W + j] = from_storage<T>(e[j]);
      }
    }
    else
    {
#pragma unroll
      for (int k = 0; k < N2; ++k)
        x[k] = from_storage<T>(src[k]);
    }
  }

  static __device__ __forceinline__ void store_slab(ST* __restrict__ dst,
                                                    const T (&x)[N2])
  {
    if constexpr (kVecSlab)
    {
      using V = typename std::conditional<sizeof(ST) == 4, float4, double2>::type;
      constexpr int W = 16 / sizeof(ST);
#pragma unroll
      for (int k = 0; k < N2 / W; ++k)
      {
        V v;
        ST* e = reinterpret_cast<ST*>(&v);
#pragma unroll
        for (int j = 0; j < W; ++j)
          e[j] = to_storage<T>(x[k * W + j]);
        reinterpret_cast<V*>(dst)[k] = v;
      }
    }
    else
    {
#pragma unroll
      for (int k = 0; k < N2; ++k)
        dst[k] = to_storage<T>(x[k]);
    }
  }

  // One pencil contraction along axis 0: forward (N -> Q) and backward
  // (Q -> N); SIG is the table's symmetry (+1 Phi, -1 Gamma) for even-odd.
  template <int SIG>
  static __device__ __forceinline__ void fwd(const T* __restrict__ t, const T (&x)[N], T (&y)[Q])
  {
    if constexpr (EVOD)
      mv_eo<Q, N, SIG>(t, x, y);
    else
      mv<Q, N, 1, Q>(t, x, y);
  }
  template <int SIG>
  static __device__ __forceinline__ void bwd(const T* __restrict__ t, const T (&x)[Q], T (&y)[N])
  {
    if constexpr (EVOD)
      mv_eo<N, Q, SIG>(t, x, y);
    else
      mv<N, Q, BSM, BSK>(t, x, y);
  }

  // Even-odd forward: the columns q2 and Q-1-q2 of a pair come from the
  // even and odd parts of the slab's rows.
  static __device__ __forceinline__ void forward_eo(const TabView<T>& p,
                                                    const ST* __restrict__ su,
                                                    T* __restrict__ sw, const Part& w)
  {
    using E = EO<Q, N>; // forward tables: Q x N
    const T* __restrict__ PF = p.P;
    const T* __restrict__ DF = p.D;
    const int bstride = w.ncb * SBC;
    for (int sl = w.c0 * N + w.tid; sl < w.c1 * N; sl += w.nthr)
    {
      const int c = sl / N, i0 = sl - c * N;
      T x[N2];
      load_slab(su + sl * US, x);
      T xe[N][E::K2], xo[N][E::K2];
#pragma unroll
      for (int i1 = 0; i1 < N; ++i1)
#pragma unroll
        for (int k = 0; k < E::K2; ++k)
        {
          xe[i1][k] = x[i1 * N + k] + x[i1 * N + N - 1 - k];
          xo[i1][k] = x[i1 * N + k] - x[i1 * N + N - 1 - k];
        }
      T* b0 = sw + c * SBC + i0 * SQ;
      T* b1 = b0 + bstride;
      T* b2 = b1 + bstride;
      // axis 1 of one column: AA, AG, BA
      auto emit = [&](int q2, const T(&a)[N], const T(&g)[N]) {
        T o[Q];
        mv_eo<Q, N, 1>(PF, a, o);
#pragma unroll
        for (int q1 = 0; q1 < Q; ++q1)
          b0[q1 * Q + q2] = o[q1];
        if constexpr (kGrad)
        {
          mv_eo<Q, N, -1>(DF, a, o);
#pragma unroll
          for (int q1 = 0; q1 < Q; ++q1)
            b1[q1 * Q + q2] = o[q1];
          mv_eo<Q, N, 1>(PF, g, o);
#pragma unroll
          for (int q1 = 0; q1 < Q; ++q1)
            b2[q1 * Q + q2] = o[q1];
        }
      };
      // even and odd sums of row i1 against row j of an even-odd table
      auto sums = [&](const T* __restrict__ t, int j, int i1, T& s, T& d) {
        acc_t<T> sa = acc_mul(t[j * N + E::E], xe[i1][0]);
#pragma unroll
        for (int k = 1; k < E::K2; ++k)
          sa = acc_fma(t[j * N + E::E + k], xe[i1][k], sa);
        if constexpr (E::KM)
          sa = acc_fma(t[j * N + E::C], x[i1 * N + E::K2], sa);
        acc_t<T> da = acc_mul(t[j * N + E::O], xo[i1][0]);
#pragma unroll
        for (int k = 1; k < E::K2; ++k)
          da = acc_fma(t[j * N + E::O + k], xo[i1][k], da);
        s = acc_val(sa);
        d = acc_val(da);
      };
#pragma unroll
      for (int j = 0; j < E::M2; ++j) // column pair (j, Q-1-j)
      {
        T a0[N], a1[N], g0[N], g1[N];
#pragma unroll
        for (int i1 = 0; i1 < N; ++i1)
        {
          T s, d;
          sums(PF, j, i1, s, d);
          a0[i1] = s + d;
          a1[i1] = s - d;
          if constexpr (kGrad)
          {
            sums(DF, j, i1, s, d);
            g0[i1] = s + d;
            g1[i1] = d - s;
          }
        }
        emit(j, a0, g0);
        emit(Q - 1 - j, a1, g1);
      }
      if constexpr (E::MM) // middle column of odd Q
      {
        constexpr int j = E::M2;
        T a[N], g[N];
#pragma unroll
        for (int i1 = 0; i1 < N; ++i1)
        {
          acc_t<T> sa = acc_mul(PF[j * N + E::E], xe[i1][0]);
#pragma unroll
          for (int k = 1; k < E::K2; ++k)
            sa = acc_fma(PF[j * N + E::E + k], xe[i1][k], sa);
          if constexpr (E::KM)
            sa = acc_fma(PF[j * N + E::C], x[i1 * N + E::K2], sa);
          a[i1] = acc_val(sa);
          if constexpr (kGrad)
          {
            acc_t<T> da = acc_mul(DF[j * N + E::O], xo[i1][0]);
#pragma unroll
            for (int k = 1; k < E::K2; ++k)
              da = acc_fma(DF[j * N + E::O + k], xo[i1][k], da);
            g[i1] = acc_val(da);
          }
        }
        emit(j, a, g);
      }
    }
  }

  // Even-odd forward with S lanes per slab: lane s takes the column pairs
  // j = s, s+S, ... (the middle column of odd Q goes to the lane with fewer
  // pairs).  The pair loop and the loop over a pair's two columns are not
  // unrolled: one copy of the (large, double-float) column code serves every
  // column of a lane, which keeps the kernel within the instruction cache.
  // A pair's table rows are read from the parameter block at the top of its
  // iteration.
  static __device__ __forceinline__ void forward_eo2(const TabView<T>& p,
                                                     const ST* __restrict__ su,
                                                     T* __restrict__ sw, const Part& w)
  {
    using E = EO<Q, N>; // forward tables: Q x N
    constexpr int JL = (E::M2 + S - 1) / S > 0 ? (E::M2 + S - 1) / S : 1; // pairs per lane
    constexpr int MIDLANE = E::M2 % S;
    const T* __restrict__ PF = p.P;
    const T* __restrict__ DF = p.D;
    const int bstride = w.ncb * SBC;
    const int ls = threadIdx.x % S;
    for (int ts = w.c0 * N * S + w.tid; ts < w.c1 * N * S; ts += w.nthr)
    {
      const int sl = ts / S;
      const int c = sl / N, i0 = sl - c * N;
      T x[N2];
      load_slab(su + sl * US, x);
      T xe[N][E::K2 > 0 ? E::K2 : 1], xo[N][E::K2 > 0 ? E::K2 : 1];
#pragma unroll
      for (int i1 = 0; i1 < N; ++i1)
#pragma unroll
        for (int k = 0; k < E::K2; ++k)
        {
          xe[i1][k] = x[i1 * N + k] + x[i1 * N + N - 1 - k];
          xo[i1][k] = x[i1 * N + k] - x[i1 * N + N - 1 - k];
        }
      T* b0 = sw + c * SBC + i0 * SQ;
      T* b1 = b0 + bstride;
      T* b2 = b1 + bstride;
      // axis 1 of one column: AA, AG, BA (the same tables in every lane)
      auto emit = [&](int q2, const T(&a)[N], const T(&g)[N]) {
        T o[Q];
        mv_eo<Q, N, 1>(PF, a, o);
#pragma unroll
        for (int q1 = 0; q1 < Q; ++q1)
          b0[q1 * Q + q2] = o[q1];
        if constexpr (kGrad)
        {
          mv_eo<Q, N, -1>(DF, a, o);
#pragma unroll
          for (int q1 = 0; q1 < Q; ++q1)
            b1[q1 * Q + q2] = o[q1];
          mv_eo<Q, N, 1>(PF, g, o);
#pragma unroll
          for (int q1 = 0; q1 < Q; ++q1)
            b2[q1 * Q + q2] = o[q1];
        }
      };
      // even and odd sums of row i1 against one even-odd table row
      auto sums = [&](const T(&t)[N], int i1, T& s, T& d) {
        acc_t<T> sa = acc_mul(t[E::E], xe[i1][0]);
#pragma unroll
        for (int k = 1; k < E::K2; ++k)
          sa = acc_fma(t[E::E + k], xe[i1][k], sa);
        if constexpr (E::KM)
          sa = acc_fma(t[E::C], x[i1 * N + E::K2], sa);
        acc_t<T> da = acc_mul(t[E::O], xo[i1][0]);
#pragma unroll
        for (int k = 1; k < E::K2; ++k)
          da = acc_fma(t[E::O + k], xo[i1][k], da);
        s = acc_val(sa);
        d = acc_val(da);
      };
#pragma unroll 1
      for (int jj = 0; jj < JL; ++jj) // this lane's column pairs (j, Q-1-j)
      {
        const int j = ls + jj * S;
        if (j >= E::M2)
          break;
        T tp[N], td[N];
#pragma unroll
        for (int k = 0; k < N; ++k)
        {
          tp[k] = PF[j * N + k];
          if constexpr (kGrad)
            td[k] = DF[j * N + k];
        }
        T a0[N], a1[N], g0[N], g1[N];
#pragma unroll
        for (int i1 = 0; i1 < N; ++i1)
        {
          T s, d;
          sums(tp, i1, s, d);
          a0[i1] = s + d;
          a1[i1] = s - d;
          if constexpr (kGrad)
          {
            sums(td, i1, s, d);
            g0[i1] = s + d;
            g1[i1] = d - s;
          }
        }
#pragma unroll 1
        for (int h = 0; h < 2; ++h) // column j, then column Q-1-j
        {
          T a[N], g[N];
#pragma unroll
          for (int i1 = 0; i1 < N; ++i1)
          {
            a[i1] = h ? a1[i1] : a0[i1];
            if constexpr (kGrad)
              g[i1] = h ? g1[i1] : g0[i1];
          }
          emit(h ? Q - 1 - j : j, a, g);
        }
      }
      if constexpr (E::MM) // middle column of odd Q
      {
        if (ls == MIDLANE)
        {
          constexpr int j = E::M2;
          T a[N], g[N];
#pragma unroll
          for (int i1 = 0; i1 < N; ++i1)
          {
            acc_t<T> sa = acc_mul(PF[j * N + E::E], xe[i1][0]);
#pragma unroll
            for (int k = 1; k < E::K2; ++k)
              sa = acc_fma(PF[j * N + E::E + k], xe[i1][k], sa);
            if constexpr (E::KM)
              sa = acc_fma(PF[j * N + E::C], x[i1 * N + E::K2], sa);
            a[i1] = acc_val(sa);
            if constexpr (kGrad)
            {
              acc_t<T> da = acc_mul(DF[j * N + E::O], xo[i1][0]);
#pragma unroll
              for (int k = 1; k < E::K2; ++k)
                da = acc_fma(DF[j * N + E::O + k], xo[i1][k], da);
              g[i1] = acc_val(da);
            }
          }
          emit(j, a, g);
        }
      }
    }
  }

  static __device__ __forceinline__ void forward(const TabView<T>& p,
                                                 const ST* __restrict__ su,
                                                 T* __restrict__ sw, int ncb)
  {
    forward(p, su, sw, cta_part(ncb));
  }

  static __device__ __forceinline__ void forward(const TabView<T>& p,
                                                 const ST* __restrict__ su,
                                                 T* __restrict__ sw, const Part& w)
  {
    if constexpr (EVOD && S == 1)
    {
      forward_eo(p, su, sw, w);
      return;
    }
    else if constexpr (EVOD)
    {
      forward_eo2(p, su, sw, w);
      return;
    }
    const T* __restrict__ P = p.P;
    const T* __restrict__ D = p.D;
    const int bstride = w.ncb * SBC;
    // With S lanes per slab the q2 columns of a lane depend on the lane, so
    // their table entries are not compile-time constants: load them into
    // registers once per call (lane_s == threadIdx.x % S for every slab of
    // this thread, since blockDim.x is a multiple of 32).
    T pc[PRE ? QS : 1][PRE ? N : 1], dc[PRE ? QS : 1][PRE ? N : 1];
    if constexpr (PRE)
    {
      const int ls = threadIdx.x % S;
#pragma unroll
      for (int jq = 0; jq < QS; ++jq)
#pragma unroll
        for (int i2 = 0; i2 < N; ++i2)
        {
          const int q2 = ls + jq * S;
          pc[jq][i2] = q2 < Q ? P[q2 + i2 * Q] : T(0);
          dc[jq][i2] = q2 < Q ? D[q2 + i2 * Q] : T(0);
        }
    }
    for (int ts = w.c0 * N * S + w.tid; ts < w.c1 * N * S; ts += w.nthr)
    {
      const int sl = ts / S, lane_s = ts - sl * S;
      const int c = sl / N, i0 = sl - c * N;
      T x[N2];
      load_slab(su + sl * US, x);
      T* b0 = sw + c * SBC + i0 * SQ;
      T* b1 = b0 + bstride;
      T* b2 = b1 + bstride;
#pragma unroll UNR
      for (int jq = 0; jq < QS; ++jq)
      {
        const int q2 = lane_s + jq * S;
        if (S > 1 && q2 >= Q)
          break;
        T a[N], g[N];
        // axis-2 table entries Phi(q2, i2), Gamma(q2, i2) of this column
        auto pq = [&](int i2) { if constexpr (PRE) return pc[jq][i2]; else return P[q2 + i2 * Q]; };
        auto dq = [&](int i2) { if constexpr (PRE) return dc[jq][i2]; else return D[q2 + i2 * Q]; };
#pragma unroll
        for (int i1 = 0; i1 < N; ++i1)
        {
          acc_t<T> acc = acc_mul(pq(0), x[i1 * N]);
#pragma unroll
          for (int i2 = 1; i2 < N; ++i2)
            acc = acc_fma(pq(i2), x[i1 * N + i2], acc);
          a[i1] = acc_val(acc);
          if constexpr (kGrad && SEM == SEM_EXACT)
          {
            acc_t<T> gcc = acc_mul(dq(0), x[i1 * N]);
#pragma unroll
            for (int i2 = 1; i2 < N; ++i2)
              gcc = acc_fma(dq(i2), x[i1 * N + i2], gcc);
            g[i1] = acc_val(gcc);
          }
        }
#pragma unroll
        for (int q1 = 0; q1 < Q; ++q1)
        {
          acc_t<T> o0 = acc_mul(P[q1], a[0]);
#pragma unroll
          for (int i1 = 1; i1 < N; ++i1)
            o0 = acc_fma(P[q1 + i1 * Q], a[i1], o0);
          b0[q1 * Q + q2] = acc_val(o0); // AA = Phi_1 Phi_2 u
          if constexpr (kGrad)
          {
            acc_t<T> o1 = acc_mul(D[q1], a[0]);
#pragma unroll
            for (int i1 = 1; i1 < N; ++i1)
              o1 = acc_fma(D[q1 + i1 * Q], a[i1], o1);
            b1[q1 * Q + q2] = acc_val(o1); // AG = Gamma_1 Phi_2 u
            if constexpr (SEM == SEM_EXACT)
            {
              acc_t<T> o2 = acc_mul(P[q1], g[0]);
#pragma unroll
              for (int i1 = 1; i1 < N; ++i1)
                o2 = acc_fma(P[q1 + i1 * Q], g[i1], o2);
              b2[q1 * Q + q2] = acc_val(o2); // BA = Phi_1 Gamma_2 u
            }
          }
        }
      }
    }
  }

  static __device__ __forceinline__ void fused(const TabView<T>& p,
                                               T* __restrict__ sw, int ncb,
                                               const ST* __restrict__ geo,
                                               long long geo_cell0, bool l2pf = false)
  {
    fused(p, sw, cta_part(ncb), geo, geo_cell0, l2pf);
  }

  // l2pf: the per-point geometry is read from device memory; each thread
  // asks L2 for its next pencil's geometry lines (one per point) while it
  // computes this pencil, so those loads wait on L2 instead of HBM.
  static __device__ __forceinline__ void fused(const TabView<T>& p,
                                               T* __restrict__ sw, const Part& w,
                                               const ST* __restrict__ geo,
                                               long long geo_cell0, bool l2pf = false)
  {
    const T* __restrict__ P = p.P;
    const T* __restrict__ D = p.D;
    // backward tables: the even-odd or weighted ones, else the forward
    // ones transposed
    const T* __restrict__ PB = (EVOD || kAffine) ? p.PB : p.P;
    const T* __restrict__ DB = (EVOD || kAffine) ? p.DB : p.D;
    const int bstride = w.ncb * SBC;
    for (int t = w.c0 * Q2 + w.tid; t < w.c1 * Q2; t += w.nthr)
    {
      const int c = t / Q2, r = t - c * Q2;
      T* b0 = sw + c * SBC + r;
      T* b1 = b0 + bstride;
      T* b2 = b1 + bstride;
      constexpr int sq = SQ;
      if constexpr (geo_nc(OP) > 0)
      {
        const int tn = t + w.nthr; // this thread's next pencil, if any
        if (l2pf && tn < w.c1 * Q2)
        {
          const int cn = tn / Q2, rn = tn - cn * Q2;
          const ST* gn = geo + ((geo_cell0 + cn) * Q3 + rn) * geo_nc(OP);
#pragma unroll
          for (int q = 0; q < Q; ++q)
            prefetch_l2(gn + (long long)q * Q2 * geo_nc(OP));
        }
      }
      if constexpr (OP == OP_MASS_AFFINE)
      {
        // detJ scales the pencil's N inputs (the weights are in PB)
        const T dj = from_storage<T>(geo[geo_cell0 + c]);
        T x[N], v[Q];
#pragma unroll
        for (int k = 0; k < N; ++k)
          x[k] = b0[k * sq] * dj;
        fwd<1>(P, x, v);
        bwd<1>(PB, v, x);
#pragma unroll
        for (int k = 0; k < N; ++k)
          b0[k * sq] = x[k];
      }
      else if constexpr (OP == OP_MASS)
      {
        const ST* dw = geo + (geo_cell0 + c) * Q3 + r;
        T x[N], v[Q];
#pragma unroll
        for (int k = 0; k < N; ++k)
          x[k] = b0[k * sq];
        fwd<1>(P, x, v);
#pragma unroll
        for (int q = 0; q < Q; ++q)
          v[q] *= from_storage<T>(dw[q * Q2]);
        bwd<1>(PB, v, x);
#pragma unroll
        for (int k = 0; k < N; ++k)
          b0[k * sq] = x[k];
      }
      else
      {
        constexpr int NCG = geo_nc(OP);
        const ST* G = geo + ((geo_cell0 + c) * Q3 + r) * NCG; // unused by affine forms
        T fx[Q], fy[Q], fz[Q];
        T fm[OP == OP_HELMHOLTZ ? Q : 1];
        if constexpr (kCompactFused)
        {
          // one copy of the contraction for d/dx (Gamma on axis 0, input
          // b0), d/dy (b1) and d/dz (b2); the outputs rotate into fx, fy, fz
#pragma unroll
          for (int q = 0; q < Q; ++q)
            fy[q] = fz[q] = T(0);
#pragma unroll 1
          for (int dir = 0; dir < 3; ++dir)
          {
            const T* src = dir == 0 ? b0 : (dir == 1 ? b1 : b2);
            T x[N], o[Q];
#pragma unroll
            for (int k = 0; k < N; ++k)
              x[k] = src[k * sq];
            mv_eo_rt<Q, N>(dir == 0 ? D : P, x, o, dir == 0);
#pragma unroll
            for (int q = 0; q < Q; ++q)
            {
              fx[q] = fy[q];
              fy[q] = fz[q];
              fz[q] = o[q];
            }
          }
        }
        else
        {
          T xa[N], xg[N];
#pragma unroll
          for (int k = 0; k < N; ++k)
          {
            xa[k] = b0[k * sq];
            xg[k] = b1[k * sq];
          }
          fwd<-1>(D, xa, fx); // d/dx: Gamma on axis 0
          fwd<1>(P, xg, fy);  // d/dy: Gamma was applied on axis 1
          if constexpr (OP == OP_HELMHOLTZ)
            fwd<1>(P, xa, fm); // the value u at the points (mass term)
          if constexpr (SEM == SEM_EXACT)
          {
            T xb[N];
#pragma unroll
            for (int k = 0; k < N; ++k)
              xb[k] = b2[k * sq];
            fwd<1>(P, xb, fz); // d/dz: Gamma was applied on axis 2
          }
          else
          {
            fwd<1>(P, xa, fz); // reference: W_z carries no derivative
          }
        }
        // G transform (src/stiffness.hpp:14-29), [zz,yz,xz,yy,xy,xx], read
        // as three 8/16-byte pairs (Helmholtz: a fourth pair holds the mass
        // factor; affine: the cell's one G for every point)
        using V2 = typename std::conditional<sizeof(ST) == 4, float2, double2>::type;
        V2 a01{}, a23{}, a45{};
        if constexpr (kAffine)
        {
          const V2* ga = reinterpret_cast<const V2*>(geo + (geo_cell0 + c) * cell_nc(OP));
          a01 = ga[0];
          a23 = ga[1];
          a45 = ga[2];
        }
#pragma unroll
        for (int q = 0; q < Q; ++q)
        {
          const V2* g2 = reinterpret_cast<const V2*>(G + (long long)q * Q2 * NCG);
          const V2 g01 = kAffine ? a01 : g2[0], g23 = kAffine ? a23 : g2[1],
                   g45 = kAffine ? a45 : g2[2];
          if constexpr (OP == OP_HELMHOLTZ)
            fm[q] *= from_storage<T>(g2[3].x);
          const T zz = from_storage<T>(g01.x), yz = from_storage<T>(g01.y),
                  xz = from_storage<T>(g23.x), yy = from_storage<T>(g23.y),
                  xy = from_storage<T>(g45.x), xx = from_storage<T>(g45.y);
          const T w0 = fx[q], w1 = fy[q], w2 = fz[q];
          if constexpr (SEM == SEM_EXACT)
          {
            fx[q] = xx * w0 + xy * w1 + xz * w2;
            fy[q] = xy * w0 + yy * w1 + yz * w2;
          }
          fz[q] = xz * w0 + yz * w1 + zz * w2;
        }
        T o[N];
        if constexpr (kCompactFused)
        {
          // one copy of the contraction for x (Gamma^T, into b0), y (b1)
          // and z (b2)
#pragma unroll 1
          for (int dir = 0; dir < 3; ++dir)
          {
            T in[Q];
#pragma unroll
            for (int q = 0; q < Q; ++q)
            {
              in[q] = fx[q];
              fx[q] = fy[q];
              fy[q] = fz[q];
            }
            mv_eo_rt<N, Q>(dir == 0 ? DB : PB, in, o, dir == 0);
            T* dst = dir == 0 ? b0 : (dir == 1 ? b1 : b2);
#pragma unroll
            for (int k = 0; k < N; ++k)
              dst[k * sq] = o[k];
          }
        }
        else if constexpr (SEM == SEM_EXACT)
        {
          bwd<-1>(DB, fx, o);
          if constexpr (OP == OP_HELMHOLTZ && EVOD)
          {
            T om[N];
            bwd<1>(PB, fm, om); // Phi_0^T (m u): same chain as x
#pragma unroll
            for (int k = 0; k < N; ++k)
              o[k] += om[k];
          }
          else if constexpr (OP == OP_HELMHOLTZ)
            mv_acc<N, Q, BSM, BSK>(P, fm, o); // Phi_0^T (m u): same chain as x
#pragma unroll
          for (int k = 0; k < N; ++k)
            b0[k * sq] = o[k];
          bwd<1>(PB, fy, o);
#pragma unroll
          for (int k = 0; k < N; ++k)
            b1[k * sq] = o[k];
          bwd<1>(PB, fz, o);
#pragma unroll
          for (int k = 0; k < N; ++k)
            b2[k * sq] = o[k];
        }
        else
        {
          bwd<1>(PB, fz, o); // (Phi, Phi, Gamma): axis 0 is Phi
#pragma unroll
          for (int k = 0; k < N; ++k)
            b0[k * sq] = o[k];
        }
      }
    }
  }

  // Even-odd backward: axis 1 back per column with mv_eo; axis 2 back over
  // the column pairs (j, Q-1-j) into accumulators of the output pairs
  // (i2, N-1-i2): A = s_Phi + d_Gamma, B = d_Phi + s_Gamma, then
  // y(i2) = A + B and y(N-1-i2) = A - B (see mv_eo for s and d).
  static __device__ __forceinline__ void backward_eo(const TabView<T>& p,
                                                     const T* __restrict__ sw,
                                                     ST* __restrict__ sy, const Part& w)
  {
    using E = EO<N, Q>; // backward tables: N x Q
    const T* __restrict__ PB = p.PB;
    const T* __restrict__ DB = p.DB;
    const int bstride = w.ncb * SBC;
    for (int sl = w.c0 * N + w.tid; sl < w.c1 * N; sl += w.nthr)
    {
      const int c = sl / N, i0 = sl - c * N;
      const T* b0 = sw + c * SBC + i0 * SQ;
      const T* b1 = b0 + bstride;
      const T* b2 = b1 + bstride;
      // accumulators (double-float: lazily renormalised, see df64acc)
      acc_t<T> A[N][E::M2 > 0 ? E::M2 : 1], B[N][E::M2 > 0 ? E::M2 : 1], Mid[N];
#pragma unroll
      for (int i1 = 0; i1 < N; ++i1)
      {
#pragma unroll
        for (int i2 = 0; i2 < E::M2; ++i2)
          A[i1][i2] = B[i1][i2] = acc_zero<T>();
        Mid[i1] = acc_zero<T>();
      }
      // axis 1 back of column q2: u1 = Phi^T X (+ Gamma^T Y), u2 = Phi^T Z
      auto column = [&](int q2, T(&u1)[N], T(&u2)[N]) {
        T X[Q];
#pragma unroll
        for (int q1 = 0; q1 < Q; ++q1)
          X[q1] = b0[q1 * Q + q2];
        mv_eo<N, Q, 1>(PB, X, u1);
        if constexpr (kGrad)
        {
          T Y[Q], Z[Q], t[N];
#pragma unroll
          for (int q1 = 0; q1 < Q; ++q1)
          {
            Y[q1] = b1[q1 * Q + q2];
            Z[q1] = b2[q1 * Q + q2];
          }
          mv_eo<N, Q, -1>(DB, Y, t);
#pragma unroll
          for (int i = 0; i < N; ++i)
            u1[i] += t[i];
          mv_eo<N, Q, 1>(PB, Z, u2);
        }
      };
#pragma unroll
      for (int j = 0; j < E::K2; ++j) // column pair (j, Q-1-j)
      {
        T u1a[N], u2a[N], u1b[N], u2b[N];
        column(j, u1a, u2a);
        column(Q - 1 - j, u1b, u2b);
#pragma unroll
        for (int i1 = 0; i1 < N; ++i1)
        {
          const T e1 = u1a[i1] + u1b[i1], o1 = u1a[i1] - u1b[i1];
#pragma unroll
          for (int i2 = 0; i2 < E::M2; ++i2)
          {
            A[i1][i2] = acc_fma(PB[i2 * Q + E::E + j], e1, A[i1][i2]);
            B[i1][i2] = acc_fma(PB[i2 * Q + E::O + j], o1, B[i1][i2]);
          }
          if constexpr (E::MM)
            Mid[i1] = acc_fma(PB[E::M2 * Q + E::E + j], e1, Mid[i1]);
          if constexpr (kGrad)
          {
            const T e2 = u2a[i1] + u2b[i1], o2 = u2a[i1] - u2b[i1];
#pragma unroll
            for (int i2 = 0; i2 < E::M2; ++i2)
            {
              A[i1][i2] = acc_fma(DB[i2 * Q + E::O + j], o2, A[i1][i2]); // d_Gamma
              B[i1][i2] = acc_fma(DB[i2 * Q + E::E + j], e2, B[i1][i2]); // s_Gamma
            }
            if constexpr (E::MM)
              Mid[i1] = acc_fma(DB[E::M2 * Q + E::O + j], o2, Mid[i1]);
          }
        }
      }
      if constexpr (E::KM) // middle column of odd Q: the C entries
      {
        T u1[N], u2[N];
        column(E::K2, u1, u2);
#pragma unroll
        for (int i1 = 0; i1 < N; ++i1)
        {
#pragma unroll
          for (int i2 = 0; i2 < E::M2; ++i2)
          {
            A[i1][i2] = acc_fma(PB[i2 * Q + E::C], u1[i1], A[i1][i2]); // s_Phi
            if constexpr (kGrad)
              B[i1][i2] = acc_fma(DB[i2 * Q + E::C], u2[i1], B[i1][i2]); // s_Gamma
          }
          if constexpr (E::MM) // Gamma^T vanishes at the centre
            Mid[i1] = acc_fma(PB[E::M2 * Q + E::C], u1[i1], Mid[i1]);
        }
      }
      T y[N2];
#pragma unroll
      for (int i1 = 0; i1 < N; ++i1)
      {
#pragma unroll
        for (int i2 = 0; i2 < E::M2; ++i2)
        {
          const T av = acc_val(A[i1][i2]), bv = acc_val(B[i1][i2]);
          y[i1 * N + i2] = av + bv;
          y[i1 * N + N - 1 - i2] = av - bv;
        }
        if constexpr (E::MM)
          y[i1 * N + E::M2] = acc_val(Mid[i1]);
      }
      store_slab(sy + sl * US, y);
    }
  }

  // Even-odd backward with S lanes per slab: lane s accumulates the column
  // pairs j = s, s+S, ... (the middle column of odd Q goes to the lane with
  // fewer pairs), then the S lanes sum their accumulators with shuffles and
  // hold the same output slab.  Every lane of a warp runs the same number of
  // rounds, so the shuffles see the whole warp.  As in forward_eo2 the pair
  // loop and the loop over a pair's two columns are not unrolled (one copy of
  // the column code), and a pair's table entries are read at the top of its
  // iteration.
  static __device__ __forceinline__ void backward_eo2(const TabView<T>& p,
                                                      const T* __restrict__ sw,
                                                      ST* __restrict__ sy, const Part& w)
  {
    using E = EO<N, Q>; // backward tables: N x Q
    constexpr int JL = (E::K2 + S - 1) / S > 0 ? (E::K2 + S - 1) / S : 1; // pairs per lane
    constexpr int MIDLANE = E::K2 % S;
    constexpr int MR = E::M2 > 0 ? E::M2 : 1;
    const T* __restrict__ PB = p.PB;
    const T* __restrict__ DB = p.DB;
    const int bstride = w.ncb * SBC;
    const int ls = threadIdx.x % S;
    const int base = w.c0 * N * S, cnt = (w.c1 - w.c0) * N * S;
    const int rounds = (cnt + w.nthr - 1) / w.nthr;
    for (int r = 0; r < rounds; ++r)
    {
      const int idx = r * w.nthr + w.tid;
      const bool live = idx < cnt;
      const int sl = live ? (base + idx) / S : w.c0 * N; // idle lanes read a valid slab
      const int c = sl / N, i0 = sl - c * N;
      const T* b0 = sw + c * SBC + i0 * SQ;
      const T* b1 = b0 + bstride;
      const T* b2 = b1 + bstride;
      acc_t<T> A[N][MR], B[N][MR], Mid[N];
#pragma unroll
      for (int i1 = 0; i1 < N; ++i1)
      {
#pragma unroll
        for (int i2 = 0; i2 < E::M2; ++i2)
          A[i1][i2] = B[i1][i2] = acc_zero<T>();
        Mid[i1] = acc_zero<T>();
      }
      // axis 1 back of column q2: u1 = Phi^T X (+ Gamma^T Y), u2 = Phi^T Z
      auto column = [&](int q2, T(&u1)[N], T(&u2)[N]) {
        T X[Q];
#pragma unroll
        for (int q1 = 0; q1 < Q; ++q1)
          X[q1] = b0[q1 * Q + q2];
        mv_eo<N, Q, 1>(PB, X, u1);
        if constexpr (kGrad)
        {
          T Y[Q], Z[Q], t[N];
#pragma unroll
          for (int q1 = 0; q1 < Q; ++q1)
          {
            Y[q1] = b1[q1 * Q + q2];
            Z[q1] = b2[q1 * Q + q2];
          }
          mv_eo<N, Q, -1>(DB, Y, t);
#pragma unroll
          for (int i = 0; i < N; ++i)
            u1[i] += t[i];
          mv_eo<N, Q, 1>(PB, Z, u2);
        }
      };
#pragma unroll 1
      for (int jj = 0; jj < JL; ++jj) // this lane's column pairs (j, Q-1-j)
      {
        const int j = ls + jj * S;
        if (j >= E::K2)
          break;
        T u1a[N], u2a[N], u1b[N], u2b[N];
#pragma unroll 1
        for (int h = 0; h < 2; ++h) // column j, then column Q-1-j
        {
          T u1[N], u2[N];
          column(h ? Q - 1 - j : j, u1, u2);
#pragma unroll
          for (int i1 = 0; i1 < N; ++i1)
          {
            u1b[i1] = u1[i1];
            u1a[i1] = h ? u1a[i1] : u1[i1];
            if constexpr (kGrad)
            {
              u2b[i1] = u2[i1];
              u2a[i1] = h ? u2a[i1] : u2[i1];
            }
          }
        }
        // this pair's entries of the backward tables
        T pe[MR], po[MR], de[MR], dq[MR], pm = T(0), dm = T(0);
#pragma unroll
        for (int i2 = 0; i2 < E::M2; ++i2)
        {
          pe[i2] = PB[i2 * Q + E::E + j];
          po[i2] = PB[i2 * Q + E::O + j];
          if constexpr (kGrad)
          {
            de[i2] = DB[i2 * Q + E::E + j];
            dq[i2] = DB[i2 * Q + E::O + j];
          }
        }
        if constexpr (E::MM)
        {
          pm = PB[E::M2 * Q + E::E + j];
          if constexpr (kGrad)
            dm = DB[E::M2 * Q + E::O + j];
        }
#pragma unroll
        for (int i1 = 0; i1 < N; ++i1)
        {
          const T e1 = u1a[i1] + u1b[i1], o1 = u1a[i1] - u1b[i1];
#pragma unroll
          for (int i2 = 0; i2 < E::M2; ++i2)
          {
            A[i1][i2] = acc_fma(pe[i2], e1, A[i1][i2]);
            B[i1][i2] = acc_fma(po[i2], o1, B[i1][i2]);
          }
          if constexpr (E::MM)
            Mid[i1] = acc_fma(pm, e1, Mid[i1]);
          if constexpr (kGrad)
          {
            const T e2 = u2a[i1] + u2b[i1], o2 = u2a[i1] - u2b[i1];
#pragma unroll
            for (int i2 = 0; i2 < E::M2; ++i2)
            {
              A[i1][i2] = acc_fma(dq[i2], o2, A[i1][i2]); // d_Gamma
              B[i1][i2] = acc_fma(de[i2], e2, B[i1][i2]); // s_Gamma
            }
            if constexpr (E::MM)
              Mid[i1] = acc_fma(dm, o2, Mid[i1]);
          }
        }
      }
      if constexpr (E::KM) // middle column of odd Q: the C entries
      {
        if (ls == MIDLANE)
        {
          T u1[N], u2[N];
          column(E::K2, u1, u2);
#pragma unroll
          for (int i1 = 0; i1 < N; ++i1)
          {
#pragma unroll
            for (int i2 = 0; i2 < E::M2; ++i2)
            {
              A[i1][i2] = acc_fma(PB[i2 * Q + E::C], u1[i1], A[i1][i2]); // s_Phi
              if constexpr (kGrad)
                B[i1][i2] = acc_fma(DB[i2 * Q + E::C], u2[i1], B[i1][i2]); // s_Gamma
            }
            if constexpr (E::MM) // Gamma^T vanishes at the centre
              Mid[i1] = acc_fma(PB[E::M2 * Q + E::C], u1[i1], Mid[i1]);
          }
        }
      }
      // the S lanes' partial sums, then the output pairs
      T y[N2];
#pragma unroll
      for (int i1 = 0; i1 < N; ++i1)
      {
#pragma unroll
        for (int i2 = 0; i2 < E::M2; ++i2)
        {
          T av = acc_val(A[i1][i2]), bv = acc_val(B[i1][i2]);
#pragma unroll
          for (int o = 1; o < S; o <<= 1)
          {
            av += shfl_xor(av, o);
            bv += shfl_xor(bv, o);
          }
          y[i1 * N + i2] = av + bv;
          y[i1 * N + N - 1 - i2] = av - bv;
        }
        if constexpr (E::MM)
        {
          T mv = acc_val(Mid[i1]);
#pragma unroll
          for (int o = 1; o < S; o <<= 1)
            mv += shfl_xor(mv, o);
          y[i1 * N + E::M2] = mv;
        }
      }
      // the S lanes of a slab hold the same sums: the store is one write
      if (live)
        store_slab(sy + sl * US, y);
    }
  }

  static __device__ __forceinline__ void backward(const TabView<T>& p,
                                                  const T* __restrict__ sw,
                                                  ST* __restrict__ sy, int ncb)
  {
    backward(p, sw, sy, cta_part(ncb));
  }

  static __device__ __forceinline__ void backward(const TabView<T>& p,
                                                  const T* __restrict__ sw,
                                                  ST* __restrict__ sy, const Part& w)
  {
    if constexpr (EVOD && S == 1)
    {
      backward_eo(p, sw, sy, w);
      return;
    }
    else if constexpr (EVOD)
    {
      backward_eo2(p, sw, sy, w);
      return;
    }
    const T* __restrict__ P = kAffine ? p.PB : p.P; // affine: weighted tables
    const T* __restrict__ D = kAffine ? p.DB : p.D;
    // every lane of a warp takes part in the shuffle reduction, so all
    // threads of the part run the same number of rounds
    const int bstride = w.ncb * SBC;
    const int base = w.c0 * N * S, cnt = (w.c1 - w.c0) * N * S;
    const int rounds = (cnt + w.nthr - 1) / w.nthr;
    // axis-2 backward table entries of this lane's q2 columns (see forward)
    const T* T2 = (OP == OP_STIFFNESS && SEM == SEM_REFERENCE) ? D : P;
    T tc[PRE ? QS : 1][PRE ? N : 1], ec[PRE ? QS : 1][PRE ? N : 1];
    if constexpr (PRE)
    {
      const int ls = threadIdx.x % S;
#pragma unroll
      for (int jq = 0; jq < QS; ++jq)
#pragma unroll
        for (int i2 = 0; i2 < N; ++i2)
        {
          const int q2 = ls + jq * S;
          tc[jq][i2] = q2 < Q ? T2[i2 * BSM + q2 * BSK] : T(0);
          ec[jq][i2] = q2 < Q ? D[i2 * BSM + q2 * BSK] : T(0);
        }
    }
    for (int r = 0; r < rounds; ++r)
    {
      const int idx = r * w.nthr + w.tid;
      const bool live = idx < cnt;
      const int ts = base + idx;
      const int sl = live ? ts / S : 0, lane_s = ts - (ts / S) * S;
      const int c = sl / N, i0 = sl - c * N;
      const T* b0 = sw + c * SBC + i0 * SQ;
      const T* b1 = b0 + bstride;
      const T* b2 = b1 + bstride;
      acc_t<T> ya[N2]; // accumulators (double-float: lazily renormalised)
#pragma unroll
      for (int k = 0; k < N2; ++k)
        ya[k] = acc_zero<T>();
#pragma unroll UNR
      for (int jq = 0; jq < QS; ++jq)
      {
        const int q2 = lane_s + jq * S;
        if (!live || (S > 1 && q2 >= Q))
          break;
        T X[Q], Y[Q], Z[Q], U1[N], U2[N];
#pragma unroll
        for (int q1 = 0; q1 < Q; ++q1)
        {
          X[q1] = b0[q1 * Q + q2];
          if constexpr (kGrad && SEM == SEM_EXACT)
          {
            Y[q1] = b1[q1 * Q + q2];
            Z[q1] = b2[q1 * Q + q2];
          }
        }
        // axis 1 back (q1 -> i1)
#pragma unroll
        for (int i1 = 0; i1 < N; ++i1)
        {
          acc_t<T> acc = acc_mul(P[i1 * BSM], X[0]);
#pragma unroll
          for (int q1 = 1; q1 < Q; ++q1)
            acc = acc_fma(P[i1 * BSM + q1 * BSK], X[q1], acc);
          if constexpr (kGrad && SEM == SEM_EXACT)
          {
#pragma unroll
            for (int q1 = 0; q1 < Q; ++q1)
              acc = acc_fma(D[i1 * BSM + q1 * BSK], Y[q1], acc);
            acc_t<T> acc2 = acc_mul(P[i1 * BSM], Z[0]);
#pragma unroll
            for (int q1 = 1; q1 < Q; ++q1)
              acc2 = acc_fma(P[i1 * BSM + q1 * BSK], Z[q1], acc2);
            U2[i1] = acc_val(acc2);
          }
          U1[i1] = acc_val(acc);
        }
        // axis 2 back (q2 -> i2), accumulated over q2
#pragma unroll
        for (int i2 = 0; i2 < N; ++i2)
        {
          T t1;
          if constexpr (PRE)
            t1 = tc[jq][i2];
          else
            t1 = T2[i2 * BSM + q2 * BSK];
#pragma unroll
          for (int i1 = 0; i1 < N; ++i1)
            ya[i1 * N + i2] = acc_fma(t1, U1[i1], ya[i1 * N + i2]);
          if constexpr (kGrad && SEM == SEM_EXACT)
          {
            T t2;
            if constexpr (PRE)
              t2 = ec[jq][i2];
            else
              t2 = D[i2 * BSM + q2 * BSK];
#pragma unroll
            for (int i1 = 0; i1 < N; ++i1)
              ya[i1 * N + i2] = acc_fma(t2, U2[i1], ya[i1 * N + i2]);
          }
        }
      }
      T y[N2];
#pragma unroll
      for (int k = 0; k < N2; ++k)
        y[k] = acc_val(ya[k]);
      if constexpr (S > 1)
      {
#pragma unroll
        for (int k = 0; k < N2; ++k)
        {
#pragma unroll
          for (int o = 1; o < S; o <<= 1)
            y[k] += shfl_xor(y[k], o);
        }
      }
      // the S lanes of a slab hold the same sums: the store is one write
      if (live)
        store_slab(sy + sl * US, y);
    }
  }
};

// ---------------------------------------------------------------------------
// FP32 slab tile on packed FP32 pairs.  sm_100 and later issue
// fma.rn.f32x2 (__ffma2_rn): one instruction carries two independent FMAs,
// each rounded as fmaf.  An operand may be a register pair, one register
// broadcast to both halves, or an entry (broadcast) or an aligned pair of
// entries of the launch's parameter block, so table operands stay constant-
// bank operands.  The FP32 slab kernels are bound by instruction issue; here
// every contraction computes two outputs per instruction:
//  * forward : stiffness: {a, g} = {Phi, Gamma}(q2, :) . x(i1, :) for one
//    column q2, then {AA, BA}(q1) = Phi(q1, :) . {a, g} and AG for two q1 at
//    once (GF); mass: two columns q2 at once, then Phi(q1, :) broadcast;
//  * fused   : {d/dy, d/dz} = Phi . {x_g, x_b} and d/dx at two points at
//    once (GF); back: {y, z} with Phi broadcast, x for two DOFs at once (GB);
//    mass: two points (PF) and two DOFs (PB) at once;
//  * backward: {x, z} with Phi broadcast, y for two DOFs at once (GB); axis
//    2 accumulates two DOFs of a row at once ((Phi or Gamma)(q2, i2..i2+1)).
// Two lanes per slab keep the lane's table columns in registers (pairs);
// one lane reads them from the pair tables.  Host-built pair tables (float2,
// padded with zeros to whole pairs) in the parameter block's table slots:
//   PG (slots 2-3) {Phi(q,i), Gamma(q,i)}      at q*N + i       (stiffness)
//   PF (slot 2)    {Phi(q,i), Phi(q+1,i)}      at (q/2)*N + i   (mass)
//   GF (slot 4)    {Gamma(q,i), Gamma(q+1,i)}  at (q/2)*N + i   (stiffness)
//   GB (slot 5)    {Gamma(q,i), Gamma(q,i+1)}  at (i/2)*Q + q   (stiffness)
//   PB (slot 6)    {Phi(q,i), Phi(q,i+1)}      at (i/2)*Q + q
// Exact semantics, per-point mass and stiffness; the tile's layout, strides
// and staging are SlabTile's.  Sums run in the order of SlabTile's except
// the backward x-gradient sum of a slab column, which adds its Gamma part
// to its Phi part at the end.
// ---------------------------------------------------------------------------
constexpr int kTabSlot = kMaxQ * kMaxN; // floats per table slot
constexpr int kSlotPG = 2, kSlotPF = 2, kSlotGF = 4, kSlotGB = 5, kSlotPB = 6;

__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c)
{
  return __ffma2_rn(a, b, c);
}
__device__ __forceinline__ float2 f2mul(float2 a, float2 b)
{
  return __fmul2_rn(a, b);
}
__device__ __forceinline__ float2 f2b(float x)
{
  return make_float2(x, x);
}

// The tiles that run on packed pairs (see SlabTileF2): FP32, exact
// semantics, per-point mass, stiffness and Helmholtz, N <= 5.  Above N = 5 the pair
// accumulators and register tables outgrow the register file (measured at
// N = 7: 255 registers against 204, and slower).
template <typename T, int N, int OP, int SEM, bool EVOD>
__host__ __device__ constexpr bool paired_tile()
{
  return std::is_same<T, float>::value && SEM == SEM_EXACT && !EVOD &&
         (OP == OP_MASS || OP == OP_STIFFNESS || OP == OP_HELMHOLTZ) && N <= 5;
}

template <int N, int Q, int OP, int LANES, bool SLOTS>
struct SlabTileF2 : SlabTile<float, N, Q, OP, SEM_EXACT, LANES, false, SLOTS>
{
  using B = SlabTile<float, N, Q, OP, SEM_EXACT, LANES, false, SLOTS>;
  static constexpr int S = B::S, N2 = B::N2, Q2 = B::Q2, Q3 = Q * Q * Q;
  static constexpr int SQ = B::SQ, SBC = B::SBC, QS = B::QS, UNR = B::UNR;
  static constexpr bool kGrad = B::kGrad;
  static_assert(OP == OP_MASS || OP == OP_STIFFNESS || OP == OP_HELMHOLTZ,
                "paired tile: per-point mass, stiffness and Helmholtz");
  static_assert(N <= 8 && 2 * Q * N <= 2 * kTabSlot, "pair tables sized for the slab degrees");
  static constexpr int NP = (N + 1) / 2, QP = (Q + 1) / 2; // whole pairs (padded)
  static constexpr int NF = N / 2;                           // full pairs of N
  static_assert(N <= 5, "see paired_tile");
  static constexpr int CP = (QS + 1) / 2; // mass, two lanes: column pairs of a lane

  static __device__ __forceinline__ const float2* slot(const TabView<float>& p, int k)
  {
    return reinterpret_cast<const float2*>(p.X + k * kTabSlot);
  }

  static __device__ __forceinline__ void forward(const TabView<float>& p,
                                                 const float* __restrict__ su,
                                                 float* __restrict__ sw, const Part& w)
  {
    const float* __restrict__ P = p.P;
    const float* __restrict__ D = p.D;
    const float2* __restrict__ PG = slot(p, kSlotPG);
    const float2* __restrict__ PF = slot(p, kSlotPF);
    const float2* __restrict__ GF = slot(p, kSlotGF);
    const int bstride = w.ncb * SBC;
    // two lanes: this lane's columns q2 = ls, ls + S, ... as register pairs
    // (stiffness {Phi, Gamma}(q2, i2); mass {Phi(q2, i2), Phi(q2 + S, i2)})
    constexpr int PR = S > 1 ? (kGrad ? QS : CP) : 1;
    float2 pc[PR][S > 1 ? N : 1];
    if constexpr (S > 1)
    {
      const int ls = threadIdx.x % S;
#pragma unroll
      for (int j = 0; j < PR; ++j)
#pragma unroll
        for (int i2 = 0; i2 < N; ++i2)
        {
          if constexpr (kGrad)
          {
            const int q2 = ls + j * S;
            pc[j][i2] = q2 < Q ? make_float2(P[q2 + i2 * Q], D[q2 + i2 * Q]) : f2b(0.f);
          }
          else
          {
            const int qa = ls + 2 * j * S, qb = qa + S;
            pc[j][i2] = make_float2(qa < Q ? P[qa + i2 * Q] : 0.f, qb < Q ? P[qb + i2 * Q] : 0.f);
          }
        }
    }
    for (int ts = w.c0 * N * S + w.tid; ts < w.c1 * N * S; ts += w.nthr)
    {
      const int sl = ts / S, lane_s = ts - sl * S;
      const int c = sl / N, i0 = sl - c * N;
      float x[N2];
      B::load_slab(su + sl * B::US, x);
      float* b0 = sw + c * SBC + i0 * SQ;
      if constexpr (kGrad)
      {
        float* b1 = b0 + bstride;
        float* b2 = b1 + bstride;
#pragma unroll UNR
        for (int jq = 0; jq < QS; ++jq)
        {
          const int q2 = S > 1 ? lane_s + jq * S : jq;
          if (S > 1 && q2 >= Q)
            break;
          auto tg = [&](int i2) -> float2 {
            if constexpr (S > 1)
              return pc[jq][i2];
            else
              return PG[q2 * N + i2];
          };
          float2 ag[N]; // {a, g}(i1): axis 2 with Phi and with Gamma
#pragma unroll
          for (int i1 = 0; i1 < N; ++i1)
          {
            float2 acc = f2mul(tg(0), f2b(x[i1 * N]));
#pragma unroll
            for (int i2 = 1; i2 < N; ++i2)
              acc = f2fma(tg(i2), f2b(x[i1 * N + i2]), acc);
            ag[i1] = acc;
          }
#pragma unroll
          for (int q1 = 0; q1 < Q; ++q1) // {AA, BA} = Phi_1 {a, g}
          {
            float2 o = f2mul(f2b(P[q1]), ag[0]);
#pragma unroll
            for (int i1 = 1; i1 < N; ++i1)
              o = f2fma(f2b(P[q1 + i1 * Q]), ag[i1], o);
            b0[q1 * Q + q2] = o.x;
            b2[q1 * Q + q2] = o.y;
          }
#pragma unroll
          for (int h = 0; h < QP; ++h) // AG = Gamma_1 a, two q1 at once
          {
            float2 o = f2mul(GF[h * N], f2b(ag[0].x));
#pragma unroll
            for (int i1 = 1; i1 < N; ++i1)
              o = f2fma(GF[h * N + i1], f2b(ag[i1].x), o);
            b1[(2 * h) * Q + q2] = o.x;
            if (2 * h + 1 < Q)
              b1[(2 * h + 1) * Q + q2] = o.y;
          }
        }
      }
      else
      {
        constexpr int NCP = S > 1 ? CP : QP;
#pragma unroll
        for (int h = 0; h < NCP; ++h) // two columns qa, qb at once
        {
          const int qa = S > 1 ? lane_s + 2 * h * S : 2 * h;
          const int qb = qa + (S > 1 ? S : 1);
          if (S > 1 && qa >= Q)
            break;
          auto tp = [&](int i2) -> float2 {
            if constexpr (S > 1)
              return pc[h][i2];
            else
              return PF[h * N + i2];
          };
          float2 a[N];
#pragma unroll
          for (int i1 = 0; i1 < N; ++i1)
          {
            float2 acc = f2mul(tp(0), f2b(x[i1 * N]));
#pragma unroll
            for (int i2 = 1; i2 < N; ++i2)
              acc = f2fma(tp(i2), f2b(x[i1 * N + i2]), acc);
            a[i1] = acc;
          }
#pragma unroll
          for (int q1 = 0; q1 < Q; ++q1)
          {
            float2 o = f2mul(f2b(P[q1]), a[0]);
#pragma unroll
            for (int i1 = 1; i1 < N; ++i1)
              o = f2fma(f2b(P[q1 + i1 * Q]), a[i1], o);
            b0[q1 * Q + qa] = o.x;
            if (qb < Q)
              b0[q1 * Q + qb] = o.y;
          }
        }
      }
    }
  }

  static __device__ __forceinline__ void fused(const TabView<float>& p,
                                               float* __restrict__ sw, const Part& w,
                                               const float* __restrict__ geo,
                                               long long geo_cell0, bool l2pf = false)
  {
    const float* __restrict__ P = p.P;
    const float2* __restrict__ PG = slot(p, kSlotPG);
    const float2* __restrict__ PF = slot(p, kSlotPF);
    const float2* __restrict__ GF = slot(p, kSlotGF);
    const float2* __restrict__ GB = slot(p, kSlotGB);
    const float2* __restrict__ PB = slot(p, kSlotPB);
    constexpr int NCG = geo_nc(OP);
    constexpr int sq = SQ;
    const int bstride = w.ncb * SBC;
    for (int t = w.c0 * Q2 + w.tid; t < w.c1 * Q2; t += w.nthr)
    {
      const int c = t / Q2, r = t - c * Q2;
      float* b0 = sw + c * SBC + r;
      const int tn = t + w.nthr; // this thread's next pencil, if any
      if (l2pf && tn < w.c1 * Q2)
      {
        const int cn = tn / Q2, rn = tn - cn * Q2;
        const float* gn = geo + ((geo_cell0 + cn) * Q3 + rn) * NCG;
#pragma unroll
        for (int q = 0; q < Q; ++q)
          prefetch_l2(gn + (long long)q * Q2 * NCG);
      }
      if constexpr (OP == OP_MASS)
      {
        const float* dw = geo + (geo_cell0 + c) * Q3 + r;
        float xk[N], v[2 * QP];
#pragma unroll
        for (int k = 0; k < N; ++k)
          xk[k] = b0[k * sq];
#pragma unroll
        for (int h = 0; h < QP; ++h) // two points at once
        {
          float2 s = f2mul(PF[h * N], f2b(xk[0]));
#pragma unroll
          for (int k = 1; k < N; ++k)
            s = f2fma(PF[h * N + k], f2b(xk[k]), s);
          v[2 * h] = s.x;
          v[2 * h + 1] = s.y;
        }
#pragma unroll
        for (int q = 0; q < Q; ++q)
          v[q] *= dw[q * Q2];
#pragma unroll
        for (int h = 0; h < NP; ++h) // two DOFs at once
        {
          float2 o = f2mul(PB[h * Q], f2b(v[0]));
#pragma unroll
          for (int q = 1; q < Q; ++q)
            o = f2fma(PB[h * Q + q], f2b(v[q]), o);
          b0[(2 * h) * sq] = o.x;
          if (2 * h + 1 < N)
            b0[(2 * h + 1) * sq] = o.y;
        }
      }
      else
      {
        float* b1 = b0 + bstride;
        float* b2 = b1 + bstride;
        const float* G = geo + ((geo_cell0 + c) * Q3 + r) * NCG;
        // the pencil's geometry, [zz,yz,xz,yy,xy,xx] per point as three
        // pairs, asked for before the contractions that precede its use
        constexpr int NG2 = NCG / 2; // pairs per point (Helmholtz: the mass factor too)
        float2 gq[Q][NG2];
#pragma unroll
        for (int q = 0; q < Q; ++q)
        {
          const float2* g2 = reinterpret_cast<const float2*>(G + (long long)q * Q2 * NCG);
#pragma unroll
          for (int j = 0; j < NG2; ++j)
            gq[q][j] = g2[j];
        }
        float xa[N];
        float2 xgb[N]; // {AG, BA} along axis 0
#pragma unroll
        for (int k = 0; k < N; ++k)
        {
          xa[k] = b0[k * sq];
          xgb[k] = make_float2(b1[k * sq], b2[k * sq]);
        }
        float2 fyz[Q]; // {d/dy, d/dz}: Phi on axis 0
        float fx[2 * QP];
        float2 fmx[OP == OP_HELMHOLTZ ? Q : 1]; // Helmholtz: {u, d/dx} at the points
#pragma unroll
        for (int q = 0; q < Q; ++q)
        {
          float2 s = f2mul(f2b(P[q]), xgb[0]);
#pragma unroll
          for (int k = 1; k < N; ++k)
            s = f2fma(f2b(P[q + k * Q]), xgb[k], s);
          fyz[q] = s;
        }
        if constexpr (OP == OP_HELMHOLTZ)
        {
#pragma unroll
          for (int q = 0; q < Q; ++q) // {Phi, Gamma} on axis 0: the value and d/dx
          {
            float2 s = f2mul(PG[q * N], f2b(xa[0]));
#pragma unroll
            for (int k = 1; k < N; ++k)
              s = f2fma(PG[q * N + k], f2b(xa[k]), s);
            fmx[q] = s;
            fx[q] = s.y;
          }
        }
        else
        {
#pragma unroll
          for (int h = 0; h < QP; ++h) // d/dx: Gamma on axis 0, two points at once
          {
            float2 s = f2mul(GF[h * N], f2b(xa[0]));
#pragma unroll
            for (int k = 1; k < N; ++k)
              s = f2fma(GF[h * N + k], f2b(xa[k]), s);
            fx[2 * h] = s.x;
            fx[2 * h + 1] = s.y;
          }
        }
        // G transform (src/stiffness.hpp:14-29), [zz,yz,xz,yy,xy,xx]
#pragma unroll
        for (int q = 0; q < Q; ++q)
        {
          const float zz = gq[q][0].x, yz = gq[q][0].y, xz = gq[q][1].x, yy = gq[q][1].y,
                      xy = gq[q][2].x, xx = gq[q][2].y;
          const float w0 = fx[q], w1 = fyz[q].x, w2 = fyz[q].y;
          fx[q] = xx * w0 + xy * w1 + xz * w2;
          fyz[q] = make_float2(xy * w0 + yy * w1 + yz * w2, xz * w0 + yz * w1 + zz * w2);
          if constexpr (OP == OP_HELMHOLTZ) // the mass term: alpha detJ w u
            fmx[q] = make_float2(fmx[q].x * gq[q][3].x, fx[q]);
        }
#pragma unroll
        for (int k = 0; k < N; ++k) // {y, z} back: Phi^T
        {
          float2 o = f2mul(f2b(P[k * Q]), fyz[0]);
#pragma unroll
          for (int q = 1; q < Q; ++q)
            o = f2fma(f2b(P[q + k * Q]), fyz[q], o);
          b1[k * sq] = o.x;
          b2[k * sq] = o.y;
        }
        if constexpr (OP == OP_HELMHOLTZ)
        {
#pragma unroll
          for (int k = 0; k < N; ++k) // Phi^T (m u) + Gamma^T x, the halves summed
          {
            float2 o = f2mul(PG[k], fmx[0]);
#pragma unroll
            for (int q = 1; q < Q; ++q)
              o = f2fma(PG[q * N + k], fmx[q], o);
            b0[k * sq] = o.x + o.y;
          }
        }
        else
        {
#pragma unroll
          for (int h = 0; h < NP; ++h) // x back: Gamma^T, two DOFs at once
          {
            float2 o = f2mul(GB[h * Q], f2b(fx[0]));
#pragma unroll
            for (int q = 1; q < Q; ++q)
              o = f2fma(GB[h * Q + q], f2b(fx[q]), o);
            b0[(2 * h) * sq] = o.x;
            if (2 * h + 1 < N)
              b0[(2 * h + 1) * sq] = o.y;
          }
        }
      }
    }
  }

  static __device__ __forceinline__ void backward(const TabView<float>& p,
                                                  const float* __restrict__ sw,
                                                  float* __restrict__ sy, const Part& w)
  {
    const float* __restrict__ P = p.P;
    const float* __restrict__ D = p.D;
    const float2* __restrict__ GB = slot(p, kSlotGB);
    const float2* __restrict__ PB = slot(p, kSlotPB);
    const int bstride = w.ncb * SBC;
    const int base = w.c0 * N * S, cnt = (w.c1 - w.c0) * N * S;
    const int rounds = (cnt + w.nthr - 1) / w.nthr;
    // two lanes: axis-2 table pairs of this lane's columns, {Phi(q2, i2),
    // Phi(q2, i2 + 1)} and the same of Gamma (odd N: the last entry alone)
    constexpr int PR = S > 1 ? QS : 1;
    constexpr int ODD = N & 1;
    float2 tp[PR][S > 1 && NF > 0 ? NF : 1], tg[PR][S > 1 && kGrad && NF > 0 ? NF : 1];
    float tpl[PR], tgl[PR];
    if constexpr (S > 1)
    {
      const int ls = threadIdx.x % S;
#pragma unroll
      for (int jq = 0; jq < PR; ++jq)
      {
        const int q2 = ls + jq * S;
        const bool ok = q2 < Q;
#pragma unroll
        for (int h = 0; h < NF; ++h)
        {
          const int i = 2 * h;
          tp[jq][h] = ok ? make_float2(P[q2 + i * Q], P[q2 + (i + 1) * Q]) : f2b(0.f);
          if constexpr (kGrad)
            tg[jq][h] = ok ? make_float2(D[q2 + i * Q], D[q2 + (i + 1) * Q]) : f2b(0.f);
        }
        if constexpr (ODD)
        {
          tpl[jq] = ok ? P[q2 + (N - 1) * Q] : 0.f;
          tgl[jq] = (ok && kGrad) ? D[q2 + (N - 1) * Q] : 0.f;
        }
      }
    }
    for (int r = 0; r < rounds; ++r)
    {
      const int idx = r * w.nthr + w.tid;
      const bool live = idx < cnt;
      const int ts = base + idx;
      const int sl = live ? ts / S : 0, lane_s = ts - (ts / S) * S;
      const int c = sl / N, i0 = sl - c * N;
      const float* b0 = sw + c * SBC + i0 * SQ;
      const float* b1 = b0 + bstride;
      const float* b2 = b1 + bstride;
      float2 ya[N][NF > 0 ? NF : 1]; // y(i1, 2h), y(i1, 2h + 1)
      float yl[N];                    // odd N: y(i1, N - 1)
#pragma unroll
      for (int i1 = 0; i1 < N; ++i1)
      {
#pragma unroll
        for (int h = 0; h < NF; ++h)
          ya[i1][h] = f2b(0.f);
        yl[i1] = 0.f;
      }
#pragma unroll UNR
      for (int jq = 0; jq < QS; ++jq)
      {
        const int q2 = S > 1 ? lane_s + jq * S : jq;
        if (!live || (S > 1 && q2 >= Q))
          break;
        auto ttp = [&](int h) -> float2 {
          if constexpr (S > 1)
            return tp[jq][h];
          else
            return PB[h * Q + q2];
        };
        auto ttpl = [&]() -> float {
          if constexpr (S > 1)
            return tpl[jq];
          else
            return P[q2 + (N - 1) * Q];
        };
        if constexpr (kGrad)
        {
          auto ttg = [&](int h) -> float2 {
            if constexpr (S > 1)
              return tg[jq][h];
            else
              return GB[h * Q + q2];
          };
          auto ttgl = [&]() -> float {
            if constexpr (S > 1)
              return tgl[jq];
            else
              return D[q2 + (N - 1) * Q];
          };
          float2 xz[Q];
          float yv[Q];
#pragma unroll
          for (int q1 = 0; q1 < Q; ++q1)
          {
            xz[q1] = make_float2(b0[q1 * Q + q2], b2[q1 * Q + q2]);
            yv[q1] = b1[q1 * Q + q2];
          }
          float u1[2 * NP], u2[N];
#pragma unroll
          for (int i1 = 0; i1 < N; ++i1) // axis 1 back, Phi^T: {x, z}
          {
            float2 s = f2mul(f2b(P[i1 * Q]), xz[0]);
#pragma unroll
            for (int q1 = 1; q1 < Q; ++q1)
              s = f2fma(f2b(P[q1 + i1 * Q]), xz[q1], s);
            u1[i1] = s.x;
            u2[i1] = s.y;
          }
#pragma unroll
          for (int h = 0; h < NP; ++h) // Gamma^T y, two DOFs at once
          {
            float2 s = f2mul(GB[h * Q], f2b(yv[0]));
#pragma unroll
            for (int q1 = 1; q1 < Q; ++q1)
              s = f2fma(GB[h * Q + q1], f2b(yv[q1]), s);
            u1[2 * h] += s.x;
            if (2 * h + 1 < N)
              u1[2 * h + 1] += s.y;
          }
#pragma unroll
          for (int i1 = 0; i1 < N; ++i1) // axis 2 back
          {
#pragma unroll
            for (int h = 0; h < NF; ++h)
            {
              ya[i1][h] = f2fma(ttp(h), f2b(u1[i1]), ya[i1][h]);
              ya[i1][h] = f2fma(ttg(h), f2b(u2[i1]), ya[i1][h]);
            }
            if constexpr (ODD)
            {
              yl[i1] = fmaf(ttpl(), u1[i1], yl[i1]);
              yl[i1] = fmaf(ttgl(), u2[i1], yl[i1]);
            }
          }
        }
        else
        {
          float X[Q], u[2 * NP];
#pragma unroll
          for (int q1 = 0; q1 < Q; ++q1)
            X[q1] = b0[q1 * Q + q2];
#pragma unroll
          for (int h = 0; h < NP; ++h) // axis 1 back, two DOFs at once
          {
            float2 s = f2mul(PB[h * Q], f2b(X[0]));
#pragma unroll
            for (int q1 = 1; q1 < Q; ++q1)
              s = f2fma(PB[h * Q + q1], f2b(X[q1]), s);
            u[2 * h] = s.x;
            u[2 * h + 1] = s.y;
          }
#pragma unroll
          for (int i1 = 0; i1 < N; ++i1) // axis 2 back
          {
#pragma unroll
            for (int h = 0; h < NF; ++h)
              ya[i1][h] = f2fma(ttp(h), f2b(u[i1]), ya[i1][h]);
            if constexpr (ODD)
              yl[i1] = fmaf(ttpl(), u[i1], yl[i1]);
          }
        }
      }
      float y[N2];
#pragma unroll
      for (int i1 = 0; i1 < N; ++i1)
#pragma unroll
        for (int i2 = 0; i2 < N; ++i2)
          y[i1 * N + i2] = (ODD && i2 == N - 1) ? yl[i1]
                                                : ((i2 & 1) ? ya[i1][i2 / 2].y : ya[i1][i2 / 2].x);
      if constexpr (S > 1)
      {
#pragma unroll
        for (int k = 0; k < N2; ++k)
        {
#pragma unroll
          for (int o = 1; o < S; o <<= 1)
            y[k] += shfl_xor(y[k], o);
        }
      }
      // the S lanes of a slab hold the same sums: the store is one write
      if (live)
        B::store_slab(sy + sl * B::US, y);
    }
  }
};

// One warp copies n elements between global (or host) memory and shared
// memory: 16-byte vector accesses when both addresses and n allow, else
// scalar; unrolled so that several requests are in flight per lane.
template <typename ST>
__device__ __forceinline__ void warp_copy(ST* __restrict__ dst, const ST* __restrict__ src, int n,
                                          int lane)
{
  constexpr int W = 16 / sizeof(ST);
  if (((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) & 15u) == 0 &&
      n % W == 0)
  {
    const uint4* s4 = reinterpret_cast<const uint4*>(src);
    uint4* d4 = reinterpret_cast<uint4*>(dst);
#pragma unroll 4
    for (int i = lane; i < n / W; i += 32)
      d4[i] = s4[i];
  }
  else
  {
#pragma unroll 4
    for (int i = lane; i < n; i += 32)
      dst[i] = src[i];
  }
}

// One warp moves the DOF slabs of cells [c0, c1) between global memory
// (cells packed, cell c0 at g) and the shared slots (slab stride US): one
// contiguous run when the slots are packed (odd N), else slab by slab
// with 16-byte vectors (even N: a slab is a multiple of 16 bytes).
template <int N, int US, bool TO_SMEM, typename ST>
__device__ __forceinline__ void warp_slabs(ST* __restrict__ sm, ST* __restrict__ g, int c0,
                                           int c1, int lane)
{
  constexpr int N2 = N * N, W = 16 / sizeof(ST);
  if constexpr (US == N2)
  {
    if constexpr (TO_SMEM)
      warp_copy(sm + c0 * N * US, g, (c1 - c0) * N * N2, lane);
    else
      warp_copy(g, sm + c0 * N * US, (c1 - c0) * N * N2, lane);
  }
  else
  {
    static_assert(N2 % W == 0, "padded slots hold whole 16-byte vectors");
    constexpr int VS = N2 / W; // vectors per slab
    const int nv = (c1 - c0) * N * VS;
#pragma unroll 4
    for (int v = lane; v < nv; v += 32)
    {
      const int sl = v / VS, k = v - sl * VS;
      uint4* a = reinterpret_cast<uint4*>(sm + (c0 * N + sl) * US) + k;
      uint4* b = reinterpret_cast<uint4*>(g + sl * N2) + k;
      if constexpr (TO_SMEM)
        *a = *b;
      else
        *b = *a;
    }
  }
}

// ---------------------------------------------------------------------------
// Streaming loop of the slab tiles with the work split by warps: each warp
// owns a block of consecutive cells of every tile (its part) and runs the
// forward, fused and backward passes on them with warp-level
// synchronisation only, then writes its cells' outputs with coalesced
// stores.  The CTA shares the TMA stages, handed over with two mbarriers
// per stage: `full` (the copy of a tile has landed) and `empty` (every warp
// has read the stage's DOF and geometry data; warp 0 waits on it before it
// refills the stage).  Without CTA-wide barriers per tile, warps overlap
// one another's passes instead of idling until the slowest is done.
// ---------------------------------------------------------------------------
template <typename T, typename Tile, int N, int Q, int NC>
__device__ __forceinline__ void stream_tiles_warp(const CellParams<T>& p)
{
  using ST = storage_t<T>;
  constexpr int N2 = N * N, N3 = N * N * N, Q3NC = Q * Q * Q * NC;
  constexpr int US = Tile::US;
  extern __shared__ __align__(128) unsigned char smem[];
  const int cb = p.cb;
  const bool staged = NC > 0 && p.geo_staged == GEO_STAGED; // affine forms: nothing to stage
  const bool tile_pf = NC > 0 && p.geo_staged == GEO_TILE_L2 && !p.host_io;
  const long long ntiles = (p.ncells + cb - 1) / cb;
  const CellLayout L = tile_layout<T, Tile, N, Q, NC>(p);
  constexpr int NS = Tile::kStages;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem); // [NS]
  uint64_t* empty = full + NS;                        // [NS]
  auto su = [&](int s) { return reinterpret_cast<ST*>(smem + L.u(s)); };
  auto sg = [&](int s) { return reinterpret_cast<ST*>(smem + L.g(s)); };
  ST* sy = reinterpret_cast<ST*>(smem + L.y);
  T* sw = reinterpret_cast<T*>(smem + L.w);
  const unsigned bslab = N2 * sizeof(ST);
  const unsigned bu = (unsigned)cb * N3 * sizeof(ST);
  const unsigned bg = staged ? (unsigned)cb * Q3NC * sizeof(ST) : 0u;
  // padded slots by tensor copies (whole boxes, padding included, land)
  const bool tma = Tile::kSlabCopies && p.tma_rows > 0 && (cb * N) % p.tma_rows == 0;
  const unsigned bx = tma ? (unsigned)cb * N * US * sizeof(ST) : bu;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  const int cw = (cb + nwarps - 1) / nwarps; // cells per warp
  const int wc0 = min(cb, warp * cw), wc1 = min(cb, wc0 + cw);
  const TabView<T> tv{p.tab[0], p.tab[1], p.sq, p.sbc, p.tab[2], p.tab[3], p.tab[0]};

  if (threadIdx.x == 0)
  {
    for (int s = 0; s < NS; ++s)
    {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], nwarps);
    }
    fence_mbar_init();
  }
  __syncthreads();

  auto is_full = [&](long long t) { return !p.host_io && (t + 1) * cb <= p.ncells; };
  // warp 0: TMA loads of tile t into stage s (the whole tile)
  auto issue = [&](long long t, int s) {
    if (lane == 0)
    {
      fence_proxy_async_smem();
      mbar_arrive_expect_tx(&full[s], bx + bg);
      if (staged)
        bulk_g2s(sg(s), p.geo + t * cb * Q3NC, bg, &full[s]);
      if constexpr (!Tile::kSlabCopies)
        bulk_g2s(su(s), p.u + t * cb * N3, bu, &full[s]);
      else if (tma)
        for (int r = 0; r < cb * N; r += p.tma_rows)
          tma_load_2d(su(s) + r * US, &p.tmu, 0, (int)(t * cb * N) + r, &full[s]);
    }
    if constexpr (Tile::kSlabCopies)
    {
      if (!tma)
      {
        __syncwarp();
        const long long slab0 = t * cb * N;
        for (int k = lane; k < cb * N; k += 32)
          bulk_g2s(su(s) + k * US, p.u + (slab0 + k) * N2, bslab, &full[s]);
      }
    }
  };

  bool ok = true;
  long long issued = -1, waited = -1; // iterations whose TMA copy was issued / landed
  long long tile = blockIdx.x;
  // prologue: the first NS-1 tiles of this CTA
  for (int j = 0; j + 1 < NS; ++j)
  {
    const long long t = tile + (long long)j * gridDim.x;
    if (warp == 0 && t < ntiles && is_full(t))
    {
      issue(t, j);
      issued = j;
    }
  }
  for (int it = 0; tile < ntiles; tile += gridDim.x, ++it)
  {
    const int s = it % NS;
    const long long ahead = tile + (long long)(NS - 1) * gridDim.x;
    // warp 0 refills stage (it-1) % NS with the tile NS-1 iterations ahead
    // once every warp has released it (one stage: only the first tile here,
    // the others after the previous tile's quadrature-point pass)
    if (warp == 0 && ahead < ntiles && is_full(ahead) && (NS > 1 || it == 0))
    {
      if (it >= 1)
        ok = __shfl_sync(0xffffffffu,
                         (int)mbar_wait(&empty[(it - 1) % NS], (unsigned)((it - 1) / NS) & 1u),
                         0) &&
             ok;
      if (ok)
      {
        issue(ahead, (it + NS - 1) % NS);
        issued = it + NS - 1;
      }
    }
    const int ncb = (int)((p.ncells - tile * cb) < cb ? (p.ncells - tile * cb) : cb);
    const int c0 = min(ncb, wc0), c1 = min(ncb, wc1);
    if (tile_pf && c1 > c0) // this warp's fused pass reads its cells' geometry from L2
      prefetch_range_l2(p.geo + (tile * cb + c0) * Q3NC, (size_t)(c1 - c0) * Q3NC * sizeof(ST),
                        lane, 32);
    if (is_full(tile))
      ok = __shfl_sync(0xffffffffu, (int)mbar_wait(&full[s], (unsigned)(it / NS) & 1u), 0) && ok;
    else
    {
      // host-resident or ragged tile: this warp loads its own cells
      warp_slabs<N, US, true>(su(s), const_cast<ST*>(p.u) + (tile * cb + c0) * N3, c0, c1,
                              lane);
      if (staged)
        warp_copy(sg(s) + c0 * Q3NC, p.geo + (tile * cb + c0) * Q3NC, (c1 - c0) * Q3NC, lane);
      __syncwarp();
    }
    if (is_full(tile) && ok)
      waited = it;
    if (!ok)
    {
      // a bounded wait ran out: stop (the other warps' waits run out too);
      // warp 0 first waits, bounded, for the copies it issued
      if (lane == 0)
        record_fault(FAULT_MBAR_TIMEOUT);
      if (warp == 0)
        for (long long k = waited + 1; k <= issued; ++k)
          mbar_wait(&full[k % NS], (unsigned)(k / NS) & 1u);
      break;
    }
    const Part w{cb, c0, c1, lane, 32};
    Tile::forward(tv, su(s), sw, w);
    __syncwarp();
    if (staged)
      Tile::fused(tv, sw, w, sg(s), 0);
    else
      Tile::fused(tv, sw, w, p.geo, tile * cb, !p.host_io && !tile_pf);
    __syncwarp();
    if (lane == 0)
      mbar_arrive(&empty[s]); // this warp is done with stage s's u and geometry
    if constexpr (NS == 1)
    {
      // one stage: warp 0 refills it with this CTA's next tile as soon as
      // every warp is done with it, while the backward passes run
      const long long nxt = tile + gridDim.x;
      if (warp == 0 && ok && nxt < ntiles && is_full(nxt))
      {
        ok = __shfl_sync(0xffffffffu, (int)mbar_wait(&empty[0], (unsigned)it & 1u), 0) && ok;
        if (ok)
        {
          issue(nxt, 0);
          issued = it + 1;
        }
      }
    }
    Tile::backward(tv, sw, sy, w);
    __syncwarp();
    // this warp's outputs: coalesced stores from the output slabs
    warp_slabs<N, US, false>(sy, p.y + (tile * cb + c0) * N3, c0, c1, lane);
    __syncwarp();
  }
}

// CTAs of 256 threads an SM must be able to hold (the register budget):
// the paired FP32 tiles keep to 128 registers per thread, as the scalar
// ones do without the bound (unbounded they took 170 at N = 5 and ran
// slower for the lost occupancy).
template <typename T, int N, int OP, int SEM, bool EVOD>
constexpr int cell_min_blocks()
{
  return paired_tile<T, N, OP, SEM, EVOD>() ? 2 : 1;
}

template <typename T, int N, int Q, int OP, int SEM, int LANES, bool EVOD = false>
__global__ void __launch_bounds__(kCellThreads, (cell_min_blocks<T, N, OP, SEM, EVOD>()))
    cell_kernel(const __grid_constant__ CellParams<T> p)
{
  using Tile = typename std::conditional<paired_tile<T, N, OP, SEM, EVOD>(),
                                         SlabTileF2<N, Q, OP, LANES, true>,
                                         SlabTile<T, N, Q, OP, SEM, LANES, EVOD, true>>::type;
  if constexpr (Tile::kWarpSplit)
    stream_tiles_warp<T, Tile, N, Q, geo_nc(OP)>(p);
  else
    stream_tiles<T, Tile, N, Q, geo_nc(OP)>(p);
}

} // namespace femtc

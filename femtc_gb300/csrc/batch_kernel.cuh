// Batched, persistent operator action over many meshes of mixed degree and
// operator in ONE launch (replayed as a CUDA graph by the host side).
//
// Work is a host-built list of tiles (mesh item, first cell, cell count,
// variant).  The list is ordered so that CTA b processes tiles b, b+G, b+2G,
// ... (G = grid size) and each CTA's sequence is a longest-processing-time
// assignment of the tiles' estimated costs: the schedule is static, so the
// kernel needs no work counter.  Per tile the CTA dispatches, with a
// warp-uniform switch, to the tile code of its variant (N = degree+1,
// Q = N+1, mass or stiffness) -- the same SlabTile / MmaTile passes as the
// single-mesh kernels -- and keeps the two-stage TMA pipeline across tiles
// of different shapes: stage buffers are sized for the largest variant of
// the batch, and each stage's mbarrier phase is tracked explicitly because
// ragged tiles are loaded without TMA.
//
// Tables ride in the parameter block, one slot per degree: the slot index is
// a compile-time constant of each dispatched variant.
#pragma once

#include "cell_kernel.cuh"
#include "mma_kernel.cuh"

namespace femtc
{

constexpr int kBatchDegrees = 7;                  // N = 2..8
constexpr int kBatchVariants = 2 * kBatchDegrees; // x {mass, stiffness}

__host__ __device__ constexpr int batch_variant(int op, int n)
{
  return op * kBatchDegrees + (n - 2);
}

struct BatchTile
{
  long long cell0; // first cell of the tile within its item
  int item;        // mesh index, -1 = padding (no work)
  int variant;     // batch_variant(op, N)
  int ncb;         // cells in this tile
  int full;        // ncb == the variant's cb: loaded and stored by TMA
};

template <typename T>
struct BatchItem
{
  const T* u;
  T* y;
  const T* geo;
};

struct BatchLayout
{
  int cb, staged, sq, sbc;
};

template <typename T>
struct BatchParams
{
  const BatchTile* tiles;
  const BatchItem<T>* items;
  long long ntiles;
  unsigned stage_u, stage_g, stage_y; // bytes of the stage regions (max)
  BatchLayout lay[kBatchVariants];
  // per degree: Phi, Gamma; the even-odd family: the even-odd tables of Phi,
  // Gamma (forward) and Phi^T, Gamma^T (backward)
  T tabs[kBatchDegrees][4][kMaxQ * kMaxN];
};

// Family of tile code: the CUDA-core slab tiles or the tensor-core tiles.
template <typename T, int FAMILY>
struct BatchFamily;

constexpr int kFamilySlab = 0;
constexpr int kFamilyF16X2 = 1;
constexpr int kFamilyBF16X3 = 2;
constexpr int kFamilySlabEO = 3; // CUDA-core tiles, even-odd contractions

__host__ __device__ constexpr bool slab_family(int family)
{
  return family == kFamilySlab || family == kFamilySlabEO;
}

// Lanes per slab of the CUDA-core tiles, per variant: two for the stiffness
// operator up to N = 5 (three outputs per slab), one elsewhere -- the same
// choice as the single-mesh launches.  Two lanes at N >= 6 would need more
// than 255 registers for the stiffness slabs.
__host__ __device__ constexpr int batch_slab_lanes(int op, int n)
{
  return (op == OP_STIFFNESS && n <= 5) ? 2 : 1;
}

template <typename T>
struct BatchFamily<T, kFamilySlab>
{
  template <int N, int OP>
  using Tile = SlabTile<T, N, N + 1, OP, SEM_EXACT, batch_slab_lanes(OP, N)>;
};
// Every even-odd tile fits in 128 registers (one lane per slab).
template <typename T>
struct BatchFamily<T, kFamilySlabEO>
{
  template <int N, int OP>
  using Tile = SlabTile<T, N, N + 1, OP, SEM_EXACT, 1, true>;
};
template <>
struct BatchFamily<float, kFamilyF16X2>
{
  template <int N, int OP>
  using Tile = MmaTile<SPLIT_F16X2, N, N + 1, OP>;
};
template <>
struct BatchFamily<float, kFamilyBF16X3>
{
  template <int N, int OP>
  using Tile = MmaTile<SPLIT_BF16X3, N, N + 1, OP>;
};

// Byte sizes of one tile's stages for a variant (host and device).
template <typename T, int FAMILY, int N, int OP>
__host__ __device__ inline void batch_tile_bytes(const BatchLayout& l,
                                                 unsigned* bu, unsigned* bg,
                                                 unsigned* bw)
{
  using Tl = typename BatchFamily<T, FAMILY>::template Tile<N, OP>;
  constexpr int Q = N + 1, NC = geo_nc(OP);
  CellParams<T> p{};
  p.cb = l.cb;
  p.geo_staged = l.staged;
  p.sq = l.sq;
  p.sbc = l.sbc;
  *bu = (unsigned)l.cb * N * Tl::US * sizeof(T);
  *bg = l.staged ? (unsigned)l.cb * Q * Q * Q * NC * sizeof(T) : 0u;
  *bw = Tl::work_bytes(p);
}

struct BatchSmem
{
  uint64_t* bar;
  unsigned char* u0;
  unsigned char* u1;
  unsigned char* g0;
  unsigned char* g1;
  unsigned char* y;
  unsigned char* w;
  __device__ __forceinline__ unsigned char* u(int s) const { return s ? u1 : u0; }
  __device__ __forceinline__ unsigned char* g(int s) const { return s ? g1 : g0; }
};

// TMA loads of one full tile of variant (N, OP) into stage s (warp 0).
template <typename T, int FAMILY, int N, int OP>
__device__ __forceinline__ void batch_issue_body(const BatchParams<T>& bp,
                                            const BatchTile& t,
                                            const BatchSmem& sm, int s)
{
  using Tl = typename BatchFamily<T, FAMILY>::template Tile<N, OP>;
  constexpr int Q = N + 1, NC = geo_nc(OP);
  constexpr int N2 = N * N, N3 = N * N * N, Q3NC = Q * Q * Q * NC;
  const BatchLayout& l = bp.lay[batch_variant(OP, N)];
  const BatchItem<T>& it = bp.items[t.item];
  const int lane = threadIdx.x & 31;
  const unsigned bu = (unsigned)l.cb * N3 * sizeof(T);
  const unsigned bg = l.staged ? (unsigned)l.cb * Q3NC * sizeof(T) : 0u;
  T* su = reinterpret_cast<T*>(sm.u(s));
  if (lane == 0)
  {
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(&sm.bar[s], bu + bg);
    if (l.staged)
      bulk_g2s(sm.g(s), it.geo + t.cell0 * Q3NC, bg, &sm.bar[s]);
    if constexpr (!Tl::kSlabCopies)
      bulk_g2s(su, it.u + t.cell0 * N3, bu, &sm.bar[s]);
  }
  if constexpr (Tl::kSlabCopies)
  {
    __syncwarp();
    const long long slab0 = t.cell0 * N;
    for (int k = lane; k < l.cb * N; k += 32)
      bulk_g2s(su + k * Tl::US, it.u + (slab0 + k) * N2, N2 * sizeof(T),
               &sm.bar[s]);
  }
}

// Compute one tile of variant (N, OP) whose inputs sit in stage s.
template <typename T, int FAMILY, int N, int OP>
__device__ __forceinline__ void batch_run_body(const BatchParams<T>& bp,
                                          const BatchTile& t,
                                          const BatchSmem& sm, int s)
{
  using Tl = typename BatchFamily<T, FAMILY>::template Tile<N, OP>;
  constexpr int Q = N + 1, NC = geo_nc(OP);
  constexpr int N2 = N * N, N3 = N * N * N, Q3NC = Q * Q * Q * NC;
  constexpr int US = Tl::US;
  const BatchLayout& l = bp.lay[batch_variant(OP, N)];
  const BatchItem<T>& it = bp.items[t.item];
  const TabView<T> tv{bp.tabs[N - 2][0], bp.tabs[N - 2][1], l.sq, l.sbc, bp.tabs[N - 2][2],
                      bp.tabs[N - 2][3]};
  const int ncb = t.ncb;
  T* su = reinterpret_cast<T*>(sm.u(s));
  T* sg = reinterpret_cast<T*>(sm.g(s));
  T* sy = reinterpret_cast<T*>(sm.y);
  T* sw = reinterpret_cast<T*>(sm.w);
  if (!t.full)
  {
    const long long u0 = t.cell0 * N3;
    for (int i = threadIdx.x; i < ncb * N3; i += blockDim.x)
      su[(i / N2) * US + (i % N2)] = it.u[u0 + i];
    if (l.staged)
    {
      const long long g0 = t.cell0 * Q3NC;
      for (int i = threadIdx.x; i < ncb * Q3NC; i += blockDim.x)
        sg[i] = it.geo[g0 + i];
    }
    __syncthreads();
  }
  Tl::forward(tv, su, sw, ncb);
  __syncthreads();
  if (l.staged)
    Tl::fused(tv, sw, ncb, sg, 0);
  else
    Tl::fused(tv, sw, ncb, it.geo, t.cell0);
  if (threadIdx.x < 32)
    bulk_wait_read0(); // the previous tile's stores have left sy
  __syncthreads();
  Tl::backward(tv, sw, sy, ncb);
  if (t.full)
  {
    fence_proxy_async_smem();
    __syncthreads();
    if constexpr (!Tl::kSlabCopies)
    {
      if (threadIdx.x == 0)
      {
        bulk_s2g(it.y + t.cell0 * N3, sy, (unsigned)ncb * N3 * sizeof(T));
        bulk_commit();
      }
    }
    else if (threadIdx.x < 32)
    {
      const int lane = threadIdx.x & 31;
      const long long slab0 = t.cell0 * N;
      for (int k = lane; k < ncb * N; k += 32)
        bulk_s2g(it.y + (slab0 + k) * N2, sy + k * US, N2 * sizeof(T));
      bulk_commit();
    }
  }
  else
  {
    __syncthreads();
    const long long y0 = t.cell0 * N3;
    for (int i = threadIdx.x; i < ncb * N3; i += blockDim.x)
      it.y[y0 + i] = sy[(i / N2) * US + (i % N2)];
  }
  __syncthreads();
}

// The same tile, this warp's part only (the CUDA-core families): its cells
// [c0, c1) of the tile, warp-level synchronisation, the stage released on
// `empty` after the fused pass, the outputs written with coalesced stores.
// Work buffers are spaced by the variant's tile capacity, so a warp's
// regions stay put from tile to tile of one variant.
template <typename T, int FAMILY, int N, int OP>
__device__ __forceinline__ void batch_run_warp_body(const BatchParams<T>& bp,
                                                    const BatchTile& t, const BatchSmem& sm,
                                                    int s, uint64_t* empty)
{
  using Tl = typename BatchFamily<T, FAMILY>::template Tile<N, OP>;
  constexpr int Q = N + 1, NC = geo_nc(OP);
  constexpr int N3 = N * N * N, Q3NC = Q * Q * Q * NC;
  constexpr int US = Tl::US;
  const BatchLayout& l = bp.lay[batch_variant(OP, N)];
  const BatchItem<T>& it = bp.items[t.item];
  const TabView<T> tv{bp.tabs[N - 2][0], bp.tabs[N - 2][1], l.sq, l.sbc, bp.tabs[N - 2][2],
                      bp.tabs[N - 2][3]};
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int cw = (l.cb + nwarps - 1) / nwarps;
  const int c0 = min(t.ncb, warp * cw), c1 = min(t.ncb, warp * cw + cw);
  T* su = reinterpret_cast<T*>(sm.u(s));
  T* sg = reinterpret_cast<T*>(sm.g(s));
  T* sy = reinterpret_cast<T*>(sm.y);
  T* sw = reinterpret_cast<T*>(sm.w);
  if (!t.full)
  {
    warp_slabs<N, US, true>(su, const_cast<T*>(it.u) + (t.cell0 + c0) * N3, c0, c1, lane);
    if (l.staged)
      warp_copy(sg + c0 * Q3NC, it.geo + (t.cell0 + c0) * Q3NC, (c1 - c0) * Q3NC, lane);
    __syncwarp();
  }
  const Part w{l.cb, c0, c1, lane, 32};
  Tl::forward(tv, su, sw, w);
  __syncwarp();
  if (l.staged)
    Tl::fused(tv, sw, w, sg, 0);
  else
    Tl::fused(tv, sw, w, it.geo, t.cell0);
  __syncwarp();
  if (lane == 0)
    mbar_arrive(&empty[s]);
  Tl::backward(tv, sw, sy, w);
  __syncwarp();
  warp_slabs<N, US, false>(sy, it.y + (t.cell0 + c0) * N3, c0, c1, lane);
  __syncwarp();
}

// Per-variant code is a separate function (one register allocation per
// variant, the kernel's count the largest) for the plain CUDA-core family,
// whose tiles need up to 255 registers: one function holding every variant
// measured slower.  The even-odd family is inlined into the kernel: it then
// fits 128 registers, where separate functions would spill kilobytes.
template <int FAMILY>
__host__ __device__ constexpr bool batch_inline()
{
  return FAMILY == kFamilySlabEO;
}

template <typename T, int FAMILY, int N, int OP>
__device__ __noinline__ void batch_issue_call(const BatchParams<T>& bp, const BatchTile& t,
                                              const BatchSmem& sm, int s)
{
  batch_issue_body<T, FAMILY, N, OP>(bp, t, sm, s);
}

template <typename T, int FAMILY, int N, int OP>
__device__ __noinline__ void batch_run_call(const BatchParams<T>& bp, const BatchTile& t,
                                            const BatchSmem& sm, int s)
{
  batch_run_body<T, FAMILY, N, OP>(bp, t, sm, s);
}

template <typename T, int FAMILY, int N, int OP>
__device__ __forceinline__ void batch_issue(const BatchParams<T>& bp, const BatchTile& t,
                                            const BatchSmem& sm, int s)
{
  if constexpr (batch_inline<FAMILY>())
    batch_issue_body<T, FAMILY, N, OP>(bp, t, sm, s);
  else
    batch_issue_call<T, FAMILY, N, OP>(bp, t, sm, s);
}

template <typename T, int FAMILY, int N, int OP>
__device__ __noinline__ void batch_run_warp_call(const BatchParams<T>& bp, const BatchTile& t,
                                                 const BatchSmem& sm, int s, uint64_t* empty)
{
  batch_run_warp_body<T, FAMILY, N, OP>(bp, t, sm, s, empty);
}

template <typename T, int FAMILY, int N, int OP>
__device__ __forceinline__ void batch_run_warp(const BatchParams<T>& bp, const BatchTile& t,
                                               const BatchSmem& sm, int s, uint64_t* empty)
{
  if constexpr (batch_inline<FAMILY>())
    batch_run_warp_body<T, FAMILY, N, OP>(bp, t, sm, s, empty);
  else
    batch_run_warp_call<T, FAMILY, N, OP>(bp, t, sm, s, empty);
}

template <typename T, int FAMILY, int N, int OP>
__device__ __forceinline__ void batch_run(const BatchParams<T>& bp, const BatchTile& t,
                                          const BatchSmem& sm, int s)
{
  if constexpr (batch_inline<FAMILY>())
    batch_run_body<T, FAMILY, N, OP>(bp, t, sm, s);
  else
    batch_run_call<T, FAMILY, N, OP>(bp, t, sm, s);
}

#define FEMTC_BATCH_CASES(X)                                                   \
  X(2, OP_MASS) X(3, OP_MASS) X(4, OP_MASS) X(5, OP_MASS) X(6, OP_MASS)        \
  X(7, OP_MASS) X(8, OP_MASS) X(2, OP_STIFFNESS) X(3, OP_STIFFNESS)            \
  X(4, OP_STIFFNESS) X(5, OP_STIFFNESS) X(6, OP_STIFFNESS)                     \
  X(7, OP_STIFFNESS) X(8, OP_STIFFNESS)

// The kernel's register budget is its largest variant's.  Tensor-core
// families and the (inlined) even-odd family fit in 128 registers: two
// 256-thread CTAs per SM.  The plain CUDA-core slab tiles of degree >= 5
// hold a whole slab per thread and spill under that cap, so that family
// keeps the full register file (one 256-thread CTA, or two of 128 threads,
// per SM).
template <int FAMILY>
__host__ __device__ constexpr int batch_min_blocks()
{
  return FAMILY == kFamilySlab ? 1 : 2;
}

// The CUDA-core families' loop: work split by warps as in
// stream_tiles_warp (cell_kernel.cuh).  Stages: `full` (TMA landed, parity
// per stage flips with each copy) and `empty` (every warp released the
// stage; one phase per iteration).  Where the variant changes from one tile
// to the next, the warps' regions of the stages and buffers move, so the
// CTA meets at a barrier there -- an mbarrier with a bounded wait, so that a
// warp that stopped on a fault cannot hang the others.
template <typename T, int FAMILY>
__device__ __forceinline__ void batch_loop_warp(const BatchParams<T>& bp,
                                                const BatchSmem& sm)
{
  uint64_t* full = sm.bar;      // [2]
  uint64_t* empty = sm.bar + 2; // [2]
  uint64_t* vsync = sm.bar + 4; // variant switches
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  if (threadIdx.x == 0)
  {
    mbar_init(&full[0], 1);
    mbar_init(&full[1], 1);
    mbar_init(&empty[0], nwarps);
    mbar_init(&empty[1], nwarps);
    mbar_init(vsync, nwarps);
    fence_mbar_init();
  }
  __syncthreads();

  auto issue = [&](long long k, int s) {
    const BatchTile t = bp.tiles[k];
    switch (t.variant)
    {
#define X(NN, OPP)                                                             \
  case batch_variant(OPP, NN):                                                 \
    batch_issue<T, FAMILY, NN, OPP>(bp, t, sm, s);                             \
    break;
      FEMTC_BATCH_CASES(X)
#undef X
    default:
      break;
    }
  };
  auto tma_tile = [&](long long k) {
    if (k >= bp.ntiles)
      return false;
    const BatchTile t = bp.tiles[k];
    return t.item >= 0 && t.full != 0;
  };

  bool ok = true;
  unsigned ph[2] = {0u, 0u}; // parity of the next `full` wait per stage
  unsigned vph = 0u;         // parity of the next variant-switch wait
  long long pend[2] = {-1, -1}; // per stage: a copy issued and not yet waited for
  int prev_variant = -1;
  long long k = blockIdx.x;
  if (warp == 0 && tma_tile(k))
  {
    issue(k, 0);
    pend[0] = k;
  }
  for (int it = 0; k < bp.ntiles; k += gridDim.x, ++it)
  {
    const int s = it & 1;
    const long long next = k + gridDim.x;
    if (warp == 0 && tma_tile(next))
    {
      if (it >= 1)
        ok = __shfl_sync(0xffffffffu,
                         (int)mbar_wait(&empty[s ^ 1], (unsigned)((it - 1) >> 1) & 1u), 0) &&
             ok;
      if (ok)
      {
        issue(next, s ^ 1);
        pend[s ^ 1] = next;
      }
    }
    const BatchTile t = bp.tiles[k];
    if (t.item < 0)
    {
      if (lane == 0)
        mbar_arrive(&empty[s]); // padding: keeps one `empty` phase per iteration
      continue;
    }
    if (t.variant != prev_variant)
    {
      if (prev_variant >= 0)
      {
        if (lane == 0)
          mbar_arrive(vsync);
        ok = __shfl_sync(0xffffffffu, (int)mbar_wait(vsync, vph), 0) && ok;
        vph ^= 1u;
      }
      prev_variant = t.variant;
    }
    if (t.full)
    {
      ok = __shfl_sync(0xffffffffu, (int)mbar_wait(&full[s], ph[s]), 0) && ok;
      ph[s] ^= 1u;
      if (ok)
        pend[s] = -1;
    }
    if (!ok)
    {
      if (lane == 0)
        record_fault(FAULT_MBAR_TIMEOUT);
      if (warp == 0) // bounded waits for copies still in flight into the stages
        for (int q = 0; q < 2; ++q)
          if (pend[q] >= 0)
            mbar_wait(&full[q], ph[q]);
      break;
    }
    switch (t.variant)
    {
#define X(NN, OPP)                                                             \
  case batch_variant(OPP, NN):                                                 \
    batch_run_warp<T, FAMILY, NN, OPP>(bp, t, sm, s, empty);                   \
    break;
      FEMTC_BATCH_CASES(X)
#undef X
    default:
      if (threadIdx.x == 0)
        record_fault(FAULT_BAD_DESCRIPTOR);
      if (lane == 0)
        mbar_arrive(&empty[s]);
      break;
    }
  }
}

template <typename T, int FAMILY>
__global__ void __launch_bounds__(kCellThreads, batch_min_blocks<FAMILY>())
    batch_kernel(const __grid_constant__ BatchParams<T> bp)
{
  extern __shared__ __align__(128) unsigned char smem[];
  BatchSmem sm;
  sm.bar = reinterpret_cast<uint64_t*>(smem);
  sm.u0 = smem + 128;
  sm.g0 = sm.u0 + bp.stage_u;
  sm.u1 = sm.g0 + bp.stage_g;
  sm.g1 = sm.u1 + bp.stage_u;
  sm.y = sm.g1 + bp.stage_g;
  sm.w = sm.y + bp.stage_y;
  if constexpr (slab_family(FAMILY))
  {
    batch_loop_warp<T, FAMILY>(bp, sm);
    return;
  }
  if (threadIdx.x == 0)
  {
    mbar_init(&sm.bar[0], 1);
    mbar_init(&sm.bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  unsigned ph0 = 0u, ph1 = 0u; // per-stage parity of the next TMA wait

  auto issue = [&](long long k, int s) {
    const BatchTile t = bp.tiles[k];
    if (t.item < 0 || !t.full)
      return;
    switch (t.variant)
    {
#define X(NN, OPP)                                                             \
  case batch_variant(OPP, NN):                                                 \
    batch_issue<T, FAMILY, NN, OPP>(bp, t, sm, s);                             \
    break;
      FEMTC_BATCH_CASES(X)
#undef X
    default:
      break;
    }
  };

  long long k = blockIdx.x;
  if (threadIdx.x < 32 && k < bp.ntiles)
    issue(k, 0);
  for (int it = 0; k < bp.ntiles; k += gridDim.x, ++it)
  {
    const int s = it & 1;
    const long long next = k + gridDim.x;
    if (threadIdx.x < 32 && next < bp.ntiles)
      issue(next, s ^ 1);
    const BatchTile t = bp.tiles[k];
    if (t.item < 0)
      continue; // padding of a shorter CTA schedule
    bool ok = true;
    if (t.full)
    {
      ok = mbar_wait(&sm.bar[s], s ? ph1 : ph0);
      if (s)
        ph1 ^= 1u;
      else
        ph0 ^= 1u;
    }
    if (__syncthreads_or(!ok))
    {
      if (threadIdx.x == 0)
        record_fault(FAULT_MBAR_TIMEOUT);
      break;
    }
    switch (t.variant)
    {
#define X(NN, OPP)                                                             \
  case batch_variant(OPP, NN):                                                 \
    batch_run<T, FAMILY, NN, OPP>(bp, t, sm, s);                               \
    break;
      FEMTC_BATCH_CASES(X)
#undef X
    default:
      if (threadIdx.x == 0)
        record_fault(FAULT_BAD_DESCRIPTOR);
      break;
    }
  }
  if (threadIdx.x < 32)
    bulk_wait0();
}

} // namespace femtc

namespace femtc
{
// Host-visible description of one compiled batch kernel family.
struct BatchKernelInfo
{
  const void* fn;
  int family;
  int dtype; // femtc_dtype of the family
  // stage / work bytes of one tile of `variant` under layout l
  void (*bytes)(int variant, const BatchLayout& l, unsigned* bu,
                unsigned* bg, unsigned* bw);
  unsigned (*read_fault)(); // reads and clears the family unit's fault word
};

template <typename T, int FAMILY>
void batch_bytes(int v, const BatchLayout& l, unsigned* bu, unsigned* bg,
                 unsigned* bw)
{
  switch (v)
  {
#define X(NN, OPP)                                                             \
  case batch_variant(OPP, NN):                                                 \
    batch_tile_bytes<T, FAMILY, NN, OPP>(l, bu, bg, bw);                       \
    break;
    FEMTC_BATCH_CASES(X)
#undef X
  default:
    *bu = *bg = *bw = 0;
  }
}

BatchKernelInfo batch_kernel_f32();
BatchKernelInfo batch_kernel_f32eo();
BatchKernelInfo batch_kernel_f16x2();
BatchKernelInfo batch_kernel_bf16x3();
} // namespace femtc

// Mixed-precision cell kernels: the same five-pass sum factorization as
// cell_kernel.cuh, with every 1D contraction on the tensor cores.
//
// Each contraction is Out^T[pencils x M] = X^T[pencils x K] . T^T[K x M],
// issued as warp-level mma.sync m16n8k16 tiles: 16 pencils per MMA row block,
// the contracted index K = N or Q (<= 10) padded to 16, the output index
// M = Q or N (<= 10) in one or two n-tiles of 8.  Storage stays FP32 (u, y,
// D/G, the shared-memory intermediates); every MMA operand is split into
// low-precision terms and the products are accumulated in FP32:
//   FEMTC_F16X2  : x = hi + lo (FP16 each), rows scaled by a power of two
//                  so the largest entry of each 16-wide row sits at 2^13
//                  (no FP16 overflow, the low term stays normal); products
//                  lo*HI + hi*LO + hi*HI                          (3 MMAs)
//   FEMTC_BF16X3 : x = hi + mid + lo (BF16 each, FP32 range, no scaling);
//                  the six products whose order is at most 2^-16  (6 MMAs)
// The tables are split the same way once per pass from the launch's
// parameter block.  In the fused pass the forward accumulator fragment is
// re-used as the A operand of the backward MMA (the C and A fragment layouts
// of m16n8k16 coincide), so the point-wise D / G work never touches shared
// memory.  Exact semantics only.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "cell_kernel.cuh"

namespace femtc
{

enum Split : int
{
  SPLIT_F16X2 = 0,
  SPLIT_BF16X3 = 1
};

template <int SPLIT>
struct SplitTraits;

template <>
struct SplitTraits<SPLIT_F16X2>
{
  static constexpr int terms = 2;
  static constexpr int nprod = 3;
  // (A term, B term) of product p, smallest first
  static __host__ __device__ constexpr int pa(int p) { return p == 0 ? 1 : 0; }
  static __host__ __device__ constexpr int pb(int p) { return p == 1 ? 1 : 0; }
  static constexpr bool scaled = true;
  static __device__ __forceinline__ uint32_t pack(float a, float b)
  {
    __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
  }
  static __device__ __forceinline__ float round(float x)
  {
    return __half2float(__float2half_rn(x));
  }
  // the two values of a pack() result (a in the low half), as floats
  static __device__ __forceinline__ float2 unpack(uint32_t r)
  {
    return __half22float2(*reinterpret_cast<const __half2*>(&r));
  }
  static __device__ __forceinline__ void mma(float (&d)[4], const uint32_t (&a)[4],
                                             uint32_t b0, uint32_t b1)
  {
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 "
                 "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
  }
  static __device__ __forceinline__ void mma8(float (&d)[4], const uint32_t (&a)[2], uint32_t b0)
  {
    asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.f16.f16.f32 "
                 "{%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(b0));
  }
};

template <>
struct SplitTraits<SPLIT_BF16X3>
{
  static constexpr int terms = 3;
  static constexpr int nprod = 6;
  // (A term, B term) of product p: (2,0) (1,1) (0,2) (1,0) (0,1) (0,0)
  static __host__ __device__ constexpr int pa(int p)
  {
    return p == 0 ? 2 : (p == 1 || p == 3) ? 1 : 0;
  }
  static __host__ __device__ constexpr int pb(int p)
  {
    return p == 2 ? 2 : (p == 1 || p == 4) ? 1 : 0;
  }
  static constexpr bool scaled = false;
  static __device__ __forceinline__ uint32_t pack(float a, float b)
  {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
  }
  static __device__ __forceinline__ float round(float x)
  {
    return __bfloat162float(__float2bfloat16_rn(x));
  }
  // the two values of a pack() result (a in the low half), as floats: a
  // BF16 value is the high half of its FP32 bit pattern
  static __device__ __forceinline__ float2 unpack(uint32_t r)
  {
    return make_float2(__uint_as_float(r << 16), __uint_as_float(r & 0xffff0000u));
  }
  static __device__ __forceinline__ void mma(float (&d)[4], const uint32_t (&a)[4],
                                             uint32_t b0, uint32_t b1)
  {
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
                 "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
  }
  static __device__ __forceinline__ void mma8(float (&d)[4], const uint32_t (&a)[2], uint32_t b0)
  {
    asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.bf16.bf16.f32 "
                 "{%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(b0));
  }
};

// Power-of-two scale that puts max|x| of a row in [2^13, 2^14) (FP16 split);
// 1 for an all-zero row.  Exact to apply and to undo.
__device__ __forceinline__ float row_scale(float m)
{
  const int e = (__float_as_int(m) >> 23) & 0xff; // biased exponent of max
  if (e == 0)
    return 1.0f;
  int se = 127 + 13 - (e - 127);
  se = se < 1 ? 1 : (se > 254 ? 254 : se);
  return __int_as_float(se << 23);
}

// K extent of the MMA instruction for a contraction of K terms: m16n8k8 for
// K <= 8 (every contraction up to degree 6 at Q <= 8), else m16n8k16.  The
// k8 form gathers and splits half the A values per thread.
__host__ __device__ constexpr int kblock(int K) { return K <= 8 ? 8 : 16; }

// A operand of one 16-row block: v[0..1] row g (k=2t,2t+1), v[2..3] row g+8,
// and for KB = 16 v[4..5] row g (k=2t+8,2t+9), v[6..7] row g+8 -- the
// m16n8k8 / m16n8k16 A layouts.
template <int SPLIT, int KB = 16>
struct AFrag
{
  using Tr = SplitTraits<SPLIT>;
  static constexpr int NV = KB / 2, NR = KB / 4;
  uint32_t r[Tr::terms][NR];
  float inv0, inv1; // undo the row scales of rows g and g+8

  __device__ __forceinline__ void build(float (&v)[NV])
  {
    float s0 = 1.0f, s1 = 1.0f;
    if constexpr (Tr::scaled)
    {
      float m0 = fmaxf(fabsf(v[0]), fabsf(v[1]));
      float m1 = fmaxf(fabsf(v[2]), fabsf(v[3]));
      if constexpr (KB == 16)
      {
        m0 = fmaxf(m0, fmaxf(fabsf(v[4]), fabsf(v[5])));
        m1 = fmaxf(m1, fmaxf(fabsf(v[6]), fabsf(v[7])));
      }
      m0 = fmaxf(m0, __shfl_xor_sync(0xffffffffu, m0, 1));
      m0 = fmaxf(m0, __shfl_xor_sync(0xffffffffu, m0, 2));
      m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, 1));
      m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, 2));
      s0 = row_scale(m0);
      s1 = row_scale(m1);
#pragma unroll
      for (int q = 0; q < NR; ++q) // values 2q, 2q+1 share a row
      {
        const float2 sv = __fmul2_rn(make_float2(v[2 * q], v[2 * q + 1]),
                                     make_float2((q & 1) ? s1 : s0, (q & 1) ? s1 : s0));
        v[2 * q] = sv.x;
        v[2 * q + 1] = sv.y;
      }
    }
    inv0 = 1.0f / s0;
    inv1 = 1.0f / s1;
    // Each term: the pair rounded and packed in one conversion, the packed
    // values read back, and the remainder v - h formed for both values in
    // one packed FMA (the same values as rounding and subtracting one at a
    // time).
#pragma unroll
    for (int j = 0; j < Tr::terms; ++j)
#pragma unroll
      for (int q = 0; q < NR; ++q)
      {
        r[j][q] = Tr::pack(v[2 * q], v[2 * q + 1]);
        if (j + 1 < Tr::terms)
        {
          const float2 h = Tr::unpack(r[j][q]);
          const float2 d = __ffma2_rn(h, make_float2(-1.0f, -1.0f),
                                      make_float2(v[2 * q], v[2 * q + 1]));
          v[2 * q] = d.x;
          v[2 * q + 1] = d.y;
        }
      }
  }
};

// B operand of one table orientation and n-tile, split into terms:
// B[k][n] = tab[n*SN + k*SK] for k < K, n < M (zero elsewhere).
template <int SPLIT, int KB = 16>
struct BFrag
{
  using Tr = SplitTraits<SPLIT>;
  static constexpr int NV = KB / 4, NR = KB / 8;
  uint32_t r[Tr::terms][NR];

  template <int K, int M, int SN, int SK>
  __device__ __forceinline__ void build(const float* __restrict__ tab, int ntile)
  {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int n = ntile * 8 + g;
    float v[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i)
    {
      const int k = 2 * t + (i & 1) + (i >> 1) * 8;
      v[i] = (k < K && n < M) ? tab[n * SN + k * SK] : 0.0f;
    }
#pragma unroll
    for (int j = 0; j < Tr::terms; ++j)
    {
      float h[NV];
#pragma unroll
      for (int i = 0; i < NV; ++i)
      {
        h[i] = (j + 1 < Tr::terms) ? Tr::round(v[i]) : v[i];
        v[i] -= h[i];
      }
#pragma unroll
      for (int q = 0; q < NR; ++q)
        r[j][q] = Tr::pack(h[2 * q], h[2 * q + 1]);
    }
  }
};

// Tables of one contraction: NT n-tiles of one orientation.
template <int SPLIT, int K, int M, bool FWD, int Q>
struct Table
{
  static constexpr int NT = (M + 7) / 8;
  static constexpr int KB = kblock(K);
  BFrag<SPLIT, KB> f[NT];
  __device__ __forceinline__ void build(const float* __restrict__ tab)
  {
#pragma unroll
    for (int j = 0; j < NT; ++j)
    {
      if constexpr (FWD) // out q, contracted i: B[k=i][n=q] = tab[q + i*Q]
        f[j].template build<K, M, 1, Q>(tab, j);
      else // exact transpose: out i, contracted q: B[k=q][n=i] = tab[q + i*Q]
        f[j].template build<K, M, Q, 1>(tab, j);
    }
  }
};

template <int SPLIT, int NT>
struct Acc
{
  float d[NT][4];
  __device__ __forceinline__ void zero()
  {
#pragma unroll
    for (int j = 0; j < NT; ++j)
      d[j][0] = d[j][1] = d[j][2] = d[j][3] = 0.0f;
  }
  template <int K, int M, bool FWD, int Q>
  __device__ __forceinline__ void mma(const AFrag<SPLIT, kblock(K)>& a,
                                      const Table<SPLIT, K, M, FWD, Q>& b)
  {
    using Tr = SplitTraits<SPLIT>;
#pragma unroll
    for (int j = 0; j < NT; ++j)
#pragma unroll
      for (int p = 0; p < Tr::nprod; ++p)
      {
        if constexpr (kblock(K) == 16)
          Tr::mma(d[j], a.r[Tr::pa(p)], b.f[j].r[Tr::pb(p)][0], b.f[j].r[Tr::pb(p)][1]);
        else
          Tr::mma8(d[j], a.r[Tr::pa(p)], b.f[j].r[Tr::pb(p)][0]);
      }
  }
  // undo the A-row scales (rows g and g+8) and add into `o`
  template <int KB>
  __device__ __forceinline__ void unscale_into(const AFrag<SPLIT, KB>& a, float (&o)[NT][4]) const
  {
#pragma unroll
    for (int j = 0; j < NT; ++j)
    {
      o[j][0] += d[j][0] * a.inv0;
      o[j][1] += d[j][1] * a.inv0;
      o[j][2] += d[j][2] * a.inv1;
      o[j][3] += d[j][3] * a.inv1;
    }
  }
};

// Gather the A values of rows r0 = base+g, r1 = base+g+8 of a pencil pass:
// element k of pencil r is src[idx(r) + k*stride], k < K; zero past K or np.
template <int K, typename Idx>
__device__ __forceinline__ void gather(const float* __restrict__ src, Idx idx,
                                       int stride, int base, int np,
                                       float (&v)[kblock(K) / 2])
{
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int r0 = base + g, r1 = base + g + 8;
  const bool ok0 = r0 < np, ok1 = r1 < np;
  const int b0 = ok0 ? idx(r0) : 0, b1 = ok1 ? idx(r1) : 0;
#pragma unroll
  for (int i = 0; i < kblock(K) / 2; ++i)
  {
    const int k = 2 * t + (i & 1) + ((i >> 2) & 1) * 8;
    const bool row1 = (i >> 1) & 1;
    const bool ok = (k < K) && (row1 ? ok1 : ok0);
    v[i] = ok ? src[(row1 ? b1 : b0) + k * stride] : 0.0f;
  }
}

// Scatter an accumulator of rows r0, r1: output m of pencil r goes to
// dst[idx(r) + m*stride], m < M.
template <int M, int NT, typename Idx>
__device__ __forceinline__ void scatter(float* __restrict__ dst, Idx idx,
                                        int stride, int base, int np,
                                        const float (&o)[NT][4])
{
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int r0 = base + g, r1 = base + g + 8;
  if (r0 < np)
  {
    const int b = idx(r0);
#pragma unroll
    for (int j = 0; j < NT; ++j)
#pragma unroll
      for (int e = 0; e < 2; ++e)
      {
        const int m = j * 8 + 2 * t + e;
        if (m < M)
          dst[b + m * stride] = o[j][e];
      }
  }
  if (r1 < np)
  {
    const int b = idx(r1);
#pragma unroll
    for (int j = 0; j < NT; ++j)
#pragma unroll
      for (int e = 0; e < 2; ++e)
      {
        const int m = j * 8 + 2 * t + e;
        if (m < M)
          dst[b + m * stride] = o[j][2 + e];
      }
  }
}

template <int NT>
__device__ __forceinline__ void zero(float (&o)[NT][4])
{
#pragma unroll
  for (int j = 0; j < NT; ++j)
    o[j][0] = o[j][1] = o[j][2] = o[j][3] = 0.0f;
}

// The rows (pencils) of a pass one warp covers: 16-row blocks starting at
// r0 + b0*16, every bs-th block, below r1.  Whole CTA: {0, np, warp,
// warps}; one warp of the warp-split loop: {its cells' rows, 0, 1}.
struct Rows
{
  int r0, r1, b0, bs;
};

__device__ __forceinline__ Rows rows_of(const Part& w, int rows_per_cell)
{
  if (w.nthr == 32 && blockDim.x != 32) // one warp's cells
    return Rows{w.c0 * rows_per_cell, w.c1 * rows_per_cell, 0, 1};
  return Rows{0, w.c1 * rows_per_cell, (int)(threadIdx.x >> 5), (int)(blockDim.x >> 5)};
}

// One contraction of a pass with up to two (input, table) terms summed:
// out = T_a^(dir) in_a [+ T_b^(dir) in_b].
template <int SPLIT, int K, int M, bool FWD, int Q, bool TWO = false,
          typename InIdx, typename OutIdx>
__device__ __forceinline__ void contract_pass(
    const float* __restrict__ in_a, const Table<SPLIT, K, M, FWD, Q>& ta,
    const float* __restrict__ in_b, const Table<SPLIT, K, M, FWD, Q>& tb,
    InIdx iidx, int istride, float* __restrict__ out, OutIdx oidx,
    int ostride, const Rows& rw)
{
  constexpr int NT = (M + 7) / 8;
  const int np = rw.r1;
  for (int base = rw.r0 + rw.b0 * 16; base < np; base += rw.bs * 16)
  {
    float o[NT][4];
    zero(o);
    {
      float v[kblock(K) / 2];
      gather<K>(in_a, iidx, istride, base, np, v);
      AFrag<SPLIT, kblock(K)> a;
      a.build(v);
      Acc<SPLIT, NT> acc;
      acc.zero();
      acc.mma(a, ta);
      acc.unscale_into(a, o);
    }
    if constexpr (TWO)
    {
      float v[kblock(K) / 2];
      gather<K>(in_b, iidx, istride, base, np, v);
      AFrag<SPLIT, kblock(K)> a;
      a.build(v);
      Acc<SPLIT, NT> acc;
      acc.zero();
      acc.mma(a, tb);
      acc.unscale_into(a, o);
    }
    scatter<M, NT>(out, oidx, ostride, base, np, o);
  }
}

// Two contractions of the same input with two tables (one gather and one
// split of A for both): out_a = T_a in, out_b = T_b in.
template <int SPLIT, int K, int M, bool FWD, int Q, typename InIdx, typename OutIdx>
__device__ __forceinline__ void contract_pass_shared(
    const float* __restrict__ in, const Table<SPLIT, K, M, FWD, Q>& ta,
    const Table<SPLIT, K, M, FWD, Q>& tb, InIdx iidx, int istride,
    float* __restrict__ out_a, float* __restrict__ out_b, OutIdx oidx, int ostride,
    const Rows& rw)
{
  constexpr int NT = (M + 7) / 8;
  const int np = rw.r1;
  for (int base = rw.r0 + rw.b0 * 16; base < np; base += rw.bs * 16)
  {
    float v[kblock(K) / 2];
    gather<K>(in, iidx, istride, base, np, v);
    AFrag<SPLIT, kblock(K)> a;
    a.build(v);
    {
      Acc<SPLIT, NT> acc;
      acc.zero();
      acc.mma(a, ta);
      float o[NT][4];
      zero(o);
      acc.unscale_into(a, o);
      scatter<M, NT>(out_a, oidx, ostride, base, np, o);
    }
    {
      Acc<SPLIT, NT> acc;
      acc.zero();
      acc.mma(a, tb);
      float o[NT][4];
      zero(o);
      acc.unscale_into(a, o);
      scatter<M, NT>(out_b, oidx, ostride, base, np, o);
    }
  }
}

template <int SPLIT, int N, int Q, int OP>
struct MmaTile
{
  static constexpr int kStages = 2;
  // CTA-wide streaming (stream_tiles).  The passes also run on one warp's
  // cells (Part/Rows), but the warp-split loop measured 10-20% slower for
  // these tiles: a warp's own rows fill fewer whole 16-row blocks.
  static constexpr bool kWarpSplit = false;
  using S = Shape<N, Q, OP, SEM_EXACT>;
  using T = float;
  static constexpr bool kSlabCopies = false;
  static constexpr int US = N * N;

  static __host__ __device__ unsigned work_bytes(const CellParams<float>& p)
  {
    return (unsigned)p.cb * S::work * sizeof(float);
  }

  // between passes: the CTA, or one warp for its own cells
  static __device__ __forceinline__ void sync(const Part& pt)
  {
    if (pt.nthr == 32)
      __syncwarp();
    else
      __syncthreads();
  }

  static __device__ __forceinline__ void forward(const TabView<float>& p,
                                                 const float* __restrict__ su,
                                                 float* __restrict__ w, int ncb)
  {
    forward(p, su, w, cta_part(ncb));
  }
  static __device__ __forceinline__ void forward(const TabView<float>& p,
                                                 const float* __restrict__ su,
                                                 float* __restrict__ w, const Part& pt)
  {
    pass1(p, su, w, pt);
    sync(pt);
    pass2(p, w, pt);
  }

  // (the last argument is the slab tiles' L2 prefetch hint; not used here)
  static __device__ __forceinline__ void fused(const TabView<float>& p,
                                               float* __restrict__ w, int ncb,
                                               const float* __restrict__ geo,
                                               long long geo_cell0, bool = false)
  {
    fused(p, w, cta_part(ncb), geo, geo_cell0);
  }
  static __device__ __forceinline__ void fused(const TabView<float>& p,
                                               float* __restrict__ w, const Part& pt,
                                               const float* __restrict__ geo,
                                               long long geo_cell0, bool = false)
  {
    pass3(p, w, pt, geo, geo_cell0);
    sync(pt);
    pass4(p, w, pt);
  }

  static __device__ __forceinline__ void backward(const TabView<float>& p,
                                                  const float* __restrict__ w,
                                                  float* __restrict__ sy, int ncb)
  {
    pass5(p, w, sy, cta_part(ncb));
  }
  static __device__ __forceinline__ void backward(const TabView<float>& p,
                                                  const float* __restrict__ w,
                                                  float* __restrict__ sy, const Part& pt)
  {
    pass5(p, w, sy, pt);
  }

  // Pass 1: axis 2, u[c][i0][i1][i2] -> A[c][i0][i1][q2]
  static __device__ __forceinline__ void pass1(const TabView<float>& p,
                                               const float* __restrict__ su,
                                               float* __restrict__ w, const Part& pt)
  {
    const int ncb = pt.ncb;
    float* A0 = w;
    float* A1 = w + ncb * S::SA;
    const Rows np = rows_of(pt, N * N);
    auto iidx = [](int r) { const int c = r / (N * N); return c * S::N3 + (r - c * (N * N)) * N; };
    auto oidx = [](int r) { const int c = r / (N * N); return c * S::SA + (r - c * (N * N)) * S::QP; };
    Table<SPLIT, N, Q, true, Q> phi;
    phi.build(p.P);
    if constexpr (OP == OP_STIFFNESS)
    {
      Table<SPLIT, N, Q, true, Q> gam;
      gam.build(p.D);
      contract_pass_shared<SPLIT, N, Q, true, Q>(su, phi, gam, iidx, 1, A0, A1, oidx, 1, np);
    }
    else
    {
      contract_pass<SPLIT, N, Q, true, Q>(su, phi, su, phi, iidx, 1, A0, oidx, 1, np);
    }
  }

  // Pass 2: axis 1, A[c][i0][i1][q2] -> B[c][i0][q1][q2]
  static __device__ __forceinline__ void pass2(const TabView<float>& p,
                                               float* __restrict__ w, const Part& pt)
  {
    const int ncb = pt.ncb;
    const float* A0 = w;
    const float* A1 = w + ncb * S::SA;
    float* B0 = w + ncb * S::nA * S::SA;
    float* B1 = B0 + ncb * S::SB;
    float* B2 = B1 + ncb * S::SB;
    const Rows np = rows_of(pt, N * Q);
    auto iidx = [](int r) {
      const int c = r / (N * Q), rr = r - c * (N * Q), i0 = rr / Q, q2 = rr - i0 * Q;
      return c * S::SA + i0 * N * S::QP + q2;
    };
    auto oidx = [](int r) {
      const int c = r / (N * Q), rr = r - c * (N * Q), i0 = rr / Q, q2 = rr - i0 * Q;
      return c * S::SB + i0 * S::QQP + q2;
    };
    Table<SPLIT, N, Q, true, Q> phi;
    phi.build(p.P);
    if constexpr (OP == OP_STIFFNESS)
    {
      Table<SPLIT, N, Q, true, Q> gam;
      gam.build(p.D);
      // A0 feeds both Phi (-> B0) and Gamma (-> B1): one gather and split
      contract_pass_shared<SPLIT, N, Q, true, Q>(A0, phi, gam, iidx, S::QP, B0, B1, oidx, S::BQ, np);
      contract_pass<SPLIT, N, Q, true, Q>(A1, phi, A1, phi, iidx, S::QP, B2, oidx, S::BQ, np);
    }
    else
    {
      contract_pass<SPLIT, N, Q, true, Q>(A0, phi, A0, phi, iidx, S::QP, B0, oidx, S::BQ, np);
    }
  }

  // Pass 3 (fused, registers only between the two MMAs): axis 0 forward,
  // D scaling / G transform, axis 0 backward; in place in B.
  static __device__ __forceinline__ void pass3(const TabView<float>& p,
                                               float* __restrict__ w, const Part& pt,
                                               const float* __restrict__ geo,
                                               long long geo_cell0)
  {
    constexpr int NTQ = (Q + 7) / 8, NTN = (N + 7) / 8;
    const int ncb = pt.ncb;
    float* B0 = w + ncb * S::nA * S::SA;
    float* B1 = B0 + ncb * S::SB;
    float* B2 = B1 + ncb * S::SB;
    const Rows rw = rows_of(pt, Q * Q);
    const int np = rw.r1;
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    auto bidx = [](int r) {
      const int c = r / (Q * Q), rr = r - c * (Q * Q), q1 = rr / Q;
      return c * S::SB + q1 * S::BQ + (rr - q1 * Q);
    };
    Table<SPLIT, N, Q, true, Q> fphi;
    Table<SPLIT, Q, N, false, Q> bphi;
    fphi.build(p.P);
    bphi.build(p.P);
    for (int base = rw.r0 + rw.b0 * 16; base < np; base += rw.bs * 16)
    {
      const int r0 = base + g, r1 = base + g + 8;
      // geometry offsets of rows r0, r1: point (c, q0, rr) at
      // ((geo_cell0 + c)*Q3 + q0*Q*Q + rr)*NC
      auto gofs = [&](int r) -> long long {
        const int c = r / (Q * Q), rr = r - c * (Q * Q);
        return ((geo_cell0 + c) * S::Q3 + rr) * S::NC;
      };
      const long long go0 = r0 < np ? gofs(r0) : -1, go1 = r1 < np ? gofs(r1) : -1;
      if constexpr (OP == OP_MASS)
      {
        float v[kblock(N) / 2];
        gather<N>(B0, bidx, S::QQP, base, np, v);
        AFrag<SPLIT, kblock(N)> a;
        a.build(v);
        Acc<SPLIT, NTQ> acc;
        acc.zero();
        acc.mma(a, fphi);
        float f[NTQ][4];
        zero(f);
        acc.unscale_into(a, f);
        // scale by D at (row, q0)
#pragma unroll
        for (int j = 0; j < NTQ; ++j)
#pragma unroll
          for (int e = 0; e < 4; ++e)
          {
            const int q0 = j * 8 + 2 * t + (e & 1);
            const long long go = (e < 2) ? go0 : go1;
            f[j][e] = (q0 < Q && go >= 0) ? f[j][e] * geo[go + q0 * Q * Q] : 0.0f;
          }
        float vb[kblock(Q) / 2];
        to_operand<NTQ>(f, vb);
        AFrag<SPLIT, kblock(Q)> ab;
        ab.build(vb);
        Acc<SPLIT, NTN> accb;
        accb.zero();
        accb.mma(ab, bphi);
        float o[NTN][4];
        zero(o);
        accb.unscale_into(ab, o);
        scatter<N, NTN>(B0, bidx, S::QQP, base, np, o);
      }
      else
      {
        Table<SPLIT, N, Q, true, Q> fgam;
        fgam.build(p.D);
        float fx[NTQ][4], fy[NTQ][4], fz[NTQ][4];
        zero(fx);
        zero(fy);
        zero(fz);
        {
          float v[kblock(N) / 2];
          gather<N>(B0, bidx, S::QQP, base, np, v); // AA -> d/dx: Gamma on axis 0
          AFrag<SPLIT, kblock(N)> a;
          a.build(v);
          Acc<SPLIT, NTQ> acc;
          acc.zero();
          acc.mma(a, fgam);
          acc.unscale_into(a, fx);
        }
        {
          float v[kblock(N) / 2];
          gather<N>(B1, bidx, S::QQP, base, np, v); // AG -> d/dy
          AFrag<SPLIT, kblock(N)> a;
          a.build(v);
          Acc<SPLIT, NTQ> acc;
          acc.zero();
          acc.mma(a, fphi);
          acc.unscale_into(a, fy);
        }
        {
          float v[kblock(N) / 2];
          gather<N>(B2, bidx, S::QQP, base, np, v); // BA -> d/dz
          AFrag<SPLIT, kblock(N)> a;
          a.build(v);
          Acc<SPLIT, NTQ> acc;
          acc.zero();
          acc.mma(a, fphi);
          acc.unscale_into(a, fz);
        }
        // G transform (src/stiffness.hpp:14-29), [zz,yz,xz,yy,xy,xx]
#pragma unroll
        for (int j = 0; j < NTQ; ++j)
#pragma unroll
          for (int e = 0; e < 4; ++e)
          {
            const int q0 = j * 8 + 2 * t + (e & 1);
            const long long go = (e < 2) ? go0 : go1;
            float a0 = 0.f, a1 = 0.f, a2 = 0.f;
            if (q0 < Q && go >= 0)
            {
              const float* G = geo + go + (long long)q0 * Q * Q * 6;
              const float w0 = fx[j][e], w1 = fy[j][e], w2 = fz[j][e];
              a0 = G[5] * w0 + G[4] * w1 + G[2] * w2;
              a1 = G[4] * w0 + G[3] * w1 + G[1] * w2;
              a2 = G[2] * w0 + G[1] * w1 + G[0] * w2;
            }
            fx[j][e] = a0;
            fy[j][e] = a1;
            fz[j][e] = a2;
          }
        Table<SPLIT, Q, N, false, Q> bgam;
        bgam.build(p.D);
        backward_store<NTQ, NTN>(fx, bgam, B0, bidx, base, np);
        backward_store<NTQ, NTN>(fy, bphi, B1, bidx, base, np);
        backward_store<NTQ, NTN>(fz, bphi, B2, bidx, base, np);
      }
    }
  }

  // accumulator fragment (rows g, g+8; cols 2t,2t+1 [+8]) -> A values
  template <int NTQ, int NV>
  static __device__ __forceinline__ void to_operand(const float (&f)[NTQ][4], float (&v)[NV])
  {
    v[0] = f[0][0];
    v[1] = f[0][1];
    v[2] = f[0][2];
    v[3] = f[0][3];
    if constexpr (NV == 8)
    {
      if constexpr (NTQ > 1)
      {
        v[4] = f[1][0];
        v[5] = f[1][1];
        v[6] = f[1][2];
        v[7] = f[1][3];
      }
      else
      {
        v[4] = v[5] = v[6] = v[7] = 0.0f;
      }
    }
  }

  template <int NTQ, int NTN, typename Idx>
  static __device__ __forceinline__ void backward_store(
      const float (&f)[NTQ][4], const Table<SPLIT, Q, N, false, Q>& tb,
      float* __restrict__ dst, Idx idx, int base, int np)
  {
    float v[kblock(Q) / 2];
    to_operand<NTQ>(f, v);
    AFrag<SPLIT, kblock(Q)> a;
    a.build(v);
    Acc<SPLIT, NTN> acc;
    acc.zero();
    acc.mma(a, tb);
    float o[NTN][4];
    zero(o);
    acc.unscale_into(a, o);
    scatter<N, NTN>(dst, idx, S::QQP, base, np, o);
  }

  // Pass 4: backward axis 1, B[c][i0][q1][q2] -> A[c][i0][i1][q2]
  static __device__ __forceinline__ void pass4(const TabView<float>& p,
                                               float* __restrict__ w, const Part& pt)
  {
    const int ncb = pt.ncb;
    float* A0 = w;
    float* A1 = w + ncb * S::SA;
    const float* B0 = w + ncb * S::nA * S::SA;
    const float* B1 = B0 + ncb * S::SB;
    const float* B2 = B1 + ncb * S::SB;
    const Rows np = rows_of(pt, N * Q);
    auto iidx = [](int r) {
      const int c = r / (N * Q), rr = r - c * (N * Q), i0 = rr / Q, q2 = rr - i0 * Q;
      return c * S::SB + i0 * S::QQP + q2;
    };
    auto oidx = [](int r) {
      const int c = r / (N * Q), rr = r - c * (N * Q), i0 = rr / Q, q2 = rr - i0 * Q;
      return c * S::SA + i0 * N * S::QP + q2;
    };
    Table<SPLIT, Q, N, false, Q> phi;
    phi.build(p.P);
    if constexpr (OP == OP_MASS)
    {
      contract_pass<SPLIT, Q, N, false, Q>(B0, phi, B0, phi, iidx, S::BQ, A0, oidx, S::QP, np);
    }
    else
    {
      Table<SPLIT, Q, N, false, Q> gam;
      gam.build(p.D);
      // U1 = Phi^T X + Gamma^T Y ; U2 = Phi^T Z
      contract_pass<SPLIT, Q, N, false, Q, true>(B0, phi, B1, gam, iidx, S::BQ, A0, oidx, S::QP, np);
      contract_pass<SPLIT, Q, N, false, Q>(B2, phi, B2, phi, iidx, S::BQ, A1, oidx, S::QP, np);
    }
  }

  // Pass 5: backward axis 2, A[c][i0][i1][q2] -> y[c][i0][i1][i2]
  static __device__ __forceinline__ void pass5(const TabView<float>& p,
                                               const float* __restrict__ w,
                                               float* __restrict__ sy, const Part& pt)
  {
    const int ncb = pt.ncb;
    const float* A0 = w;
    const float* A1 = w + ncb * S::SA;
    const Rows np = rows_of(pt, N * N);
    auto iidx = [](int r) { const int c = r / (N * N); return c * S::SA + (r - c * (N * N)) * S::QP; };
    auto oidx = [](int r) { const int c = r / (N * N); return c * S::N3 + (r - c * (N * N)) * N; };
    Table<SPLIT, Q, N, false, Q> phi;
    phi.build(p.P);
    if constexpr (OP == OP_MASS)
    {
      contract_pass<SPLIT, Q, N, false, Q>(A0, phi, A0, phi, iidx, 1, sy, oidx, 1, np);
    }
    else
    {
      Table<SPLIT, Q, N, false, Q> gam;
      gam.build(p.D);
      contract_pass<SPLIT, Q, N, false, Q, true>(A0, phi, A1, gam, iidx, 1, sy, oidx, 1, np);
    }
  }
};

template <int SPLIT, int N, int Q, int OP>
__global__ void __launch_bounds__(kCellThreads)
    mma_kernel(const __grid_constant__ CellParams<float> p)
{
  stream_tiles<float, MmaTile<SPLIT, N, Q, OP>, N, Q, geo_nc(OP)>(p);
}

} // namespace femtc

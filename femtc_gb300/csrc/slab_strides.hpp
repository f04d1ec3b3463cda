// Work-buffer strides of the slab kernels (cell_kernel.cuh), per (N, Q,
// bytes per arithmetic value, lanes per slab): a slab (cell c, i0) of the
// B buffers starts at c*sbc + i0*sq.  The forward and backward passes
// access the buffers with one thread (or `lanes` threads) per slab, the
// fused pass with one thread per pencil; the strides minimise the modelled
// shared-memory wavefronts of both patterns (32 four-byte banks; 8-byte
// values served per half warp) over sq in [Q^2, Q^2+32) and sbc in
// [N*sq, N*sq+32), then the footprint.  slab_strides_gen.cpp computes this
// table; tests/test_slab_strides.py checks it against the generator.
// Device code takes the strides as compile-time constants (immediate
// offsets in every shared-memory access); the host sizes tiles with the
// same values.
#pragma once

namespace femtc
{
struct SlabStride
{
  int n, q, esize, lanes, sq, sbc;
};

constexpr SlabStride kSlabStrides[] = {
    {2, 2, 4, 1, 5, 10},
    {2, 3, 4, 1, 16, 41},
    {2, 4, 4, 1, 16, 33},
    {3, 3, 4, 1, 35, 105},
    {3, 4, 4, 1, 17, 51},
    {3, 5, 4, 1, 51, 153},
    {4, 4, 4, 1, 17, 68},
    {4, 5, 4, 1, 40, 185},
    {4, 6, 4, 1, 37, 164},
    {5, 5, 4, 1, 37, 185},
    {5, 6, 4, 1, 37, 185},
    {5, 7, 4, 1, 61, 305},
    {6, 6, 4, 1, 37, 222},
    {6, 7, 4, 1, 49, 294},
    {6, 8, 4, 1, 65, 390},
    {7, 7, 4, 1, 71, 497},
    {7, 8, 4, 1, 65, 455},
    {7, 9, 4, 1, 103, 721},
    {8, 8, 4, 1, 65, 520},
    {8, 9, 4, 1, 84, 689},
    {8, 10, 4, 1, 100, 801},
    {9, 9, 4, 1, 105, 945},
    {9, 10, 4, 1, 101, 909},
    {2, 2, 4, 2, 6, 12},
    {2, 3, 4, 2, 10, 20},
    {2, 4, 4, 2, 16, 34},
    {3, 3, 4, 2, 10, 41},
    {3, 4, 4, 2, 18, 54},
    {3, 5, 4, 2, 26, 78},
    {4, 4, 4, 2, 18, 72},
    {4, 5, 4, 2, 26, 104},
    {4, 6, 4, 2, 38, 152},
    {5, 5, 4, 2, 26, 130},
    {5, 6, 4, 2, 38, 190},
    {5, 7, 4, 2, 50, 250},
    {6, 6, 4, 2, 38, 228},
    {6, 7, 4, 2, 50, 300},
    {6, 8, 4, 2, 66, 396},
    {7, 7, 4, 2, 50, 350},
    {7, 8, 4, 2, 66, 462},
    {7, 9, 4, 2, 82, 574},
    {8, 8, 4, 2, 66, 528},
    {8, 9, 4, 2, 82, 656},
    {8, 10, 4, 2, 100, 802},
    {9, 9, 4, 2, 82, 738},
    {9, 10, 4, 2, 102, 918},
    {2, 2, 8, 1, 5, 10},
    {2, 3, 8, 1, 24, 57},
    {2, 4, 8, 1, 17, 34},
    {3, 3, 8, 1, 19, 57},
    {3, 4, 8, 1, 17, 51},
    {3, 5, 8, 1, 35, 105},
    {4, 4, 8, 1, 17, 68},
    {4, 5, 8, 1, 28, 121},
    {4, 6, 8, 1, 37, 148},
    {5, 5, 8, 1, 37, 185},
    {5, 6, 8, 1, 37, 185},
    {5, 7, 8, 1, 61, 305},
    {6, 6, 8, 1, 37, 222},
    {6, 7, 8, 1, 49, 294},
    {6, 8, 8, 1, 65, 390},
    {7, 7, 8, 1, 55, 385},
    {7, 8, 8, 1, 65, 455},
    {7, 9, 8, 1, 87, 609},
    {8, 8, 8, 1, 65, 520},
    {8, 9, 8, 1, 82, 657},
    {8, 10, 8, 1, 101, 808},
    {9, 9, 8, 1, 89, 801},
    {9, 10, 8, 1, 101, 909},
    {2, 2, 8, 2, 6, 12},
    {2, 3, 8, 2, 9, 25},
    {2, 4, 8, 2, 18, 36},
    {3, 3, 8, 2, 10, 30},
    {3, 4, 8, 2, 18, 54},
    {3, 5, 8, 2, 26, 78},
    {4, 4, 8, 2, 18, 72},
    {4, 5, 8, 2, 26, 104},
    {4, 6, 8, 2, 36, 146},
    {5, 5, 8, 2, 26, 130},
    {5, 6, 8, 2, 38, 190},
    {5, 7, 8, 2, 50, 250},
    {6, 6, 8, 2, 38, 228},
    {6, 7, 8, 2, 50, 300},
    {6, 8, 8, 2, 66, 396},
    {7, 7, 8, 2, 50, 350},
    {7, 8, 8, 2, 66, 462},
    {7, 9, 8, 2, 82, 574},
    {8, 8, 8, 2, 66, 528},
    {8, 9, 8, 2, 82, 657},
    {8, 10, 8, 2, 102, 820},
    {9, 9, 8, 2, 82, 738},
    {9, 10, 8, 2, 102, 918}
};

// {sq, sbc} of (n, q, esize, lanes); sq = 0 when the table has no entry.
// Host function: device code uses it only in constant expressions.
constexpr SlabStride slab_strides(int n, int q, int esize, int lanes)
{
  for (const SlabStride& s : kSlabStrides)
    if (s.n == n && s.q == q && s.esize == esize && s.lanes == lanes)
      return s;
  return SlabStride{n, q, esize, lanes, 0, 0};
}
} // namespace femtc

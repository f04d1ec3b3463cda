// Generator of slab_strides.hpp (a maintainer's tool, not part of the
// library build): prints the work-buffer strides {n, q, esize, lanes, sq,
// sbc} of every slab-kernel variant.
//   g++ -O2 slab_strides_gen.cpp -o gen && ./gen
// Cost model: for each candidate (sq in [Q^2, Q^2+32), sbc in [N*sq,
// N*sq+32)), the shared-memory wavefronts of the slab passes' warp accesses
// (thread t of a warp takes slab (t / lanes), lane t % lanes: address
// (sl / N)*sbc + (sl % N)*sq + t % lanes) and of the fused pass's (thread t
// takes pencil t: (t / Q^2)*sbc + t % Q^2), averaged over the accesses of
// one pass; ties go to the smaller footprint.  32 four-byte banks; 8-byte
// values are served per half warp (16 x 8 bytes = one 128-byte wavefront
// when the element indices differ modulo 16).
#include <algorithm>
#include <cstdio>
#include <utility>
int wavefronts(const long long* a, int esize)
{
  if (esize == 4)
  {
    int worst = 0;
    for (int b = 0; b < 32; ++b)
    {
      long long seen[32];
      int n = 0;
      for (int t = 0; t < 32; ++t)
        if (((a[t] % 32) + 32) % 32 == b)
        {
          bool dup = false;
          for (int k = 0; k < n; ++k)
            dup = dup || seen[k] == a[t];
          if (!dup)
            seen[n++] = a[t];
        }
      worst = std::max(worst, n);
    }
    return worst;
  }
  int total = 0;
  for (int h = 0; h < 2; ++h)
  {
    int worst = 0;
    for (int b = 0; b < 16; ++b)
    {
      long long seen[16];
      int n = 0;
      for (int t = 16 * h; t < 16 * h + 16; ++t)
        if (((a[t] % 16) + 16) % 16 == b)
        {
          bool dup = false;
          for (int k = 0; k < n; ++k)
            dup = dup || seen[k] == a[t];
          if (!dup)
            seen[n++] = a[t];
        }
      worst = std::max(worst, n);
    }
    total += worst;
  }
  return total;
}
std::pair<int, int> slab_layout(int n, int q, int esize, int lanes)
{
  const int q2 = q * q;
  double best = 1e30;
  std::pair<int, int> res{q2, n * q2};
  long long a[32];
  for (int sq = q2; sq < q2 + 32; ++sq)
    for (int sbc = n * sq; sbc < n * sq + 32; ++sbc)
    {
      double cost = 0.0;
      for (int mm = 0; mm < n; ++mm)
      {
        for (int t = 0; t < 32; ++t)
        {
          const long long ts = 32LL * mm + t, sl = ts / lanes;
          a[t] = (sl / n) * sbc + (sl % n) * sq + ts % lanes;
        }
        cost += double(wavefronts(a, esize)) / n;
      }
      for (int mm = 0; mm < q2; ++mm)
      {
        for (int t = 0; t < 32; ++t)
        {
          const long long pp = 32LL * mm + t;
          a[t] = (pp / q2) * sbc + pp % q2;
        }
        cost += double(wavefronts(a, esize)) / q2;
      }
      cost += 1e-6 * sbc;
      if (cost < best)
      {
        best = cost;
        res = {sq, sbc};
      }
    }
  return res;
}
int main()
{
  for (int esize : {4, 8})
    for (int lanes : {1, 2})
      for (int n = 2; n <= 9; ++n)
        for (int q = n; q <= n + 2 && q <= 10; ++q)
        {
          auto r = slab_layout(n, q, esize, lanes);
          printf("    {%d, %d, %d, %d, %d, %d},\n", n, q, esize, lanes, r.first, r.second);
        }
}

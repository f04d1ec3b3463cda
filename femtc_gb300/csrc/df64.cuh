// Double-float arithmetic: a value is hi + lo, two FP32 numbers, giving
// about 48 significand bits (unit roundoff ~2^-48) on the FP32 pipes.  On
// GB300 the FP32 FMA rate is about 60x the FP64 rate, so FP64-accurate
// operator results are cheaper this way than with FP64 instructions.
//
// The algorithms are the classical error-free transformations: Dekker's and
// Knuth's TwoSum (Knuth, TAOCP vol. 2, 4.2.2), the FMA-based TwoProduct
// (exact product error e = fma(a, b, -a*b)), and FastTwoSum renormalisation;
// see also Hida, Li and Bailey, "Library for double-double and quad-double
// arithmetic" (2000), whose double-double operations these mirror with FP32
// halves.
//
// Conversions from and to the FP64 storage format use integer bit
// manipulation (no FP64 instructions).  Range: the hi part must be a normal
// FP32 number, |x| in about [1e-30, 3e38]; smaller magnitudes flush to zero
// and lose the low part first (the operator's tolerance is relative to the
// largest entry, so such entries do not matter to it).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace femtc
{
using ::fma; // the float/double overloads stay visible next to df64's

struct df64
{
  float h, l;
  df64() = default;
  __host__ __device__ constexpr df64(float hi, float lo) : h(hi), l(lo) {}
  __host__ __device__ constexpr explicit df64(int v) : h((float)v), l(0.f) {}
};

// s + err = a + b exactly (Knuth's TwoSum, no ordering assumption)
__device__ __forceinline__ float two_sum(float a, float b, float& err)
{
  const float s = a + b;
  const float bb = s - a;
  err = (a - (s - bb)) + (b - bb);
  return s;
}

// s + err = a + b exactly when |a| >= |b| (FastTwoSum)
__device__ __forceinline__ float fast_two_sum(float a, float b, float& err)
{
  const float s = a + b;
  err = b - (s - a);
  return s;
}

// a * b as an unevaluated pair: p + e
__device__ __forceinline__ float two_prod(float a, float b, float& e)
{
  const float p = a * b;
  e = __fmaf_rn(a, b, -p);
  return p;
}

__device__ __forceinline__ df64 operator*(df64 a, df64 b)
{
  float e;
  const float p = two_prod(a.h, b.h, e);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  float lo;
  const float hi = fast_two_sum(p, e, lo);
  return df64(hi, lo);
}

__device__ __forceinline__ df64 operator+(df64 a, df64 b)
{
  float e;
  const float s = two_sum(a.h, b.h, e);
  e += a.l + b.l;
  float lo;
  const float hi = fast_two_sum(s, e, lo);
  return df64(hi, lo);
}

__device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.h, -a.l); }

__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }

__device__ __forceinline__ df64& operator+=(df64& a, df64 b)
{
  a = a + b;
  return a;
}

__device__ __forceinline__ df64& operator*=(df64& a, df64 b)
{
  a = a * b;
  return a;
}

// a * b + c
__device__ __forceinline__ df64 fma(df64 a, df64 b, df64 c)
{
  float e;
  const float p = two_prod(a.h, b.h, e);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  float t;
  const float s = two_sum(p, c.h, t);
  t += e + c.l;
  float lo;
  const float hi = fast_two_sum(s, t, lo);
  return df64(hi, lo);
}

// ---------------------------------------------------------------------------
// Lazy accumulation of a sum of products, sum_k a_k x_k, in double-float:
// the high parts are summed with TwoSum and every rounding error (of the
// products, by the FMA-based TwoProduct, and of the sums) is gathered in one
// FP32 word; the pair is renormalised once, when the value is read.  That is
// the compensated dot product of Ogita, Rump and Oishi ("Accurate sum and
// dot product", SIAM J. Sci. Comput. 26, 2005, Dot2) applied to double-float
// operands: 12 FP32 operations per term instead of 15 for a renormalised
// df64 fma, and only the high-part addition lies on the chain from one term
// to the next.  The result keeps double-float accuracy (about 2^-48
// relative to the sum of |a_k x_k|).
struct df64acc
{
  float s, e; // value s + e, not normalised
};

__device__ __forceinline__ df64acc acc_mul(df64 a, df64 b)
{
  df64acc r;
  r.s = two_prod(a.h, b.h, r.e);
  r.e = __fmaf_rn(a.h, b.l, r.e);
  r.e = __fmaf_rn(a.l, b.h, r.e);
  return r;
}

__device__ __forceinline__ df64acc acc_fma(df64 a, df64 b, df64acc c)
{
  float pe;
  const float p = two_prod(a.h, b.h, pe);
  pe = __fmaf_rn(a.h, b.l, pe);
  pe = __fmaf_rn(a.l, b.h, pe);
  float t;
  c.s = two_sum(c.s, p, t);
  c.e += t + pe;
  return c;
}

__device__ __forceinline__ df64 acc_val(df64acc c)
{
  float lo;
  const float hi = fast_two_sum(c.s, c.e, lo);
  return df64(hi, lo);
}

__device__ __forceinline__ df64acc acc_from(df64 v) { return df64acc{v.h, v.l}; }

// The same interface for plain FP32 / FP64 arithmetic: the accumulator is
// the value and every call is the ordinary operation.
template <typename T>
struct acc_of
{
  using type = T;
};
template <>
struct acc_of<df64>
{
  using type = df64acc;
};
template <typename T>
using acc_t = typename acc_of<T>::type;

template <typename T>
__device__ __forceinline__ acc_t<T> acc_zero();
template <>
__device__ __forceinline__ float acc_zero<float>()
{
  return 0.f;
}
template <>
__device__ __forceinline__ double acc_zero<double>()
{
  return 0.0;
}
template <>
__device__ __forceinline__ df64acc acc_zero<df64>()
{
  return df64acc{0.f, 0.f};
}
__device__ __forceinline__ float acc_mul(float a, float b) { return a * b; }
__device__ __forceinline__ double acc_mul(double a, double b) { return a * b; }
__device__ __forceinline__ float acc_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double acc_fma(double a, double b, double c) { return ::fma(a, b, c); }
__device__ __forceinline__ float acc_val(float c) { return c; }
__device__ __forceinline__ double acc_val(double c) { return c; }
__device__ __forceinline__ float acc_from(float v) { return v; }
__device__ __forceinline__ double acc_from(double v) { return v; }

__device__ __forceinline__ df64 shfl_xor(df64 v, int lane_mask)
{
  return df64(__shfl_xor_sync(0xffffffffu, v.h, lane_mask),
              __shfl_xor_sync(0xffffffffu, v.l, lane_mask));
}

// FP64 -> hi + lo by bit manipulation: hi takes the sign, exponent and the
// top 23 fraction bits (truncation, exact); lo is the remaining 29 fraction
// bits, converted from integer and scaled by the exact power of two.
__device__ __forceinline__ df64 to_df64(double d)
{
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7ffu);
  if (e < 1023 - 126 || e > 1023 + 127) // below FP32 normal range: flush
    return df64(0.f, 0.f);              // (above: not produced by the operators' data)
  const unsigned long long frac = b & 0x000fffffffffffffull;
  const unsigned hb = sign | ((unsigned)(e - 1023 + 127) << 23) | (unsigned)(frac >> 29);
  const unsigned low = (unsigned)(frac & ((1ull << 29) - 1));
  // low * 2^(e - 1023 - 52): integer to float (rounded to 24 bits), exact scale
  const int se = e - 1023 - 52 + 127;
  float lo = 0.f;
  if (se >= 1)
    lo = __uint2float_rn(low) * __int_as_float(se << 23);
  if (sign)
    lo = -lo;
  return df64(__int_as_float((int)hb), lo);
}

__device__ __forceinline__ double to_double(df64 v)
{
  return (double)v.h + (double)v.l;
}

// Host: split an FP64 table entry into hi + lo (for launch parameters).
inline df64 host_df64(double d)
{
  const float h = (float)d;
  return df64(h, (float)(d - (double)h));
}

} // namespace femtc

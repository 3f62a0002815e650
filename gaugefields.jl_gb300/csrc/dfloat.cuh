// Double-float arithmetic: a value is an unevaluated sum hi + lo of two fp32
// numbers with |lo| <= ulp(hi)/2, giving a 48-bit significand (relative
// rounding 2^-48 ~ 3.6e-15 per operation). On GB300 fp32 issues about 64
// times faster than fp64, so the fp64-class parts of the mixed-precision MD
// (the link update with re-unitarisation and the Hamiltonian) run on the fp32
// pipes in this form, with fp64 storage and fp64 global sums.
//
// The building blocks are the error-free transformations of Knuth (TwoSum)
// and Dekker (FastTwoSum, product via fused multiply-add), as collected in
// Hida, Li, Bailey, "Algorithms for quad-double precision floating point
// arithmetic" (ARITH-15, 2001) and Joldes, Muller, Popescu, "Tight and
// rigorous error bounds for basic building blocks of double-word arithmetic"
// (ACM TOMS 44, 2017). The additions below are the "accurate" double-word sum
// (relative error <= 3u^2), the product is DWTimesDW with FMA.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

#define GF_DF_HD __host__ __device__ __forceinline__

namespace gf {
// The type and its operators live in their own namespace so that fabs/sqrt
// for double-floats are found only by argument-dependent lookup and never
// shadow the float/double overloads used elsewhere in namespace gf.
namespace dfns {

struct dfl {
  float hi, lo;
  GF_DF_HD constexpr dfl() : hi(0.f), lo(0.f) {}
  GF_DF_HD constexpr dfl(float h, float l) : hi(h), lo(l) {}
  GF_DF_HD constexpr dfl(int v) : hi((float)v), lo(0.f) {}
  GF_DF_HD constexpr explicit dfl(float v) : hi(v), lo(0.f) {}
  // constexpr so that literal constants are split at compile time
  GF_DF_HD constexpr explicit dfl(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
  GF_DF_HD explicit operator double() const { return (double)hi + (double)lo; }
};

// The rounded product fl(a*b) as a value the compiler cannot fuse into a
// following add (nvcc contracts a*b + c into one FMA by default, which would
// make the error-free transformations below count the product error twice).
GF_DF_HD float df_mul_rn(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}

GF_DF_HD dfl df_two_sum(float a, float b) {
  float s = a + b;
  float bb = s - a;
  float e = (a - (s - bb)) + (b - bb);
  return dfl(s, e);
}
GF_DF_HD dfl df_fast_two_sum(float a, float b) {
  float s = a + b;
  float e = b - (s - a);
  return dfl(s, e);
}
GF_DF_HD dfl df_two_prod(float a, float b) {
  float p = df_mul_rn(a, b);
  float e = fmaf(a, b, -p);
  return dfl(p, e);
}

GF_DF_HD dfl operator+(dfl a, dfl b) {
  dfl s = df_two_sum(a.hi, b.hi);
  dfl t = df_two_sum(a.lo, b.lo);
  float c = s.lo + t.hi;
  dfl v = df_fast_two_sum(s.hi, c);
  float w = t.lo + v.lo;
  return df_fast_two_sum(v.hi, w);
}
// The "sloppy" double-word sum (one TwoSum on the high parts, the low parts
// added plainly): error at most ~2^-47 of max(|a|, |b|) rather than of
// |a + b|, for accumulations whose terms do not cancel to far below their
// own size (the Cayley-Hamilton power series). Eleven operations against
// the twenty of operator+.
GF_DF_HD dfl df_add_fast(dfl a, dfl b) {
  const dfl s = df_two_sum(a.hi, b.hi);
  return df_fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}
GF_DF_HD dfl operator-(dfl a) { return dfl(-a.hi, -a.lo); }
GF_DF_HD dfl operator-(dfl a, dfl b) { return a + (-b); }
GF_DF_HD dfl operator*(dfl a, dfl b) {
  dfl p = df_two_prod(a.hi, b.hi);
  float t = fmaf(a.hi, b.lo, df_mul_rn(a.lo, b.hi));
  return df_fast_two_sum(p.hi, p.lo + t);
}
GF_DF_HD dfl operator/(dfl a, dfl b) {
  float q1 = a.hi / b.hi;
  dfl r = a - b * dfl(q1);
  float q2 = r.hi / b.hi;
  return df_fast_two_sum(q1, q2);
}
GF_DF_HD dfl& operator+=(dfl& a, dfl b) {
  a = a + b;
  return a;
}
GF_DF_HD dfl& operator-=(dfl& a, dfl b) {
  a = a - b;
  return a;
}
GF_DF_HD dfl& operator*=(dfl& a, dfl b) {
  a = a * b;
  return a;
}
GF_DF_HD bool operator<(dfl a, dfl b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
GF_DF_HD bool operator>(dfl a, dfl b) { return b < a; }
GF_DF_HD dfl fabs(dfl a) { return a.hi < 0.f ? -a : a; }
GF_DF_HD dfl sqrt(dfl a) {
  if (a.hi <= 0.f) return dfl(0.f, 0.f);
  float s = sqrtf(a.hi);
  // one Newton step on s: s + (a - s^2) / (2 s)
  dfl s2 = df_two_prod(s, s);
  dfl r = a - s2;
  float c = r.hi / (2.f * s);
  return df_fast_two_sum(s, c);
}

}  // namespace dfns
using dfns::dfl;
using dfns::df_two_sum;
using dfns::df_fast_two_sum;
using dfns::df_two_prod;
using dfns::df_mul_rn;
using dfns::df_add_fast;

// Split an fp64 value into hi + lo fp32 parts without fp64 instructions (on
// GB300 one fp64 warp instruction occupies the fp64 pipe for as long as ~64
// fp32 ones, and these conversions run on every load of a double-float
// kernel): hi keeps the sign, exponent and leading 23 fraction bits
// (truncated), lo the remaining 29 bits rounded to fp32, so hi + lo equals the
// double to 2^-48 relative, the precision of double-float arithmetic. The
// 29-bit remainder becomes a float through two exact 2^23-offset
// constructions and one fused multiply-add (no integer conversion
// instruction). Magnitudes in [2^-74, 2^128) take this path; smaller ones
// flush to a signed zero (far below 2^-48 of every value they meet on this
// path; keeping hi alone for them measured 5-12% slower in every
// double-float kernel), larger ones and infinities give a signed infinity and
// NaN a NaN.
__device__ __forceinline__ dfl df_from_double(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned int w1 = (unsigned int)(b >> 32), w0 = (unsigned int)b;
  const unsigned int sign = w1 & 0x80000000u;
  const int e = (int)((w1 >> 20) & 0x7FFu);
  const unsigned int m23 = ((w1 & 0xFFFFFu) << 3) | (w0 >> 29);
  const unsigned int r = w0 & 0x1FFFFFFFu;
  const float two23 = 8388608.0f;
  const float rl = __uint_as_float(0x4B000000u | (r & 0x7FFFFFu)) - two23;  // exact
  const float rh = __uint_as_float(0x4B000000u | (r >> 23)) - two23;        // exact
  const float rv = fmaf(rh, two23, rl);                                      // r rounded to fp32
  // lo = r * 2^(e - 1023 - 52): the scale's exponent field is e - 948
  const float scale = __uint_as_float((unsigned int)(e - 948) << 23);
  float hi = __uint_as_float(sign | ((unsigned int)(e - 896) << 23) | m23);
  float lo = __uint_as_float(__float_as_uint(rv * scale) ^ sign);
  if (e < 949) {
    hi = __uint_as_float(sign);
    lo = 0.f;
  } else if (e > 1150) {
    const bool nan = e == 0x7FF && (m23 | r) != 0u;
    hi = __uint_as_float(sign | 0x7F800000u | (nan ? 0x400000u : 0u));
    lo = 0.f;
  }
  return dfl(hi, lo);
}

// fp32 -> fp64 widening with integer operations only. Zero and subnormal
// parts (only ever the lo part of a value below 2^-100) map to a signed zero;
// infinities and NaN keep their class.
__device__ __forceinline__ double widen_f32(float f) {
  const unsigned int b = __float_as_uint(f);
  const unsigned int e = (b >> 23) & 0xFFu;
  const unsigned long long sign = (unsigned long long)(b >> 31) << 63;
  const unsigned long long ex = e == 0u ? 0ull : (e == 0xFFu ? 0x7FFull : (unsigned long long)(e + 896u));
  const unsigned long long man = e == 0u ? 0ull : (unsigned long long)(b & 0x7FFFFFu) << 29;
  return __longlong_as_double((long long)(sign | (ex << 52) | man));
}

// hi + lo as fp64: two integer widenings and one fp64 add
__device__ __forceinline__ double df_to_double(dfl a) { return widen_f32(a.hi) + widen_f32(a.lo); }

// a kernel result of any arithmetic type as fp64
__device__ __forceinline__ double to_f64(double v) { return v; }
__device__ __forceinline__ double to_f64(float v) { return (double)v; }
__device__ __forceinline__ double to_f64(dfl v) { return df_to_double(v); }

}  // namespace gf

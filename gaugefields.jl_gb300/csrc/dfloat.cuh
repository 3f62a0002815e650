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

// Split an fp64 value into hi + lo fp32 parts with integer operations only:
// hi keeps the sign, exponent and leading 23 fraction bits (truncated), lo the
// remaining 29 bits rounded to fp32, so hi + lo equals the double to 2^-53
// relative. Zero maps to zero; magnitudes between 2^-70 and 2^100 (all link,
// momentum and staple entries) take the integer path, others (never met on
// this path) an fp64 conversion.
__device__ __forceinline__ dfl df_from_double(double d) {
  unsigned long long b = (unsigned long long)__double_as_longlong(d);
  if ((b << 1) == 0ull) return dfl(0.f, 0.f);
  unsigned int sign = (unsigned int)(b >> 63);
  int e = (int)((b >> 52) & 0x7FF);
  if (e < 1023 - 70 || e > 1023 + 100) return dfl((float)d, 0.f);
  unsigned long long mant = b & 0xFFFFFFFFFFFFFull;
  unsigned int hbits = (sign << 31) | ((unsigned int)(e - 1023 + 127) << 23) | (unsigned int)(mant >> 29);
  float hi = __int_as_float((int)hbits);
  unsigned int r = (unsigned int)(mant & 0x1FFFFFFFull);
  // lo = r * 2^(e - 1023 - 52), built from the exponent bits of the scale
  float scale = __int_as_float((int)((unsigned int)(e - 1023 - 52 + 127) << 23));
  float lo = __uint2float_rn(r) * scale;
  return dfl(hi, sign ? -lo : lo);
}

// fp32 -> fp64 widening with integer operations. Zero and subnormal parts
// (only ever the lo part of a value below 2^-100) map to zero; infinities and
// NaN take the fp64 conversion so that they propagate.
__device__ __forceinline__ double widen_f32(float f) {
  unsigned int b = (unsigned int)__float_as_int(f);
  unsigned int e = (b >> 23) & 0xFFu;
  if (e == 0u) return 0.0;
  if (e == 0xFFu) return (double)f;
  unsigned long long d = ((unsigned long long)(b >> 31) << 63) | ((unsigned long long)(e - 127u + 1023u) << 52) |
                         ((unsigned long long)(b & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)d);
}

// hi + lo as fp64: two integer widenings and one fp64 add
__device__ __forceinline__ double df_to_double(dfl a) { return widen_f32(a.hi) + widen_f32(a.lo); }

// a kernel result of any arithmetic type as fp64
__device__ __forceinline__ double to_f64(double v) { return v; }
__device__ __forceinline__ double to_f64(float v) { return (double)v; }
__device__ __forceinline__ double to_f64(dfl v) { return df_to_double(v); }

}  // namespace gf

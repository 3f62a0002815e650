// SU(3) / 3x3 complex matrix arithmetic shared by every kernel of the
// library. Templated on the real type (float for the mixed-precision force
// path, double for the plain FP64 path and for the Hamiltonian pieces).
//
// Conventions follow Gaugefields.jl:
//  * link matrices are row-major 3x3 complex (element (i,j) = row i, column j);
//  * the su(3) coefficient map of a matrix M is the one of
//    Traceless_antihermitian_add! (src/4D/TA_gaugefields_4D_serial.jl:181-269):
//    TA(M) = (M - M^dag)/2 - tr(M - M^dag)/6 = i * sum_a c_a lambda_a / 2;
//  * momenta P = sum_a p_a lambda_a / 2 are Hermitian and the link update is
//    U <- exp(i eps P) U (exptU! of src/4D/TA_gaugefields_4D_serial.jl:760).
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>
#include <type_traits>
#include "dfloat.cuh"

#define GF_HD __host__ __device__ __forceinline__

namespace gf {

template <typename R>
struct cplx {
  R re, im;
};

template <typename R>
GF_HD cplx<R> mk(R re, R im) {
  cplx<R> c;
  c.re = re;
  c.im = im;
  return c;
}
template <typename R>
GF_HD cplx<R> operator+(cplx<R> a, cplx<R> b) { return mk(a.re + b.re, a.im + b.im); }
template <typename R>
GF_HD cplx<R> operator-(cplx<R> a, cplx<R> b) { return mk(a.re - b.re, a.im - b.im); }
template <typename R>
GF_HD cplx<R> operator*(cplx<R> a, cplx<R> b) {
  return mk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
template <typename R>
GF_HD cplx<R> operator*(R s, cplx<R> a) { return mk(s * a.re, s * a.im); }
template <typename R>
GF_HD cplx<R> conj(cplx<R> a) { return mk(a.re, -a.im); }
// a * conj(b)
template <typename R>
GF_HD cplx<R> mulc(cplx<R> a, cplx<R> b) {
  return mk(a.re * b.re + a.im * b.im, a.im * b.re - a.re * b.im);
}
// conj(a) * conj(b)
template <typename R>
GF_HD cplx<R> cmulc(cplx<R> a, cplx<R> b) {
  return mk(a.re * b.re - a.im * b.im, -(a.re * b.im + a.im * b.re));
}
// c += a*b
template <typename R>
GF_HD void fma_(cplx<R>& c, cplx<R> a, cplx<R> b) {
  c.re += a.re * b.re - a.im * b.im;
  c.im += a.re * b.im + a.im * b.re;
}

template <typename R>
struct mat3 {
  cplx<R> e[3][3];
};

template <typename R>
GF_HD mat3<R> zero3() {
  mat3<R> m;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) m.e[i][j] = mk<R>(0, 0);
  return m;
}
template <typename R>
GF_HD mat3<R> ident3() {
  mat3<R> m = zero3<R>();
  m.e[0][0].re = m.e[1][1].re = m.e[2][2].re = R(1);
  return m;
}

// A*B
template <typename R>
GF_HD mat3<R> mul_nn(const mat3<R>& a, const mat3<R>& b) {
  mat3<R> c;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      cplx<R> s = a.e[i][0] * b.e[0][j];
      fma_(s, a.e[i][1], b.e[1][j]);
      fma_(s, a.e[i][2], b.e[2][j]);
      c.e[i][j] = s;
    }
  return c;
}
// A*B^dag
template <typename R>
GF_HD mat3<R> mul_na(const mat3<R>& a, const mat3<R>& b) {
  mat3<R> c;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      cplx<R> s = mulc(a.e[i][0], b.e[j][0]);
      s = s + mulc(a.e[i][1], b.e[j][1]);
      s = s + mulc(a.e[i][2], b.e[j][2]);
      c.e[i][j] = s;
    }
  return c;
}
// A^dag*B
template <typename R>
GF_HD mat3<R> mul_an(const mat3<R>& a, const mat3<R>& b) {
  mat3<R> c;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      cplx<R> s = conj(a.e[0][i]) * b.e[0][j];
      fma_(s, conj(a.e[1][i]), b.e[1][j]);
      fma_(s, conj(a.e[2][i]), b.e[2][j]);
      c.e[i][j] = s;
    }
  return c;
}
// A^dag*B^dag
template <typename R>
GF_HD mat3<R> mul_aa(const mat3<R>& a, const mat3<R>& b) {
  mat3<R> c;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      cplx<R> s = cmulc(a.e[0][i], b.e[j][0]);
      s = s + cmulc(a.e[1][i], b.e[j][1]);
      s = s + cmulc(a.e[2][i], b.e[j][2]);
      c.e[i][j] = s;
    }
  return c;
}
template <typename R>
GF_HD mat3<R> dag(const mat3<R>& a) {
  mat3<R> c;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) c.e[i][j] = conj(a.e[j][i]);
  return c;
}
template <typename R>
GF_HD void add_to(mat3<R>& c, const mat3<R>& a) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) c.e[i][j] = c.e[i][j] + a.e[i][j];
}
// c += s*a
template <typename R>
GF_HD void axpy_to(mat3<R>& c, R s, const mat3<R>& a) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      c.e[i][j].re += s * a.e[i][j].re;
      c.e[i][j].im += s * a.e[i][j].im;
    }
}
template <typename R>
GF_HD mat3<R> scale(R s, const mat3<R>& a) {
  mat3<R> c;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) c.e[i][j] = s * a.e[i][j];
  return c;
}
template <typename R>
GF_HD cplx<R> trace(const mat3<R>& a) {
  return a.e[0][0] + a.e[1][1] + a.e[2][2];
}
// Re tr(A B^dag) = sum_ij Re(A_ij conj(B_ij))
template <typename R>
GF_HD R retr_na(const mat3<R>& a, const mat3<R>& b) {
  R s = R(0);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) s += a.e[i][j].re * b.e[i][j].re + a.e[i][j].im * b.e[i][j].im;
  return s;
}
// tr(A B)
template <typename R>
GF_HD cplx<R> tr_nn(const mat3<R>& a, const mat3<R>& b) {
  cplx<R> s = mk<R>(0, 0);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k) fma_(s, a.e[i][k], b.e[k][i]);
  return s;
}

// Traceless anti-Hermitian projection as a matrix:
// TA(M) = (M - M^dag)/2 - tr(M - M^dag)/6 * 1.
template <typename R>
GF_HD mat3<R> ta_proj(const mat3<R>& m) {
  mat3<R> y;
  constexpr R third = R(1.0 / 3.0), half = R(0.5), mhalf = R(-0.5);
  R tri = (m.e[0][0].im + m.e[1][1].im + m.e[2][2].im) * third;
#pragma unroll
  for (int i = 0; i < 3; ++i) y.e[i][i] = mk<R>(R(0), m.e[i][i].im - tri);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = i + 1; j < 3; ++j) {
      cplx<R> x = m.e[i][j] - conj(m.e[j][i]);
      y.e[i][j] = half * x;
      y.e[j][i] = mk<R>(mhalf * x.re, half * x.im);
    }
  return y;
}

// su(3) coefficients c_a (a = 1..8 stored 0..7) of TA(M), with
// TA(M) = i sum_a c_a lambda_a / 2. This is the coefficient map of
// Traceless_antihermitian_add! for NC = 3.
template <typename R>
GF_HD void ta_coeffs(const mat3<R>& m, R c[8]) {
  constexpr R sr3i = R(0.57735026918962576451);  // 1/sqrt(3)
  // off-diagonal: x_ij = M_ij - conj(M_ji) = 2 y_ij
  cplx<R> x12 = m.e[0][1] - conj(m.e[1][0]);
  cplx<R> x13 = m.e[0][2] - conj(m.e[2][0]);
  cplx<R> x23 = m.e[1][2] - conj(m.e[2][1]);
  c[0] = x12.im;
  c[1] = x12.re;
  c[3] = x13.im;
  c[4] = x13.re;
  c[5] = x23.im;
  c[6] = x23.re;
  R d1 = m.e[0][0].im, d2 = m.e[1][1].im, d3 = m.e[2][2].im;
  c[2] = d1 - d2;
  c[7] = sr3i * (d1 + d2 - R(2) * d3);
}

// Hermitian matrix Q = sum_a p_a lambda_a / 2 (Gell-Mann basis).
template <typename R>
GF_HD mat3<R> herm_from_coeffs(const R p[8]) {
  constexpr R sr3i = R(0.57735026918962576451);
  constexpr R h = R(0.5), two = R(2.0);
  mat3<R> q;
  q.e[0][0] = mk<R>(h * (p[2] + sr3i * p[7]), R(0));
  q.e[1][1] = mk<R>(h * (-p[2] + sr3i * p[7]), R(0));
  q.e[2][2] = mk<R>(-h * two * sr3i * p[7], R(0));
  q.e[0][1] = mk<R>(h * p[0], -h * p[1]);
  q.e[1][0] = mk<R>(h * p[0], h * p[1]);
  q.e[0][2] = mk<R>(h * p[3], -h * p[4]);
  q.e[2][0] = mk<R>(h * p[3], h * p[4]);
  q.e[1][2] = mk<R>(h * p[5], -h * p[6]);
  q.e[2][1] = mk<R>(h * p[5], h * p[6]);
  return q;
}

// Third row of an SU(3) matrix from its first two rows: row3 = conj(row1 x row2)
// (m3complv3! of src/AbstractGaugefields.jl:3431).
template <typename R>
GF_HD void reconstruct_row3(mat3<R>& u) {
  u.e[2][0] = conj(u.e[0][1] * u.e[1][2] - u.e[0][2] * u.e[1][1]);
  u.e[2][1] = conj(u.e[0][2] * u.e[1][0] - u.e[0][0] * u.e[1][2]);
  u.e[2][2] = conj(u.e[0][0] * u.e[1][1] - u.e[0][1] * u.e[1][0]);
}

// Re-unitarisation: Gram-Schmidt of rows 1-2, row 3 from the cross product
// (normalize3! of src/AbstractGaugefields.jl:3378-3429).
template <typename R>
GF_HD void reunitarize(mat3<R>& u) {
  R n1 = R(0);
#pragma unroll
  for (int j = 0; j < 3; ++j) n1 += u.e[0][j].re * u.e[0][j].re + u.e[0][j].im * u.e[0][j].im;
  // w = <row1, row2> = sum_j u2j conj(u1j)
  cplx<R> w = mk<R>(0, 0);
#pragma unroll
  for (int j = 0; j < 3; ++j) w = w + mulc(u.e[1][j], u.e[0][j]);
  R inv1 = R(1) / n1;
  w = mk<R>(-w.re * inv1, -w.im * inv1);
#pragma unroll
  for (int j = 0; j < 3; ++j) fma_(u.e[1][j], w, u.e[0][j]);
  R n2 = R(0);
#pragma unroll
  for (int j = 0; j < 3; ++j) n2 += u.e[1][j].re * u.e[1][j].re + u.e[1][j].im * u.e[1][j].im;
  R s1 = R(1) / sqrt(n1), s2 = R(1) / sqrt(n2);
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    u.e[0][j] = s1 * u.e[0][j];
    u.e[1][j] = s2 * u.e[1][j];
  }
  reconstruct_row3(u);
}

// ---------------------------------------------------------------------------
// Cayley-Hamilton exponential of i*Q for a traceless Hermitian 3x3 Q:
//   exp(iQ) = f0 + f1 Q + f2 Q^2,
// with c0 = det Q, c1 = tr(Q^2)/2 and Q^3 = c1 Q + c0 (Cayley-Hamilton).
// The coefficients f_j(c0, c1) and their derivatives b1_j = df_j/dc1,
// b2_j = df_j/dc0 (the B1, B2 matrices of the stout derivative,
// calc_coefficients_Q in src/AbstractGaugefields.jl:3284) are summed from the
// power series exp(iQ) = sum_n (iQ)^n/n!, with every power reduced to
// a_n + b_n Q + c_n Q^2 by the recursion
//   a_{n+1} = c0 c_n,  b_{n+1} = a_n + c1 c_n,  c_{n+1} = b_n .
// The series is stable for the small |Q| of link updates, flow steps and
// stout layers (no division by (9u^2 - w^2)^2 as in the closed form), and it
// is summed until the term falls below the working precision.
// ---------------------------------------------------------------------------
template <typename R>
struct ch_coef {
  cplx<R> f[3];
  cplx<R> b1[3];  // d f_j / d c1
  cplx<R> b2[3];  // d f_j / d c0
};

template <typename R>
__device__ __forceinline__ R ch_eps();
template <>
__device__ __forceinline__ float ch_eps<float>() { return 3.0e-8f; }
template <>
__device__ __forceinline__ double ch_eps<double>() { return 5.0e-18; }

#define GF_CH_TERMS 44
// 1/n! for n = 0 .. GF_CH_TERMS-1
static __constant__ double c_inv_fact_d[GF_CH_TERMS] = {1.0, 1.0, 0.5, 0.16666666666666666, 0.041666666666666664, 0.008333333333333333, 0.001388888888888889, 0.0001984126984126984, 2.48015873015873e-05, 2.7557319223985893e-06, 2.755731922398589e-07, 2.505210838544172e-08, 2.08767569878681e-09, 1.6059043836821613e-10, 1.1470745597729725e-11, 7.647163731819816e-13, 4.779477332387385e-14, 2.8114572543455206e-15, 1.5619206968586225e-16, 8.22063524662433e-18, 4.110317623312165e-19, 1.9572941063391263e-20, 8.896791392450574e-22, 3.8681701706306835e-23, 1.6117375710961184e-24, 6.446950284384474e-26, 2.4795962632247972e-27, 9.183689863795546e-29, 3.279889237069838e-30, 1.1309962886447718e-31, 3.7699876288159054e-33, 1.2161250415535181e-34, 3.800390754854744e-36, 1.151633562077195e-37, 3.387157535521162e-39, 9.67759295863189e-41, 2.688220266286636e-42, 7.265460179153071e-44, 1.911963205040282e-45, 4.902469756513544e-47, 1.225617439128386e-48, 2.9893108271424046e-50, 7.117406731291439e-52, 1.6552108677421951e-53};
static __constant__ float c_inv_fact_f[GF_CH_TERMS] = {1.0f, 1.0f, 0.5f, 0.166666672f, 0.0416666679f, 0.00833333377f, 0.00138888892f, 0.000198412701f, 2.48015876e-05f, 2.75573188e-06f, 2.755732e-07f, 2.50521079e-08f, 2.08767559e-09f, 1.60590444e-10f, 1.14707454e-11f, 7.64716361e-13f, 4.77947726e-14f, 2.81145736e-15f, 1.56192068e-16f, 8.22063508e-18f, 4.11031759e-19f, 1.95729415e-20f, 8.89679096e-22f, 3.8681703e-23f, 1.61173759e-24f, 6.44695034e-26f, 2.47959628e-27f, 9.18368981e-29f, 3.27988916e-30f, 1.13099625e-31f, 3.76998781e-33f, 1.21612501e-34f, 3.80039067e-36f, 1.1516336e-37f, 3.38715699e-39f, 9.67764745e-41f, 2.68769045e-42f, 7.28675201e-44f, 1.40129846e-45f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};

// 1/n! as double-float pairs (hi, lo)
static __constant__ float c_inv_fact_df[2 * GF_CH_TERMS] = {
    1.000000000e+00f, 0.000000000e+00f,
    1.000000000e+00f, 0.000000000e+00f,
    5.000000000e-01f, 0.000000000e+00f,
    1.666666716e-01f, -4.967053879e-09f,
    4.166666791e-02f, -1.241763470e-09f,
    8.333333768e-03f, -4.346172033e-10f,
    1.388888923e-03f, -3.363109444e-11f,
    1.984127011e-04f, -2.725596875e-12f,
    2.480158764e-05f, -3.406996094e-13f,
    2.755731884e-06f, 3.793571224e-14f,
    2.755731998e-07f, -7.575112209e-15f,
    2.505210794e-08f, 4.417623045e-16f,
    2.087675588e-09f, 1.108283981e-16f,
    1.605904437e-10f, -5.352526512e-18f,
    1.147074536e-11f, 2.372207689e-19f,
    7.647163610e-13f, 1.220071047e-20f,
    4.779477256e-14f, 7.625444044e-22f,
    2.811457359e-15f, -1.046208474e-22f,
    1.561920681e-16f, 1.540447147e-24f,
    8.220635078e-18f, 1.681478097e-25f,
    4.110317591e-19f, 3.237511733e-27f,
    1.957294152e-20f, -4.612945514e-28f,
    8.896790960e-22f, 4.328837203e-29f,
    3.868170298e-23f, -1.273340432e-30f,
    1.611737591e-24f, -2.018664841e-32f,
    6.446950340e-26f, -5.609469144e-34f,
    2.479596285e-27f, -2.157488154e-35f,
    9.183689810e-29f, 5.383816950e-37f,
    3.279889164e-30f, 7.296480389e-38f,
    1.130996247e-31f, 4.137399577e-39f,
    3.769987809e-33f, -1.804494071e-40f,
    1.216125015e-34f, 2.696098245e-42f,
    3.800390671e-36f, 8.407790786e-44f,
    1.151633601e-37f, -4.203895393e-45f,
    3.387156991e-39f, 0.000000000e+00f,
    9.677647454e-41f, -0.000000000e+00f,
    2.687690455e-42f, 0.000000000e+00f,
    7.286752014e-44f, -0.000000000e+00f,
    1.401298464e-45f, 0.000000000e+00f,
    0.000000000e+00f, 0.000000000e+00f,
    0.000000000e+00f, 0.000000000e+00f,
    0.000000000e+00f, 0.000000000e+00f,
    0.000000000e+00f, 0.000000000e+00f,
    0.000000000e+00f, 0.000000000e+00f};

template <>
__device__ __forceinline__ dfl ch_eps<dfl>() { return dfl(2.0e-16f); }

template <typename R>
__device__ __forceinline__ R inv_fact(int n);
template <>
__device__ __forceinline__ double inv_fact<double>(int n) { return c_inv_fact_d[n]; }
template <>
__device__ __forceinline__ float inv_fact<float>(int n) { return c_inv_fact_f[n]; }
template <>
__device__ __forceinline__ dfl inv_fact<dfl>(int n) { return dfl(c_inv_fact_df[2 * n], c_inv_fact_df[2 * n + 1]); }

// Accumulation and convergence helpers of the series: fp32/fp64 use the
// plain operators; double-float accumulates with the sloppy double-word sum
// (the terms shrink geometrically, so no cancellation) and measures the
// term sizes on the fp32 high parts.
template <typename R>
struct ch_ops {
  typedef R mag_t;
  static __device__ __forceinline__ R sum(R x, R y) { return x + y; }
  static __device__ __forceinline__ void add(R& x, R y) { x += y; }
  static __device__ __forceinline__ void sub(R& x, R y) { x -= y; }
  static __device__ __forceinline__ mag_t mag(R x) { return fabs(x); }
  static __device__ __forceinline__ mag_t eps() { return ch_eps<R>(); }
};
template <>
struct ch_ops<dfl> {
  typedef float mag_t;
  static __device__ __forceinline__ dfl sum(dfl x, dfl y) { return df_add_fast(x, y); }
  static __device__ __forceinline__ void add(dfl& x, dfl y) { x = df_add_fast(x, y); }
  static __device__ __forceinline__ void sub(dfl& x, dfl y) { x = df_add_fast(x, -y); }
  static __device__ __forceinline__ float mag(dfl x) { return fabsf(x.hi); }
  static __device__ __forceinline__ float eps() { return 2.0e-16f; }
};

// One term of the series: advance the power coefficients from Q^{n-1} to
// Q^n and add i^n/n! times them; the phase i^n is the compile-time PH
// (0: 1, 1: i, 2: -1, 3: -i), so each term costs adds only.
template <typename R, bool DERIV, int PH>
struct ch_state {
  typedef ch_ops<R> O;
  static __device__ __forceinline__ typename O::mag_t step(int n, R c0, R c1, R& a, R& b, R& c, R& a0, R& b0, R& c0d,
                                                          R& a1, R& b1, R& c1d, R* fr, R* fi, R* d1r, R* d1i,
                                                          R* d2r, R* d2i) {
    R na = c0 * c, nb = O::sum(a, c1 * c), nc = b;
    R na0 = 0, nb0 = 0, nc0 = 0, na1 = 0, nb1 = 0, nc1 = 0;
    if (DERIV) {
      na0 = O::sum(c, c0 * c0d);
      nb0 = O::sum(a0, c1 * c0d);
      nc0 = b0;
      na1 = c0 * c1d;
      nb1 = O::sum(O::sum(a1, c), c1 * c1d);
      nc1 = b1;
    }
    a = na; b = nb; c = nc;
    const R fact = inv_fact<R>(n);
    R t[3] = {a * fact, b * fact, c * fact};
    typename O::mag_t mag = O::mag(t[0]) + O::mag(t[1]) + O::mag(t[2]);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      if (PH == 0) O::add(fr[j], t[j]);
      if (PH == 1) O::add(fi[j], t[j]);
      if (PH == 2) O::sub(fr[j], t[j]);
      if (PH == 3) O::sub(fi[j], t[j]);
    }
    if (DERIV) {
      a0 = na0; b0 = nb0; c0d = nc0;
      a1 = na1; b1 = nb1; c1d = nc1;
      R u0[3] = {a0 * fact, b0 * fact, c0d * fact};
      R u1[3] = {a1 * fact, b1 * fact, c1d * fact};
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        if (PH == 0) { O::add(d2r[j], u0[j]); O::add(d1r[j], u1[j]); }
        if (PH == 1) { O::add(d2i[j], u0[j]); O::add(d1i[j], u1[j]); }
        if (PH == 2) { O::sub(d2r[j], u0[j]); O::sub(d1r[j], u1[j]); }
        if (PH == 3) { O::sub(d2i[j], u0[j]); O::sub(d1i[j], u1[j]); }
      }
      mag += O::mag(u0[0]) + O::mag(u0[1]) + O::mag(u0[2]) + O::mag(u1[0]) + O::mag(u1[1]) + O::mag(u1[2]);
    }
    return mag;
  }
};

// One term of the series with the phase i^n split into its target (odd n:
// the imaginary part, even n: the real part; compile-time ODD) and its sign
// ((n & 2) ? -1 : +1, at run time), so a loop over pairs of terms holds two
// step bodies instead of four (the double-float kernels are instruction-fetch
// bound).
template <typename R, bool DERIV, bool ODD>
struct ch_pair_state {
  typedef ch_ops<R> O;
  static __device__ __forceinline__ typename O::mag_t step(int n, R c0, R c1, R& a, R& b, R& c, R& a0, R& b0,
                                                          R& c0d, R& a1, R& b1, R& c1d, R* fr, R* fi, R* d1r,
                                                          R* d1i, R* d2r, R* d2i) {
    R na = c0 * c, nb = O::sum(a, c1 * c), nc = b;
    R na0 = 0, nb0 = 0, nc0 = 0, na1 = 0, nb1 = 0, nc1 = 0;
    if (DERIV) {
      na0 = O::sum(c, c0 * c0d);
      nb0 = O::sum(a0, c1 * c0d);
      nc0 = b0;
      na1 = c0 * c1d;
      nb1 = O::sum(O::sum(a1, c), c1 * c1d);
      nc1 = b1;
    }
    a = na; b = nb; c = nc;
    R fact = inv_fact<R>(n);
    if (n & 2) fact = -fact;
    const R t[3] = {a * fact, b * fact, c * fact};
    typename O::mag_t mag = O::mag(t[0]) + O::mag(t[1]) + O::mag(t[2]);
#pragma unroll
    for (int j = 0; j < 3; ++j) O::add(ODD ? fi[j] : fr[j], t[j]);
    if (DERIV) {
      a0 = na0; b0 = nb0; c0d = nc0;
      a1 = na1; b1 = nb1; c1d = nc1;
      const R u0[3] = {a0 * fact, b0 * fact, c0d * fact};
      const R u1[3] = {a1 * fact, b1 * fact, c1d * fact};
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        O::add(ODD ? d2i[j] : d2r[j], u0[j]);
        O::add(ODD ? d1i[j] : d1r[j], u1[j]);
      }
      mag += O::mag(u0[0]) + O::mag(u0[1]) + O::mag(u0[2]) + O::mag(u1[0]) + O::mag(u1[1]) + O::mag(u1[2]);
    }
    return mag;
  }
};

// Double-float form: the terms are summed in double-float while the last
// term of a group of four is at least 1e-8; the rest of the series, terms
// below 1e-8, runs in fp32 (its rounding, ~1e-7 of the tail, is below 1e-15
// absolute) and is added to the double-float sums at the end. For the
// |Q| ~ 0.1-0.3 of stout layers and link updates this halves the number of
// double-float terms.
template <bool DERIV>
__device__ __forceinline__ void ch_coefficients_df(dfl c0, dfl c1, ch_coef<dfl>& out) {
  dfl a = dfl(1.f), b = dfl(0.f), c = dfl(0.f);
  dfl a0 = 0, b0 = 0, c0d = 0, a1 = 0, b1 = 0, c1d = 0;
  dfl fr[3] = {dfl(1.f), dfl(0.f), dfl(0.f)}, fi[3] = {0, 0, 0};
  dfl d1r[3] = {0, 0, 0}, d1i[3] = {0, 0, 0}, d2r[3] = {0, 0, 0}, d2i[3] = {0, 0, 0};
  int n = 1;
  for (; n + 1 < GF_CH_TERMS; n += 2) {
    ch_pair_state<dfl, DERIV, true>::step(n, c0, c1, a, b, c, a0, b0, c0d, a1, b1, c1d, fr, fi, d1r, d1i, d2r, d2i);
    const float mag = ch_pair_state<dfl, DERIV, false>::step(n + 1, c0, c1, a, b, c, a0, b0, c0d, a1, b1, c1d, fr,
                                                              fi, d1r, d1i, d2r, d2i);
    if (mag < 1.0e-8f) {
      n += 2;
      break;
    }
  }
  // fp32 tail from term n (n odd, so the pairs continue in order)
  float fa = a.hi + a.lo, fb = b.hi + b.lo, fc = c.hi + c.lo;
  float fa0 = a0.hi + a0.lo, fb0 = b0.hi + b0.lo, fc0 = c0d.hi + c0d.lo;
  float fa1 = a1.hi + a1.lo, fb1 = b1.hi + b1.lo, fc1 = c1d.hi + c1d.lo;
  const float g0 = c0.hi + c0.lo, g1 = c1.hi + c1.lo;
  float tr[3] = {0.f, 0.f, 0.f}, ti[3] = {0.f, 0.f, 0.f};
  float e1r[3] = {0.f, 0.f, 0.f}, e1i[3] = {0.f, 0.f, 0.f}, e2r[3] = {0.f, 0.f, 0.f}, e2i[3] = {0.f, 0.f, 0.f};
  for (; n + 1 < GF_CH_TERMS; n += 2) {
    ch_pair_state<float, DERIV, true>::step(n, g0, g1, fa, fb, fc, fa0, fb0, fc0, fa1, fb1, fc1, tr, ti, e1r, e1i,
                                            e2r, e2i);
    const float mag = ch_pair_state<float, DERIV, false>::step(n + 1, g0, g1, fa, fb, fc, fa0, fb0, fc0, fa1, fb1,
                                                                fc1, tr, ti, e1r, e1i, e2r, e2i);
    if (mag < 2.0e-16f) break;
  }
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    out.f[j] = mk(df_add_fast(fr[j], dfl(tr[j])), df_add_fast(fi[j], dfl(ti[j])));
    if (DERIV) {
      out.b1[j] = mk(df_add_fast(d1r[j], dfl(e1r[j])), df_add_fast(d1i[j], dfl(e1i[j])));
      out.b2[j] = mk(df_add_fast(d2r[j], dfl(e2r[j])), df_add_fast(d2i[j], dfl(e2i[j])));
    }
  }
}

template <typename R, bool DERIV>
__device__ __forceinline__ void ch_coefficients(R c0, R c1, ch_coef<R>& out) {
  if constexpr (std::is_same<R, dfl>::value) {
    ch_coefficients_df<DERIV>(c0, c1, out);
    return;
  }
  // power coefficients of Q^n and their partial derivatives
  R a = R(1), b = R(0), c = R(0);
  R a0 = 0, b0 = 0, c0d = 0;  // d/dc0
  R a1 = 0, b1 = 0, c1d = 0;  // d/dc1
  R fr[3] = {R(1), R(0), R(0)}, fi[3] = {R(0), R(0), R(0)};
  R d1r[3] = {0, 0, 0}, d1i[3] = {0, 0, 0}, d2r[3] = {0, 0, 0}, d2i[3] = {0, 0, 0};
  // terms n = 4k+1 .. 4k+4 have phases i, -1, -i, 1
  for (int n = 1; n + 3 < GF_CH_TERMS; n += 4) {
    ch_state<R, DERIV, 1>::step(n, c0, c1, a, b, c, a0, b0, c0d, a1, b1, c1d, fr, fi, d1r, d1i, d2r, d2i);
    ch_state<R, DERIV, 2>::step(n + 1, c0, c1, a, b, c, a0, b0, c0d, a1, b1, c1d, fr, fi, d1r, d1i, d2r, d2i);
    ch_state<R, DERIV, 3>::step(n + 2, c0, c1, a, b, c, a0, b0, c0d, a1, b1, c1d, fr, fi, d1r, d1i, d2r, d2i);
    const auto mag =
        ch_state<R, DERIV, 0>::step(n + 3, c0, c1, a, b, c, a0, b0, c0d, a1, b1, c1d, fr, fi, d1r, d1i, d2r, d2i);
    if (mag < ch_ops<R>::eps()) break;
  }
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    out.f[j] = mk(fr[j], fi[j]);
    if (DERIV) {
      out.b1[j] = mk(d1r[j], d1i[j]);
      out.b2[j] = mk(d2r[j], d2i[j]);
    }
  }
}

// Q^2 of a Hermitian Q: Hermitian, so six entries are computed.
template <typename R>
__device__ __forceinline__ mat3<R> herm_square(const mat3<R>& q) {
  mat3<R> r;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    R d = q.e[i][i].re * q.e[i][i].re;
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (k != i) d += q.e[i][k].re * q.e[i][k].re + q.e[i][k].im * q.e[i][k].im;
    r.e[i][i] = mk(d, R(0));
  }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = i + 1; j < 3; ++j) {
      // sum_k Q_ik Q_kj with Q_ii, Q_jj real
      cplx<R> v = q.e[i][i].re * q.e[i][j] + q.e[j][j].re * q.e[i][j];
      int k = 3 - i - j;
      fma_(v, q.e[i][k], q.e[k][j]);
      r.e[i][j] = v;
      r.e[j][i] = conj(v);
    }
  return r;
}

// c1 = tr(Q^2)/2 and c0 = det(Q) of a traceless Hermitian matrix.
template <typename R>
GF_HD void herm_invariants(const mat3<R>& q, R& c0, R& c1) {
  R q11 = q.e[0][0].re, q22 = q.e[1][1].re, q33 = q.e[2][2].re;
  cplx<R> q12 = q.e[0][1], q13 = q.e[0][2], q23 = q.e[1][2];
  R a12 = q12.re * q12.re + q12.im * q12.im;
  R a13 = q13.re * q13.re + q13.im * q13.im;
  R a23 = q23.re * q23.re + q23.im * q23.im;
  constexpr R half = R(0.5);
  c1 = half * (q11 * q11 + q22 * q22 + q33 * q33) + a12 + a13 + a23;
  // det = q11 q22 q33 + 2 Re(q12 q23 q31) - q11|q23|^2 - q22|q13|^2 - q33|q12|^2
  cplx<R> t = q12 * q23;
  R re3 = t.re * q13.re + t.im * q13.im;  // Re(q12 q23 conj(q13))
  c0 = q11 * q22 * q33 + R(2) * re3 - q11 * a23 - q22 * a13 - q33 * a12;
}

// Entry (i,j) of f0 + f1 Q + f2 Q^2 with the type's operators
template <typename R>
__device__ __forceinline__ cplx<R> ch_combine_ops(const ch_coef<R>& cc, const mat3<R>& q, const mat3<R>& q2, int i,
                                                  int j) {
  cplx<R> v = cc.f[1] * q.e[i][j];
  fma_(v, cc.f[2], q2.e[i][j]);
  if (i == j) v = v + cc.f[0];
  return v;
}
template <typename R>
__device__ __forceinline__ cplx<R> ch_combine(const ch_coef<R>& cc, const mat3<R>& q, const mat3<R>& q2, int i, int j) {
  return ch_combine_ops(cc, q, q2, i, j);
}
// exp(iQ) for traceless Hermitian Q. Q2 receives Q^2 (callers reuse it).
// ROWS = 2 forms rows 1-2 only (row 3 left zero), for products whose row 3 is
// rebuilt or not stored. OPS = true combines f0 + f1 Q + f2 Q^2 with the
// type's operators (for double-float: the accurate double-word sums, ~2^-48,
// which chains of link updates keep to 1e-12 of fp64), false with the
// fixed-grid sum (rms ~2^-43 of the bound) where one is given.
template <typename R, int ROWS = 3, bool OPS = false>
__device__ __forceinline__ mat3<R> expiq(const mat3<R>& q, mat3<R>* q2out = nullptr) {
  R c0, c1;
  herm_invariants(q, c0, c1);
  ch_coef<R> cc;
  ch_coefficients<R, false>(c0, c1, cc);
  // OPS: the generic (operator) square as well; otherwise the type's best
  mat3<R> q2 = OPS ? herm_square<R>(q) : herm_square(q);
  mat3<R> e = zero3<R>();
#pragma unroll
  for (int i = 0; i < ROWS; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) e.e[i][j] = OPS ? ch_combine_ops(cc, q, q2, i, j) : ch_combine(cc, q, q2, i, j);
  if (q2out) *q2out = q2;
  return e;
}

}  // namespace gf

// ---------------------------------------------------------------------------
// Double-float 3x3 products as compensated dot products (Ogita, Rump, Oishi,
// "Accurate sum and dot product", SIAM J. Sci. Comput. 26, 2005, Dot2 with
// double-float inputs): the high parts are summed with TwoSum, the product
// errors (FMA), the TwoSum errors and the cross terms hi*lo + lo*hi go into a
// single fp32 correction. Error ~ u^2 * sum |terms|, about half the operations
// of composing double-float multiplies and adds.
// ---------------------------------------------------------------------------
namespace gf {

struct dacc {
  float s, c;
};

GF_HD void dacc_add(dacc& a, float xh, float xl, float yh, float yl) {
  float p = df_mul_rn(xh, yh);  // not fusible: TwoSum below needs fl(xh*yh)
  float pe = fmaf(xh, yh, -p);
  float t = a.s + p;
  float z = t - a.s;
  float e = (a.s - (t - z)) + (p - z);
  a.s = t;
  a.c += e + pe;
  a.c = fmaf(xh, yl, a.c);
  a.c = fmaf(xl, yh, a.c);
}

GF_HD dfl dacc_get(const dacc& a) { return df_two_sum(a.s, a.c); }

// acc(i,j) (+)= sum_k op(a)_ik op(b)_kj with op = identity or dagger.
// Fully unrolled and inlined: an out-of-line form with rolled entry loops
// (matrices by value) was 1.3x slower in the stencil kernels, and the forms
// that indexed the caller's matrices through pointers or dynamic indices came
// out wrong under nvcc 13.0 -O3 (products of matrices built in registers read
// stale values).
template <bool DA, bool DB, bool ACC, int ROWS = 3>
GF_HD mat3<dfl> df_matmul(const mat3<dfl>& a, const mat3<dfl>& b, const mat3<dfl>* c) {
  mat3<dfl> r;
#pragma unroll
  for (int i = 0; i < ROWS; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      dacc re, im;
      if (ACC) {
        re.s = c->e[i][j].re.hi; re.c = c->e[i][j].re.lo;
        im.s = c->e[i][j].im.hi; im.c = c->e[i][j].im.lo;
      } else {
        re.s = re.c = im.s = im.c = 0.f;
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const cplx<dfl> x = DA ? conj(a.e[k][i]) : a.e[i][k];
        const cplx<dfl> y = DB ? conj(b.e[j][k]) : b.e[k][j];
        dacc_add(re, x.re.hi, x.re.lo, y.re.hi, y.re.lo);
        dacc_add(re, -x.im.hi, -x.im.lo, y.im.hi, y.im.lo);
        dacc_add(im, x.re.hi, x.re.lo, y.im.hi, y.im.lo);
        dacc_add(im, x.im.hi, x.im.lo, y.re.hi, y.re.lo);
      }
      r.e[i][j] = mk(dacc_get(re), dacc_get(im));
    }
  return r;
}

// ---------------------------------------------------------------------------
// Fixed-grid compensated product. The high parts of the terms of each output
// are accumulated onto a grid: the accumulator starts at a constant
// K = 1.5 * 2^k chosen from a norm bound so that every partial sum stays in
// [2^k, 2^(k+1)), where fp32 spacing is the constant g = 2^(k-23). Then each
// fused multiply-add a_h b_h + A rounds onto that grid, A - A_new is exact,
// and a second fused multiply-add recovers the rounding residual
// a_h b_h + (A - A_new) (about 24 bits, exact to 2^-48 relative). Residuals
// and the cross terms a_h b_l + a_l b_h go to a plain fp32 correction. Six
// fp32 operations per real term instead of the twelve of the TwoSum-based
// accumulation above; the error per entry is rms ~2^-43 and at most ~2^-38
// of |op(A)| |op(B)| (+ |C|) (the correction word sums up to twelve
// residuals of half a grid step in fp32), against rms ~2^-48 there. The bound: partial sums of entry (i,j) are at
// most |row i of op(A)| |column j of op(B)| (Cauchy-Schwarz), so
// M^2 = max_i |a_i|^2 max_j |b_j|^2 (+ the accumulator's entries), and k is
// taken from M^2's exponent with a factor 2 of headroom.
// ---------------------------------------------------------------------------
GF_HD float df_grid_const(float m2) {
#ifdef __CUDA_ARCH__
  const int e2 = (int)(__float_as_uint(m2) >> 23);
#else
  unsigned int u;
  memcpy(&u, &m2, 4);
  const int e2 = (int)(u >> 23);
#endif
  // 2^(k-1) >= 2 M with M^2 < 2^(e2-126): k = ceil((e2 - 122) / 2)
  const int k = (e2 - 121) >> 1;
  const unsigned int bits = ((unsigned int)(k + 127) << 23) | 0x400000u;
#ifdef __CUDA_ARCH__
  return __uint_as_float(bits);
#else
  float f;
  memcpy(&f, &bits, 4);
  return f;
#endif
}

GF_HD void grid_term(float& A, float& L, float xh, float xl, float yh, float yl) {
  const float An = fmaf(xh, yh, A);
  const float t = A - An;  // exact: both on the grid of one binade
  L += fmaf(xh, yh, t);    // the rounding residual of xh*yh onto the grid
  L = fmaf(xh, yl, L);
  L = fmaf(xl, yh, L);
  A = An;
}

//
// NORM = false leaves each entry as the raw pair (A - K, L) instead of the
// normalised double-float fast_two_sum(A - K, L): the same value, with a low
// word of up to ~2^-19 of the bound instead of half an ulp of the high word.
// The next product's grid sees only high words, so it stays exact; its cross
// terms carry the larger low word at fp32 precision (rms 1.5x the error).
//
// GF_DF_PACKED = 1 runs the real and imaginary accumulators of an entry as one
// pair through the paired fp32 instructions of sm_100-class GPUs (__ffma2_rn,
// __fadd2_rn; per component the same correctly rounded operations as fmaf and
// +), the terms of each accumulator in the scalar order, so the results are
// bitwise those of the scalar form with half the arithmetic instructions. The
// operand pairs (x.re, x.re), (-x.im, x.im), (y.re, y.im), (y.im, y.re) are
// rebuilt with moves for every term, and at 32^4 the paired form measured
// 1.55 trajectories/s against 1.84 (gather 6.3 against 4.9 ms, small spills
// at the gather's 128 registers), so the scalar form is the default.
#ifndef GF_DF_PACKED
#define GF_DF_PACKED 0
#endif
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000 && GF_DF_PACKED
#define GF_DF_PAIRED 1
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
// grid_term on the pair (re, im): the same six operations per component
__device__ __forceinline__ void grid_term2(float2& A, float2& L, float2 xh, float2 xl, float2 yh, float2 yl) {
  const float2 An = __ffma2_rn(xh, yh, A);
  const float2 t = __fadd2_rn(A, neg2(An));
  L = __fadd2_rn(L, __ffma2_rn(xh, yh, t));
  L = __ffma2_rn(xh, yl, L);
  L = __ffma2_rn(xl, yh, L);
  A = An;
}
#else
#define GF_DF_PAIRED 0
#endif

template <bool DA, bool DB, bool ACC, int ROWS = 3, bool NORM = true>
GF_HD mat3<dfl> dfg_matmul(const mat3<dfl>& a, const mat3<dfl>& b, const mat3<dfl>* c) {
  float ra = 0.f, cb = 0.f;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    float r = 0.f, q = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const cplx<dfl> x = DA ? conj(a.e[k][i]) : a.e[i][k];  // row i of op(a)
      const cplx<dfl> y = DB ? conj(b.e[i][k]) : b.e[k][i];  // column i of op(b)
      r = fmaf(x.re.hi, x.re.hi, fmaf(x.im.hi, x.im.hi, r));
      q = fmaf(y.re.hi, y.re.hi, fmaf(y.im.hi, y.im.hi, q));
    }
    if (i < ROWS) ra = fmaxf(ra, r);
    cb = fmaxf(cb, q);
  }
  float m2 = ra * cb;
  if (ACC) {
    float cm = 0.f;
#pragma unroll
    for (int i = 0; i < ROWS; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) cm = fmaxf(cm, fmaxf(fabsf(c->e[i][j].re.hi), fabsf(c->e[i][j].im.hi)));
    m2 = 2.f * fmaf(cm, cm, m2);  // (x + y)^2 <= 2 (x^2 + y^2)
  }
  const float K = df_grid_const(m2);
  mat3<dfl> r = zero3<dfl>();
#if GF_DF_PAIRED
  const float2 K2 = f2(K, K);
#pragma unroll
  for (int i = 0; i < ROWS; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      float2 A2 = K2, L2 = f2(0.f, 0.f);
      if (ACC) {
        const cplx<dfl> v = c->e[i][j];
        const float2 vh = f2(v.re.hi, v.im.hi);
        A2 = __fadd2_rn(K2, vh);
        L2 = __fadd2_rn(__fadd2_rn(vh, neg2(__fadd2_rn(A2, neg2(K2)))), f2(v.re.lo, v.im.lo));
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const cplx<dfl> x = DA ? conj(a.e[k][i]) : a.e[i][k];
        const cplx<dfl> y = DB ? conj(b.e[j][k]) : b.e[k][j];
        // (re, im) += (x.re y.re, x.re y.im), then (-x.im y.im, x.im y.re)
        grid_term2(A2, L2, f2(x.re.hi, x.re.hi), f2(x.re.lo, x.re.lo), f2(y.re.hi, y.im.hi), f2(y.re.lo, y.im.lo));
        grid_term2(A2, L2, f2(-x.im.hi, x.im.hi), f2(-x.im.lo, x.im.lo), f2(y.im.hi, y.re.hi),
                   f2(y.im.lo, y.re.lo));
      }
      const float2 sv = __fadd2_rn(A2, neg2(K2));
      if (NORM) {
        const float2 h = __fadd2_rn(sv, L2);
        const float2 e = __fadd2_rn(L2, neg2(__fadd2_rn(h, neg2(sv))));
        r.e[i][j] = mk(dfl(h.x, e.x), dfl(h.y, e.y));
      } else {
        r.e[i][j] = mk(dfl(sv.x, L2.x), dfl(sv.y, L2.y));
      }
    }
  return r;
#else
#pragma unroll
  for (int i = 0; i < ROWS; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      float Ar = K, Ai = K, Lr = 0.f, Li = 0.f;
      if (ACC) {
        const cplx<dfl> v = c->e[i][j];
        Ar = K + v.re.hi;
        Lr = (v.re.hi - (Ar - K)) + v.re.lo;
        Ai = K + v.im.hi;
        Li = (v.im.hi - (Ai - K)) + v.im.lo;
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const cplx<dfl> x = DA ? conj(a.e[k][i]) : a.e[i][k];
        const cplx<dfl> y = DB ? conj(b.e[j][k]) : b.e[k][j];
        grid_term(Ar, Lr, x.re.hi, x.re.lo, y.re.hi, y.re.lo);
        grid_term(Ar, Lr, -x.im.hi, -x.im.lo, y.im.hi, y.im.lo);
        grid_term(Ai, Li, x.re.hi, x.re.lo, y.im.hi, y.im.lo);
        grid_term(Ai, Li, x.im.hi, x.im.lo, y.re.hi, y.re.lo);
      }
      if (NORM) r.e[i][j] = mk(df_fast_two_sum(Ar - K, Lr), df_fast_two_sum(Ai - K, Li));
      else r.e[i][j] = mk(dfl(Ar - K, Lr), dfl(Ai - K, Li));
    }
  return r;
#endif
}

// Fixed-grid accumulators for single sums of products (traces, Q^2 and the
// coefficient combinations of the stout adjoint): the same grid scheme as
// dfg_matmul, with the bound M on |partial sums| given by the caller (sums
// of |x||y| over the terms, from the fp32 high parts; |x| of a complex value
// bounded by |re| + |im|). About 28 fp32 operations per complex multiply-add
// against ~110 through the double-float operators.
struct dfg_acc {
  float K, A, L;
};
struct dfg_cacc {
  float K, Ar, Ai, Lr, Li;
};
GF_HD float cabs1(const cplx<dfl>& x) { return fabsf(x.re.hi) + fabsf(x.im.hi); }
GF_HD dfg_acc dfg_begin(float M) {
  const float K = df_grid_const(M * M);
  return dfg_acc{K, K, 0.f};
}
GF_HD dfg_cacc dfg_cbegin(float M) {
  const float K = df_grid_const(M * M);
  return dfg_cacc{K, K, K, 0.f, 0.f};
}
// real += x y
GF_HD void dfg_term(dfg_acc& a, dfl x, dfl y) { grid_term(a.A, a.L, x.hi, x.lo, y.hi, y.lo); }
// complex += x y
GF_HD void dfg_cterm(dfg_cacc& a, const cplx<dfl>& x, const cplx<dfl>& y) {
  grid_term(a.Ar, a.Lr, x.re.hi, x.re.lo, y.re.hi, y.re.lo);
  grid_term(a.Ar, a.Lr, -x.im.hi, -x.im.lo, y.im.hi, y.im.lo);
  grid_term(a.Ai, a.Li, x.re.hi, x.re.lo, y.im.hi, y.im.lo);
  grid_term(a.Ai, a.Li, x.im.hi, x.im.lo, y.re.hi, y.re.lo);
}
// complex += r y with r real
GF_HD void dfg_rcterm(dfg_cacc& a, dfl r, const cplx<dfl>& y) {
  grid_term(a.Ar, a.Lr, r.hi, r.lo, y.re.hi, y.re.lo);
  grid_term(a.Ai, a.Li, r.hi, r.lo, y.im.hi, y.im.lo);
}
// real part += c
GF_HD void dfg_cadd_re(dfg_cacc& a, dfl c) { grid_term(a.Ar, a.Lr, c.hi, c.lo, 1.f, 0.f); }
GF_HD dfl dfg_end(const dfg_acc& a) { return df_fast_two_sum(a.A - a.K, a.L); }
GF_HD cplx<dfl> dfg_cend(const dfg_cacc& a) {
  return mk(df_fast_two_sum(a.Ar - a.K, a.Lr), df_fast_two_sum(a.Ai - a.K, a.Li));
}

// tr(A B) for double-float matrices, one fixed-grid sum
__device__ __forceinline__ cplx<dfl> tr_nn(const mat3<dfl>& a, const mat3<dfl>& b) {
  float M = 0.f;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k) M = fmaf(cabs1(a.e[i][k]), cabs1(b.e[k][i]), M);
  dfg_cacc acc = dfg_cbegin(M);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k) dfg_cterm(acc, a.e[i][k], b.e[k][i]);
  return dfg_cend(acc);
}

// Q^2 of a Hermitian double-float Q with fixed-grid sums
__device__ __forceinline__ mat3<dfl> herm_square(const mat3<dfl>& q) {
  mat3<dfl> r;
  float a[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k) a[i][k] = cabs1(q.e[i][k]);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    float M = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) M = fmaf(a[i][k], a[i][k], M);
    dfg_acc d = dfg_begin(M);
    dfg_term(d, q.e[i][i].re, q.e[i][i].re);
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (k != i) {
        dfg_term(d, q.e[i][k].re, q.e[i][k].re);
        dfg_term(d, q.e[i][k].im, q.e[i][k].im);
      }
    r.e[i][i] = mk(dfg_end(d), dfl(0.f));
  }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = i + 1; j < 3; ++j) {
      // sum_k Q_ik Q_kj with Q_ii, Q_jj real
      const int k = 3 - i - j;
      const float M = (a[i][i] + a[j][j]) * a[i][j] + a[i][k] * a[k][j];
      dfg_cacc v = dfg_cbegin(M);
      dfg_rcterm(v, q.e[i][i].re, q.e[i][j]);
      dfg_rcterm(v, q.e[j][j].re, q.e[i][j]);
      dfg_cterm(v, q.e[i][k], q.e[k][j]);
      r.e[i][j] = dfg_cend(v);
      r.e[j][i] = conj(r.e[i][j]);
    }
  return r;
}

// f0 + f1 Q + f2 Q^2 (ch_combine, found by argument-dependent lookup from expiq):
// the double-float entry as one fixed-grid sum
__device__ __forceinline__ cplx<dfl> ch_combine(const ch_coef<dfl>& cc, const mat3<dfl>& q, const mat3<dfl>& q2,
                                                int i, int j) {
  dfg_cacc w = dfg_cbegin(cabs1(cc.f[1]) * cabs1(q.e[i][j]) + cabs1(cc.f[2]) * cabs1(q2.e[i][j]) +
                          (i == j ? cabs1(cc.f[0]) : 0.f));
  dfg_cterm(w, cc.f[1], q.e[i][j]);
  dfg_cterm(w, cc.f[2], q2.e[i][j]);
  if (i == j) dfg_cterm(w, cc.f[0], mk(dfl(1.f), dfl(0.f)));
  return dfg_cend(w);
}

// Rows 1-2 of A*B (row 3 left zero), for updates that re-unitarise right
// after the product: re-unitarisation rebuilds row 3 from rows 1-2.
template <typename R>
GF_HD mat3<R> mul_nn_rows12(const mat3<R>& a, const mat3<R>& b) {
  mat3<R> r = zero3<R>();
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      cplx<R> v = a.e[i][0] * b.e[0][j];
      fma_(v, a.e[i][1], b.e[1][j]);
      fma_(v, a.e[i][2], b.e[2][j]);
      r.e[i][j] = v;
    }
  return r;
}
__device__ __forceinline__ mat3<dfl> mul_nn_rows12(const mat3<dfl>& a, const mat3<dfl>& b) {
  return df_matmul<false, false, false, 2>(a, b, nullptr);
}

template <bool DA, bool DB>
__device__ __forceinline__ mat3<dfl> df_mul(const mat3<dfl>& a, const mat3<dfl>& b) {
  return df_matmul<DA, DB, false>(a, b, nullptr);
}
template <bool DA, bool DB>
__device__ __forceinline__ void df_mac(mat3<dfl>& acc, const mat3<dfl>& a, const mat3<dfl>& b) {
  acc = df_matmul<DA, DB, true>(a, b, &acc);
}

__device__ __forceinline__ mat3<dfl> mul_nn(const mat3<dfl>& a, const mat3<dfl>& b) { return df_mul<false, false>(a, b); }
__device__ __forceinline__ mat3<dfl> mul_na(const mat3<dfl>& a, const mat3<dfl>& b) { return df_mul<false, true>(a, b); }
__device__ __forceinline__ mat3<dfl> mul_an(const mat3<dfl>& a, const mat3<dfl>& b) { return df_mul<true, false>(a, b); }
__device__ __forceinline__ mat3<dfl> mul_aa(const mat3<dfl>& a, const mat3<dfl>& b) { return df_mul<true, true>(a, b); }

}  // namespace gf

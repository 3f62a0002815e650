// Lattice geometry and the HBM layout of every field.
//
// Sites are even/odd ordered: site index s = parity * V/2 + lex/2 with
// lex = x + NX*(y + NY*(z + NZ*t)) and parity = (x+y+z+t) & 1 (NX even).
// Periodic neighbours come from index arithmetic; there are no halo copies
// (the reference keeps a halo of width 1 and refreshes it with set_halo!,
// src/4D/mpi_jacc/gaugefields_4D_MPILattice.jl:509-512).
//
// Field storage is site-major structure-of-arrays: for direction mu and
// component c the V site values are contiguous, so a warp of consecutive
// sites issues one coalesced 128-bit (or 64-bit) load per component.
//   LINK64 : double2 [4][9][V]   (3x3 complex, row-major components)
//   MAT64  : double2 [4][9][V]   (general 3x3 complex, same layout)
//   LINK32 : float4  [4][3][V]   (rows 1-2 = 12 reals; row 3 rebuilt)
//   MAT32  : float2  [4][9][V]   (general 3x3 complex in fp32)
//   MOM64  : double  [4][8][V]   (su(3) coefficients p_1..p_8)
#pragma once
#include "su3.cuh"
#include <stdint.h>

namespace gf {

struct Geom {
  int L[4];      // NX, NY, NZ, NT
  int vol;       // V
  int vh;        // V/2
  int stride[4]; // lexicographic strides 1, NX, NX*NY, NX*NY*NZ
};

struct Site {
  int x[4];
  int lex;
  int par;
};

GF_HD Site site_of(const Geom& g, int s) {
  Site st;
  st.par = s >= g.vh ? 1 : 0;
  int h = s - st.par * g.vh;
  int nxh = g.L[0] >> 1;
  int xh = h % nxh;
  int r = h / nxh;
  st.x[1] = r % g.L[1];
  r /= g.L[1];
  st.x[2] = r % g.L[2];
  st.x[3] = r / g.L[2];
  st.x[0] = 2 * xh + ((st.par + st.x[1] + st.x[2] + st.x[3]) & 1);
  st.lex = st.x[0] + g.L[0] * (st.x[1] + g.L[1] * (st.x[2] + g.L[2] * st.x[3]));
  return st;
}

GF_HD int eo_of_lex(const Geom& g, int lex, int par) { return par * g.vh + (lex >> 1); }

// lexicographic index after a unit step d = +-1 along the compile-time axis MU
// (periodic wrap), starting from a site whose MU coordinate is `c`.
template <int MU>
GF_HD int step_lex(const Geom& g, int lex, int c, int d) {
  int n = c + d;
  if (n < 0) return lex + (g.L[MU] - 1) * g.stride[MU];
  if (n >= g.L[MU]) return lex - (g.L[MU] - 1) * g.stride[MU];
  return lex + d * g.stride[MU];
}

// even/odd index of x + d e_MU
template <int MU>
GF_HD int nbr(const Geom& g, const Site& st, int d) {
  return eo_of_lex(g, step_lex<MU>(g, st.lex, st.x[MU], d), st.par ^ 1);
}

// even/odd index of x + d0 e_MU + d1 e_NU  (MU != NU)
template <int MU, int NU>
GF_HD int nbr2(const Geom& g, const Site& st, int d0, int d1) {
  int lex = step_lex<MU>(g, st.lex, st.x[MU], d0);
  lex = step_lex<NU>(g, lex, st.x[NU], d1);
  return eo_of_lex(g, lex, st.par);
}

// Minimum resident blocks per SM requested for the stencil kernels (register
// budget 65536 / (128 threads * min blocks)): fp32 and double-float kernels are
// latency-bound and gain from occupancy; fp64 kernels are fp64-issue-bound and
// keep the full register file.
#ifndef GF_FP32_MINB
#define GF_FP32_MINB 4
#endif
#ifndef GF_DF_MINB
#define GF_DF_MINB 3
#endif
template <typename R>
struct minblocks {
  static constexpr int value = 1;
};
template <>
struct minblocks<float> {
  static constexpr int value = GF_FP32_MINB;
};
template <>
struct minblocks<dfl> {
  static constexpr int value = GF_DF_MINB;
};
#define GF_MINB(R) (minblocks<R>::value)
// The double-float adjoint kernels hold twice the fp32 state; at three blocks
// per SM they spill heavily, so they keep two (255 registers a thread).
#ifndef GF_DF_ADJ_MINB
#define GF_DF_ADJ_MINB 2
#endif
template <typename R>
struct minblocks_adj {
  static constexpr int value = minblocks<R>::value;
};
template <>
struct minblocks_adj<dfl> {
  static constexpr int value = GF_DF_ADJ_MINB;
};
#define GF_MINB_ADJ(R) (minblocks_adj<R>::value)

// Link index of a stencil thread. With GF_INTERLEAVE the grid is 1-D with
// 4 * ceil(V/bs) blocks and block b handles direction b % 4 of the sites of
// block b / 4 (the four directions of the same sites run back to back, so
// their shared neighbours stay in L2); otherwise blockIdx.y is the direction.
#ifndef GF_INTERLEAVE
#define GF_INTERLEAVE 1
#endif
__device__ __forceinline__ void link_of_thread(int& s, int& mu) {
#if GF_INTERLEAVE
  mu = blockIdx.x & 3;
  s = (blockIdx.x >> 2) * blockDim.x + threadIdx.x;
#else
  mu = blockIdx.y;
  s = blockIdx.x * blockDim.x + threadIdx.x;
#endif
}
inline dim3 stencil_grid(int vol, int bs) {
#if GF_INTERLEAVE
  return dim3(4 * ((vol + bs - 1) / bs));
#else
  return dim3((vol + bs - 1) / bs, 4);
#endif
}

// Runtime-axis forms of the same steps. The stencil kernels loop over the
// other axes at run time (one loop body instead of one unrolled copy per axis
// pair), which keeps their code within the instruction cache.
GF_HD int coord(const Site& st, int mu) {
  return mu == 0 ? st.x[0] : (mu == 1 ? st.x[1] : (mu == 2 ? st.x[2] : st.x[3]));
}
GF_HD int step_lex_rt(const Geom& g, int lex, int c, int mu, int d) {
  const int L = g.L[mu], str = g.stride[mu];
  const int n = c + d;
  if (n < 0) return lex + (L - 1) * str;
  if (n >= L) return lex - (L - 1) * str;
  return lex + d * str;
}
// even/odd index of x + d e_mu
GF_HD int nbr_rt(const Geom& g, const Site& st, int mu, int d) {
  return eo_of_lex(g, step_lex_rt(g, st.lex, coord(st, mu), mu, d), st.par ^ 1);
}
// even/odd index of x + d0 e_mu + d1 e_nu  (mu != nu)
GF_HD int nbr2_rt(const Geom& g, const Site& st, int mu, int d0, int nu, int d1) {
  int lex = step_lex_rt(g, st.lex, coord(st, mu), mu, d0);
  lex = step_lex_rt(g, lex, coord(st, nu), nu, d1);
  return eo_of_lex(g, lex, st.par);
}

// ---------------------------------------------------------------------------
// Field accessors. `V` is the site count, `s` the even/odd site index.
// ---------------------------------------------------------------------------
template <typename R>
struct LinkFull;  // 18-real storage (LINK64 / MAT64 / MAT32)

template <>
struct LinkFull<double> {
  typedef double2 elem;
  static __device__ __forceinline__ mat3<double> load(const double2* __restrict__ p, int mu, int s, int V) {
    mat3<double> m;
    const double2* b = p + (size_t)mu * 9 * V + s;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      double2 v = __ldg(b + (size_t)k * V);
      m.e[k / 3][k % 3] = mk(v.x, v.y);
    }
    return m;
  }
  static __device__ __forceinline__ void store(double2* __restrict__ p, int mu, int s, int V, const mat3<double>& m) {
    double2* b = p + (size_t)mu * 9 * V + s;
#pragma unroll
    for (int k = 0; k < 9; ++k) b[(size_t)k * V] = make_double2(m.e[k / 3][k % 3].re, m.e[k / 3][k % 3].im);
  }
};

template <>
struct LinkFull<float> {
  typedef float2 elem;
  static __device__ __forceinline__ mat3<float> load(const float2* __restrict__ p, int mu, int s, int V) {
    mat3<float> m;
    const float2* b = p + (size_t)mu * 9 * V + s;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      float2 v = __ldg(b + (size_t)k * V);
      m.e[k / 3][k % 3] = mk(v.x, v.y);
    }
    return m;
  }
  static __device__ __forceinline__ void store(float2* __restrict__ p, int mu, int s, int V, const mat3<float>& m) {
    float2* b = p + (size_t)mu * 9 * V + s;
#pragma unroll
    for (int k = 0; k < 9; ++k) b[(size_t)k * V] = make_float2(m.e[k / 3][k % 3].re, m.e[k / 3][k % 3].im);
  }
};

// fp64 storage, double-float arithmetic (the mixed form's fp64-class kernels)
template <>
struct LinkFull<dfl> {
  typedef double2 elem;
  static __device__ __forceinline__ mat3<dfl> load(const double2* __restrict__ p, int mu, int s, int V) {
    mat3<dfl> m;
    const double2* b = p + (size_t)mu * 9 * V + s;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      double2 v = __ldg(b + (size_t)k * V);
      m.e[k / 3][k % 3] = mk(df_from_double(v.x), df_from_double(v.y));
    }
    return m;
  }
  static __device__ __forceinline__ void store(double2* __restrict__ p, int mu, int s, int V, const mat3<dfl>& m) {
    double2* b = p + (size_t)mu * 9 * V + s;
#pragma unroll
    for (int k = 0; k < 9; ++k)
      b[(size_t)k * V] = make_double2(df_to_double(m.e[k / 3][k % 3].re), df_to_double(m.e[k / 3][k % 3].im));
  }
};

// Double-float-native 18-real storage (the internal fields of double-float
// stout stacks): each complex element is one float4 (re.hi, re.lo, im.hi,
// im.lo), laid out like LINK64 / MAT64 (16 bytes per element, 144 per
// link), so loads and stores need no fp64 <-> double-float conversion.
struct LinkDfn {
  typedef float4 elem;
  static __device__ __forceinline__ mat3<dfl> load(const float4* __restrict__ p, int mu, int s, int V) {
    mat3<dfl> m;
    const float4* b = p + (size_t)mu * 9 * V + s;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      float4 v = __ldg(b + (size_t)k * V);
      m.e[k / 3][k % 3] = mk(dfl(v.x, v.y), dfl(v.z, v.w));
    }
    return m;
  }
  // fp64 view of a double-float-native link (hi + lo in fp64; fp64 kernels)
  static __device__ __forceinline__ mat3<double> load64(const float4* __restrict__ p, int mu, int s, int V) {
    mat3<double> m;
    const float4* b = p + (size_t)mu * 9 * V + s;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      float4 v = __ldg(b + (size_t)k * V);
      m.e[k / 3][k % 3] = mk((double)v.x + (double)v.y, (double)v.z + (double)v.w);
    }
    return m;
  }
  static __device__ __forceinline__ void store(float4* __restrict__ p, int mu, int s, int V, const mat3<dfl>& m) {
    float4* b = p + (size_t)mu * 9 * V + s;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const cplx<dfl> v = m.e[k / 3][k % 3];
      b[(size_t)k * V] = make_float4(v.re.hi, v.re.lo, v.im.hi, v.im.lo);
    }
  }
};

// double-float loads and stores from either storage: fp64 (double2,
// converted) or double-float-native (float4)
template <typename E>
struct DfIO;
template <>
struct DfIO<double2> {
  static __device__ __forceinline__ mat3<dfl> load(const double2* __restrict__ p, int mu, int s, int V) {
    return LinkFull<dfl>::load(p, mu, s, V);
  }
  static __device__ __forceinline__ void store(double2* __restrict__ p, int mu, int s, int V, const mat3<dfl>& m) {
    LinkFull<dfl>::store(p, mu, s, V, m);
  }
};
template <>
struct DfIO<float4> {
  static __device__ __forceinline__ mat3<dfl> load(const float4* __restrict__ p, int mu, int s, int V) {
    return LinkDfn::load(p, mu, s, V);
  }
  static __device__ __forceinline__ void store(float4* __restrict__ p, int mu, int s, int V, const mat3<dfl>& m) {
    LinkDfn::store(p, mu, s, V, m);
  }
};

// 12-real two-row fp32 link storage: 3 float4 per link
struct Link12f {
  static __device__ __forceinline__ mat3<float> load(const float4* __restrict__ p, int mu, int s, int V) {
    mat3<float> m;
    const float4* b = p + (size_t)mu * 3 * V + s;
    float4 a0 = __ldg(b);
    float4 a1 = __ldg(b + (size_t)V);
    float4 a2 = __ldg(b + (size_t)2 * V);
    m.e[0][0] = mk(a0.x, a0.y);
    m.e[0][1] = mk(a0.z, a0.w);
    m.e[0][2] = mk(a1.x, a1.y);
    m.e[1][0] = mk(a1.z, a1.w);
    m.e[1][1] = mk(a2.x, a2.y);
    m.e[1][2] = mk(a2.z, a2.w);
    reconstruct_row3(m);
    return m;
  }
  static __device__ __forceinline__ void store(float4* __restrict__ p, int mu, int s, int V, const mat3<float>& m) {
    float4* b = p + (size_t)mu * 3 * V + s;
    b[0] = make_float4(m.e[0][0].re, m.e[0][0].im, m.e[0][1].re, m.e[0][1].im);
    b[(size_t)V] = make_float4(m.e[0][2].re, m.e[0][2].im, m.e[1][0].re, m.e[1][0].im);
    b[(size_t)2 * V] = make_float4(m.e[1][1].re, m.e[1][1].im, m.e[1][2].re, m.e[1][2].im);
  }
};

// Link source policy used by the stencil kernels: full 18-real storage in
// precision R, or 12-real fp32 storage (R = float only).
template <typename R, bool TWELVE>
struct LinkSrc;
template <typename R>
struct LinkSrc<R, false> {
  typedef typename LinkFull<R>::elem elem;
  const elem* __restrict__ p;
  __device__ __forceinline__ mat3<R> operator()(int mu, int s, int V) const { return LinkFull<R>::load(p, mu, s, V); }
};
// fp64 arithmetic on double-float-native storage (plaquette of a
// double-float stack's top level)
struct LinkSrcDfn64 {
  typedef float4 elem;
  const float4* __restrict__ p;
  __device__ __forceinline__ mat3<double> operator()(int mu, int s, int V) const { return LinkDfn::load64(p, mu, s, V); }
};
template <>
struct LinkSrc<float, true> {
  typedef float4 elem;
  const float4* __restrict__ p;
  __device__ __forceinline__ mat3<float> operator()(int mu, int s, int V) const { return Link12f::load(p, mu, s, V); }
};

}  // namespace gf

// Nearest-neighbour staple stencils shared by the Wilson force, the stout
// layers and the gradient flow.
//
// S_mu(x) is the sum of the six staples in dS/dU order, i.e. the rest of each
// plaquette after U_mu(x):
//   S_mu(x) = sum_{nu != mu} [ U_nu(x+mu) U_mu(x+nu)^dag U_nu(x)^dag
//                            + U_nu(x+mu-nu)^dag U_mu(x-nu)^dag U_nu(x-nu) ].
// It is the Wilsonloop staple list of GaugeAction_dataset
// (src/action/GaugeActions.jl:48-62) for the loops plaq U plaq^dag, and its
// Hermitian conjugate is the staple V of construct_double_staple! /
// construct_staple! (src/AbstractGaugefields.jl:2856-2923) and the stout C_mu/rho.
#pragma once
#include "lattice.cuh"

namespace gf {

// acc += A*B
template <typename R>
__device__ __forceinline__ void mac_nn(mat3<R>& acc, const mat3<R>& a, const mat3<R>& b) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      fma_(acc.e[i][j], a.e[i][0], b.e[0][j]);
      fma_(acc.e[i][j], a.e[i][1], b.e[1][j]);
      fma_(acc.e[i][j], a.e[i][2], b.e[2][j]);
    }
}
// acc += A*B^dag
template <typename R>
__device__ __forceinline__ void mac_na(mat3<R>& acc, const mat3<R>& a, const mat3<R>& b) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      fma_(acc.e[i][j], a.e[i][0], conj(b.e[j][0]));
      fma_(acc.e[i][j], a.e[i][1], conj(b.e[j][1]));
      fma_(acc.e[i][j], a.e[i][2], conj(b.e[j][2]));
    }
}
// acc += A^dag*B
template <typename R>
__device__ __forceinline__ void mac_an(mat3<R>& acc, const mat3<R>& a, const mat3<R>& b) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      fma_(acc.e[i][j], conj(a.e[0][i]), b.e[0][j]);
      fma_(acc.e[i][j], conj(a.e[1][i]), b.e[1][j]);
      fma_(acc.e[i][j], conj(a.e[2][i]), b.e[2][j]);
    }
}

// acc += A^dag*B^dag
template <typename R>
__device__ __forceinline__ void mac_aa(mat3<R>& acc, const mat3<R>& a, const mat3<R>& b) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      fma_(acc.e[i][j], conj(a.e[0][i]), conj(b.e[j][0]));
      fma_(acc.e[i][j], conj(a.e[1][i]), conj(b.e[j][1]));
      fma_(acc.e[i][j], conj(a.e[2][i]), conj(b.e[j][2]));
    }
}

// double-float accumulating products as compensated dot products
__device__ __forceinline__ void mac_nn(mat3<dfl>& acc, const mat3<dfl>& a, const mat3<dfl>& b) { df_mac<false, false>(acc, a, b); }
__device__ __forceinline__ void mac_na(mat3<dfl>& acc, const mat3<dfl>& a, const mat3<dfl>& b) { df_mac<false, true>(acc, a, b); }
__device__ __forceinline__ void mac_an(mat3<dfl>& acc, const mat3<dfl>& a, const mat3<dfl>& b) { df_mac<true, false>(acc, a, b); }
__device__ __forceinline__ void mac_aa(mat3<dfl>& acc, const mat3<dfl>& a, const mat3<dfl>& b) { df_mac<true, true>(acc, a, b); }

template <typename R, class SRC>
__device__ __forceinline__ void add_staple_pair(mat3<R>& acc, const SRC& U, const Geom& g, const Site& st, int s,
                                                int mu, int nu) {
  const int V = g.vol;
  const int xpm = nbr_rt(g, st, mu, +1);
  const int xpn = nbr_rt(g, st, nu, +1);
  const int xmn = nbr_rt(g, st, nu, -1);
  const int xpm_mn = nbr2_rt(g, st, mu, +1, nu, -1);
  // up: U_nu(x+mu) U_mu(x+nu)^dag U_nu(x)^dag
  mat3<R> t = mul_na(U(nu, xpm, V), U(mu, xpn, V));
  mac_na(acc, t, U(nu, s, V));
  // down: U_nu(x+mu-nu)^dag U_mu(x-nu)^dag U_nu(x-nu)
  t = mul_aa(U(nu, xpm_mn, V), U(mu, xmn, V));
  mac_nn(acc, t, U(nu, xmn, V));
}

// S_mu(x); the three other axes nu = mu+1, mu+2, mu+3 (mod 4) in a run-time loop
template <typename R, class SRC>
__device__ __forceinline__ mat3<R> staple_sum(int mu, const SRC& U, const Geom& g, const Site& st, int s) {
  mat3<R> acc = zero3<R>();
#pragma unroll 1
  for (int k = 1; k < 4; ++k) add_staple_pair<R>(acc, U, g, st, s, mu, (mu + k) & 3);
  return acc;
}

// Sum over mu<nu of Re tr P_munu(x) at one site.
template <typename R, class SRC, int MU, int NU>
__device__ __forceinline__ R plaq_pair(const SRC& U, const Geom& g, const Site& st, int s) {
  const int V = g.vol;
  mat3<R> a = mul_nn(U(MU, s, V), U(NU, nbr<MU>(g, st, +1), V));  // U_mu(x) U_nu(x+mu)
  mat3<R> b = mul_nn(U(NU, s, V), U(MU, nbr<NU>(g, st, +1), V));  // U_nu(x) U_mu(x+nu)
  return retr_na(a, b);
}

template <typename R, class SRC>
__device__ __forceinline__ R plaq_site(const SRC& U, const Geom& g, const Site& st, int s) {
  R v = plaq_pair<R, SRC, 0, 1>(U, g, st, s);
  v += plaq_pair<R, SRC, 0, 2>(U, g, st, s);
  v += plaq_pair<R, SRC, 0, 3>(U, g, st, s);
  v += plaq_pair<R, SRC, 1, 2>(U, g, st, s);
  v += plaq_pair<R, SRC, 1, 3>(U, g, st, s);
  v += plaq_pair<R, SRC, 2, 3>(U, g, st, s);
  return v;
}

__device__ __forceinline__ void block_partial_sum(double v, double* __restrict__ part) {
  __shared__ double sh[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    v = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) part[blockIdx.x] = v;
  }
}

}  // namespace gf

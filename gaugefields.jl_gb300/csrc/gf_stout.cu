// Stout smearing (Morningstar-Peardon) forward and adjoint kernels.
//
// Forward, per level and link (forward!, src/smearing/stout_fast.jl:250-275):
//   C_mu  = rho * sum_{nu != mu} [U_nu(x) U_mu(x+nu) U_nu(x+mu)^dag
//                                 + U_nu(x-nu)^dag U_mu(x-nu) U_nu(x-nu+mu)] = rho S_mu^dag
//   Omega = C_mu U_mu^dag,  Q = TA(Omega),  Ubar_mu = exp(Q) U_mu.
//
// Adjoint, per level (backward_dSdUαUβρ_add!, stout_fast.jl:317-408). With
// Dbar = dS/dUbar (Wirtinger derivative, dS = 2 Re tr(dUbar Dbar)):
//   Lambda = U Dbar, Gamma = C star dexp(Q)/dQ (CdexpQdQ!, stout_fast.jl:888-946)
//   Y  = TA(Gamma)            (calc_dSdΩ!, :678-685)
//   Z  = U^dag Y = dS/dC      (calc_dSdC!, :687)
//   Dp = Dbar exp(Q) + (Y C)^dag   (calc_dSdu1! :629 and calc_dSdUdag! :692)
//   D_nu(x) = Dp_nu(x) + rho * [pull-back of Z through C(U)]   (calc_dSdUν_fromdSCμ_add!, :712-785)
// The last step is written as a gather over the 18 staple positions in which
// a link U_nu(x) enters some C_kappa(y), so no atomics are needed.
//
// Two kernels per backward level: k_bwd_local (Lambda .. Dp, Z) and
// k_bwd_gather (the pull-back through C, fused with the thin-link MD force
// and momentum update at the bottom level).
#include "gf_internal.h"
#include "stencil.cuh"
#include "dfslots.cuh"
#include <type_traits>



namespace gf {

template <typename R>
struct Prec;
template <>
struct Prec<double> {
  typedef LinkSrc<double, false> Src;
  typedef double2 LinkElem;
  typedef double2 MatElem;
  static constexpr int link_kind = GF_LINK64;
  static constexpr int mat_kind = GF_MAT64;
  static __device__ __forceinline__ void store_link(double2* p, int mu, int s, int V, const mat3<double>& m) {
    LinkFull<double>::store(p, mu, s, V, m);
  }
};
template <>
struct Prec<float> {
  typedef LinkSrc<float, true> Src;
  typedef float4 LinkElem;
  typedef float2 MatElem;
  static constexpr int link_kind = GF_LINK32;
  static constexpr int mat_kind = GF_MAT32;
  static __device__ __forceinline__ void store_link(float4* p, int mu, int s, int V, const mat3<float>& m) {
    Link12f::store(p, mu, s, V, m);
  }
};

// i * r * A  (elementwise)
template <typename R>
__device__ __forceinline__ mat3<R> times_i(R r, const mat3<R>& a) {
  mat3<R> b;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) b.e[i][j] = mk(-r * a.e[i][j].im, r * a.e[i][j].re);
  return b;
}

// --------------------------------------------------------------------------
// forward level
// --------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(128, GF_MINB(R))
    k_stout_fwd(typename Prec<R>::Src U, typename Prec<R>::LinkElem* __restrict__ Uout,
                typename Prec<R>::MatElem* __restrict__ Cout, Geom g, R rho) {
  int s, mu;
  link_of_thread(s, mu);
  if (s >= g.vol) return;
  const int V = g.vol;
  Site st = site_of(g, s);
  mat3<R> S = staple_sum<R>(mu, U, g, st, s);
  mat3<R> u = U(mu, s, V);
  // Omega = rho (U S)^dag, Q = TA(Omega) = -rho TA(U S), exp(Q) = exp(i Qh), Qh = i rho TA(U S)
  mat3<R> M = mul_nn(u, S);
  mat3<R> qh = times_i(rho, ta_proj(M));
  if constexpr (std::is_same<R, float>::value) {
    // 12-real output: rows 1-2 of e^Q U are all that is stored
    Prec<R>::store_link(Uout, mu, s, V, mul_nn_rows12(expiq<R, 2>(qh), u));
  } else {
    Prec<R>::store_link(Uout, mu, s, V, mul_nn(expiq(qh), u));
  }
  if (Cout) LinkFull<R>::store(Cout, mu, s, V, scale(rho, dag(S)));
}

// --------------------------------------------------------------------------
// backward, local part
// --------------------------------------------------------------------------
template <typename R, bool TOP>
__global__ void __launch_bounds__(128, GF_MINB_ADJ(R))
    k_bwd_local(typename Prec<R>::Src U, typename Prec<R>::Src Utop, const typename Prec<R>::MatElem* __restrict__ Dbar,
                const typename Prec<R>::MatElem* __restrict__ Cst, typename Prec<R>::MatElem* __restrict__ Zout,
                typename Prec<R>::MatElem* __restrict__ Dpout, Geom g, R rho, R halfbeta) {
  int s, mu;
  link_of_thread(s, mu);
  if (s >= g.vol) return;
  const int V = g.vol;
  Site st = site_of(g, s);
  mat3<R> u = U(mu, s, V);
  mat3<R> C;
  if (Cst) C = LinkFull<R>::load(Cst, mu, s, V);
  else C = scale(rho, dag(staple_sum<R>(mu, U, g, st, s)));
  // Qh = -i TA(C U^dag)
  mat3<R> qh = times_i(R(-1), ta_proj(mul_na(C, u)));
  R c0, c1;
  herm_invariants(qh, c0, c1);
  ch_coef<R> cc;
  ch_coefficients<R, true>(c0, c1, cc);
  mat3<R> qh2 = herm_square(qh);
  mat3<R> db;
  if (TOP) db = scale(halfbeta, staple_sum<R>(mu, Utop, g, st, s));
  else db = LinkFull<R>::load(Dbar, mu, s, V);
  mat3<R> lam = mul_nn(u, db);
  cplx<R> trL = trace(lam), trLQ = tr_nn(lam, qh), trLQ2 = tr_nn(lam, qh2);
  cplx<R> trB1 = cc.b1[0] * trL + cc.b1[1] * trLQ + cc.b1[2] * trLQ2;
  cplx<R> trB2 = cc.b2[0] * trL + cc.b2[1] * trLQ + cc.b2[2] * trLQ2;
  // Gamma_MP = trB1 Qh + trB2 Qh^2 + f1 Lambda + f2 (Qh Lambda + Lambda Qh)
  mat3<R> gam = mul_nn(qh, lam);
  mac_nn(gam, lam, qh);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      cplx<R> v = cc.f[2] * gam.e[i][j];
      fma_(v, cc.f[1], lam.e[i][j]);
      fma_(v, trB1, qh.e[i][j]);
      fma_(v, trB2, qh2.e[i][j]);
      gam.e[i][j] = v;
    }
  // dS/dQ = -i Gamma_MP, Y = TA(dS/dQ)
  mat3<R> Y = ta_proj(times_i(R(-1), gam));
  LinkFull<R>::store(Zout, mu, s, V, mul_an(u, Y));
  // exp(Q) = f0 + f1 Qh + f2 Qh^2
  mat3<R> E;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      cplx<R> v = cc.f[1] * qh.e[i][j];
      fma_(v, cc.f[2], qh2.e[i][j]);
      if (i == j) v = v + cc.f[0];
      E.e[i][j] = v;
    }
  mat3<R> dp = mul_nn(db, E);
  mac_aa(dp, C, Y);  // (Y C)^dag = C^dag Y^dag
  LinkFull<R>::store(Dpout, mu, s, V, dp);
}

// --------------------------------------------------------------------------
// backward, gather of the pull-back through C(U)
// --------------------------------------------------------------------------
// Six contributions to D_nu(x) from the staples that involve the axis K:
//  (a) U_K(x+nu) U_nu(x+K)^dag Z_K(x)          (b) U_K(x-K+nu)^dag U_nu(x-K)^dag Z_K(x-K)^dag
//  (c) Z_K(x+nu)^dag U_nu(x+K)^dag U_K(x)^dag  (d) Z_K(x+nu-K) U_nu(x-K)^dag U_K(x-K)
//  (e) U_K(x-K+nu)^dag Z_nu(x-K) U_K(x-K)      (f) U_K(x+nu) Z_nu(x+K) U_K(x)^dag
template <typename R>
__device__ __forceinline__ void gather_axis(mat3<R>& acc, const typename Prec<R>::Src& U,
                                            const typename Prec<R>::MatElem* __restrict__ Z, const Geom& g,
                                            const Site& st, int s, int NU, int K) {
  const int V = g.vol;
  const int xpn = nbr_rt(g, st, NU, +1);
  const int xpk = nbr_rt(g, st, K, +1);
  const int xmk = nbr_rt(g, st, K, -1);
  const int xmk_pn = nbr2_rt(g, st, K, -1, NU, +1);
  {
    mat3<R> a1 = U(K, xpn, V);   // U_K(x+nu)
    mat3<R> a2 = U(NU, xpk, V);  // U_nu(x+K)
    mat3<R> a6 = U(K, s, V);     // U_K(x)
    // (a) + (f) = U_K(x+nu) [U_nu(x+K)^dag Z_K(x) + Z_nu(x+K) U_K(x)^dag]
    mat3<R> t = mul_an(a2, LinkFull<R>::load(Z, K, s, V));
    mac_na(t, LinkFull<R>::load(Z, NU, xpk, V), a6);
    mac_nn(acc, a1, t);
    // (c) = Z_K(x+nu)^dag [U_K(x) U_nu(x+K)]^dag
    t = mul_nn(a6, a2);
    mac_aa(acc, LinkFull<R>::load(Z, K, xpn, V), t);
  }
  {
    mat3<R> a3 = U(K, xmk_pn, V);  // U_K(x-K+nu)
    mat3<R> a4 = U(NU, xmk, V);    // U_nu(x-K)
    mat3<R> a5 = U(K, xmk, V);     // U_K(x-K)
    // (b) = [U_nu(x-K) U_K(x-K+nu)]^dag Z_K(x-K)^dag
    mat3<R> t = mul_nn(a4, a3);
    mac_aa(acc, t, LinkFull<R>::load(Z, K, xmk, V));
    // (d) + (e) = [Z_K(x+nu-K) U_nu(x-K)^dag + U_K(x-K+nu)^dag Z_nu(x-K)] U_K(x-K)
    t = mul_na(LinkFull<R>::load(Z, K, xmk_pn, V), a4);
    mac_an(t, a3, LinkFull<R>::load(Z, NU, xmk, V));
    mac_nn(acc, t, a5);
  }
}

template <typename R, bool FORCE>
__global__ void __launch_bounds__(128, GF_MINB_ADJ(R))
    k_bwd_gather(typename Prec<R>::Src U, const typename Prec<R>::MatElem* __restrict__ Z,
                 const typename Prec<R>::MatElem* __restrict__ Dp, typename Prec<R>::MatElem* __restrict__ Dout,
                 double* __restrict__ P, Geom g, R rho, double coef) {
  int s, nu;
  link_of_thread(s, nu);
  if (s >= g.vol) return;
  const int V = g.vol;
  Site st = site_of(g, s);
  mat3<R> acc = zero3<R>();
#pragma unroll 1
  for (int k = 1; k < 4; ++k) gather_axis<R>(acc, U, Z, g, st, s, nu, (nu + k) & 3);
  mat3<R> d = LinkFull<R>::load(Dp, nu, s, V);
  axpy_to(d, rho, acc);
  if (FORCE) {
    // thin-link MD force F = -(1/3) TA(U dS/dU), P += eps F  (coef = -eps/3)
    mat3<R> M = mul_nn(U(nu, s, V), d);
    R c[8];
    ta_coeffs(M, c);
    double* p = P + (size_t)nu * 8 * V + s;
#pragma unroll
    for (int a = 0; a < 8; ++a) p[(size_t)a * V] += coef * to_f64(c[a]);
  } else {
    LinkFull<R>::store(Dout, nu, s, V, d);
  }
}

// --------------------------------------------------------------------------
// Double-float kernels as loops over tables of products. Inlined, every
// double-float 3x3 product is about 1,400 instructions; the stout kernels hold
// 14-30 of them, overflow the instruction cache and stall on instruction
// fetch (ncu). Here one product sits in the body of a run-time loop over a
// table of operations. Each operand is a link of one of up to three fields
// (at one of five sites, in one of two directions) or a per-thread slot in
// shared memory, optionally daggered; the result goes to a slot, optionally
// added to it. The order of the operations is that of the inlined kernels, so
// the results are the same. Out-of-line forms of the product were slower (argument passing) or
// miscompiled (pointers into the caller's registers), which this avoids.
// --------------------------------------------------------------------------
// Products of the table kernels: the fixed-grid form (dfg_matmul, six fp32
// operations per term) or the TwoSum-based one (df_matmul, twelve).
#ifndef GF_DF_GRID
#define GF_DF_GRID 1
#endif

struct DfOp {
  // src: 0, 1, 2 fields F0, F1, F2, 3 + k slot k; dir: 0 the kernel's link
  // direction, 1 the loop axis; site: index into the kernel's five sites
  unsigned char a_src, a_dir, a_site, a_dag, b_src, b_dir, b_site, b_dag, out, accumulate;
};

struct DfSites {
  int x[5];
};
__device__ __forceinline__ int pick_site(const DfSites& st, int i) {
  return i == 0 ? st.x[0] : i == 1 ? st.x[1] : i == 2 ? st.x[2] : i == 3 ? st.x[3] : st.x[4];
}
// The operand fields of a table kernel: F0 in storage E0 (fp64 for the
// level-0 forward of a forward-only stack, which reads the thin links in
// place), F1 and F2 double-float-native.
template <typename E0>
struct DfFields {
  const E0* f0;
  const float4* f1;
  const float4* f2;
};
// Daggered operands: GF_DF_DAG_LOAD = 1 takes the transposition in the load
// addresses (element (i, j) of M^dag is read from (j, i)) and negates the
// imaginary parts after the loads; 0 loads M and forms dag(M) in registers.
// Same results; at 32^4 the address form measured 0.4% slower per trajectory
// alone (gather slower, local adjoint faster) and 2% faster with raw pairs
// (GF_DF_NORM = 0).
#ifndef GF_DF_DAG_LOAD
#define GF_DF_DAG_LOAD 0
#endif
__device__ __forceinline__ int op_elem(int e, int dagger) { return dagger ? (e % 3) * 3 + e / 3 : e; }
template <typename E0>
__device__ __forceinline__ mat3<dfl> df_operand(int src, int dir, int site, int dagger, const float* sm, int tid,
                                                const DfFields<E0>& F, int V, int d0, int d1, const DfSites& st) {
  mat3<dfl> m;
  const int mu = dir ? d1 : d0, x = pick_site(st, site);
#if GF_DF_DAG_LOAD
  if (src == 0 && !std::is_same<E0, float4>::value) {
    m = DfIO<E0>::load(F.f0, mu, x, V);
    if (dagger) m = dag(m);
    return m;
  }
  if (src >= 3) {
    const float4* q = reinterpret_cast<const float4*>(sm) + (src - 3) * 9 * 128 + tid;
#pragma unroll
    for (int e = 0; e < 9; ++e) {
      const float4 v = q[op_elem(e, dagger) * 128];
      m.e[e / 3][e % 3] = mk(dfl(v.x, v.y), dfl(v.z, v.w));
    }
  } else {
    const float4* f = src == 0 ? reinterpret_cast<const float4*>(F.f0) : (src == 1 ? F.f1 : F.f2);
    const float4* b = f + (size_t)mu * 9 * V + x;
#pragma unroll
    for (int e = 0; e < 9; ++e) {
      const float4 v = __ldg(b + (size_t)op_elem(e, dagger) * V);
      m.e[e / 3][e % 3] = mk(dfl(v.x, v.y), dfl(v.z, v.w));
    }
  }
  if (dagger) {
#pragma unroll
    for (int e = 0; e < 9; ++e) m.e[e / 3][e % 3].im = dfl(-m.e[e / 3][e % 3].im.hi, -m.e[e / 3][e % 3].im.lo);
  }
#else
  if (src >= 3) m = slot_load(sm, src - 3, tid);
  else if (src == 0) m = DfIO<E0>::load(F.f0, mu, x, V);
  else m = LinkDfn::load(src == 1 ? F.f1 : F.f2, mu, x, V);
  if (dagger) m = dag(m);
#endif
  return m;
}
template <typename E0>
__device__ __forceinline__ void df_exec(const DfOp op, float* sm, int tid, const DfFields<E0>& F, int V, int d0,
                                        int d1, const DfSites& st) {
  const mat3<dfl> A = df_operand(op.a_src, op.a_dir, op.a_site, op.a_dag, sm, tid, F, V, d0, d1, st);
  const mat3<dfl> B = df_operand(op.b_src, op.b_dir, op.b_site, op.b_dag, sm, tid, F, V, d0, d1, st);
  // one inlined product, always accumulating (into zero when the op does not
  // accumulate): a second, non-accumulating copy in the loop body measured
  // 3% slower per trajectory (larger body)
  const mat3<dfl> C = op.accumulate ? slot_load(sm, op.out, tid) : zero3<dfl>();
#if GF_DF_GRID
  slot_store(sm, op.out, tid, dfg_matmul<false, false, true, 3, GF_DF_NORM>(A, B, &C));
#else
  slot_store(sm, op.out, tid, df_matmul<false, false, true>(A, B, &C));
#endif
}

// The gather: F0 = U, F1 = Z, d0 = nu, d1 = kappa; sites x, x+nu, x+kappa,
// x-kappa, x-kappa+nu; slot 0 = t, slot 1 = acc. The terms (a)..(f) of
// gather_axis in the same factored order.
__constant__ DfOp c_gather_ops[10] = {
    {0, 0, 2, 1, 1, 1, 0, 0, 0, 0},  // t  = U_nu(x+k)^dag Z_k(x)
    {1, 0, 2, 0, 0, 1, 0, 1, 0, 1},  // t += Z_nu(x+k) U_k(x)^dag
    {0, 1, 1, 0, 3, 0, 0, 0, 1, 1},  // acc += U_k(x+nu) t
    {0, 1, 0, 0, 0, 0, 2, 0, 0, 0},  // t  = U_k(x) U_nu(x+k)
    {1, 1, 1, 1, 3, 0, 0, 1, 1, 1},  // acc += Z_k(x+nu)^dag t^dag
    {0, 0, 3, 0, 0, 1, 4, 0, 0, 0},  // t  = U_nu(x-k) U_k(x-k+nu)
    {3, 0, 0, 1, 1, 1, 3, 1, 1, 1},  // acc += t^dag Z_k(x-k)^dag
    {1, 1, 4, 0, 0, 0, 3, 1, 0, 0},  // t  = Z_k(x-k+nu) U_nu(x-k)^dag
    {0, 1, 4, 1, 1, 0, 3, 0, 0, 1},  // t += U_k(x-k+nu)^dag Z_nu(x-k)
    {3, 0, 0, 0, 0, 1, 3, 0, 1, 1},  // acc += t U_k(x-k)
};

// four blocks per SM: 128 registers without spills, 36 KB of shared memory
// each; at 32^4 4.85 ms per launch against 5.42 ms with three blocks (168
// registers) and 6.46 ms with two; five spill (96 registers)
#ifndef GF_DF_GATHER_MINB
#define GF_DF_GATHER_MINB 4
#endif
template <bool FORCE, typename EOUT>
__global__ void __launch_bounds__(128, GF_DF_GATHER_MINB)
    k_bwd_gather_df(const float4* __restrict__ U, const float4* __restrict__ Z, const float4* __restrict__ Dp,
                    EOUT* __restrict__ Dout, double* __restrict__ P, Geom g, dfl rho, double coef) {
  __shared__ __align__(16) float sm[2 * 36 * 128];
  const int tid = threadIdx.x;
  int s, nu;
  link_of_thread(s, nu);
  const bool live = s < g.vol;  // every thread runs the loop; only live ones write global memory
  const int V = g.vol;
  const int sc = live ? s : 0;
  const Site st = site_of(g, sc);
  slot_store(sm, 1, tid, zero3<dfl>());
  DfSites ss;
  ss.x[0] = sc;
  ss.x[1] = nbr_rt(g, st, nu, +1);
#pragma unroll 1
  for (int k = 1; k < 4; ++k) {
    const int K = (nu + k) & 3;
    ss.x[2] = nbr_rt(g, st, K, +1);
    ss.x[3] = nbr_rt(g, st, K, -1);
    ss.x[4] = nbr2_rt(g, st, K, -1, nu, +1);
#pragma unroll 1
    for (int q = 0; q < 10; ++q) df_exec(c_gather_ops[q], sm, tid, DfFields<float4>{U, Z, Z}, V, nu, K, ss);
  }
  if (!live) return;
  mat3<dfl> d = LinkDfn::load(Dp, nu, s, V);
  axpy_to(d, rho, slot_load_n(sm, 1, tid));
  if (FORCE) {
    const mat3<dfl> M = mul_nn(LinkDfn::load(U, nu, s, V), d);
    dfl c[8];
    ta_coeffs(M, c);
    double* p = P + (size_t)nu * 8 * V + s;
#pragma unroll
    for (int a = 0; a < 8; ++a) p[(size_t)a * V] += coef * to_f64(c[a]);
  } else {
    DfIO<EOUT>::store(Dout, nu, s, V, d);
  }
}

// The stout forward: F0 = U, d0 = mu, d1 = nu; sites x, x+mu, x+nu,
// x+mu-nu, x-nu; slot 0 = t, slot 1 = acc. Ops 0-3 (per nu) build S_mu in
// dS/dU order as add_staple_pair does; op 4 forms U S; op 5 e^Q U.
__constant__ DfOp c_stout_ops[6] = {
    {0, 1, 1, 0, 0, 0, 2, 1, 0, 0},  // t  = U_nu(x+mu) U_mu(x+nu)^dag
    {3, 0, 0, 0, 0, 1, 0, 1, 1, 1},  // acc += t U_nu(x)^dag
    {0, 1, 3, 1, 0, 0, 4, 1, 0, 0},  // t  = U_nu(x+mu-nu)^dag U_mu(x-nu)^dag
    {3, 0, 0, 0, 0, 1, 4, 0, 1, 1},  // acc += t U_nu(x-nu)
    {0, 0, 0, 0, 4, 0, 0, 0, 0, 0},  // t  = U_mu(x) S
    {3, 0, 0, 0, 0, 0, 0, 0, 1, 0},  // acc = e^Q U_mu(x)   (slot 0 holds e^Q by then)
};

// three blocks per SM (168 registers); four fit without spills at 128
// registers but measured 4% slower
#ifndef GF_DF_FWD_MINB
#define GF_DF_FWD_MINB 3
#endif
template <typename EIN>
__global__ void __launch_bounds__(128, GF_DF_FWD_MINB)
    k_stout_fwd_df(const EIN* __restrict__ U, float4* __restrict__ Uout, float4* __restrict__ Cout, Geom g,
                   dfl rho) {
  __shared__ __align__(16) float sm[2 * 36 * 128];
  const int tid = threadIdx.x;
  int s, mu;
  link_of_thread(s, mu);
  const bool live = s < g.vol;
  const int V = g.vol;
  const int sc = live ? s : 0;
  const Site st = site_of(g, sc);
  slot_store(sm, 1, tid, zero3<dfl>());
  DfSites ss;
  ss.x[0] = sc;
  ss.x[1] = nbr_rt(g, st, mu, +1);
  int nu = 0;
#pragma unroll 1
  for (int q = 0; q < 14; ++q) {
    if (q < 12 && (q & 3) == 0) {
      nu = (mu + 1 + (q >> 2)) & 3;
      ss.x[2] = nbr_rt(g, st, nu, +1);
      ss.x[3] = nbr2_rt(g, st, mu, +1, nu, -1);
      ss.x[4] = nbr_rt(g, st, nu, -1);
    }
    if (q == 13) {
      // Q = TA(rho S^dag U^dag) = -rho TA(U S): exp(Q) = exp(i Qh), Qh = i rho TA(U S)
      const mat3<dfl> qh = times_i(rho, ta_proj(slot_load_n(sm, 0, tid)));
      slot_store(sm, 0, tid, expiq(qh));
      if (Cout && live) LinkDfn::store(Cout, mu, s, V, scale(rho, dag(slot_load_n(sm, 1, tid))));
    }
    df_exec(c_stout_ops[q < 12 ? (q & 3) : q - 8], sm, tid, DfFields<EIN>{U, nullptr, nullptr}, V, mu, nu, ss);
  }
  if (live) LinkDfn::store(Uout, mu, s, V, slot_load_n(sm, 1, tid));
}

// The coefficient algebra of the double-float local adjoint, as fixed-grid
// sums: on entry gam holds Qh Lambda + Lambda Qh; on exit
//   gam = f2 (Qh Lambda + Lambda Qh) + f1 Lambda + trB1 Qh + trB2 Qh^2,
//   E   = f0 + f1 Qh + f2 Qh^2 = exp(Q),
// with trB_k = b_k[0] tr(Lambda) + b_k[1] tr(Lambda Qh) + b_k[2] tr(Lambda Qh^2)
// (CdexpQdQ!, src/smearing/stout_fast.jl:888-946).
__device__ __forceinline__ void df_gamma_and_exp(const ch_coef<dfl>& cc, const mat3<dfl>& lam, const mat3<dfl>& qh,
                                                 const mat3<dfl>& qh2, mat3<dfl>& gam, mat3<dfl>& E) {
  const cplx<dfl> trL = trace(lam), trLQ = tr_nn(lam, qh), trLQ2 = tr_nn(lam, qh2);
  cplx<dfl> trB[2];
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const cplx<dfl>* b = k ? cc.b2 : cc.b1;
    dfg_cacc t = dfg_cbegin(cabs1(b[0]) * cabs1(trL) + cabs1(b[1]) * cabs1(trLQ) + cabs1(b[2]) * cabs1(trLQ2));
    dfg_cterm(t, b[0], trL);
    dfg_cterm(t, b[1], trLQ);
    dfg_cterm(t, b[2], trLQ2);
    trB[k] = dfg_cend(t);
  }
  const float m2 = cabs1(cc.f[2]), m1 = cabs1(cc.f[1]), m0 = cabs1(cc.f[0]);
  const float b1 = cabs1(trB[0]), b2 = cabs1(trB[1]);
  const cplx<dfl> one = mk(dfl(1.f), dfl(0.f));
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      dfg_cacc v = dfg_cbegin(m2 * cabs1(gam.e[i][j]) + m1 * cabs1(lam.e[i][j]) + b1 * cabs1(qh.e[i][j]) +
                              b2 * cabs1(qh2.e[i][j]));
      dfg_cterm(v, cc.f[2], gam.e[i][j]);
      dfg_cterm(v, cc.f[1], lam.e[i][j]);
      dfg_cterm(v, trB[0], qh.e[i][j]);
      dfg_cterm(v, trB[1], qh2.e[i][j]);
      gam.e[i][j] = dfg_cend(v);
      dfg_cacc w = dfg_cbegin(m1 * cabs1(qh.e[i][j]) + m2 * cabs1(qh2.e[i][j]) + (i == j ? m0 : 0.f));
      dfg_cterm(w, cc.f[1], qh.e[i][j]);
      dfg_cterm(w, cc.f[2], qh2.e[i][j]);
      if (i == j) dfg_cterm(w, cc.f[0], one);
      E.e[i][j] = dfg_cend(w);
    }
}

// The local adjoint: F0 = U, F1 = Dbar (or the top level's smeared links),
// F2 = the stored C; d0 = mu, d1 = nu; sites x, x+mu, x+nu, x+mu-nu, x-nu.
// Slots: 0 work (U C^dag, then Gamma, then Y), 1 Qh, 2 Qh^2 then e^Q,
// 3 Lambda then Z then Dp, 4 Dbar of the top level, 5 a recomputed C.
// Operand codes 14 and 15 stand for C and Dbar, resolved per launch.
#define GF_LOCAL_SLOTS 6
__constant__ DfOp c_local_ops[31] = {
    // 0-11: S_mu of F0 into slot 5 (C recomputed), in dS/dU order
    {0, 1, 1, 0, 0, 0, 2, 1, 0, 0}, {3, 0, 0, 0, 0, 1, 0, 1, 5, 1},
    {0, 1, 3, 1, 0, 0, 4, 1, 0, 0}, {3, 0, 0, 0, 0, 1, 4, 0, 5, 1},
    {0, 1, 1, 0, 0, 0, 2, 1, 0, 0}, {3, 0, 0, 0, 0, 1, 0, 1, 5, 1},
    {0, 1, 3, 1, 0, 0, 4, 1, 0, 0}, {3, 0, 0, 0, 0, 1, 4, 0, 5, 1},
    {0, 1, 1, 0, 0, 0, 2, 1, 0, 0}, {3, 0, 0, 0, 0, 1, 0, 1, 5, 1},
    {0, 1, 3, 1, 0, 0, 4, 1, 0, 0}, {3, 0, 0, 0, 0, 1, 4, 0, 5, 1},
    // 12-23: S_mu of F1 into slot 4 (top level: Dbar = beta/2 S)
    {1, 1, 1, 0, 1, 0, 2, 1, 0, 0}, {3, 0, 0, 0, 1, 1, 0, 1, 4, 1},
    {1, 1, 3, 1, 1, 0, 4, 1, 0, 0}, {3, 0, 0, 0, 1, 1, 4, 0, 4, 1},
    {1, 1, 1, 0, 1, 0, 2, 1, 0, 0}, {3, 0, 0, 0, 1, 1, 0, 1, 4, 1},
    {1, 1, 3, 1, 1, 0, 4, 1, 0, 0}, {3, 0, 0, 0, 1, 1, 4, 0, 4, 1},
    {1, 1, 1, 0, 1, 0, 2, 1, 0, 0}, {3, 0, 0, 0, 1, 1, 0, 1, 4, 1},
    {1, 1, 3, 1, 1, 0, 4, 1, 0, 0}, {3, 0, 0, 0, 1, 1, 4, 0, 4, 1},
    {14, 0, 0, 0, 0, 0, 0, 1, 0, 0},  // 24: work = C U^dag
    {0, 0, 0, 0, 15, 0, 0, 0, 3, 0},  // 25: Lambda = U Dbar
    {4, 0, 0, 0, 6, 0, 0, 0, 0, 0},   // 26: work = Qh Lambda
    {6, 0, 0, 0, 4, 0, 0, 0, 0, 1},   // 27: work += Lambda Qh
    {0, 0, 0, 1, 3, 0, 0, 0, 3, 0},   // 28: Z = U^dag Y
    {15, 0, 0, 0, 5, 0, 0, 0, 3, 0},  // 29: Dp = Dbar e^Q
    {14, 0, 0, 1, 3, 0, 0, 1, 3, 1},  // 30: Dp += C^dag Y^dag
};

// Blocks per SM of the local adjoint below the top level. Its slots 0-3
// (72 KB) would let three blocks share an SM, but at the 168 registers that
// takes it spills and measured 4.47 ms per 32^4 launch against 4.31 ms with
// two blocks at 255 registers.
#ifndef GF_DF_LOCAL_MINB_LOWER
#define GF_DF_LOCAL_MINB_LOWER 2
#endif
template <bool TOP>
__global__ void __launch_bounds__(128, TOP ? GF_MINB_ADJ(dfl) : GF_DF_LOCAL_MINB_LOWER)
    k_bwd_local_df(const float4* __restrict__ U, const float4* __restrict__ F1, const float4* __restrict__ Cst,
                   float4* __restrict__ Zout, float4* __restrict__ Dpout, Geom g, dfl rho, dfl halfbeta) {
  extern __shared__ float sm[];  // GF_LOCAL_SLOTS slots of 36 x 128 floats
  const int tid = threadIdx.x;
  int s, mu;
  link_of_thread(s, mu);
  const bool live = s < g.vol;
  const int V = g.vol;
  const int sc = live ? s : 0;
  const Site st = site_of(g, sc);
  const bool recompute = Cst == nullptr;
  const DfFields<float4> F{U, F1, Cst ? Cst : U};
  DfSites ss;
  ss.x[0] = sc;
  ss.x[1] = nbr_rt(g, st, mu, +1);
  int nu = 0;
  ch_coef<dfl> cc;
#pragma unroll 1
  for (int q = 0; q < 31; ++q) {
    if (q < 12 && !recompute) continue;
    if (q >= 12 && q < 24 && !TOP) continue;
    if (q < 24) {
      const int r = q < 12 ? q : q - 12;
      if ((r & 3) == 0) {
        nu = (mu + 1 + (r >> 2)) & 3;
        ss.x[2] = nbr_rt(g, st, nu, +1);
        ss.x[3] = nbr2_rt(g, st, mu, +1, nu, -1);
        ss.x[4] = nbr_rt(g, st, nu, -1);
      }
      if (r == 0) slot_store(sm, q < 12 ? 5 : 4, tid, zero3<dfl>());
    }
    DfOp op = c_local_ops[q];
    if (op.a_src == 14) op.a_src = recompute ? 8 : 2;
    if (op.b_src == 14) op.b_src = recompute ? 8 : 2;
    if (op.a_src == 15) op.a_src = TOP ? 7 : 1;
    if (op.b_src == 15) op.b_src = TOP ? 7 : 1;
    df_exec(op, sm, tid, F, V, mu, nu, ss);
    if (q == 11) slot_store(sm, 5, tid, scale(rho, dag(slot_load_n(sm, 5, tid))));  // C = rho S^dag
    if (q == 23) slot_store(sm, 4, tid, scale(halfbeta, slot_load_n(sm, 4, tid)));  // Dbar = beta/2 S
    if (q == 24) {
      // Qh = -i TA(C U^dag)
      const mat3<dfl> qh = times_i(dfl(-1), ta_proj(slot_load_n(sm, 0, tid)));
      dfl c0, c1;
      herm_invariants(qh, c0, c1);
      ch_coefficients<dfl, true>(c0, c1, cc);
      slot_store(sm, 1, tid, qh);
      slot_store(sm, 2, tid, herm_square(qh));
    }
    if (q == 27) {
      const mat3<dfl> lam = slot_load_n(sm, 3, tid), qh = slot_load(sm, 1, tid), qh2 = slot_load(sm, 2, tid);
      mat3<dfl> gam = slot_load_n(sm, 0, tid);
      mat3<dfl> E;
      df_gamma_and_exp(cc, lam, qh, qh2, gam, E);
      slot_store(sm, 0, tid, ta_proj(times_i(dfl(-1), gam)));  // Y
      slot_store(sm, 2, tid, E);                                // e^Q
    }
    if (q == 28 && live) LinkDfn::store(Zout, mu, s, V, slot_load_n(sm, 3, tid));
  }
  if (live) LinkDfn::store(Dpout, mu, s, V, slot_load_n(sm, 3, tid));
}

// --------------------------------------------------------------------------
// dS/drho of one level (parameter_derivatives, the rho part of
// backward_dSdUαUβρ_add!, src/smearing/stout_fast.jl:371-386). With
// C = rho S^dag and Z = dS/dC from the level's local adjoint,
//   dS/drho = 2 Re sum_{x,mu} tr(Z_mu(x) S_mu(x)^dag),
// S recomputed from the level input (valid at rho = 0 too). One partial sum
// per block (deterministic two-stage reduction).
// --------------------------------------------------------------------------
template <typename R, class SRC, class ZL>
__global__ void __launch_bounds__(128) k_dsdrho(SRC U, ZL Z, Geom g, double* __restrict__ part) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  double v = 0.0;
  if (s < g.vol) {
    const Site st = site_of(g, s);
#pragma unroll 1
    for (int mu = 0; mu < 4; ++mu) {
      const mat3<R> S = staple_sum<R>(mu, U, g, st, s);
      const mat3<R> z = Z(mu, s, g.vol);
      R t = R(0);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) t += z.e[i][j].re * S.e[i][j].re + z.e[i][j].im * S.e[i][j].im;
      v += 2.0 * (double)t;
    }
  }
  block_partial_sum(v, part);
}

// dS/drho of level `l` from the stack's Z (after that level's local adjoint)
static double level_dsdrho(gf_ctx* ctx, gf_stout* st, int l) {
  const int nb = blocks_for(ctx->geom.vol, 128);
  const gf_field* u = st->lev_in[l];
  if (st->precision == GF_FP64) {
    k_dsdrho<double><<<nb, 128, 0, ctx->stream>>>(LinkSrc<double, false>{(const double2*)u->ptr},
                                                  LinkSrc<double, false>{(const double2*)st->Z->ptr}, ctx->geom,
                                                  ctx->d_partials);
  } else if (st->precision == GF_MIXED) {
    k_dsdrho<float><<<nb, 128, 0, ctx->stream>>>(LinkSrc<float, true>{(const float4*)u->ptr},
                                                 LinkSrc<float, false>{(const float2*)st->Z->ptr}, ctx->geom,
                                                 ctx->d_partials);
  } else if (u->kind == GF_LINKDF) {
    // double-float stack: fp64 arithmetic on hi + lo
    k_dsdrho<double><<<nb, 128, 0, ctx->stream>>>(LinkSrcDfn64{(const float4*)u->ptr},
                                                  LinkSrcDfn64{(const float4*)st->Z->ptr}, ctx->geom,
                                                  ctx->d_partials);
  } else {
    throw gf_error(GF_EINVAL, "dS/drho: unexpected level storage");
  }
  GF_CHECK_LAUNCH();
  return finish_reduction(ctx, nb);
}

// --------------------------------------------------------------------------
// host drivers
// --------------------------------------------------------------------------
template <typename R>
static typename Prec<R>::Src src_of(const gf_field* f) {
  typename Prec<R>::Src s;
  s.p = (const typename Prec<R>::LinkElem*)f->ptr;
  return s;
}

// profiling class of a kernel stage in arithmetic type R
template <typename R>
static int kclass(int f32, int f64, int df) {
  return std::is_same<R, float>::value ? f32 : (std::is_same<R, double>::value ? f64 : df);
}

template <typename R>
static void forward_impl(gf_ctx* ctx, gf_stout* st) {
  dim3 grid = stencil_grid(ctx->geom.vol, 128);
  for (int l = 0; l < st->nlev; ++l) {
    ProfScope prof(ctx, kclass<R>(GF_K_STOUT_FWD, GF_K_STOUT_FWD64, GF_K_STOUT_FWD_DF));
    if constexpr (std::is_same<R, dfl>::value) {
      // double-float stacks store every level natively; level 0 of a
      // forward-only stack is the fp64 thin links, read in place
      float4* cout = st->store ? (float4*)st->C[l]->ptr : nullptr;
      float4* uout = (float4*)st->lev_in[l + 1]->ptr;
      if (st->lev_in[l]->kind == GF_LINK64)
        k_stout_fwd_df<double2><<<grid, 128, 0, ctx->stream>>>((const double2*)st->lev_in[l]->ptr, uout, cout,
                                                               ctx->geom, (R)st->rho[l]);
      else
        k_stout_fwd_df<float4><<<grid, 128, 0, ctx->stream>>>((const float4*)st->lev_in[l]->ptr, uout, cout,
                                                              ctx->geom, (R)st->rho[l]);
    } else {
      k_stout_fwd<R><<<grid, 128, 0, ctx->stream>>>(
          src_of<R>(st->lev_in[l]), (typename Prec<R>::LinkElem*)st->lev_in[l + 1]->ptr,
          st->store ? (typename Prec<R>::MatElem*)st->C[l]->ptr : nullptr, ctx->geom, (R)st->rho[l]);
    }
    GF_CHECK_LAUNCH();
  }
}

// Kind of a stack's level-0 input: fp32 12-real (mixed), double-float-native
// (a double-float stack with an adjoint keeps its own copy of the thin
// links), or the caller's fp64 links (plain form; forward-only double-float
// stacks read them in place).
static int level0_kind(const gf_stout* st) {
  if (st->precision == GF_MIXED) return GF_LINK32;
  if (st->precision == GF_PREC_DF && !st->fwd_only) return GF_LINKDF;
  return GF_LINK64;
}

void stout_forward(gf_ctx* ctx, gf_stout* st, const gf_field* U, gf_field* Uout) {
  const int lk = level0_kind(st);
  gf_field* old = st->lev_in[0];
  if (U->kind == lk) {
    // alias the caller's thin links (not owned by the stack)
    gf_field* a = new gf_field(*U);
    a->owned = 0;
    st->lev_in[0] = a;
    field_delete(old);  // frees storage only if the old entry was owned
  } else if ((lk == GF_LINK32 || lk == GF_LINKDF) && U->kind == GF_LINK64) {
    // keep an owned copy of the fp64 thin links in the stack's storage
    if (!old || !old->owned) {
      st->lev_in[0] = field_new(ctx, lk);
      field_delete(old);
    }
    copy_field(ctx, st->lev_in[0], U);
  } else {
    throw gf_error(GF_EINVAL, "stout forward: link field kind does not match the stack precision");
  }
  if (st->precision == GF_FP64) forward_impl<double>(ctx, st);
  else if (st->precision == GF_PREC_DF) forward_impl<dfl>(ctx, st);
  else forward_impl<float>(ctx, st);
  st->have_forward = 1;
  if (Uout) copy_field(ctx, Uout, st->lev_in[st->nlev]);
}

const gf_field* stout_top(const gf_stout* st) { return st->lev_in[st->nlev]; }

// Double-float adjoint on native storage. A caller's dS/dUbar (fp64) is
// converted into D[1] first: the top level's local kernel reads it before
// that level's gather overwrites D[1] (an internal caller may have written it
// there, double-float-native, already). A caller's dS/dU receives the bottom
// gather's output in fp64.
static void backward_df(gf_ctx* ctx, gf_stout* st, const gf_field* dSdUbar, double beta, gf_field* dSdU,
                        gf_field* P, double eps, double* dsdrho) {
  dim3 grid = stencil_grid(ctx->geom.vol, 128);
  const float4* dbar = nullptr;
  if (dSdUbar) {
    if (dSdUbar != st->D[1]) copy_field(ctx, st->D[1], dSdUbar);
    dbar = (const float4*)st->D[1]->ptr;
  }
  int cur = 0;
  for (int l = st->nlev - 1; l >= 0; --l) {
    const bool top = (l == st->nlev - 1) && dSdUbar == nullptr;
    const float4* Cst = st->store ? (const float4*)st->C[l]->ptr : nullptr;
    const float4* din = (l == st->nlev - 1) ? dbar : (const float4*)st->D[cur]->ptr;
    const float4* u = (const float4*)st->lev_in[l]->ptr;
    {
      ProfScope prof(ctx, GF_K_BWD_LOCAL_DF);
      const float4* f1 = top ? (const float4*)st->lev_in[l + 1]->ptr : din;
      // slots used: 0-3, 4 (the top level's Dbar), 5 (a recomputed C)
      const int nslots = Cst == nullptr ? GF_LOCAL_SLOTS : (top ? 5 : 4);
      const size_t smem = (size_t)nslots * 36 * 128 * sizeof(float);
      auto kern = top ? k_bwd_local_df<true> : k_bwd_local_df<false>;
      GF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      kern<<<grid, 128, smem, ctx->stream>>>(u, f1, Cst, (float4*)st->Z->ptr, (float4*)st->Dp->ptr, ctx->geom,
                                             (dfl)st->rho[l], (dfl)(0.5 * beta));
      GF_CHECK_LAUNCH();
    }
    if (dsdrho) dsdrho[l] = level_dsdrho(ctx, st, l);
    const int nxt = cur ^ 1;
    ProfScope prof(ctx, GF_K_BWD_GATHER_DF);
    const float4* z = (const float4*)st->Z->ptr;
    const float4* dp = (const float4*)st->Dp->ptr;
    if (l == 0 && P) {
      k_bwd_gather_df<true, float4><<<grid, 128, 0, ctx->stream>>>(u, z, dp, nullptr, (double*)P->ptr, ctx->geom,
                                                                   (dfl)st->rho[0], -eps / 3.0);
    } else if (l == 0 && dSdU) {
      k_bwd_gather_df<false, double2><<<grid, 128, 0, ctx->stream>>>(u, z, dp, (double2*)dSdU->ptr, nullptr,
                                                                     ctx->geom, (dfl)st->rho[0], 0.0);
    } else {
      k_bwd_gather_df<false, float4><<<grid, 128, 0, ctx->stream>>>(u, z, dp, (float4*)st->D[nxt]->ptr, nullptr,
                                                                    ctx->geom, (dfl)st->rho[l], 0.0);
    }
    GF_CHECK_LAUNCH();
    cur = nxt;
  }
}

template <typename R>
static void backward_impl(gf_ctx* ctx, gf_stout* st, const gf_field* dSdUbar, double beta, gf_field* dSdU,
                          gf_field* P, double eps, double* dsdrho) {
  dim3 grid = stencil_grid(ctx->geom.vol, 128);
  typedef typename Prec<R>::MatElem ME;
  const ME* dbar = dSdUbar ? (const ME*)dSdUbar->ptr : nullptr;
  int cur = 0;
  for (int l = st->nlev - 1; l >= 0; --l) {
    bool top = (l == st->nlev - 1) && dSdUbar == nullptr;
    const ME* Cst = st->store ? (const ME*)st->C[l]->ptr : nullptr;
    const ME* din = (l == st->nlev - 1) ? dbar : (const ME*)st->D[cur]->ptr;
    {
      ProfScope prof(ctx, kclass<R>(GF_K_BWD_LOCAL, GF_K_BWD_LOCAL64, GF_K_BWD_LOCAL_DF));
      if (top) {
        k_bwd_local<R, true><<<grid, 128, 0, ctx->stream>>>(src_of<R>(st->lev_in[l]), src_of<R>(st->lev_in[l + 1]),
                                                            nullptr, Cst, (ME*)st->Z->ptr, (ME*)st->Dp->ptr,
                                                            ctx->geom, (R)st->rho[l], (R)(0.5 * beta));
      } else {
        k_bwd_local<R, false><<<grid, 128, 0, ctx->stream>>>(src_of<R>(st->lev_in[l]), src_of<R>(st->lev_in[l + 1]),
                                                             din, Cst, (ME*)st->Z->ptr, (ME*)st->Dp->ptr, ctx->geom,
                                                             (R)st->rho[l], (R)(0.5 * beta));
      }
      GF_CHECK_LAUNCH();
    }
    if (dsdrho) dsdrho[l] = level_dsdrho(ctx, st, l);
    int nxt = cur ^ 1;
    ProfScope prof(ctx, kclass<R>(GF_K_BWD_GATHER, GF_K_BWD_GATHER64, GF_K_BWD_GATHER_DF));
    if (l == 0 && P) {
      k_bwd_gather<R, true><<<grid, 128, 0, ctx->stream>>>(src_of<R>(st->lev_in[0]), (const ME*)st->Z->ptr,
                                                           (const ME*)st->Dp->ptr, nullptr, (double*)P->ptr,
                                                           ctx->geom, (R)st->rho[0], -eps / 3.0);
    } else {
      ME* out = (l == 0 && dSdU) ? (ME*)dSdU->ptr : (ME*)st->D[nxt]->ptr;
      k_bwd_gather<R, false><<<grid, 128, 0, ctx->stream>>>(src_of<R>(st->lev_in[l]), (const ME*)st->Z->ptr,
                                                            (const ME*)st->Dp->ptr, out, nullptr, ctx->geom,
                                                            (R)st->rho[l], 0.0);
    }
    GF_CHECK_LAUNCH();
    cur = nxt;
  }
}

void stout_backward(gf_ctx* ctx, gf_stout* st, const gf_field* dSdUbar, double beta, gf_field* dSdU, gf_field* P,
                    double eps, double* dsdrho) {
  if (!st->have_forward) throw gf_error(GF_ESTATE, "stout backward called before forward");
  if (st->fwd_only) throw gf_error(GF_EINVAL, "stout backward: forward-only stack");
  if (st->nlev < 1) throw gf_error(GF_EINVAL, "stout backward needs at least one level");
  int mk = st->precision == GF_MIXED ? GF_MAT32 : GF_MAT64;
  // a dS/dUbar in the stack's own D[1] (written there by the caller) is read in place
  if (dSdUbar && dSdUbar != st->D[1] && dSdUbar->kind != mk) throw gf_error(GF_EINVAL, "stout backward: dS/dUbar kind does not match the stack precision");
  // dSdU == NULL without P: only dS/drho is wanted (the thin-link result stays internal)
  if (!P && dSdU && dSdU->kind != mk) throw gf_error(GF_EINVAL, "stout backward: dS/dU kind does not match the stack precision");
  if (!P && !dSdU && !dsdrho) throw gf_error(GF_EINVAL, "stout backward: no output");
  if (st->precision == GF_FP64) backward_impl<double>(ctx, st, dSdUbar, beta, dSdU, P, eps, dsdrho);
  else if (st->precision == GF_PREC_DF) backward_df(ctx, st, dSdUbar, beta, dSdU, P, eps, dsdrho);
  else backward_impl<float>(ctx, st, dSdUbar, beta, dSdU, P, eps, dsdrho);
}

}  // namespace gf

// Wilson-action kernels: plaquette/action reduction, staples and the fused
// force + momentum update, for fp64 links (fp64 or double-float arithmetic)
// and for fp32 12-real links.
#include "gf_internal.h"
#include "stencil.cuh"

namespace gf {

typedef LinkSrc<double, false> Src64;
typedef LinkSrc<float, true> Src32;
typedef LinkSrc<dfl, false> SrcDF;

// Per-site plaquette sum, one partial per block (calculate_Plaquette,
// src/AbstractGaugefields.jl:2684-2699, evaluated plaquette by plaquette).
template <typename R, class SRC>
__global__ void __launch_bounds__(128, GF_MINB(R)) k_plaquette(SRC U, Geom g, double* __restrict__ part) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  double v = 0.0;
  if (s < g.vol) {
    Site st = site_of(g, s);
    v = (double)plaq_site<R>(U, g, st, s);
  }
  block_partial_sum(v, part);
}

double plaquette_sum(gf_ctx* ctx, const gf_field* U, bool df) {
  int V = ctx->geom.vol;
  int nb = blocks_for(V, 128);
  ProfScope prof(ctx, GF_K_PLAQ);
  if (df && U->kind == GF_LINK64) {
    LinkSrc<dfl, false> src{(const double2*)U->ptr};
    k_plaquette<dfl><<<nb, 128, 0, ctx->stream>>>(src, ctx->geom, ctx->d_partials);
  } else if (U->kind == GF_LINK64 || U->kind == GF_MAT64) {
    Src64 src{(const double2*)U->ptr};
    k_plaquette<double><<<nb, 128, 0, ctx->stream>>>(src, ctx->geom, ctx->d_partials);
  } else if (U->kind == GF_LINK32) {
    Src32 src{(const float4*)U->ptr};
    k_plaquette<float><<<nb, 128, 0, ctx->stream>>>(src, ctx->geom, ctx->d_partials);
  } else if (U->kind == GF_LINKDF) {
    // top level of a double-float stack: fp64 arithmetic on hi + lo
    LinkSrcDfn64 src{(const float4*)U->ptr};
    k_plaquette<double><<<nb, 128, 0, ctx->stream>>>(src, ctx->geom, ctx->d_partials);
  } else {
    throw gf_error(GF_EINVAL, "plaquette: links must be LINK64 or LINK32");
  }
  GF_CHECK_LAUNCH();
  return finish_reduction(ctx, nb);
}

// Polyakov loop (calculate_Polyakov_loop, src/AbstractGaugefields.jl:
// 2929-2956): for each site x of the t = 0 slice, Re or Im (comp 0 / 1) of
// tr(U_T(x, 0) U_T(x, 1) ... U_T(x, NT - 1)), one partial per block. One
// thread per spatial site, the product along T in fp64.
__global__ void __launch_bounds__(128) k_polyakov(Src64 U, Geom g, int comp, double* __restrict__ part) {
  const int vs = g.stride[3];  // NX NY NZ
  const int sp = blockIdx.x * blockDim.x + threadIdx.x;
  double v = 0.0;
  if (sp < vs) {
    const int x = sp % g.L[0], r = sp / g.L[0];
    const int par0 = (x + r % g.L[1] + r / g.L[1]) & 1;
    mat3<double> p = U(3, eo_of_lex(g, sp, par0), g.vol);
#pragma unroll 1
    for (int t = 1; t < g.L[3]; ++t) p = mul_nn(p, U(3, eo_of_lex(g, sp + t * vs, par0 ^ (t & 1)), g.vol));
    const cplx<double> tr = trace(p);
    v = comp ? tr.im : tr.re;
  }
  block_partial_sum(v, part);
}

void polyakov_loop(gf_ctx* ctx, const gf_field* U, double out[2]) {
  if (U->kind != GF_LINK64) throw gf_error(GF_EINVAL, "Polyakov loop: links must be LINK64");
  const int vs = ctx->geom.stride[3];
  const int nb = blocks_for(vs, 128);
  ProfScope prof(ctx, GF_K_PLAQ);
  for (int c = 0; c < 2; ++c) {
    k_polyakov<<<nb, 128, 0, ctx->stream>>>(Src64{(const double2*)U->ptr}, ctx->geom, c, ctx->d_partials);
    GF_CHECK_LAUNCH();
    out[c] = finish_reduction(ctx, nb) / vs;
  }
}

// construct_staple!: V_mu = sum_{nu != mu} U_nu(x) U_mu(x+nu) U_nu(x+mu)^dag = S_mu^dag
__global__ void __launch_bounds__(128) k_staple_up(Src64 U, Geom g, int mu, double2* __restrict__ out) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= g.vol) return;
  Site st = site_of(g, s);
  // up staples only (construct_staple! has no down staples)
  mat3<double> acc = zero3<double>();
  const int V = g.vol;
#pragma unroll
  for (int nu = 0; nu < 4; ++nu) {
    if (nu == mu) continue;
    // x+nu and x+mu with a runtime axis (this kernel is off the hot path)
    int lex = st.lex;
    int cnu = st.x[nu] + 1 == g.L[nu] ? -(g.L[nu] - 1) : 1;
    int cmu = st.x[mu] + 1 == g.L[mu] ? -(g.L[mu] - 1) : 1;
    int xpn = eo_of_lex(g, lex + cnu * g.stride[nu], st.par ^ 1);
    int xpm = eo_of_lex(g, lex + cmu * g.stride[mu], st.par ^ 1);
    mat3<double> t = mul_nn(U(nu, s, V), U(mu, xpn, V));
    mac_na(acc, t, U(nu, xpm, V));
  }
  LinkFull<double>::store(out, mu, s, V, acc);
}

void staple_up(gf_ctx* ctx, const gf_field* U, int mu, gf_field* Vout) {
  if (U->kind != GF_LINK64 && U->kind != GF_MAT64) throw gf_error(GF_EINVAL, "staple: U must be LINK64");
  if (Vout->kind != GF_MAT64 && Vout->kind != GF_LINK64) throw gf_error(GF_EINVAL, "staple: V must be MAT64");
  if (mu < 0 || mu > 3) throw gf_error(GF_EINVAL, "staple: mu out of range");
  Src64 src{(const double2*)U->ptr};
  k_staple_up<<<blocks_for(ctx->geom.vol, 128), 128, 0, ctx->stream>>>(src, ctx->geom, mu, (double2*)Vout->ptr);
  GF_CHECK_LAUNCH();
}

// P_mu(x) <- keep * P_mu(x) + coef * c(U_mu(x) S_mu(x)), c = su(3) coefficients
// of TA (keep = 0 overwrites without reading P).
//  * md_force!:        coef = -(1/3) * beta/2, keep = 0
//  * update_momenta!:  coef = eps * (-(1/3) * beta/2), keep = 1
//  * add_force! flow:  coef = factor
template <typename R, class SRC>
__global__ void __launch_bounds__(128, GF_MINB(R)) k_force_ta(SRC U, double* __restrict__ P, Geom g, double coef, double keep) {
  int s, mu;
  link_of_thread(s, mu);
  if (s >= g.vol) return;
  Site st = site_of(g, s);
  const int V = g.vol;
  mat3<R> S = staple_sum<R>(mu, U, g, st, s);
  mat3<R> M = mul_nn(U(mu, s, V), S);
  R c[8];
  ta_coeffs(M, c);
  double* p = P + (size_t)mu * 8 * V + s;
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    double old = (keep != 0.0) ? keep * p[(size_t)a * V] : 0.0;
    p[(size_t)a * V] = old + coef * to_f64(c[a]);
  }
}

void wilson_force_coef(gf_ctx* ctx, const gf_field* U, gf_field* P, double coef, double keep, bool df) {
  if (P->kind != GF_MOM64) throw gf_error(GF_EINVAL, "force: output must be MOM64");
  dim3 grid = stencil_grid(ctx->geom.vol, 128);
  ProfScope prof(ctx, df ? GF_K_FORCE_DF : GF_K_FORCE);
  if (df && U->kind == GF_LINK64) {
    SrcDF src{(const double2*)U->ptr};
    k_force_ta<dfl><<<grid, 128, 0, ctx->stream>>>(src, (double*)P->ptr, ctx->geom, coef, keep);
  } else if (df) {
    throw gf_error(GF_EINVAL, "force: the double-float force needs LINK64 links");
  } else if (U->kind == GF_LINK64) {
    Src64 src{(const double2*)U->ptr};
    k_force_ta<double><<<grid, 128, 0, ctx->stream>>>(src, (double*)P->ptr, ctx->geom, coef, keep);
  } else if (U->kind == GF_LINK32) {
    Src32 src{(const float4*)U->ptr};
    k_force_ta<float><<<grid, 128, 0, ctx->stream>>>(src, (double*)P->ptr, ctx->geom, coef, keep);
  } else {
    throw gf_error(GF_EINVAL, "force: links must be LINK64 or LINK32");
  }
  GF_CHECK_LAUNCH();
}

// add_force!(F, U; plaqonly=true): F += factor * TA(U_mu V_mu^dag), V^dag = S
// the flow's force; double-float: the plaquette-staple table kernel of
// gf_rect.cu (fixed-grid products, 2.4x the inlined double-float force)
void flow_force(gf_ctx* ctx, const gf_field* U, gf_field* F, double factor, double keep, bool df) {
  if (df) plaquette_force_df(ctx, U, F, factor, keep);
  else wilson_force_coef(ctx, U, F, factor, keep);
}

}  // namespace gf

// Rectangle (2x1) loops of the gauge action, fp64 links in fp64 arithmetic:
// the loop sum, and the force (+ momentum update) of an action with
// plaquette and rectangle terms, push!(action, c_plaq, plaq U plaq') and
// push!(action, c_rect, rect U rect') (src/action/GaugeActions.jl:48-142; the
// loops of make_rect, src/autostaples/wilsonloops.jl:304-330).
//
// For a link U_mu(x) and each nu != mu, the six rectangles that contain it,
// as the rest of each loop after U_mu(x) (the staple of its forward
// occurrence):
//   (a) 1x2 up      U_nu(x+mu) U_nu(x+mu+nu) U_mu(x+2nu)^+ U_nu(x+nu)^+ U_nu(x)^+
//   (b) 1x2 down    U_nu(x+mu-nu)^+ U_nu(x+mu-2nu)^+ U_mu(x-2nu)^+ U_nu(x-2nu) U_nu(x-nu)
//   (c) 2x1 first   U_mu(x+mu) U_nu(x+2mu) U_mu(x+mu+nu)^+ U_mu(x+nu)^+ U_nu(x)^+
//   (d) 2x1 first   U_mu(x+mu) U_nu(x+2mu-nu)^+ U_mu(x+mu-nu)^+ U_mu(x-nu)^+ U_nu(x-nu)
//   (e) 2x1 second  U_nu(x+mu) U_mu(x+nu)^+ U_mu(x-mu+nu)^+ U_nu(x-mu)^+ U_mu(x-mu)
//   (f) 2x1 second  U_nu(x+mu-nu)^+ U_mu(x-nu)^+ U_mu(x-mu-nu)^+ U_nu(x-mu-nu) U_mu(x-mu)
// Each geometric rectangle holding the link appears once, as the six
// plaquette-staple terms do for the plaquettes, so dS/dU_mu = c_plaq S_plaq +
// c_rect S_rect and F = -(1/3) TA(U_mu dS/dU_mu), as for the Wilson action.
#include "gf_internal.h"
#include "stencil.cuh"

namespace gf {

typedef LinkSrc<double, false> SrcRect;

// even/odd index of x + a e_mu + b e_nu (mu != nu, any a, b; periodic)
__device__ __forceinline__ int site_off(const Geom& g, const Site& st, int mu, int a, int nu, int b) {
  int lex = st.lex;
  int c = coord(st, mu);
  int n = (c + a) % g.L[mu];
  if (n < 0) n += g.L[mu];
  lex += (n - c) * g.stride[mu];
  c = coord(st, nu);
  n = (c + b) % g.L[nu];
  if (n < 0) n += g.L[nu];
  lex += (n - c) * g.stride[nu];
  return eo_of_lex(g, lex, st.par ^ ((a + b) & 1));
}

// Sum over mu < nu of Re tr (R^{1x2}_{mu nu}(x) + R^{2x1}_{mu nu}(x)) at one
// site, each rectangle as Re tr(A B^+) of its two three-link halves.
__device__ double rect_site(const SrcRect& U, const Geom& g, const Site& st, int s) {
  const int V = g.vol;
  double v = 0.0;
#pragma unroll 1
  for (int p = 0; p < 6; ++p) {
    const int mu = p < 3 ? 0 : (p < 5 ? 1 : 2);
    const int nu = p < 3 ? p + 1 : (p < 5 ? p - 1 : 3);
    // 1x2: A = U_mu(x) U_nu(x+mu) U_nu(x+mu+nu), B = U_nu(x) U_nu(x+nu) U_mu(x+2nu)
    mat3<double> a = mul_nn(U(mu, s, V), U(nu, site_off(g, st, mu, 1, nu, 0), V));
    a = mul_nn(a, U(nu, site_off(g, st, mu, 1, nu, 1), V));
    mat3<double> b = mul_nn(U(nu, s, V), U(nu, site_off(g, st, mu, 0, nu, 1), V));
    b = mul_nn(b, U(mu, site_off(g, st, mu, 0, nu, 2), V));
    v += retr_na(a, b);
    // 2x1: A = U_mu(x) U_mu(x+mu) U_nu(x+2mu), B = U_nu(x) U_mu(x+nu) U_mu(x+mu+nu)
    a = mul_nn(U(mu, s, V), U(mu, site_off(g, st, mu, 1, nu, 0), V));
    a = mul_nn(a, U(nu, site_off(g, st, mu, 2, nu, 0), V));
    b = mul_nn(U(nu, s, V), U(mu, site_off(g, st, mu, 0, nu, 1), V));
    b = mul_nn(b, U(mu, site_off(g, st, mu, 1, nu, 1), V));
    v += retr_na(a, b);
  }
  return v;
}

__global__ void __launch_bounds__(128) k_rect_sum(SrcRect U, Geom g, double* __restrict__ part) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  double v = 0.0;
  if (s < g.vol) {
    Site st = site_of(g, s);
    v = rect_site(U, g, st, s);
  }
  block_partial_sum(v, part);
}

// acc += the six rectangle staples (a)-(f) of U_mu(x) in the mu-nu plane
__device__ __forceinline__ void add_rect_staples(mat3<double>& acc, const SrcRect& U, const Geom& g, const Site& st,
                                                 int s, int mu, int nu) {
  const int V = g.vol;
  mat3<double> t;
  // (a)
  t = mul_nn(U(nu, site_off(g, st, mu, 1, nu, 0), V), U(nu, site_off(g, st, mu, 1, nu, 1), V));
  t = mul_na(t, U(mu, site_off(g, st, mu, 0, nu, 2), V));
  t = mul_na(t, U(nu, site_off(g, st, mu, 0, nu, 1), V));
  mac_na(acc, t, U(nu, s, V));
  // (b)
  t = mul_aa(U(nu, site_off(g, st, mu, 1, nu, -1), V), U(nu, site_off(g, st, mu, 1, nu, -2), V));
  t = mul_na(t, U(mu, site_off(g, st, mu, 0, nu, -2), V));
  t = mul_nn(t, U(nu, site_off(g, st, mu, 0, nu, -2), V));
  mac_nn(acc, t, U(nu, site_off(g, st, mu, 0, nu, -1), V));
  // (c)
  t = mul_nn(U(mu, site_off(g, st, mu, 1, nu, 0), V), U(nu, site_off(g, st, mu, 2, nu, 0), V));
  t = mul_na(t, U(mu, site_off(g, st, mu, 1, nu, 1), V));
  t = mul_na(t, U(mu, site_off(g, st, mu, 0, nu, 1), V));
  mac_na(acc, t, U(nu, s, V));
  // (d)
  t = mul_na(U(mu, site_off(g, st, mu, 1, nu, 0), V), U(nu, site_off(g, st, mu, 2, nu, -1), V));
  t = mul_na(t, U(mu, site_off(g, st, mu, 1, nu, -1), V));
  t = mul_na(t, U(mu, site_off(g, st, mu, 0, nu, -1), V));
  mac_nn(acc, t, U(nu, site_off(g, st, mu, 0, nu, -1), V));
  // (e)
  t = mul_na(U(nu, site_off(g, st, mu, 1, nu, 0), V), U(mu, site_off(g, st, mu, 0, nu, 1), V));
  t = mul_na(t, U(mu, site_off(g, st, mu, -1, nu, 1), V));
  t = mul_na(t, U(nu, site_off(g, st, mu, -1, nu, 0), V));
  mac_nn(acc, t, U(mu, site_off(g, st, mu, -1, nu, 0), V));
  // (f)
  t = mul_aa(U(nu, site_off(g, st, mu, 1, nu, -1), V), U(mu, site_off(g, st, mu, 0, nu, -1), V));
  t = mul_na(t, U(mu, site_off(g, st, mu, -1, nu, -1), V));
  t = mul_nn(t, U(nu, site_off(g, st, mu, -1, nu, -1), V));
  mac_nn(acc, t, U(mu, site_off(g, st, mu, -1, nu, 0), V));
}

// P_mu(x) <- keep * P_mu(x) + c(U_mu(x) (cp S_mu(x) + cr R_mu(x))), c = su(3)
// coefficients of TA; S the six plaquette staples, R the eighteen rectangle
// staples (keep = 0 overwrites without reading P).
__global__ void __launch_bounds__(128) k_force_rect(SrcRect U, double* __restrict__ P, Geom g, double cp, double cr,
                                                    double keep) {
  int s, mu;
  link_of_thread(s, mu);
  if (s >= g.vol) return;
  Site st = site_of(g, s);
  const int V = g.vol;
  mat3<double> S = zero3<double>();
  mat3<double> R = zero3<double>();
#pragma unroll 1
  for (int k = 1; k < 4; ++k) {
    const int nu = (mu + k) & 3;
    add_staple_pair<double>(S, U, g, st, s, mu, nu);
    add_rect_staples(R, U, g, st, s, mu, nu);
  }
  mat3<double> T = scale(cp, S);
  axpy_to(T, cr, R);
  mat3<double> M = mul_nn(U(mu, s, V), T);
  double c[8];
  ta_coeffs(M, c);
  double* p = P + (size_t)mu * 8 * V + s;
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    double old = (keep != 0.0) ? keep * p[(size_t)a * V] : 0.0;
    p[(size_t)a * V] = old + c[a];
  }
}

double rectangle_sum(gf_ctx* ctx, const gf_field* U) {
  if (U->kind != GF_LINK64 && U->kind != GF_MAT64) throw gf_error(GF_EINVAL, "rectangle: links must be LINK64");
  const int V = ctx->geom.vol;
  const int nb = blocks_for(V, 128);
  ProfScope prof(ctx, GF_K_RECT);
  SrcRect src{(const double2*)U->ptr};
  k_rect_sum<<<nb, 128, 0, ctx->stream>>>(src, ctx->geom, ctx->d_partials);
  GF_CHECK_LAUNCH();
  return finish_reduction(ctx, nb);
}

void loops_force_coef(gf_ctx* ctx, const gf_field* U, gf_field* P, double cp, double cr, double keep) {
  if (P->kind != GF_MOM64) throw gf_error(GF_EINVAL, "force: output must be MOM64");
  if (U->kind != GF_LINK64 && U->kind != GF_MAT64)
    throw gf_error(GF_EINVAL, "force: the rectangle force takes LINK64 links");
  dim3 grid = stencil_grid(ctx->geom.vol, 128);
  ProfScope prof(ctx, GF_K_RECT);
  SrcRect src{(const double2*)U->ptr};
  k_force_rect<<<grid, 128, 0, ctx->stream>>>(src, (double*)P->ptr, ctx->geom, cp, cr, keep);
  GF_CHECK_LAUNCH();
}

}  // namespace gf

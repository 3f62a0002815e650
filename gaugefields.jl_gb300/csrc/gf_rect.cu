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
#include "dfslots.cuh"

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
template <class SRC>
__device__ double rect_site(const SRC& U, const Geom& g, const Site& st, int s) {
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

template <class SRC>
__global__ void __launch_bounds__(128) k_rect_sum(SRC U, Geom g, double* __restrict__ part) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  double v = 0.0;
  if (s < g.vol) {
    Site st = site_of(g, s);
    v = rect_site(U, g, st, s);
  }
  block_partial_sum(v, part);
}

// acc += the six rectangle staples (a)-(f) of U_mu(x) in the mu-nu plane
template <typename R, class SRC>
__device__ __forceinline__ void add_rect_staples(mat3<R>& acc, const SRC& U, const Geom& g, const Site& st, int s,
                                                 int mu, int nu) {
  const int V = g.vol;
  mat3<R> t;
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

// cp S_mu(x) + cr R_mu(x): S the six plaquette staples, R the eighteen
// rectangle staples of U_mu(x)
template <typename R, class SRC>
__device__ __forceinline__ mat3<R> loops_dsdu(const SRC& U, const Geom& g, const Site& st, int s, int mu, R cp,
                                              R cr) {
  mat3<R> S = zero3<R>();
  mat3<R> Q = zero3<R>();
#pragma unroll 1
  for (int k = 1; k < 4; ++k) {
    const int nu = (mu + k) & 3;
    add_staple_pair<R>(S, U, g, st, s, mu, nu);
    add_rect_staples<R>(Q, U, g, st, s, mu, nu);
  }
  mat3<R> T = scale(cp, S);
  axpy_to(T, cr, Q);
  return T;
}

// P_mu(x) <- keep * P_mu(x) + c(U_mu(x) (cp S_mu(x) + cr R_mu(x))), c = su(3)
// coefficients of TA (keep = 0 overwrites without reading P); arithmetic in
// R (fp64 on the plain form's links, fp32 on the mixed form's 12-real links)
template <typename R, class SRC>
__global__ void __launch_bounds__(128) k_force_rect(SRC U, double* __restrict__ P, Geom g, R cp, R cr, double keep) {
  int s, mu;
  link_of_thread(s, mu);
  if (s >= g.vol) return;
  Site st = site_of(g, s);
  const int V = g.vol;
  const mat3<R> T = loops_dsdu<R>(U, g, st, s, mu, cp, cr);
  mat3<R> M = mul_nn(U(mu, s, V), T);
  R c[8];
  ta_coeffs(M, c);
  double* p = P + (size_t)mu * 8 * V + s;
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    double old = (keep != 0.0) ? keep * p[(size_t)a * V] : 0.0;
    p[(size_t)a * V] = old + to_f64(c[a]);
  }
}

// D_mu(x) = cp S_mu(x) + cr R_mu(x): dS/dUbar of the plaquette + rectangle
// action on the top level of a stout stack (the input of its adjoint)
template <typename R, class SRC>
__global__ void __launch_bounds__(128) k_dsdu_rect(SRC U, typename LinkFull<R>::elem* __restrict__ D, Geom g, R cp,
                                                   R cr) {
  int s, mu;
  link_of_thread(s, mu);
  if (s >= g.vol) return;
  Site st = site_of(g, s);
  LinkFull<R>::store(D, mu, s, g.vol, loops_dsdu<R>(U, g, st, s, mu, cp, cr));
}

// --------------------------------------------------------------------------
// The same force in double-float arithmetic (the GF_DFLOAT form: the force
// on thin links, or dS/dUbar on a stack's top level), as a loop over a table
// of products with one inlined fixed-grid
// product (the double-float stencils overflow the instruction cache when
// their products are inlined). Per plane (mu, nu): ops 0-3 add the two
// plaquette staples to S (add_staple_pair), ops 4-27 the six rectangle
// staples (a)-(f) above to R, four products each. An operand is the link of
// direction mu or nu at x + mo e_mu + no e_nu (optionally daggered) or the
// running product t; results go to t, S or R.
// --------------------------------------------------------------------------
struct DfOpR {
  // src 0: link (dir 0 = mu, 1 = nu; offsets mo, no), src 1: slot t
  signed char a_src, a_dir, a_mo, a_no, a_dag, b_src, b_dir, b_mo, b_no, b_dag, out, accumulate;
};
#define GF_RECT_T 0
#define GF_RECT_S 1
#define GF_RECT_R 2
#define GF_RECT_SLOTS 3
__constant__ DfOpR c_rect_ops[28] = {
    // plaquette staples: U_nu(x+mu) U_mu(x+nu)^+ U_nu(x)^+ and U_nu(x+mu-nu)^+ U_mu(x-nu)^+ U_nu(x-nu)
    {0, 1, 1, 0, 0, 0, 0, 0, 1, 1, 0, 0}, {1, 0, 0, 0, 0, 0, 1, 0, 0, 1, 1, 1},
    {0, 1, 1, -1, 1, 0, 0, 0, -1, 1, 0, 0}, {1, 0, 0, 0, 0, 0, 1, 0, -1, 0, 1, 1},
    // (a) U_nu(x+mu) U_nu(x+mu+nu) U_mu(x+2nu)^+ U_nu(x+nu)^+ U_nu(x)^+
    {0, 1, 1, 0, 0, 0, 1, 1, 1, 0, 0, 0}, {1, 0, 0, 0, 0, 0, 0, 0, 2, 1, 0, 0},
    {1, 0, 0, 0, 0, 0, 1, 0, 1, 1, 0, 0}, {1, 0, 0, 0, 0, 0, 1, 0, 0, 1, 2, 1},
    // (b) U_nu(x+mu-nu)^+ U_nu(x+mu-2nu)^+ U_mu(x-2nu)^+ U_nu(x-2nu) U_nu(x-nu)
    {0, 1, 1, -1, 1, 0, 1, 1, -2, 1, 0, 0}, {1, 0, 0, 0, 0, 0, 0, 0, -2, 1, 0, 0},
    {1, 0, 0, 0, 0, 0, 1, 0, -2, 0, 0, 0}, {1, 0, 0, 0, 0, 0, 1, 0, -1, 0, 2, 1},
    // (c) U_mu(x+mu) U_nu(x+2mu) U_mu(x+mu+nu)^+ U_mu(x+nu)^+ U_nu(x)^+
    {0, 0, 1, 0, 0, 0, 1, 2, 0, 0, 0, 0}, {1, 0, 0, 0, 0, 0, 0, 1, 1, 1, 0, 0},
    {1, 0, 0, 0, 0, 0, 0, 0, 1, 1, 0, 0}, {1, 0, 0, 0, 0, 0, 1, 0, 0, 1, 2, 1},
    // (d) U_mu(x+mu) U_nu(x+2mu-nu)^+ U_mu(x+mu-nu)^+ U_mu(x-nu)^+ U_nu(x-nu)
    {0, 0, 1, 0, 0, 0, 1, 2, -1, 1, 0, 0}, {1, 0, 0, 0, 0, 0, 0, 1, -1, 1, 0, 0},
    {1, 0, 0, 0, 0, 0, 0, 0, -1, 1, 0, 0}, {1, 0, 0, 0, 0, 0, 1, 0, -1, 0, 2, 1},
    // (e) U_nu(x+mu) U_mu(x+nu)^+ U_mu(x-mu+nu)^+ U_nu(x-mu)^+ U_mu(x-mu)
    {0, 1, 1, 0, 0, 0, 0, 0, 1, 1, 0, 0}, {1, 0, 0, 0, 0, 0, 0, -1, 1, 1, 0, 0},
    {1, 0, 0, 0, 0, 0, 1, -1, 0, 1, 0, 0}, {1, 0, 0, 0, 0, 0, 0, -1, 0, 0, 2, 1},
    // (f) U_nu(x+mu-nu)^+ U_mu(x-nu)^+ U_mu(x-mu-nu)^+ U_nu(x-mu-nu) U_mu(x-mu)
    {0, 1, 1, -1, 1, 0, 0, 0, -1, 1, 0, 0}, {1, 0, 0, 0, 0, 0, 0, -1, -1, 1, 0, 0},
    {1, 0, 0, 0, 0, 0, 1, -1, -1, 0, 0, 0}, {1, 0, 0, 0, 0, 0, 0, -1, 0, 0, 2, 1},
};

__device__ __forceinline__ mat3<dfl> rect_operand(int src, int dir, int mo, int no, int dagger, const float* sm, int tid,
                                                  const float4* __restrict__ U, const Geom& g, const Site& st, int mu,
                                                  int nu) {
  mat3<dfl> m;
  if (src == 1) m = slot_load(sm, GF_RECT_T, tid);
  else m = LinkDfn::load(U, dir ? nu : mu, site_off(g, st, mu, mo, nu, no), g.vol);
  if (dagger) m = dag(m);
  return m;
}

// P_mu(x) <- keep * P_mu(x) + c(U_mu(x) (cp S_mu(x) + cr R_mu(x))) as
// k_force_rect, the staples, the combination and the projection in
// double-float, on double-float-native links; DSDU: D_mu(x) = cp S + cr R
// (as k_dsdu_rect, double-float-native) instead. NOPS = 4 runs only the
// plaquette staples (the Wilson force; R stays zero).
template <bool DSDU, int NOPS>
__global__ void __launch_bounds__(128, 3)
    k_force_rect_df(const float4* __restrict__ U, double* __restrict__ P, float4* __restrict__ D, Geom g, dfl cp,
                    dfl cr, double keep) {
  extern __shared__ __align__(16) float sm[];  // GF_RECT_SLOTS slots of 36 x 128 floats
  const int tid = threadIdx.x;
  int s, mu;
  link_of_thread(s, mu);
  if (s >= g.vol) return;  // the slots are per thread: no block-wide synchronisation
  const Site st = site_of(g, s);
  slot_store(sm, GF_RECT_S, tid, zero3<dfl>());
  slot_store(sm, GF_RECT_R, tid, zero3<dfl>());
#pragma unroll 1
  for (int k = 1; k < 4; ++k) {
    const int nu = (mu + k) & 3;
#pragma unroll 1
    for (int q = 0; q < NOPS; ++q) {
      const DfOpR op = c_rect_ops[q];
      const mat3<dfl> A = rect_operand(op.a_src, op.a_dir, op.a_mo, op.a_no, op.a_dag, sm, tid, U, g, st, mu, nu);
      const mat3<dfl> B = rect_operand(op.b_src, op.b_dir, op.b_mo, op.b_no, op.b_dag, sm, tid, U, g, st, mu, nu);
      const mat3<dfl> C = op.accumulate ? slot_load(sm, op.out, tid) : zero3<dfl>();
      slot_store(sm, op.out, tid, dfg_matmul<false, false, true>(A, B, &C));
    }
  }
  const mat3<dfl> S = slot_load(sm, GF_RECT_S, tid), R = slot_load(sm, GF_RECT_R, tid);
  mat3<dfl> T;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      dfg_cacc a = dfg_cbegin(fabsf(cp.hi) * cabs1(S.e[i][j]) + fabsf(cr.hi) * cabs1(R.e[i][j]));
      dfg_rcterm(a, cp, S.e[i][j]);
      dfg_rcterm(a, cr, R.e[i][j]);
      T.e[i][j] = dfg_cend(a);
    }
  if (DSDU) {
    LinkDfn::store(D, mu, s, g.vol, T);
    return;
  }
  const mat3<dfl> M = dfg_matmul<false, false, false>(LinkDfn::load(U, mu, s, g.vol), T, nullptr);
  dfl c[8];
  ta_coeffs(M, c);
  double* p = P + (size_t)mu * 8 * g.vol + s;
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const double old = (keep != 0.0) ? keep * p[(size_t)a * g.vol] : 0.0;
    p[(size_t)a * g.vol] = old + to_f64(c[a]);
  }
}

static void rect_df(gf_ctx* ctx, const float4* U, gf_field* P, gf_field* D, double cp, double cr, double keep,
                    bool plaquette_only = false) {
  const size_t smem = (size_t)GF_RECT_SLOTS * 36 * 128 * sizeof(float);
  auto kern = plaquette_only ? k_force_rect_df<false, 4> : (D ? k_force_rect_df<true, 28> : k_force_rect_df<false, 28>);
  GF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid = stencil_grid(ctx->geom.vol, 128);
  ProfScope prof(ctx, GF_K_RECT_DF);
  kern<<<grid, 128, smem, ctx->stream>>>(U, P ? (double*)P->ptr : nullptr, D ? (float4*)D->ptr : nullptr, ctx->geom,
                                         dfl(cp), dfl(cr), keep);
  GF_CHECK_LAUNCH();
}

template <class SRC>
static double rect_sum_of(gf_ctx* ctx, SRC src) {
  const int nb = blocks_for(ctx->geom.vol, 128);
  ProfScope prof(ctx, GF_K_RECT);
  k_rect_sum<<<nb, 128, 0, ctx->stream>>>(src, ctx->geom, ctx->d_partials);
  GF_CHECK_LAUNCH();
  return finish_reduction(ctx, nb);
}

double rectangle_sum(gf_ctx* ctx, const gf_field* U) {
  if (U->kind == GF_LINK64 || U->kind == GF_MAT64) return rect_sum_of(ctx, SrcRect{(const double2*)U->ptr});
  // top level of a double-float stack: fp64 arithmetic on hi + lo
  if (U->kind == GF_LINKDF) return rect_sum_of(ctx, LinkSrcDfn64{(const float4*)U->ptr});
  throw gf_error(GF_EINVAL, "rectangle: links must be LINK64");
}

void loops_force_coef(gf_ctx* ctx, const gf_field* U, gf_field* P, double cp, double cr, double keep, bool df) {
  if (P->kind != GF_MOM64) throw gf_error(GF_EINVAL, "force: output must be MOM64");
  dim3 grid = stencil_grid(ctx->geom.vol, 128);
  if (df) {
    if (U->kind != GF_LINK64) throw gf_error(GF_EINVAL, "force: the double-float rectangle force takes LINK64 links");
    // a double-float-native copy of the links, converted once per force
    if (!ctx->w_linkdf) ctx->w_linkdf = field_new(ctx, GF_LINKDF);
    copy_field(ctx, ctx->w_linkdf, U);
    rect_df(ctx, (const float4*)ctx->w_linkdf->ptr, P, nullptr, cp, cr, keep);
    return;
  }
  if (U->kind == GF_LINK64 || U->kind == GF_MAT64) {
    ProfScope prof(ctx, GF_K_RECT);
    k_force_rect<double><<<grid, 128, 0, ctx->stream>>>(SrcRect{(const double2*)U->ptr}, (double*)P->ptr, ctx->geom,
                                                        cp, cr, keep);
  } else if (U->kind == GF_LINK32) {
    ProfScope prof(ctx, GF_K_RECT);
    k_force_rect<float><<<grid, 128, 0, ctx->stream>>>(LinkSrc<float, true>{(const float4*)U->ptr}, (double*)P->ptr,
                                                       ctx->geom, (float)cp, (float)cr, keep);
  } else {
    throw gf_error(GF_EINVAL, "force: the rectangle force takes LINK64 or LINK32 links");
  }
  GF_CHECK_LAUNCH();
}

void plaquette_force_df(gf_ctx* ctx, const gf_field* U, gf_field* P, double coef, double keep) {
  if (P->kind != GF_MOM64) throw gf_error(GF_EINVAL, "force: output must be MOM64");
  if (U->kind != GF_LINK64) throw gf_error(GF_EINVAL, "force: the double-float force takes LINK64 links");
  if (!ctx->w_linkdf) ctx->w_linkdf = field_new(ctx, GF_LINKDF);
  copy_field(ctx, ctx->w_linkdf, U);
  rect_df(ctx, (const float4*)ctx->w_linkdf->ptr, P, nullptr, coef, 0.0, keep, true);
}

void loops_dsdu(gf_ctx* ctx, const gf_field* Ubar, gf_field* D, double cp, double cr) {
  dim3 grid = stencil_grid(ctx->geom.vol, 128);
  if (Ubar->kind == GF_LINKDF && D->kind == GF_MATDF) {
    rect_df(ctx, (const float4*)Ubar->ptr, nullptr, D, cp, cr, 0.0);
    return;
  }
  ProfScope prof(ctx, GF_K_RECT);
  if (Ubar->kind == GF_LINK64 && D->kind == GF_MAT64) {
    k_dsdu_rect<double><<<grid, 128, 0, ctx->stream>>>(SrcRect{(const double2*)Ubar->ptr}, (double2*)D->ptr,
                                                       ctx->geom, cp, cr);
  } else if (Ubar->kind == GF_LINK32 && D->kind == GF_MAT32) {
    k_dsdu_rect<float><<<grid, 128, 0, ctx->stream>>>(LinkSrc<float, true>{(const float4*)Ubar->ptr},
                                                      (float2*)D->ptr, ctx->geom, (float)cp, (float)cr);
  } else {
    throw gf_error(GF_EINVAL, "loops dS/dU: link and matrix kinds do not match");
  }
  GF_CHECK_LAUNCH();
}

}  // namespace gf

// Link update U <- exp(i eps P) U (update_gaugefields!,
// src/molecular_dynamics.jl:513-531; exptU!, src/4D/TA_gaugefields_4D_serial.jl:760)
// with the Cayley-Hamilton exponential, optional re-unitarisation
// (normalize3!, src/AbstractGaugefields.jl:3378) and an optional fp32
// 12-real shadow copy for the mixed-precision force path. All in fp64.
#include "gf_internal.h"

namespace gf {

__global__ void __launch_bounds__(128) k_link_update(const double2* Uin, double2* Uout,
                                                     const double* __restrict__ P, Geom g, double eps, int reunit,
                                                     float4* __restrict__ sh32) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  int mu = blockIdx.y;
  if (s >= g.vol) return;
  const int V = g.vol;
  double p[8];
#pragma unroll
  for (int a = 0; a < 8; ++a) p[a] = eps * P[((size_t)mu * 8 + a) * V + s];
  mat3<double> q = herm_from_coeffs(p);
  mat3<double> e = expiq(q);
  mat3<double> u = LinkFull<double>::load(Uin, mu, s, V);
  mat3<double> w = mul_nn(e, u);
  if (reunit) reunitarize(w);
  LinkFull<double>::store(Uout, mu, s, V, w);
  if (sh32) {
    mat3<float> f;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) f.e[i][j] = mk((float)w.e[i][j].re, (float)w.e[i][j].im);
    Link12f::store(sh32, mu, s, V, f);
  }
}

void link_update(gf_ctx* ctx, gf_field* U, const gf_field* P, double eps, int reunit, gf_field* shadow32) {
  if (U->kind != GF_LINK64) throw gf_error(GF_EINVAL, "link update: U must be LINK64");
  if (P->kind != GF_MOM64) throw gf_error(GF_EINVAL, "link update: P must be MOM64");
  dim3 grid(blocks_for(ctx->geom.vol, 128), 4);
  ProfScope prof(ctx, GF_K_LINK_UPDATE);
  k_link_update<<<grid, 128, 0, ctx->stream>>>((const double2*)U->ptr, (double2*)U->ptr, (const double*)P->ptr,
                                                 ctx->geom, eps, reunit,
                                                 shadow32 ? (float4*)shadow32->ptr : nullptr);
  GF_CHECK_LAUNCH();
}

// exp_aF_U!(W, a, F, U) (src/AbstractGaugefields.jl:2810-2842): W_mu = exp(a F_mu) U_mu
// with F in su(3) coefficients, i.e. exp(i a sum_a F_a lambda_a / 2) U.
void exp_mom_links(gf_ctx* ctx, gf_field* W, const gf_field* P, double a, const gf_field* U) {
  dim3 grid(blocks_for(ctx->geom.vol, 128), 4);
  ProfScope prof(ctx, GF_K_LINK_UPDATE);
  k_link_update<<<grid, 128, 0, ctx->stream>>>((const double2*)U->ptr, (double2*)W->ptr, (const double*)P->ptr,
                                                 ctx->geom, a, 0, nullptr);
  GF_CHECK_LAUNCH();
}

__global__ void k_reunit(double2* __restrict__ U, int V) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  int mu = blockIdx.y;
  if (s >= V) return;
  mat3<double> u = LinkFull<double>::load(U, mu, s, V);
  reunitarize(u);
  LinkFull<double>::store(U, mu, s, V, u);
}

void reunitarize_links(gf_ctx* ctx, gf_field* U) {
  if (U->kind != GF_LINK64) throw gf_error(GF_EINVAL, "reunitarize: U must be LINK64");
  dim3 grid(blocks_for(ctx->geom.vol, 128), 4);
  k_reunit<<<grid, 128, 0, ctx->stream>>>((double2*)U->ptr, ctx->geom.vol);
  GF_CHECK_LAUNCH();
}

}  // namespace gf

// Link update U <- exp(i eps P) U (update_gaugefields!,
// src/molecular_dynamics.jl:513-531; exptU!, src/4D/TA_gaugefields_4D_serial.jl:760)
// with the Cayley-Hamilton exponential, optional re-unitarisation
// (normalize3!, src/AbstractGaugefields.jl:3378) and an optional fp32
// 12-real shadow copy for the mixed-precision force path. All in fp64.
#include "gf_internal.h"

namespace gf {

template <typename R>
__device__ __forceinline__ R from_f64(double v);
template <>
__device__ __forceinline__ double from_f64<double>(double v) { return v; }
template <>
__device__ __forceinline__ dfl from_f64<dfl>(double v) { return df_from_double(v); }

__device__ __forceinline__ float to_f32(double v) { return (float)v; }
__device__ __forceinline__ float to_f32(dfl v) { return v.hi; }

// R = double: fp64 arithmetic. R = dfl: double-float arithmetic on the fp32
// pipes with the same fp64 storage (the mixed form).
template <typename R>
__global__ void __launch_bounds__(128) k_link_update(const double2* Uin, double2* Uout, const double* __restrict__ P,
                                                     Geom g, R eps, int reunit, float4* __restrict__ sh32) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  int mu = blockIdx.y;
  if (s >= g.vol) return;
  const int V = g.vol;
  R p[8];
#pragma unroll
  for (int a = 0; a < 8; ++a) p[a] = eps * from_f64<R>(P[((size_t)mu * 8 + a) * V + s]);
  mat3<R> q = herm_from_coeffs(p);
  mat3<R> u = LinkFull<R>::load(Uin, mu, s, V);
  // re-unitarisation rebuilds row 3 from rows 1-2, so only those are formed
  mat3<R> w;
  if (reunit) {
    w = mul_nn_rows12(expiq<R, 2, true>(q), u);
    reunitarize(w);
  } else {
    w = mul_nn(expiq<R, 3, true>(q), u);
  }
  LinkFull<R>::store(Uout, mu, s, V, w);
  if (sh32) {
    mat3<float> f;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) f.e[i][j] = mk(to_f32(w.e[i][j].re), to_f32(w.e[i][j].im));
    Link12f::store(sh32, mu, s, V, f);
  }
}

void link_update(gf_ctx* ctx, gf_field* U, const gf_field* P, double eps, int reunit, gf_field* shadow32, bool df) {
  if (U->kind != GF_LINK64) throw gf_error(GF_EINVAL, "link update: U must be LINK64");
  if (P->kind != GF_MOM64) throw gf_error(GF_EINVAL, "link update: P must be MOM64");
  dim3 grid(blocks_for(ctx->geom.vol, 128), 4);
  ProfScope prof(ctx, df ? GF_K_LINK_UPDATE_DF : GF_K_LINK_UPDATE);
  float4* sh = shadow32 ? (float4*)shadow32->ptr : nullptr;
  if (df)
    k_link_update<dfl><<<grid, 128, 0, ctx->stream>>>((const double2*)U->ptr, (double2*)U->ptr, (const double*)P->ptr,
                                                      ctx->geom, dfl(eps), reunit, sh);
  else
    k_link_update<double><<<grid, 128, 0, ctx->stream>>>((const double2*)U->ptr, (double2*)U->ptr,
                                                         (const double*)P->ptr, ctx->geom, eps, reunit, sh);
  GF_CHECK_LAUNCH();
}

// exp_aF_U!(W, a, F, U) (src/AbstractGaugefields.jl:2810-2842): W_mu = exp(a F_mu) U_mu
// with F in su(3) coefficients, i.e. exp(i a sum_a F_a lambda_a / 2) U.
void exp_mom_links(gf_ctx* ctx, gf_field* W, const gf_field* P, double a, const gf_field* U, bool df) {
  dim3 grid(blocks_for(ctx->geom.vol, 128), 4);
  ProfScope prof(ctx, df ? GF_K_LINK_UPDATE_DF : GF_K_LINK_UPDATE);
  if (df)
    k_link_update<dfl><<<grid, 128, 0, ctx->stream>>>((const double2*)U->ptr, (double2*)W->ptr,
                                                      (const double*)P->ptr, ctx->geom, dfl(a), 0, nullptr);
  else
    k_link_update<double><<<grid, 128, 0, ctx->stream>>>((const double2*)U->ptr, (double2*)W->ptr,
                                                         (const double*)P->ptr, ctx->geom, a, 0, nullptr);
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

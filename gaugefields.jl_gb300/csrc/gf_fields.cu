// Field allocation, host<->device transfer in the reference layout, cold and
// hot starts, Gaussian momenta, field copies/conversions and the deterministic
// two-stage reductions used by every global sum.
#include "gf_internal.h"
#include <vector>

namespace gf {

// ---------------------------------------------------------------------------
// storage sizes
// ---------------------------------------------------------------------------
size_t field_bytes(const Geom& g, int kind) {
  size_t V = (size_t)g.vol;
  switch (kind) {
    case GF_LINK64:
    case GF_MAT64: return 4 * 9 * V * sizeof(double2);
    case GF_LINKDF:
    case GF_MATDF: return 4 * 9 * V * sizeof(float4);
    case GF_LINK32: return 4 * 3 * V * sizeof(float4);
    case GF_MAT32: return 4 * 9 * V * sizeof(float2);
    case GF_MOM64: return 4 * 8 * V * sizeof(double);
  }
  throw gf_error(GF_EINVAL, "unknown field kind " + std::to_string(kind));
}

gf_field* field_new(gf_ctx* ctx, int kind) {
  size_t bytes = field_bytes(ctx->geom, kind);
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw gf_error(GF_ENOMEM, "cudaMalloc of " + std::to_string(bytes) + " bytes failed: " + cudaGetErrorString(e));
  }
  gf_field* f = new gf_field;
  f->ctx = ctx;
  f->kind = kind;
  f->ptr = p;
  f->bytes = bytes;
  f->owned = 1;
  return f;
}

gf_field* arena_view(gf_ctx* ctx, int which, size_t off, int kind) {
  const size_t cap = field_bytes(ctx->geom, GF_LINK64);
  if (!ctx->arena[which]) {
    cudaError_t e = cudaMalloc(&ctx->arena[which], cap);
    if (e != cudaSuccess) {
      cudaGetLastError();
      ctx->arena[which] = nullptr;
      throw gf_error(GF_ENOMEM, "cudaMalloc of " + std::to_string(cap) + " bytes failed: " + cudaGetErrorString(e));
    }
  }
  const size_t bytes = field_bytes(ctx->geom, kind);
  if (off + bytes > cap) throw gf_error(GF_EINVAL, "scratch view beyond its block");
  gf_field* f = new gf_field;
  f->ctx = ctx;
  f->kind = kind;
  f->ptr = (char*)ctx->arena[which] + off;
  f->bytes = bytes;
  f->owned = 0;
  return f;
}

void field_delete(gf_field* f) {
  if (!f) return;
  if (f->owned && f->ptr) cudaFree(f->ptr);
  delete f;
}

// ---------------------------------------------------------------------------
// deterministic reductions
// ---------------------------------------------------------------------------
__global__ void k_reduce_final(const double* __restrict__ part, int n, double* __restrict__ out) {
  __shared__ double sh[32];
  double v = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) v += part[i];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    v = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) *out = v;
  }
}

double finish_reduction(gf_ctx* ctx, int nblocks) {
  k_reduce_final<<<1, 1024, 0, ctx->stream>>>(ctx->d_partials, nblocks, ctx->d_result);
  GF_CHECK_LAUNCH();
  GF_CUDA(cudaMemcpyAsync(ctx->h_result, ctx->d_result, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  GF_CUDA(cudaStreamSynchronize(ctx->stream));
  return *ctx->h_result;
}

__device__ __forceinline__ void block_partial(double v, double* __restrict__ part) {
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

__global__ void k_kinetic(const double* __restrict__ P, int V, double* __restrict__ part) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  double v = 0.0;
  if (s < V) {
#pragma unroll
    for (int mu = 0; mu < 4; ++mu)
#pragma unroll
      for (int a = 0; a < 8; ++a) {
        double p = P[((size_t)mu * 8 + a) * V + s];
        v += p * p;
      }
  }
  block_partial(v, part);
}

double kinetic(gf_ctx* ctx, const gf_field* P) {
  int V = ctx->geom.vol;
  int nb = blocks_for(V, 256);
  k_kinetic<<<nb, 256, 0, ctx->stream>>>((const double*)P->ptr, V, ctx->d_partials);
  GF_CHECK_LAUNCH();
  return finish_reduction(ctx, nb);
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  // splitmix64 finaliser (Steele, Lea, Flood, "Fast splittable pseudorandom
  // number generators", OOPSLA 2014)
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__global__ void k_hash(const unsigned long long* __restrict__ w, size_t n, unsigned long long* __restrict__ out) {
  unsigned long long h = 0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    h += mix64(w[i] ^ (i * 0x9E3779B97F4A7C15ull));
  for (int o = 16; o > 0; o >>= 1) h += __shfl_down_sync(0xffffffffu, h, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, h);
}

unsigned long long field_hash(gf_ctx* ctx, const gf_field* f) {
  GF_CUDA(cudaMemsetAsync(ctx->d_hash, 0, sizeof(unsigned long long), ctx->stream));
  // a grid-stride loop over the field: eight blocks of 256 threads per SM
  k_hash<<<ctx->sm_count * 8, 256, 0, ctx->stream>>>((const unsigned long long*)f->ptr, f->bytes / 8, ctx->d_hash);
  GF_CHECK_LAUNCH();
  GF_CUDA(cudaMemcpyAsync(ctx->h_hash, ctx->d_hash, sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream));
  GF_CUDA(cudaStreamSynchronize(ctx->stream));
  return *ctx->h_hash;
}

// ---------------------------------------------------------------------------
// reference layout <-> device layout
// host links: complex (i,j,x,y,z,t) column-major, element (i,j) of direction
// mu at complex index mu*9V + i + 3j + 9*lex.
// ---------------------------------------------------------------------------
__global__ void k_links_from_ref(const double2* __restrict__ ref, double2* __restrict__ out, Geom g) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  int mu = blockIdx.y;
  if (s >= g.vol) return;
  Site st = site_of(g, s);
  const double2* src = ref + (size_t)mu * 9 * g.vol + (size_t)9 * st.lex;
  double2* dst = out + (size_t)mu * 9 * g.vol + s;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) dst[(size_t)(3 * i + j) * g.vol] = src[i + 3 * j];
}

__global__ void k_links_to_ref(const double2* __restrict__ in, double2* __restrict__ ref, Geom g) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  int mu = blockIdx.y;
  if (s >= g.vol) return;
  Site st = site_of(g, s);
  double2* dst = ref + (size_t)mu * 9 * g.vol + (size_t)9 * st.lex;
  const double2* src = in + (size_t)mu * 9 * g.vol + s;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) dst[i + 3 * j] = src[(size_t)(3 * i + j) * g.vol];
}

// host momenta: (a, x,y,z,t) per direction -> index mu*8V + a + 8*lex
__global__ void k_mom_from_ref(const double* __restrict__ ref, double* __restrict__ out, Geom g) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  int mu = blockIdx.y;
  if (s >= g.vol) return;
  Site st = site_of(g, s);
  const double* src = ref + (size_t)mu * 8 * g.vol + (size_t)8 * st.lex;
#pragma unroll
  for (int a = 0; a < 8; ++a) out[((size_t)mu * 8 + a) * g.vol + s] = src[a];
}

__global__ void k_mom_to_ref(const double* __restrict__ in, double* __restrict__ ref, Geom g) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  int mu = blockIdx.y;
  if (s >= g.vol) return;
  Site st = site_of(g, s);
  double* dst = ref + (size_t)mu * 8 * g.vol + (size_t)8 * st.lex;
#pragma unroll
  for (int a = 0; a < 8; ++a) dst[a] = in[((size_t)mu * 8 + a) * g.vol + s];
}

// One staging buffer per context, kept between transfers (a fresh 0.6 GB
// allocation per call cost more than the copy itself).
static void* staging(gf_ctx* ctx, size_t bytes) {
  if (ctx->stage_bytes < bytes) {
    if (ctx->d_stage) {
      GF_CUDA(cudaStreamSynchronize(ctx->stream));
      cudaFree(ctx->d_stage);
      ctx->d_stage = nullptr;
      ctx->stage_bytes = 0;
    }
    cudaError_t e = cudaMalloc(&ctx->d_stage, bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      throw gf_error(GF_ENOMEM, std::string("staging allocation failed: ") + cudaGetErrorString(e));
    }
    ctx->stage_bytes = bytes;
  }
  return ctx->d_stage;
}

static void require_kind(const gf_field* f, int k1, int k2, const char* what) {
  if (!f || (f->kind != k1 && f->kind != k2))
    throw gf_error(GF_EINVAL, std::string(what) + ": field has the wrong kind");
}

void upload_links(gf_ctx* ctx, gf_field* U, const double* host) {
  require_kind(U, GF_LINK64, GF_MAT64, "upload_links");
  size_t bytes = field_bytes(ctx->geom, GF_LINK64);
  void* tmp = staging(ctx, bytes);
  GF_CUDA(cudaMemcpyAsync(tmp, host, bytes, cudaMemcpyHostToDevice, ctx->stream));
  dim3 grid(blocks_for(ctx->geom.vol, 256), 4);
  k_links_from_ref<<<grid, 256, 0, ctx->stream>>>((const double2*)tmp, (double2*)U->ptr, ctx->geom);
  GF_CHECK_LAUNCH();
  GF_CUDA(cudaStreamSynchronize(ctx->stream));
}

void download_links(gf_ctx* ctx, const gf_field* U, double* host) {
  require_kind(U, GF_LINK64, GF_MAT64, "download_links");
  size_t bytes = field_bytes(ctx->geom, GF_LINK64);
  void* tmp = staging(ctx, bytes);
  dim3 grid(blocks_for(ctx->geom.vol, 256), 4);
  k_links_to_ref<<<grid, 256, 0, ctx->stream>>>((const double2*)U->ptr, (double2*)tmp, ctx->geom);
  GF_CHECK_LAUNCH();
  GF_CUDA(cudaMemcpyAsync(host, tmp, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  GF_CUDA(cudaStreamSynchronize(ctx->stream));
}

void upload_mom(gf_ctx* ctx, gf_field* P, const double* host) {
  require_kind(P, GF_MOM64, GF_MOM64, "upload_mom");
  size_t bytes = field_bytes(ctx->geom, GF_MOM64);
  void* tmp = staging(ctx, bytes);
  GF_CUDA(cudaMemcpyAsync(tmp, host, bytes, cudaMemcpyHostToDevice, ctx->stream));
  dim3 grid(blocks_for(ctx->geom.vol, 256), 4);
  k_mom_from_ref<<<grid, 256, 0, ctx->stream>>>((const double*)tmp, (double*)P->ptr, ctx->geom);
  GF_CHECK_LAUNCH();
  GF_CUDA(cudaStreamSynchronize(ctx->stream));
}

void download_mom(gf_ctx* ctx, const gf_field* P, double* host) {
  require_kind(P, GF_MOM64, GF_MOM64, "download_mom");
  size_t bytes = field_bytes(ctx->geom, GF_MOM64);
  void* tmp = staging(ctx, bytes);
  dim3 grid(blocks_for(ctx->geom.vol, 256), 4);
  k_mom_to_ref<<<grid, 256, 0, ctx->stream>>>((const double*)P->ptr, (double*)tmp, ctx->geom);
  GF_CHECK_LAUNCH();
  GF_CUDA(cudaMemcpyAsync(host, tmp, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  GF_CUDA(cudaStreamSynchronize(ctx->stream));
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11): counter-based, so every (site, direction, block) draw
// is independent of the launch shape.
// ---------------------------------------------------------------------------
struct u4 {
  uint32_t v[4];
};

__device__ __forceinline__ u4 philox4x32_10(u4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0 = __umulhi(M0, c.v[0]), lo0 = M0 * c.v[0];
    uint32_t hi1 = __umulhi(M1, c.v[2]), lo1 = M1 * c.v[2];
    u4 n;
    n.v[0] = hi1 ^ c.v[1] ^ k0;
    n.v[1] = lo1;
    n.v[2] = hi0 ^ c.v[3] ^ k1;
    n.v[3] = lo0;
    c = n;
    k0 += W0;
    k1 += W1;
  }
  return c;
}

// 53-bit uniform in (0,1) from two 32-bit words
__device__ __forceinline__ double u01(uint32_t a, uint32_t b) {
  uint64_t m = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
  return ((double)m + 0.5) * (1.0 / 9007199254740992.0);
}

// Box-Muller pair with standard deviation sigma
__device__ __forceinline__ void gauss_pair(u4 r, double sigma, double& g1, double& g2) {
  double u1 = u01(r.v[0], r.v[1]);
  double u2 = u01(r.v[2], r.v[3]);
  double rad = sigma * sqrt(-2.0 * log(u1));
  double sn, cs;
  sincospi(2.0 * u2, &sn, &cs);
  g1 = rad * cs;
  g2 = rad * sn;
}

#define GF_TAG_LINK 0x48415252u /* link hot start */
#define GF_TAG_MOM 0x4D4F4D30u  /* momenta */

__global__ void k_hot_start(double2* __restrict__ U, Geom g, uint32_t k0, uint32_t k1) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  int mu = blockIdx.y;
  if (s >= g.vol) return;
  Site st = site_of(g, s);
  mat3<double> m;
  const double sig = 0.70710678118654752440;  // re, im ~ N(0, 1/2)
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    u4 c;
    c.v[0] = (uint32_t)st.lex;
    c.v[1] = ((uint32_t)mu << 8) | (uint32_t)k;
    c.v[2] = 0u;
    c.v[3] = GF_TAG_LINK;
    u4 r = philox4x32_10(c, k0, k1);
    double a, b;
    gauss_pair(r, sig, a, b);
    m.e[k / 3][k % 3] = mk(a, b);
  }
  // Gram-Schmidt of the three rows
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int j = 0; j < i; ++j) {
      cplx<double> pr = mk(0.0, 0.0);  // <row_j, row_i> = sum conj(r_j) r_i
#pragma unroll
      for (int k = 0; k < 3; ++k) pr = pr + conj(m.e[j][k]) * m.e[i][k];
#pragma unroll
      for (int k = 0; k < 3; ++k) m.e[i][k] = m.e[i][k] - pr * m.e[j][k];
    }
    double n = 0.0;
#pragma unroll
    for (int k = 0; k < 3; ++k) n += m.e[i][k].re * m.e[i][k].re + m.e[i][k].im * m.e[i][k].im;
    double inv = 1.0 / sqrt(n);
#pragma unroll
    for (int k = 0; k < 3; ++k) m.e[i][k] = inv * m.e[i][k];
  }
  // divide out the determinant phase: U <- U * exp(-i arg(det U)/3)
  cplx<double> d = m.e[0][0] * (m.e[1][1] * m.e[2][2] - m.e[1][2] * m.e[2][1]) -
                   m.e[0][1] * (m.e[1][0] * m.e[2][2] - m.e[1][2] * m.e[2][0]) +
                   m.e[0][2] * (m.e[1][0] * m.e[2][1] - m.e[1][1] * m.e[2][0]);
  double phi = atan2(d.im, d.re) / 3.0;
  double sn, cs;
  sincos(phi, &sn, &cs);
  cplx<double> ph = mk(cs, -sn);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) m.e[i][j] = m.e[i][j] * ph;
  LinkFull<double>::store(U, mu, s, g.vol, m);
}

void hot_start(gf_ctx* ctx, gf_field* U, uint64_t seed) {
  require_kind(U, GF_LINK64, GF_LINK64, "hot_start");
  dim3 grid(blocks_for(ctx->geom.vol, 128), 4);
  k_hot_start<<<grid, 128, 0, ctx->stream>>>((double2*)U->ptr, ctx->geom, (uint32_t)seed, (uint32_t)(seed >> 32));
  GF_CHECK_LAUNCH();
}

__global__ void k_cold_start(double2* __restrict__ U, int V) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t n = (size_t)4 * 9 * V;
  if (i >= n) return;
  int k = (int)((i / V) % 9);
  U[i] = make_double2((k == 0 || k == 4 || k == 8) ? 1.0 : 0.0, 0.0);
}

void cold_start(gf_ctx* ctx, gf_field* U) {
  require_kind(U, GF_LINK64, GF_LINK64, "cold_start");
  size_t n = (size_t)36 * ctx->geom.vol;
  k_cold_start<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>((double2*)U->ptr, ctx->geom.vol);
  GF_CHECK_LAUNCH();
}

__global__ void k_gauss_mom(double* __restrict__ P, Geom g, uint32_t k0, uint32_t k1, uint32_t sw0, uint32_t sw1) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  int mu = blockIdx.y;
  if (s >= g.vol) return;
  Site st = site_of(g, s);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    u4 c;
    c.v[0] = (uint32_t)st.lex;
    c.v[1] = ((uint32_t)mu << 8) | (uint32_t)k;
    c.v[2] = sw0;
    c.v[3] = GF_TAG_MOM ^ sw1;
    u4 r = philox4x32_10(c, k0, k1);
    double a, b;
    gauss_pair(r, 1.0, a, b);
    P[((size_t)mu * 8 + 2 * k) * g.vol + s] = a;
    P[((size_t)mu * 8 + 2 * k + 1) * g.vol + s] = b;
  }
}

void gaussian_momenta(gf_ctx* ctx, gf_field* P, uint64_t seed, uint64_t sweep) {
  require_kind(P, GF_MOM64, GF_MOM64, "gaussian_momenta");
  dim3 grid(blocks_for(ctx->geom.vol, 256), 4);
  k_gauss_mom<<<grid, 256, 0, ctx->stream>>>((double*)P->ptr, ctx->geom, (uint32_t)seed, (uint32_t)(seed >> 32),
                                               (uint32_t)sweep, (uint32_t)(sweep >> 32));
  GF_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// copies and conversions
// ---------------------------------------------------------------------------
__global__ void k_link64_to_32(const double2* __restrict__ in, float4* __restrict__ out, int V) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  int mu = blockIdx.y;
  if (s >= V) return;
  mat3<double> m = LinkFull<double>::load(in, mu, s, V);
  mat3<float> f;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) f.e[i][j] = mk((float)m.e[i][j].re, (float)m.e[i][j].im);
  Link12f::store(out, mu, s, V, f);
}

__global__ void k_link32_to_64(const float4* __restrict__ in, double2* __restrict__ out, int V) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  int mu = blockIdx.y;
  if (s >= V) return;
  mat3<float> f = Link12f::load(in, mu, s, V);
  mat3<double> m;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) m.e[i][j] = mk((double)f.e[i][j].re, (double)f.e[i][j].im);
  LinkFull<double>::store(out, mu, s, V, m);
}

__global__ void k_mat64_to_32(const double2* __restrict__ in, float2* __restrict__ out, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    double2 v = in[i];
    out[i] = make_float2((float)v.x, (float)v.y);
  }
}

__global__ void k_mat32_to_64(const float2* __restrict__ in, double2* __restrict__ out, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    float2 v = in[i];
    out[i] = make_double2((double)v.x, (double)v.y);
  }
}

void link64_to_32(gf_ctx* ctx, gf_field* dst, const gf_field* src) {
  dim3 grid(blocks_for(ctx->geom.vol, 256), 4);
  k_link64_to_32<<<grid, 256, 0, ctx->stream>>>((const double2*)src->ptr, (float4*)dst->ptr, ctx->geom.vol);
  GF_CHECK_LAUNCH();
}

// fp64 <-> double-float-native storage, one complex element per thread
__global__ void k_f64_to_dfn(const double2* __restrict__ in, float4* __restrict__ out, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2 v = in[i];
  const dfl re = df_from_double(v.x), im = df_from_double(v.y);
  out[i] = make_float4(re.hi, re.lo, im.hi, im.lo);
}
__global__ void k_dfn_to_f64(const float4* __restrict__ in, double2* __restrict__ out, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 v = in[i];
  out[i] = make_double2(df_to_double(dfl(v.x, v.y)), df_to_double(dfl(v.z, v.w)));
}

static bool is_f64_full(int k) { return k == GF_LINK64 || k == GF_MAT64; }
static bool is_dfn(int k) { return k == GF_LINKDF || k == GF_MATDF; }

void copy_field(gf_ctx* ctx, gf_field* dst, const gf_field* src) {
  if (!dst || !src) throw gf_error(GF_EINVAL, "copy: null field");
  if (dst == src) return;
  int a = src->kind, b = dst->kind;
  bool full64 = (is_f64_full(a) && is_f64_full(b)) || (is_dfn(a) && is_dfn(b));
  if (a == b || full64) {
    GF_CUDA(cudaMemcpyAsync(dst->ptr, src->ptr, src->bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    return;
  }
  size_t n = (size_t)36 * ctx->geom.vol;
  unsigned nb = (unsigned)((n + 255) / 256);
  dim3 grid(blocks_for(ctx->geom.vol, 256), 4);
  if (a == GF_LINK64 && b == GF_LINK32) {
    link64_to_32(ctx, dst, src);
  } else if (a == GF_LINK32 && (b == GF_LINK64 || b == GF_MAT64)) {
    k_link32_to_64<<<grid, 256, 0, ctx->stream>>>((const float4*)src->ptr, (double2*)dst->ptr, ctx->geom.vol);
  } else if ((a == GF_LINK64 || a == GF_MAT64) && b == GF_MAT32) {
    k_mat64_to_32<<<nb, 256, 0, ctx->stream>>>((const double2*)src->ptr, (float2*)dst->ptr, n);
  } else if (a == GF_MAT32 && (b == GF_MAT64 || b == GF_LINK64)) {
    k_mat32_to_64<<<nb, 256, 0, ctx->stream>>>((const float2*)src->ptr, (double2*)dst->ptr, n);
  } else if (is_f64_full(a) && is_dfn(b)) {
    k_f64_to_dfn<<<nb, 256, 0, ctx->stream>>>((const double2*)src->ptr, (float4*)dst->ptr, n);
  } else if (is_dfn(a) && is_f64_full(b)) {
    k_dfn_to_f64<<<nb, 256, 0, ctx->stream>>>((const float4*)src->ptr, (double2*)dst->ptr, n);
  } else {
    throw gf_error(GF_EINVAL, "copy: unsupported kind conversion " + std::to_string(a) + " -> " + std::to_string(b));
  }
  GF_CHECK_LAUNCH();
}

void zero_field(gf_ctx* ctx, gf_field* f) { GF_CUDA(cudaMemsetAsync(f->ptr, 0, f->bytes, ctx->stream)); }

__global__ void k_axpy(double* __restrict__ y, double a, const double* __restrict__ x, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] += a * x[i];
}
__global__ void k_scale(double* __restrict__ y, double a, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] *= a;
}

void mom_axpy(gf_ctx* ctx, gf_field* y, double a, const gf_field* x) {
  size_t n = (size_t)32 * ctx->geom.vol;
  k_axpy<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>((double*)y->ptr, a, (const double*)x->ptr, n);
  GF_CHECK_LAUNCH();
}
void field_axpy(gf_ctx* ctx, gf_field* y, double a, const gf_field* x) {
  size_t n = y->bytes / sizeof(double);
  k_axpy<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>((double*)y->ptr, a, (const double*)x->ptr, n);
  GF_CHECK_LAUNCH();
}
void mom_scale(gf_ctx* ctx, gf_field* y, double a) {
  size_t n = (size_t)32 * ctx->geom.vol;
  k_scale<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>((double*)y->ptr, a, n);
  GF_CHECK_LAUNCH();
}

}  // namespace gf

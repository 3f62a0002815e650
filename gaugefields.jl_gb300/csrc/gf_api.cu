// C-ABI of libgfgb300: argument checking, status codes and the host-side
// drivers (MD trajectory, HMC update, RK3 flow) that sequence the kernels on
// the context's stream.
#include "gf_internal.h"
#include <cmath>
#include <cstring>
#include <new>

using namespace gf;

#include <atomic>

static thread_local std::string g_last_error;
static std::atomic<long long> g_launches(0);

namespace gf {
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void set_global_error(const std::string& m) { g_last_error = m; }

void prof_begin(gf_ctx* ctx, int kid) {
  if (!ctx->prof_on) return;
  if (ctx->prof_n == GF_PROF_CAP) prof_flush(ctx);
  ctx->prof_kid[ctx->prof_n] = kid;
  cudaEventRecord(ctx->prof_ev[2 * ctx->prof_n], ctx->stream);
}

void prof_end(gf_ctx* ctx, int kid) {
  if (!ctx->prof_on) return;
  (void)kid;
  cudaEventRecord(ctx->prof_ev[2 * ctx->prof_n + 1], ctx->stream);
  ctx->prof_n++;
}

void prof_flush(gf_ctx* ctx) {
  if (ctx->prof_n == 0) return;
  GF_CUDA(cudaEventSynchronize(ctx->prof_ev[2 * ctx->prof_n - 1]));
  for (int i = 0; i < ctx->prof_n; ++i) {
    float ms = 0.f;
    GF_CUDA(cudaEventElapsedTime(&ms, ctx->prof_ev[2 * i], ctx->prof_ev[2 * i + 1]));
    ctx->prof_ms[ctx->prof_kid[i]] += ms;
    ctx->prof_cnt[ctx->prof_kid[i]] += 1;
  }
  ctx->prof_n = 0;
}
}  // namespace gf

static void set_err(const gf_ctx* ctx, const std::string& m) {
  g_last_error = m;
  if (ctx) const_cast<gf_ctx*>(ctx)->err = m;
}

#define API_BEGIN try {
#define API_END(ctx)                           \
  }                                            \
  catch (const gf_error& e) {                  \
    set_err(ctx, e.what());                    \
    return e.code;                             \
  }                                            \
  catch (const std::bad_alloc&) {              \
    set_err(ctx, "host allocation failed");    \
    return GF_ENOMEM;                          \
  }                                            \
  catch (const std::exception& e) {            \
    set_err(ctx, e.what());                    \
    return GF_ECUDA;                           \
  }                                            \
  return GF_OK;

static void need(bool ok, const char* msg) {
  if (!ok) throw gf_error(GF_EINVAL, msg);
}

static void need_kind(const gf_field* f, int kind, const char* what) {
  need(f != nullptr, what);
  if (f->kind != kind) throw gf_error(GF_EINVAL, std::string(what) + ": wrong field kind");
}

static void need_ctx(const gf_ctx* ctx, const gf_field* f) {
  if (f && f->ctx != ctx) throw gf_error(GF_EINVAL, "field belongs to another context");
}

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
extern "C" int gf_ctx_create(const int L[4], int device, gf_ctx** out) {
  gf_ctx* ctx = nullptr;
  API_BEGIN
  need(L != nullptr && out != nullptr, "gf_ctx_create: null argument");
  *out = nullptr;
  long long V = 1;
  for (int i = 0; i < 4; ++i) {
    need(L[i] >= 2 && (L[i] % 2) == 0, "gf_ctx_create: every lattice extent must be even and >= 2");
    V *= L[i];
    // checked after every factor: the running product stays below 2^28 before
    // the next multiply, so it cannot overflow
    need(V <= (1LL << 28), "gf_ctx_create: volume too large for 32-bit site indices");
  }
  GF_CUDA(cudaSetDevice(device));
  ctx = new gf_ctx();
  ctx->device = device;
  GF_CUDA(cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device));
  for (int i = 0; i < 4; ++i) ctx->geom.L[i] = L[i];
  ctx->geom.vol = (int)V;
  ctx->geom.vh = (int)(V / 2);
  ctx->geom.stride[0] = 1;
  ctx->geom.stride[1] = L[0];
  ctx->geom.stride[2] = L[0] * L[1];
  ctx->geom.stride[3] = L[0] * L[1] * L[2];
  GF_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
  ctx->own_stream = 1;
  ctx->partial_cap = blocks_for((int)V, 128) + 1;
  GF_CUDA(cudaMalloc(&ctx->d_partials, sizeof(double) * ctx->partial_cap));
  GF_CUDA(cudaMalloc(&ctx->d_result, sizeof(double) * 4));
  GF_CUDA(cudaMallocHost(&ctx->h_result, sizeof(double) * 4));
  GF_CUDA(cudaMalloc(&ctx->d_hash, sizeof(unsigned long long)));
  GF_CUDA(cudaMallocHost(&ctx->h_hash, sizeof(unsigned long long)));
  *out = ctx;
  return GF_OK;
  }
  catch (const gf_error& e) {
    set_err(nullptr, e.what());
    if (ctx) gf_ctx_destroy(ctx);
    return e.code;
  }
  catch (const std::exception& e) {
    set_err(nullptr, e.what());
    if (ctx) gf_ctx_destroy(ctx);
    return GF_ECUDA;
  }
}

extern "C" int gf_stout_destroy(gf_stout* st);

extern "C" int gf_ctx_destroy(gf_ctx* ctx) {
  if (!ctx) return GF_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  field_delete(ctx->w_link64);
  field_delete(ctx->w_link64b);
  for (int i = 0; i < 4; ++i) field_delete(ctx->w_mom[i]);
  field_delete(ctx->w_link32);
  field_delete(ctx->w_linkdf);
  if (ctx->w_stout64) gf_stout_destroy(ctx->w_stout64);
  if (ctx->w_stout32) gf_stout_destroy(ctx->w_stout32);
  if (ctx->w_stoutdf) gf_stout_destroy(ctx->w_stoutdf);
  if (ctx->d_partials) cudaFree(ctx->d_partials);
  if (ctx->d_result) cudaFree(ctx->d_result);
  if (ctx->h_result) cudaFreeHost(ctx->h_result);
  if (ctx->d_hash) cudaFree(ctx->d_hash);
  if (ctx->d_stage) cudaFree(ctx->d_stage);
  for (int i = 0; i < 2; ++i)
    if (ctx->arena[i]) cudaFree(ctx->arena[i]);
  if (ctx->h_hash) cudaFreeHost(ctx->h_hash);
  if (ctx->prof_ev) {
    for (int i = 0; i < 2 * GF_PROF_CAP; ++i) cudaEventDestroy(ctx->prof_ev[i]);
    delete[] ctx->prof_ev;
  }
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return GF_OK;
}

extern "C" int gf_ctx_set_stream(gf_ctx* ctx, void* cuda_stream) {
  API_BEGIN
  need(ctx != nullptr, "gf_ctx_set_stream: null context");
  GF_CUDA(cudaStreamSynchronize(ctx->stream));
  if (ctx->own_stream) {
    GF_CUDA(cudaStreamDestroy(ctx->stream));
    ctx->own_stream = 0;
  }
  if (cuda_stream) {
    ctx->stream = (cudaStream_t)cuda_stream;
  } else {
    GF_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    ctx->own_stream = 1;
  }
  API_END(ctx)
}

extern "C" int gf_ctx_synchronize(gf_ctx* ctx) {
  API_BEGIN
  need(ctx != nullptr, "gf_ctx_synchronize: null context");
  GF_CUDA(cudaStreamSynchronize(ctx->stream));
  API_END(ctx)
}

extern "C" const char* gf_last_error(const gf_ctx* ctx) {
  if (ctx) return ctx->err.c_str();
  return g_last_error.c_str();
}

extern "C" int gf_ctx_volume(const gf_ctx* ctx, int64_t* out) {
  API_BEGIN
  need(ctx && out, "gf_ctx_volume: null argument");
  *out = ctx->geom.vol;
  API_END(ctx)
}

// ---------------------------------------------------------------------------
// fields
// ---------------------------------------------------------------------------
extern "C" int gf_field_alloc(gf_ctx* ctx, int kind, gf_field** out) {
  API_BEGIN
  need(ctx && out, "gf_field_alloc: null argument");
  need(kind >= GF_LINK64 && kind <= GF_MAT32, "gf_field_alloc: unknown kind");
  GF_CUDA(cudaSetDevice(ctx->device));
  *out = field_new(ctx, kind);
  API_END(ctx)
}

extern "C" int gf_field_free(gf_field* f) {
  // cudaFree waits for outstanding work on the buffer; the context is not
  // touched, so a field may be freed after its context.
  if (!f) return GF_OK;
  field_delete(f);
  return GF_OK;
}

extern "C" int gf_field_kind(const gf_field* f, int* kind) {
  if (!f || !kind) return GF_EINVAL;
  *kind = f->kind;
  return GF_OK;
}

extern "C" int gf_field_bytes(const gf_field* f, size_t* bytes) {
  if (!f || !bytes) return GF_EINVAL;
  *bytes = f->bytes;
  return GF_OK;
}

extern "C" int gf_field_device_ptr(const gf_field* f, void** ptr) {
  if (!f || !ptr) return GF_EINVAL;
  *ptr = f->ptr;
  return GF_OK;
}

extern "C" int gf_field_copy(gf_ctx* ctx, gf_field* dst, const gf_field* src) {
  API_BEGIN
  need(ctx && dst && src, "gf_field_copy: null argument");
  need_ctx(ctx, dst);
  need_ctx(ctx, src);
  copy_field(ctx, dst, src);
  API_END(ctx)
}

extern "C" int gf_field_zero(gf_ctx* ctx, gf_field* f) {
  API_BEGIN
  need(ctx && f, "gf_field_zero: null argument");
  need_ctx(ctx, f);
  zero_field(ctx, f);
  API_END(ctx)
}

extern "C" int gf_field_axpy(gf_ctx* ctx, gf_field* y, double a, const gf_field* x) {
  API_BEGIN
  need(ctx && y && x, "gf_field_axpy: null argument");
  need_ctx(ctx, y);
  need_ctx(ctx, x);
  need(y->kind == x->kind, "gf_field_axpy: the fields must be of one kind");
  need(y->kind == GF_LINK64 || y->kind == GF_MAT64 || y->kind == GF_MOM64,
       "gf_field_axpy: fp64 fields (LINK64, MAT64, MOM64) only");
  need(std::isfinite(a), "gf_field_axpy: the factor must be finite");
  field_axpy(ctx, y, a, x);
  API_END(ctx)
}

// ---------------------------------------------------------------------------
// host transfer
// ---------------------------------------------------------------------------
extern "C" int gf_upload_links(gf_ctx* ctx, gf_field* U, const double* host) {
  API_BEGIN
  need(ctx && U && host, "gf_upload_links: null argument");
  need_ctx(ctx, U);
  upload_links(ctx, U, host);
  API_END(ctx)
}
extern "C" int gf_download_links(gf_ctx* ctx, const gf_field* U, double* host) {
  API_BEGIN
  need(ctx && U && host, "gf_download_links: null argument");
  need_ctx(ctx, U);
  download_links(ctx, U, host);
  API_END(ctx)
}
extern "C" int gf_upload_mom(gf_ctx* ctx, gf_field* P, const double* host) {
  API_BEGIN
  need(ctx && P && host, "gf_upload_mom: null argument");
  need_ctx(ctx, P);
  upload_mom(ctx, P, host);
  API_END(ctx)
}
extern "C" int gf_download_mom(gf_ctx* ctx, const gf_field* P, double* host) {
  API_BEGIN
  need(ctx && P && host, "gf_download_mom: null argument");
  need_ctx(ctx, P);
  download_mom(ctx, P, host);
  API_END(ctx)
}

// ---------------------------------------------------------------------------
// starts
// ---------------------------------------------------------------------------
extern "C" int gf_cold_start(gf_ctx* ctx, gf_field* U) {
  API_BEGIN
  need(ctx && U, "gf_cold_start: null argument");
  need_ctx(ctx, U);
  cold_start(ctx, U);
  API_END(ctx)
}
extern "C" int gf_hot_start(gf_ctx* ctx, gf_field* U, uint64_t seed) {
  API_BEGIN
  need(ctx && U, "gf_hot_start: null argument");
  need_ctx(ctx, U);
  hot_start(ctx, U, seed);
  API_END(ctx)
}
extern "C" int gf_gaussian_momenta(gf_ctx* ctx, gf_field* P, uint64_t seed, uint64_t sweep) {
  API_BEGIN
  need(ctx && P, "gf_gaussian_momenta: null argument");
  need_ctx(ctx, P);
  gaussian_momenta(ctx, P, seed, sweep);
  API_END(ctx)
}

extern "C" int gf_mom_scale(gf_ctx* ctx, gf_field* P, double a) {
  API_BEGIN
  need(ctx && P, "gf_mom_scale: null argument");
  need_ctx(ctx, P);
  need_kind(P, GF_MOM64, "gf_mom_scale: P");
  need(std::isfinite(a), "gf_mom_scale: the factor must be finite");
  mom_scale(ctx, P, a);
  API_END(ctx)
}
extern "C" int gf_reunitarize(gf_ctx* ctx, gf_field* U) {
  API_BEGIN
  need(ctx && U, "gf_reunitarize: null argument");
  need_ctx(ctx, U);
  reunitarize_links(ctx, U);
  API_END(ctx)
}

// ---------------------------------------------------------------------------
// measurements
// ---------------------------------------------------------------------------
extern "C" int gf_plaquette(gf_ctx* ctx, const gf_field* U, double* out) {
  API_BEGIN
  need(ctx && U && out, "gf_plaquette: null argument");
  need_ctx(ctx, U);
  *out = plaquette_sum(ctx, U);
  API_END(ctx)
}
extern "C" int gf_polyakov_loop(gf_ctx* ctx, const gf_field* U, double* out) {
  API_BEGIN
  need(ctx && U && out, "gf_polyakov_loop: null argument");
  need_ctx(ctx, U);
  need_kind(U, GF_LINK64, "gf_polyakov_loop: U");
  polyakov_loop(ctx, U, out);
  API_END(ctx)
}
extern "C" int gf_action(gf_ctx* ctx, const gf_field* U, double beta, double* out) {
  API_BEGIN
  need(ctx && U && out, "gf_action: null argument");
  need_ctx(ctx, U);
  need(std::isfinite(beta), "gf_action: beta must be finite");
  *out = -(beta / 3.0) * plaquette_sum(ctx, U);
  API_END(ctx)
}
extern "C" int gf_rectangle(gf_ctx* ctx, const gf_field* U, double* out) {
  API_BEGIN
  need(ctx && U && out, "gf_rectangle: null argument");
  need_ctx(ctx, U);
  need_kind(U, GF_LINK64, "gf_rectangle: U");
  *out = rectangle_sum(ctx, U);
  API_END(ctx)
}
extern "C" int gf_action_loops(gf_ctx* ctx, const gf_field* U, double c_plaq, double c_rect, double* out) {
  API_BEGIN
  need(ctx && U && out, "gf_action_loops: null argument");
  need_ctx(ctx, U);
  need(std::isfinite(c_plaq) && std::isfinite(c_rect), "gf_action_loops: the coefficients must be finite");
  need_kind(U, GF_LINK64, "gf_action_loops: U");
  double v = c_plaq * plaquette_sum(ctx, U);
  if (c_rect != 0.0) v += c_rect * rectangle_sum(ctx, U);
  *out = -(2.0 / 3.0) * v;
  API_END(ctx)
}
extern "C" int gf_kinetic(gf_ctx* ctx, const gf_field* P, double* out) {
  API_BEGIN
  need(ctx && P && out, "gf_kinetic: null argument");
  need_ctx(ctx, P);
  need_kind(P, GF_MOM64, "gf_kinetic");
  *out = kinetic(ctx, P);
  API_END(ctx)
}
extern "C" int gf_staple(gf_ctx* ctx, const gf_field* U, int mu, gf_field* V) {
  API_BEGIN
  need(ctx && U && V, "gf_staple: null argument");
  need_ctx(ctx, U);
  need_ctx(ctx, V);
  staple_up(ctx, U, mu, V);
  API_END(ctx)
}

// ---------------------------------------------------------------------------
// stout workspace
// ---------------------------------------------------------------------------
static gf_stout* stout_new(gf_ctx* ctx, int nlev, const double* rho, int precision, int store,
                           bool fwd_only = false, bool arena = false) {
  need(nlev >= 1 && nlev <= GF_MAX_STOUT, "stout: number of levels must be 1..GF_MAX_STOUT");
  need(precision == GF_FP64 || precision == GF_MIXED || precision == GF_DFLOAT,
       "stout: precision must be GF_FP64, GF_MIXED or GF_DFLOAT");
  for (int l = 0; l < nlev; ++l) need(std::isfinite(rho[l]), "stout: rho must be finite");
  gf_stout* st = new gf_stout();
  st->ctx = ctx;
  st->nlev = nlev;
  for (int l = 0; l < nlev; ++l) st->rho[l] = rho[l];
  st->precision = precision;
  st->store = store ? 1 : 0;
  // double-float stacks keep their levels and adjoint fields as fp32 hi/lo
  // pairs (no conversion on the kernels' loads)
  int lk = precision == GF_MIXED ? GF_LINK32 : (precision == GF_PREC_DF ? GF_LINKDF : GF_LINK64);
  int mk = precision == GF_MIXED ? GF_MAT32 : (precision == GF_PREC_DF ? GF_MATDF : GF_MAT64);
  try {
    for (int l = 1; l <= nlev; ++l) {
      if (fwd_only && arena && l <= 2) {
        st->lev_in[l] = arena_view(ctx, l - 1, 0, lk);
      } else if (fwd_only && l > 2) {
        // a forward-only stack holds one level's input and output at a time:
        // level l writes where level l - 2 wrote (two buffers in turn)
        gf_field* a = new gf_field(*st->lev_in[l - 2]);
        a->owned = 0;
        st->lev_in[l] = a;
      } else {
        st->lev_in[l] = field_new(ctx, lk);
      }
    }
    if (fwd_only) {
      st->store = 0;  // forward only: no C, no back-propagation buffers
      st->fwd_only = 1;
      return st;
    }
    if (st->store)
      for (int l = 0; l < nlev; ++l) st->C[l] = field_new(ctx, mk);
    if (arena && mk == GF_MAT32) {
      // two fp32 matrix fields fill one fp64 link-sized block
      const size_t half = field_bytes(ctx->geom, GF_MAT32);
      st->Z = arena_view(ctx, 0, 0, mk);
      st->Dp = arena_view(ctx, 0, half, mk);
      st->D[0] = arena_view(ctx, 1, 0, mk);
      st->D[1] = arena_view(ctx, 1, half, mk);
    } else {
      st->Z = field_new(ctx, mk);
      st->Dp = field_new(ctx, mk);
      st->D[0] = field_new(ctx, mk);
      st->D[1] = field_new(ctx, mk);
    }
  } catch (...) {
    gf_stout_destroy(st);
    throw;
  }
  return st;
}

extern "C" int gf_stout_create(gf_ctx* ctx, int nlev, const double* rho, int precision, int store, gf_stout** out) {
  API_BEGIN
  need(ctx && rho && out, "gf_stout_create: null argument");
  need(precision == GF_FP64 || precision == GF_MIXED || precision == GF_DFLOAT,
       "gf_stout_create: precision must be GF_FP64, GF_MIXED or GF_DFLOAT");
  *out = stout_new(ctx, nlev, rho, precision, store);
  API_END(ctx)
}

extern "C" int gf_stout_destroy(gf_stout* st) {
  if (!st) return GF_OK;
  for (int l = 0; l <= GF_MAX_STOUT; ++l) field_delete(st->lev_in[l]);
  for (int l = 0; l < GF_MAX_STOUT; ++l) field_delete(st->C[l]);
  field_delete(st->Z);
  field_delete(st->Dp);
  field_delete(st->D[0]);
  field_delete(st->D[1]);
  delete st;
  return GF_OK;
}

extern "C" int gf_stout_forward(gf_ctx* ctx, gf_stout* st, const gf_field* U, gf_field* Uout) {
  API_BEGIN
  need(ctx && st && U, "gf_stout_forward: null argument");
  need_ctx(ctx, U);
  need_ctx(ctx, Uout);
  need(st->ctx == ctx, "gf_stout_forward: stack belongs to another context");
  stout_forward(ctx, st, U, Uout);
  API_END(ctx)
}

extern "C" int gf_stout_backward(gf_ctx* ctx, gf_stout* st, const gf_field* dSdUbar, gf_field* dSdU) {
  API_BEGIN
  need(ctx && st && dSdUbar && dSdU, "gf_stout_backward: null argument");
  need_ctx(ctx, dSdUbar);
  need_ctx(ctx, dSdU);
  stout_backward(ctx, st, dSdUbar, 0.0, dSdU, nullptr, 0.0);
  API_END(ctx)
}

extern "C" int gf_stout_param_derivatives(gf_ctx* ctx, gf_stout* st, const gf_field* U, const gf_field* dSdUbar,
                                          double* dSdrho) {
  API_BEGIN
  need(ctx && st && U && dSdUbar && dSdrho, "gf_stout_param_derivatives: null argument");
  need_ctx(ctx, U);
  need_ctx(ctx, dSdUbar);
  need(st->ctx == ctx, "gf_stout_param_derivatives: stack belongs to another context");
  stout_forward(ctx, st, U, nullptr);
  stout_backward(ctx, st, dSdUbar, 0.0, nullptr, nullptr, 0.0, dSdrho);
  API_END(ctx)
}

extern "C" int gf_stout_mom_update(gf_ctx* ctx, gf_stout* st, gf_field* P, const gf_field* U, double eps,
                                   double beta) {
  API_BEGIN
  need(ctx && st && P && U, "gf_stout_mom_update: null argument");
  need_ctx(ctx, P);
  need_ctx(ctx, U);
  need_kind(P, GF_MOM64, "gf_stout_mom_update");
  need(std::isfinite(eps) && std::isfinite(beta), "gf_stout_mom_update: eps and beta must be finite");
  stout_forward(ctx, st, U, nullptr);
  stout_backward(ctx, st, nullptr, beta, nullptr, P, eps);
  API_END(ctx)
}

// ---------------------------------------------------------------------------
// molecular dynamics
// ---------------------------------------------------------------------------
static void check_md(const gf_md_params* p) {
  need(p != nullptr, "md: null parameters");
  need(p->steps > 0, "md: steps must be positive");
  need(std::isfinite(p->tau), "md: trajectory_length must be finite");
  need(p->tau != 0.0, "md: trajectory_length must not be zero");
  need(std::isfinite(p->beta), "md: beta must be finite");
  need(p->integrator == GF_QPQ || p->integrator == GF_PQP || p->integrator == GF_OMELYAN,
       "md: integrator must be GF_QPQ, GF_PQP or GF_OMELYAN");
  need(p->integrator != GF_OMELYAN || std::isfinite(p->lambda), "md: the Omelyan lambda must be finite");
  need(p->precision == GF_FP64 || p->precision == GF_MIXED || p->precision == GF_DFLOAT,
       "md: precision must be GF_FP64, GF_MIXED or GF_DFLOAT");
  need(p->nstout >= 0 && p->nstout <= GF_MAX_STOUT, "md: nstout must be 0..GF_MAX_STOUT");
  for (int l = 0; l < p->nstout; ++l) need(std::isfinite(p->rho[l]), "md: rho must be finite");
  need(std::isfinite(p->c_rect), "md: c_rect must be finite");
}

// The context's stack for a stack precision. The mixed form's Hamiltonian
// uses a forward-only double-float stack; the GF_DFLOAT form shares one full
// double-float stack between its force and its Hamiltonian.
static gf_stout* ctx_stout(gf_ctx* ctx, const gf_md_params* p, int precision) {
  gf_stout** slot = precision == GF_FP64 ? &ctx->w_stout64
                    : (precision == GF_MIXED ? &ctx->w_stout32 : &ctx->w_stoutdf);
  const bool fwd_only = precision == GF_PREC_DF && p->precision == GF_MIXED;
  int store = fwd_only ? 0 : (p->stout_recompute ? 0 : 1);
  bool same = *slot && (*slot)->nlev == p->nstout && (*slot)->store == store && (*slot)->fwd_only == (int)fwd_only;
  if (same)
    for (int l = 0; l < p->nstout; ++l) same = same && (*slot)->rho[l] == p->rho[l];
  if (!same) {
    if (*slot) gf_stout_destroy(*slot);
    *slot = nullptr;
    // the mixed form's two internal stacks share the context's scratch blocks
    *slot = stout_new(ctx, p->nstout, p->rho, precision, store, fwd_only, p->precision == GF_MIXED);
  }
  return *slot;
}

// The potential on the (smeared) fp64 links, plaquette and rectangle loops.
// The plain form evaluates it in fp64. The mixed and double-float forms smear
// in double-float arithmetic (compensated products, ~1e-13 of the operands'
// norms) on the fp32 pipes, which on GB300 is 2.1x faster than the fp64 stout
// forward; the loop sums over the smeared links stay fp64
// (GF_DF_HAMILTONIAN=0 keeps the mixed form's potential fp64).
#ifndef GF_DF_HAMILTONIAN
#define GF_DF_HAMILTONIAN 1
#endif
static double potential(gf_ctx* ctx, const gf_field* U, const gf_md_params* p) {
  bool df = (GF_DF_HAMILTONIAN && p->precision == GF_MIXED) || p->precision == GF_DFLOAT;
  const gf_field* links = U;
  if (p->nstout > 0) {
    gf_stout* st = ctx_stout(ctx, p, df ? GF_PREC_DF : GF_FP64);
    stout_forward(ctx, st, U, nullptr);
    links = stout_top(st);
  }
  double v = -(p->beta / 3.0) * plaquette_sum(ctx, links);
  if (p->c_rect != 0.0) v -= (2.0 / 3.0) * p->c_rect * rectangle_sum(ctx, links);
  return v;
}

static double hamiltonian(gf_ctx* ctx, const gf_field* U, const gf_field* P, const gf_md_params* p) {
  double v = potential(ctx, U, p);
  return v + 0.5 * kinetic(ctx, P);
}

// P += eps * F(U) with the force of the (smeared) Wilson action
static void mom_update(gf_ctx* ctx, gf_field* P, const gf_field* U, const gf_field* U32, double eps,
                       const gf_md_params* p) {
  const gf_field* links = (p->precision == GF_MIXED) ? U32 : U;
  if (p->nstout == 0 && p->c_rect != 0.0) {
    loops_force_coef(ctx, links, P, eps * (-1.0 / 3.0) * (0.5 * p->beta), eps * (-1.0 / 3.0) * p->c_rect, 1.0,
                     p->precision == GF_DFLOAT);
    return;
  }
  if (p->c_rect != 0.0) {
    // smeared plaquette + rectangle action: dS/dUbar = beta/2 S + c_rect R on
    // the top level, written into the stack's D[1] and back-propagated
    gf_stout* st = ctx_stout(ctx, p, p->precision);
    stout_forward(ctx, st, links, nullptr);
    loops_dsdu(ctx, stout_top(st), st->D[1], 0.5 * p->beta, p->c_rect);
    stout_backward(ctx, st, st->D[1], p->beta, nullptr, P, eps);
    return;
  }
  if (p->nstout == 0) {
    wilson_force_coef(ctx, links, P, eps * (-1.0 / 3.0) * (0.5 * p->beta), 1.0, p->precision == GF_DFLOAT);
    return;
  }
  gf_stout* st = ctx_stout(ctx, p, p->precision);
  stout_forward(ctx, st, links, nullptr);
  stout_backward(ctx, st, nullptr, p->beta, nullptr, P, eps);
}

// The potential at the start of a trajectory is the one the previous MD call
// ended on (accepted) or started from (rejected: gf_hmc_update restores the
// links, and a caller doing its own Metropolis around gf_md_trajectory
// uploads or copies the old links back). Both are kept, each keyed by a
// 64-bit hash of the fp64 links and the action parameters; a match saves one
// stout forward + plaquette per trajectory. Any change of the links changes
// the hash, so a reused value is bitwise the recomputed one.
static bool vcache_lookup(const gf_ctx* ctx, const gf_md_params* p, unsigned long long h, double* V) {
  for (int e = 0; e < 2; ++e) {
    const auto& c = ctx->vc[e];
    if (!c.valid || c.hash != h || c.beta != p->beta || c.c_rect != p->c_rect || c.nstout != p->nstout ||
        c.precision != p->precision)
      continue;
    bool same = true;
    for (int l = 0; l < p->nstout; ++l) same = same && c.rho[l] == p->rho[l];
    if (same) {
      *V = c.V;
      return true;
    }
  }
  return false;
}

static void vcache_clear(gf_ctx* ctx) {
  ctx->vc[0].valid = 0;
  ctx->vc[1].valid = 0;
}

// entry 0: the configuration an MD call ended on, entry 1: the one it started from
static void vcache_set(gf_ctx* ctx, const gf_md_params* p, int e, unsigned long long h, double V) {
  auto& c = ctx->vc[e];
  c.valid = std::isfinite(V) ? 1 : 0;
  c.hash = h;
  c.V = V;
  c.beta = p->beta;
  c.c_rect = p->c_rect;
  c.nstout = p->nstout;
  c.precision = p->precision;
  for (int l = 0; l < GF_MAX_STOUT; ++l) c.rho[l] = l < p->nstout ? p->rho[l] : 0.0;
}

struct MDResult {
  double H0, H1, V0, V1;
  unsigned long long h0, h1;
};

static MDResult md_run(gf_ctx* ctx, gf_field* U, gf_field* P, const gf_md_params* p) {
  need_kind(U, GF_LINK64, "md: U");
  need_kind(P, GF_MOM64, "md: P");
  gf_field* U32 = nullptr;
  if (p->precision == GF_MIXED) {
    if (!ctx->w_link32) ctx->w_link32 = field_new(ctx, GF_LINK32);
    U32 = ctx->w_link32;
    link64_to_32(ctx, U32, U);
  }
  MDResult r;
  r.h0 = field_hash(ctx, U);
  if (!vcache_lookup(ctx, p, r.h0, &r.V0)) r.V0 = potential(ctx, U, p);
  r.H0 = r.V0 + 0.5 * kinetic(ctx, P);
  double eps = p->tau / p->steps;
  // Adjacent half steps of consecutive QPQ (PQP) steps act with the same P
  // (the same U), so they are applied as one full step, as the reference's
  // _md_fast_qpq! does (molecular_dynamics.jl:618-633): n+1 link updates and
  // n forces (QPQ), or n+1 forces and n link updates (PQP). The trajectory
  // is the one of md_step! up to rounding.
  const bool df = p->precision != GF_FP64;  // link updates in double-float
  if (p->integrator == GF_QPQ) {
    link_update(ctx, U, P, 0.5 * eps, p->reunitarize, U32, df);
    for (int n = 0; n < p->steps; ++n) {
      mom_update(ctx, P, U, U32, eps, p);
      link_update(ctx, U, P, (n == p->steps - 1) ? 0.5 * eps : eps, p->reunitarize, U32, df);
    }
  } else if (p->integrator == GF_PQP) {
    mom_update(ctx, P, U, U32, 0.5 * eps, p);
    for (int n = 0; n < p->steps; ++n) {
      link_update(ctx, U, P, eps, p->reunitarize, U32, df);
      mom_update(ctx, P, U, U32, (n == p->steps - 1) ? 0.5 * eps : eps, p);
    }
  } else {
    // Omelyan PQPQP: P(l eps) Q(eps/2) P((1-2l) eps) Q(eps/2) P(l eps); the
    // closing and opening kicks of consecutive steps merge into P(2 l eps).
    const double lam = p->lambda;
    mom_update(ctx, P, U, U32, lam * eps, p);
    for (int n = 0; n < p->steps; ++n) {
      link_update(ctx, U, P, 0.5 * eps, p->reunitarize, U32, df);
      mom_update(ctx, P, U, U32, (1.0 - 2.0 * lam) * eps, p);
      link_update(ctx, U, P, 0.5 * eps, p->reunitarize, U32, df);
      mom_update(ctx, P, U, U32, (n == p->steps - 1 ? 1.0 : 2.0) * lam * eps, p);
    }
  }
  r.V1 = potential(ctx, U, p);
  r.H1 = r.V1 + 0.5 * kinetic(ctx, P);
  r.h1 = field_hash(ctx, U);
  return r;
}

extern "C" int gf_force(gf_ctx* ctx, const gf_field* U, double beta, gf_field* F) {
  API_BEGIN
  need(ctx && U && F, "gf_force: null argument");
  need_ctx(ctx, U);
  need_ctx(ctx, F);
  need(std::isfinite(beta), "gf_force: beta must be finite");
  wilson_force_coef(ctx, U, F, -(1.0 / 3.0) * (0.5 * beta), 0.0);
  API_END(ctx)
}

extern "C" int gf_force_loops(gf_ctx* ctx, const gf_field* U, double c_plaq, double c_rect, gf_field* F) {
  API_BEGIN
  need(ctx && U && F, "gf_force_loops: null argument");
  need_ctx(ctx, U);
  need_ctx(ctx, F);
  need(std::isfinite(c_plaq) && std::isfinite(c_rect), "gf_force_loops: the coefficients must be finite");
  need_kind(U, GF_LINK64, "gf_force_loops: U");
  loops_force_coef(ctx, U, F, -(1.0 / 3.0) * c_plaq, -(1.0 / 3.0) * c_rect, 0.0);
  API_END(ctx)
}

extern "C" int gf_mom_update(gf_ctx* ctx, gf_field* P, const gf_field* U, double eps, double beta) {
  API_BEGIN
  need(ctx && U && P, "gf_mom_update: null argument");
  need_ctx(ctx, U);
  need_ctx(ctx, P);
  need(std::isfinite(eps), "gf_mom_update: the momentum step size must be finite");
  need(std::isfinite(beta), "gf_mom_update: beta must be finite");
  wilson_force_coef(ctx, U, P, eps * (-(1.0 / 3.0) * (0.5 * beta)), 1.0);
  API_END(ctx)
}

extern "C" int gf_link_update(gf_ctx* ctx, gf_field* U, const gf_field* P, double eps, int reunit) {
  API_BEGIN
  need(ctx && U && P, "gf_link_update: null argument");
  need_ctx(ctx, U);
  need_ctx(ctx, P);
  need(std::isfinite(eps), "gf_link_update: the gauge-field step size must be finite");
  link_update(ctx, U, P, eps, reunit, nullptr);
  API_END(ctx)
}

extern "C" int gf_hamiltonian(gf_ctx* ctx, const gf_field* U, const gf_field* P, const gf_md_params* prm,
                              double* out) {
  API_BEGIN
  need(ctx && U && P && out, "gf_hamiltonian: null argument");
  need_ctx(ctx, U);
  need_ctx(ctx, P);
  check_md(prm);
  need_kind(U, GF_LINK64, "gf_hamiltonian: U");
  need_kind(P, GF_MOM64, "gf_hamiltonian: P");
  *out = hamiltonian(ctx, U, P, prm);
  API_END(ctx)
}

extern "C" int gf_md_mom_update(gf_ctx* ctx, gf_field* P, const gf_field* U, double eps, const gf_md_params* prm) {
  API_BEGIN
  need(ctx && U && P, "gf_md_mom_update: null argument");
  need_ctx(ctx, U);
  need_ctx(ctx, P);
  check_md(prm);
  need_kind(U, GF_LINK64, "gf_md_mom_update: U");
  need_kind(P, GF_MOM64, "gf_md_mom_update: P");
  need(std::isfinite(eps), "gf_md_mom_update: the momentum step size must be finite");
  gf_field* U32 = nullptr;
  if (prm->precision == GF_MIXED) {
    if (!ctx->w_link32) ctx->w_link32 = field_new(ctx, GF_LINK32);
    U32 = ctx->w_link32;
    link64_to_32(ctx, U32, U);
  }
  mom_update(ctx, P, U, U32, eps, prm);
  API_END(ctx)
}

extern "C" int gf_md_link_update(gf_ctx* ctx, gf_field* U, const gf_field* P, double eps, const gf_md_params* prm) {
  API_BEGIN
  need(ctx && U && P, "gf_md_link_update: null argument");
  need_ctx(ctx, U);
  need_ctx(ctx, P);
  check_md(prm);
  need_kind(U, GF_LINK64, "gf_md_link_update: U");
  need_kind(P, GF_MOM64, "gf_md_link_update: P");
  need(std::isfinite(eps), "gf_md_link_update: the gauge-field step size must be finite");
  link_update(ctx, U, P, eps, prm->reunitarize, nullptr, prm->precision != GF_FP64);
  API_END(ctx)
}

extern "C" int gf_md_trajectory(gf_ctx* ctx, gf_field* U, gf_field* P, const gf_md_params* prm, double out[3]) {
  API_BEGIN
  need(ctx && U && P && out, "gf_md_trajectory: null argument");
  need_ctx(ctx, U);
  need_ctx(ctx, P);
  check_md(prm);
  MDResult r = md_run(ctx, U, P, prm);
  out[0] = r.H0;
  out[1] = r.H1;
  out[2] = r.H1 - r.H0;
  if (!std::isfinite(out[2])) {
    vcache_clear(ctx);
    throw gf_error(GF_ENAN, "gf_md_trajectory: Delta H is not finite");
  }
  vcache_set(ctx, prm, 0, r.h1, r.V1);
  vcache_set(ctx, prm, 1, r.h0, r.V0);
  API_END(ctx)
}

extern "C" int gf_hmc_update(gf_ctx* ctx, gf_field* U, gf_field* P, const gf_md_params* prm, uint64_t seed,
                             uint64_t sweep, double unif, double out[4]) {
  API_BEGIN
  need(ctx && U && P && out, "gf_hmc_update: null argument");
  need_ctx(ctx, U);
  need_ctx(ctx, P);
  check_md(prm);
  need(unif >= 0.0 && unif < 1.0, "gf_hmc_update: unif must be in [0,1)");
  need_kind(U, GF_LINK64, "gf_hmc_update: U");
  if (!ctx->w_link64) ctx->w_link64 = field_new(ctx, GF_LINK64);
  copy_field(ctx, ctx->w_link64, U);
  gaussian_momenta(ctx, P, seed, sweep);
  MDResult r = md_run(ctx, U, P, prm);
  double h[3] = {r.H0, r.H1, r.H1 - r.H0};
  bool finite = std::isfinite(h[2]);
  bool accept = finite && (h[2] <= 0.0 || unif < std::exp(-h[2]));
  if (!accept) copy_field(ctx, U, ctx->w_link64);
  GF_CUDA(cudaStreamSynchronize(ctx->stream));
  vcache_set(ctx, prm, 0, r.h1, r.V1);
  vcache_set(ctx, prm, 1, r.h0, r.V0);
  out[0] = h[0];
  out[1] = h[1];
  out[2] = h[2];
  out[3] = accept ? 1.0 : 0.0;
  if (!finite) throw gf_error(GF_ENAN, "gf_hmc_update: Delta H is not finite; configuration restored");
  API_END(ctx)
}

// ---------------------------------------------------------------------------
// gradient flow: Luescher RK3 (flow!, src/smearing/gradientflow.jl:171-238)
//   W1 = exp(-eps/4 F0) U
//   W2 = exp(-8eps/9 F1 + 17eps/36 F0) W1
//   U  = exp(-3eps/4 F2 + 8eps/9 F1 - 17eps/36 F0) W2
// with F = TA(U V^dag) in su(3) coefficients. One coefficient field G holds
// the running combination: G = 17eps/36 F0 -> G - 8eps/9 F1 -> -G - 3eps/4 F2.
// ---------------------------------------------------------------------------
extern "C" int gf_flow_force(gf_ctx* ctx, const gf_field* U, gf_field* F, double factor) {
  API_BEGIN
  need(ctx && U && F, "gf_flow_force: null argument");
  need_ctx(ctx, U);
  need_ctx(ctx, F);
  need_kind(F, GF_MOM64, "gf_flow_force: F");
  flow_force(ctx, U, F, factor, 1.0);
  API_END(ctx)
}

// RK3 Wilson-flow steps (flow!, src/smearing/gradientflow.jl:171-238) in fp64
// or, df, with the force and the exponentials in double-float arithmetic on
// the fp64 fields
static void flow_steps(gf_ctx* ctx, gf_field* U, double eps, int nsteps, bool df) {
  if (!ctx->w_link64) ctx->w_link64 = field_new(ctx, GF_LINK64);
  if (!ctx->w_link64b) ctx->w_link64b = field_new(ctx, GF_LINK64);
  if (!ctx->w_mom[0]) ctx->w_mom[0] = field_new(ctx, GF_MOM64);
  gf_field* W1 = ctx->w_link64;
  gf_field* W2 = ctx->w_link64b;
  gf_field* G = ctx->w_mom[0];
  const double c0 = 17.0 * eps / 36.0;
  for (int n = 0; n < nsteps; ++n) {
    flow_force(ctx, U, G, c0, 0.0, df);                 // G = 17eps/36 F0
    exp_mom_links(ctx, W1, G, -9.0 / 17.0, U, df);      // W1 = exp(-eps/4 F0) U
    flow_force(ctx, W1, G, -8.0 * eps / 9.0, 1.0, df);  // G = 17eps/36 F0 - 8eps/9 F1
    exp_mom_links(ctx, W2, G, 1.0, W1, df);             // W2 = exp(G) W1
    flow_force(ctx, W2, G, -0.75 * eps, -1.0, df);      // G = -G - 3eps/4 F2
    exp_mom_links(ctx, U, G, 1.0, W2, df);              // U = exp(G) W2
  }
}

extern "C" int gf_flow(gf_ctx* ctx, gf_field* U, double eps, int nsteps) {
  return gf_flow_precision(ctx, U, eps, nsteps, GF_FP64);
}

extern "C" int gf_flow_precision(gf_ctx* ctx, gf_field* U, double eps, int nsteps, int precision) {
  API_BEGIN
  need(ctx && U, "gf_flow: null argument");
  need_ctx(ctx, U);
  need_kind(U, GF_LINK64, "gf_flow: U");
  need(std::isfinite(eps) && eps != 0.0, "gf_flow: eps must be finite and nonzero");
  need(nsteps >= 0, "gf_flow: nsteps must be nonnegative");
  need(precision == GF_FP64 || precision == GF_DFLOAT, "gf_flow: precision must be GF_FP64 or GF_DFLOAT");
  flow_steps(ctx, U, eps, nsteps, precision == GF_DFLOAT);
  API_END(ctx)
}

// The same RK3 steps with the force TA(U dS/dU) of the plaquette + rectangle
// action (Gradientflow_general); (c_plaq, c_rect) = (1, 0) is the Wilson flow.
extern "C" int gf_flow_loops(gf_ctx* ctx, gf_field* U, double eps, int nsteps, double c_plaq, double c_rect) {
  API_BEGIN
  need(ctx && U, "gf_flow_loops: null argument");
  need_ctx(ctx, U);
  need_kind(U, GF_LINK64, "gf_flow_loops: U");
  need(std::isfinite(eps) && eps != 0.0, "gf_flow_loops: eps must be finite and nonzero");
  need(nsteps >= 0, "gf_flow_loops: nsteps must be nonnegative");
  need(std::isfinite(c_plaq) && std::isfinite(c_rect), "gf_flow_loops: the coefficients must be finite");
  if (!ctx->w_link64) ctx->w_link64 = field_new(ctx, GF_LINK64);
  if (!ctx->w_link64b) ctx->w_link64b = field_new(ctx, GF_LINK64);
  if (!ctx->w_mom[0]) ctx->w_mom[0] = field_new(ctx, GF_MOM64);
  gf_field* W1 = ctx->w_link64;
  gf_field* W2 = ctx->w_link64b;
  gf_field* G = ctx->w_mom[0];
  const double c0 = 17.0 * eps / 36.0;
  const double c1 = -8.0 * eps / 9.0;
  const double c2 = -0.75 * eps;
  for (int n = 0; n < nsteps; ++n) {
    loops_force_coef(ctx, U, G, c0 * c_plaq, c0 * c_rect, 0.0);    // G = 17eps/36 F0
    exp_mom_links(ctx, W1, G, -9.0 / 17.0, U);                    // W1 = exp(-eps/4 F0) U
    loops_force_coef(ctx, W1, G, c1 * c_plaq, c1 * c_rect, 1.0);   // G += -8eps/9 F1
    exp_mom_links(ctx, W2, G, 1.0, W1);                           // W2 = exp(G) W1
    loops_force_coef(ctx, W2, G, c2 * c_plaq, c2 * c_rect, -1.0);  // G = -G - 3eps/4 F2
    exp_mom_links(ctx, U, G, 1.0, W2);                            // U = exp(G) W2
  }
  API_END(ctx)
}

// ---------------------------------------------------------------------------
// instrumentation
// ---------------------------------------------------------------------------
extern "C" int gf_prof_enable(gf_ctx* ctx, int on) {
  API_BEGIN
  need(ctx != nullptr, "gf_prof_enable: null context");
  if (on && !ctx->prof_ev) {
    ctx->prof_ev = new cudaEvent_t[2 * GF_PROF_CAP];
    for (int i = 0; i < 2 * GF_PROF_CAP; ++i) GF_CUDA(cudaEventCreate(&ctx->prof_ev[i]));
  }
  if (ctx->prof_on) prof_flush(ctx);
  ctx->prof_on = on ? 1 : 0;
  if (on) {
    ctx->prof_n = 0;
    for (int k = 0; k < GF_K_COUNT; ++k) {
      ctx->prof_ms[k] = 0.0;
      ctx->prof_cnt[k] = 0;
    }
  }
  API_END(ctx)
}

extern "C" int gf_prof_read(gf_ctx* ctx, int kernel_class, double* total_ms, long long* launches) {
  API_BEGIN
  need(ctx && total_ms && launches, "gf_prof_read: null argument");
  need(kernel_class >= 0 && kernel_class < GF_K_COUNT, "gf_prof_read: unknown kernel class");
  if (ctx->prof_on) prof_flush(ctx);
  *total_ms = ctx->prof_ms[kernel_class];
  *launches = ctx->prof_cnt[kernel_class];
  API_END(ctx)
}

extern "C" int gf_launch_count(long long* out) {
  if (!out) return GF_EINVAL;
  *out = g_launches.load();
  return GF_OK;
}

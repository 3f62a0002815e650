// Internal declarations shared by the translation units of libgfgb300.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <stdexcept>
#include "lattice.cuh"
#include "../../include/gaugefields_gb300.h"

// Error carried from the CUDA layer to the C-ABI wrappers, which turn it into
// a status code and keep the message for gf_last_error().
struct gf_error : std::runtime_error {
  int code;
  gf_error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define GF_CUDA(call)                                                                    \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      throw gf_error(GF_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_));     \
  } while (0)

namespace gf {
// process-wide count of kernels launched by this library
void count_launch();
}
#define GF_CHECK_LAUNCH()          \
  do {                             \
    gf::count_launch();            \
    GF_CUDA(cudaGetLastError());   \
  } while (0)

#define GF_PROF_CAP 4096

// Stack precision with double-float arithmetic: the GF_DFLOAT form, and the
// Hamiltonian of the mixed form (forward only).
#define GF_PREC_DF GF_DFLOAT

// Internal field kinds of double-float stacks: 18-real links and general
// matrices stored as fp32 hi/lo pairs (one float4 per complex element, the
// size of GF_LINK64). They never cross the C-ABI: the API converts at the
// boundary.
#define GF_LINKDF 101
#define GF_MATDF 102

struct gf_field {
  gf_ctx* ctx;
  int kind;
  void* ptr;
  size_t bytes;
  int owned;
};

struct gf_ctx {
  int device;
  int sm_count;  // streaming multiprocessors of the device (grid sizing)
  gf::Geom geom;
  cudaStream_t stream;
  int own_stream;
  std::string err;
  // deterministic reductions: per-block partial sums and a pinned result slot
  double* d_partials;
  int partial_cap;
  double* d_result;
  double* h_result;
  // work fields of the MD / flow drivers, allocated on first use
  gf_field* w_link64;     // backup / W1 of the flow
  gf_field* w_link64b;    // W2 of the flow
  gf_field* w_mom[4];     // F0, F1, F2, Ftmp of the RK3 flow (fp64 coefficients)
  gf_field* w_link32;     // fp32 12-real shadow of the thin links (mixed form)
  gf_field* w_linkdf;     // double-float-native copy of the thin links (double-float rectangle force)
  // Two scratch blocks of one fp64 link field each, shared by the mixed form's
  // internal stacks: the Hamiltonian's double-float level buffers and the
  // force adjoint's Z, Dp, D[0], D[1] (fp32). They are never live together:
  // the potential runs before and after the MD steps, the adjoint within them.
  void* arena[2];
  gf_stout* w_stout64;    // stout workspace, fp64
  gf_stout* w_stout32;    // stout workspace, fp32
  gf_stout* w_stoutdf;    // double-float stack: mixed-form Hamiltonian (forward only) or GF_DFLOAT
  int w_stout_nlev;
  double w_stout_rho[GF_MAX_STOUT];
  // potentials of the configurations the last MD call started and ended on,
  // keyed by a 64-bit hash of their fp64 links and the action parameters
  unsigned long long* d_hash;
  unsigned long long* h_hash;
  struct {
    int valid;
    unsigned long long hash;
    double V, beta, c_rect;
    int nstout, precision;
    double rho[GF_MAX_STOUT];
  } vc[2];
  // staging buffer for host transfers in the reference layout (grown on demand)
  void* d_stage;
  size_t stage_bytes;
  // per-kernel CUDA-event timing on the context's stream (gf_prof_*)
  int prof_on;
  int prof_n;
  cudaEvent_t* prof_ev;  // 2 * GF_PROF_CAP events
  int prof_kid[GF_PROF_CAP];
  double prof_ms[GF_K_COUNT];
  long long prof_cnt[GF_K_COUNT];
};

struct gf_stout {
  gf_ctx* ctx;
  int nlev;
  double rho[GF_MAX_STOUT];
  int precision;  // GF_FP64, GF_MIXED or GF_PREC_DF
  int store;      // 1: keep C of every level from the forward pass
  int fwd_only;   // 1: no adjoint buffers (a Hamiltonian-only stack)
  gf_field* lev_in[GF_MAX_STOUT + 1];  // lev_in[0] aliases the thin links
  gf_field* C[GF_MAX_STOUT];
  gf_field* Z;   // dS/dC of the level being pulled back
  gf_field* Dp;  // local part of dS/dU (alpha term + (Y C)^dag)
  gf_field* D[2];
  int have_forward;
};

namespace gf {

size_t field_bytes(const Geom& g, int kind);
gf_field* field_new(gf_ctx* ctx, int kind);
// a non-owning field of `kind` over scratch block `which` at byte offset `off`
gf_field* arena_view(gf_ctx* ctx, int which, size_t off, int kind);
void field_delete(gf_field* f);

inline int blocks_for(int n, int bs) { return (n + bs - 1) / bs; }

// CUDA-event timing of one kernel launch (no-op unless gf_prof_enable is on)
void prof_begin(gf_ctx* ctx, int kid);
void prof_end(gf_ctx* ctx, int kid);
void prof_flush(gf_ctx* ctx);
struct ProfScope {
  gf_ctx* c;
  int k;
  ProfScope(gf_ctx* c_, int k_) : c(c_), k(k_) { prof_begin(c, k); }
  ~ProfScope() { prof_end(c, k); }
};

// message returned by gf_last_error(NULL) for calls without a context
void set_global_error(const std::string& m);

// ---- reductions (gf_fields.cu) ----
// Deterministic two-stage sum of per-site doubles produced by a kernel that
// writes one partial per block; returns the total on the host.
double finish_reduction(gf_ctx* ctx, int nblocks);
double kinetic(gf_ctx* ctx, const gf_field* P);
// order-independent 64-bit hash of a field's bytes (sum of mixed words)
unsigned long long field_hash(gf_ctx* ctx, const gf_field* f);

// ---- field plumbing (gf_fields.cu) ----
void upload_links(gf_ctx* ctx, gf_field* U, const double* host);
void download_links(gf_ctx* ctx, const gf_field* U, double* host);
void upload_mom(gf_ctx* ctx, gf_field* P, const double* host);
void download_mom(gf_ctx* ctx, const gf_field* P, double* host);
void cold_start(gf_ctx* ctx, gf_field* U);
void hot_start(gf_ctx* ctx, gf_field* U, uint64_t seed);
void gaussian_momenta(gf_ctx* ctx, gf_field* P, uint64_t seed, uint64_t sweep);
void copy_field(gf_ctx* ctx, gf_field* dst, const gf_field* src);
void zero_field(gf_ctx* ctx, gf_field* f);
void mom_axpy(gf_ctx* ctx, gf_field* y, double a, const gf_field* x);  // y += a x
void field_axpy(gf_ctx* ctx, gf_field* y, double a, const gf_field* x);  // y += a x, fp64 fields of one kind
void mom_scale(gf_ctx* ctx, gf_field* y, double a);                      // y *= a

// ---- Wilson action pieces (gf_wilson.cu) ----
double plaquette_sum(gf_ctx* ctx, const gf_field* U, bool df = false);  // sum_x sum_{mu<nu} Re tr P
// mean over the t = 0 slice of tr prod_t U_T: out = {Re, Im}
void polyakov_loop(gf_ctx* ctx, const gf_field* U, double out[2]);
void staple_up(gf_ctx* ctx, const gf_field* U, int mu, gf_field* V);  // construct_staple! (mu field slot)
// P <- keep * P + coef * TA-coefficients(U_mu * S_mu), S = sum of the six
// staples (dS/dU order); keep = 0 overwrites P without reading it.
void wilson_force_coef(gf_ctx* ctx, const gf_field* U, gf_field* P, double coef, double keep, bool df = false);

// ---- rectangle loops (gf_rect.cu) ----
double rectangle_sum(gf_ctx* ctx, const gf_field* U);  // sum_x sum_{mu<nu} Re tr (R1x2 + R2x1)
// P <- keep * P + TA-coefficients(U_mu (cp S_mu + cr R_mu)), S the six
// plaquette staples and R the eighteen rectangle staples of U_mu.
void loops_force_coef(gf_ctx* ctx, const gf_field* U, gf_field* P, double cp, double cr, double keep,
                      bool df = false);
// D = cp S + cr R (plaquette and rectangle staples) on a stack's top level:
// LINK64 -> MAT64, LINK32 -> MAT32, LINKDF -> MATDF (double-float)
void loops_dsdu(gf_ctx* ctx, const gf_field* Ubar, gf_field* D, double cp, double cr);
// P <- keep P + coef c(U S), S the six plaquette staples, as a double-float
// table loop of fixed-grid products on a double-float-native copy of U
void plaquette_force_df(gf_ctx* ctx, const gf_field* U, gf_field* P, double coef, double keep);

// ---- link update (gf_update.cu) ----
// U <- exp(i eps P) U, optional re-unitarisation, optional fp32 shadow copy.
// df: double-float arithmetic on the fp32 pipes (the mixed form), else fp64.
void link_update(gf_ctx* ctx, gf_field* U, const gf_field* P, double eps, int reunit, gf_field* shadow32,
                 bool df = false);
// W = exp(i a P) U (fp64, or double-float arithmetic on the fp64 fields)
void exp_mom_links(gf_ctx* ctx, gf_field* W, const gf_field* P, double a, const gf_field* U, bool df = false);
void reunitarize_links(gf_ctx* ctx, gf_field* U);
void link64_to_32(gf_ctx* ctx, gf_field* dst, const gf_field* src);

// ---- stout (gf_stout.cu) ----
void stout_forward(gf_ctx* ctx, gf_stout* st, const gf_field* U, gf_field* Uout);
// Pull dS/dUbar back to the thin links. If dSdUbar is null the top-level
// derivative is taken from the Wilson action (coefficient beta/2 per staple)
// on the smeared links. If P is non-null the thin-link result is turned into
// the MD force and added as P += eps * F; otherwise it is written to dSdU.
// dsdrho (optional, nlev entries): dS/drho of every level
void stout_backward(gf_ctx* ctx, gf_stout* st, const gf_field* dSdUbar, double beta, gf_field* dSdU,
                    gf_field* P, double eps, double* dsdrho = nullptr);
const gf_field* stout_top(const gf_stout* st);

// ---- flow (gf_flow.cu) ----
// F <- keep * F + factor * TA-coefficients(U_mu V_mu^dag), V = six-staple sum
// (add_force!, plaqonly)
void flow_force(gf_ctx* ctx, const gf_field* U, gf_field* F, double factor, double keep, bool df = false);

}  // namespace gf

/*
 * gaugefields_gb300.h -- C-ABI of libgfgb300.so, the GB300 (sm_103a) backend
 * for the SU(3) gauge-link hot path of Gaugefields.jl.
 *
 * Every entry point returns an int status (GF_OK = 0, negative on error) and
 * never lets a C++ exception cross the ABI; gf_last_error() returns the text
 * of the last failure on a context. Plain pointers and sizes only.
 *
 * Host arrays use the reference's layouts:
 *   links   : complex128 (3,3,NX,NY,NZ,NT) column-major per direction, the four
 *             directions contiguous (Gaugefields_4D_nowing.U, or the
 *             LatticeMatrix interior of Gaugefields_4D_MPILattice without halo)
 *             -> 4*9*V complex = 72*V doubles (re,im interleaved)
 *   momenta : Float64 (8,NX,NY,NZ,NT) per direction, contiguous over the four
 *             directions (TA_Gaugefields_4D_serial.a) -> 32*V doubles
 * Device storage is the library's own (even/odd site-major SoA) and is opaque.
 *
 * Reference citations are paths inside the Gaugefields.jl source tree.
 */
#ifndef GAUGEFIELDS_GB300_H
#define GAUGEFIELDS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define GF_OK 0
#define GF_EINVAL (-1)  /* bad argument: ArgumentError in the reference */
#define GF_ENOMEM (-2)  /* device allocation failed */
#define GF_ECUDA (-3)   /* CUDA runtime error */
#define GF_ENAN (-4)    /* non-finite value detected (e.g. Delta H) */
#define GF_ESTATE (-5)  /* call out of order (e.g. backward before forward) */

/* field kinds */
#define GF_LINK64 1 /* SU(3) links, complex128, 18 reals per link */
#define GF_LINK32 2 /* SU(3) links, fp32 two-row 12-real storage */
#define GF_MOM64 3  /* su(3) momenta / forces, 8 fp64 coefficients per link */
#define GF_MAT64 4  /* general 3x3 complex per link, fp64 (dS/dU, staples) */
#define GF_MAT32 5  /* general 3x3 complex per link, fp32 */

/* precision of the force / stout path */
#define GF_FP64 0  /* plain form: fp64 throughout */
#define GF_MIXED 1 /* fp32 force and stout (12-real links), fp64 H / updates */
#define GF_DFLOAT 2 /* force, stout forward/adjoint and link updates in
                       double-float arithmetic (fp32 pairs, ~48-bit
                       significand, on the fp32 pipes) on fp64 links; fp64
                       H, Delta H and Metropolis. No counterpart in the
                       reference: a third form between GF_FP64 and GF_MIXED */

/* integrators of the MD driver (molecular_dynamics.jl:604-616); GF_OMELYAN is
 * the second-order minimum-norm PQPQP scheme of the reference's custom
 * integrator example OmelyanPQP(lambda) (docs/src/hmc.md:250-270) */
#define GF_QPQ 0
#define GF_PQP 1
#define GF_OMELYAN 2

#define GF_MAX_STOUT 4

typedef struct gf_ctx gf_ctx;
typedef struct gf_field gf_field;
typedef struct gf_stout gf_stout;

/* MD parameters: md_driver(U, action; steps, trajectory_length, integrator)
 * (src/molecular_dynamics.jl:440-483) with the GaugeAction
 * push!(action, beta/2, plaq U plaq^dag), optionally a rectangle term
 * push!(action, c_rect, rect U rect^dag), and an optional stout stack
 * (STOUT_Layer, src/smearing/stout_fast.jl:6-121). */
typedef struct gf_md_params {
  double beta;           /* Wilson coupling */
  double tau;            /* trajectory_length, finite and nonzero */
  int steps;             /* > 0 */
  int integrator;        /* GF_QPQ, GF_PQP or GF_OMELYAN */
  int precision;         /* GF_FP64, GF_MIXED or GF_DFLOAT */
  int nstout;            /* 0 .. GF_MAX_STOUT smearing levels */
  double rho[GF_MAX_STOUT];
  int reunitarize;       /* re-unitarise links after every link update */
  int stout_recompute;   /* 1: the adjoint recomputes each level's C_mu from the
                            stored level input instead of keeping it from the
                            forward pass (less memory, more flops) */
  double lambda;         /* Omelyan parameter (GF_OMELYAN only) */
  double c_rect;         /* coefficient of the rectangle loops,
                            push!(action, c_rect, rect U rect') (make_rect,
                            src/autostaples/wilsonloops.jl:304-330); 0 for the
                            plain Wilson action. Every precision form; with
                            stout levels the loops are those of the smeared
                            links (dS/dUbar = beta/2 S + c_rect R on the top
                            level, back-propagated by the stout adjoint). */
} gf_md_params;

/* ---- context ------------------------------------------------------------ */
/* Replaces the lattice/PE bookkeeping of Gaugefields_4D_MPILattice
 * (src/4D/mpi_jacc/gaugefields_4D_MPILattice.jl:34-121). L = {NX,NY,NZ,NT};
 * NX must be even (even/odd site order); one CUDA device per context. */
int gf_ctx_create(const int L[4], int device, gf_ctx** out);
int gf_ctx_destroy(gf_ctx* ctx);
/* Run all work of the context on a caller-owned cudaStream_t (NULL restores
 * the context's own stream). */
int gf_ctx_set_stream(gf_ctx* ctx, void* cuda_stream);
int gf_ctx_synchronize(gf_ctx* ctx);
const char* gf_last_error(const gf_ctx* ctx);
int gf_ctx_volume(const gf_ctx* ctx, int64_t* out);

/* ---- fields ------------------------------------------------------------- */
/* similar(U[1]) / initialize_TA_Gaugefields(U) (AbstractGaugefields.jl,
 * TA_Gaugefields.jl:140-160): allocate a device field of the given kind. */
int gf_field_alloc(gf_ctx* ctx, int kind, gf_field** out);
int gf_field_free(gf_field* f);
int gf_field_kind(const gf_field* f, int* kind);
int gf_field_bytes(const gf_field* f, size_t* bytes);
/* Device pointer of a field (for CUDA.jl / torch interop, library layout). */
int gf_field_device_ptr(const gf_field* f, void** ptr);
/* substitute_U! (gaugefields_4D_MPILattice.jl:509-611): dst <- src. LINK64 ->
 * LINK32 converts to the fp32 12-real form; other kinds must match. */
int gf_field_copy(gf_ctx* ctx, gf_field* dst, const gf_field* src);
/* clear_U! */
int gf_field_zero(gf_ctx* ctx, gf_field* f);
/* add_U!(c, t, a) (src/4D/mpi_jacc/gaugefields_4D_MPILattice.jl:739-745):
 * y += a x for fp64 fields of one kind (LINK64, MAT64 or MOM64). */
int gf_field_axpy(gf_ctx* ctx, gf_field* y, double a, const gf_field* x);

/* ---- host transfer in the reference layout ----------------------------- */
/* Upload/download link fields (LINK64 or MAT64) and momenta (MOM64); the
 * round trip is exact. Replaces getindex/setindex!/substitute_U! host access
 * (gaugefields_4D_MPILattice.jl:166-199) and the rank-0 gather of API.jl:531. */
int gf_upload_links(gf_ctx* ctx, gf_field* U, const double* host);
int gf_download_links(gf_ctx* ctx, const gf_field* U, double* host);
int gf_upload_mom(gf_ctx* ctx, gf_field* P, const double* host);
int gf_download_mom(gf_ctx* ctx, const gf_field* P, double* host);

/* ---- starts and random fields ------------------------------------------ */
/* gauge_configuration(L; start=:cold) (API.jl:178-251): all links = 1. */
int gf_cold_start(gf_ctx* ctx, gf_field* U);
/* gauge_configuration(L; start=:hot, seed): Haar-random SU(3) per link from a
 * Gaussian 3x3 complex matrix (re, im ~ N(0,1/2)), Gram-Schmidt of the rows
 * and the determinant phase divided out; counter-based Philox4x32-10 keyed by
 * seed, so the start is independent of the launch shape. */
int gf_hot_start(gf_ctx* ctx, gf_field* U, uint64_t seed);
/* gaussian_momenta!(P; seed, sweep) (API.jl:341-368): p_a ~ N(0,1). */
int gf_gaussian_momenta(gf_ctx* ctx, gf_field* P, uint64_t seed, uint64_t sweep);
/* P <- a P on a MOM64 field: gaussian_momenta!(P; sigma) (API.jl:341-368)
 * draws unit-variance momenta and scales them by sigma. */
int gf_mom_scale(gf_ctx* ctx, gf_field* P, double a);
/* normalize_U! (AbstractGaugefields.jl:3378-3457) on every link. */
int gf_reunitarize(gf_ctx* ctx, gf_field* U);

/* ---- measurements ------------------------------------------------------- */
/* calculate_Plaquette(U, temp, staple) (AbstractGaugefields.jl:2684-2699):
 * sum_mu Re tr(U_mu V_mu^dag)/2 = sum_x sum_{mu<nu} Re tr P_munu(x).
 * measure_plaquette divides by 6*V*3 (API.jl:395-404). Deterministic. */
int gf_plaquette(gf_ctx* ctx, const gf_field* U, double* out);
/* calculate_Polyakov_loop(U, temp1, temp2) (AbstractGaugefields.jl:
 * 2929-2956): the mean over the sites of the t = 0 slice of
 * tr(U_T(x,0) U_T(x,1) ... U_T(x,NT-1)); out[0] = Re, out[1] = Im.
 * measure_polyakov_loop (API.jl:412-417) divides by 3. Deterministic. */
int gf_polyakov_loop(gf_ctx* ctx, const gf_field* U, double* out);
/* md_potential(::GaugeAction) (molecular_dynamics.jl:247) for the Wilson
 * action beta/2 * (plaq U plaq^dag): -(beta/3) sum Re tr P. */
int gf_action(gf_ctx* ctx, const gf_field* U, double beta, double* out);
/* P*P (TA_gaugefields_4D_serial.jl:106-129): sum of p_a^2. */
int gf_kinetic(gf_ctx* ctx, const gf_field* P, double* out);
/* construct_staple!(V, U, mu, temp) (AbstractGaugefields.jl:2873-2923): the
 * up staples sum_{nu != mu} U_nu(x) U_mu(x+nu) U_nu(x+mu)^dag into direction
 * slot mu (0-based) of the MAT64/LINK64 field V. */
int gf_staple(gf_ctx* ctx, const gf_field* U, int mu, gf_field* V);
/* evaluate_GaugeAction over the rectangle loops of make_rect
 * (GaugeActions.jl:132-142, wilsonloops.jl:304-330) without the conjugates:
 * sum_x sum_{mu<nu} Re tr (R^{1x2}_{mu nu}(x) + R^{2x1}_{mu nu}(x)), the loops
 * (mu,1),(nu,2),(mu,-1),(nu,-2) and (mu,2),(nu,1),(mu,-2),(nu,-1). fp64,
 * deterministic. */
int gf_rectangle(gf_ctx* ctx, const gf_field* U, double* out);
/* md_potential(::GaugeAction) (molecular_dynamics.jl:247) of
 * push!(action, c_plaq, plaq U plaq') and push!(action, c_rect, rect U rect')
 * (e.g. Iwasaki: c_plaq = beta (1 - 8 c1)/2, c_rect = beta c1/2, c1 = -0.331):
 * -(2/3) (c_plaq sum Re tr P + c_rect sum Re tr R). fp64 links (LINK64). */
int gf_action_loops(gf_ctx* ctx, const gf_field* U, double c_plaq, double c_rect, double* out);

/* ---- molecular dynamics ------------------------------------------------- */
/* md_force!(F, ::GaugeAction, U, ws) (molecular_dynamics.jl:251-267):
 * F_mu = -(1/3) TA(U_mu dS/dU_mu), dS/dU_mu = beta/2 * sum of six staples. */
int gf_force(gf_ctx* ctx, const gf_field* U, double beta, gf_field* F);
/* md_force! of the plaquette + rectangle action of gf_action_loops
 * (calc_dSdUμ!, GaugeActions.jl:95-123): F_mu = -(1/3) TA(U_mu dS/dU_mu),
 * dS/dU_mu = c_plaq * (6 plaquette staples) + c_rect * (18 rectangle staples).
 * fp64, one fused kernel. */
int gf_force_loops(gf_ctx* ctx, const gf_field* U, double c_plaq, double c_rect, gf_field* F);
/* update_momenta!(P, U, eps, driver) (molecular_dynamics.jl:539-551):
 * P += eps * F(U), fused in one kernel. */
int gf_mom_update(gf_ctx* ctx, gf_field* P, const gf_field* U, double eps, double beta);
/* update_gaugefields!(U, P, eps, driver) (molecular_dynamics.jl:513-531):
 * U_mu <- exp(i eps P_mu) U_mu (Cayley-Hamilton), reunit != 0 re-unitarises. */
int gf_link_update(gf_ctx* ctx, gf_field* U, const gf_field* P, double eps, int reunit);
/* md_hamiltonian (molecular_dynamics.jl:494-505): potential (on the smeared
 * links when nstout > 0) + P*P/2, in fp64. */
int gf_hamiltonian(gf_ctx* ctx, const gf_field* U, const gf_field* P, const gf_md_params* prm, double* out);
/* update_momenta!(P, U, eps, driver) and update_gaugefields!(U, P, eps,
 * driver) (molecular_dynamics.jl:539-551, :513-531) with the driver's action,
 * smearing and precision, as one step of gf_md_trajectory takes them: the
 * building blocks of custom integrators (md_step! of user types, :593-602).
 * gf_md_link_update re-unitarises when prm->reunitarize != 0. */
int gf_md_mom_update(gf_ctx* ctx, gf_field* P, const gf_field* U, double eps, const gf_md_params* prm);
int gf_md_link_update(gf_ctx* ctx, gf_field* U, const gf_field* P, double eps, const gf_md_params* prm);
/* md_trajectory!(U, P, driver) (molecular_dynamics.jl:712-730): one QPQ/PQP
 * trajectory. out[0..2] = initial H, final H, Delta H. prm->precision selects
 * the plain fp64, the mixed or the double-float form. */
int gf_md_trajectory(gf_ctx* ctx, gf_field* U, gf_field* P, const gf_md_params* prm, double out[3]);
/* One HMC update of the application loop (docs/src/hmc.md:22-81): momenta
 * refresh (seed, sweep), md_trajectory!, Metropolis test with the uniform
 * `unif` in [0,1), rejection restores U. out = {H0, H1, dH, accepted}. */
int gf_hmc_update(gf_ctx* ctx, gf_field* U, gf_field* P, const gf_md_params* prm, uint64_t seed,
                  uint64_t sweep, double unif, double out[4]);

/* ---- stout smearing ----------------------------------------------------- */
/* STOUT_Layer stack (stout_fast.jl:6-121) / CovNeuralnet of nlev plaquette
 * layers with coefficients rho[0..nlev-1]. precision GF_FP64, GF_MIXED
 * (fp32 12-real links) or GF_DFLOAT (fp64 links and MAT64 derivatives,
 * double-float arithmetic); store != 0 keeps C_mu of every level from the
 * forward pass, store == 0 recomputes it in the backward pass. */
int gf_stout_create(gf_ctx* ctx, int nlev, const double* rho, int precision, int store, gf_stout** out);
int gf_stout_destroy(gf_stout* st);
/* calc_smearedU / apply_layer! -> forward! (stout_fast.jl:250-275):
 * Ubar_mu = exp(TA(C_mu U_mu^dag)) U_mu per level. Uout may be NULL. */
int gf_stout_forward(gf_ctx* ctx, gf_stout* st, const gf_field* U, gf_field* Uout);
/* back_prop (Abstractsmearing.jl:316-411) -> layer_pullback! ->
 * backward_dSdUαUβρ_add! (stout_fast.jl:317-408): dS/dU on the thin links
 * from dS/dUbar (MAT64/MAT32 in the precision of the stack). */
int gf_stout_backward(gf_ctx* ctx, gf_stout* st, const gf_field* dSdUbar, gf_field* dSdU);
/* parameter_derivatives / get_parameter_derivatives (Abstractsmearing.jl:
 * 416-436, 505; the rho part of backward_dSdUαUβρ_add!, stout_fast.jl:
 * 371-386): forward on U, then the adjoint from dS/dUbar (MAT64, or MAT32
 * for a GF_MIXED stack), writing dS/drho of every level to dSdrho[0..nlev-1]:
 * dS/drho_l = 2 Re sum tr(Z_l S_l^dag), Z_l = dS/dC_l, C_l = rho_l S_l^dag. */
int gf_stout_param_derivatives(gf_ctx* ctx, gf_stout* st, const gf_field* U, const gf_field* dSdUbar,
                               double* dSdrho);
/* Smeared Wilson-action MD force on the thin links, the stout-HMC P_update!
 * (test/HMCstout_test_nowing.jl:99-118): forward, dS/dUbar = beta/2 * staples
 * of Ubar, back-propagation, P += eps * (-(1/3) TA(U dS/dU)). */
int gf_stout_mom_update(gf_ctx* ctx, gf_stout* st, gf_field* P, const gf_field* U, double eps, double beta);

/* ---- gradient flow ------------------------------------------------------ */
/* flow!(U, ::Gradientflow) (smearing/gradientflow.jl:171-238): nsteps RK3
 * Wilson-flow steps of size eps. */
int gf_flow(gf_ctx* ctx, gf_field* U, double eps, int nsteps);
/* The same flow with the force and the exponentials in double-float
 * arithmetic on the fp32 pipes (precision GF_DFLOAT; the fields stay fp64)
 * or in fp64 (GF_FP64, = gf_flow). */
int gf_flow_precision(gf_ctx* ctx, gf_field* U, double eps, int nsteps, int precision);
/* flow!(U, ::Gradientflow_general) (smearing/gradientflow.jl:240-336) for the
 * action with the plaquette loops at c_plaq and the rectangle loops at c_rect
 * (gradient_flow(U, [:plaquette, :rectangular], [c_plaq, c_rect]), API.jl:
 * 426-438): the same RK3 steps with the force TA(U dS/dU) (F_update!,
 * gradientflow.jl:319-334), fp64. (1, 0) is the Wilson flow of gf_flow. */
int gf_flow_loops(gf_ctx* ctx, gf_field* U, double eps, int nsteps, double c_plaq, double c_rect);
/* add_force!(F, U, temps; plaqonly=true) (AbstractGaugefields.jl:2717-2763):
 * F += factor * TA(U_mu V_mu^dag) with V the six-staple sum. */
int gf_flow_force(gf_ctx* ctx, const gf_field* U, gf_field* F, double factor);

/* ---- allocation-free plaquette (no counterpart in the reference) -------- */
/* The plaquette sum of gf_plaquette for callers that cannot allocate device
 * memory: applications whose device memory belongs to another allocator
 * (CUDA.jl's pool, PyTorch's caching allocator) and loops where a cudaMalloc
 * would synchronise the device. It needs no context (creating one
 * allocates). `links` is the device storage of a GF_LINK64 field
 * (gf_field_device_ptr) for the lattice L = {NX,NY,NZ,NT}; `out` is one
 * double in device memory; `stream` a cudaStream_t (NULL: default stream).
 * Kernels are only enqueued: read `out` after the stream has finished.
 * The per-block partial sums live in a fixed 1 MiB device array inside the
 * library (held by every GPU that loads it until the process exits), so the
 * lattice may have at most 16,777,216 sites (64^4); larger lattices return
 * GF_EINVAL. All calls share that array: calls whose kernels overlap on the
 * GPU race and must be serialised by the caller. The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress) with that device
 * current; make it before any stream capture. That address is kept for the
 * life of the process, so do not call this entry point again after
 * cudaDeviceReset (or any teardown of the device's primary context).
 * gf_last_error(NULL) gives the message of a failed call. */
int gf_plaquette_noalloc(const void* links, const int L[4], double* out, void* stream);

/* ---- instrumentation (no counterpart in the reference) ----------------- */
/* Kernel classes timed by gf_prof_*: */
#define GF_K_PLAQ 0         /* plaquette / action reduction (fp64) */
#define GF_K_FORCE 1        /* Wilson staple force (+ momentum update) */
#define GF_K_LINK_UPDATE 2  /* exp(i eps P) U link update (fp64) */
#define GF_K_STOUT_FWD 3    /* stout forward level, fp32 */
#define GF_K_BWD_LOCAL 4    /* stout adjoint, local part, fp32 */
#define GF_K_BWD_GATHER 5   /* stout adjoint, pull-back gather (+ force), fp32 */
#define GF_K_STOUT_FWD64 6  /* the same three stages in fp64 */
#define GF_K_BWD_LOCAL64 7
#define GF_K_BWD_GATHER64 8
#define GF_K_OTHER 9        /* starts, conversions, kinetic, copies */
#define GF_K_LINK_UPDATE_DF 10  /* link update in double-float (mixed form) */
#define GF_K_STOUT_FWD_DF 11    /* stout forward in double-float (Hamiltonian, GF_DFLOAT force) */
#define GF_K_FORCE_DF 12        /* Wilson staple force in double-float */
#define GF_K_BWD_LOCAL_DF 13    /* stout adjoint, local part, double-float */
#define GF_K_BWD_GATHER_DF 14   /* stout adjoint, gather (+ force), double-float */
#define GF_K_RECT 15            /* rectangle loop sum and plaquette + rectangle force (fp64) */
#define GF_K_RECT_DF 16         /* plaquette + rectangle force in double-float */
#define GF_K_COUNT 17
/* Enable (on != 0) or disable CUDA-event timing of every kernel launch on the
 * context's stream; enabling clears the accumulators. */
int gf_prof_enable(gf_ctx* ctx, int on);
/* Total device milliseconds and launch count of one kernel class since the
 * last gf_prof_enable(ctx, 1); synchronises the context's stream. */
int gf_prof_read(gf_ctx* ctx, int kernel_class, double* total_ms, long long* launches);
/* Process-wide number of kernels this library has launched. */
int gf_launch_count(long long* out);

#ifdef __cplusplus
}
#endif
#endif /* GAUGEFIELDS_GB300_H */

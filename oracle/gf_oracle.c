/*
 * gf_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * CPU restatement, in FP64 C99, of the Gaugefields.jl algorithms on the SU(3)
 * gauge-link hot path. Only the tests, __graft_entry__.smoke() and the
 * cpu_baseline / reference leg of bench.py load it, and only as the checker or
 * the timed CPU baseline; the product library never links it.
 *
 * It follows the reference's own in-tree CPU code (paths inside Gaugefields.jl):
 *   construct_staple!, calculate_Plaquette  src/AbstractGaugefields.jl:2684-2699, 2873-2923
 *   GaugeAction staples / calc_dSdUμ!      src/action/GaugeActions.jl:48-123, 132-213
 *   md_force!, update_*!, md_trajectory!    src/molecular_dynamics.jl:243-267, 494-730
 *   Traceless_antihermitian_add! (NC=3)     src/4D/TA_gaugefields_4D_serial.jl:181-269
 *   exptU! eigen method + exp_T4 fallback   src/4D/TA_gaugefields_4D_serial.jl:690-1078
 *   P*P                                     src/4D/TA_gaugefields_4D_serial.jl:106-129
 *   normalize3! / m3complv3!                src/AbstractGaugefields.jl:3378-3457
 *   calc_coefficients_Q                     src/AbstractGaugefields.jl:3284-3344
 *   STOUT forward!/backward + CdexpQdQ!     src/smearing/stout_fast.jl:250-408, 603-785, 888-946, 1031-1081
 *   STOUT_dataset (Cμ, dCμ/dUν lists)       src/smearing/stout_dataset.jl:10-80
 *   plaquette / rectangle loop sets         src/autostaples/wilsonloops.jl:233-330 (make_plaq, make_rect)
 *   calculate_Polyakov_loop                 src/AbstractGaugefields.jl:2929-2956
 *   flow! (RK3), add_force!, exp_aF_U!      src/smearing/gradientflow.jl:171-238,
 *                                           src/AbstractGaugefields.jl:2717-2842
 * The Wilson-loop path lists come from the external package Wilsonloop.jl
 * (compat 0.1.3, not vendored); they are restated here from their published
 * definitions (plaquette staples; derive_U of a path as left/right link
 * products around each occurrence of U_nu).
 *
 * Parity pinning: the reference is Julia and cannot run in this environment,
 * and its default arithmetic lives in LatticeMatrices.jl (not vendored). The
 * oracle is pinned by the reference's own invariant tests (cold-start
 * plaquette == 1 exactly, cold-start Delta H == 0 and P*P == 0, reversibility
 * to 2e-12, force additivity) and by the gradient-flow golden value at the
 * reference test's tolerance; see tests/test_oracle.py.
 *
 * Layouts are the reference's host layouts: links complex128 (3,3,NX,NY,NZ,NT)
 * column-major per direction with the four directions contiguous; momenta
 * (8,NX,NY,NZ,NT) per direction.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cdbl;
typedef struct {
  cdbl m[3][3];
} M3;

typedef struct {
  int L[4];
  long V;
} Lat;

static Lat mklat(const int L[4]) {
  Lat l;
  l.V = 1;
  for (int i = 0; i < 4; ++i) {
    l.L[i] = L[i];
    l.V *= L[i];
  }
  return l;
}

static inline void coords(const Lat* l, long lex, int x[4]) {
  x[0] = (int)(lex % l->L[0]);
  lex /= l->L[0];
  x[1] = (int)(lex % l->L[1]);
  lex /= l->L[1];
  x[2] = (int)(lex % l->L[2]);
  x[3] = (int)(lex / l->L[2]);
}
static inline long lexof(const Lat* l, const int x[4]) {
  return x[0] + (long)l->L[0] * (x[1] + (long)l->L[1] * (x[2] + (long)l->L[2] * x[3]));
}
/* site x + sum_k off[k] e_k with periodic wrap */
static inline long shifted(const Lat* l, long lex, const int off[4]) {
  int x[4];
  coords(l, lex, x);
  for (int k = 0; k < 4; ++k) {
    int c = (x[k] + off[k]) % l->L[k];
    if (c < 0) c += l->L[k];
    x[k] = c;
  }
  return lexof(l, x);
}
static inline long shift1(const Lat* l, long lex, int mu, int d) {
  int off[4] = {0, 0, 0, 0};
  off[mu] = d;
  return shifted(l, lex, off);
}

static inline M3 ld(const cdbl* U, const Lat* l, int mu, long lex) {
  const cdbl* p = U + ((size_t)mu * l->V + lex) * 9;
  M3 a;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) a.m[i][j] = p[i + 3 * j];
  return a;
}
static inline void stm(cdbl* U, const Lat* l, int mu, long lex, const M3* a) {
  cdbl* p = U + ((size_t)mu * l->V + lex) * 9;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) p[i + 3 * j] = a->m[i][j];
}

/* Neumaier (improved Kahan) summation of n doubles: the oracle's global sums
 * are accurate to a few ulp of the total, independent of their order. */
static double sum_accurate(const double* v, long n) {
  double s = 0.0, c = 0.0;
  for (long i = 0; i < n; ++i) {
    double t = s + v[i];
    if (fabs(s) >= fabs(v[i])) c += (s - t) + v[i];
    else c += (v[i] - t) + s;
    s = t;
  }
  return s + c;
}

static inline M3 mzero(void) {
  M3 a;
  memset(&a, 0, sizeof a);
  return a;
}
static inline M3 meye(void) {
  M3 a = mzero();
  a.m[0][0] = a.m[1][1] = a.m[2][2] = 1.0;
  return a;
}
static inline M3 mmul(const M3* a, const M3* b) {
  M3 c;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      cdbl s = 0;
      for (int k = 0; k < 3; ++k) s += a->m[i][k] * b->m[k][j];
      c.m[i][j] = s;
    }
  return c;
}
static inline M3 mdag(const M3* a) {
  M3 c;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) c.m[i][j] = conj(a->m[j][i]);
  return c;
}
static inline void madd(M3* c, cdbl s, const M3* a) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) c->m[i][j] += s * a->m[i][j];
}
static inline cdbl mtr(const M3* a) { return a->m[0][0] + a->m[1][1] + a->m[2][2]; }

/* ------------------------------------------------------------------------ */
/* Traceless_antihermitian! (matrix) and the coefficient map of             */
/* Traceless_antihermitian_add! (NC = 3)                                     */
/* ------------------------------------------------------------------------ */
static const double sr3i = 0.57735026918962576451;

static M3 ta_matrix(const M3* v) {
  M3 y;
  double tri = (cimag(v->m[0][0]) + cimag(v->m[1][1]) + cimag(v->m[2][2])) / 3.0;
  for (int i = 0; i < 3; ++i) y.m[i][i] = I * (cimag(v->m[i][i]) - tri);
  for (int i = 0; i < 3; ++i)
    for (int j = i + 1; j < 3; ++j) {
      cdbl x = v->m[i][j] - conj(v->m[j][i]);
      y.m[i][j] = 0.5 * x;
      y.m[j][i] = -0.5 * conj(x);
    }
  return y;
}

/* c[a] += factor * (coefficient a of TA(v)), as Traceless_antihermitian_add! */
static void ta_add(double* c, double factor, const M3* v) {
  M3 y = ta_matrix(v);
  c[0] += (cimag(y.m[0][1]) + cimag(y.m[1][0])) * factor;
  c[1] += (creal(y.m[0][1]) - creal(y.m[1][0])) * factor;
  c[2] += (cimag(y.m[0][0]) - cimag(y.m[1][1])) * factor;
  c[3] += (cimag(y.m[0][2]) + cimag(y.m[2][0])) * factor;
  c[4] += (creal(y.m[0][2]) - creal(y.m[2][0])) * factor;
  c[5] += (cimag(y.m[1][2]) + cimag(y.m[2][1])) * factor;
  c[6] += (creal(y.m[1][2]) - creal(y.m[2][1])) * factor;
  c[7] += sr3i * (cimag(y.m[0][0]) + cimag(y.m[1][1]) - 2 * cimag(y.m[2][2])) * factor;
}

/* ------------------------------------------------------------------------ */
/* exptU! for TA fields (eigen method, TA_gaugefields_4D_serial.jl:760-1078) */
/* uout = exp(t * i sum_a u_a lambda_a / 2)                                   */
/* ------------------------------------------------------------------------ */
static long g_taylor_fallbacks = 0;

static M3 exp_t4(double v1, double v3, double v4, double v5, double v6, double v7, double v8, double v9, double v11,
                 double v12, double v13, double v14, double v15, double v16, double v17) {
  /* exp(iV) ~ 1 + iV - V^2/2 - iV^3/6 + V^4/24  (exp_T4, :690-758) */
  M3 V;
  V.m[0][0] = v1;
  V.m[0][1] = v3 + I * v4;
  V.m[0][2] = v5 + I * v6;
  V.m[1][0] = v7 + I * v8;
  V.m[1][1] = v9;
  V.m[1][2] = v11 + I * v12;
  V.m[2][0] = v13 + I * v14;
  V.m[2][1] = v15 + I * v16;
  V.m[2][2] = v17;
  M3 V2 = mmul(&V, &V), V3 = mmul(&V2, &V), V4 = mmul(&V2, &V2);
  M3 E = meye();
  madd(&E, I, &V);
  madd(&E, -0.5, &V2);
  madd(&E, -I / 6.0, &V3);
  madd(&E, 1.0 / 24.0, &V4);
  return E;
}

/* Which exponential the oracle's link updates use: 0 = the reference's eigen
 * method (default), 1 = Taylor series with scaling and squaring to full
 * double precision (used to separate the eigen method's own ~1e-14 error
 * from differences of the GPU path). */
static int g_exp_method = 0;
void or_set_exp_method(int m) { g_exp_method = m; }

static M3 expt_taylor(double t, const double* u) {
  /* X = i t sum_a u_a lambda_a / 2, exp(X) = (exp(X / 2^k))^(2^k) */
  M3 X;
  double c[8];
  for (int a = 0; a < 8; ++a) c[a] = t * u[a] * 0.5;
  X.m[0][0] = I * (c[2] + sr3i * c[7]);
  X.m[1][1] = I * (-c[2] + sr3i * c[7]);
  X.m[2][2] = I * (-2 * sr3i * c[7]);
  X.m[0][1] = I * (c[0] - I * c[1]);
  X.m[1][0] = I * (c[0] + I * c[1]);
  X.m[0][2] = I * (c[3] - I * c[4]);
  X.m[2][0] = I * (c[3] + I * c[4]);
  X.m[1][2] = I * (c[5] - I * c[6]);
  X.m[2][1] = I * (c[5] + I * c[6]);
  double nrm = 0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) nrm += creal(X.m[i][j] * conj(X.m[i][j]));
  nrm = sqrt(nrm);
  int k = 0;
  while (nrm > 0.25) {
    nrm *= 0.5;
    ++k;
  }
  double sc = ldexp(1.0, -k);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) X.m[i][j] *= sc;
  M3 E = meye(), term = meye();
  for (int n = 1; n <= 24; ++n) {
    term = mmul(&term, &X);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) term.m[i][j] /= n;
    madd(&E, 1.0, &term);
  }
  for (int r = 0; r < k; ++r) E = mmul(&E, &E);
  return E;
}

static M3 expt_eigen_ref(double t, const double* u);

static M3 expt_eigen(double t, const double* u) {
  return g_exp_method == 1 ? expt_taylor(t, u) : expt_eigen_ref(t, u);
}

static M3 expt_eigen_ref(double t, const double* u) {
  const double pi23 = 2.0 * M_PI / 3.0;
  const double tinyvalue = 1e-100;
  double c1 = t * u[0] * 0.5, c2 = t * u[1] * 0.5, c3 = t * u[2] * 0.5, c4 = t * u[3] * 0.5;
  double c5 = t * u[4] * 0.5, c6 = t * u[5] * 0.5, c7 = t * u[6] * 0.5, c8 = t * u[7] * 0.5;
  double csum = c1 + c2 + c3 + c4 + c5 + c6 + c7 + c8;
  if (csum == 0) return meye();
  double v1 = c3 + sr3i * c8, v3 = c1, v4 = -c2, v5 = c4, v6 = -c5;
  double v7 = c1, v8 = c2, v9 = -c3 + sr3i * c8, v11 = c6, v12 = -c7;
  double v13 = c4, v14 = c5, v15 = c6, v16 = c7, v17 = -2.0 * sr3i * c8;
  double trv3 = (v1 + v9 + v17) / 3.0;
  double cofac = v1 * v9 - v3 * v3 - v4 * v4 + v1 * v17 - v5 * v5 - v6 * v6 + v9 * v17 - v11 * v11 - v12 * v12;
  double det = v1 * v9 * v17 - v1 * (v11 * v11 + v12 * v12) - v9 * (v5 * v5 + v6 * v6) - v17 * (v3 * v3 + v4 * v4) +
               (v5 * (v3 * v11 - v4 * v12) + v6 * (v3 * v12 + v4 * v11)) * 2.0;
  double p3 = cofac / 3.0 - trv3 * trv3;
  double q = trv3 * cofac - det - 2.0 * trv3 * trv3 * trv3;
  double x = sqrt(-4.0 * p3) + tinyvalue;
  double arg = q / (x * p3);
  if (arg > 1) arg = 1;
  if (arg < -1) arg = -1;
  double theta = acos(arg) / 3.0;
  double e1 = x * cos(theta) + trv3;
  theta = theta + pi23;
  double e2 = x * cos(theta) + trv3;
  double e3 = 3.0 * trv3 - e1 - e2;
  double e[3] = {e1, e2, e3};
  double w[3][6];
  for (int k = 0; k < 3; ++k) {
    double ek = e[k];
    w[k][0] = v5 * (v9 - ek) - v3 * v11 + v4 * v12;
    w[k][1] = -v6 * (v9 - ek) + v4 * v11 + v3 * v12;
    w[k][2] = (v1 - ek) * v11 - v3 * v5 - v4 * v6;
    w[k][3] = -(v1 - ek) * v12 - v4 * v5 + v3 * v6;
    w[k][4] = -(v1 - ek) * (v9 - ek) + v3 * v3 + v4 * v4;
    w[k][5] = 0.0;
    double nrm2 = w[k][0] * w[k][0] + w[k][1] * w[k][1] + w[k][2] * w[k][2] + w[k][3] * w[k][3] + w[k][4] * w[k][4];
    if (nrm2 < 1e-24) {
      /* degenerate eigenvectors: the reference falls back to the 4th-order
       * Taylor series (an approximation, not the exact exponential) */
#pragma omp atomic
      g_taylor_fallbacks++;
      return exp_t4(v1, v3, v4, v5, v6, v7, v8, v9, v11, v12, v13, v14, v15, v16, v17);
    }
    double coeff = 1.0 / sqrt(nrm2);
    for (int j = 0; j < 5; ++j) w[k][j] *= coeff;
  }
  /* uout = w^dag * ww, ww_k = exp(i e_k) w_k (row k) */
  M3 W, WW;
  for (int k = 0; k < 3; ++k) {
    double ck = cos(e[k]), sk = sin(e[k]);
    for (int j = 0; j < 3; ++j) {
      double re = w[k][2 * j], im = w[k][2 * j + 1];
      W.m[k][j] = re + I * im;
      WW.m[k][j] = (re * ck - im * sk) + I * (im * ck + re * sk);
    }
  }
  M3 Wd = mdag(&W);
  return mmul(&Wd, &WW);
}

/* ------------------------------------------------------------------------ */
/* calc_coefficients_Q (AbstractGaugefields.jl:3284-3344), Q Hermitian        */
/* ------------------------------------------------------------------------ */
typedef struct {
  cdbl f0, f1, f2, b10, b11, b12, b20, b21, b22;
} QCoef;

static QCoef calc_coefficients_Q(const M3* Q) {
  QCoef r;
  cdbl c0 = Q->m[0][0] * Q->m[1][1] * Q->m[2][2] + Q->m[0][1] * Q->m[1][2] * Q->m[2][0] +
            Q->m[0][2] * Q->m[1][0] * Q->m[2][1] - Q->m[0][2] * Q->m[1][1] * Q->m[2][0] -
            Q->m[0][1] * Q->m[1][0] * Q->m[2][2] - Q->m[0][0] * Q->m[1][2] * Q->m[2][1];
  cdbl c1c = 0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) c1c += Q->m[i][j] * Q->m[j][i];
  double c1 = creal(c1c) / 2;
  double c0r = creal(c0);
  double c0max = 2 * pow(c1 / 3, 1.5);
  double th = acos(c0r / c0max);
  double u = sqrt(c1 / 3) * cos(th / 3);
  double w = sqrt(c1) * sin(th / 3);
  double xi0 = sin(w) / w;
  double xi1 = cos(w) / (w * w) - sin(w) / (w * w * w);
  cdbl emiu = cexp(-I * u), e2iu = cexp(2 * I * u);
  double cw = cos(w);
  cdbl h0 = (u * u - w * w) * e2iu + emiu * (8 * u * u * cw + 2 * I * u * (3 * u * u + w * w) * xi0);
  cdbl h1 = 2 * u * e2iu - emiu * (2 * u * cw - I * (3 * u * u - w * w) * xi0);
  cdbl h2 = e2iu - emiu * (cw + 3 * I * u * xi0);
  double den = 9 * u * u - w * w;
  r.f0 = h0 / den;
  r.f1 = h1 / den;
  r.f2 = h2 / den;
  cdbl r10 = 2 * (u + I * (u * u - w * w)) * e2iu +
             2 * emiu * (4 * u * (2 - I * u) * cw + I * (9 * u * u + w * w - I * u * (3 * u * u + w * w)) * xi0);
  cdbl r11 = 2 * (1 + 2 * I * u) * e2iu + emiu * (-2 * (1 - I * u) * cw + I * (6 * u + I * (w * w - 3 * u * u)) * xi0);
  cdbl r12 = 2 * I * e2iu + I * emiu * (cw - 3 * (1 - I * u) * xi0);
  cdbl r20 = -2 * e2iu + 2 * I * u * emiu * (cw + (1 + 4 * I * u) * xi0 + 3 * u * u * xi1);
  cdbl r21 = -I * emiu * (cw + (1 + 2 * I * u) * xi0 - 3 * u * u * xi1);
  cdbl r22 = emiu * (xi0 - 3 * I * u * xi1);
  double d2 = 2 * den * den;
  r.b10 = (2 * u * r10 + (3 * u * u - w * w) * r20 - 2 * (15 * u * u + w * w) * r.f0) / d2;
  r.b11 = (2 * u * r11 + (3 * u * u - w * w) * r21 - 2 * (15 * u * u + w * w) * r.f1) / d2;
  r.b12 = (2 * u * r12 + (3 * u * u - w * w) * r22 - 2 * (15 * u * u + w * w) * r.f2) / d2;
  r.b20 = (r10 - 3 * u * r20 - 24 * u * r.f0) / d2;
  r.b21 = (r11 - 3 * u * r21 - 24 * u * r.f1) / d2;
  r.b22 = (r12 - 3 * u * r22 - 24 * u * r.f2) / d2;
  return r;
}

/* C star dexp(Q)/dQ for antihermitian Q (CdexpQdQ! NC=3, stout_fast.jl:888-946) */
static M3 cdexpqdq(const M3* C, const M3* Q) {
  cdbl trQ2 = 0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) trQ2 += Q->m[i][j] * Q->m[j][i];
  M3 out = mzero();
  /* At Q = 0 the reference leaves the output untouched (its commented-out
   * assignment copies C); the exact pull-back there is C itself. */
  if (!(cabs(trQ2) > 1e-18)) return *C;
  M3 Qn;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Qn.m[i][j] = Q->m[i][j] / I;
  QCoef k = calc_coefficients_Q(&Qn);
  M3 Q2 = mmul(&Qn, &Qn);
  M3 B1 = mzero(), B2 = mzero();
  for (int i = 0; i < 3; ++i) {
    B1.m[i][i] = k.b10;
    B2.m[i][i] = k.b20;
  }
  madd(&B1, k.b11, &Qn);
  madd(&B1, k.b12, &Q2);
  madd(&B2, k.b21, &Qn);
  madd(&B2, k.b22, &Q2);
  M3 CB1 = mmul(C, &B1), CB2 = mmul(C, &B2);
  cdbl trCB1 = mtr(&CB1), trCB2 = mtr(&CB2);
  M3 QC = mmul(&Qn, C), CQ = mmul(C, &Qn);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      out.m[i][j] = (trCB1 * Qn.m[i][j] + k.f1 * C->m[i][j] + trCB2 * Q2.m[i][j] + k.f2 * (QC.m[i][j] + CQ.m[i][j])) / I;
  return out;
}

/* ------------------------------------------------------------------------ */
/* normalize3! (AbstractGaugefields.jl:3378-3457)                             */
/* ------------------------------------------------------------------------ */
static void normalize3(M3* u) {
  cdbl w1 = 0, w2 = 0;
  for (int ic = 0; ic < 3; ++ic) {
    w1 += u->m[1][ic] * conj(u->m[0][ic]);
    w2 += u->m[0][ic] * conj(u->m[0][ic]);
  }
  w1 = -w1 / w2;
  cdbl x4 = u->m[1][0] + w1 * u->m[0][0];
  cdbl x5 = u->m[1][1] + w1 * u->m[0][1];
  cdbl x6 = u->m[1][2] + w1 * u->m[0][2];
  cdbl w3 = x4 * conj(x4) + x5 * conj(x5) + x6 * conj(x6);
  u->m[1][0] = x4;
  u->m[1][1] = x5;
  u->m[1][2] = x6;
  double s3 = 1 / sqrt(creal(w3)), s2 = 1 / sqrt(creal(w2));
  for (int j = 0; j < 3; ++j) {
    u->m[0][j] *= s2;
    u->m[1][j] *= s3;
  }
  /* m3complv3! */
  u->m[2][0] = conj(u->m[0][1] * u->m[1][2] - u->m[0][2] * u->m[1][1]);
  u->m[2][1] = conj(u->m[0][2] * u->m[1][0] - u->m[0][0] * u->m[1][2]);
  u->m[2][2] = conj(u->m[0][0] * u->m[1][1] - u->m[0][1] * u->m[1][0]);
}

/* ------------------------------------------------------------------------ */
/* Wilson lines: a path is a list of steps (dir, +-1) from an origin; each   */
/* step is a link U_dir(base)^(dagger) at an absolute offset (the GLink of   */
/* Wilsonloop.jl).                                                           */
/* ------------------------------------------------------------------------ */
typedef struct {
  int dir;
  int dag;
  int off[4];
} Link;

typedef struct {
  int n;
  Link l[8];
} Path;

static Path path_from_steps(const int (*steps)[2], int n) {
  Path p;
  p.n = n;
  int c[4] = {0, 0, 0, 0};
  for (int k = 0; k < n; ++k) {
    int d = steps[k][0], s = steps[k][1];
    p.l[k].dir = d;
    if (s > 0) {
      p.l[k].dag = 0;
      memcpy(p.l[k].off, c, sizeof c);
      c[d] += 1;
    } else {
      c[d] -= 1;
      p.l[k].dag = 1;
      memcpy(p.l[k].off, c, sizeof c);
    }
  }
  return p;
}

static Path path_dag(const Path* p) {
  Path q;
  q.n = p->n;
  for (int k = 0; k < p->n; ++k) {
    q.l[k] = p->l[p->n - 1 - k];
    q.l[k].dag ^= 1;
  }
  return q;
}

/* product of links k0..k1-1 of a path anchored at site `lex` */
static M3 eval_links(const cdbl* U, const Lat* lat, const Path* p, int k0, int k1, long lex) {
  M3 r = meye();
  for (int k = k0; k < k1; ++k) {
    long s = shifted(lat, lex, p->l[k].off);
    M3 u = ld(U, lat, p->l[k].dir, s);
    if (p->l[k].dag) u = mdag(&u);
    r = mmul(&r, &u);
  }
  return r;
}

/* MP staples of C_mu (make_Cμ on the plaquette loops): up and down per nu */
static int cmu_staples(int mu, Path* out) {
  int n = 0;
  for (int nu = 0; nu < 4; ++nu) {
    if (nu == mu) continue;
    int up[3][2] = {{nu, +1}, {mu, +1}, {nu, -1}};
    int dn[3][2] = {{nu, -1}, {mu, +1}, {nu, +1}};
    out[n++] = path_from_steps((const int (*)[2])up, 3);
    out[n++] = path_from_steps((const int (*)[2])dn, 3);
  }
  return n;
}

/* Staples of GaugeAction (plaq U plaq^dag) for U_mu: the rest of each closed
 * loop after U_mu(x); make_staple(loop, mu) over plaq U plaq^dag. */
static int action_staples(int mu, Path* out) {
  int n = 0;
  for (int nu = 0; nu < 4; ++nu) {
    if (nu == mu) continue;
    int up[3][2] = {{nu, +1}, {mu, -1}, {nu, -1}};  /* loop U_mu(x) U_nu(x+mu) U_mu^dag(x+nu) U_nu^dag(x) */
    int dn[3][2] = {{nu, -1}, {mu, -1}, {nu, +1}};  /* loop U_mu(x) U_nu^dag(x+mu-nu) U_mu^dag(x-nu) U_nu(x-nu) */
    Path a = path_from_steps((const int (*)[2])up, 3);
    Path b = path_from_steps((const int (*)[2])dn, 3);
    /* the staple starts at x + e_mu */
    for (int k = 0; k < 3; ++k) {
      a.l[k].off[mu] += 1;
      b.l[k].off[mu] += 1;
    }
    out[n++] = a;
    out[n++] = b;
  }
  return n;
}

/* ------------------------------------------------------------------------ */
/* exported API                                                              */
/* ------------------------------------------------------------------------ */
int or_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void or_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
long or_taylor_fallbacks(void) { return g_taylor_fallbacks; }

/* construct_staple!: V = sum_{nu != mu} U_nu(x) U_mu(x+nu) U_nu(x+mu)^dag */
void or_staple(const int L[4], const cdbl* U, int mu, cdbl* Vout) {
  Lat lat = mklat(L);
#pragma omp parallel for schedule(static)
  for (long x = 0; x < lat.V; ++x) {
    M3 acc = mzero();
    for (int nu = 0; nu < 4; ++nu) {
      if (nu == mu) continue;
      M3 a = ld(U, &lat, nu, x);
      M3 b = ld(U, &lat, mu, shift1(&lat, x, nu, 1));
      M3 c = ld(U, &lat, nu, shift1(&lat, x, mu, 1));
      M3 ab = mmul(&a, &b);
      M3 cd = mdag(&c);
      M3 t = mmul(&ab, &cd);
      madd(&acc, 1.0, &t);
    }
    stm(Vout, &lat, 0, x, &acc);
  }
}

/* calculate_Plaquette: real(sum_mu tr(U_mu V_mu^dag) * 0.5) */
/* calculate_Polyakov_loop(U, temp1, temp2) (src/AbstractGaugefields.jl:
 * 2929-2956): the products U_T(x) U_T(x+T) ... U_T(x+(NT-1)T) from the
 * sites of the first time slice, traced and averaged over that slice
 * (partial_tr over the slice / NX NY NZ); out = {Re, Im} */
void or_polyakov_loop(const int L[4], const cdbl* U, double out[2]) {
  Lat lat = mklat(L);
  const long vs = (long)L[0] * L[1] * L[2];
  double* pr = (double*)calloc((size_t)vs, sizeof(double));
  double* pi = (double*)calloc((size_t)vs, sizeof(double));
#pragma omp parallel for schedule(static)
  for (long s = 0; s < vs; ++s) {
    long x = s;  /* lexicographic index of (x, y, z, t = 0) */
    M3 p = ld(U, &lat, 3, x);
    for (int t = 1; t < L[3]; ++t) {
      x = shift1(&lat, x, 3, 1);
      M3 u = ld(U, &lat, 3, x);
      p = mmul(&p, &u);
    }
    cdbl tr = mtr(&p);
    pr[s] = creal(tr);
    pi[s] = cimag(tr);
  }
  out[0] = sum_accurate(pr, vs) / (double)vs;
  out[1] = sum_accurate(pi, vs) / (double)vs;
  free(pr);
  free(pi);
}

double or_plaquette(const int L[4], const cdbl* U) {
  Lat lat = mklat(L);
  double* part = (double*)calloc((size_t)lat.V, sizeof(double));
#pragma omp parallel for schedule(static)
  for (long x = 0; x < lat.V; ++x) {
    cdbl s = 0;
    for (int mu = 0; mu < 4; ++mu) {
      M3 V = mzero();
      for (int nu = 0; nu < 4; ++nu) {
        if (nu == mu) continue;
        M3 a = ld(U, &lat, nu, x);
        M3 b = ld(U, &lat, mu, shift1(&lat, x, nu, 1));
        M3 c = ld(U, &lat, nu, shift1(&lat, x, mu, 1));
        M3 ab = mmul(&a, &b);
        M3 cd = mdag(&c);
        M3 t = mmul(&ab, &cd);
        madd(&V, 1.0, &t);
      }
      M3 u = ld(U, &lat, mu, x);
      M3 vd = mdag(&V);
      M3 t = mmul(&u, &vd);
      s += mtr(&t);
    }
    part[x] = creal(s * 0.5);
  }
  double sum = sum_accurate(part, lat.V);
  free(part);
  return sum;
}

/* calc_dSdUμ!: dS/dU_mu = beta/2 * (staples of plaq U plaq^dag for U_mu) */
static void dsdu_mu(const Lat* lat, const cdbl* U, double coef, int mu, cdbl* D) {
  Path st[6];
  int ns = action_staples(mu, st);
#pragma omp parallel for schedule(static)
  for (long x = 0; x < lat->V; ++x) {
    M3 acc = mzero();
    for (int k = 0; k < ns; ++k) {
      M3 t = eval_links(U, lat, &st[k], 0, st[k].n, x);
      madd(&acc, coef, &t);
    }
    stm(D, lat, 0, x, &acc);
  }
}

void or_dsdu(const int L[4], const cdbl* U, double beta, int mu, cdbl* D) {
  Lat lat = mklat(L);
  dsdu_mu(&lat, U, 0.5 * beta, mu, D);
}

/* md_potential(::GaugeAction) = -Re(evaluate_GaugeAction)/NC with the loops
 * plaq U plaq^dag at coefficient beta/2 */
double or_action(const int L[4], const cdbl* U, double beta) {
  Lat lat = mklat(L);
  double* part = (double*)calloc((size_t)lat.V, sizeof(double));
#pragma omp parallel for schedule(static)
  for (long x = 0; x < lat.V; ++x) {
    cdbl s = 0;
    for (int mu = 0; mu < 4; ++mu)
      for (int nu = mu + 1; nu < 4; ++nu) {
        int stp[4][2] = {{mu, 1}, {nu, 1}, {mu, -1}, {nu, -1}};
        Path p = path_from_steps((const int (*)[2])stp, 4);
        Path q = path_dag(&p);
        M3 a = eval_links(U, &lat, &p, 0, 4, x);
        M3 b = eval_links(U, &lat, &q, 0, 4, x);
        s += 0.5 * beta * (mtr(&a) + mtr(&b));
      }
    part[x] = creal(s);
  }
  double sum = sum_accurate(part, lat.V);
  free(part);
  return -sum / 3.0;
}

/* md_force!(::GaugeAction): F_mu = TA-coefficients of -(1/3) U_mu dS/dU_mu */
void or_force(const int L[4], const cdbl* U, double beta, double* F) {
  Lat lat = mklat(L);
  cdbl* D = (cdbl*)malloc(sizeof(cdbl) * 9 * (size_t)lat.V);
  for (int mu = 0; mu < 4; ++mu) {
    dsdu_mu(&lat, U, 0.5 * beta, mu, D);
#pragma omp parallel for schedule(static)
    for (long x = 0; x < lat.V; ++x) {
      M3 u = ld(U, &lat, mu, x);
      M3 d = ld(D, &lat, 0, x);
      M3 w = mmul(&u, &d);
      double* f = F + ((size_t)mu * lat.V + x) * 8;
      for (int a = 0; a < 8; ++a) f[a] = 0;
      ta_add(f, -1.0 / 3.0, &w);
    }
  }
  free(D);
}

/* ------------------------------------------------------------------------ */
/* general loop sets (push!(action, c, loops U loops'))                      */
/* ------------------------------------------------------------------------ */
/* A closed loop as unit steps (direction, +-1) from its origin. Kind 0 is the
 * plaquette set, kind 1 the rectangle set of make_loops_fromname
 * ("plaquette" / "rectangular"): for mu < nu the loops (mu,1),(nu,1),(mu,-1),
 * (nu,-1), and (mu,1),(nu,2),(mu,-1),(nu,-2) with (mu,2),(nu,1),(mu,-2),(nu,-1)
 * (make_plaq / make_rect, src/autostaples/wilsonloops.jl:233-330), each
 * followed by its Hermitian conjugate (the reversed loop with every step
 * inverted), as the action's loops U loops' holds it. */
typedef struct {
  int n;
  int st[8][2];
} Loop;

static void loop_push(Loop* l, int dir, int sign, int count) {
  for (int i = 0; i < count; ++i) {
    l->st[l->n][0] = dir;
    l->st[l->n][1] = sign;
    l->n++;
  }
}

static int loop_set(int kind, Loop* out) {
  int n = 0;
  for (int mu = 0; mu < 4; ++mu)
    for (int nu = mu + 1; nu < 4; ++nu) {
      const int shapes[2][2] = {{1, 2}, {2, 1}}; /* extent along mu, along nu */
      const int nshape = kind == 0 ? 1 : 2;
      for (int k = 0; k < nshape; ++k) {
        int a = kind == 0 ? 1 : shapes[k][0], b = kind == 0 ? 1 : shapes[k][1];
        Loop l;
        l.n = 0;
        loop_push(&l, mu, +1, a);
        loop_push(&l, nu, +1, b);
        loop_push(&l, mu, -1, a);
        loop_push(&l, nu, -1, b);
        Loop d;
        d.n = l.n;
        for (int i = 0; i < l.n; ++i) {
          d.st[i][0] = l.st[l.n - 1 - i][0];
          d.st[i][1] = -l.st[l.n - 1 - i][1];
        }
        out[n++] = l;
        out[n++] = d;
      }
    }
  return n;
}

/* Staples of a loop set for U_mu (Wilsonloop's make_staple over the set):
 * every forward occurrence of U_mu in a loop contributes the rest of that
 * loop, cyclically, as a path starting at x + e_mu. */
static int loop_staples(int mu, const Loop* loops, int nloops, Path* out) {
  int n = 0;
  for (int i = 0; i < nloops; ++i)
    for (int k = 0; k < loops[i].n; ++k) {
      if (loops[i].st[k][0] != mu || loops[i].st[k][1] != 1) continue;
      int rot[8][2];
      int m = 0;
      for (int j = 1; j < loops[i].n; ++j) {
        int q = (k + j) % loops[i].n;
        rot[m][0] = loops[i].st[q][0];
        rot[m][1] = loops[i].st[q][1];
        ++m;
      }
      Path p = path_from_steps((const int (*)[2])rot, m);
      for (int j = 0; j < m; ++j) p.l[j].off[mu] += 1;
      out[n++] = p;
    }
  return n;
}

/* Re sum_x sum_{loops of the set and their conjugates} tr loop(x) */
double or_loop_trace(const int L[4], const cdbl* U, int kind) {
  Lat lat = mklat(L);
  Loop loops[24];
  Path paths[24];
  int nl = loop_set(kind, loops);
  for (int i = 0; i < nl; ++i) paths[i] = path_from_steps((const int (*)[2])loops[i].st, loops[i].n);
  double* part = (double*)calloc((size_t)lat.V, sizeof(double));
#pragma omp parallel for schedule(static)
  for (long x = 0; x < lat.V; ++x) {
    cdbl s = 0;
    for (int i = 0; i < nl; ++i) {
      M3 a = eval_links(U, &lat, &paths[i], 0, paths[i].n, x);
      s += mtr(&a);
    }
    part[x] = creal(s);
  }
  double sum = sum_accurate(part, lat.V);
  free(part);
  return sum;
}

/* md_potential of push!(c_plaq, plaq U plaq'), push!(c_rect, rect U rect'):
 * -Re(evaluate_GaugeAction)/NC (src/action/GaugeActions.jl:132-142) */
double or_action_loops(const int L[4], const cdbl* U, double c_plaq, double c_rect) {
  double v = c_plaq * or_loop_trace(L, U, 0);
  if (c_rect != 0.0) v += c_rect * or_loop_trace(L, U, 1);
  return -v / 3.0;
}

/* dS/dU_mu(x) = sum over the sets of c * (staples of U_mu) (calc_dSdUμ!,
 * src/action/GaugeActions.jl:95-123): stp/srp hold the plaquette and
 * rectangle staples of direction mu */
static M3 loops_dsdu_at(const Lat* lat, const cdbl* U, const Path* sp, int nsp, const Path* sr, int nsr,
                        double c_plaq, double c_rect, long x) {
  M3 acc = mzero();
  for (int k = 0; k < nsp; ++k) {
    M3 t = eval_links(U, lat, &sp[k], 0, sp[k].n, x);
    madd(&acc, c_plaq, &t);
  }
  if (c_rect != 0.0)
    for (int k = 0; k < nsr; ++k) {
      M3 t = eval_links(U, lat, &sr[k], 0, sr[k].n, x);
      madd(&acc, c_rect, &t);
    }
  return acc;
}

/* D_mu(x) = dS/dU_mu(x) of every link, in the links' layout (the dS/dUbar
 * input of the stout adjoint for an action with rectangles) */
static void loops_dsdu(const Lat* lat, const cdbl* U, double c_plaq, double c_rect, cdbl* D) {
  Loop lp[12], lr[24];
  int np = loop_set(0, lp), nr = loop_set(1, lr);
  for (int mu = 0; mu < 4; ++mu) {
    Path sp[8], sr[32];
    int nsp = loop_staples(mu, lp, np, sp);
    int nsr = loop_staples(mu, lr, nr, sr);
#pragma omp parallel for schedule(static)
    for (long x = 0; x < lat->V; ++x) {
      M3 acc = loops_dsdu_at(lat, U, sp, nsp, sr, nsr, c_plaq, c_rect, x);
      stm(D, lat, mu, x, &acc);
    }
  }
}

/* dS/dU_mu(x) of the plaquette + rectangle action for every link, in the
 * links' layout (exported for the tests of the device's staple tables) */
void or_dsdu_loops(const int L[4], const cdbl* U, double c_plaq, double c_rect, cdbl* D) {
  Lat lat = mklat(L);
  loops_dsdu(&lat, U, c_plaq, c_rect, D);
}

/* F_mu (+)= factor * TA-coefficients of U_mu dS/dU_mu; accumulate = 0
 * overwrites F. */
static void loops_force(const int L[4], const cdbl* U, double c_plaq, double c_rect, double factor, int accumulate,
                        double* F) {
  Lat lat = mklat(L);
  Loop lp[12], lr[24];
  int np = loop_set(0, lp), nr = loop_set(1, lr);
  for (int mu = 0; mu < 4; ++mu) {
    Path sp[8], sr[32];
    int nsp = loop_staples(mu, lp, np, sp);
    int nsr = loop_staples(mu, lr, nr, sr);
#pragma omp parallel for schedule(static)
    for (long x = 0; x < lat.V; ++x) {
      M3 acc = loops_dsdu_at(&lat, U, sp, nsp, sr, nsr, c_plaq, c_rect, x);
      M3 u = ld(U, &lat, mu, x);
      M3 w = mmul(&u, &acc);
      double* f = F + ((size_t)mu * lat.V + x) * 8;
      if (!accumulate)
        for (int a = 0; a < 8; ++a) f[a] = 0;
      ta_add(f, factor, &w);
    }
  }
}

/* md_force! of the same action: F_mu = TA-coefficients of -(1/3) U_mu dS/dU_mu */
void or_force_loops(const int L[4], const cdbl* U, double c_plaq, double c_rect, double* F) {
  loops_force(L, U, c_plaq, c_rect, -1.0 / 3.0, 0, F);
}

/* number of staples of U_mu in a set (6 for the plaquettes, 18 for the
 * rectangles) */
int or_loop_staple_count(int kind, int mu) {
  Loop loops[24];
  Path st[32];
  int nl = loop_set(kind, loops);
  return loop_staples(mu, loops, nl, st);
}

/* add_U!(P, eps, F) over all directions */
static void mom_axpy(const Lat* lat, double* P, double eps, const double* F) {
  size_t n = (size_t)32 * lat->V;
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < n; ++i) P[i] += eps * F[i];
}

/* exptU! on one link: TA coefficients -> matrix */
void or_expt(double t, const double* u, cdbl* out) {
  M3 e = expt_eigen(t, u);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) out[i + 3 * j] = e.m[i][j];
}

/* update_gaugefields!: U_mu <- exptU!(eps, P_mu) * U_mu */
void or_link_update(const int L[4], cdbl* U, const double* P, double eps) {
  Lat lat = mklat(L);
#pragma omp parallel for schedule(static)
  for (long x = 0; x < lat.V; ++x)
    for (int mu = 0; mu < 4; ++mu) {
      M3 e = expt_eigen(eps, P + ((size_t)mu * lat.V + x) * 8);
      M3 u = ld(U, &lat, mu, x);
      M3 w = mmul(&e, &u);
      stm(U, &lat, mu, x, &w);
    }
}

/* exp_aF_U!: W_mu = exptU!(a, F_mu) U_mu */
static void exp_af_u(const Lat* lat, cdbl* W, double a, const double* F, const cdbl* U) {
#pragma omp parallel for schedule(static)
  for (long x = 0; x < lat->V; ++x)
    for (int mu = 0; mu < 4; ++mu) {
      M3 e = expt_eigen(a, F + ((size_t)mu * lat->V + x) * 8);
      M3 u = ld(U, lat, mu, x);
      M3 w = mmul(&e, &u);
      stm(W, lat, mu, x, &w);
    }
}

double or_kinetic(const int L[4], const double* P) {
  Lat lat = mklat(L);
  size_t n = (size_t)32 * lat.V;
  double* sq = (double*)malloc(sizeof(double) * n);
  for (size_t i = 0; i < n; ++i) sq[i] = P[i] * P[i];
  double s = sum_accurate(sq, (long)n);
  free(sq);
  return s;
}

void or_normalize(const int L[4], cdbl* U) {
  Lat lat = mklat(L);
#pragma omp parallel for schedule(static)
  for (long x = 0; x < lat.V; ++x)
    for (int mu = 0; mu < 4; ++mu) {
      M3 u = ld(U, &lat, mu, x);
      normalize3(&u);
      stm(U, &lat, mu, x, &u);
    }
}

/* ------------------------------------------------------------------------ */
/* stout smearing                                                            */
/* ------------------------------------------------------------------------ */
typedef struct {
  cdbl* Uin;  /* 4 directions */
  cdbl* C;
  cdbl* Q;
  cdbl* eQ;
} Level;

static void stout_level_forward(const Lat* lat, double rho, const cdbl* Uin, cdbl* Uout, Level* keep) {
  Path st[4][6];
  int ns[4];
  for (int mu = 0; mu < 4; ++mu) ns[mu] = cmu_staples(mu, st[mu]);
#pragma omp parallel for schedule(static)
  for (long x = 0; x < lat->V; ++x)
    for (int mu = 0; mu < 4; ++mu) {
      M3 C = mzero();
      for (int k = 0; k < ns[mu]; ++k) {
        M3 t = eval_links(Uin, lat, &st[mu][k], 0, st[mu][k].n, x);
        madd(&C, rho, &t);
      }
      M3 u = ld(Uin, lat, mu, x);
      M3 ud = mdag(&u);
      M3 om = mmul(&C, &ud);
      M3 Q = ta_matrix(&om);
      double c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      ta_add(c, 1.0, &Q);
      M3 eQ = expt_eigen(1.0, c);
      M3 ub = mmul(&eQ, &u);
      stm(Uout, lat, mu, x, &ub);
      if (keep) {
        stm(keep->C, lat, mu, x, &C);
        stm(keep->Q, lat, mu, x, &Q);
        stm(keep->eQ, lat, mu, x, &eQ);
      }
    }
}

/* Forward smearing through nlev plaquette stout layers. */
void or_stout_forward(const int L[4], const cdbl* U, int nlev, const double* rho, cdbl* Uout) {
  Lat lat = mklat(L);
  size_t n = (size_t)36 * lat.V;
  cdbl* a = (cdbl*)malloc(sizeof(cdbl) * n);
  cdbl* b = (cdbl*)malloc(sizeof(cdbl) * n);
  memcpy(a, U, sizeof(cdbl) * n);
  for (int l = 0; l < nlev; ++l) {
    stout_level_forward(&lat, rho[l], a, b, NULL);
    cdbl* t = a;
    a = b;
    b = t;
  }
  memcpy(Uout, a, sizeof(cdbl) * n);
  free(a);
  free(b);
}

/* One layer pull-back (backward_dSdUαUβρ_add! with dSdU cleared first):
 * dSdU = dSdUout e^Q + ((TA(dSdQ)) C)^dag + sum over dC/dU terms. */
static void stout_level_backward(const Lat* lat, double rho, const Level* lv, const cdbl* dSdUout, cdbl* dSdU,
                                 double* dsdrho) {
  size_t n = (size_t)36 * lat->V;
  cdbl* dSdC = (cdbl*)malloc(sizeof(cdbl) * n);
  double rsum = 0;
#pragma omp parallel for schedule(static) reduction(+ : rsum)
  for (long x = 0; x < lat->V; ++x)
    for (int mu = 0; mu < 4; ++mu) {
      M3 dout = ld(dSdUout, lat, mu, x);
      M3 eQ = ld(lv->eQ, lat, mu, x);
      M3 Q = ld(lv->Q, lat, mu, x);
      M3 C = ld(lv->C, lat, mu, x);
      M3 u = ld(lv->Uin, lat, mu, x);
      M3 acc = mmul(&dout, &eQ);                 /* calc_dSdu1! */
      M3 udout = mmul(&u, &dout);
      M3 dsdq = cdexpqdq(&udout, &Q);             /* calc_dSdQ! */
      M3 dsdom = ta_matrix(&dsdq);                /* calc_dSdΩ! */
      M3 ud = mdag(&u);
      M3 dsdc = mmul(&ud, &dsdom);                /* calc_dSdC! */
      M3 dsdudag = mmul(&dsdom, &C);              /* calc_dSdUdag! */
      M3 t = mdag(&dsdudag);
      madd(&acc, 1.0, &t);
      stm(dSdU, lat, mu, x, &acc);
      stm(dSdC, lat, mu, x, &dsdc);
      /* dS/drho = 2 Re tr(dSdC C_unit) with C_unit = C / rho */
      M3 cc = mmul(&dsdc, &C);
      if (rho != 0) rsum += 2 * creal(mtr(&cc)) / rho;
    }
  if (dsdrho) *dsdrho += rsum;
  /* calc_dSdUν_fromdSCμ_add!: for every staple W of C_mu and for W^dag,
   * every forward U_nu inside it at offset pos contributes
   *   dSdU_nu(x) += rho * right(x) * L(x - pos) * left(x - pos)
   * with L = dSdC_mu (W) or dSdC_mu^dag (W^dag). */
  for (int mu = 0; mu < 4; ++mu) {
    Path st[6];
    int ns = cmu_staples(mu, st);
    for (int k = 0; k < 2 * ns; ++k) {
      Path w = (k < ns) ? st[k] : path_dag(&st[k - ns]);
      int dg = (k >= ns);
      for (int j = 0; j < w.n; ++j) {
        if (w.l[j].dag) continue;
        int nu = w.l[j].dir;
        int mpos[4];
        for (int c = 0; c < 4; ++c) mpos[c] = -w.l[j].off[c];
#pragma omp parallel for schedule(static)
        for (long x = 0; x < lat->V; ++x) {
          long y = shifted(lat, x, mpos); /* anchor of W */
          M3 A = eval_links(lv->Uin, lat, &w, 0, j, y);
          M3 B = eval_links(lv->Uin, lat, &w, j + 1, w.n, y);
          M3 Lm = ld(dSdC, lat, mu, y);
          if (dg) Lm = mdag(&Lm);
          M3 BL = mmul(&B, &Lm);
          M3 BLA = mmul(&BL, &A);
          M3 cur = ld(dSdU, lat, nu, x);
          madd(&cur, rho, &BLA);
          stm(dSdU, lat, nu, x, &cur);
        }
      }
    }
  }
  free(dSdC);
}

static void alloc_level(Level* lv, size_t n) {
  lv->Uin = (cdbl*)malloc(sizeof(cdbl) * n);
  lv->C = (cdbl*)malloc(sizeof(cdbl) * n);
  lv->Q = (cdbl*)malloc(sizeof(cdbl) * n);
  lv->eQ = (cdbl*)malloc(sizeof(cdbl) * n);
}
static void free_level(Level* lv) {
  free(lv->Uin);
  free(lv->C);
  free(lv->Q);
  free(lv->eQ);
}

/* back_prop through nlev layers: dSdU (thin) from dSdUbar. Also returns the
 * dS/drho of every layer in dsdrho (may be NULL). */
void or_stout_backward(const int L[4], const cdbl* U, int nlev, const double* rho, const cdbl* dSdUbar, cdbl* dSdU,
                       double* dsdrho) {
  Lat lat = mklat(L);
  size_t n = (size_t)36 * lat.V;
  Level lv[8];
  cdbl* cur = (cdbl*)malloc(sizeof(cdbl) * n);
  memcpy(cur, U, sizeof(cdbl) * n);
  for (int l = 0; l < nlev; ++l) {
    alloc_level(&lv[l], n);
    memcpy(lv[l].Uin, cur, sizeof(cdbl) * n);
    stout_level_forward(&lat, rho[l], lv[l].Uin, cur, &lv[l]);
  }
  cdbl* d = (cdbl*)malloc(sizeof(cdbl) * n);
  cdbl* e = (cdbl*)malloc(sizeof(cdbl) * n);
  memcpy(d, dSdUbar, sizeof(cdbl) * n);
  for (int l = nlev - 1; l >= 0; --l) {
    double r = 0;
    stout_level_backward(&lat, rho[l], &lv[l], d, e, &r);
    if (dsdrho) dsdrho[l] = r;
    cdbl* t = d;
    d = e;
    e = t;
  }
  memcpy(dSdU, d, sizeof(cdbl) * n);
  for (int l = 0; l < nlev; ++l) free_level(&lv[l]);
  free(cur);
  free(d);
  free(e);
}

/* MD force of the Wilson action evaluated on stout-smeared links
 * (P_update! of test/HMCstout_test_nowing.jl:99-118 without the step):
 * F = -(1/3) TA(U dS/dU) with dS/dU back-propagated from beta/2 staples(Ubar). */
void or_stout_force(const int L[4], const cdbl* U, int nlev, const double* rho, double beta, double* F) {
  Lat lat = mklat(L);
  size_t n = (size_t)36 * lat.V;
  if (nlev == 0) {
    or_force(L, U, beta, F);
    return;
  }
  cdbl* Ub = (cdbl*)malloc(sizeof(cdbl) * n);
  cdbl* dbar = (cdbl*)malloc(sizeof(cdbl) * n);
  cdbl* dthin = (cdbl*)malloc(sizeof(cdbl) * n);
  or_stout_forward(L, U, nlev, rho, Ub);
  for (int mu = 0; mu < 4; ++mu) dsdu_mu(&lat, Ub, 0.5 * beta, mu, dbar + (size_t)mu * 9 * lat.V);
  or_stout_backward(L, U, nlev, rho, dbar, dthin, NULL);
#pragma omp parallel for schedule(static)
  for (long x = 0; x < lat.V; ++x)
    for (int mu = 0; mu < 4; ++mu) {
      M3 u = ld(U, &lat, mu, x);
      M3 d = ld(dthin, &lat, mu, x);
      M3 w = mmul(&u, &d);
      double* f = F + ((size_t)mu * lat.V + x) * 8;
      for (int a = 0; a < 8; ++a) f[a] = 0;
      ta_add(f, -1.0 / 3.0, &w);
    }
  free(Ub);
  free(dbar);
  free(dthin);
}

double or_stout_action(const int L[4], const cdbl* U, int nlev, const double* rho, double beta) {
  if (nlev == 0) return or_action(L, U, beta);
  Lat lat = mklat(L);
  size_t n = (size_t)36 * lat.V;
  cdbl* Ub = (cdbl*)malloc(sizeof(cdbl) * n);
  or_stout_forward(L, U, nlev, rho, Ub);
  double v = or_action(L, Ub, beta);
  free(Ub);
  return v;
}

/* ------------------------------------------------------------------------ */
/* MD driver                                                                 */
/* ------------------------------------------------------------------------ */
/* Coefficient of the rectangle loops rect U rect' in the MD action (0: the
 * plain Wilson action); with it the action is thin-link. */
static double g_c_rect = 0.0;
void or_set_rect(double c_rect) { g_c_rect = c_rect; }

/* Force of the plaquette + rectangle action on stout-smeared links: the
 * action's dS/dUbar on the top level (loops_dsdu), back-propagated by the
 * stout adjoint, F = -(1/3) TA(U dS/dU) (the smeared-action force of
 * src/molecular_dynamics.jl:539-551 with a loop-set action) */
void or_stout_force_loops(const int L[4], const cdbl* U, int nlev, const double* rho, double c_plaq, double c_rect,
                          double* F) {
  if (nlev == 0) {
    or_force_loops(L, U, c_plaq, c_rect, F);
    return;
  }
  Lat lat = mklat(L);
  size_t n = (size_t)36 * lat.V;
  cdbl* Ub = (cdbl*)malloc(sizeof(cdbl) * n);
  cdbl* dbar = (cdbl*)malloc(sizeof(cdbl) * n);
  cdbl* dthin = (cdbl*)malloc(sizeof(cdbl) * n);
  or_stout_forward(L, U, nlev, rho, Ub);
  loops_dsdu(&lat, Ub, c_plaq, c_rect, dbar);
  or_stout_backward(L, U, nlev, rho, dbar, dthin, NULL);
#pragma omp parallel for schedule(static)
  for (long x = 0; x < lat.V; ++x)
    for (int mu = 0; mu < 4; ++mu) {
      M3 u = ld(U, &lat, mu, x);
      M3 d = ld(dthin, &lat, mu, x);
      M3 w = mmul(&u, &d);
      double* f = F + ((size_t)mu * lat.V + x) * 8;
      for (int a = 0; a < 8; ++a) f[a] = 0;
      ta_add(f, -1.0 / 3.0, &w);
    }
  free(Ub);
  free(dbar);
  free(dthin);
}

double or_stout_action_loops(const int L[4], const cdbl* U, int nlev, const double* rho, double c_plaq,
                             double c_rect) {
  if (nlev == 0) return or_action_loops(L, U, c_plaq, c_rect);
  Lat lat = mklat(L);
  cdbl* Ub = (cdbl*)malloc(sizeof(cdbl) * (size_t)36 * lat.V);
  or_stout_forward(L, U, nlev, rho, Ub);
  double v = or_action_loops(L, Ub, c_plaq, c_rect);
  free(Ub);
  return v;
}

static void mom_update(const int L[4], double* P, const cdbl* U, double eps, double beta, int nstout, const double* rho,
                       double* F) {
  Lat lat = mklat(L);
  if (g_c_rect != 0.0)
    or_stout_force_loops(L, U, nstout, rho, 0.5 * beta, g_c_rect, F);
  else
    or_stout_force(L, U, nstout, rho, beta, F);
  mom_axpy(&lat, P, eps, F);
}

double or_hamiltonian(const int L[4], const cdbl* U, const double* P, double beta, int nstout, const double* rho) {
  double v = (g_c_rect != 0.0) ? or_stout_action_loops(L, U, nstout, rho, 0.5 * beta, g_c_rect)
                               : or_stout_action(L, U, nstout, rho, beta);
  return v + or_kinetic(L, P) / 2;
}

static double g_omelyan_lambda = 0.1931833275037836;
void or_set_omelyan_lambda(double lam) { g_omelyan_lambda = lam; }

/* md_trajectory!: integrator 0 = QPQ, 1 = PQP, 2 = Omelyan PQPQP (the custom
 * integrator of docs/src/hmc.md:250-270); out = {H0, H1, dH} */
void or_md_trajectory(const int L[4], cdbl* U, double* P, double beta, double tau, int steps, int integrator,
                      int nstout, const double* rho, double* out) {
  Lat lat = mklat(L);
  double* F = (double*)malloc(sizeof(double) * 32 * (size_t)lat.V);
  double H0 = or_hamiltonian(L, U, P, beta, nstout, rho);
  double eps = tau / steps;
  for (int s = 0; s < steps; ++s) {
    if (integrator == 0) {
      or_link_update(L, U, P, eps / 2);
      mom_update(L, P, U, eps, beta, nstout, rho, F);
      or_link_update(L, U, P, eps / 2);
    } else if (integrator == 1) {
      mom_update(L, P, U, eps / 2, beta, nstout, rho, F);
      or_link_update(L, U, P, eps);
      mom_update(L, P, U, eps / 2, beta, nstout, rho, F);
    } else {
      double lam = g_omelyan_lambda;
      mom_update(L, P, U, lam * eps, beta, nstout, rho, F);
      or_link_update(L, U, P, eps / 2);
      mom_update(L, P, U, (1 - 2 * lam) * eps, beta, nstout, rho, F);
      or_link_update(L, U, P, eps / 2);
      mom_update(L, P, U, lam * eps, beta, nstout, rho, F);
    }
  }
  double H1 = or_hamiltonian(L, U, P, beta, nstout, rho);
  out[0] = H0;
  out[1] = H1;
  out[2] = H1 - H0;
  free(F);
}

/* One MD step only (for the bounded CPU-baseline sample). */
void or_md_steps(const int L[4], cdbl* U, double* P, double beta, double eps, int nsteps, int nstout, const double* rho) {
  Lat lat = mklat(L);
  double* F = (double*)malloc(sizeof(double) * 32 * (size_t)lat.V);
  for (int s = 0; s < nsteps; ++s) {
    or_link_update(L, U, P, eps / 2);
    mom_update(L, P, U, eps, beta, nstout, rho, F);
    or_link_update(L, U, P, eps / 2);
  }
  free(F);
}

/* ------------------------------------------------------------------------ */
/* gradient flow                                                             */
/* ------------------------------------------------------------------------ */
/* add_force!(F, U; plaqonly=true): F += factor * TA(U_mu V_mu^dag) with V the
 * six MP staples (construct_double_staple!) */
void or_flow_force(const int L[4], const cdbl* U, double* F, double factor) {
  Lat lat = mklat(L);
  Path st[4][6];
  int ns[4];
  for (int mu = 0; mu < 4; ++mu) ns[mu] = cmu_staples(mu, st[mu]);
#pragma omp parallel for schedule(static)
  for (long x = 0; x < lat.V; ++x)
    for (int mu = 0; mu < 4; ++mu) {
      M3 V = mzero();
      for (int k = 0; k < ns[mu]; ++k) {
        M3 t = eval_links(U, &lat, &st[mu][k], 0, st[mu][k].n, x);
        madd(&V, 1.0, &t);
      }
      M3 u = ld(U, &lat, mu, x);
      M3 vd = mdag(&V);
      M3 w = mmul(&u, &vd);
      ta_add(F + ((size_t)mu * lat.V + x) * 8, factor, &w);
    }
}

void or_flow(const int L[4], cdbl* U, double eps, int nsteps) {
  Lat lat = mklat(L);
  size_t nf = (size_t)32 * lat.V, nl = (size_t)36 * lat.V;
  double* F0 = (double*)malloc(sizeof(double) * nf);
  double* F1 = (double*)malloc(sizeof(double) * nf);
  double* F2 = (double*)malloc(sizeof(double) * nf);
  double* Ft = (double*)malloc(sizeof(double) * nf);
  cdbl* W1 = (cdbl*)malloc(sizeof(cdbl) * nl);
  cdbl* W2 = (cdbl*)malloc(sizeof(cdbl) * nl);
  for (int s = 0; s < nsteps; ++s) {
    memset(F0, 0, sizeof(double) * nf);
    or_flow_force(L, U, F0, 1.0);
    exp_af_u(&lat, W1, -eps / 4, F0, U);
    memset(F1, 0, sizeof(double) * nf);
    or_flow_force(L, W1, F1, 1.0);
    memset(Ft, 0, sizeof(double) * nf);
    mom_axpy(&lat, Ft, -(8 * eps / 9), F1);
    mom_axpy(&lat, Ft, 17 * eps / 36, F0);
    exp_af_u(&lat, W2, 1.0, Ft, W1);
    memset(F2, 0, sizeof(double) * nf);
    or_flow_force(L, W2, F2, 1.0);
    memset(Ft, 0, sizeof(double) * nf);
    mom_axpy(&lat, Ft, -(3 * eps / 4), F2);
    mom_axpy(&lat, Ft, 8 * eps / 9, F1);
    mom_axpy(&lat, Ft, -(17 * eps / 36), F0);
    exp_af_u(&lat, U, 1.0, Ft, W2);
  }
  free(F0);
  free(F1);
  free(F2);
  free(Ft);
  free(W1);
  free(W2);
}

/* flow!(U, ::Gradientflow_general) (src/smearing/gradientflow.jl:240-336): the
 * same RK3 steps with the force F_update!(F, U, 1, Dim, action) = TA(U dS/dU)
 * of the action holding c_plaq (plaq U plaq') and c_rect (rect U rect'),
 * gradient_flow(U, loops, coefficients) of src/API.jl:426-438. */
void or_flow_loops(const int L[4], cdbl* U, double eps, int nsteps, double c_plaq, double c_rect) {
  Lat lat = mklat(L);
  size_t nf = (size_t)32 * lat.V, nl = (size_t)36 * lat.V;
  double* F0 = (double*)malloc(sizeof(double) * nf);
  double* F1 = (double*)malloc(sizeof(double) * nf);
  double* F2 = (double*)malloc(sizeof(double) * nf);
  double* Ft = (double*)malloc(sizeof(double) * nf);
  cdbl* W1 = (cdbl*)malloc(sizeof(cdbl) * nl);
  cdbl* W2 = (cdbl*)malloc(sizeof(cdbl) * nl);
  for (int s = 0; s < nsteps; ++s) {
    loops_force(L, U, c_plaq, c_rect, 1.0, 0, F0);
    exp_af_u(&lat, W1, -eps / 4, F0, U);
    loops_force(L, W1, c_plaq, c_rect, 1.0, 0, F1);
    memset(Ft, 0, sizeof(double) * nf);
    mom_axpy(&lat, Ft, -(8 * eps / 9), F1);
    mom_axpy(&lat, Ft, 17 * eps / 36, F0);
    exp_af_u(&lat, W2, 1.0, Ft, W1);
    loops_force(L, W2, c_plaq, c_rect, 1.0, 0, F2);
    memset(Ft, 0, sizeof(double) * nf);
    mom_axpy(&lat, Ft, -(3 * eps / 4), F2);
    mom_axpy(&lat, Ft, 8 * eps / 9, F1);
    mom_axpy(&lat, Ft, -(17 * eps / 36), F0);
    exp_af_u(&lat, U, 1.0, Ft, W2);
  }
  free(F0);
  free(F1);
  free(F2);
  free(Ft);
  free(W1);
  free(W2);
}

/* ------------------------------------------------------------------------ */
/* random starts: Philox4x32-10 (Salmon et al., SC'11) with the same counter  */
/* layout as the library, so the oracle can regenerate the GPU's inputs.      */
/* counter = (lex, (mu << 8) | block, word2, tag ^ word3), key = seed.        */
/* ------------------------------------------------------------------------ */
static void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}
static double u01(uint32_t a, uint32_t b) {
  uint64_t m = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
  return ((double)m + 0.5) * (1.0 / 9007199254740992.0);
}
static void gauss_pair(const uint32_t r[4], double sigma, double* g1, double* g2) {
  double u1 = u01(r[0], r[1]), u2 = u01(r[2], r[3]);
  double rad = sigma * sqrt(-2.0 * log(u1));
  *g1 = rad * cos(2.0 * M_PI * u2);
  *g2 = rad * sin(2.0 * M_PI * u2);
}

/* Haar-random SU(3): Gaussian 3x3 (re, im ~ N(0,1/2)), Gram-Schmidt of the
 * rows, determinant phase divided out (principal branch). */
void or_hot_start(const int L[4], cdbl* U, uint64_t seed) {
  Lat lat = mklat(L);
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
#pragma omp parallel for schedule(static)
  for (long x = 0; x < lat.V; ++x)
    for (int mu = 0; mu < 4; ++mu) {
      M3 m;
      for (int k = 0; k < 9; ++k) {
        uint32_t c[4] = {(uint32_t)x, ((uint32_t)mu << 8) | (uint32_t)k, 0u, 0x48415252u};
        philox(c, k0, k1);
        double a, b;
        gauss_pair(c, 0.70710678118654752440, &a, &b);
        m.m[k / 3][k % 3] = a + I * b;
      }
      for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < i; ++j) {
          cdbl pr = 0;
          for (int k = 0; k < 3; ++k) pr += conj(m.m[j][k]) * m.m[i][k];
          for (int k = 0; k < 3; ++k) m.m[i][k] -= pr * m.m[j][k];
        }
        double nn = 0;
        for (int k = 0; k < 3; ++k) nn += creal(m.m[i][k] * conj(m.m[i][k]));
        double inv = 1.0 / sqrt(nn);
        for (int k = 0; k < 3; ++k) m.m[i][k] *= inv;
      }
      cdbl d = m.m[0][0] * (m.m[1][1] * m.m[2][2] - m.m[1][2] * m.m[2][1]) -
               m.m[0][1] * (m.m[1][0] * m.m[2][2] - m.m[1][2] * m.m[2][0]) +
               m.m[0][2] * (m.m[1][0] * m.m[2][1] - m.m[1][1] * m.m[2][0]);
      double phi = atan2(cimag(d), creal(d)) / 3.0;
      cdbl ph = cos(phi) - I * sin(phi);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) m.m[i][j] *= ph;
      stm(U, &lat, mu, x, &m);
    }
}

/* The reference's legacy hot start distribution
 * (randomGaugefields_4D_nowing, gaugefields_4D_nowing.jl:240-279):
 * entries rand()-0.5 + i(rand()-0.5), then normalize_U!. The uniform stream
 * here is Philox (the reference uses StableRNG(123), not reproducible here). */
void or_uniform_hot_start(const int L[4], cdbl* U, uint64_t seed) {
  Lat lat = mklat(L);
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
#pragma omp parallel for schedule(static)
  for (long x = 0; x < lat.V; ++x)
    for (int mu = 0; mu < 4; ++mu) {
      M3 m;
      for (int k = 0; k < 9; ++k) {
        uint32_t c[4] = {(uint32_t)x, ((uint32_t)mu << 8) | (uint32_t)k, 0u, 0x554E4946u};
        philox(c, k0, k1);
        m.m[k % 3][k / 3] = (u01(c[0], c[1]) - 0.5) + I * (u01(c[2], c[3]) - 0.5);
      }
      normalize3(&m);
      stm(U, &lat, mu, x, &m);
    }
}

void or_gauss_mom(const int L[4], double* P, uint64_t seed, uint64_t sweep) {
  Lat lat = mklat(L);
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
#pragma omp parallel for schedule(static)
  for (long x = 0; x < lat.V; ++x)
    for (int mu = 0; mu < 4; ++mu)
      for (int k = 0; k < 4; ++k) {
        uint32_t c[4] = {(uint32_t)x, ((uint32_t)mu << 8) | (uint32_t)k, (uint32_t)sweep,
                         0x4D4F4D30u ^ (uint32_t)(sweep >> 32)};
        philox(c, k0, k1);
        double a, b;
        gauss_pair(c, 1.0, &a, &b);
        P[((size_t)mu * lat.V + x) * 8 + 2 * k] = a;
        P[((size_t)mu * lat.V + x) * 8 + 2 * k + 1] = b;
      }
}

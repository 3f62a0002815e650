// Host-side accuracy check of the double-float 3x3 products of su3.cuh
// (their device and host forms are the same source): random complex
// Gaussian matrices in double-float, products against long double. Prints
// one line per measurement: name, max and rms error relative to
// |row i of A| |column j of B| (+ |C_ij| when accumulating).
#include <cmath>
#include <cstdio>
#include <random>

#include "su3.cuh"

using namespace gf;
typedef long double ld;

static ld val(const dfl& x) { return (ld)x.hi + (ld)x.lo; }

static void rnd(mat3<dfl>& m, std::mt19937_64& g, double s) {
  std::normal_distribution<double> nd(0.0, s);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) m.e[i][j] = mk(dfl(nd(g)), dfl(nd(g)));
}

// max and rms of |R - (A B + C)| / (|a_i| |b_j| + |C_ij|) over the entries
static void err(const mat3<dfl>& A, const mat3<dfl>& B, const mat3<dfl>* C, const mat3<dfl>& R, double& mx,
                double& s2, long& n) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      ld sr = C ? val(C->e[i][j].re) : 0, si = C ? val(C->e[i][j].im) : 0, ra = 0, cb = 0;
      for (int k = 0; k < 3; ++k) {
        const ld ar = val(A.e[i][k].re), ai = val(A.e[i][k].im), br = val(B.e[k][j].re), bi = val(B.e[k][j].im);
        sr += ar * br - ai * bi;
        si += ar * bi + ai * br;
        ra += ar * ar + ai * ai;
        cb += br * br + bi * bi;
      }
      const ld m = sqrtl(ra * cb) + (C ? sqrtl(val(C->e[i][j].re) * val(C->e[i][j].re) +
                                                 val(C->e[i][j].im) * val(C->e[i][j].im))
                                       : 0);
      const double e = (double)(fmaxl(fabsl(val(R.e[i][j].re) - sr), fabsl(val(R.e[i][j].im) - si)) / m);
      mx = fmax(mx, e);
      s2 += e * e;
      ++n;
    }
}

int main() {
  std::mt19937_64 g(11);
  const int N = 40000;
  double gm = 0, gs = 0, tm = 0, ts = 0, am = 0, as = 0, rm = 0, rs = 0;
  long gn = 0, tn = 0, an = 0, rn = 0;
  for (int t = 0; t < N; ++t) {
    const double s = std::pow(10.0, (t % 7) - 3);  // scales 1e-3 .. 1e3
    mat3<dfl> A, B, C;
    rnd(A, g, s);
    rnd(B, g, 1.0 / std::sqrt(3.0));
    rnd(C, g, s);
    err(A, B, nullptr, dfg_matmul<false, false, false>(A, B, nullptr), gm, gs, gn);
    err(A, B, nullptr, df_matmul<false, false, false>(A, B, nullptr), tm, ts, tn);
    err(A, B, &C, dfg_matmul<false, false, true>(A, B, &C), am, as, an);
    // a raw grid pair (NORM = false) used as the next product's operand
    const mat3<dfl> raw = dfg_matmul<false, false, false, 3, false>(A, B, nullptr);
    const mat3<dfl> nrm = dfg_matmul<false, false, false>(A, B, nullptr);
    err(nrm, C, nullptr, dfg_matmul<false, false, false>(raw, C, nullptr), rm, rs, rn);
  }
  std::printf("grid %.4e %.4e\n", gm, std::sqrt(gs / gn));
  std::printf("twosum %.4e %.4e\n", tm, std::sqrt(ts / tn));
  std::printf("grid_acc %.4e %.4e\n", am, std::sqrt(as / an));
  std::printf("grid_raw_operand %.4e %.4e\n", rm, std::sqrt(rs / rn));
  return 0;
}

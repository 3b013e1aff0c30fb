// Tabulated pair functions of the FP64 form: cubic Hermite tables in s = r^2
// of the vdW + Coulomb energy and force factor (vdW_Coulomb_Energy_Full_C,
// reaxc_nonbonded_sw64.c:40-258) and of the QEq matrix element H_ij
// (compute_H_Full_C, fix_qeq_reax_sw64.c:768-911), per unordered type pair.
//
// The reference has a cubic-spline long-range table (LR_lookup_table,
// reaxc_ctypes_sunway.h:832-860) that its NULL control path leaves off
// (tabulate = 0).  Here the table replaces the FP64 transcendental work of
// the pair kernels (two exp, two log and a cube root per pair, ~240 FP64
// instructions, on a GPU whose FP64 rate is 1/64 of its FP32 rate) by ~30
// FP64 instructions and 96 L2-resident bytes.  Interpolating in s needs no
// square root, and (1/r) dE/dr = 2 dE/ds.  Each node holds the function
// and its s-derivative (the reference's own force expression, halved), and
// for the force factor its s-derivative by a fourth-order central
// difference; with 65536 intervals on [0.25, rc^2] A^2 the interpolants
// agree with the analytic expressions to ~1e-10 (relative to
// max(|f|, 1e-4 max|f|); checked here, rg_table_info), inside the 1e-9
// parity bars.
#include <algorithm>
#include <cmath>
#include <thread>
#include <utility>
#include <vector>

#include "rg_internal.h"

namespace {

double taper_poly(const double *T, double r) {
  double t = T[7];
  for (int k = 6; k >= 0; --k) t = t * r + T[k];
  return t;
}

// (1/r) dTap/dr
double taper_dr(const double *T, double r) {
  double d = 7 * T[7];
  for (int k = 6; k >= 2; --k) d = d * r + k * T[k];
  return d + T[1] / r;
}

// The reference's pair terms at distance r (reaxc_nonbonded_sw64.c:40-258):
// vdW energy (with core and low-gradient terms) and its (1/r) dE/dr, and the
// Coulomb energy and force factor per unit C_ele qi qj.
void pair_funcs(const ForceField &F, const Control &C, int ti, int tj, double r, double *ev,
                double *cv, double *ec, double *cc) {
  const Tbp &tw = F.tbp[ti][tj];
  const double d2 = r * r;
  const double Tp = taper_poly(C.Tap, r), dTap = taper_dr(C.Tap, r);
  const double p_vdW1 = F.gp[28];
  double e_vdW, CEvd, e_core = 0, e_lg = 0;
  if (F.vdw_type == 1 || F.vdw_type == 3) {
    const double powr = std::pow(r, p_vdW1);
    const double S = powr + tw.powgi_vdW1;
    const double fn13 = std::pow(S, 1.0 / p_vdW1);
    const double exp1 = std::exp(tw.alpha * (1.0 - fn13 / tw.r_vdW));
    const double exp2 = std::exp(0.5 * tw.alpha * (1.0 - fn13 / tw.r_vdW));
    e_vdW = tw.D * (exp1 - 2.0 * exp2);
    const double dfn13 = std::pow(S, 1.0 / p_vdW1 - 1.0) * std::pow(r, p_vdW1 - 2.0);
    CEvd = dTap * e_vdW - Tp * tw.D * (tw.alpha / tw.r_vdW) * (exp1 - exp2) * dfn13;
  } else {
    const double exp1 = std::exp(tw.alpha * (1.0 - r / tw.r_vdW));
    const double exp2 = std::exp(0.5 * tw.alpha * (1.0 - r / tw.r_vdW));
    e_vdW = tw.D * (exp1 - 2.0 * exp2);
    CEvd = dTap * e_vdW - Tp * tw.D * (tw.alpha / tw.r_vdW) * (exp1 - exp2) / r;
  }
  if (F.vdw_type == 2 || F.vdw_type == 3) {
    e_core = tw.ecore * std::exp(tw.acore * (1.0 - r / tw.rcore));
    const double de_core = -(tw.acore / tw.rcore) * e_core;
    CEvd += dTap * e_core + Tp * de_core / r;
    if (C.lgflag) {
      const double r5 = d2 * d2 * r, r6 = d2 * d2 * d2, re6 = std::pow(tw.lgre, 6.0);
      e_lg = -(tw.lgcij / (r6 + re6));
      const double de_lg = -6.0 * e_lg * r5 / (r6 + re6);
      CEvd += dTap * e_lg + Tp * de_lg / r;
    }
  }
  *ev = Tp * (e_vdW + e_core + e_lg);
  *cv = CEvd;
  const double dr3 = d2 * r + tw.gamma;
  const double inv3 = std::pow(dr3, -0.33333333333333);
  *ec = Tp * inv3;
  *cc = (dTap - Tp * r / dr3) * inv3;
}

// QEq H_ij = Tap_q(r) 14.4 / (r^3 + shld)^0.3333333333333 (fix_qeq_reax_sw64.c:146-181)
double h_func(const ForceField &F, const Control &C, int ti, int tj, double r) {
  const double Tp = taper_poly(C.qTap, r);
  return Tp * 14.4 * std::pow(r * r * r + F.tbp[ti][tj].gamma, -0.3333333333333);
}

// fourth-order central difference of g at s (step h)
template <typename G>
double deriv(G g, double s, double h) {
  return (-g(s + 2 * h) + 8 * g(s + h) - 8 * g(s - h) + g(s - 2 * h)) / (12 * h);
}

double hermite(double y0, double d0, double y1, double d1, double u, double ds) {
  const double u2 = u * u;
  const double h01 = u2 * (3.0 - 2.0 * u), h00 = 1.0 - h01;
  const double h10 = ds * u * (1.0 - u) * (1.0 - u), h11 = ds * u2 * (u - 1.0);
  return h00 * y0 + h01 * y1 + h10 * d0 + h11 * d1;
}

}  // namespace

int rg_pair_index(int ti, int tj, int nt) {
  if (ti > tj) std::swap(ti, tj);
  return ti * nt - ti * (ti - 1) / 2 + (tj - ti);
}

// Fills nb[npair][n+1][6] = {Ev, Dv, ds Dv', Ec, Dc, ds Dc'} (D = dE/ds,
// ' = d/ds, ds the node spacing) per node and hq[npair][n][4] = the Hermite
// cubic of H (nodes H, ds H') per interval in the power basis
// c0 + u (c1 + u (c2 + u c3)), u in [0, 1] (three FMAs and no weights on the
// device; the same 32 bytes per evaluation), over s in [s0, s1] with n
// intervals; with
// check, returns the largest deviation of the interpolants from the
// analytic functions at 5 interior points of every interval (else 0).
double rg_build_tables(const ForceField &F, const Control &C, int n, double s0, double s1,
                       std::vector<double> &nb, std::vector<double> &hq, bool check) {
  const int nt = F.ntypes;
  const int np = nt * (nt + 1) / 2;
  const double ds = (s1 - s0) / n;
  nb.assign((size_t)np * (n + 1) * 6, 0.0);
  hq.assign((size_t)np * n * 4, 0.0);
  std::vector<std::pair<int, int>> pairs;
  for (int ti = 0; ti < nt; ++ti)
    for (int tj = ti; tj < nt; ++tj) pairs.emplace_back(ti, tj);
  std::vector<double> worst_of(pairs.size(), 0.0);
  // one host thread per type pair
  auto build_pair = [&](size_t w) {
    const int ti = pairs[w].first, tj = pairs[w].second;
    double worst = 0.0;
    {
      const int p = rg_pair_index(ti, tj, nt);
      auto ev = [&](double s) { double a, b, c, d; pair_funcs(F, C, ti, tj, std::sqrt(s), &a, &b, &c, &d); return a; };
      auto dv = [&](double s) { double a, b, c, d; pair_funcs(F, C, ti, tj, std::sqrt(s), &a, &b, &c, &d); return 0.5 * b; };
      auto ecf = [&](double s) { double a, b, c, d; pair_funcs(F, C, ti, tj, std::sqrt(s), &a, &b, &c, &d); return c; };
      auto dc = [&](double s) { double a, b, c, d; pair_funcs(F, C, ti, tj, std::sqrt(s), &a, &b, &c, &d); return 0.5 * d; };
      auto hf = [&](double s) { return h_func(F, C, ti, tj, std::sqrt(s)); };
      const double h = 1e-4;
      double hy0 = 0.0, hp0 = 0.0;
      for (int k = 0; k <= n; ++k) {
        const double s = s0 + k * ds;
        double *e = &nb[((size_t)p * (n + 1) + k) * 6];
        e[0] = ev(s);
        e[1] = dv(s);
        e[2] = ds * deriv(dv, s, h);
        e[3] = ecf(s);
        e[4] = dc(s);
        e[5] = ds * deriv(dc, s, h);
        // H: the Hermite cubic of each interval in the power basis of u
        const double hy1 = hf(s), hp1 = ds * deriv(hf, s, h);
        if (k > 0) {
          double *q = &hq[((size_t)p * n + (k - 1)) * 4];
          q[0] = hy0;
          q[1] = hp0;
          q[2] = 3.0 * (hy1 - hy0) - 2.0 * hp0 - hp1;
          q[3] = 2.0 * (hy0 - hy1) + hp0 + hp1;
        }
        hy0 = hy1;
        hp0 = hp1;
      }
      if (!check) return;
      // accuracy of the interpolants against the analytic functions:
      // relative error where |f| >= 1e-4 max|f|, absolute error in units of
      // 1e-4 max|f| below (near zero crossings and the taper's end, where the
      // analytic form itself carries the expanded polynomial's cancellation)
      double M[5] = {0, 0, 0, 0, 0};
      for (int k = 0; k <= n; ++k) {
        const double *e = &nb[((size_t)p * (n + 1) + k) * 6];
        M[0] = std::max(M[0], std::fabs(e[0]));
        M[1] = std::max(M[1], std::fabs(2.0 * e[1]));
        M[2] = std::max(M[2], std::fabs(e[3]));
        M[3] = std::max(M[3], std::fabs(2.0 * e[4]));
        if (k < n) M[4] = std::max(M[4], std::fabs(hq[((size_t)p * n + k) * 4]));
      }
      for (int k = 0; k < n; ++k) {
        const double *a = &nb[((size_t)p * (n + 1) + k) * 6], *b = a + 6;
        const double *qc = &hq[((size_t)p * n + k) * 4];
        for (int m = 1; m <= 5; ++m) {
          const double u = m / 6.0, s = s0 + (k + u) * ds;
          double x[4];
          pair_funcs(F, C, ti, tj, std::sqrt(s), &x[0], &x[1], &x[2], &x[3]);
          const double iv[4] = {hermite(a[0], a[1], b[0], b[1], u, ds),
                                2.0 * hermite(a[1], a[2], b[1], b[2], u, 1.0),
                                hermite(a[3], a[4], b[3], b[4], u, ds),
                                2.0 * hermite(a[4], a[5], b[4], b[5], u, 1.0)};
          for (int c = 0; c < 4; ++c) {
            const double scale = std::max(std::fabs(x[c]), 1e-4 * M[c]);
            if (scale > 0.0) worst = std::max(worst, std::fabs(iv[c] - x[c]) / scale);
          }
          const double hv = ((qc[3] * u + qc[2]) * u + qc[1]) * u + qc[0], hx = hf(s);
          const double hs = std::max(std::fabs(hx), 1e-4 * M[4]);
          if (hs > 0.0) worst = std::max(worst, std::fabs(hv - hx) / hs);
        }
      }
    }
    worst_of[w] = worst;
  };
  std::vector<std::thread> th;
  for (size_t w = 0; w < pairs.size(); ++w) th.emplace_back(build_pair, w);
  for (auto &x : th) x.join();
  double worst = 0.0;
  for (double v : worst_of) worst = std::max(worst, v);
  return worst;
}

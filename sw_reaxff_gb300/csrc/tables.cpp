// Tabulated pair functions of the FP64 form: cubic Hermite tables in s = r^2
// of the vdW + Coulomb energy and force factor (vdW_Coulomb_Energy_Full_C,
// reaxc_nonbonded_sw64.c:40-258) and of the QEq matrix element H_ij
// (compute_H_Full_C, fix_qeq_reax_sw64.c:768-911), per unordered type pair.
//
// The reference has a cubic-spline long-range table (LR_lookup_table,
// reaxc_ctypes_sunway.h:832-860) that its NULL control path leaves off
// (tabulate = 0).  Here the table replaces the FP64 transcendental work of
// the pair kernels (two exp, two log and a cube root per pair, ~240 FP64
// instructions, on a GPU whose FP64 rate is 1/64 of its FP32 rate) by ten
// FP64 instructions and 64 L2-resident bytes per pair on force-only steps.  Interpolating in s needs no
// square root, and (1/r) dE/dr = 2 dE/ds.  Each interval's cubic matches
// the function and its s-derivative at both ends (the energies' derivative
// is the reference's own force expression, halved; the force factors'
// derivatives are fourth-order central differences); with 65536 intervals on [0.25, rc^2] A^2 the interpolants
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


}  // namespace

int rg_pair_index(int ti, int tj, int nt) {
  if (ti > tj) std::swap(ti, tj);
  return ti * nt - ti * (ti - 1) / 2 + (tj - ti);
}

// Fills, per type pair and interval of s in [s0, s1] (n intervals of width
// ds), the Hermite cubic of each tabulated function in the power basis of
// u in [0, 1]: c0 + u (c1 + u (c2 + u c3)) (three FMAs, no weights):
//   nb[npair][n][16] = { Fv[4], Fc[4], Ev[4], Ec[4] }
//     Fv = (1/r) dE_vdW/dr = 2 dE_vdW/ds, Fc = C_ele (1/r) dE_ele/dr per
//     unit qi qj, Ev = the tapered vdW energy, Ec = C_ele Tap/(r^3+g)^c;
//     the force factors come first (the 64 bytes a force-only step reads)
//   hq[npair][n][4] = H_ij
// from node values and s-derivatives (the force factors' own derivatives by
// a fourth-order central difference).  With check, returns the largest
// deviation of the interpolants from the analytic functions at 5 interior
// points of every interval (else 0).
double rg_build_tables(const ForceField &F, const Control &C, int n, double s0, double s1,
                       std::vector<double> &nb, std::vector<double> &hq, bool check) {
  const int nt = F.ntypes;
  const int np = nt * (nt + 1) / 2;
  const double ds = (s1 - s0) / n;
  nb.assign((size_t)np * n * 16, 0.0);
  hq.assign((size_t)np * n * 4, 0.0);
  std::vector<std::pair<int, int>> pairs;
  for (int ti = 0; ti < nt; ++ti)
    for (int tj = ti; tj < nt; ++tj) pairs.emplace_back(ti, tj);
  std::vector<double> worst_of(pairs.size(), 0.0);
  // one host thread per type pair
  auto build_pair = [&](size_t w) {
    const int ti = pairs[w].first, tj = pairs[w].second;
    const int p = rg_pair_index(ti, tj, nt);
    auto funcs = [&](double s, double *o) {
      pair_funcs(F, C, ti, tj, std::sqrt(s), &o[0], &o[1], &o[2], &o[3]);
      o[2] *= RG_C_ELE;
      o[3] *= RG_C_ELE;
    };
    auto fv = [&](double s) { double o[4]; funcs(s, o); return o[1]; };
    auto fc = [&](double s) { double o[4]; funcs(s, o); return o[3]; };
    auto hf = [&](double s) { return h_func(F, C, ti, tj, std::sqrt(s)); };
    const double h = 1e-4;
    // node values y and s-derivatives dy of Fv, Fc, Ev, Ec, H
    std::vector<double> y((size_t)(n + 1) * 5), dy((size_t)(n + 1) * 5);
    for (int k = 0; k <= n; ++k) {
      const double s = s0 + k * ds;
      double o[4];
      funcs(s, o);
      double *Y = &y[(size_t)k * 5], *D = &dy[(size_t)k * 5];
      Y[0] = o[1];
      D[0] = deriv(fv, s, h);
      Y[1] = o[3];
      D[1] = deriv(fc, s, h);
      Y[2] = o[0];
      D[2] = 0.5 * o[1];      // dEv/ds = (1/2)(1/r) dEv/dr
      Y[3] = o[2];
      D[3] = 0.5 * o[3];
      Y[4] = hf(s);
      D[4] = deriv(hf, s, h);
    }
    auto coeffs = [&](int k, int f, double *c) {
      const double y0 = y[(size_t)k * 5 + f], y1 = y[(size_t)(k + 1) * 5 + f];
      const double p0 = ds * dy[(size_t)k * 5 + f], p1 = ds * dy[(size_t)(k + 1) * 5 + f];
      c[0] = y0;
      c[1] = p0;
      c[2] = 3.0 * (y1 - y0) - 2.0 * p0 - p1;
      c[3] = 2.0 * (y0 - y1) + p0 + p1;
    };
    for (int k = 0; k < n; ++k) {
      double *e = &nb[((size_t)p * n + k) * 16];
      for (int f = 0; f < 4; ++f) coeffs(k, f, e + 4 * f);
      coeffs(k, 4, &hq[((size_t)p * n + k) * 4]);
    }
    if (!check) return;
    // accuracy of the interpolants against the analytic functions:
    // relative error where |f| >= 1e-4 max|f|, absolute error in units of
    // 1e-4 max|f| below (near zero crossings and the taper's end, where the
    // analytic form itself carries the expanded polynomial's cancellation)
    double M[5] = {0, 0, 0, 0, 0};
    for (int k = 0; k <= n; ++k)
      for (int f = 0; f < 5; ++f) M[f] = std::max(M[f], std::fabs(y[(size_t)k * 5 + f]));
    double worst = 0.0;
    for (int k = 0; k < n; ++k) {
      const double *e = &nb[((size_t)p * n + k) * 16];
      const double *qc = &hq[((size_t)p * n + k) * 4];
      for (int m = 1; m <= 5; ++m) {
        const double u = m / 6.0, s = s0 + (k + u) * ds;
        double o[4];
        funcs(s, o);
        const double x[5] = {o[1], o[3], o[0], o[2], hf(s)};
        for (int f = 0; f < 5; ++f) {
          const double *c = f < 4 ? e + 4 * f : qc;
          const double iv = ((c[3] * u + c[2]) * u + c[1]) * u + c[0];
          const double scale = std::max(std::fabs(x[f]), 1e-4 * M[f]);
          if (scale > 0.0) worst = std::max(worst, std::fabs(iv - x[f]) / scale);
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

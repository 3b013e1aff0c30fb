// Force-field reader.  Restates the reference's Read_Force_Field
// (reaxc_ffield_sunway.cpp:35-714): global parameters, per-element (sbp),
// bond (tbp), off-diagonal, angle (thbp), torsion (fbp, with the 0-X-Y-0
// wildcard form) and hydrogen-bond (hbp) blocks, plus the mixing rules and
// the vdW-type selection.  The layout of ForceField is this library's own.
#include <cctype>
#include <cmath>
#include <cstring>
#include <fstream>
#include <sstream>

#include "rg_internal.h"

namespace {

struct LineReader {
  std::ifstream in;
  std::vector<std::string> tok;
  bool next() {
    std::string line;
    if (!std::getline(in, line)) return false;
    tok.clear();
    // '!' starts a comment in the ffield header lines
    for (char &c : line)
      if (c == '!') c = ' ';
    std::istringstream ss(line);
    std::string t;
    while (ss >> t) tok.push_back(t);
    return true;
  }
  double d(size_t i) const { return i < tok.size() ? std::atof(tok[i].c_str()) : 0.0; }
  int i(size_t k) const { return k < tok.size() ? std::atoi(tok[k].c_str()) : 0; }
};

}  // namespace

void rg_init_taper(double swa, double swb, double *Tap) {
  // 7th-order taper, Init_Taper reaxc_init_md_sunway.cpp:100-136
  const double d7 = std::pow(swb - swa, 7.0);
  const double a2 = swa * swa, a3 = a2 * swa, b2 = swb * swb, b3 = b2 * swb;
  Tap[7] = 20.0 / d7;
  Tap[6] = -70.0 * (swa + swb) / d7;
  Tap[5] = 84.0 * (a2 + 3.0 * swa * swb + b2) / d7;
  Tap[4] = -35.0 * (a3 + 9.0 * a2 * swb + 9.0 * swa * b2 + b3) / d7;
  Tap[3] = 140.0 * (a3 * swb + 3.0 * a2 * b2 + swa * b3) / d7;
  Tap[2] = -210.0 * (a3 * b2 + a2 * b3) / d7;
  Tap[1] = 140.0 * a3 * b3 / d7;
  Tap[0] = (-35.0 * a3 * b2 * b2 + 21.0 * a2 * b3 * b2 + 7.0 * swa * b3 * b3 +
            b3 * b3 * swb) / d7;
}

std::string rg_read_ffield(const char *path, int lgflag, ForceField *ff) {
  LineReader r;
  r.in.open(path);
  if (!r.in) return std::string("cannot open force field file ") + path;
  std::memset(ff, 0, sizeof(*ff));
  auto need = [&](void) { return r.next(); };
  if (!need() || !need()) return "force field: truncated header";
  const int ngp = r.i(0);
  if (ngp < 1 || ngp > 64) return "force field: bad number of global parameters";
  ff->ngp = ngp;
  for (int k = 0; k < ngp; ++k) {
    if (!need()) return "force field: truncated global parameters";
    ff->gp[k] = r.d(0);
  }
  if (!need()) return "force field: missing atom block";
  const int nt = r.i(0);
  if (nt < 1 || nt > RG_MAXT) return "force field: unsupported number of atom types";
  ff->ntypes = nt;
  for (int k = 0; k < 3; ++k)
    if (!need()) return "force field: truncated atom block header";
  ff->vdw_type = 0;
  for (int t = 0; t < nt; ++t) {
    Sbp &s = ff->sbp[t];
    if (!need() || r.tok.size() < 9) return "force field: bad atom line 1";
    std::string nm = r.tok[0];
    for (size_t c = 0; c < nm.size() && c < 7; ++c) s.name[c] = (char)std::toupper((unsigned char)nm[c]);
    s.is_carbon = (std::strcmp(s.name, "C") == 0);
    s.r_s = r.d(1); s.valency = r.d(2); s.mass = r.d(3); s.r_vdw = r.d(4);
    s.epsilon = r.d(5); s.gamma = r.d(6); s.r_pi = r.d(7); s.valency_e = r.d(8);
    s.nlp_opt = 0.5 * (s.valency_e - s.valency);
    if (!need() || r.tok.size() < 8) return "force field: bad atom line 2";
    s.alpha = r.d(0); s.gamma_w = r.d(1); s.valency_boc = r.d(2); s.p_ovun5 = r.d(3);
    s.chi = r.d(5); s.eta = 2.0 * r.d(6); s.p_hbond = (int)r.d(7);
    if (!need() || r.tok.size() < 6) return "force field: bad atom line 3";
    s.r_pi_pi = r.d(0); s.p_lp2 = r.d(1);
    s.b_o_131 = r.d(3); s.b_o_132 = r.d(4); s.b_o_133 = r.d(5);
    if (!need() || r.tok.size() < 3) return "force field: inconsistent ffield file (atom line 4)";
    s.p_ovun2 = r.d(0); s.p_val3 = r.d(1); s.valency_val = r.d(3); s.p_val5 = r.d(4);
    s.rcore2 = r.d(5); s.ecore2 = r.d(6); s.acore2 = r.d(7);
    if (lgflag) {
      if (!need()) return "force field: missing lg line";
      s.lgcij = r.d(0); s.lgre = r.d(1);
    }
    // vdW flavour: 1 shielded, 2 inner wall, 3 both (reaxc_ffield_sunway.cpp:229-284)
    const bool wall = s.rcore2 > 0.01 && s.acore2 > 0.01;
    const bool shield = s.gamma_w > 0.5;
    int want = wall ? (shield ? 3 : 2) : (shield ? 1 : 0);
    if (want == 0) return std::string("force field: no shielding or inner wall for element ") + s.name;
    if (ff->vdw_type == 0) ff->vdw_type = want;
  }
  for (int t = 0; t < nt; ++t) {
    Sbp &s = ff->sbp[t];
    if (s.mass < 21 && s.valency_val != s.valency_boc) s.valency_val = s.valency_boc;
  }
  // bonds
  if (!need()) return "force field: missing bond block";
  int nl = r.i(0);
  if (!need()) return "force field: truncated bond block";
  for (int l = 0; l < nl; ++l) {
    if (!need()) return "force field: truncated bond block";
    int j = r.i(0) - 1, k = r.i(1) - 1;
    double a[8];
    for (int m = 0; m < 8; ++m) a[m] = r.d(2 + m);
    if (!need()) return "force field: truncated bond block";
    if (j < 0 || k < 0 || j >= nt || k >= nt) continue;
    for (int pass = 0; pass < 2; ++pass) {
      Tbp &b = pass ? ff->tbp[k][j] : ff->tbp[j][k];
      b.De_s = a[0]; b.De_p = a[1]; b.De_pp = a[2]; b.p_be1 = a[3];
      b.p_bo5 = a[4]; b.v13cor = a[5]; b.p_bo6 = a[6]; b.p_ovun1 = a[7];
      b.p_be2 = r.d(0); b.p_bo3 = r.d(1); b.p_bo4 = r.d(2);
      b.p_bo1 = r.d(4); b.p_bo2 = r.d(5); b.ovc = r.d(6);
    }
  }
  // mixing rules (reaxc_ffield_sunway.cpp:368-436)
  for (int i = 0; i < nt; ++i)
    for (int j = 0; j < nt; ++j) {
      const Sbp &a = ff->sbp[i], &b = ff->sbp[j];
      Tbp &t = ff->tbp[i][j];
      t.r_s = 0.5 * (a.r_s + b.r_s);
      t.r_p = 0.5 * (a.r_pi + b.r_pi);
      t.r_pp = 0.5 * (a.r_pi_pi + b.r_pi_pi);
      t.p_boc3 = std::sqrt(a.b_o_132 * b.b_o_132);
      t.p_boc4 = std::sqrt(a.b_o_131 * b.b_o_131);
      t.p_boc5 = std::sqrt(a.b_o_133 * b.b_o_133);
      t.D = std::sqrt(a.epsilon * b.epsilon);
      t.alpha = std::sqrt(a.alpha * b.alpha);
      t.r_vdW = 2.0 * std::sqrt(a.r_vdw * b.r_vdw);
      t.gamma_w = std::sqrt(a.gamma_w * b.gamma_w);
      t.gamma = std::pow(a.gamma * b.gamma, -1.5);
      t.rcore = std::sqrt(a.rcore2 * b.rcore2);
      t.ecore = std::sqrt(a.ecore2 * b.ecore2);
      t.acore = std::sqrt(a.acore2 * b.acore2);
      t.lgcij = std::sqrt(a.lgcij * b.lgcij);
      t.lgre = 2.0 * ff->gp[35] * std::sqrt(a.lgre * b.lgre);
    }
  // off-diagonal overrides
  if (!need()) return "force field: missing off-diagonal block";
  nl = r.i(0);
  for (int l = 0; l < nl; ++l) {
    if (!need()) return "force field: truncated off-diagonal block";
    int j = r.i(0) - 1, k = r.i(1) - 1;
    if (j < 0 || k < 0 || j >= nt || k >= nt) continue;
    for (int pass = 0; pass < 2; ++pass) {
      Tbp &b = pass ? ff->tbp[k][j] : ff->tbp[j][k];
      double v;
      if ((v = r.d(2)) > 0.0) b.D = v;
      if ((v = r.d(3)) > 0.0) b.r_vdW = 2 * v;
      if ((v = r.d(4)) > 0.0) b.alpha = v;
      if ((v = r.d(5)) > 0.0) b.r_s = v;
      if ((v = r.d(6)) > 0.0) b.r_p = v;
      if ((v = r.d(7)) > 0.0) b.r_pp = v;
      if (r.tok.size() > 8 && (v = r.d(8)) >= 0.0) b.lgcij = v;
    }
  }
  // angles: both counters advance even when the end types coincide
  // (reaxc_ffield_sunway.cpp:552-586)
  if (!need()) return "force field: missing angle block";
  nl = r.i(0);
  for (int l = 0; l < nl; ++l) {
    if (!need()) return "force field: truncated angle block";
    int j = r.i(0) - 1, k = r.i(1) - 1, m = r.i(2) - 1;
    if (j < 0 || k < 0 || m < 0 || j >= nt || k >= nt || m >= nt) continue;
    int cnt = ff->thbp[j][k][m].cnt;
    if (cnt >= RG_MAX3 - 1) continue;
    ff->thbp[j][k][m].cnt++;
    ff->thbp[m][k][j].cnt++;
    Thbp p{r.d(3), r.d(4), r.d(5), r.d(6), r.d(7), r.d(8), r.d(9)};
    ff->thbp[j][k][m].prm[cnt] = p;
    ff->thbp[m][k][j].prm[cnt] = p;
  }
  // torsions (explicit entries win over 0-X-Y-0 wildcards)
  if (!need()) return "force field: missing torsion block";
  nl = r.i(0);
  {
    std::vector<char> flag((size_t)RG_MAXT * RG_MAXT * RG_MAXT * RG_MAXT, 0);
    auto F = [&](int a, int b, int c, int d) -> char & {
      return flag[((a * RG_MAXT + b) * RG_MAXT + c) * RG_MAXT + d];
    };
    for (int l = 0; l < nl; ++l) {
      if (!need()) return "force field: truncated torsion block";
      int j = r.i(0) - 1, k = r.i(1) - 1, m = r.i(2) - 1, n = r.i(3) - 1;
      Fbp p{r.d(4), r.d(5), r.d(6), r.d(7), r.d(8)};
      if (j >= 0 && n >= 0) {
        if (j < nt && k < nt && m < nt && n < nt && k >= 0 && m >= 0) {
          F(j, k, m, n) = F(n, m, k, j) = 1;
          ff->fbp[j][k][m][n].cnt = ff->fbp[n][m][k][j].cnt = 1;
          ff->fbp[j][k][m][n].prm = p;
          ff->fbp[n][m][k][j].prm = p;
        }
      } else if (k >= 0 && m >= 0 && k < nt && m < nt) {
        for (int a = 0; a < nt; ++a)
          for (int o = 0; o < nt; ++o) {
            ff->fbp[a][k][m][o].cnt = 1;
            ff->fbp[o][m][k][a].cnt = 1;
            if (!F(a, k, m, o)) ff->fbp[a][k][m][o].prm = p;
            if (!F(o, m, k, a)) ff->fbp[o][m][k][a].prm = p;
          }
      }
    }
  }
  // hydrogen bonds
  for (int i = 0; i < nt; ++i)
    for (int j = 0; j < nt; ++j)
      for (int k = 0; k < nt; ++k) ff->hbp[i][j][k].r0_hb = -1.0;
  if (need()) {
    nl = r.i(0);
    for (int l = 0; l < nl; ++l) {
      if (!need()) break;
      if (r.tok.size() < 7) continue;
      int j = r.i(0) - 1, k = r.i(1) - 1, m = r.i(2) - 1;
      if (j < 0 || k < 0 || m < 0 || j >= nt || k >= nt || m >= nt) continue;
      Hbp &h = ff->hbp[j][k][m];
      h.r0_hb = r.d(3); h.p_hb1 = r.d(4); h.p_hb2 = r.d(5); h.p_hb3 = r.d(6);
      h.inv_r0_hb = h.r0_hb > 0.0 ? 1.0 / h.r0_hb : 0.0;
    }
  }
  const double p_vdW1 = ff->gp[28];
  for (int i = 0; i < nt; ++i)
    for (int j = 0; j < nt; ++j)
      ff->tbp[i][j].powgi_vdW1 = std::pow(1.0 / ff->tbp[i][j].gamma_w, p_vdW1);
  return "";
}

// Bond-order correction and the bonded energy terms.
//
//  k_bo_deltap / k_bo_correct / k_bo_atom: BO_Section1/2/3
//      (reaxc_bond_orders_sw64.c:56-64, :162-377, :451-482)
//  k_atom_energy: bond energy, lone pair, over/under-coordination and
//      polarisation, Merge_Bonds_Atom_Energy_C_New (reaxc_multi_body_sw64.c:21-333)
//  k_hbonds: Hydrogen_Bonds_C (reaxc_hydrogen_bonds_sw64.c:146-248)
//  k_vt_* / k_valence / k_torsion: Merge_Torsion_Valence_Angles
//      (reaxc_torsion_angles_sw64.c:813-1367) with Calculate_Omega (:21-102)
//  k_dbond: Add_All_dBond_to_Forces_C (reaxc_forces_sw64.c:499-588)
//
// Every term is evaluated once per centre atom as in the reference; the
// reference's ghost atoms become (atom, periodic image) pairs carried in the
// bond entries, so forces and CdDelta land directly on the owning atoms.
// Scattered accumulations use FP64 atomics.
#include <type_traits>

#include "rg_internal.h"

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr double constPI = 3.14159265;          // reaxc_defs_sunway.h:58
constexpr double KCALpMOL_to_EV = 23.02;        // reaxc_defs_sunway.h:69
constexpr double HB_THRESHOLD = 1e-2;           // reaxc_defs_sunway.h:91
constexpr double MIN_SINE = 1e-10;

template <typename R>
__device__ __forceinline__ R deg2rad(R a) { return a * R(constPI) / R(180); }
template <typename R>
__device__ __forceinline__ R sqr(R x) { return x * x; }

// per-block reduction of one energy term into segment seg's entry E
__device__ __forceinline__ void energy_add(const Dev &d, double v, int seg, int E) {
  seg_block_add<1>(&v, seg, d.energy + E, RG_NE);
}

__device__ __forceinline__ void add3(double *fC, int n, int a, double s, double x, double y, double z) {
  atomicAdd(&fC[a], s * x);
  atomicAdd(&fC[n + a], s * y);
  atomicAdd(&fC[2 * n + a], s * z);
}

__device__ __forceinline__ int nbr_of(uint32_t e) { return (int)(e >> 8); }

// diagnostics: keeps the first non-finite term (kind 1 angle, 2 torsion)
__device__ void debug_record(const Dev &d, int kind, int a, int b, int c, int e, const double *v,
                             int nv) {
  if (atomicCAS(d.dbg_flag, 0, 1) != 0) return;
  d.dbg[0] = kind; d.dbg[1] = a; d.dbg[2] = b; d.dbg[3] = c; d.dbg[4] = e;
  for (int k = 0; k < nv && k < 35; ++k) d.dbg[5 + k] = v[k];
}

// (tag, position) order deciding which end of a bond / central torsion
// bond carries the term, reaxc_multi_body_sw64.c:256-267
__device__ __forceinline__ bool tag_first(const Dev &d, int i, int j, uint32_t e) {
  const int ti = d.tags[i], tj = d.tags[j];
  if (ti > tj) return false;
  if (ti == tj) {
    int sx, sy, sz;
    img_unpack((int)(e & 255u), &sx, &sy, &sz);
    const double4 xi = d.xs[i], xj0 = d.xs[j];
    const double *L = d.seg[d.seg_s[i]].L;
    const double xj = xj0.x + sx * L[0], yj = xj0.y + sy * L[1], zj = xj0.z + sz * L[2];
    if (zj < xi.z) return false;
    if (zj == xi.z && yj < xi.y) return false;
    if (zj == xi.z && yj == xi.y && xj < xi.x) return false;
  }
  return true;
}

// Calculate_Theta / Calculate_dCos_Theta, reaxc_valence_angles_sunway.cpp:49-79
// (R = double: the FP64 form; R = float: the mixed form)
template <typename R, bool THETA = true>
__device__ __forceinline__ void theta_dcos(const R *dji, R d_ji, const R *djk, R d_jk, R &theta,
                                           R &cos_theta, R *di, R *dj, R *dk) {
  const R dot = dji[0] * djk[0] + dji[1] * djk[1] + dji[2] * djk[2];
  cos_theta = dot / (d_ji * d_jk);
  if (cos_theta > R(1)) cos_theta = R(1);
  if (cos_theta < R(-1)) cos_theta = R(-1);
  if (THETA) theta = acos(cos_theta);
  const R sqr_d_ji = d_ji * d_ji, sqr_d_jk = d_jk * d_jk;
  const R inv_dists = R(1) / (d_ji * d_jk);
  const R inv_dists3 = inv_dists * inv_dists * inv_dists;
  const R Cdot_inv3 = dot * inv_dists3;
  // the three gradients of cos theta sum to zero: dj = -(di + dk)
#pragma unroll
  for (int t = 0; t < 3; ++t) {
    di[t] = djk[t] * inv_dists - Cdot_inv3 * sqr_d_jk * dji[t];
    dk[t] = dji[t] * inv_dists - Cdot_inv3 * sqr_d_ji * djk[t];
    dj[t] = -(di[t] + dk[t]);
  }
}

// ------------------------------------------------------------------
// bond orders

__global__ void k_bo_deltap(Dev d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n) return;
  const Sbp &s = d.ff->sbp[d.ts[i]];
  const double b = d.bo0[i];
  const double Dp = b - s.valency;
  d.Deltap[i] = Dp;
  d.Deltap_boc[i] = b - s.valency_val;
  // the per-atom exponentials of the f1 correction, once per atom instead
  // of once per bond end
  d.exp_boc[i] = exp(-d.ff->gp[0] * Dp);
  d.exp_boc[d.n + i] = exp(-d.ff->gp[1] * Dp);
}

// the corrected bond order of bond slot k of atom i (f1 with f4 f5; the
// reference's quotients taken as products with five reciprocals)
__device__ __forceinline__ void bo_correct_item(const Dev &d, int i, int k) {
  const int n = d.n;
  const long long s = (long long)k * n + i, S = (long long)d.bond_cap * n;
  const ForceField &F = *d.ff;
  const int j = nbr_of(d.b_nbr[s]);
  const int ti = d.ts[i], tj = d.ts[j];
  const Tbp &tw = F.tbp[ti][tj];
  double BO = d.b_BO[s], BOs = d.b_BOs[s], BOpi = d.b_BOpi[s], BOpi2 = d.b_BOpi2[s];
  double C[11];
  if (tw.ovc < 0.001 && tw.v13cor < 0.001) {
    C[0] = 1.0; C[1] = 0.0; C[2] = 0.0;
    C[3] = BOpi; C[4] = 0.0; C[5] = 0.0; C[6] = 0.0;
    C[7] = BOpi2; C[8] = 0.0; C[9] = 0.0; C[10] = 0.0;
  } else {
    const double p_boc1 = F.gp[0], p_boc2 = F.gp[1];
    const double val_i = F.sbp[ti].valency, val_j = F.sbp[tj].valency;
    const double Dboc_i = d.Deltap_boc[i], Dboc_j = d.Deltap_boc[j];
    double f1, Cf1_ij, Cf1_ji, f4, f5, f4f5, Cf45_ij, Cf45_ji;
    if (tw.ovc >= 0.001) {
      const double exp_p1i = d.exp_boc[i], exp_p2i = d.exp_boc[n + i];
      const double exp_p1j = d.exp_boc[j], exp_p2j = d.exp_boc[n + j];
      const double f2 = exp_p1i + exp_p1j;
      const double e22 = exp_p2i + exp_p2j, ie22 = 1.0 / e22;
      const double f3 = -1.0 / p_boc2 * log(0.5 * e22);
      const double temp = f2 + f3;
      const double u1_ij = val_i + temp, u1_ji = val_j + temp;
      const double a = 1.0 / u1_ij, b = 1.0 / u1_ji, a2 = a * a, b2 = b * b;
      f1 = 0.5 * ((val_i + f2) * a + (val_j + f2) * b);
      const double Cf1A_ij = 0.5 * f3 * (a2 + b2);
      const double Cf1B_ij = -0.5 * ((u1_ij - f3) * a2 + (u1_ji - f3) * b2);
      const double ep = exp_p2i * ie22;
      Cf1_ij = 0.50 * (-p_boc1 * exp_p1i * a - ((val_i + f2) * a2) * (-p_boc1 * exp_p1i + ep) +
                       -p_boc1 * exp_p1i * b - ((val_j + f2) * b2) * (-p_boc1 * exp_p1i + ep));
      Cf1_ji = -Cf1A_ij * p_boc1 * exp_p1j + Cf1B_ij * exp_p2j * ie22;
    } else {
      f1 = 1.0;
      Cf1_ij = Cf1_ji = 0.0;
    }
    if (tw.v13cor >= 0.001) {
      const double exp_f4 = exp(-(tw.p_boc4 * sqr(BO) - Dboc_i) * tw.p_boc3 + tw.p_boc5);
      const double exp_f5 = exp(-(tw.p_boc4 * sqr(BO) - Dboc_j) * tw.p_boc3 + tw.p_boc5);
      f4 = 1. / (1. + exp_f4);
      f5 = 1. / (1. + exp_f5);
      f4f5 = f4 * f5;
      Cf45_ij = -f4 * exp_f4;
      Cf45_ji = -f5 * exp_f5;
    } else {
      f4 = f5 = f4f5 = 1.0;
      Cf45_ij = Cf45_ji = 0.0;
    }
    const double A0 = f1 * f4f5;
    const double A1 = -2 * tw.p_boc3 * tw.p_boc4 * BO * (Cf45_ij + Cf45_ji);
    const double if1 = 1.0 / f1;
    const double A2_ij = Cf1_ij * if1 + tw.p_boc3 * Cf45_ij;
    const double A2_ji = Cf1_ji * if1 + tw.p_boc3 * Cf45_ji;
    const double A3_ij = A2_ij + Cf1_ij * if1;
    const double A3_ji = A2_ji + Cf1_ji * if1;
    BO = BO * A0;
    BOpi = BOpi * A0 * f1;
    BOpi2 = BOpi2 * A0 * f1;
    BOs = BO - (BOpi + BOpi2);
    C[0] = A0 + BO * A1; C[1] = BO * A2_ij; C[2] = BO * A2_ji;
    C[3] = f1 * f1 * f4 * f5; C[4] = BOpi * A1; C[5] = BOpi * A3_ij; C[6] = BOpi * A3_ji;
    C[7] = f1 * f1 * f4 * f5; C[8] = BOpi2 * A1; C[9] = BOpi2 * A3_ij; C[10] = BOpi2 * A3_ji;
  }
  if (BO < 1e-10) BO = 0.0;
  if (BOs < 1e-10) BOs = 0.0;
  if (BOpi < 1e-10) BOpi = 0.0;
  if (BOpi2 < 1e-10) BOpi2 = 0.0;
  d.b_BO[s] = BO; d.b_BOs[s] = BOs; d.b_BOpi[s] = BOpi; d.b_BOpi2[s] = BOpi2;
#pragma unroll
  for (int c = 0; c < 11; ++c) d.b_C[c * S + s] = C[c];
}

__global__ void __launch_bounds__(256) k_bo_correct(Dev d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int cnt = i < d.n ? min(d.nbonds[i], d.bond_cap) : 0;
  warp_items(cnt, i, [&](int a, int k) { bo_correct_item(d, a, k); });
}

__global__ void k_bo_atom(Dev d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n) return;
  const int n = d.n;
  const ForceField &F = *d.ff;
  const Sbp &s = F.sbp[d.ts[i]];
  const int nb = min(d.nbonds[i], d.bond_cap);
  double tot = 0.0;
  for (int k = 0; k < nb; ++k) tot += d.b_BO[(long long)k * n + i];
  d.bo0[i] = tot;
  const double p_lp1 = F.gp[15];
  const double Delta = tot - s.valency, Delta_e = tot - s.valency_e;
  d.Delta[i] = Delta;
  d.Delta_e[i] = Delta_e;
  d.Delta_boc[i] = tot - s.valency_boc;
  d.Delta_val[i] = tot - s.valency_val;
  const double vlpex = Delta_e - 2.0 * (int)(Delta_e / 2.0);
  const double explp1 = exp(-p_lp1 * sqr(2.0 + vlpex));
  const double nlp = explp1 - (int)(Delta_e / 2.0);
  d.vlpex[i] = vlpex;
  d.nlp[i] = nlp;
  d.Delta_lp[i] = s.nlp_opt - nlp;
  const double Clp = 2.0 * p_lp1 * explp1 * (2.0 + vlpex);
  d.dDelta_lp[i] = Clp;
  double nlp_temp;
  if (s.mass > 21.0) nlp_temp = 0.5 * (s.valency_e - s.valency);
  else nlp_temp = nlp;
  d.nlp_temp[i] = nlp_temp;
  d.Delta_lp_temp[i] = s.nlp_opt - nlp_temp;
}

// ------------------------------------------------------------------
// bond + lone pair + over/under-coordination + polarisation

__global__ void k_atom_energy(Dev d, int eflag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = d.n;
  double e_lph = 0, e_lp = 0, e_ov = 0, e_un = 0;
  double pol = 0, pol_w = 0;
  if (i < n) {
    const ForceField &F = *d.ff;
    const double p_lp3 = F.gp[5], p_ovun3 = F.gp[32], p_ovun4 = F.gp[31];
    const double p_ovun6 = F.gp[6], p_ovun7 = F.gp[8], p_ovun8 = F.gp[9];
    double *CdD = d.fC + 3 * (long long)n;
    const int ti = d.ts[i];
    const Sbp &si = F.sbp[ti];
    const int nb = min(d.nbonds[i], d.bond_cap);
    // polarisation (Compute_Polarization_Energy inlined at :93-104); the
    // reference's pvector value is the running sum, = sum_k pol_k*(n-k) over
    // the original atom order of the segment
    const double q = d.xs[i].w;
    pol = KCALpMOL_to_EV * (si.chi * q + (si.eta / 2.) * sqr(q));
    const SegGeom &g = d.seg[d.seg_s[i]];
    pol_w = pol * (double)(g.atom0 + g.natoms - d.perm[i]);
    const double p_lp2 = si.p_lp2;
    const double Dlp_i = d.Delta_lp[i];
    const double expvd2 = exp(-75 * Dlp_i);
    const double inv_expvd2 = 1. / (1. + expvd2);
    const double p_ovun2 = si.p_ovun2;
    const double dfvl = (si.mass > 21.0) ? 0.0 : 1.0;
    double sum_ovun1 = 0, sum_ovun2 = 0;
    for (int k = 0; k < nb; ++k) {
      const long long s = (long long)k * n + i;
      const int j = nbr_of(d.b_nbr[s]);
      const Tbp &tw = F.tbp[ti][d.ts[j]];
      sum_ovun1 += tw.p_ovun1 * tw.De_s * d.b_BO[s];
      sum_ovun2 += (d.Delta[j] - dfvl * d.Delta_lp_temp[j]) * (d.b_BOpi[s] + d.b_BOpi2[s]);
    }
    const double dElp = p_lp2 * inv_expvd2 + 75 * p_lp2 * Dlp_i * expvd2 * sqr(inv_expvd2);
    const double CElp = dElp * d.dDelta_lp[i];
    double cd_i = 0.0;
    if (p_lp3 > 0.001 && si.is_carbon) {
      for (int k = 0; k < nb; ++k) {
        const long long s = (long long)k * n + i;
        const int j = nbr_of(d.b_nbr[s]);
        if (!F.sbp[d.ts[j]].is_carbon) continue;
        const double Di = d.Delta[i];
        const double Di2 = Di * Di;
        const double vov3 = d.b_BO[s] - Di - 0.040 * (Di2 * Di2);
        if (vov3 > 3.) {
          e_lph += p_lp3 * sqr(vov3 - 3.0);
          d.b_Cdbo[s] += 2. * p_lp3 * (vov3 - 3.);
          cd_i += 2. * p_lp3 * (vov3 - 3.) * (-1. - 0.16 * (Di2 * Di));
        }
      }
    }
    const double exp_ovun1 = p_ovun3 * exp(p_ovun4 * sum_ovun2);
    const double inv_exp_ovun1 = 1.0 / (1 + exp_ovun1);
    const double Delta_lpcorr = d.Delta[i] - (dfvl * d.Delta_lp_temp[i]) * inv_exp_ovun1;
    const double exp_ovun2 = exp(p_ovun2 * Delta_lpcorr);
    const double inv_exp_ovun2 = 1.0 / (1.0 + exp_ovun2);
    const double DlpVi = 1.0 / (Delta_lpcorr + si.valency + 1e-8);
    const double CEover1 = Delta_lpcorr * DlpVi * inv_exp_ovun2;
    e_ov = sum_ovun1 * CEover1;
    const double CEover2 = sum_ovun1 * DlpVi * inv_exp_ovun2 *
                           (1.0 - Delta_lpcorr * (DlpVi + p_ovun2 * exp_ovun2 * inv_exp_ovun2));
    const double CEover3 = CEover2 * (1.0 - dfvl * d.dDelta_lp[i] * inv_exp_ovun1);
    const double CEover4 = CEover2 * (dfvl * d.Delta_lp_temp[i]) * p_ovun4 * exp_ovun1 * sqr(inv_exp_ovun1);
    const double p_ovun5 = si.p_ovun5;
    const double exp_ovun2n = 1.0 / exp_ovun2;
    const double exp_ovun6 = exp(p_ovun6 * Delta_lpcorr);
    const double exp_ovun8 = p_ovun7 * exp(p_ovun8 * sum_ovun2);
    const double inv_exp_ovun2n = 1.0 / (1.0 + exp_ovun2n);
    const double inv_exp_ovun8 = 1.0 / (1.0 + exp_ovun8);
    cd_i += CEover3;
    double CEunder1, CEunder2, CEunder4;
    double eun = 0.0;
    if (nb > 0 || d.ctl->enobondsflag) {
      eun = -p_ovun5 * (1.0 - exp_ovun6) * inv_exp_ovun2n * inv_exp_ovun8;
      e_un = eun;
      e_lp += p_lp2 * Dlp_i * inv_expvd2;
    }
    CEunder1 = inv_exp_ovun2n * (p_ovun5 * p_ovun6 * exp_ovun6 * inv_exp_ovun8 + p_ovun2 * eun * exp_ovun2n);
    CEunder2 = -eun * p_ovun8 * exp_ovun8 * inv_exp_ovun8;
    const double CEunder3 = CEunder1 * (1.0 - dfvl * d.dDelta_lp[i] * inv_exp_ovun1);
    CEunder4 = CEunder1 * (dfvl * d.Delta_lp_temp[i]) * p_ovun4 * exp_ovun1 * sqr(inv_exp_ovun1) + CEunder2;
    if (nb > 0 || d.ctl->enobondsflag) {
      cd_i += CEunder3;
      cd_i += CElp;
    }
    for (int k = 0; k < nb; ++k) {
      const long long s = (long long)k * n + i;
      const uint32_t e = d.b_nbr[s];
      const int j = nbr_of(e);
      const int tj = d.ts[j];
      const Tbp &tw = F.tbp[ti][tj];
      const double BOpi = d.b_BOpi[s], BOpi2 = d.b_BOpi2[s];
      const double cdbo = CEover1 * tw.p_ovun1 * tw.De_s;
      const double ftmp2 = (1.0 - dfvl * d.dDelta_lp[j]) * (BOpi + BOpi2);
      const double dj = d.Delta[j] - dfvl * d.Delta_lp_temp[j];
      const double cdj = CEover4 * ftmp2 + CEunder4 * ftmp2;
      const double cdpi = CEover4 * dj + CEunder4 * dj;
      const double cdpi2 = cdpi;
      // the bond energy of the bond's first end: k_bond_energy
      d.b_Cdbo[s] += cdbo;
      d.b_Cdbopi[s] += cdpi;
      d.b_Cdbopi2[s] += cdpi2;
      if (cdj != 0.0) atomicAdd(&CdD[j], cdj);
    }
    atomicAdd(&CdD[i], cd_i);
  }
  if (eflag) {
    const int sg = i < n ? d.seg_s[i] : -1;
    energy_add(d, e_ov + e_un, sg, E_OVUN);
    energy_add(d, e_lp + e_lph, sg, E_LP);
    energy_add(d, e_lph + e_lp + e_ov + e_un, sg, E_ENG_VDWL);
    energy_add(d, pol, sg, E_ENG_COUL);
    energy_add(d, pol, sg, E_POL_PHYS);
    energy_add(d, pol_w, sg, E_POL);
  }
}

// Bond energy (with the triple-bond stabilisation) of every bond, at its
// first end (tag_first), the reference's Bonds (reaxc_bonds_sw64.c): one
// warp per 32 atoms over the bond slots that carry the energy
// (warp_items_mask), so their log/exp keep the lanes busy.
__global__ void __launch_bounds__(256) k_bond_energy(Dev d, int eflag) {
  const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = d.n;
  const int cnt = i0 < n ? min(d.nbonds[i0], d.bond_cap) : 0;
  double eb = 0.0;
  int sg = -1;
  auto item = [&](int i, int k) {
    const long long s = (long long)k * n + i;
    const uint32_t e = d.b_nbr[s];
    const int j = nbr_of(e);
    if (!tag_first(d, i, j, e)) return;
    const ForceField &F = *d.ff;
    const int ti = d.ts[i], tj = d.ts[j];
    const Tbp &tw = F.tbp[ti][tj];
    const Sbp &si = F.sbp[ti], &sj = F.sbp[tj];
    const double BOpi = d.b_BOpi[s], BOpi2 = d.b_BOpi2[s], BO = d.b_BO[s], BOs = d.b_BOs[s];
    // BOs^p_be2 as exp(p_be2 ln BOs) (to ~1e-15 relative, without pow's
    // extended-precision logarithm)
    const double pow_BOs_be2 = (BOs <= 0.0) ? 0.0 : exp(tw.p_be2 * log(BOs));
    const double exp_be12 = exp(tw.p_be1 * (1.0 - pow_BOs_be2));
    const double CEbo = -tw.De_s * exp_be12 * (1.0 - tw.p_be1 * tw.p_be2 * pow_BOs_be2);
    double ebond = -tw.De_s * BOs * exp_be12 - tw.De_p * BOpi - tw.De_pp * BOpi2;
    double cdbo = CEbo;
    const int gp37 = (int)F.gp[37];
    if (BO >= 1.00 && (gp37 == 2 || (si.mass == 12.0000 && sj.mass == 15.9990) ||
                       (sj.mass == 12.0000 && si.mass == 15.9990))) {
      const double gp3 = F.gp[3], gp4 = F.gp[4], gp7 = F.gp[7], gp10 = F.gp[10];
      double *CdD = d.fC + 3 * (long long)n;
      const double exphu = exp(-gp7 * sqr(BO - 2.50));
      const double exphua1 = exp(-gp3 * (d.bo0[i] - BO));
      const double exphub1 = exp(-gp3 * (d.bo0[j] - BO));
      const double exphuov = exp(gp4 * (d.Delta[i] + d.Delta[j]));
      const double hulpov = 1.0 / (1.0 + 25.0 * exphuov);
      ebond += gp10 * exphu * hulpov * (exphua1 + exphub1);
      cdbo += gp10 * exphu * hulpov * (exphua1 + exphub1) * (gp3 - 2.0 * gp7 * (BO - 2.50));
      atomicAdd(&CdD[i], -gp10 * exphu * hulpov *
                             (gp3 * exphua1 + 25.0 * gp4 * exphuov * hulpov * (exphua1 + exphub1)));
      atomicAdd(&CdD[j], -gp10 * exphu * hulpov *
                             (gp3 * exphub1 + 25.0 * gp4 * exphuov * hulpov * (exphua1 + exphub1)));
    }
    d.b_Cdbo[s] += cdbo;
    d.b_Cdbopi[s] -= CEbo + tw.De_p;
    d.b_Cdbopi2[s] -= CEbo + tw.De_pp;
    if (eflag) {
      // a lane's items can reach into the next segment (batches): the
      // finished segment's sum goes out directly
      const int si_seg = d.seg_s[i];
      if (si_seg != sg) {
        if (sg >= 0 && eb != 0.0) {
          atomicAdd(&d.energy[(long long)sg * RG_NE + E_BOND], eb);
          atomicAdd(&d.energy[(long long)sg * RG_NE + E_ENG_VDWL], eb);
        }
        sg = si_seg;
        eb = 0.0;
      }
      eb += ebond;
    }
  };
  if (d.bond_cap <= 32) {
    // only the slots that carry the energy (a bit per slot)
    unsigned first = 0;
    for (int k = 0; k < cnt; ++k) {
      const uint32_t e = d.b_nbr[(long long)k * n + i0];
      if (tag_first(d, i0, nbr_of(e), e)) first |= 1u << k;
    }
    warp_items_mask(first, i0, item);
  } else {
    warp_items(cnt, i0, item);
  }
  if (eflag) {
    energy_add(d, eb, sg, E_BOND);
    energy_add(d, eb, sg, E_ENG_VDWL);
  }
}

// ------------------------------------------------------------------
// hydrogen bonds: one warp per H atom j; for each bonded acceptor i
// (p_hbond 2, BO >= 0.01) the lanes take the H-bond partners k

__device__ __forceinline__ double warp_sum_d(double v) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(FULL, v, off);
  return v;
}

// FP64 form (the mixed form runs k_hbonds32 below).  Per acceptor bond the
// lanes hold exp(-p_hb2 BO) for every partner type (p_hb2 depends on the
// partner's type, BO on the bond only), and 1/r_ij; per partner one
// reciprocal square root gives 1/r_jk and r_jk, and 1/r0_hb comes with the
// parameters, so no division is left in the triple loop.  The partners are
// taken 32 at a time with all lanes in step (the per-type exponential is a
// shuffle).
template <bool VIR>
__global__ void __launch_bounds__(256) k_hbonds(Dev d, int eflag) {
  const int lane = threadIdx.x & 31;
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int n = d.n;
  double ehb = 0.0;
  double w[6] = {0, 0, 0, 0, 0, 0};
  if (j < n && d.ff->sbp[d.ts[j]].p_hbond == 1) {
    const ForceField &F = *d.ff;
    const int tj = d.ts[j];
    const int nb = min(d.nbonds[j], d.bond_cap);
    const int nh = min(d.nhb[j], d.hb_cap);
    const double4 xj = d.xs[j];
    const SegGeom &g = d.seg[d.seg_s[j]];
    double *fC = d.fC;
    double fjx = 0, fjy = 0, fjz = 0;
    for (int q = 0; q < nb; ++q) {
      const long long s = (long long)q * n + j;
      const int i = nbr_of(d.b_nbr[s]);
      const int ti = d.ts[i];
      const double BO = d.b_BO[s];
      if (F.sbp[ti].p_hbond != 2 || !(BO >= HB_THRESHOLD)) continue;
      const double dij[3] = {d.b_dx[s], d.b_dy[s], d.b_dz[s]};
      const double r_ij = d.b_d[s];
      const double inv_rij = 1.0 / r_ij, sqr_d_ji = r_ij * r_ij;
      double e2 = 0.0;
      if (lane < F.ntypes && F.hbp[ti][tj][lane].r0_hb > 0.0)
        e2 = exp(-F.hbp[ti][tj][lane].p_hb2 * BO);
      const int tag_i = d.tags[i];
      double fix = 0, fiy = 0, fiz = 0, cdbo = 0;
      for (int base = 0; base < nh; base += 32) {
        const int pk = base + lane;
        uint32_t ek = 0;
        int k = 0, tk = 0;
        bool ok = pk < nh;
        if (ok) {
          ek = d.hb_nbr[(long long)j * d.hb_cap + pk];
          k = nbr_of(ek);
          tk = d.ts[k];
          ok = d.tags[k] != tag_i && F.hbp[ti][tj][tk].r0_hb > 0.0;
        }
        const double exp_hb2 = __shfl_sync(FULL, e2, tk);
        if (!ok) continue;
        const Hbp &hbp = F.hbp[ti][tj][tk];
        int sx, sy, sz;
        img_unpack((int)(ek & 255u), &sx, &sy, &sz);
        const double4 xk = d.xs[k];
        double djk[3];
        disp64(g, xk, xj, sx, sy, sz, djk[0], djk[1], djk[2]);
        const double sqr_d_jk = fma(djk[0], djk[0], fma(djk[1], djk[1], djk[2] * djk[2]));
        const double inv_rjk = rsqrt(sqr_d_jk);
        const double r_jk = sqr_d_jk * inv_rjk;
        // the angle and d(cos theta) (theta_dcos with the reciprocals)
        const double dot = dij[0] * djk[0] + dij[1] * djk[1] + dij[2] * djk[2];
        const double inv_dists = inv_rij * inv_rjk;
        double cos_theta = dot * inv_dists;
        if (cos_theta > 1.0) cos_theta = 1.0;
        if (cos_theta < -1.0) cos_theta = -1.0;
        const double Cdot_inv3 = dot * inv_dists * inv_dists * inv_dists;
        double di[3], djv[3], dk[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          di[c] = djk[c] * inv_dists - Cdot_inv3 * sqr_d_jk * dij[c];
          dk[c] = dij[c] * inv_dists - Cdot_inv3 * sqr_d_ji * djk[c];
          djv[c] = -(di[c] + dk[c]);   // the gradients sum to zero
        }
        // sin^4(theta/2) = ((1 - cos theta) / 2)^2: the reference's
        // sin(acos(c) / 2) without the two transcendentals
        const double cos_xhz1 = 1.0 - cos_theta;
        const double sin_xhz4 = 0.25 * cos_xhz1 * cos_xhz1;
        const double p_hb1 = hbp.p_hb1, p_hb2 = hbp.p_hb2, p_hb3 = hbp.p_hb3;
        const double r0_hb = hbp.r0_hb, inv_r0 = hbp.inv_r0_hb;
        const double exp_hb3 = exp(-p_hb3 * (r0_hb * inv_rjk + r_jk * inv_r0 - 2.0));
        const double e_hb = p_hb1 * (1.0 - exp_hb2) * exp_hb3 * sin_xhz4;
        ehb += e_hb;
        const double CEhb1 = p_hb1 * p_hb2 * exp_hb2 * exp_hb3 * sin_xhz4;
        const double CEhb2 = -0.5 * p_hb1 * (1.0 - exp_hb2) * exp_hb3 * cos_xhz1;
        const double CEhb3 = -p_hb3 * (inv_r0 - r0_hb * inv_rjk * inv_rjk) * e_hb;
        cdbo += CEhb1;
        fix += CEhb2 * di[0]; fiy += CEhb2 * di[1]; fiz += CEhb2 * di[2];
        const double c3 = CEhb3 * inv_rjk;
        fjx += CEhb2 * djv[0] - c3 * djk[0];
        fjy += CEhb2 * djv[1] - c3 * djk[1];
        fjz += CEhb2 * djv[2] - c3 * djk[2];
        const double fk[3] = {CEhb2 * dk[0] + c3 * djk[0], CEhb2 * dk[1] + c3 * djk[1],
                              CEhb2 * dk[2] + c3 * djk[2]};
        add3(fC, n, k, 1.0, fk[0], fk[1], fk[2]);
        if (VIR) vir_acc(w, djk[0], djk[1], djk[2], fk[0], fk[1], fk[2]);
      }
      if (VIR) vir_acc(w, d.b_dx[s], d.b_dy[s], d.b_dz[s], fix, fiy, fiz);
      cdbo = warp_sum_d(cdbo);
      fix = warp_sum_d(fix);
      fiy = warp_sum_d(fiy);
      fiz = warp_sum_d(fiz);
      if (lane == 0) {
        d.b_Cdbo[s] += cdbo;
        if (fix != 0.0 || fiy != 0.0 || fiz != 0.0) add3(fC, n, i, 1.0, fix, fiy, fiz);
      }
    }
    fjx = warp_sum_d(fjx);
    fjy = warp_sum_d(fjy);
    fjz = warp_sum_d(fjz);
    if (lane == 0 && (fjx != 0.0 || fjy != 0.0 || fjz != 0.0)) add3(fC, n, j, 1.0, fjx, fjy, fjz);
  }
  if (eflag) {
    const int sg = j < n ? d.seg_s[j] : -1;
    energy_add(d, ehb, sg, E_HB);
    energy_add(d, ehb, sg, E_ENG_VDWL);
  }
  if (VIR) seg_block_add<6>(w, j < n ? d.seg_s[j] : -1, d.virial, 6);
}

// Mixed form: the same terms entirely in FP32 per (H, acceptor bond,
// partner) triple: the H...Z displacement from the FP32 (hi, lo) positions,
// parameters from the control block's FP32 copies, forces summed in FP32
// (the atoms' into the FP32 force array), energies and the bond's Cdbo in
// FP64 once per lane and bond.
template <bool VIR>
__global__ void __launch_bounds__(256) k_hbonds32(Dev d, int eflag) {
  const int lane = threadIdx.x & 31;
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int n = d.n;
  double ehb = 0.0;
  double w[6] = {0, 0, 0, 0, 0, 0};
  if (j < n && d.ff->sbp[d.ts[j]].p_hbond == 1) {
    const ForceField &F = *d.ff;
    const Control &C = *d.ctl;
    const int tj = d.ts[j];
    const int nb = min(d.nbonds[j], d.bond_cap);
    const int nh = min(d.nhb[j], d.hb_cap);
    const float4 hjf = d.xf[j], ljf = d.xl[j];
    const SegGeom &g = d.seg[d.seg_s[j]];
    float *f32 = d.fC32;
    float fjx = 0.f, fjy = 0.f, fjz = 0.f;
    for (int q = 0; q < nb; ++q) {
      const long long s = (long long)q * n + j;
      const int i = nbr_of(d.b_nbr[s]);
      const int ti = d.ts[i];
      const double BO64 = d.b_BO[s];
      if (F.sbp[ti].p_hbond != 2 || !(BO64 >= HB_THRESHOLD)) continue;
      const float BO = (float)BO64;
      const float dij[3] = {(float)d.b_dx[s], (float)d.b_dy[s], (float)d.b_dz[s]};
      const float r_ij = (float)d.b_d[s];
      const int tag_i = d.tags[i];
      float fix = 0.f, fiy = 0.f, fiz = 0.f, cdbo = 0.f, el = 0.f;
      for (int pk = lane; pk < nh; pk += 32) {
        const uint32_t ek = d.hb_nbr[(long long)j * d.hb_cap + pk];
        const int k = nbr_of(ek), tk = d.ts[k];
        if (d.tags[k] == tag_i) continue;
        const Control::HbF &hp = C.hb32[ti][tj][tk];
        if (hp.r0_hb <= 0.f) continue;
        int sx, sy, sz;
        img_unpack((int)(ek & 255u), &sx, &sy, &sz);
        float djk[3];
        disp32(g, d.xf[k], d.xl[k], hjf, ljf, sx, sy, sz, djk[0], djk[1], djk[2]);
        const float r_jk = sqrtf(djk[0] * djk[0] + djk[1] * djk[1] + djk[2] * djk[2]);
        float theta, cos_theta, di[3], djv[3], dk[3];
        theta_dcos<float>(dij, r_ij, djk, r_jk, theta, cos_theta, di, djv, dk);
        const float sin_theta2 = sinf(theta / 2.f);
        float sin_xhz4 = sin_theta2 * sin_theta2;
        sin_xhz4 *= sin_xhz4;
        const float cos_xhz1 = 1.f - cos_theta;
        const float exp_hb2 = expf(-hp.p_hb2 * BO);
        const float exp_hb3 = expf(-hp.p_hb3 * (hp.r0_hb / r_jk + r_jk / hp.r0_hb - 2.f));
        const float e_hb = hp.p_hb1 * (1.f - exp_hb2) * exp_hb3 * sin_xhz4;
        el += e_hb;
        const float CEhb1 = hp.p_hb1 * hp.p_hb2 * exp_hb2 * exp_hb3 * sin_xhz4;
        const float CEhb2 = -hp.p_hb1 / 2.f * (1.f - exp_hb2) * exp_hb3 * cos_xhz1;
        const float CEhb3 = -hp.p_hb3 * (-hp.r0_hb / (r_jk * r_jk) + 1.f / hp.r0_hb) * e_hb;
        cdbo += CEhb1;
        fix += CEhb2 * di[0]; fiy += CEhb2 * di[1]; fiz += CEhb2 * di[2];
        const float c3 = CEhb3 / r_jk;
        fjx += CEhb2 * djv[0] - c3 * djk[0];
        fjy += CEhb2 * djv[1] - c3 * djk[1];
        fjz += CEhb2 * djv[2] - c3 * djk[2];
        const float fkx = CEhb2 * dk[0] + c3 * djk[0], fky = CEhb2 * dk[1] + c3 * djk[1],
                    fkz = CEhb2 * dk[2] + c3 * djk[2];
        atomicAdd(&f32[k], fkx);
        atomicAdd(&f32[n + k], fky);
        atomicAdd(&f32[2 * n + k], fkz);
        if (VIR) vir_acc(w, djk[0], djk[1], djk[2], fkx, fky, fkz);
      }
      if (eflag) ehb += (double)el;
      if (VIR) vir_acc(w, d.b_dx[s], d.b_dy[s], d.b_dz[s], fix, fiy, fiz);
      for (int off = 16; off > 0; off >>= 1) {
        cdbo += __shfl_down_sync(FULL, cdbo, off);
        fix += __shfl_down_sync(FULL, fix, off);
        fiy += __shfl_down_sync(FULL, fiy, off);
        fiz += __shfl_down_sync(FULL, fiz, off);
      }
      if (lane == 0) {
        d.b_Cdbo[s] += (double)cdbo;
        if (fix != 0.f || fiy != 0.f || fiz != 0.f) {
          atomicAdd(&f32[i], fix);
          atomicAdd(&f32[n + i], fiy);
          atomicAdd(&f32[2 * n + i], fiz);
        }
      }
    }
    for (int off = 16; off > 0; off >>= 1) {
      fjx += __shfl_down_sync(FULL, fjx, off);
      fjy += __shfl_down_sync(FULL, fjy, off);
      fjz += __shfl_down_sync(FULL, fjz, off);
    }
    if (lane == 0 && (fjx != 0.f || fjy != 0.f || fjz != 0.f)) {
      atomicAdd(&f32[j], fjx);
      atomicAdd(&f32[n + j], fjy);
      atomicAdd(&f32[2 * n + j], fjz);
    }
  }
  if (eflag) {
    const int sg = j < n ? d.seg_s[j] : -1;
    energy_add(d, ehb, sg, E_HB);
    energy_add(d, ehb, sg, E_ENG_VDWL);
  }
  if (VIR) seg_block_add<6>(w, j < n ? d.seg_s[j] : -1, d.virial, 6);
}

// ------------------------------------------------------------------
// Calculate_Omega, reaxc_torsion_angles_sw64.c:21-102
template <typename R>
struct Thb {
  R theta, sin, cos, di[3], dj[3], dk[3];
};

// the dihedral's derivative vectors; returns the unnormalised cosine and
// sine of omega (omega = atan2(us, uc)); the two angles' sines and cosines
// come with p_ijk and p_jkl
template <typename R>
__device__ void calc_omega(const R *dvec_ij, R r_ij, const R *dvec_jk, R r_jk, const R *dvec_kl,
                           R r_kl, const R *dvec_li, R r_li, const Thb<R> &p_ijk,
                           const Thb<R> &p_jkl, R *doi, R *doj, R *dok, R *dol, R &uc, R &us) {
  R sin_ijk = p_ijk.sin, cos_ijk = p_ijk.cos, sin_jkl = p_jkl.sin, cos_jkl = p_jkl.cos;
  const R dij_jk = dvec_ij[0] * dvec_jk[0] + dvec_ij[1] * dvec_jk[1] + dvec_ij[2] * dvec_jk[2];
  const R djk_kl = dvec_jk[0] * dvec_kl[0] + dvec_jk[1] * dvec_kl[1] + dvec_jk[2] * dvec_kl[2];
  const R dij_kl = dvec_ij[0] * dvec_kl[0] + dvec_ij[1] * dvec_kl[1] + dvec_ij[2] * dvec_kl[2];
  const R unnorm_cos_omega = -dij_jk * djk_kl + sqr(r_jk) * dij_kl;
  const R cr0 = dvec_jk[1] * dvec_kl[2] - dvec_jk[2] * dvec_kl[1];
  const R cr1 = dvec_jk[2] * dvec_kl[0] - dvec_jk[0] * dvec_kl[2];
  const R cr2 = dvec_jk[0] * dvec_kl[1] - dvec_jk[1] * dvec_kl[0];
  const R unnorm_sin_omega = -r_jk * (dvec_ij[0] * cr0 + dvec_ij[1] * cr1 + dvec_ij[2] * cr2);
  uc = unnorm_cos_omega;
  us = unnorm_sin_omega;
  const R htra = r_ij + cos_ijk * (r_kl * cos_jkl - r_jk);
  const R htrb = r_jk - r_ij * cos_ijk - r_kl * cos_jkl;
  const R htrc = r_kl + cos_jkl * (r_ij * cos_ijk - r_jk);
  const R hthd = r_ij * sin_ijk * (r_jk - r_kl * cos_jkl);
  const R hthe = r_kl * sin_jkl * (r_jk - r_ij * cos_ijk);
  const R hnra = r_kl * sin_ijk * sin_jkl;
  const R hnrc = r_ij * sin_ijk * sin_jkl;
  const R hnhd = r_ij * r_kl * cos_ijk * sin_jkl;
  const R hnhe = r_ij * r_kl * sin_ijk * cos_jkl;
  R poem = R(2) * r_ij * r_kl * sin_ijk * sin_jkl;
  if (poem < R(1e-20)) poem = R(1e-20);
  const R tel = sqr(r_ij) + sqr(r_jk) + sqr(r_kl) - sqr(r_li) -
                R(2) * (r_ij * r_jk * cos_ijk - r_ij * r_kl * cos_ijk * cos_jkl + r_jk * r_kl * cos_jkl);
  R arg = tel / poem;
  if (arg > R(1)) arg = R(1);
  if (arg < R(-1)) arg = R(-1);
  const R ms = (R)MIN_SINE;
  if (sin_ijk >= R(0) && sin_ijk <= ms) sin_ijk = ms;
  else if (sin_ijk <= R(0) && sin_ijk >= -ms) sin_ijk = -ms;
  if (sin_jkl >= R(0) && sin_jkl <= ms) sin_jkl = ms;
  else if (sin_jkl <= R(0) && sin_jkl >= -ms) sin_jkl = -ms;
  const R p2 = R(2) / poem;
  const R a1 = (htra - arg * hnra) / r_ij, a2 = (hthd - arg * hnhd) / sin_ijk;
  const R a3 = (hthe - arg * hnhe) / sin_jkl, a4 = (htrc - arg * hnrc) / r_kl;
  const R a5 = htrb / r_jk;
#pragma unroll
  for (int t = 0; t < 3; ++t) {
    doi[t] = p2 * (a1 * dvec_ij[t] - dvec_li[t] - a2 * p_ijk.dk[t]);
    doj[t] = p2 * (-a1 * dvec_ij[t] - a5 * dvec_jk[t] - a2 * p_ijk.dj[t] - a3 * p_jkl.di[t]);
    dok[t] = p2 * (-a4 * dvec_kl[t] + a5 * dvec_jk[t] - a2 * p_ijk.di[t] - a3 * p_jkl.dj[t]);
    dol[t] = p2 * (a4 * dvec_kl[t] + dvec_li[t] - a3 * p_jkl.dk[t]);
  }
}

// ------------------------------------------------------------------
// valence angles and torsions as work lists: every angle (centre j, bonds
// pk < ph) and every torsion (centre bond j-k counted at one end, bonds ph
// of j and pw of k) that passes the reference's bond-order tests becomes
// one item, so each thread evaluates one term with uniform work.  Torsions
// whose four parameters V1, V2, V3 and p_cot1 are all zero contribute
// exactly zero and are not listed.

// per centre: SBO2, CSBO2, dSBO1, dSBO2, expval6
__global__ void k_vt_prep_center(Dev d) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = d.n;
  if (j >= n) return;
  const ForceField &F = *d.ff;
  const double p_val6 = F.gp[14], p_val8 = F.gp[33], p_val9 = F.gp[16];
  const int nbj = min(d.nbonds[j], d.bond_cap);
  double SBOp = 0, prod_SBO = 1;
  for (int q = 0; q < nbj; ++q) {
    const long long sq = (long long)q * n + j;
    SBOp += d.b_BOpi[sq] + d.b_BOpi2[sq];
    double tmp = sqr(d.b_BO[sq]);
    tmp *= tmp;
    tmp *= tmp;
    prod_SBO *= exp(-tmp);
  }
  const double Delta_j = d.Delta_boc[j];
  double vlpadj, dSBO2;
  if (d.vlpex[j] >= 0) {
    vlpadj = 0;
    dSBO2 = prod_SBO - 1;
  } else {
    vlpadj = d.nlp[j];
    dSBO2 = (prod_SBO - 1) * (1 - p_val8 * d.dDelta_lp[j]);
  }
  const double SBO = SBOp + (1 - prod_SBO) * (-Delta_j - p_val8 * vlpadj);
  const double dSBO1 = -8 * prod_SBO * (Delta_j + p_val8 * vlpadj);
  double SBO2, CSBO2;
  if (SBO <= 0) SBO2 = 0, CSBO2 = 0;
  else if (SBO > 0 && SBO <= 1) {
    // x^p and p x^(p-1) from one logarithm and one exponential
    const double xp = exp(p_val9 * log(SBO));
    SBO2 = xp;
    CSBO2 = p_val9 * xp / SBO;
  } else if (SBO > 1 && SBO < 2) {
    const double y = 2 - SBO, yp = exp(p_val9 * log(y));
    SBO2 = 2 - yp;
    CSBO2 = p_val9 * yp / y;
  } else SBO2 = 2, CSBO2 = 0;
  d.c_sbo[j] = SBO2;
  d.c_sbo[n + j] = CSBO2;
  d.c_sbo[2 * n + j] = dSBO1;
  d.c_sbo[3 * n + j] = dSBO2;
  d.c_sbo[4 * n + j] = exp(p_val6 * Delta_j);
  if (!d.mixed) {
    // the FP64 form's per-centre factors of its angles (penalty f9 and
    // Cf9/f9, coalition 1/(1 + e) and -p_coa2 e/(1 + e), theta_0's
    // exponential); the mixed form's few FP64 fallback angles evaluate
    // them in place
    const double p_pen3 = F.gp[20], p_pen4 = F.gp[21], p_coa2 = F.gp[2];
    const double e3 = exp(-p_pen3 * d.Delta[j]), e4 = exp(p_pen4 * d.Delta[j]);
    const double trm = 1.0 + e3 + e4, f9 = (2.0 + e3) / trm;
    const double Cf9 = (-p_pen3 * e3 * trm - (2.0 + e3) * (-p_pen3 * e3 + p_pen4 * e4)) / sqr(trm);
    const double ec = exp(p_coa2 * d.Delta_val[j]), ic = 1.0 / (1.0 + ec);
    d.c_sbo[5 * n + j] = f9;
    d.c_sbo[6 * n + j] = Cf9 / f9;
    d.c_sbo[7 * n + j] = ic;
    d.c_sbo[8 * n + j] = exp(-F.gp[17] * (2.0 - SBO2));
    d.c_sbo[9 * n + j] = -p_coa2 * ec * ic;
  }
}

// per bond slot: exp(-p_tor2 BOA), exp(-p_cot2 (BOA - 1.5)^2)
__device__ __forceinline__ void vt_prep_bond_item(const Dev &d, int i, int k) {
  const int n = d.n;
  const long long s = (long long)k * n + i;
  const double BO = d.b_BO[s], BOA = BO - d.ctl->thb_cut;
  d.b_et2[s] = exp(-d.ff->gp[23] * BOA);
  d.b_ec2[s] = exp(-d.ff->gp[27] * sqr(BOA - 1.5));
  d.b_BOf[s] = BO > d.ctl->thb_cut ? (float)BO : 0.f;
  if (!d.mixed) {
    // the FP64 form's per-bond exponentials of its angles (penalty and
    // coalition)
    const long long S = (long long)d.bond_cap * n;
    d.b_vexp[s] = exp(-d.ff->gp[19] * sqr(BOA - 2.0));
    d.b_vexp[S + s] = exp(-d.ff->gp[38] * sqr(d.bo0[nbr_of(d.b_nbr[s])] - BOA));
    d.b_vexp[2 * S + s] = exp(-d.ff->gp[30] * sqr(BOA - 1.5));
  }
}

__global__ void __launch_bounds__(256) k_vt_prep_bond(Dev d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int cnt = i < d.n ? min(d.nbonds[i], d.bond_cap) : 0;
  warp_items(cnt, i, [&](int a, int k) { vt_prep_bond_item(d, a, k); });
}

__device__ __forceinline__ bool fbp_nonzero(const Fbp &p) {
  return p.V1 != 0.0 || p.V2 != 0.0 || p.V3 != 0.0 || p.p_cot1 != 0.0;
}

// a > b (b > 0) decided in FP32 away from the threshold and in FP64 within
// 1e-5 of it, so the outcome is the FP64 one
__device__ __forceinline__ bool above(float af, float bf, double a, double b) {
  if (af > bf * (1.f + 1e-5f)) return true;
  if (af < bf * (1.f - 1e-5f)) return false;
  return a > b;
}

// enumerate the items of slot (j, kk); FILL writes them at the offsets.
// The single-bond tests BO > thb_cut are the exact flags of b_BOf (0 =
// below), the product tests are FP32 away from their thresholds, and the
// parameter tests are the control block's tables: no FP64 in the common
// case.
template <bool FILL>
__device__ void vt_enumerate(const Dev &d, int j, int kk, int &cv, int &ct, long long ov,
                             long long ot) {
  const int n = d.n;
  const Control &C = *d.ctl;
  cv = ct = 0;
  const int nbj = min(d.nbonds[j], d.bond_cap);
  if (kk >= nbj) return;
  const long long spk = (long long)kk * n + j;
  const float BO_jk = d.b_BOf[spk];
  if (BO_jk == 0.f || d.b_sym[spk] < 0) return;
  const uint32_t ejk = d.b_nbr[spk];
  const int k = nbr_of(ejk), tj = d.ts[j], tk = d.ts[k];
  const long long spj = d.b_sym[spk];
  const int nbk = min(d.nbonds[k], d.bond_cap);
  const bool do_tor = tag_first(d, j, k, ejk);
  int sjk[3];
  img_unpack((int)(ejk & 255u), &sjk[0], &sjk[1], &sjk[2]);
  for (int ph = 0; ph < nbj; ++ph) {
    if (ph == kk) continue;
    const long long sph = (long long)ph * n + j;
    const float BO_hj = d.b_BOf[sph];
    if (BO_hj == 0.f) continue;   // below thb_cut: neither an angle nor a torsion end
    const uint32_t ehj = d.b_nbr[sph];
    const int h = nbr_of(ehj), th = d.ts[h];
    if (ph > kk && C.thb_any[tk][tj][th] &&
        above(BO_jk * BO_hj, C.thb_cutsq_f, d.b_BO[spk] * d.b_BO[sph], C.thb_cutsq)) {
      // (the regular path sizes the list on the host first; a captured
      // step may meet a list past its capacity: the scan total says so)
      if (FILL && ov + cv < d.cap_val)
        d.w_val[ov + cv] = ((unsigned long long)j << 16) | ((unsigned long long)kk << 8) | ph;
      ++cv;
    }
    if (!do_tor) continue;
    int shj[3];
    img_unpack((int)(ehj & 255u), &shj[0], &shj[1], &shj[2]);
    for (int pw = 0; pw < nbk; ++pw) {
      const long long spw = (long long)pw * n + k;
      if (spw == spj) continue;
      const float BO_kl = d.b_BOf[spw];
      if (BO_kl == 0.f) continue;
      const uint32_t ekl = d.b_nbr[spw];
      const int l = nbr_of(ekl);
      if (!C.fb_on[th][tj][tk][d.ts[l]]) continue;
      if (!above(BO_hj * BO_jk * BO_kl, C.thb_cut_f,
                 d.b_BO[sph] * d.b_BO[spk] * d.b_BO[spw], C.thb_cut))
        continue;
      int skl[3];
      img_unpack((int)(ekl & 255u), &skl[0], &skl[1], &skl[2]);
      if (l == h && sjk[0] + skl[0] == shj[0] && sjk[1] + skl[1] == shj[1] &&
          sjk[2] + skl[2] == shj[2])
        continue;   // i and l are the same atom instance
      if (FILL && ot + ct < d.cap_tor)
        d.w_tor[ot + ct] = ((unsigned long long)j << 24) | ((unsigned long long)kk << 16) |
                           ((unsigned long long)ph << 8) | pw;
      ++ct;
    }
  }
}

// items per bond slot (kk of centre j): one warp per 32 centres over their
// bond slots (warp_items); the slots past a centre's bond count, and the
// trailing entry of the exclusive scans, get zero
__global__ void __launch_bounds__(256) k_vt_count(Dev d) {
  const int n = d.n;
  const int j0 = blockIdx.x * blockDim.x + threadIdx.x;
  const int cnt = j0 < n ? min(d.nbonds[j0], d.bond_cap) : 0;
  if (j0 < n)
    for (int k = cnt; k < d.bond_cap; ++k) {
      d.w_cnt_v[(long long)k * n + j0] = 0;
      d.w_cnt_t[(long long)k * n + j0] = 0;
    }
  if (j0 == 0) {
    const long long slots = (long long)d.bond_cap * n;
    d.w_cnt_v[slots] = 0;
    d.w_cnt_t[slots] = 0;
  }
  warp_items(cnt, j0, [&](int j, int kk) {
    int cv, ct;
    vt_enumerate<false>(d, j, kk, cv, ct, 0, 0);
    d.w_cnt_v[(long long)kk * n + j] = cv;
    d.w_cnt_t[(long long)kk * n + j] = ct;
  });
}

__global__ void __launch_bounds__(256) k_vt_fill(Dev d) {
  const int n = d.n;
  const int j0 = blockIdx.x * blockDim.x + threadIdx.x;
  const int cnt = j0 < n ? min(d.nbonds[j0], d.bond_cap) : 0;
  warp_items(cnt, j0, [&](int j, int kk) {
    const long long t = (long long)kk * n + j;
    if (d.w_cnt_v[t] == 0 && d.w_cnt_t[t] == 0) return;
    int cv, ct;
    vt_enumerate<true>(d, j, kk, cv, ct, d.w_off_v[t], d.w_off_t[t]);
  });
}

// one valence angle h-j-k (with its penalty and coalition terms); R as in
// k_hbonds: the per-angle arithmetic in R from the FP64 per-bond and
// per-centre quantities, accumulation in FP64
template <typename R, bool VIR>
__device__ __forceinline__ void valence_item(const Dev &d, unsigned long long it, double &e_ang,
                                             double &e_pen, double &e_coa, double *w) {
  {
    const int j = (int)(it >> 16), kk = (int)((it >> 8) & 255), ph = (int)(it & 255);
    const int n = d.n;
    const ForceField &F = *d.ff;
    const double thb_cut = d.ctl->thb_cut;
    const R p_val6 = (R)F.gp[14], p_val10 = (R)F.gp[17];
    const R p_pen2 = (R)F.gp[19], p_pen3 = (R)F.gp[20], p_pen4 = (R)F.gp[21];
    const R p_coa2 = (R)F.gp[2], p_coa3 = (R)F.gp[38], p_coa4 = (R)F.gp[30];
    double *fC = d.fC;
    double *CdD = d.fC + 3 * (long long)n;
    const int tj = d.ts[j];
    const R p_val3 = (R)F.sbp[tj].p_val3, p_val5 = (R)F.sbp[tj].p_val5;
    const R SBO2 = (R)d.c_sbo[j], CSBO2 = (R)d.c_sbo[n + j];
    const R dSBO1 = (R)d.c_sbo[2 * n + j], dSBO2 = (R)d.c_sbo[3 * n + j];
    const R expval6 = (R)d.c_sbo[4 * n + j];
    const R Delta_j = (R)d.Delta_boc[j];
    const long long spk = (long long)kk * n + j, sph = (long long)ph * n + j;
    const int k = nbr_of(d.b_nbr[spk]), h = nbr_of(d.b_nbr[sph]);
    const int tk = d.ts[k], th = d.ts[h];
    const R BOA_jk = (R)(d.b_BO[spk] - thb_cut), BOA_hj = (R)(d.b_BO[sph] - thb_cut);
    const R djk[3] = {(R)d.b_dx[spk], (R)d.b_dy[spk], (R)d.b_dz[spk]};
    const R dhj[3] = {(R)d.b_dx[sph], (R)d.b_dy[sph], (R)d.b_dz[sph]};
    constexpr bool F64 = std::is_same<R, double>::value;
    // the per-centre and per-bond exponentials exist in the FP64 form only
    const bool pre = F64 && !d.mixed;
    R theta_hjk, cos_theta_hjk, di[3], dj[3], dk[3];
    theta_dcos<R>(djk, (R)d.b_d[spk], dhj, (R)d.b_d[sph], theta_hjk, cos_theta_hjk, di, dj, dk);
    // sin(acos c) = sqrt((1 - c)(1 + c)) in FP64 (no sine evaluation)
    R sin_theta_hjk = F64 ? sqrt((R(1) - cos_theta_hjk) * (R(1) + cos_theta_hjk)) : sin(theta_hjk);
    if (sin_theta_hjk < R(1.0e-5)) sin_theta_hjk = R(1.0e-5);
    const Thbh &thbh = F.thbp[tk][tj][th];
    const R Dj = (R)d.Delta[j], Dval_j = (R)d.Delta_val[j];
    const R bo0k = (R)d.bo0[k], bo0h = (R)d.bo0[h];
    // FP64: BOA^p_val4 from one logarithm per bond order and angle, and the
    // per-centre and per-bond exponentials of k_vt_prep_center/_bond
    const long long S = (long long)d.bond_cap * n;
    const R Ljk = F64 ? log(BOA_jk) : R(0), Lhj = F64 ? log(BOA_hj) : R(0);
    const R iBjk = F64 ? R(1) / BOA_jk : R(0), iBhj = F64 ? R(1) / BOA_hj : R(0);
    for (int cnt = 0; cnt < thbh.cnt; ++cnt) {
      const Thbp &tp = thbh.prm[cnt];
      if (!(fabs(tp.p_val1) > 0.001)) continue;
      const R p_val1 = (R)tp.p_val1, p_val2 = (R)tp.p_val2, p_val4 = (R)tp.p_val4, p_val7 = (R)tp.p_val7;
      const R theta_00 = (R)tp.theta_00;
      R exp3jk, Cf7jk, exp3hj, Cf7hj;
      if (F64) {
        const R pjk = exp(p_val4 * Ljk), phj = exp(p_val4 * Lhj);
        exp3jk = exp(-p_val3 * pjk);
        Cf7jk = p_val3 * p_val4 * (pjk * iBjk) * exp3jk;
        exp3hj = exp(-p_val3 * phj);
        Cf7hj = p_val3 * p_val4 * (phj * iBhj) * exp3hj;
      } else {
        exp3jk = exp(-p_val3 * pow(BOA_jk, p_val4));
        Cf7jk = p_val3 * p_val4 * pow(BOA_jk, p_val4 - R(1)) * exp3jk;
        exp3hj = exp(-p_val3 * pow(BOA_hj, p_val4));
        Cf7hj = p_val3 * p_val4 * pow(BOA_hj, p_val4 - R(1)) * exp3hj;
      }
      const R f7_jk = R(1) - exp3jk;
      const R f7_hj = R(1) - exp3hj;
      const R expval7 = exp(-p_val7 * Delta_j);
      const R trm8 = R(1) + expval6 + expval7;
      const R f8_Dj = p_val5 - ((p_val5 - R(1)) * (R(2) + expval6) / trm8);
      const R Cf8j = ((R(1) - p_val5) / sqr(trm8)) *
                     (p_val6 * expval6 * trm8 - (R(2) + expval6) * (p_val6 * expval6 - p_val7 * expval7));
      const R exp_val10 = pre ? (R)d.c_sbo[8 * n + j] : exp(-p_val10 * (R(2) - SBO2));
      R theta_0 = R(180) - theta_00 * (R(1) - exp_val10);
      theta_0 = deg2rad(theta_0);
      const R expval2theta = exp(-p_val2 * sqr(theta_0 - theta_hjk));
      const R expval12theta = (p_val1 >= R(0)) ? p_val1 * (R(1) - expval2theta) : p_val1 * -expval2theta;
      const R CEval1 = Cf7jk * f7_hj * f8_Dj * expval12theta;
      const R CEval2 = Cf7hj * f7_jk * f8_Dj * expval12theta;
      const R CEval3 = Cf8j * f7_hj * f7_jk * expval12theta;
      const R CEval4 = R(-2) * p_val1 * p_val2 * f7_jk * f7_hj * f8_Dj * expval2theta * (theta_0 - theta_hjk);
      const R Ctheta_0 = p_val10 * deg2rad(theta_00) * exp_val10;
      const R CEval5 = -CEval4 * Ctheta_0 * CSBO2;
      const R CEval6 = CEval5 * dSBO1;
      const R CEval7 = CEval5 * dSBO2;
      const R CEval8 = -CEval4 / sin_theta_hjk;
      e_ang += (double)(f7_jk * f7_hj * f8_Dj * expval12theta);
      const R exp_pen2jk = pre ? (R)d.b_vexp[spk] : exp(-p_pen2 * sqr(BOA_jk - R(2)));
      const R exp_pen2hj = pre ? (R)d.b_vexp[sph] : exp(-p_pen2 * sqr(BOA_hj - R(2)));
      // f9(Delta_j) and Cf9j / f9 per centre (FP64 form: k_vt_prep_center)
      R f9_Dj, Cf9_f9;
      if (pre) {
        f9_Dj = (R)d.c_sbo[5 * n + j];
        Cf9_f9 = (R)d.c_sbo[6 * n + j];
      } else {
        const R exp_pen3 = exp(-p_pen3 * Dj), exp_pen4 = exp(p_pen4 * Dj);
        const R trm_pen34 = R(1) + exp_pen3 + exp_pen4;
        f9_Dj = (R(2) + exp_pen3) / trm_pen34;
        const R Cf9j = (-p_pen3 * exp_pen3 * trm_pen34 -
                        (R(2) + exp_pen3) * (-p_pen3 * exp_pen3 + p_pen4 * exp_pen4)) / sqr(trm_pen34);
        Cf9_f9 = Cf9j / f9_Dj;
      }
      const R epen = (R)tp.p_pen1 * f9_Dj * exp_pen2jk * exp_pen2hj;
      e_pen += (double)epen;
      const R CEpen1 = epen * Cf9_f9;
      const R temp = R(-2) * p_pen2 * epen;
      const R CEpen2 = temp * (BOA_jk - R(2));
      const R CEpen3 = temp * (BOA_hj - R(2));
      // 1 / (1 + exp(p_coa2 Delta_val)) and -p_coa2 exp(..) / (1 + exp(..))
      // per centre in the FP64 form
      R icoa, kcoa;
      if (pre) {
        icoa = (R)d.c_sbo[7 * n + j];
        kcoa = (R)d.c_sbo[9 * n + j];
      } else {
        const R exp_coa2 = exp(p_coa2 * Dval_j);
        icoa = R(1) / (R(1) + exp_coa2);
        kcoa = -p_coa2 * exp_coa2 * icoa;
      }
      const R ecoa =
          pre ? (R)tp.p_coa1 * icoa * (R)d.b_vexp[S + spk] * (R)d.b_vexp[S + sph] *
                    (R)d.b_vexp[2 * S + spk] * (R)d.b_vexp[2 * S + sph]
              : (R)tp.p_coa1 * icoa * exp(-p_coa3 * sqr(bo0k - BOA_jk)) *
                    exp(-p_coa3 * sqr(bo0h - BOA_hj)) * exp(-p_coa4 * sqr(BOA_jk - R(1.5))) *
                    exp(-p_coa4 * sqr(BOA_hj - R(1.5)));
      e_coa += (double)ecoa;
      const R CEcoa1 = R(-2) * p_coa4 * (BOA_jk - R(1.5)) * ecoa;
      const R CEcoa2 = R(-2) * p_coa4 * (BOA_hj - R(1.5)) * ecoa;
      const R CEcoa3 = kcoa * ecoa;
      const R CEcoa4 = R(-2) * p_coa3 * (bo0k - BOA_jk) * ecoa;
      const R CEcoa5 = R(-2) * p_coa3 * (bo0h - BOA_hj) * ecoa;
      atomicAdd(&d.b_Cdbo[spk], (double)(CEval1 + CEpen2 + (CEcoa1 - CEcoa4)));
      atomicAdd(&d.b_Cdbo[sph], (double)(CEval2 + CEpen3 + (CEcoa2 - CEcoa5)));
      atomicAdd(&CdD[j], (double)((CEval3 + CEval7) + CEpen1 + CEcoa3));
      atomicAdd(&CdD[k], (double)CEcoa4);
      atomicAdd(&CdD[h], (double)CEcoa5);
      // CEval6 BO^7 to Cdbo and CEval5 to Cdbopi, Cdbopi2 of every bond of
      // j: summed per centre here, applied per bond in k_dbond
      atomicAdd(&d.vsum[j], (double)CEval5);
      atomicAdd(&d.vsum[n + j], (double)CEval6);
      if (d.debug) {
        const double v[] = {BOA_jk, BOA_hj, theta_hjk, sin_theta_hjk, SBO2, CSBO2, dSBO1, dSBO2,
                            expval6, Delta_j, f7_jk, f7_hj, f8_Dj, expval2theta, theta_0, CEval1,
                            CEval2, CEval3, CEval4, CEval5, CEval8, epen, ecoa, icoa, Cf7jk,
                            Cf7hj, Cf8j, CEpen1, CEcoa3, (double)cnt};
        double sum = 0.0;
        for (double x : v) sum += x;
        if (!isfinite(sum)) debug_record(d, 1, j, kk, ph, 0, v, (int)(sizeof(v) / sizeof(v[0])));
      }
      const double c8 = (double)CEval8;
      add3(fC, n, k, c8, (double)di[0], (double)di[1], (double)di[2]);
      add3(fC, n, j, c8, (double)dj[0], (double)dj[1], (double)dj[2]);
      add3(fC, n, h, c8, (double)dk[0], (double)dk[1], (double)dk[2]);
      if (VIR) {
        vir_acc(w, d.b_dx[spk], d.b_dy[spk], d.b_dz[spk], c8 * di[0], c8 * di[1], c8 * di[2]);
        vir_acc(w, d.b_dx[sph], d.b_dy[sph], d.b_dz[sph], c8 * dk[0], c8 * dk[1], c8 * dk[2]);
      }
    }
  }
}

// FP32 is not used for angles within about 1.1 degrees of 0 or 180 (sine
// below 0.02): there the reference's 1/sin factors (MIN_SINE clamps at
// 1e-10) overflow FP32 and its cancellations lose the result.  The FP32
// kernels queue those items (and the over-coordination cases below) for an
// FP64 pass.
__device__ __forceinline__ bool near_linear(const Dev &d, long long sa, long long sb) {
  const float ax = (float)d.b_dx[sa], ay = (float)d.b_dy[sa], az = (float)d.b_dz[sa];
  const float bx = (float)d.b_dx[sb], by = (float)d.b_dy[sb], bz = (float)d.b_dz[sb];
  const float c = (ax * bx + ay * by + az * bz) / ((float)d.b_d[sa] * (float)d.b_d[sb]);
  return fabsf(c) > 0.9998f;
}

__device__ __forceinline__ void valence_energies(const Dev &d, int eflag, int sg, double e_ang,
                                                 double e_pen, double e_coa) {
  if (eflag) {
    energy_add(d, e_ang, sg, E_ANG);
    energy_add(d, e_pen, sg, E_PEN);
    energy_add(d, e_coa, sg, E_COA);
    energy_add(d, e_ang + e_pen + e_coa, sg, E_ENG_VDWL);
  }
}

template <typename R, bool VIR>
__global__ void __launch_bounds__(128) k_valence(Dev d, int eflag, long long nitems,
                                                 const int *ntot) {
  const long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (ntot) nitems = min(nitems, (long long)*ntot);
  double e_ang = 0, e_pen = 0, e_coa = 0;
  double vw[6] = {0, 0, 0, 0, 0, 0};
  int sg = -1;
  if (w < nitems) {
    const unsigned long long it = d.w_val[w];
    sg = d.seg_s[(int)(it >> 16)];
    if (std::is_same<R, float>::value) {
      const int j = (int)(it >> 16), kk = (int)((it >> 8) & 255), ph = (int)(it & 255);
      // FP64 as well for strongly over-coordinated centres, where
      // exp(p_val6 Delta) (p_val6 ~ 34) and exp(p_coa2 Delta_val) and their
      // products leave the FP32 range
      if (near_linear(d, (long long)kk * d.n + j, (long long)ph * d.n + j) ||
          d.Delta_boc[j] > 1.0 || d.Delta_val[j] > 2.0)
        d.w_fb_val[atomicAdd(&d.fb_cnt[0], 1)] = it;
      else
        valence_item<R, VIR>(d, it, e_ang, e_pen, e_coa, vw);
    } else {
      valence_item<R, VIR>(d, it, e_ang, e_pen, e_coa, vw);
    }
  }
  valence_energies(d, eflag, sg, e_ang, e_pen, e_coa);
  if (VIR) seg_block_add<6>(vw, sg, d.virial, 6);
}

// the FP64 pass over the queued near-linear angles (grid-stride over the
// device-side count; few items, so energies go straight to their segment)
template <bool VIR>
__device__ void valence_fb(const Dev &d, int eflag, long long first, long long stride) {
  const long long cnt = d.fb_cnt[0];
  for (long long w = first; w < cnt; w += stride) {
    double e_ang = 0, e_pen = 0, e_coa = 0;
    double vw[6] = {0, 0, 0, 0, 0, 0};
    const unsigned long long it = d.w_fb_val[w];
    valence_item<double, VIR>(d, it, e_ang, e_pen, e_coa, vw);
    const int sg = d.seg_s[(int)(it >> 16)];
    if (eflag) {
      double *E = d.energy + (long long)sg * RG_NE;
      atomicAdd(&E[E_ANG], e_ang);
      atomicAdd(&E[E_PEN], e_pen);
      atomicAdd(&E[E_COA], e_coa);
      atomicAdd(&E[E_ENG_VDWL], e_ang + e_pen + e_coa);
    }
    if (VIR)
      for (int c = 0; c < 6; ++c) atomicAdd(&d.virial[(long long)sg * 6 + c], vw[c]);
  }
}

// one torsion h-j-k-l (with its 4-body conjugation term); R as in k_valence
template <typename R, bool VIR>
__device__ __forceinline__ void torsion_item(const Dev &d, unsigned long long it, double &e_tor,
                                             double &e_con, double *w) {
  {
    const int j = (int)(it >> 24), kk = (int)((it >> 16) & 255);
    const int ph = (int)((it >> 8) & 255), pw = (int)(it & 255);
    const int n = d.n;
    const ForceField &F = *d.ff;
    const double thb_cut = d.ctl->thb_cut;
    const R p_tor2 = (R)F.gp[23], p_tor3 = (R)F.gp[24], p_tor4 = (R)F.gp[25], p_cot2 = (R)F.gp[27];
    double *fC = d.fC;
    double *CdD = d.fC + 3 * (long long)n;
    const long long spk = (long long)kk * n + j, sph = (long long)ph * n + j;
    const int k = nbr_of(d.b_nbr[spk]), i = nbr_of(d.b_nbr[sph]);
    const long long spj = d.b_sym[spk];
    const long long spw = (long long)pw * n + k;
    const int l = nbr_of(d.b_nbr[spw]);
    const Fbp &fbp = F.fbp[d.ts[i]][d.ts[j]][d.ts[k]][d.ts[l]].prm;
    const R V1 = (R)fbp.V1, V2 = (R)fbp.V2, V3 = (R)fbp.V3;
    const R p_tor1 = (R)fbp.p_tor1, p_cot1 = (R)fbp.p_cot1;
    const R BOA_jk = (R)(d.b_BO[spk] - thb_cut), BOA_ij = (R)(d.b_BO[sph] - thb_cut);
    const R BOA_kl = (R)(d.b_BO[spw] - thb_cut);
    const R Delta_j = (R)d.Delta_boc[j], Delta_k = (R)d.Delta_boc[k];
    const R exp_tor3_DjDk = exp(-p_tor3 * (Delta_j + Delta_k));
    const R exp_tor4_DjDk = exp(p_tor4 * (Delta_j + Delta_k));
    const R exp_tor34_inv = R(1) / (R(1) + exp_tor3_DjDk + exp_tor4_DjDk);
    const R f11_DjDk = (R(2) + exp_tor3_DjDk) * exp_tor34_inv;
    const R exp_tor2_jk = (R)d.b_et2[spk], exp_cot2_jk = (R)d.b_ec2[spk];
    const R exp_tor2_ij = (R)d.b_et2[sph], exp_cot2_ij = (R)d.b_ec2[sph];
    const R exp_tor2_kl = (R)d.b_et2[spw], exp_cot2_kl = (R)d.b_ec2[spw];
    const R djk[3] = {(R)d.b_dx[spk], (R)d.b_dy[spk], (R)d.b_dz[spk]};
    const R dhj[3] = {(R)d.b_dx[sph], (R)d.b_dy[sph], (R)d.b_dz[sph]};
    const R dkl[3] = {(R)d.b_dx[spw], (R)d.b_dy[spw], (R)d.b_dz[spw]};
    const R dpj[3] = {(R)d.b_dx[spj], (R)d.b_dy[spj], (R)d.b_dz[spj]};
    const R r_jk = (R)d.b_d[spk], r_ij = (R)d.b_d[sph], r_kl = (R)d.b_d[spw];
    // FP64: the angles' sines from their cosines, sqrt((1 - c)(1 + c)) =
    // sin(acos c), and omega's cosines from its two components (no acos,
    // sincos, atan2 or cos evaluation); FP32: the reference's sequence
    constexpr bool F64 = std::is_same<R, double>::value;
    Thb<R> p_ijk, p_jkl;
    theta_dcos<R, !F64>(djk, r_jk, dhj, r_ij, p_ijk.theta, p_ijk.cos, p_ijk.di, p_ijk.dj, p_ijk.dk);
    theta_dcos<R, !F64>(dpj, (R)d.b_d[spj], dkl, r_kl, p_jkl.theta, p_jkl.cos, p_jkl.di, p_jkl.dj,
                        p_jkl.dk);
    if (F64) {
      p_ijk.sin = sqrt((R(1) - p_ijk.cos) * (R(1) + p_ijk.cos));
      p_jkl.sin = sqrt((R(1) - p_jkl.cos) * (R(1) + p_jkl.cos));
    } else {
      sincos(p_ijk.theta, &p_ijk.sin, &p_ijk.cos);
      sincos(p_jkl.theta, &p_jkl.sin, &p_jkl.cos);
    }
    const R ms = (R)MIN_SINE;
    R tan_ijk_i, tan_jkl_i;
    const R sin_ijk = p_ijk.sin, cos_ijk = p_ijk.cos, sin_jkl = p_jkl.sin, cos_jkl = p_jkl.cos;
    if (sin_ijk >= R(0) && sin_ijk <= ms) tan_ijk_i = cos_ijk / ms;
    else if (sin_ijk <= R(0) && sin_ijk >= -ms) tan_ijk_i = cos_ijk / -ms;
    else tan_ijk_i = cos_ijk / sin_ijk;
    if (sin_jkl >= R(0) && sin_jkl <= ms) tan_jkl_i = cos_jkl / ms;
    else if (sin_jkl <= R(0) && sin_jkl >= -ms) tan_jkl_i = cos_jkl / -ms;
    else tan_jkl_i = cos_jkl / sin_jkl;
    R dli[3];
    dli[0] = dhj[0] - djk[0] - dkl[0];
    dli[1] = dhj[1] - djk[1] - dkl[1];
    dli[2] = dhj[2] - djk[2] - dkl[2];
    const R r_li = sqrt(sqr(dli[0]) + sqr(dli[1]) + sqr(dli[2]));
    R doi[3], doj[3], dok[3], dol[3];
    R uc, us;
    calc_omega<R>(dhj, r_ij, djk, r_jk, dkl, r_kl, dli, r_li, p_ijk, p_jkl, doi, doj, dok, dol, uc,
                  us);
    R cos_omega, cos2omega, cos3omega;
    if (F64) {
      const R hyp = sqrt(uc * uc + us * us);
      cos_omega = hyp > R(0) ? uc / hyp : R(1);   // atan2(0, 0) = 0
      cos2omega = R(2) * cos_omega * cos_omega - R(1);
      cos3omega = cos_omega * (R(4) * cos_omega * cos_omega - R(3));
    } else {
      const R omega = atan2(us, uc);
      cos_omega = cos(omega);
      cos2omega = cos(R(2) * omega);
      cos3omega = cos(R(3) * omega);
    }
    const R BOpi_jk = (R)d.b_BOpi[spk];
    const R exp_tor1 = exp(p_tor1 * sqr(R(2) - BOpi_jk - f11_DjDk));
    const R fn10 = (R(1) - exp_tor2_ij) * (R(1) - exp_tor2_jk) * (R(1) - exp_tor2_kl);
    const R CV = R(0.5) * (V1 * (R(1) + cos_omega) + V2 * exp_tor1 * (R(1) - cos2omega) +
                           V3 * (R(1) + cos3omega));
    e_tor = (double)(fn10 * sin_ijk * sin_jkl * CV);
    R dfn11;
    if (std::is_same<R, double>::value) {
      dfn11 = (-p_tor3 * exp_tor3_DjDk +
               (p_tor3 * exp_tor3_DjDk - p_tor4 * exp_tor4_DjDk) * (R(2) + exp_tor3_DjDk) * exp_tor34_inv) *
              exp_tor34_inv;
    } else {
      // the same value with every product bounded: for Delta_j + Delta_k
      // near -4 the product of the two exponentials above exceeds FP32
      const R a3 = p_tor3 * (exp_tor3_DjDk * exp_tor34_inv);
      const R a4 = p_tor4 * (exp_tor4_DjDk * exp_tor34_inv);
      dfn11 = -a3 + (a3 - a4) * f11_DjDk;
    }
    const R CEtors1 = sin_ijk * sin_jkl * CV;
    const R CEtors2 = -fn10 * R(2) * p_tor1 * V2 * exp_tor1 * (R(2) - BOpi_jk - f11_DjDk) *
                      (R(1) - sqr(cos_omega)) * sin_ijk * sin_jkl;
    const R CEtors3 = CEtors2 * dfn11;
    const R CEtors4 = CEtors1 * p_tor2 * exp_tor2_ij * (R(1) - exp_tor2_jk) * (R(1) - exp_tor2_kl);
    const R CEtors5 = CEtors1 * p_tor2 * (R(1) - exp_tor2_ij) * exp_tor2_jk * (R(1) - exp_tor2_kl);
    const R CEtors6 = CEtors1 * p_tor2 * (R(1) - exp_tor2_ij) * (R(1) - exp_tor2_jk) * exp_tor2_kl;
    const R cmn = -fn10 * CV;
    const R CEtors7 = cmn * sin_jkl * tan_ijk_i;
    const R CEtors8 = cmn * sin_ijk * tan_jkl_i;
    const R CEtors9 = fn10 * sin_ijk * sin_jkl *
                      (R(0.5) * V1 - R(2) * V2 * exp_tor1 * cos_omega +
                       R(1.5) * V3 * (cos2omega + R(2) * sqr(cos_omega)));
    const R fn12 = exp_cot2_ij * exp_cot2_jk * exp_cot2_kl;
    e_con = (double)(p_cot1 * fn12 * (R(1) + (sqr(cos_omega) - R(1)) * sin_ijk * sin_jkl));
    const R Cconj = R(-2) * fn12 * p_cot1 * p_cot2 * (R(1) + (sqr(cos_omega) - R(1)) * sin_ijk * sin_jkl);
    const R CEconj1 = Cconj * (BOA_ij - R(1.5));
    const R CEconj2 = Cconj * (BOA_jk - R(1.5));
    const R CEconj3 = Cconj * (BOA_kl - R(1.5));
    const R CEconj4 = -p_cot1 * fn12 * (sqr(cos_omega) - R(1)) * sin_jkl * tan_ijk_i;
    const R CEconj5 = -p_cot1 * fn12 * (sqr(cos_omega) - R(1)) * sin_ijk * tan_jkl_i;
    const R CEconj6 = R(2) * p_cot1 * fn12 * cos_omega * sin_ijk * sin_jkl;
    atomicAdd(&d.b_Cdbopi[spk], (double)CEtors2);
    atomicAdd(&CdD[j], (double)CEtors3);
    atomicAdd(&CdD[k], (double)CEtors3);
    atomicAdd(&d.b_Cdbo[sph], (double)(CEtors4 + CEconj1));
    atomicAdd(&d.b_Cdbo[spk], (double)(CEtors5 + CEconj2));
    atomicAdd(&d.b_Cdbo[spw], (double)(CEtors6 + CEconj3));
    const R c78 = CEtors7 + CEconj4, c85 = CEtors8 + CEconj5, c96 = CEtors9 + CEconj6;
    if (d.debug) {
      const double v[] = {BOA_ij, BOA_jk, BOA_kl, cos_ijk, cos_jkl, sin_ijk, sin_jkl,
                          tan_ijk_i, tan_jkl_i, cos_omega, r_li, exp_tor1, fn10, CV, c78, c85, c96,
                          CEtors2, CEtors3, CEtors4, CEtors5, CEtors6, doi[0], doj[0], dok[0],
                          dol[0], f11_DjDk, dfn11, Delta_j, Delta_k};
      double sum = 0.0;
      for (double x : v) sum += x;
      if (!isfinite(sum)) debug_record(d, 2, j, kk, ph, pw, v, (int)(sizeof(v) / sizeof(v[0])));
    }
    add3(fC, n, i, 1.0, (double)(c78 * p_ijk.dk[0] + c96 * doi[0]), (double)(c78 * p_ijk.dk[1] + c96 * doi[1]),
         (double)(c78 * p_ijk.dk[2] + c96 * doi[2]));
    add3(fC, n, j, 1.0, (double)(c78 * p_ijk.dj[0] + c85 * p_jkl.di[0] + c96 * doj[0]),
         (double)(c78 * p_ijk.dj[1] + c85 * p_jkl.di[1] + c96 * doj[1]),
         (double)(c78 * p_ijk.dj[2] + c85 * p_jkl.di[2] + c96 * doj[2]));
    add3(fC, n, k, 1.0, (double)(c78 * p_ijk.di[0] + c85 * p_jkl.dj[0] + c96 * dok[0]),
         (double)(c78 * p_ijk.di[1] + c85 * p_jkl.dj[1] + c96 * dok[1]),
         (double)(c78 * p_ijk.di[2] + c85 * p_jkl.dj[2] + c96 * dok[2]));
    add3(fC, n, l, 1.0, (double)(c85 * p_jkl.dk[0] + c96 * dol[0]), (double)(c85 * p_jkl.dk[1] + c96 * dol[1]),
         (double)(c85 * p_jkl.dk[2] + c96 * dol[2]));
    if (VIR) {
      // positions relative to j: i = j + d(j->i), k = j + d(j->k), l = k + d(k->l)
      const double ax = d.b_dx[sph], ay = d.b_dy[sph], az = d.b_dz[sph];
      const double bx = d.b_dx[spk], by = d.b_dy[spk], bz = d.b_dz[spk];
      const double lx = bx + d.b_dx[spw], ly = by + d.b_dy[spw], lz = bz + d.b_dz[spw];
      vir_acc(w, ax, ay, az, (double)(c78 * p_ijk.dk[0] + c96 * doi[0]),
              (double)(c78 * p_ijk.dk[1] + c96 * doi[1]), (double)(c78 * p_ijk.dk[2] + c96 * doi[2]));
      vir_acc(w, bx, by, bz, (double)(c78 * p_ijk.di[0] + c85 * p_jkl.dj[0] + c96 * dok[0]),
              (double)(c78 * p_ijk.di[1] + c85 * p_jkl.dj[1] + c96 * dok[1]),
              (double)(c78 * p_ijk.di[2] + c85 * p_jkl.dj[2] + c96 * dok[2]));
      vir_acc(w, lx, ly, lz, (double)(c85 * p_jkl.dk[0] + c96 * dol[0]),
              (double)(c85 * p_jkl.dk[1] + c96 * dol[1]), (double)(c85 * p_jkl.dk[2] + c96 * dol[2]));
    }
  }
}

__device__ __forceinline__ void torsion_energies(const Dev &d, int eflag, int sg, double e_tor,
                                                 double e_con) {
  if (eflag) {
    energy_add(d, e_tor, sg, E_TOR);
    energy_add(d, e_con, sg, E_CON);
    energy_add(d, e_tor + e_con, sg, E_ENG_VDWL);
  }
}

template <typename R, bool VIR>
__global__ void __launch_bounds__(128) k_torsion(Dev d, int eflag, long long nitems,
                                                 const int *ntot) {
  const long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (ntot) nitems = min(nitems, (long long)*ntot);
  double e_tor = 0, e_con = 0;
  double vw[6] = {0, 0, 0, 0, 0, 0};
  int sg = -1;
  if (w < nitems) {
    const unsigned long long it = d.w_tor[w];
    sg = d.seg_s[(int)(it >> 24)];
    if (std::is_same<R, float>::value) {
      const int n = d.n;
      const int j = (int)(it >> 24), kk = (int)((it >> 16) & 255);
      const int ph = (int)((it >> 8) & 255), pw = (int)(it & 255);
      const long long spk = (long long)kk * n + j, sph = (long long)ph * n + j;
      const int k = nbr_of(d.b_nbr[spk]);
      const long long spj = d.b_sym[spk], spw = (long long)pw * n + k;
      if (near_linear(d, spk, sph) || near_linear(d, spj, spw))
        d.w_fb_tor[atomicAdd(&d.fb_cnt[1], 1)] = it;
      else
        torsion_item<R, VIR>(d, it, e_tor, e_con, vw);
    } else {
      torsion_item<R, VIR>(d, it, e_tor, e_con, vw);
    }
  }
  torsion_energies(d, eflag, sg, e_tor, e_con);
  if (VIR) seg_block_add<6>(vw, sg, d.virial, 6);
}

template <bool VIR>
__device__ void torsion_fb(const Dev &d, int eflag, long long first, long long stride) {
  const long long cnt = d.fb_cnt[1];
  for (long long w = first; w < cnt; w += stride) {
    double e_tor = 0, e_con = 0;
    double vw[6] = {0, 0, 0, 0, 0, 0};
    const unsigned long long it = d.w_fb_tor[w];
    torsion_item<double, VIR>(d, it, e_tor, e_con, vw);
    const int sg = d.seg_s[(int)(it >> 24)];
    if (eflag) {
      double *E = d.energy + (long long)sg * RG_NE;
      atomicAdd(&E[E_TOR], e_tor);
      atomicAdd(&E[E_CON], e_con);
      atomicAdd(&E[E_ENG_VDWL], e_tor + e_con);
    }
    if (VIR)
      for (int c = 0; c < 6; ++c) atomicAdd(&d.virial[(long long)sg * 6 + c], vw[c]);
  }
}

// the FP64 passes over the queued angles (first half of the blocks) and
// torsions (second half) in one launch, so their latencies overlap
template <bool VIR>
__global__ void __launch_bounds__(128) k_vt_fb(Dev d, int eflag) {
  const int half = gridDim.x / 2;
  const bool val = (int)blockIdx.x < half;
  const long long first = (long long)(val ? blockIdx.x : blockIdx.x - half) * blockDim.x + threadIdx.x;
  const long long stride = (long long)half * blockDim.x;
  if (val) valence_fb<VIR>(d, eflag, first, stride);
  else torsion_fb<VIR>(d, eflag, first, stride);
}

// ------------------------------------------------------------------
// bond-order derivative forces: one thread per atom i over its bonds

template <bool VIR>
__global__ void k_dbond(Dev d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = d.n;
  // virial: the pieces along a bond i-k that act on i here and on k in k's
  // pass count half each; the Delta' pieces (on i and on all of i's
  // neighbours m, both here) count whole
  double w[6] = {0, 0, 0, 0, 0, 0};
  if (i < n) {
    const long long S = (long long)d.bond_cap * n;
    const int nb = min(d.nbonds[i], d.bond_cap);
    const double *CdD = d.fC + 3 * (long long)n;
    const double Ddx = d.dDeltap[i], Ddy = d.dDeltap[n + i], Ddz = d.dDeltap[2 * n + i];
    const double cdi = CdD[i];
    const double v5i = d.vsum[i], v6i = d.vsum[n + i];
    double fx = 0, fy = 0, fz = 0, buf_c = 0;
    for (int k = 0; k < nb; ++k) {
      const long long s = (long long)k * n + i;
      const int j = nbr_of(d.b_nbr[s]);
      const long long sy = d.b_sym[s];
      // the valence centres' shares: CEval6 BO^7 and CEval5 from both ends
      const double bs = d.b_BO[s], bs3 = bs * bs * bs;
      double cdbo = d.b_Cdbo[s] + v6i * (bs3 * bs3 * bs);
      double cdbopi = d.b_Cdbopi[s] + v5i, cdbopi2 = d.b_Cdbopi2[s] + v5i;
      if (sy >= 0) {
        const double by = d.b_BO[sy], by3 = by * by * by;
        const double v5j = d.vsum[j], v6j = d.vsum[n + j];
        cdbo += d.b_Cdbo[sy] + v6j * (by3 * by3 * by);
        cdbopi += d.b_Cdbopi[sy] + v5j;
        cdbopi2 += d.b_Cdbopi2[sy] + v5j;
      }
      const double C1dbo = d.b_C[0 * S + s], C2dbo = d.b_C[1 * S + s];
      const double C1pi = d.b_C[3 * S + s], C2pi = d.b_C[4 * S + s], C3pi = d.b_C[5 * S + s];
      const double C1pi2 = d.b_C[7 * S + s], C2pi2 = d.b_C[8 * S + s], C3pi2 = d.b_C[9 * S + s];
      const double cdd = cdi + CdD[j];
      const double a = C1dbo * cdbo + C1dbo * cdd + C2pi * cdbopi + C2pi2 * cdbopi2;  // along dBOp
      const double b = C2dbo * cdbo + C2dbo * cdd + C3pi * cdbopi + C3pi2 * cdbopi2;  // along dDeltap_i
      const double cpi = C1pi * cdbopi, cpi2 = C1pi2 * cdbopi2;
      const double gx = d.b_dBOp[s], gy = d.b_dBOp[S + s], gz = d.b_dBOp[2 * S + s];
      const double px = a * gx + cpi * d.b_dlnpi[s] + cpi2 * d.b_dlnpi2[s];
      const double py = a * gy + cpi * d.b_dlnpi[S + s] + cpi2 * d.b_dlnpi2[S + s];
      const double pz = a * gz + cpi * d.b_dlnpi[2 * S + s] + cpi2 * d.b_dlnpi2[2 * S + s];
      fx += px + b * Ddx;
      fy += py + b * Ddy;
      fz += pz + b * Ddz;
      buf_c -= b;
      if (VIR) vir_acc(w, d.b_dx[s], d.b_dy[s], d.b_dz[s], -0.5 * px, -0.5 * py, -0.5 * pz);
    }
    double *fC = d.fC;
    atomicAdd(&fC[i], fx);
    atomicAdd(&fC[n + i], fy);
    atomicAdd(&fC[2 * n + i], fz);
    if (buf_c != 0.0)
      for (int k = 0; k < nb; ++k) {
        const long long s = (long long)k * n + i;
        const int j = nbr_of(d.b_nbr[s]);
        const double gx = d.b_dBOp[s], gy = d.b_dBOp[S + s], gz = d.b_dBOp[2 * S + s];
        add3(fC, n, j, buf_c, gx, gy, gz);
        if (VIR) vir_acc(w, d.b_dx[s], d.b_dy[s], d.b_dz[s], buf_c * gx, buf_c * gy, buf_c * gz);
      }
  }
  if (VIR) seg_block_add<6>(w, i < n ? d.seg_s[i] : -1, d.virial, 6);
}

// forces back to the original atom order: f = -dE/dx
__global__ void k_force_out(Dev d) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= d.n) return;
  const int n = d.n, i = d.perm[s];
  double fx = -d.fC[s], fy = -d.fC[n + s], fz = -d.fC[2 * n + s];
  if (d.fC32) {   // mixed form: the FP32 pair terms' forces
    fx -= (double)d.fC32[s];
    fy -= (double)d.fC32[n + s];
    fz -= (double)d.fC32[2 * n + s];
  }
  if (!(isfinite(fx) && isfinite(fy) && isfinite(fz))) atomicOr(&d.status[ST_NAN], 1);
  d.f_o[3 * i + 0] = fx;
  d.f_o[3 * i + 1] = fy;
  d.f_o[3 * i + 2] = fz;
}

// failure detection: sets *flag if any of a[0..count) is not finite
__global__ void k_check_finite(const double *a, long long count, int *flag) {
  bool bad = false;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x)
    bad |= !isfinite(a[i]);
  if (__any_sync(FULL, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

}  // namespace

void launch_check_finite(const double *a, long long count, int *flag, cudaStream_t st) {
  k_check_finite<<<152 * 4, 256, 0, st>>>(a, count, flag);
}

void launch_bond_orders(const Dev &d, cudaStream_t st) {
  const int B = 256;
  k_bo_deltap<<<(d.n + B - 1) / B, B, 0, st>>>(d);
  k_bo_correct<<<(unsigned)((d.n + 255) / 256), 256, 0, st>>>(d);
  k_bo_atom<<<(d.n + B - 1) / B, B, 0, st>>>(d);
}

void launch_atom_energy(const Dev &d, cudaStream_t st, int eflag) {
  k_atom_energy<<<(d.n + 255) / 256, 256, 0, st>>>(d, eflag);
  k_bond_energy<<<(d.n + 255) / 256, 256, 0, st>>>(d, eflag);
}

void launch_hbonds(const Dev &d, cudaStream_t st, int eflag) {
  const long long threads = (long long)d.n * 32;
  const unsigned G = (unsigned)((threads + 255) / 256);
  if (d.vflag) {
    if (d.mixed) k_hbonds32<true><<<G, 256, 0, st>>>(d, eflag);
    else k_hbonds<true><<<G, 256, 0, st>>>(d, eflag);
  } else {
    if (d.mixed) k_hbonds32<false><<<G, 256, 0, st>>>(d, eflag);
    else k_hbonds<false><<<G, 256, 0, st>>>(d, eflag);
  }
}

void launch_vt_count(const Dev &d, cudaStream_t st) {
  const int B = 256;
  const long long slots = (long long)d.n * d.bond_cap;
  k_vt_prep_center<<<(d.n + B - 1) / B, B, 0, st>>>(d);
  k_vt_prep_bond<<<(unsigned)((d.n + 255) / 256), 256, 0, st>>>(d);
  k_vt_count<<<(unsigned)((d.n + 255) / 256), 256, 0, st>>>(d);
  launch_scan(d.w_cnt_v, d.w_off_v, (int)(slots + 1), d.w_bsum, st);
  launch_scan(d.w_cnt_t, d.w_off_t, (int)(slots + 1), d.w_bsum, st);
}

template <bool VIR>
static void vt_kernels(const Dev &d, cudaStream_t st, int eflag, long long nval, long long ntor,
                       unsigned gv, unsigned gt, const int *tv, const int *tt) {
  if (d.mixed) {
    cudaMemsetAsync(d.fb_cnt, 0, 2 * sizeof(int), st);
    if (nval > 0) k_valence<float, VIR><<<gv, 128, 0, st>>>(d, eflag, nval, tv);
    if (ntor > 0) k_torsion<float, VIR><<<gt, 128, 0, st>>>(d, eflag, ntor, tt);
    // FP64 passes over the near-linear items (count read on the device;
    // usually none or a few, so a small grid that strides)
    k_vt_fb<VIR><<<32, 128, 0, st>>>(d, eflag);
  } else {
    if (nval > 0) k_valence<double, VIR><<<gv, 128, 0, st>>>(d, eflag, nval, tv);
    if (ntor > 0) k_torsion<double, VIR><<<gt, 128, 0, st>>>(d, eflag, ntor, tt);
  }
}

// nval, ntor: the item counts the host read back, or (device_counts) the
// list capacities, the kernels then taking the counts from the scan totals
void launch_vt_run(const Dev &d, cudaStream_t st, int eflag, long long nval, long long ntor,
                   bool device_counts) {
  k_vt_fill<<<(unsigned)((d.n + 255) / 256), 256, 0, st>>>(d);
  const unsigned gv = (unsigned)((nval + 127) / 128), gt = (unsigned)((ntor + 127) / 128);
  const long long slots = (long long)d.n * d.bond_cap;
  const int *tv = device_counts ? d.w_off_v + slots : nullptr;
  const int *tt = device_counts ? d.w_off_t + slots : nullptr;
  if (d.vflag) vt_kernels<true>(d, st, eflag, nval, ntor, gv, gt, tv, tt);
  else vt_kernels<false>(d, st, eflag, nval, ntor, gv, gt, tv, tt);
}

void launch_dbond_forces(const Dev &d, cudaStream_t st) {
  const int B = 256;
  if (d.vflag) k_dbond<true><<<(d.n + B - 1) / B, B, 0, st>>>(d);
  else k_dbond<false><<<(d.n + B - 1) / B, B, 0, st>>>(d);
}

void launch_force_out(const Dev &d, cudaStream_t st) {
  const int B = 256;
  k_force_out<<<(d.n + B - 1) / B, B, 0, st>>>(d);
}


// Bond-order correction and the bonded energy terms.
//
//  k_bo_deltap / k_bo_correct / k_bo_atom: BO_Section1/2/3
//      (reaxc_bond_orders_sw64.c:56-64, :162-377, :451-482)
//  k_atom_energy: bond energy, lone pair, over/under-coordination and
//      polarisation, Merge_Bonds_Atom_Energy_C_New (reaxc_multi_body_sw64.c:21-333)
//  k_hbonds: Hydrogen_Bonds_C (reaxc_hydrogen_bonds_sw64.c:146-248)
//  k_valence_torsion: Merge_Torsion_Valence_Angles
//      (reaxc_torsion_angles_sw64.c:813-1367) with Calculate_Omega (:21-102)
//  k_dbond: Add_All_dBond_to_Forces_C (reaxc_forces_sw64.c:499-588)
//
// Every term is evaluated once per centre atom as in the reference; the
// reference's ghost atoms become (atom, periodic image) pairs carried in the
// bond entries, so forces and CdDelta land directly on the owning atoms.
// Scattered accumulations use FP64 atomics.
#include "rg_internal.h"

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr double constPI = 3.14159265;          // reaxc_defs_sunway.h:58
constexpr double KCALpMOL_to_EV = 23.02;        // reaxc_defs_sunway.h:69
constexpr double HB_THRESHOLD = 1e-2;           // reaxc_defs_sunway.h:91
constexpr double MIN_SINE = 1e-10;

__device__ __forceinline__ double deg2rad(double a) { return a * constPI / 180.0; }
__device__ __forceinline__ double sqr(double x) { return x * x; }

// per-block reduction of one value into dst (FP64 atomic)
__device__ __forceinline__ void block_add(double v, double *dst) {
  __shared__ double red[32];
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(FULL, v, off);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = (l < (int)(blockDim.x >> 5)) ? red[l] : 0.0;
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(FULL, v, off);
    if (l == 0 && v != 0.0) atomicAdd(dst, v);
  }
}

__device__ __forceinline__ void add3(double *fC, int n, int a, double s, double x, double y, double z) {
  atomicAdd(&fC[a], s * x);
  atomicAdd(&fC[n + a], s * y);
  atomicAdd(&fC[2 * n + a], s * z);
}

__device__ __forceinline__ int nbr_of(uint32_t e) { return (int)(e >> 8); }

// (tag, position) order deciding which end of a bond / central torsion
// bond carries the term, reaxc_multi_body_sw64.c:256-267
__device__ __forceinline__ bool tag_first(const Dev &d, int i, int j, uint32_t e) {
  const int ti = d.tags[i], tj = d.tags[j];
  if (ti > tj) return false;
  if (ti == tj) {
    int sx, sy, sz;
    img_unpack((int)(e & 255u), &sx, &sy, &sz);
    const double4 xi = d.xs[i], xj0 = d.xs[j];
    const double xj = xj0.x + sx * d.L[0], yj = xj0.y + sy * d.L[1], zj = xj0.z + sz * d.L[2];
    if (zj < xi.z) return false;
    if (zj == xi.z && yj < xi.y) return false;
    if (zj == xi.z && yj == xi.y && xj < xi.x) return false;
  }
  return true;
}

// Calculate_Theta / Calculate_dCos_Theta, reaxc_valence_angles_sunway.cpp:49-79
__device__ __forceinline__ void theta_dcos(const double *dji, double d_ji, const double *djk,
                                           double d_jk, double &theta, double &cos_theta,
                                           double *di, double *dj, double *dk) {
  const double dot = dji[0] * djk[0] + dji[1] * djk[1] + dji[2] * djk[2];
  cos_theta = dot / (d_ji * d_jk);
  if (cos_theta > 1.) cos_theta = 1.0;
  if (cos_theta < -1.) cos_theta = -1.0;
  theta = acos(cos_theta);
  const double sqr_d_ji = d_ji * d_ji, sqr_d_jk = d_jk * d_jk;
  const double inv_dists = 1.0 / (d_ji * d_jk);
  const double inv_dists3 = inv_dists * inv_dists * inv_dists;
  const double Cdot_inv3 = dot * inv_dists3;
#pragma unroll
  for (int t = 0; t < 3; ++t) {
    di[t] = djk[t] * inv_dists - Cdot_inv3 * sqr_d_jk * dji[t];
    dj[t] = -(djk[t] + dji[t]) * inv_dists + Cdot_inv3 * (sqr_d_jk * dji[t] + sqr_d_ji * djk[t]);
    dk[t] = dji[t] * inv_dists - Cdot_inv3 * sqr_d_ji * djk[t];
  }
}

// ------------------------------------------------------------------
// bond orders

__global__ void k_bo_deltap(Dev d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n) return;
  const Sbp &s = d.ff->sbp[d.ts[i]];
  const double b = d.bo0[i];
  d.Deltap[i] = b - s.valency;
  d.Deltap_boc[i] = b - s.valency_val;
}

__global__ void k_bo_correct(Dev d) {
  const int n = d.n;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int i = (int)(t % n), k = (int)(t / n);
  if (k >= d.bond_cap || i >= n || k >= d.nbonds[i]) return;
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
    const double Deltap_i = d.Deltap[i], Deltap_j = d.Deltap[j];
    const double Dboc_i = d.Deltap_boc[i], Dboc_j = d.Deltap_boc[j];
    double f1, Cf1_ij, Cf1_ji, f4, f5, f4f5, Cf45_ij, Cf45_ji;
    if (tw.ovc >= 0.001) {
      const double exp_p1i = exp(-p_boc1 * Deltap_i), exp_p2i = exp(-p_boc2 * Deltap_i);
      const double exp_p1j = exp(-p_boc1 * Deltap_j), exp_p2j = exp(-p_boc2 * Deltap_j);
      const double f2 = exp_p1i + exp_p1j;
      const double f3 = -1.0 / p_boc2 * log(0.5 * (exp_p2i + exp_p2j));
      f1 = 0.5 * ((val_i + f2) / (val_i + f2 + f3) + (val_j + f2) / (val_j + f2 + f3));
      const double temp = f2 + f3;
      const double u1_ij = val_i + temp, u1_ji = val_j + temp;
      const double Cf1A_ij = 0.5 * f3 * (1.0 / sqr(u1_ij) + 1.0 / sqr(u1_ji));
      const double Cf1B_ij = -0.5 * ((u1_ij - f3) / sqr(u1_ij) + (u1_ji - f3) / sqr(u1_ji));
      const double ep = exp_p2i / (exp_p2i + exp_p2j);
      Cf1_ij = 0.50 * (-p_boc1 * exp_p1i / u1_ij - ((val_i + f2) / sqr(u1_ij)) * (-p_boc1 * exp_p1i + ep) +
                       -p_boc1 * exp_p1i / u1_ji - ((val_j + f2) / sqr(u1_ji)) * (-p_boc1 * exp_p1i + ep));
      Cf1_ji = -Cf1A_ij * p_boc1 * exp_p1j + Cf1B_ij * exp_p2j / (exp_p2i + exp_p2j);
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
    const double A2_ij = Cf1_ij / f1 + tw.p_boc3 * Cf45_ij;
    const double A2_ji = Cf1_ji / f1 + tw.p_boc3 * Cf45_ji;
    const double A3_ij = A2_ij + Cf1_ij / f1;
    const double A3_ji = A2_ji + Cf1_ji / f1;
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
  double e_lph = 0, e_lp = 0, e_ov = 0, e_un = 0, ebond = 0, estriph = 0;
  double pol = 0, pol_w = 0;
  if (i < n) {
    const ForceField &F = *d.ff;
    const double p_lp3 = F.gp[5], p_ovun3 = F.gp[32], p_ovun4 = F.gp[31];
    const double p_ovun6 = F.gp[6], p_ovun7 = F.gp[8], p_ovun8 = F.gp[9];
    const double gp3 = F.gp[3], gp4 = F.gp[4], gp7 = F.gp[7], gp10 = F.gp[10];
    const int gp37 = (int)F.gp[37];
    double *CdD = d.fC + 3 * (long long)n;
    const int ti = d.ts[i];
    const Sbp &si = F.sbp[ti];
    const int nb = min(d.nbonds[i], d.bond_cap);
    // polarisation (Compute_Polarization_Energy inlined at :93-104); the
    // reference's pvector value is the running sum, = sum_k pol_k*(n-k) over
    // the original atom order
    const double q = d.xs[i].w;
    pol = KCALpMOL_to_EV * (si.chi * q + (si.eta / 2.) * sqr(q));
    pol_w = pol * (double)(n - d.perm[i]);
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
        const double vov3 = d.b_BO[s] - Di - 0.040 * pow(Di, 4.);
        if (vov3 > 3.) {
          e_lph += p_lp3 * sqr(vov3 - 3.0);
          d.b_Cdbo[s] += 2. * p_lp3 * (vov3 - 3.);
          cd_i += 2. * p_lp3 * (vov3 - 3.) * (-1. - 0.16 * pow(Di, 3.));
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
      const double BOpi = d.b_BOpi[s], BOpi2 = d.b_BOpi2[s], BO = d.b_BO[s];
      double cdbo = CEover1 * tw.p_ovun1 * tw.De_s;
      const double ftmp2 = (1.0 - dfvl * d.dDelta_lp[j]) * (BOpi + BOpi2);
      const double dj = d.Delta[j] - dfvl * d.Delta_lp_temp[j];
      double cdj = CEover4 * ftmp2 + CEunder4 * ftmp2;
      double cdpi = CEover4 * dj + CEunder4 * dj;
      double cdpi2 = cdpi;
      if (tag_first(d, i, j, e)) {
        const Sbp &sj = F.sbp[tj];
        const double BOs = d.b_BOs[s];
        const double pow_BOs_be2 = (BOs == 0.0) ? 0.0 : pow(BOs, tw.p_be2);
        const double exp_be12 = exp(tw.p_be1 * (1.0 - pow_BOs_be2));
        const double CEbo = -tw.De_s * exp_be12 * (1.0 - tw.p_be1 * tw.p_be2 * pow_BOs_be2);
        ebond += -tw.De_s * BOs * exp_be12 - tw.De_p * BOpi - tw.De_pp * BOpi2;
        cdbo += CEbo;
        cdpi -= (CEbo + tw.De_p);
        cdpi2 -= (CEbo + tw.De_pp);
        if (BO >= 1.00 && (gp37 == 2 || (si.mass == 12.0000 && sj.mass == 15.9990) ||
                           (sj.mass == 12.0000 && si.mass == 15.9990))) {
          const double exphu = exp(-gp7 * sqr(BO - 2.50));
          const double exphua1 = exp(-gp3 * (d.bo0[i] - BO));
          const double exphub1 = exp(-gp3 * (d.bo0[j] - BO));
          const double exphuov = exp(gp4 * (d.Delta[i] + d.Delta[j]));
          const double hulpov = 1.0 / (1.0 + 25.0 * exphuov);
          estriph += gp10 * exphu * hulpov * (exphua1 + exphub1);
          cdbo += gp10 * exphu * hulpov * (exphua1 + exphub1) * (gp3 - 2.0 * gp7 * (BO - 2.50));
          cd_i += -gp10 * exphu * hulpov * (gp3 * exphua1 + 25.0 * gp4 * exphuov * hulpov * (exphua1 + exphub1));
          cdj += -gp10 * exphu * hulpov * (gp3 * exphub1 + 25.0 * gp4 * exphuov * hulpov * (exphua1 + exphub1));
        }
      }
      d.b_Cdbo[s] += cdbo;
      d.b_Cdbopi[s] += cdpi;
      d.b_Cdbopi2[s] += cdpi2;
      if (cdj != 0.0) atomicAdd(&CdD[j], cdj);
    }
    atomicAdd(&CdD[i], cd_i);
  }
  if (eflag) {
    block_add(ebond + estriph, &d.energy[E_BOND]);
    block_add(e_ov + e_un, &d.energy[E_OVUN]);
    block_add(e_lp + e_lph, &d.energy[E_LP]);
    block_add(e_lph + e_lp + e_ov + ebond + estriph + e_un, &d.energy[E_ENG_VDWL]);
    block_add(pol, &d.energy[E_ENG_COUL]);
    block_add(pol, &d.energy[E_POL_PHYS]);
    block_add(pol_w, &d.energy[E_POL]);
  }
}

// ------------------------------------------------------------------
// hydrogen bonds: one warp per H atom j; for each bonded acceptor i
// (p_hbond 2, BO >= 0.01) the lanes take the H-bond partners k

__device__ __forceinline__ double warp_sum_d(double v) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(FULL, v, off);
  return v;
}

__global__ void __launch_bounds__(256) k_hbonds(Dev d, int eflag) {
  const int lane = threadIdx.x & 31;
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int n = d.n;
  double ehb = 0.0;
  if (j < n && d.ff->sbp[d.ts[j]].p_hbond == 1) {
    const ForceField &F = *d.ff;
    const int tj = d.ts[j];
    const int nb = min(d.nbonds[j], d.bond_cap);
    const int nh = min(d.nhb[j], d.hb_cap);
    const double4 xj = d.xs[j];
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
      const int tag_i = d.tags[i];
      double fix = 0, fiy = 0, fiz = 0, cdbo = 0;
      for (int pk = lane; pk < nh; pk += 32) {
        const uint32_t ek = d.hb_nbr[(long long)j * d.hb_cap + pk];
        const int k = nbr_of(ek), tk = d.ts[k];
        if (d.tags[k] == tag_i) continue;
        const Hbp &hbp = F.hbp[ti][tj][tk];
        if (hbp.r0_hb <= 0.0) continue;
        int sx, sy, sz;
        img_unpack((int)(ek & 255u), &sx, &sy, &sz);
        const double4 xk = d.xs[k];
        double djk[3];
        djk[0] = __dsub_rn(__dadd_rn(xk.x, sx * d.L[0]), xj.x);
        djk[1] = __dsub_rn(__dadd_rn(xk.y, sy * d.L[1]), xj.y);
        djk[2] = __dsub_rn(__dadd_rn(xk.z, sz * d.L[2]), xj.z);
        const double r_jk = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(djk[0], djk[0]),
                                                           __dmul_rn(djk[1], djk[1])),
                                                 __dmul_rn(djk[2], djk[2])));
        double theta, cos_theta, di[3], djv[3], dk[3];
        theta_dcos(dij, r_ij, djk, r_jk, theta, cos_theta, di, djv, dk);
        const double sin_theta2 = sin(theta / 2.0);
        double sin_xhz4 = sqr(sin_theta2);
        sin_xhz4 *= sin_xhz4;
        const double cos_xhz1 = 1.0 - cos_theta;
        const double exp_hb2 = exp(-hbp.p_hb2 * BO);
        const double exp_hb3 = exp(-hbp.p_hb3 * (hbp.r0_hb / r_jk + r_jk / hbp.r0_hb - 2.0));
        const double e_hb = hbp.p_hb1 * (1.0 - exp_hb2) * exp_hb3 * sin_xhz4;
        ehb += e_hb;
        const double CEhb1 = hbp.p_hb1 * hbp.p_hb2 * exp_hb2 * exp_hb3 * sin_xhz4;
        const double CEhb2 = -hbp.p_hb1 / 2.0 * (1.0 - exp_hb2) * exp_hb3 * cos_xhz1;
        const double CEhb3 = -hbp.p_hb3 * (-hbp.r0_hb / sqr(r_jk) + 1.0 / hbp.r0_hb) * e_hb;
        cdbo += CEhb1;
        fix += CEhb2 * di[0]; fiy += CEhb2 * di[1]; fiz += CEhb2 * di[2];
        const double c3 = CEhb3 / r_jk;
        fjx += CEhb2 * djv[0] - c3 * djk[0];
        fjy += CEhb2 * djv[1] - c3 * djk[1];
        fjz += CEhb2 * djv[2] - c3 * djk[2];
        add3(fC, n, k, 1.0, CEhb2 * dk[0] + c3 * djk[0], CEhb2 * dk[1] + c3 * djk[1],
             CEhb2 * dk[2] + c3 * djk[2]);
      }
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
    block_add(ehb, &d.energy[E_HB]);
    block_add(ehb, &d.energy[E_ENG_VDWL]);
  }
}

// ------------------------------------------------------------------
// Calculate_Omega, reaxc_torsion_angles_sw64.c:21-102
struct Thb {
  double theta, di[3], dj[3], dk[3];
};

__device__ double calc_omega(const double *dvec_ij, double r_ij, const double *dvec_jk, double r_jk,
                             const double *dvec_kl, double r_kl, const double *dvec_li, double r_li,
                             const Thb &p_ijk, const Thb &p_jkl, double *doi, double *doj,
                             double *dok, double *dol) {
  double sin_ijk, cos_ijk, sin_jkl, cos_jkl;
  sincos(p_ijk.theta, &sin_ijk, &cos_ijk);
  sincos(p_jkl.theta, &sin_jkl, &cos_jkl);
  const double dij_jk = dvec_ij[0] * dvec_jk[0] + dvec_ij[1] * dvec_jk[1] + dvec_ij[2] * dvec_jk[2];
  const double djk_kl = dvec_jk[0] * dvec_kl[0] + dvec_jk[1] * dvec_kl[1] + dvec_jk[2] * dvec_kl[2];
  const double dij_kl = dvec_ij[0] * dvec_kl[0] + dvec_ij[1] * dvec_kl[1] + dvec_ij[2] * dvec_kl[2];
  const double unnorm_cos_omega = -dij_jk * djk_kl + sqr(r_jk) * dij_kl;
  const double cr0 = dvec_jk[1] * dvec_kl[2] - dvec_jk[2] * dvec_kl[1];
  const double cr1 = dvec_jk[2] * dvec_kl[0] - dvec_jk[0] * dvec_kl[2];
  const double cr2 = dvec_jk[0] * dvec_kl[1] - dvec_jk[1] * dvec_kl[0];
  const double unnorm_sin_omega = -r_jk * (dvec_ij[0] * cr0 + dvec_ij[1] * cr1 + dvec_ij[2] * cr2);
  const double omega = atan2(unnorm_sin_omega, unnorm_cos_omega);
  const double htra = r_ij + cos_ijk * (r_kl * cos_jkl - r_jk);
  const double htrb = r_jk - r_ij * cos_ijk - r_kl * cos_jkl;
  const double htrc = r_kl + cos_jkl * (r_ij * cos_ijk - r_jk);
  const double hthd = r_ij * sin_ijk * (r_jk - r_kl * cos_jkl);
  const double hthe = r_kl * sin_jkl * (r_jk - r_ij * cos_ijk);
  const double hnra = r_kl * sin_ijk * sin_jkl;
  const double hnrc = r_ij * sin_ijk * sin_jkl;
  const double hnhd = r_ij * r_kl * cos_ijk * sin_jkl;
  const double hnhe = r_ij * r_kl * sin_ijk * cos_jkl;
  double poem = 2.0 * r_ij * r_kl * sin_ijk * sin_jkl;
  if (poem < 1e-20) poem = 1e-20;
  const double tel = sqr(r_ij) + sqr(r_jk) + sqr(r_kl) - sqr(r_li) -
                     2.0 * (r_ij * r_jk * cos_ijk - r_ij * r_kl * cos_ijk * cos_jkl + r_jk * r_kl * cos_jkl);
  double arg = tel / poem;
  if (arg > 1.0) arg = 1.0;
  if (arg < -1.0) arg = -1.0;
  if (sin_ijk >= 0 && sin_ijk <= MIN_SINE) sin_ijk = MIN_SINE;
  else if (sin_ijk <= 0 && sin_ijk >= -MIN_SINE) sin_ijk = -MIN_SINE;
  if (sin_jkl >= 0 && sin_jkl <= MIN_SINE) sin_jkl = MIN_SINE;
  else if (sin_jkl <= 0 && sin_jkl >= -MIN_SINE) sin_jkl = -MIN_SINE;
  const double p2 = 2.0 / poem;
  const double a1 = (htra - arg * hnra) / r_ij, a2 = (hthd - arg * hnhd) / sin_ijk;
  const double a3 = (hthe - arg * hnhe) / sin_jkl, a4 = (htrc - arg * hnrc) / r_kl;
  const double a5 = htrb / r_jk;
#pragma unroll
  for (int t = 0; t < 3; ++t) {
    doi[t] = p2 * (a1 * dvec_ij[t] - dvec_li[t] - a2 * p_ijk.dk[t]);
    doj[t] = p2 * (-a1 * dvec_ij[t] - a5 * dvec_jk[t] - a2 * p_ijk.dj[t] - a3 * p_jkl.di[t]);
    dok[t] = p2 * (-a4 * dvec_kl[t] + a5 * dvec_jk[t] - a2 * p_ijk.di[t] - a3 * p_jkl.dj[t]);
    dol[t] = p2 * (a4 * dvec_kl[t] + dvec_li[t] - a3 * p_jkl.dk[t]);
  }
  return omega;
}

// ------------------------------------------------------------------
// valence + penalty + coalition + torsion + conjugation:
// one thread per (centre j, bond pk of j)

__global__ void __launch_bounds__(128) k_valence_torsion(Dev d, int eflag) {
  const int n = d.n;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int j = (int)(t % n), kk = (int)(t / n);
  double e_ang = 0, e_pen = 0, e_coa = 0, e_tor = 0, e_con = 0;
  const bool active = (kk < d.bond_cap) && (j < n) && (kk < min(d.nbonds[j], d.bond_cap));
  if (active) {
    const ForceField &F = *d.ff;
    const Control &C = *d.ctl;
    const double p_tor2 = F.gp[23], p_tor3 = F.gp[24], p_tor4 = F.gp[25];
    const double p_cot2 = F.gp[27], p_val6 = F.gp[14], p_val8 = F.gp[33];
    const double p_val9 = F.gp[16], p_val10 = F.gp[17];
    const double p_pen2 = F.gp[19], p_pen3 = F.gp[20], p_pen4 = F.gp[21];
    const double p_coa2 = F.gp[2], p_coa3 = F.gp[38], p_coa4 = F.gp[30];
    const double thb_cut = C.thb_cut, thb_cutsq = C.thb_cutsq;
    double *fC = d.fC;
    double *CdD = d.fC + 3 * (long long)n;
    const int nbj = min(d.nbonds[j], d.bond_cap);
    const int tj = d.ts[j];
    const long long spk = (long long)kk * n + j;
    const double BO_jk = d.b_BO[spk];
    const double BOA_jk = BO_jk - thb_cut;
    if (BOA_jk > 0.0 && d.b_sym[spk] >= 0) {
      const uint32_t ejk = d.b_nbr[spk];
      const int k = nbr_of(ejk), tk = d.ts[k];
      const int nbk = min(d.nbonds[k], d.bond_cap);
      const long long spj = d.b_sym[spk];  // j on k's list
      // per-centre quantities (SBO etc.), recomputed per thread
      const double Delta_j = d.Delta_boc[j];
      const double p_val3 = F.sbp[tj].p_val3, p_val5 = F.sbp[tj].p_val5;
      double SBOp = 0, prod_SBO = 1;
      for (int q = 0; q < nbj; ++q) {
        const long long sq = (long long)q * n + j;
        SBOp += d.b_BOpi[sq] + d.b_BOpi2[sq];
        double tmp = sqr(d.b_BO[sq]);
        tmp *= tmp;
        tmp *= tmp;
        prod_SBO *= exp(-tmp);
      }
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
        SBO2 = pow(SBO, p_val9);
        CSBO2 = p_val9 * pow(SBO, p_val9 - 1);
      } else if (SBO > 1 && SBO < 2) {
        SBO2 = 2 - pow(2 - SBO, p_val9);
        CSBO2 = p_val9 * pow(2 - SBO, p_val9 - 1);
      } else SBO2 = 2, CSBO2 = 0;
      const double expval6 = exp(p_val6 * Delta_j);
      const double Delta_k = d.Delta_boc[k];
      const double r_jk = d.b_d[spk];
      const double djk[3] = {d.b_dx[spk], d.b_dy[spk], d.b_dz[spk]};
      const double exp_tor2_jk = exp(-p_tor2 * BOA_jk);
      const double exp_cot2_jk = exp(-p_cot2 * sqr(BOA_jk - 1.5));
      const double exp_tor3_DjDk = exp(-p_tor3 * (Delta_j + Delta_k));
      const double exp_tor4_DjDk = exp(p_tor4 * (Delta_j + Delta_k));
      const double exp_tor34_inv = 1.0 / (1.0 + exp_tor3_DjDk + exp_tor4_DjDk);
      const double f11_DjDk = (2.0 + exp_tor3_DjDk) * exp_tor34_inv;
      const bool do_tor = tag_first(d, j, k, ejk);
      const double BOpi_jk = d.b_BOpi[spk];
      int sjk[3];
      img_unpack((int)(ejk & 255u), &sjk[0], &sjk[1], &sjk[2]);
      const double dpj[3] = {d.b_dx[spj], d.b_dy[spj], d.b_dz[spj]};
      const double r_pj = d.b_d[spj];
      for (int ph = 0; ph < nbj; ++ph) {
        if (ph == kk) continue;
        const long long sph = (long long)ph * n + j;
        const double BO_hj = d.b_BO[sph];
        const double BOA_hj = BO_hj - thb_cut;
        const uint32_t ehj = d.b_nbr[sph];
        const int h = nbr_of(ehj), th = d.ts[h];
        const double dhj[3] = {d.b_dx[sph], d.b_dy[sph], d.b_dz[sph]};
        const double r_hj = d.b_d[sph];
        Thb p_hjk;
        double cos_theta_hjk;
        theta_dcos(djk, r_jk, dhj, r_hj, p_hjk.theta, cos_theta_hjk, p_hjk.di, p_hjk.dj, p_hjk.dk);
        const double theta_hjk = p_hjk.theta;
        double sin_theta_hjk = sin(theta_hjk);
        if (sin_theta_hjk < 1.0e-5) sin_theta_hjk = 1.0e-5;
        // valence angle h-j-k, each unordered bond pair once
        if (ph > kk && BO_jk > thb_cut && BO_hj > thb_cut && BO_jk * BO_hj > thb_cutsq) {
          const Thbh &thbh = F.thbp[tk][tj][th];
          for (int cnt = 0; cnt < thbh.cnt; ++cnt) {
            const Thbp &tp = thbh.prm[cnt];
            if (!(fabs(tp.p_val1) > 0.001)) continue;
            const double p_val1 = tp.p_val1, p_val2 = tp.p_val2, p_val4 = tp.p_val4, p_val7 = tp.p_val7;
            const double theta_00 = tp.theta_00;
            const double exp3jk = exp(-p_val3 * pow(BOA_jk, p_val4));
            const double f7_jk = 1.0 - exp3jk;
            const double Cf7jk = p_val3 * p_val4 * pow(BOA_jk, p_val4 - 1.0) * exp3jk;
            const double exp3hj = exp(-p_val3 * pow(BOA_hj, p_val4));
            const double f7_hj = 1.0 - exp3hj;
            const double Cf7hj = p_val3 * p_val4 * pow(BOA_hj, p_val4 - 1.0) * exp3hj;
            const double expval7 = exp(-p_val7 * Delta_j);
            const double trm8 = 1.0 + expval6 + expval7;
            const double f8_Dj = p_val5 - ((p_val5 - 1.0) * (2.0 + expval6) / trm8);
            const double Cf8j = ((1.0 - p_val5) / sqr(trm8)) *
                                (p_val6 * expval6 * trm8 - (2.0 + expval6) * (p_val6 * expval6 - p_val7 * expval7));
            double theta_0 = 180.0 - theta_00 * (1.0 - exp(-p_val10 * (2.0 - SBO2)));
            theta_0 = deg2rad(theta_0);
            const double expval2theta = exp(-p_val2 * sqr(theta_0 - theta_hjk));
            const double expval12theta = (p_val1 >= 0) ? p_val1 * (1.0 - expval2theta) : p_val1 * -expval2theta;
            const double CEval1 = Cf7jk * f7_hj * f8_Dj * expval12theta;
            const double CEval2 = Cf7hj * f7_jk * f8_Dj * expval12theta;
            const double CEval3 = Cf8j * f7_hj * f7_jk * expval12theta;
            const double CEval4 = -2.0 * p_val1 * p_val2 * f7_jk * f7_hj * f8_Dj * expval2theta * (theta_0 - theta_hjk);
            const double Ctheta_0 = p_val10 * deg2rad(theta_00) * exp(-p_val10 * (2.0 - SBO2));
            const double CEval5 = -CEval4 * Ctheta_0 * CSBO2;
            const double CEval6 = CEval5 * dSBO1;
            const double CEval7 = CEval5 * dSBO2;
            const double CEval8 = -CEval4 / sin_theta_hjk;
            e_ang += f7_jk * f7_hj * f8_Dj * expval12theta;
            const double p_pen1 = tp.p_pen1;
            const double exp_pen2jk = exp(-p_pen2 * sqr(BOA_jk - 2.0));
            const double exp_pen2hj = exp(-p_pen2 * sqr(BOA_hj - 2.0));
            const double exp_pen3 = exp(-p_pen3 * d.Delta[j]);
            const double exp_pen4 = exp(p_pen4 * d.Delta[j]);
            const double trm_pen34 = 1.0 + exp_pen3 + exp_pen4;
            const double f9_Dj = (2.0 + exp_pen3) / trm_pen34;
            const double Cf9j = (-p_pen3 * exp_pen3 * trm_pen34 -
                                 (2.0 + exp_pen3) * (-p_pen3 * exp_pen3 + p_pen4 * exp_pen4)) / sqr(trm_pen34);
            const double epen = p_pen1 * f9_Dj * exp_pen2jk * exp_pen2hj;
            e_pen += epen;
            const double CEpen1 = epen * Cf9j / f9_Dj;
            const double temp = -2.0 * p_pen2 * epen;
            const double CEpen2 = temp * (BOA_jk - 2.0);
            const double CEpen3 = temp * (BOA_hj - 2.0);
            const double p_coa1 = tp.p_coa1;
            const double exp_coa2 = exp(p_coa2 * d.Delta_val[j]);
            const double bo0k = d.bo0[k], bo0h = d.bo0[h];
            const double ecoa = p_coa1 / (1. + exp_coa2) * exp(-p_coa3 * sqr(bo0k - BOA_jk)) *
                                exp(-p_coa3 * sqr(bo0h - BOA_hj)) * exp(-p_coa4 * sqr(BOA_jk - 1.5)) *
                                exp(-p_coa4 * sqr(BOA_hj - 1.5));
            e_coa += ecoa;
            const double CEcoa1 = -2 * p_coa4 * (BOA_jk - 1.5) * ecoa;
            const double CEcoa2 = -2 * p_coa4 * (BOA_hj - 1.5) * ecoa;
            const double CEcoa3 = -p_coa2 * exp_coa2 * ecoa / (1 + exp_coa2);
            const double CEcoa4 = -2 * p_coa3 * (bo0k - BOA_jk) * ecoa;
            const double CEcoa5 = -2 * p_coa3 * (bo0h - BOA_hj) * ecoa;
            atomicAdd(&d.b_Cdbo[spk], CEval1 + CEpen2 + (CEcoa1 - CEcoa4));
            atomicAdd(&d.b_Cdbo[sph], CEval2 + CEpen3 + (CEcoa2 - CEcoa5));
            atomicAdd(&CdD[j], (CEval3 + CEval7) + CEpen1 + CEcoa3);
            atomicAdd(&CdD[k], CEcoa4);
            atomicAdd(&CdD[h], CEcoa5);
            for (int q = 0; q < nbj; ++q) {
              const long long sq = (long long)q * n + j;
              const double b = d.b_BO[sq];
              const double b3 = b * b * b;
              atomicAdd(&d.b_Cdbo[sq], CEval6 * (b3 * b3 * b));
              atomicAdd(&d.b_Cdbopi[sq], CEval5);
              atomicAdd(&d.b_Cdbopi2[sq], CEval5);
            }
            add3(fC, n, k, CEval8, p_hjk.di[0], p_hjk.di[1], p_hjk.di[2]);
            add3(fC, n, j, CEval8, p_hjk.dj[0], p_hjk.dj[1], p_hjk.dj[2]);
            add3(fC, n, h, CEval8, p_hjk.dk[0], p_hjk.dk[1], p_hjk.dk[2]);
          }
        }
        // torsion h-j-k-l about the central bond j-k (counted at one end)
        if (!do_tor) continue;
        if (!(BO_hj > thb_cut) || nbk <= 0) continue;
        const int i = h, ti = th;
        const double r_ij = r_hj;
        const double BOA_ij = BOA_hj;
        const double theta_ijk = theta_hjk;
        double sin_ijk, cos_ijk, tan_ijk_i;
        sincos(theta_ijk, &sin_ijk, &cos_ijk);
        if (sin_ijk >= 0 && sin_ijk <= MIN_SINE) tan_ijk_i = cos_ijk / MIN_SINE;
        else if (sin_ijk <= 0 && sin_ijk >= -MIN_SINE) tan_ijk_i = cos_ijk / -MIN_SINE;
        else tan_ijk_i = cos_ijk / sin_ijk;
        const double exp_tor2_ij = exp(-p_tor2 * BOA_ij);
        const double exp_cot2_ij = exp(-p_cot2 * sqr(BOA_ij - 1.5));
        int shj[3];
        img_unpack((int)(ehj & 255u), &shj[0], &shj[1], &shj[2]);
        for (int pw = 0; pw < nbk; ++pw) {
          const long long spw = (long long)pw * n + k;
          if (spw == spj) continue;
          const double BO_kl = d.b_BO[spw];
          const uint32_t ekl = d.b_nbr[spw];
          const int l = nbr_of(ekl), tl = d.ts[l];
          // i and l are the same atom instance when owners and images agree
          int skl[3];
          img_unpack((int)(ekl & 255u), &skl[0], &skl[1], &skl[2]);
          const bool same = (l == i) && (sjk[0] + skl[0] == shj[0]) && (sjk[1] + skl[1] == shj[1]) &&
                            (sjk[2] + skl[2] == shj[2]);
          const Fbh &fbh = F.fbp[ti][tj][tk][tl];
          if (same || !fbh.cnt || !(BO_kl > thb_cut) || !(BO_hj * BO_jk * BO_kl > thb_cut)) continue;
          const Fbp &fbp = fbh.prm;
          const double dkl[3] = {d.b_dx[spw], d.b_dy[spw], d.b_dz[spw]};
          const double r_kl = d.b_d[spw];
          Thb p_jkl;
          double cos_theta_jkl;
          theta_dcos(dpj, r_pj, dkl, r_kl, p_jkl.theta, cos_theta_jkl, p_jkl.di, p_jkl.dj, p_jkl.dk);
          const double BOA_kl = BO_kl - thb_cut;
          double sin_jkl, cos_jkl, tan_jkl_i;
          sincos(p_jkl.theta, &sin_jkl, &cos_jkl);
          if (sin_jkl >= 0 && sin_jkl <= MIN_SINE) tan_jkl_i = cos_jkl / MIN_SINE;
          else if (sin_jkl <= 0 && sin_jkl >= -MIN_SINE) tan_jkl_i = cos_jkl / -MIN_SINE;
          else tan_jkl_i = cos_jkl / sin_jkl;
          double dli[3];
          dli[0] = dhj[0] - djk[0] - dkl[0];
          dli[1] = dhj[1] - djk[1] - dkl[1];
          dli[2] = dhj[2] - djk[2] - dkl[2];
          const double r_li = sqrt(sqr(dli[0]) + sqr(dli[1]) + sqr(dli[2]));
          double doi[3], doj[3], dok[3], dol[3];
          const double omega = calc_omega(dhj, r_ij, djk, r_jk, dkl, r_kl, dli, r_li, p_hjk, p_jkl,
                                          doi, doj, dok, dol);
          const double cos_omega = cos(omega);
          const double cos2omega = cos(2. * omega);
          const double cos3omega = cos(3. * omega);
          const double exp_tor1 = exp(fbp.p_tor1 * sqr(2.0 - BOpi_jk - f11_DjDk));
          const double exp_tor2_kl = exp(-p_tor2 * BOA_kl);
          const double exp_cot2_kl = exp(-p_cot2 * sqr(BOA_kl - 1.5));
          const double fn10 = (1.0 - exp_tor2_ij) * (1.0 - exp_tor2_jk) * (1.0 - exp_tor2_kl);
          const double CV = 0.5 * (fbp.V1 * (1.0 + cos_omega) + fbp.V2 * exp_tor1 * (1.0 - cos2omega) +
                                   fbp.V3 * (1.0 + cos3omega));
          e_tor += fn10 * sin_ijk * sin_jkl * CV;
          const double dfn11 = (-p_tor3 * exp_tor3_DjDk +
                                (p_tor3 * exp_tor3_DjDk - p_tor4 * exp_tor4_DjDk) * (2.0 + exp_tor3_DjDk) * exp_tor34_inv) *
                               exp_tor34_inv;
          const double CEtors1 = sin_ijk * sin_jkl * CV;
          const double CEtors2 = -fn10 * 2.0 * fbp.p_tor1 * fbp.V2 * exp_tor1 * (2.0 - BOpi_jk - f11_DjDk) *
                                 (1.0 - sqr(cos_omega)) * sin_ijk * sin_jkl;
          const double CEtors3 = CEtors2 * dfn11;
          const double CEtors4 = CEtors1 * p_tor2 * exp_tor2_ij * (1.0 - exp_tor2_jk) * (1.0 - exp_tor2_kl);
          const double CEtors5 = CEtors1 * p_tor2 * (1.0 - exp_tor2_ij) * exp_tor2_jk * (1.0 - exp_tor2_kl);
          const double CEtors6 = CEtors1 * p_tor2 * (1.0 - exp_tor2_ij) * (1.0 - exp_tor2_jk) * exp_tor2_kl;
          const double cmn = -fn10 * CV;
          const double CEtors7 = cmn * sin_jkl * tan_ijk_i;
          const double CEtors8 = cmn * sin_ijk * tan_jkl_i;
          const double CEtors9 = fn10 * sin_ijk * sin_jkl *
                                 (0.5 * fbp.V1 - 2.0 * fbp.V2 * exp_tor1 * cos_omega +
                                  1.5 * fbp.V3 * (cos2omega + 2.0 * sqr(cos_omega)));
          const double fn12 = exp_cot2_ij * exp_cot2_jk * exp_cot2_kl;
          const double econ = fbp.p_cot1 * fn12 * (1.0 + (sqr(cos_omega) - 1.0) * sin_ijk * sin_jkl);
          e_con += econ;
          const double Cconj = -2.0 * fn12 * fbp.p_cot1 * p_cot2 * (1.0 + (sqr(cos_omega) - 1.0) * sin_ijk * sin_jkl);
          const double CEconj1 = Cconj * (BOA_ij - 1.5e0);
          const double CEconj2 = Cconj * (BOA_jk - 1.5e0);
          const double CEconj3 = Cconj * (BOA_kl - 1.5e0);
          const double CEconj4 = -fbp.p_cot1 * fn12 * (sqr(cos_omega) - 1.0) * sin_jkl * tan_ijk_i;
          const double CEconj5 = -fbp.p_cot1 * fn12 * (sqr(cos_omega) - 1.0) * sin_ijk * tan_jkl_i;
          const double CEconj6 = 2.0 * fbp.p_cot1 * fn12 * cos_omega * sin_ijk * sin_jkl;
          atomicAdd(&d.b_Cdbopi[spk], CEtors2);
          atomicAdd(&CdD[j], CEtors3);
          atomicAdd(&CdD[k], CEtors3);
          atomicAdd(&d.b_Cdbo[sph], CEtors4 + CEconj1);
          atomicAdd(&d.b_Cdbo[spk], CEtors5 + CEconj2);
          atomicAdd(&d.b_Cdbo[spw], CEtors6 + CEconj3);
          const double c78 = CEtors7 + CEconj4, c85 = CEtors8 + CEconj5, c96 = CEtors9 + CEconj6;
          add3(fC, n, i, 1.0, c78 * p_hjk.dk[0] + c96 * doi[0], c78 * p_hjk.dk[1] + c96 * doi[1],
               c78 * p_hjk.dk[2] + c96 * doi[2]);
          add3(fC, n, j, 1.0, c78 * p_hjk.dj[0] + c85 * p_jkl.di[0] + c96 * doj[0],
               c78 * p_hjk.dj[1] + c85 * p_jkl.di[1] + c96 * doj[1],
               c78 * p_hjk.dj[2] + c85 * p_jkl.di[2] + c96 * doj[2]);
          add3(fC, n, k, 1.0, c78 * p_hjk.di[0] + c85 * p_jkl.dj[0] + c96 * dok[0],
               c78 * p_hjk.di[1] + c85 * p_jkl.dj[1] + c96 * dok[1],
               c78 * p_hjk.di[2] + c85 * p_jkl.dj[2] + c96 * dok[2]);
          add3(fC, n, l, 1.0, c85 * p_jkl.dk[0] + c96 * dol[0], c85 * p_jkl.dk[1] + c96 * dol[1],
               c85 * p_jkl.dk[2] + c96 * dol[2]);
        }
      }
    }
  }
  if (eflag) {
    block_add(e_ang, &d.energy[E_ANG]);
    block_add(e_pen, &d.energy[E_PEN]);
    block_add(e_coa, &d.energy[E_COA]);
    block_add(e_tor, &d.energy[E_TOR]);
    block_add(e_con, &d.energy[E_CON]);
    block_add(e_ang + e_pen + e_coa + e_tor + e_con, &d.energy[E_ENG_VDWL]);
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
    SBO2 = pow(SBO, p_val9);
    CSBO2 = p_val9 * pow(SBO, p_val9 - 1);
  } else if (SBO > 1 && SBO < 2) {
    SBO2 = 2 - pow(2 - SBO, p_val9);
    CSBO2 = p_val9 * pow(2 - SBO, p_val9 - 1);
  } else SBO2 = 2, CSBO2 = 0;
  d.c_sbo[j] = SBO2;
  d.c_sbo[n + j] = CSBO2;
  d.c_sbo[2 * n + j] = dSBO1;
  d.c_sbo[3 * n + j] = dSBO2;
  d.c_sbo[4 * n + j] = exp(p_val6 * Delta_j);
}

// per bond slot: exp(-p_tor2 BOA), exp(-p_cot2 (BOA - 1.5)^2)
__global__ void k_vt_prep_bond(Dev d) {
  const int n = d.n;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int i = (int)(t % n), k = (int)(t / n);
  if (k >= d.bond_cap || i >= n || k >= d.nbonds[i]) return;
  const long long s = (long long)k * n + i;
  const double BOA = d.b_BO[s] - d.ctl->thb_cut;
  d.b_et2[s] = exp(-d.ff->gp[23] * BOA);
  d.b_ec2[s] = exp(-d.ff->gp[27] * sqr(BOA - 1.5));
}

__device__ __forceinline__ bool fbp_nonzero(const Fbp &p) {
  return p.V1 != 0.0 || p.V2 != 0.0 || p.V3 != 0.0 || p.p_cot1 != 0.0;
}

// enumerate the items of slot (j, kk); FILL writes them at the offsets
template <bool FILL>
__device__ void vt_enumerate(const Dev &d, int j, int kk, int &cv, int &ct, long long ov,
                             long long ot) {
  const int n = d.n;
  const ForceField &F = *d.ff;
  const double thb_cut = d.ctl->thb_cut, thb_cutsq = d.ctl->thb_cutsq;
  cv = ct = 0;
  const int nbj = min(d.nbonds[j], d.bond_cap);
  if (kk >= nbj) return;
  const long long spk = (long long)kk * n + j;
  const double BO_jk = d.b_BO[spk];
  if (!(BO_jk - thb_cut > 0.0) || d.b_sym[spk] < 0) return;
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
    const double BO_hj = d.b_BO[sph];
    const uint32_t ehj = d.b_nbr[sph];
    const int h = nbr_of(ehj), th = d.ts[h];
    if (ph > kk && BO_jk > thb_cut && BO_hj > thb_cut && BO_jk * BO_hj > thb_cutsq) {
      const Thbh &thbh = F.thbp[tk][tj][th];
      bool any = false;
      for (int c = 0; c < thbh.cnt; ++c) any |= fabs(thbh.prm[c].p_val1) > 0.001;
      if (any) {
        if (FILL)
          d.w_val[ov + cv] = ((unsigned long long)j << 16) | ((unsigned long long)kk << 8) | ph;
        ++cv;
      }
    }
    if (!do_tor || !(BO_hj > thb_cut)) continue;
    int shj[3];
    img_unpack((int)(ehj & 255u), &shj[0], &shj[1], &shj[2]);
    for (int pw = 0; pw < nbk; ++pw) {
      const long long spw = (long long)pw * n + k;
      if (spw == spj) continue;
      const double BO_kl = d.b_BO[spw];
      if (!(BO_kl > thb_cut) || !(BO_hj * BO_jk * BO_kl > thb_cut)) continue;
      const uint32_t ekl = d.b_nbr[spw];
      const int l = nbr_of(ekl);
      const Fbh &fbh = F.fbp[th][tj][tk][d.ts[l]];
      if (!fbh.cnt || !fbp_nonzero(fbh.prm)) continue;
      int skl[3];
      img_unpack((int)(ekl & 255u), &skl[0], &skl[1], &skl[2]);
      if (l == h && sjk[0] + skl[0] == shj[0] && sjk[1] + skl[1] == shj[1] &&
          sjk[2] + skl[2] == shj[2])
        continue;   // i and l are the same atom instance
      if (FILL)
        d.w_tor[ot + ct] = ((unsigned long long)j << 24) | ((unsigned long long)kk << 16) |
                           ((unsigned long long)ph << 8) | pw;
      ++ct;
    }
  }
}

__global__ void k_vt_count(Dev d) {
  const int n = d.n;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long slots = (long long)d.bond_cap * n;
  if (t > slots) return;
  if (t == slots) {   // trailing zero for the exclusive scans
    d.w_cnt_v[t] = 0;
    d.w_cnt_t[t] = 0;
    return;
  }
  int cv, ct;
  vt_enumerate<false>(d, (int)(t % n), (int)(t / n), cv, ct, 0, 0);
  d.w_cnt_v[t] = cv;
  d.w_cnt_t[t] = ct;
}

__global__ void k_vt_fill(Dev d) {
  const int n = d.n;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)d.bond_cap * n) return;
  if (d.w_cnt_v[t] == 0 && d.w_cnt_t[t] == 0) return;
  int cv, ct;
  vt_enumerate<true>(d, (int)(t % n), (int)(t / n), cv, ct, d.w_off_v[t], d.w_off_t[t]);
}

// one valence angle h-j-k (with its penalty and coalition terms)
__global__ void __launch_bounds__(128) k_valence(Dev d, int eflag, long long nitems) {
  const long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double e_ang = 0, e_pen = 0, e_coa = 0;
  if (w < nitems) {
    const unsigned long long it = d.w_val[w];
    const int j = (int)(it >> 16), kk = (int)((it >> 8) & 255), ph = (int)(it & 255);
    const int n = d.n;
    const ForceField &F = *d.ff;
    const double thb_cut = d.ctl->thb_cut;
    const double p_val6 = F.gp[14], p_val10 = F.gp[17];
    const double p_pen2 = F.gp[19], p_pen3 = F.gp[20], p_pen4 = F.gp[21];
    const double p_coa2 = F.gp[2], p_coa3 = F.gp[38], p_coa4 = F.gp[30];
    double *fC = d.fC;
    double *CdD = d.fC + 3 * (long long)n;
    const int tj = d.ts[j];
    const double p_val3 = F.sbp[tj].p_val3, p_val5 = F.sbp[tj].p_val5;
    const double SBO2 = d.c_sbo[j], CSBO2 = d.c_sbo[n + j];
    const double dSBO1 = d.c_sbo[2 * n + j], dSBO2 = d.c_sbo[3 * n + j];
    const double expval6 = d.c_sbo[4 * n + j];
    const double Delta_j = d.Delta_boc[j];
    const long long spk = (long long)kk * n + j, sph = (long long)ph * n + j;
    const int k = nbr_of(d.b_nbr[spk]), h = nbr_of(d.b_nbr[sph]);
    const int tk = d.ts[k], th = d.ts[h];
    const double BOA_jk = d.b_BO[spk] - thb_cut, BOA_hj = d.b_BO[sph] - thb_cut;
    const double djk[3] = {d.b_dx[spk], d.b_dy[spk], d.b_dz[spk]};
    const double dhj[3] = {d.b_dx[sph], d.b_dy[sph], d.b_dz[sph]};
    double theta_hjk, cos_theta_hjk, di[3], dj[3], dk[3];
    theta_dcos(djk, d.b_d[spk], dhj, d.b_d[sph], theta_hjk, cos_theta_hjk, di, dj, dk);
    double sin_theta_hjk = sin(theta_hjk);
    if (sin_theta_hjk < 1.0e-5) sin_theta_hjk = 1.0e-5;
    const Thbh &thbh = F.thbp[tk][tj][th];
    const int nbj = min(d.nbonds[j], d.bond_cap);
    for (int cnt = 0; cnt < thbh.cnt; ++cnt) {
      const Thbp &tp = thbh.prm[cnt];
      if (!(fabs(tp.p_val1) > 0.001)) continue;
      const double p_val1 = tp.p_val1, p_val2 = tp.p_val2, p_val4 = tp.p_val4, p_val7 = tp.p_val7;
      const double theta_00 = tp.theta_00;
      const double exp3jk = exp(-p_val3 * pow(BOA_jk, p_val4));
      const double f7_jk = 1.0 - exp3jk;
      const double Cf7jk = p_val3 * p_val4 * pow(BOA_jk, p_val4 - 1.0) * exp3jk;
      const double exp3hj = exp(-p_val3 * pow(BOA_hj, p_val4));
      const double f7_hj = 1.0 - exp3hj;
      const double Cf7hj = p_val3 * p_val4 * pow(BOA_hj, p_val4 - 1.0) * exp3hj;
      const double expval7 = exp(-p_val7 * Delta_j);
      const double trm8 = 1.0 + expval6 + expval7;
      const double f8_Dj = p_val5 - ((p_val5 - 1.0) * (2.0 + expval6) / trm8);
      const double Cf8j = ((1.0 - p_val5) / sqr(trm8)) *
                          (p_val6 * expval6 * trm8 - (2.0 + expval6) * (p_val6 * expval6 - p_val7 * expval7));
      double theta_0 = 180.0 - theta_00 * (1.0 - exp(-p_val10 * (2.0 - SBO2)));
      theta_0 = deg2rad(theta_0);
      const double expval2theta = exp(-p_val2 * sqr(theta_0 - theta_hjk));
      const double expval12theta = (p_val1 >= 0) ? p_val1 * (1.0 - expval2theta) : p_val1 * -expval2theta;
      const double CEval1 = Cf7jk * f7_hj * f8_Dj * expval12theta;
      const double CEval2 = Cf7hj * f7_jk * f8_Dj * expval12theta;
      const double CEval3 = Cf8j * f7_hj * f7_jk * expval12theta;
      const double CEval4 = -2.0 * p_val1 * p_val2 * f7_jk * f7_hj * f8_Dj * expval2theta * (theta_0 - theta_hjk);
      const double Ctheta_0 = p_val10 * deg2rad(theta_00) * exp(-p_val10 * (2.0 - SBO2));
      const double CEval5 = -CEval4 * Ctheta_0 * CSBO2;
      const double CEval6 = CEval5 * dSBO1;
      const double CEval7 = CEval5 * dSBO2;
      const double CEval8 = -CEval4 / sin_theta_hjk;
      e_ang += f7_jk * f7_hj * f8_Dj * expval12theta;
      const double exp_pen2jk = exp(-p_pen2 * sqr(BOA_jk - 2.0));
      const double exp_pen2hj = exp(-p_pen2 * sqr(BOA_hj - 2.0));
      const double exp_pen3 = exp(-p_pen3 * d.Delta[j]);
      const double exp_pen4 = exp(p_pen4 * d.Delta[j]);
      const double trm_pen34 = 1.0 + exp_pen3 + exp_pen4;
      const double f9_Dj = (2.0 + exp_pen3) / trm_pen34;
      const double Cf9j = (-p_pen3 * exp_pen3 * trm_pen34 -
                           (2.0 + exp_pen3) * (-p_pen3 * exp_pen3 + p_pen4 * exp_pen4)) / sqr(trm_pen34);
      const double epen = tp.p_pen1 * f9_Dj * exp_pen2jk * exp_pen2hj;
      e_pen += epen;
      const double CEpen1 = epen * Cf9j / f9_Dj;
      const double temp = -2.0 * p_pen2 * epen;
      const double CEpen2 = temp * (BOA_jk - 2.0);
      const double CEpen3 = temp * (BOA_hj - 2.0);
      const double exp_coa2 = exp(p_coa2 * d.Delta_val[j]);
      const double bo0k = d.bo0[k], bo0h = d.bo0[h];
      const double ecoa = tp.p_coa1 / (1. + exp_coa2) * exp(-p_coa3 * sqr(bo0k - BOA_jk)) *
                          exp(-p_coa3 * sqr(bo0h - BOA_hj)) * exp(-p_coa4 * sqr(BOA_jk - 1.5)) *
                          exp(-p_coa4 * sqr(BOA_hj - 1.5));
      e_coa += ecoa;
      const double CEcoa1 = -2 * p_coa4 * (BOA_jk - 1.5) * ecoa;
      const double CEcoa2 = -2 * p_coa4 * (BOA_hj - 1.5) * ecoa;
      const double CEcoa3 = -p_coa2 * exp_coa2 * ecoa / (1 + exp_coa2);
      const double CEcoa4 = -2 * p_coa3 * (bo0k - BOA_jk) * ecoa;
      const double CEcoa5 = -2 * p_coa3 * (bo0h - BOA_hj) * ecoa;
      atomicAdd(&d.b_Cdbo[spk], CEval1 + CEpen2 + (CEcoa1 - CEcoa4));
      atomicAdd(&d.b_Cdbo[sph], CEval2 + CEpen3 + (CEcoa2 - CEcoa5));
      atomicAdd(&CdD[j], (CEval3 + CEval7) + CEpen1 + CEcoa3);
      atomicAdd(&CdD[k], CEcoa4);
      atomicAdd(&CdD[h], CEcoa5);
      for (int q = 0; q < nbj; ++q) {
        const long long sq = (long long)q * n + j;
        const double b = d.b_BO[sq];
        const double b3 = b * b * b;
        atomicAdd(&d.b_Cdbo[sq], CEval6 * (b3 * b3 * b));
        atomicAdd(&d.b_Cdbopi[sq], CEval5);
        atomicAdd(&d.b_Cdbopi2[sq], CEval5);
      }
      add3(fC, n, k, CEval8, di[0], di[1], di[2]);
      add3(fC, n, j, CEval8, dj[0], dj[1], dj[2]);
      add3(fC, n, h, CEval8, dk[0], dk[1], dk[2]);
    }
  }
  if (eflag) {
    block_add(e_ang, &d.energy[E_ANG]);
    block_add(e_pen, &d.energy[E_PEN]);
    block_add(e_coa, &d.energy[E_COA]);
    block_add(e_ang + e_pen + e_coa, &d.energy[E_ENG_VDWL]);
  }
}

// one torsion h-j-k-l (with its 4-body conjugation term)
__global__ void __launch_bounds__(128) k_torsion(Dev d, int eflag, long long nitems) {
  const long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double e_tor = 0, e_con = 0;
  if (w < nitems) {
    const unsigned long long it = d.w_tor[w];
    const int j = (int)(it >> 24), kk = (int)((it >> 16) & 255);
    const int ph = (int)((it >> 8) & 255), pw = (int)(it & 255);
    const int n = d.n;
    const ForceField &F = *d.ff;
    const double thb_cut = d.ctl->thb_cut;
    const double p_tor2 = F.gp[23], p_tor3 = F.gp[24], p_tor4 = F.gp[25], p_cot2 = F.gp[27];
    double *fC = d.fC;
    double *CdD = d.fC + 3 * (long long)n;
    const long long spk = (long long)kk * n + j, sph = (long long)ph * n + j;
    const int k = nbr_of(d.b_nbr[spk]), i = nbr_of(d.b_nbr[sph]);
    const long long spj = d.b_sym[spk];
    const long long spw = (long long)pw * n + k;
    const int l = nbr_of(d.b_nbr[spw]);
    const Fbp &fbp = F.fbp[d.ts[i]][d.ts[j]][d.ts[k]][d.ts[l]].prm;
    const double BOA_jk = d.b_BO[spk] - thb_cut, BOA_ij = d.b_BO[sph] - thb_cut;
    const double BOA_kl = d.b_BO[spw] - thb_cut;
    const double Delta_j = d.Delta_boc[j], Delta_k = d.Delta_boc[k];
    const double exp_tor3_DjDk = exp(-p_tor3 * (Delta_j + Delta_k));
    const double exp_tor4_DjDk = exp(p_tor4 * (Delta_j + Delta_k));
    const double exp_tor34_inv = 1.0 / (1.0 + exp_tor3_DjDk + exp_tor4_DjDk);
    const double f11_DjDk = (2.0 + exp_tor3_DjDk) * exp_tor34_inv;
    const double exp_tor2_jk = d.b_et2[spk], exp_cot2_jk = d.b_ec2[spk];
    const double exp_tor2_ij = d.b_et2[sph], exp_cot2_ij = d.b_ec2[sph];
    const double exp_tor2_kl = d.b_et2[spw], exp_cot2_kl = d.b_ec2[spw];
    const double djk[3] = {d.b_dx[spk], d.b_dy[spk], d.b_dz[spk]};
    const double dhj[3] = {d.b_dx[sph], d.b_dy[sph], d.b_dz[sph]};
    const double dkl[3] = {d.b_dx[spw], d.b_dy[spw], d.b_dz[spw]};
    const double dpj[3] = {d.b_dx[spj], d.b_dy[spj], d.b_dz[spj]};
    const double r_jk = d.b_d[spk], r_ij = d.b_d[sph], r_kl = d.b_d[spw];
    Thb p_ijk, p_jkl;
    double cth;
    theta_dcos(djk, r_jk, dhj, r_ij, p_ijk.theta, cth, p_ijk.di, p_ijk.dj, p_ijk.dk);
    theta_dcos(dpj, d.b_d[spj], dkl, r_kl, p_jkl.theta, cth, p_jkl.di, p_jkl.dj, p_jkl.dk);
    double sin_ijk, cos_ijk, tan_ijk_i, sin_jkl, cos_jkl, tan_jkl_i;
    sincos(p_ijk.theta, &sin_ijk, &cos_ijk);
    if (sin_ijk >= 0 && sin_ijk <= MIN_SINE) tan_ijk_i = cos_ijk / MIN_SINE;
    else if (sin_ijk <= 0 && sin_ijk >= -MIN_SINE) tan_ijk_i = cos_ijk / -MIN_SINE;
    else tan_ijk_i = cos_ijk / sin_ijk;
    sincos(p_jkl.theta, &sin_jkl, &cos_jkl);
    if (sin_jkl >= 0 && sin_jkl <= MIN_SINE) tan_jkl_i = cos_jkl / MIN_SINE;
    else if (sin_jkl <= 0 && sin_jkl >= -MIN_SINE) tan_jkl_i = cos_jkl / -MIN_SINE;
    else tan_jkl_i = cos_jkl / sin_jkl;
    double dli[3];
    dli[0] = dhj[0] - djk[0] - dkl[0];
    dli[1] = dhj[1] - djk[1] - dkl[1];
    dli[2] = dhj[2] - djk[2] - dkl[2];
    const double r_li = sqrt(sqr(dli[0]) + sqr(dli[1]) + sqr(dli[2]));
    double doi[3], doj[3], dok[3], dol[3];
    const double omega = calc_omega(dhj, r_ij, djk, r_jk, dkl, r_kl, dli, r_li, p_ijk, p_jkl,
                                    doi, doj, dok, dol);
    const double cos_omega = cos(omega);
    const double cos2omega = cos(2. * omega);
    const double cos3omega = cos(3. * omega);
    const double BOpi_jk = d.b_BOpi[spk];
    const double exp_tor1 = exp(fbp.p_tor1 * sqr(2.0 - BOpi_jk - f11_DjDk));
    const double fn10 = (1.0 - exp_tor2_ij) * (1.0 - exp_tor2_jk) * (1.0 - exp_tor2_kl);
    const double CV = 0.5 * (fbp.V1 * (1.0 + cos_omega) + fbp.V2 * exp_tor1 * (1.0 - cos2omega) +
                             fbp.V3 * (1.0 + cos3omega));
    e_tor = fn10 * sin_ijk * sin_jkl * CV;
    const double dfn11 = (-p_tor3 * exp_tor3_DjDk +
                          (p_tor3 * exp_tor3_DjDk - p_tor4 * exp_tor4_DjDk) * (2.0 + exp_tor3_DjDk) * exp_tor34_inv) *
                         exp_tor34_inv;
    const double CEtors1 = sin_ijk * sin_jkl * CV;
    const double CEtors2 = -fn10 * 2.0 * fbp.p_tor1 * fbp.V2 * exp_tor1 * (2.0 - BOpi_jk - f11_DjDk) *
                           (1.0 - sqr(cos_omega)) * sin_ijk * sin_jkl;
    const double CEtors3 = CEtors2 * dfn11;
    const double CEtors4 = CEtors1 * p_tor2 * exp_tor2_ij * (1.0 - exp_tor2_jk) * (1.0 - exp_tor2_kl);
    const double CEtors5 = CEtors1 * p_tor2 * (1.0 - exp_tor2_ij) * exp_tor2_jk * (1.0 - exp_tor2_kl);
    const double CEtors6 = CEtors1 * p_tor2 * (1.0 - exp_tor2_ij) * (1.0 - exp_tor2_jk) * exp_tor2_kl;
    const double cmn = -fn10 * CV;
    const double CEtors7 = cmn * sin_jkl * tan_ijk_i;
    const double CEtors8 = cmn * sin_ijk * tan_jkl_i;
    const double CEtors9 = fn10 * sin_ijk * sin_jkl *
                           (0.5 * fbp.V1 - 2.0 * fbp.V2 * exp_tor1 * cos_omega +
                            1.5 * fbp.V3 * (cos2omega + 2.0 * sqr(cos_omega)));
    const double fn12 = exp_cot2_ij * exp_cot2_jk * exp_cot2_kl;
    e_con = fbp.p_cot1 * fn12 * (1.0 + (sqr(cos_omega) - 1.0) * sin_ijk * sin_jkl);
    const double Cconj = -2.0 * fn12 * fbp.p_cot1 * p_cot2 * (1.0 + (sqr(cos_omega) - 1.0) * sin_ijk * sin_jkl);
    const double CEconj1 = Cconj * (BOA_ij - 1.5e0);
    const double CEconj2 = Cconj * (BOA_jk - 1.5e0);
    const double CEconj3 = Cconj * (BOA_kl - 1.5e0);
    const double CEconj4 = -fbp.p_cot1 * fn12 * (sqr(cos_omega) - 1.0) * sin_jkl * tan_ijk_i;
    const double CEconj5 = -fbp.p_cot1 * fn12 * (sqr(cos_omega) - 1.0) * sin_ijk * tan_jkl_i;
    const double CEconj6 = 2.0 * fbp.p_cot1 * fn12 * cos_omega * sin_ijk * sin_jkl;
    atomicAdd(&d.b_Cdbopi[spk], CEtors2);
    atomicAdd(&CdD[j], CEtors3);
    atomicAdd(&CdD[k], CEtors3);
    atomicAdd(&d.b_Cdbo[sph], CEtors4 + CEconj1);
    atomicAdd(&d.b_Cdbo[spk], CEtors5 + CEconj2);
    atomicAdd(&d.b_Cdbo[spw], CEtors6 + CEconj3);
    const double c78 = CEtors7 + CEconj4, c85 = CEtors8 + CEconj5, c96 = CEtors9 + CEconj6;
    add3(fC, n, i, 1.0, c78 * p_ijk.dk[0] + c96 * doi[0], c78 * p_ijk.dk[1] + c96 * doi[1],
         c78 * p_ijk.dk[2] + c96 * doi[2]);
    add3(fC, n, j, 1.0, c78 * p_ijk.dj[0] + c85 * p_jkl.di[0] + c96 * doj[0],
         c78 * p_ijk.dj[1] + c85 * p_jkl.di[1] + c96 * doj[1],
         c78 * p_ijk.dj[2] + c85 * p_jkl.di[2] + c96 * doj[2]);
    add3(fC, n, k, 1.0, c78 * p_ijk.di[0] + c85 * p_jkl.dj[0] + c96 * dok[0],
         c78 * p_ijk.di[1] + c85 * p_jkl.dj[1] + c96 * dok[1],
         c78 * p_ijk.di[2] + c85 * p_jkl.dj[2] + c96 * dok[2]);
    add3(fC, n, l, 1.0, c85 * p_jkl.dk[0] + c96 * dol[0], c85 * p_jkl.dk[1] + c96 * dol[1],
         c85 * p_jkl.dk[2] + c96 * dol[2]);
  }
  if (eflag) {
    block_add(e_tor, &d.energy[E_TOR]);
    block_add(e_con, &d.energy[E_CON]);
    block_add(e_tor + e_con, &d.energy[E_ENG_VDWL]);
  }
}

// ------------------------------------------------------------------
// bond-order derivative forces: one thread per atom i over its bonds

__global__ void k_dbond(Dev d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = d.n;
  if (i >= n) return;
  const long long S = (long long)d.bond_cap * n;
  const int nb = min(d.nbonds[i], d.bond_cap);
  const double *CdD = d.fC + 3 * (long long)n;
  const double Ddx = d.dDeltap[i], Ddy = d.dDeltap[n + i], Ddz = d.dDeltap[2 * n + i];
  const double cdi = CdD[i];
  double fx = 0, fy = 0, fz = 0, buf_c = 0;
  for (int k = 0; k < nb; ++k) {
    const long long s = (long long)k * n + i;
    const int j = nbr_of(d.b_nbr[s]);
    const long long sy = d.b_sym[s];
    double cdbo = d.b_Cdbo[s], cdbopi = d.b_Cdbopi[s], cdbopi2 = d.b_Cdbopi2[s];
    if (sy >= 0) {
      cdbo += d.b_Cdbo[sy];
      cdbopi += d.b_Cdbopi[sy];
      cdbopi2 += d.b_Cdbopi2[sy];
    }
    const double C1dbo = d.b_C[0 * S + s], C2dbo = d.b_C[1 * S + s];
    const double C1pi = d.b_C[3 * S + s], C2pi = d.b_C[4 * S + s], C3pi = d.b_C[5 * S + s];
    const double C1pi2 = d.b_C[7 * S + s], C2pi2 = d.b_C[8 * S + s], C3pi2 = d.b_C[9 * S + s];
    const double cdd = cdi + CdD[j];
    const double a = C1dbo * cdbo + C1dbo * cdd + C2pi * cdbopi + C2pi2 * cdbopi2;  // along dBOp
    const double b = C2dbo * cdbo + C2dbo * cdd + C3pi * cdbopi + C3pi2 * cdbopi2;  // along dDeltap_i
    const double cpi = C1pi * cdbopi, cpi2 = C1pi2 * cdbopi2;
    const double gx = d.b_dBOp[s], gy = d.b_dBOp[S + s], gz = d.b_dBOp[2 * S + s];
    fx += a * gx + b * Ddx + cpi * d.b_dlnpi[s] + cpi2 * d.b_dlnpi2[s];
    fy += a * gy + b * Ddy + cpi * d.b_dlnpi[S + s] + cpi2 * d.b_dlnpi2[S + s];
    fz += a * gz + b * Ddz + cpi * d.b_dlnpi[2 * S + s] + cpi2 * d.b_dlnpi2[2 * S + s];
    buf_c -= b;
  }
  double *fC = d.fC;
  atomicAdd(&fC[i], fx);
  atomicAdd(&fC[n + i], fy);
  atomicAdd(&fC[2 * n + i], fz);
  if (buf_c != 0.0)
    for (int k = 0; k < nb; ++k) {
      const long long s = (long long)k * n + i;
      const int j = nbr_of(d.b_nbr[s]);
      add3(fC, n, j, buf_c, d.b_dBOp[s], d.b_dBOp[S + s], d.b_dBOp[2 * S + s]);
    }
}

// forces back to the original atom order: f = -dE/dx
__global__ void k_force_out(Dev d) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= d.n) return;
  const int n = d.n, i = d.perm[s];
  const double fx = -d.fC[s], fy = -d.fC[n + s], fz = -d.fC[2 * n + s];
  if (!(isfinite(fx) && isfinite(fy) && isfinite(fz))) atomicOr(&d.status[ST_NAN], 1);
  d.f_o[3 * i + 0] = fx;
  d.f_o[3 * i + 1] = fy;
  d.f_o[3 * i + 2] = fz;
}

}  // namespace

void launch_bond_orders(const Dev &d, cudaStream_t st) {
  const int B = 256;
  k_bo_deltap<<<(d.n + B - 1) / B, B, 0, st>>>(d);
  const long long slots = (long long)d.n * d.bond_cap;
  k_bo_correct<<<(unsigned)((slots + B - 1) / B), B, 0, st>>>(d);
  k_bo_atom<<<(d.n + B - 1) / B, B, 0, st>>>(d);
}

void launch_atom_energy(const Dev &d, cudaStream_t st, int eflag) {
  k_atom_energy<<<(d.n + 255) / 256, 256, 0, st>>>(d, eflag);
}

void launch_hbonds(const Dev &d, cudaStream_t st, int eflag) {
  const long long threads = (long long)d.n * 32;
  k_hbonds<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(d, eflag);
}

void launch_valence_torsion(const Dev &d, cudaStream_t st, int eflag) {
  const long long slots = (long long)d.n * d.bond_cap;
  k_valence_torsion<<<(unsigned)((slots + 127) / 128), 128, 0, st>>>(d, eflag);
}

void launch_vt_count(const Dev &d, cudaStream_t st) {
  const int B = 256;
  const long long slots = (long long)d.n * d.bond_cap;
  k_vt_prep_center<<<(d.n + B - 1) / B, B, 0, st>>>(d);
  k_vt_prep_bond<<<(unsigned)((slots + B - 1) / B), B, 0, st>>>(d);
  k_vt_count<<<(unsigned)((slots + 1 + B - 1) / B), B, 0, st>>>(d);
  launch_scan(d.w_cnt_v, d.w_off_v, (int)(slots + 1), d.w_bsum, st);
  launch_scan(d.w_cnt_t, d.w_off_t, (int)(slots + 1), d.w_bsum, st);
}

void launch_vt_run(const Dev &d, cudaStream_t st, int eflag, long long nval, long long ntor) {
  const int B = 256;
  const long long slots = (long long)d.n * d.bond_cap;
  k_vt_fill<<<(unsigned)((slots + B - 1) / B), B, 0, st>>>(d);
  if (nval > 0) k_valence<<<(unsigned)((nval + 127) / 128), 128, 0, st>>>(d, eflag, nval);
  if (ntor > 0) k_torsion<<<(unsigned)((ntor + 127) / 128), 128, 0, st>>>(d, eflag, ntor);
}

void launch_dbond_forces(const Dev &d, cudaStream_t st) {
  const int B = 256;
  k_dbond<<<(d.n + B - 1) / B, B, 0, st>>>(d);
}

void launch_force_out(const Dev &d, cudaStream_t st) {
  const int B = 256;
  k_force_out<<<(d.n + B - 1) / B, B, 0, st>>>(d);
}


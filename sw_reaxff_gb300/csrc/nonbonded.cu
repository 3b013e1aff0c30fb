// vdW + Coulomb with the 7th-order taper.
//
// The reference loops the full far list of each local atom and puts the
// force on i only (vdW_Coulomb_Energy_Full_C_test_err,
// reaxc_nonbonded_sw64.c:40-258).  Here each unordered pair is evaluated
// once (Newton's third law, equal and opposite forces via FP64 atomics),
// which halves the FP64 work; the full-list energy sums the reference
// reports in pvector (e_vdW, e_ele = twice the physical value) are recovered
// by doubling, and eng_vdwl / eng_coul get the physical (half-tallied) sums
// like ev_tally_full (reaxc_inlines_sw64.h:178-222).
#include <type_traits>

#include "rg_internal.h"

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr double C_ele = RG_C_ELE;
constexpr int IMG0 = 62;              // img_pack(0,0,0)

__device__ __forceinline__ double warp_sum(double v) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(FULL, v, off);
  return v;
}

constexpr int NBW = 8;     // warps per block
constexpr int QC = 64;     // queue slots per warp

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

struct PairQueue {
  uint32_t e[QC];
};

// Tap(r) and (1/r) dTap/dr (FP64 form)
__device__ __forceinline__ void taper(const Control &C, double r, double rinv, double &Tp,
                                      double &dTap) {
  const double *Tap = C.Tap;
  Tp = fma(Tap[7], r, Tap[6]);
  Tp = fma(Tp, r, Tap[5]);
  Tp = fma(Tp, r, Tap[4]);
  Tp = fma(Tp, r, Tap[3]);
  Tp = fma(Tp, r, Tap[2]);
  Tp = fma(Tp, r, Tap[1]);
  Tp = fma(Tp, r, Tap[0]);
  dTap = fma(7 * Tap[7], r, 6 * Tap[6]);
  dTap = fma(dTap, r, 5 * Tap[5]);
  dTap = fma(dTap, r, 4 * Tap[4]);
  dTap = fma(dTap, r, 3 * Tap[3]);
  dTap = fma(dTap, r, 2 * Tap[2]);
  dTap = fma(Tap[1], rinv, dTap);
}

__device__ __forceinline__ double cubic_u(const double2 &c01, const double2 &c23, double u) {
  return fma(fma(fma(c23.y, u, c23.x), u, c01.y), u, c01.x);
}

// FP64 form: vdW + Coulomb of one queued pair, from the pair-function
// tables (tabulate > 0) or the reference's expressions; returns whether the
// pair is inside the cutoff, (1/r) dE/dr in c and the displacement; with EF
// the energies are added to evdw and eele
template <bool EF>
__device__ __forceinline__ bool pair_terms(const Dev &d, const ForceField &F, const Control &C,
                                          uint32_t e, bool act, const double4 &xi,
                                          const float4 &xif, const float4 &xil, fpair qi, int ti,
                                          const SegGeom &g, double &ev, double &ee,
                                          double &c, double &dx, double &dy, double &dz,
                                          int &j) {
  c = 0.0; dx = dy = dz = 0.0; ev = ee = 0.0;
  j = (int)(e >> 8);
  if (!act) return false;
  int sx, sy, sz;
  img_unpack((int)(e & 255u), &sx, &sy, &sz);
  const double4 xj = d.xs[j];
  const double qj = xj.w;
  disp64(g, xj, xi, sx, sy, sz, dx, dy, dz);
  // the cutoff test with the reference's rounding where the list reaches
  // beyond nonb_cut; r^2 for the pair functions by FMAs
  if (!C.nonb_all_listed &&
      __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)) > C.nonb_cut2)
    return false;
  if (d.tab_nb_fp && !g.tri) {
    // orthogonal segments: the table lookup with r^2, the interval offset,
    // the cubics and q_i q_j as FP32 pairs (~1e-13 relative, far below the
    // tables' 1e-10); the FP64 pipe takes the conversions, the
    // displacement and the force products only
    const float4 hj = d.xf[j], lj = d.xl[j];
    const fpair s2 = fp_d2(g, hj, lj, xif, xil, sx, sy, sz);
    if (s2.hi >= C.tab_s0_f) {
      int k;
      fpair u;
      fp_interval(C, s2, k, u);
      const float4 *T = d.tab_nb_fp + ((long long)C.tab_pair[ti][__float_as_int(hj.w)] * C.tab_n + k) * 8;
      const fpair qq = fp_mul(qi, {lj.w, d.qlo[j]});
      c = fp_to_double(fp_add(fp_cubic(T[0], T[1], u), fp_mul(qq, fp_cubic(T[2], T[3], u))));
      if (EF) {
        ev = fp_to_double(fp_cubic(T[4], T[5], u));
        ee = fp_to_double(fp_mul(qq, fp_cubic(T[6], T[7], u)));
      }
      return true;
    }
  }
  const double d2 = fma(dx, dx, fma(dy, dy, dz * dz));
  if (C.tab_n && d2 >= C.tab_s0) {
    // FP64 tables in s = r^2: (1/r) dE/dr of vdW and of Coulomb per unit
    // qi qj (C_ele folded in) as cubics in u of the interval; the energies'
    // cubics follow and are read on energy steps only
    const double x = fma(d2, C.tab_inv_ds, C.tab_x0);
    int k = (int)x;
    if (k > C.tab_n - 1) k = C.tab_n - 1;
    const double u = x - (double)k;
    const double2 *T = reinterpret_cast<const double2 *>(
        d.tab_nb + ((long long)C.tab_pair[ti][d.ts[j]] * C.tab_n + k) * 16);
    const double qq = xi.w * qj;
    c = fma(cubic_u(T[2], T[3], u), qq, cubic_u(T[0], T[1], u));
    if (EF) {
      ev = cubic_u(T[4], T[5], u);
      ee = qq * cubic_u(T[6], T[7], u);
    }
    return true;
  }
  const double rinv = rsqrt(d2);
  const double r = d2 * rinv;
  const Tbp &tw = F.tbp[ti][d.ts[j]];
  double Tp, dTap;
  taper(C, r, rinv, Tp, dTap);
  const double p_vdW1 = F.gp[28];
  const int vdw_type = F.vdw_type;
  const double alpha = tw.alpha, r_vdW = tw.r_vdW, D = tw.D;
  const double ar = alpha / r_vdW;
  double e_vdW, CEvd, e_core = 0, e_lg = 0;
  if (vdw_type == 1 || vdw_type == 3) {
    // shielded Morse: fn13 = (r^p + gamma_w^-p)^(1/p)
    const double powr = exp(p_vdW1 * log(r));                 // r^p
    const double S = powr + tw.powgi_vdW1;
    const double fn13 = exp(log(S) / p_vdW1);                 // S^(1/p)
    const double exp2 = exp(0.5 * alpha * (1.0 - fn13 / r_vdW));
    const double exp1 = exp2 * exp2;
    e_vdW = D * (exp1 - 2.0 * exp2);
    const double dfn13 = (fn13 / S) * (powr / d2);            // S^(1/p-1) r^(p-2)
    CEvd = dTap * e_vdW - Tp * D * ar * (exp1 - exp2) * dfn13;
  } else {
    const double exp2 = exp(0.5 * alpha * (1.0 - r / r_vdW));
    const double exp1 = exp2 * exp2;
    e_vdW = D * (exp1 - 2.0 * exp2);
    CEvd = dTap * e_vdW - Tp * D * ar * (exp1 - exp2) * rinv;
  }
  if (vdw_type == 2 || vdw_type == 3) {
    const double acore = tw.acore, rcore = tw.rcore;
    e_core = tw.ecore * exp(acore * (1.0 - (r / rcore)));
    const double de_core = -(acore / rcore) * e_core;
    CEvd += dTap * e_core + Tp * de_core * rinv;
    if (C.lgflag) {
      const double r5 = d2 * d2 * r, r6 = d2 * d2 * d2;
      const double lg2 = tw.lgre * tw.lgre;
      const double re6 = lg2 * lg2 * lg2;
      e_lg = -(tw.lgcij / (r6 + re6));
      const double de_lg = -6.0 * e_lg * r5 / (r6 + re6);
      CEvd += dTap * e_lg + Tp * de_lg * rinv;
    }
  }
  // shielded Coulomb: Tap qi qj / (r^3 + gamma)^c
  const double dr3gamij_1 = fma(d2, r, tw.gamma);
  const double inv3 = rpow_third(dr3gamij_1, RG_C3_ELE);
  const double qq = C_ele * xi.w * qj;
  const double CEclmb = qq * (dTap - Tp * r / dr3gamij_1) * inv3;
  if (EF) {
    ev = Tp * (e_vdW + e_core + e_lg);
    ee = qq * Tp * inv3;
  }
  c = CEvd + CEclmb;
  return true;
}

__device__ __forceinline__ fpair fp_split(double v) {
  const float h = __double2float_rn(v);
  return {h, __double2float_rn(v - (double)h)};
}

// FP64 form, orthogonal segment, every listed pair inside the cutoff, no
// virial or per-atom tally: the pair's force g = (1/r) dE/dr (x_j - x_i)
// with the displacement, the table lookup and the products as FP32 pairs
// (~1e-13 relative); the FP64 pipe converts g for the partner's atomics
// only.  Pairs below the tables take the FP64 expressions.
template <bool EF>
__device__ __forceinline__ bool pair_fp(const Dev &d, const ForceField &F, const Control &C,
                                       uint32_t e, bool act, const double4 &xi, const float4 &xif,
                                       const float4 &xil, fpair qi, int ti, const SegGeom &g,
                                       double &ev, double &ee, fpair &gx, fpair &gy, fpair &gz,
                                       int &j) {
  gx = gy = gz = {0.f, 0.f};
  ev = ee = 0.0;
  j = (int)(e >> 8);
  if (!act) return false;
  int sx, sy, sz;
  img_unpack((int)(e & 255u), &sx, &sy, &sz);
  const float4 hj = d.xf[j], lj = d.xl[j];
  const fpair dx = fp_disp(hj.x, lj.x, xif.x, xil.x, sx, g.Lh[0], g.Ll[0]);
  const fpair dy = fp_disp(hj.y, lj.y, xif.y, xil.y, sy, g.Lh[1], g.Ll[1]);
  const fpair dz = fp_disp(hj.z, lj.z, xif.z, xil.z, sz, g.Lh[2], g.Ll[2]);
  const fpair s2 = fp_add(fp_add(fp_sqr(dx), fp_sqr(dy)), fp_sqr(dz));
  if (!(s2.hi >= C.tab_s0_f)) {
    double c, ex, ey, ez;
    if (!pair_terms<EF>(d, F, C, e, act, xi, xif, xil, qi, ti, g, ev, ee, c, ex, ey, ez, j))
      return false;
    gx = fp_split(c * ex);
    gy = fp_split(c * ey);
    gz = fp_split(c * ez);
    return true;
  }
  int k;
  fpair u;
  fp_interval(C, s2, k, u);
  const float4 *T = d.tab_nb_fp + ((long long)C.tab_pair[ti][__float_as_int(hj.w)] * C.tab_n + k) * 8;
  const fpair qq = fp_mul(qi, {lj.w, d.qlo[j]});
  const fpair c = fp_add(fp_cubic(T[0], T[1], u), fp_mul(qq, fp_cubic(T[2], T[3], u)));
  gx = fp_mul(c, dx);
  gy = fp_mul(c, dy);
  gz = fp_mul(c, dz);
  if (EF) {
    ev = fp_to_double(fp_cubic(T[4], T[5], u));
    ee = fp_to_double(fp_mul(qq, fp_cubic(T[6], T[7], u)));
  }
  return true;
}

__device__ __forceinline__ float cubic_uf(const float4 &c, float u) {
  return fmaf(fmaf(fmaf(c.w, u, c.z), u, c.y), u, c.x);
}

// Mixed form: vdW + Coulomb of one pair entirely in FP32, parameters from
// the control block's FP32 copies (no double is read or converted per
// pair), or from the FP32 copy of the pair-function tables (their index
// and fraction from the FP32 r^2, whose rounding the fraction inherits);
// returns (1/r) dE/dr in c, the displacement and, with EF, the energies.
template <bool EF>
__device__ __forceinline__ void pair32(const Dev &d, const Control &C, int vdw_type, uint32_t e,
                                       bool act, const double4 &xi, const float4 &xif,
                                       const float4 &xil, int ti, const SegGeom &g, float &ev,
                                       float &ee, float &c, float &dx, float &dy, float &dz,
                                       int &j) {
  c = 0.f; dx = dy = dz = 0.f; ev = ee = 0.f;
  j = (int)(e >> 8);
  if (!act) return;
  int sx, sy, sz;
  img_unpack((int)(e & 255u), &sx, &sy, &sz);
  const float4 hj = d.xf[j], lj = d.xl[j];
  disp32(g, hj, lj, xif, xil, sx, sy, sz, dx, dy, dz);
  const float d2 = dx * dx + dy * dy + dz * dz;
  if (!C.nonb_all_listed) {
    // the list reaches the QEq taper radius beyond nonb_cut: FP64 only near
    // the cutoff
    const float nc2 = C.nonb_cut2_f;
    bool out;
    if (d2 <= nc2 * (1.f - 1e-5f)) out = false;
    else if (d2 > nc2 * (1.f + 1e-5f)) out = true;
    else {
      double ex, ey, ez;
      disp64(g, d.xs[j], xi, sx, sy, sz, ex, ey, ez);
      out = __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez)) > C.nonb_cut2;
    }
    if (out) {
      dx = dy = dz = 0.f;
      return;
    }
  }
  const int tj = __float_as_int(hj.w);
  if (C.tab_n && d2 >= C.tab_s0_f) {
    const float x = fmaf(d2, C.tab_inv_ds_f, C.tab_x0_f);
    int k = (int)x;
    if (k > C.tab_n - 1) k = C.tab_n - 1;
    const float u = x - (float)k;
    const float4 *T = reinterpret_cast<const float4 *>(
        d.tab_nb32 + ((long long)C.tab_pair[ti][tj] * C.tab_n + k) * 16);
    const float qq = xil.w * lj.w;   // C_ele is in the Coulomb cubics
    c = fmaf(cubic_uf(T[1], u), qq, cubic_uf(T[0], u));
    if (EF) {
      ev = cubic_uf(T[2], u);
      ee = qq * cubic_uf(T[3], u);
    }
    return;
  }
  const Control::NbF &P = C.nb32[ti][tj];
  const float rinv = rsqrtf(d2);
  const float r = d2 * rinv;
  float Tp, dTap;
  if (C.tap_factored) {
    // (1-t)^4 (1 + 4t + 10t^2 + 20t^3), t = r/swb;  (1/r) d/dr = -140 t^2 (1-t)^3 / swb^2
    const float is = C.inv_swb_nb_f;
    const float t = r * is, u = 1.f - t, u2 = u * u;
    Tp = u2 * u2 * (1.f + t * (4.f + t * (10.f + t * 20.f)));
    dTap = -140.f * t * t * u2 * u * is * is;
  } else {
    const float *T = C.Tap_f, *D = C.dTap_f;
    Tp = fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(T[7], r, T[6]), r, T[5]), r, T[4]), r, T[3]), r, T[2]),
                   r, T[1]), r, T[0]);
    dTap = fmaf(fmaf(fmaf(fmaf(fmaf(D[7], r, D[6]), r, D[5]), r, D[4]), r, D[3]), r, D[2]);
    dTap = fmaf(T[1], rinv, dTap);
  }
  float e_vdW, CEvd, e_core = 0.f, e_lg = 0.f;
  if (vdw_type == 1 || vdw_type == 3) {
    const float p = C.p_vdW1_f;
    const float powr = expf(p * logf(r));                // r^p
    const float S = powr + P.powgi;
    const float fn13 = expf(logf(S) / p);                // S^(1/p)
    const float exp2 = expf(0.5f * P.alpha * (1.f - fn13 / P.r_vdW));
    const float exp1 = exp2 * exp2;
    e_vdW = P.D * (exp1 - 2.f * exp2);
    const float dfn13 = (fn13 / S) * (powr / d2);            // S^(1/p-1) r^(p-2)
    CEvd = dTap * e_vdW - Tp * P.D * P.ar * (exp1 - exp2) * dfn13;
  } else {
    const float exp2 = expf(0.5f * P.alpha * (1.f - r / P.r_vdW));
    const float exp1 = exp2 * exp2;
    e_vdW = P.D * (exp1 - 2.f * exp2);
    CEvd = dTap * e_vdW - Tp * P.D * P.ar * (exp1 - exp2) * rinv;
  }
  if (vdw_type == 2 || vdw_type == 3) {
    e_core = P.ecore * expf(P.acore * (1.f - r / P.rcore));
    const float de_core = -(P.acore / P.rcore) * e_core;
    CEvd += dTap * e_core + Tp * de_core * rinv;
    if (C.lgflag) {
      const float r5 = d2 * d2 * r, r6 = d2 * d2 * d2;
      e_lg = -(P.lgcij / (r6 + P.re6));
      const float de_lg = -6.f * e_lg * r5 / (r6 + P.re6);
      CEvd += dTap * e_lg + Tp * de_lg * rinv;
    }
  }
  // shielded Coulomb: Tap qi qj / (r^3 + gamma)^(1/3)
  const float dr3 = fmaf(d2, r, P.gamma);
  const float inv3 = rcbrtf(dr3);
  const float qq = (float)C_ele * xil.w * lj.w;
  ee = qq * Tp * inv3;
  ev = Tp * (e_vdW + e_core + e_lg);
  c = CEvd + qq * (dTap - Tp * r / dr3) * inv3;
}

// AT: one pair's halves of energy and virial to atom i (registers, summed
// per warp at the end) and to atom j (atomics); dx = x_j - x_i and c =
// (1/r) dE/dr here, so del (x) del fpair = -c dx (x) dx
__device__ __forceinline__ void atom_tally(const Dev &d, double *ta, int j, double ev, double ee,
                                           double c, double dx, double dy, double dz) {
  const double e = 0.5 * (ev + ee), h = -0.5 * c;
  const double v[6] = {h * dx * dx, h * dy * dy, h * dz * dz, h * dx * dy, h * dx * dz, h * dy * dz};
  ta[0] += e;
  atomicAdd(&d.eatom[j], e);
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    ta[1 + k] += v[k];
    atomicAdd(&d.vatom[(long long)k * d.n + j], v[k]);
  }
}

// one warp per atom i; the pairs (i,j,image) with j > i, or j == i with the
// "positive" image, are queued and evaluated 32 at a time
// the FP64 form is FP64-pipe bound: three blocks per SM (80 registers, a
// few spilled) keep the pipe busier than two (7 % faster); the FP32 form
// has no minimum (0) and keeps its 66-80 registers
// AT (only with EF): per-atom tallies of LAMMPS's eflag_atom / vflag_atom,
// as the reference's ev_tally_full over the full list
// (reaxc_nonbonded_sw64.c:198-213): each directed pair gives its centre
// half of the pair's vdW + Coulomb energy and half of del (x) del fpair
// (del = x_i - x_j, fpair = -(1/r) dE/dr).  An unordered pair here gives
// both atoms those halves (the two directions have the same values).
template <typename R, bool VIR, bool EF, bool AT = false>
__global__ void __launch_bounds__(NBW * 32, std::is_same<R, double>::value ? 3 : 0)
    k_nonbonded(Dev d) {
  __shared__ PairQueue queues[NBW];
  const int lane = threadIdx.x & 31;
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  double evdw = 0.0, eele = 0.0;
  double w[6] = {0, 0, 0, 0, 0, 0};
  if (i < d.n) {
    PairQueue &Q = queues[threadIdx.x >> 5];
    const ForceField &F = *d.ff;
    const Control &C = *d.ctl;
    const int n = d.n;
    const double4 xi = d.xs[i];
    const float4 xif = d.xf[i];
    const float4 xil = d.xl[i];
    const fpair qi = {xil.w, d.mixed ? 0.f : d.qlo[i]};
    const int ti = d.ts[i];
    const SegGeom &g = d.seg[d.seg_s[i]];
    const long long row = (long long)i * d.nb_cap;
    const int nn = nbr_near_count(d, i), nf = nbr_far_count(d, i);
    const int capN = d.nb_capN;
    const int tot = nn + nf;
    double fx = 0, fy = 0, fz = 0;
    fpair gxs = {0.f, 0.f}, gys = gxs, gzs = gxs;  // pair_fp: sum of the pairs' g
    const bool fast = !VIR && !AT && d.tab_nb_fp && !g.tri && C.nonb_all_listed;
    float fx32 = 0.f, fy32 = 0.f, fz32 = 0.f;   // mixed form: FP32 force sums
    double ta[7] = {0, 0, 0, 0, 0, 0, 0};        // AT: atom i's energy and virial
    double *fC = d.fC;
    const int vdw_type = F.vdw_type;
    int qn = 0;
    for (int base = 0; base < tot + 32; base += 32) {
      if (base < tot) {
        const int p = base + lane;
        bool take = false;
        uint32_t e = 0;
        if (p < tot) {
          const int slot = p < nn ? p : capN + (p - nn);
          e = d.nbr[row + slot];
          const int j = (int)(e >> 8);
          take = j > i || (j == i && (int)(e & 255u) > IMG0);
        }
        const unsigned m = __ballot_sync(FULL, take);
        if (take) Q.e[qn + __popc(m & lanemask_lt())] = e;
        qn += __popc(m);
        __syncwarp();
      }
      // evaluate a full batch, or the remainder after the last entry
      while (qn >= 32 || (base >= tot && qn > 0)) {
        const int cnt = min(qn, 32);
        const bool act = lane < cnt;
        const uint32_t e = act ? Q.e[lane] : 0u;
        int j;
        if constexpr (std::is_same<R, float>::value) {
          float ev, ee, c, dx, dy, dz;
          pair32<EF>(d, C, vdw_type, e, act, xi, xif, xil, ti, g, ev, ee, c, dx, dy, dz, j);
          if (EF) {   // energies summed in FP64 (only on energy steps)
            evdw += (double)ev;
            eele += (double)ee;
          }
          if (act && c != 0.f) {
            fx32 -= c * dx;
            fy32 -= c * dy;
            fz32 -= c * dz;
            atomicAdd(&d.fC32[j], c * dx);
            atomicAdd(&d.fC32[n + j], c * dy);
            atomicAdd(&d.fC32[2 * n + j], c * dz);
            if (VIR) vir_acc(w, dx, dy, dz, (double)(c * dx), (double)(c * dy), (double)(c * dz));
          }
          if (AT && act)
            atom_tally(d, ta, j, (double)ev, (double)ee, (double)c, (double)dx, (double)dy,
                       (double)dz);
        } else if (fast) {
          fpair gx, gy, gz;
          double ev, ee;
          if (pair_fp<EF>(d, F, C, e, act, xi, xif, xil, qi, ti, g, ev, ee, gx, gy, gz, j)) {
            gxs = fp_add(gxs, gx);
            gys = fp_add(gys, gy);
            gzs = fp_add(gzs, gz);
            atomicAdd(&fC[j], fp_to_double(gx));
            atomicAdd(&fC[n + j], fp_to_double(gy));
            atomicAdd(&fC[2 * n + j], fp_to_double(gz));
            if (EF) {
              evdw += ev;
              eele += ee;
            }
          }
        } else {
          double c, dx, dy, dz, ev, ee;
          if (pair_terms<EF>(d, F, C, e, act, xi, xif, xil, qi, ti, g, ev, ee, c, dx, dy, dz, j)) {
            fx -= c * dx;
            fy -= c * dy;
            fz -= c * dz;
            atomicAdd(&fC[j], c * dx);
            atomicAdd(&fC[n + j], c * dy);
            atomicAdd(&fC[2 * n + j], c * dz);
            if (VIR) vir_acc(w, dx, dy, dz, c * dx, c * dy, c * dz);
            if (EF) {
              evdw += ev;
              eele += ee;
            }
            if (AT) atom_tally(d, ta, j, ev, ee, c, dx, dy, dz);
          }
        }
        __syncwarp();
        const int left = qn - cnt;
        uint32_t le = 0;
        if (lane < left) le = Q.e[cnt + lane];
        __syncwarp();
        if (lane < left) Q.e[lane] = le;
        qn = left;
        __syncwarp();
      }
    }
    if constexpr (std::is_same<R, float>::value) {
      for (int off = 16; off > 0; off >>= 1) {
        fx32 += __shfl_down_sync(FULL, fx32, off);
        fy32 += __shfl_down_sync(FULL, fy32, off);
        fz32 += __shfl_down_sync(FULL, fz32, off);
      }
      if (lane == 0) {
        atomicAdd(&d.fC32[i], fx32);
        atomicAdd(&d.fC32[n + i], fy32);
        atomicAdd(&d.fC32[2 * n + i], fz32);
      }
    } else {
      if (fast) {
        fx -= fp_to_double(gxs);
        fy -= fp_to_double(gys);
        fz -= fp_to_double(gzs);
      }
      fx = warp_sum(fx);
      fy = warp_sum(fy);
      fz = warp_sum(fz);
      if (lane == 0) {
        atomicAdd(&fC[i], fx);
        atomicAdd(&fC[n + i], fy);
        atomicAdd(&fC[2 * n + i], fz);
      }
    }
    if (AT) {
#pragma unroll
      for (int k = 0; k < 7; ++k) ta[k] = warp_sum(ta[k]);
      if (lane == 0) {
        atomicAdd(&d.eatom[i], ta[0]);
#pragma unroll
        for (int k = 0; k < 6; ++k) atomicAdd(&d.vatom[(long long)k * n + i], ta[1 + k]);
      }
    }
  }
  if (EF) {
    const int sg = i < d.n ? d.seg_s[i] : -1;
    const double v[4] = {2.0 * evdw, 2.0 * eele, evdw, eele};
    static_assert(E_ELE == E_VDW + 1, "energy slots");
    seg_block_add<2>(v, sg, d.energy + E_VDW, RG_NE);
    seg_block_add<1>(v + 2, sg, d.energy + E_ENG_VDWL, RG_NE);
    seg_block_add<1>(v + 3, sg, d.energy + E_ENG_COUL, RG_NE);
  }
  if (VIR) seg_block_add<6>(w, i < d.n ? d.seg_s[i] : -1, d.virial, 6);
}

}  // namespace

template <typename R, bool VIR>
void launch_nb(const Dev &d, cudaStream_t st, int eflag, unsigned G) {
  if (d.atom_tally) k_nonbonded<R, VIR, true, true><<<G, NBW * 32, 0, st>>>(d);
  else if (eflag) k_nonbonded<R, VIR, true><<<G, NBW * 32, 0, st>>>(d);
  else k_nonbonded<R, VIR, false><<<G, NBW * 32, 0, st>>>(d);
}

void launch_nonbonded(const Dev &d, cudaStream_t st, int eflag) {
  const long long threads = (long long)d.n * 32;
  const unsigned G = (unsigned)((threads + NBW * 32 - 1) / (NBW * 32));
  if (d.vflag) {
    if (d.mixed) launch_nb<float, true>(d, st, eflag, G);
    else launch_nb<double, true>(d, st, eflag, G);
  } else {
    if (d.mixed) launch_nb<float, false>(d, st, eflag, G);
    else launch_nb<double, false>(d, st, eflag, G);
  }
}

// Internal types of the reaxgpu library (host + device).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#define RG_MAXT 8       // force-field atom types supported
#define RG_MAX3 5       // three-body parameter sets per type triple
#define RG_NE 17        // energy vector length (RG_NENERGY)

// energy slots (pvector order of pair_reaxc_sunway.cpp:657-670, then
// eng_vdwl, eng_coul, physical e_pol)
enum {
  E_BOND = 0, E_OVUN, E_LP, E_3, E_ANG, E_PEN, E_COA, E_HB, E_TOR, E_CON,
  E_VDW, E_ELE, E_12, E_POL, E_ENG_VDWL, E_ENG_COUL, E_POL_PHYS
};

struct Sbp {
  double r_s, valency, mass, r_vdw, epsilon, gamma, r_pi, valency_e, nlp_opt;
  double alpha, gamma_w, valency_boc, p_ovun5, chi, eta;
  double r_pi_pi, p_lp2, b_o_131, b_o_132, b_o_133;
  double p_ovun2, p_val3, valency_val, p_val5, rcore2, ecore2, acore2;
  double lgcij, lgre;
  int p_hbond;
  int is_carbon;
  char name[8];
};

struct Tbp {
  double r_s, r_p, r_pp, p_bo1, p_bo2, p_bo3, p_bo4, p_bo5, p_bo6;
  double p_boc3, p_boc4, p_boc5, v13cor, ovc;
  double De_s, De_p, De_pp, p_be1, p_be2, p_ovun1;
  double D, alpha, r_vdW, gamma_w, gamma, rcore, ecore, acore, lgcij, lgre;
  // derived for the nonbonded kernel
  double powgi_vdW1;   // pow(1/gamma_w, p_vdW1)
};

struct Thbp {
  double theta_00, p_val1, p_val2, p_coa1, p_val7, p_pen1, p_val4;
};
struct Thbh {
  int cnt;
  Thbp prm[RG_MAX3];
};
struct Fbp {
  double V1, V2, V3, p_tor1, p_cot1;
};
struct Fbh {
  int cnt;
  Fbp prm;
};
struct Hbp {
  double r0_hb, p_hb1, p_hb2, p_hb3;
  double inv_r0_hb;   // 1 / r0_hb (derived at load)
};

// Whole force field, plain data, copied once to device memory.
struct ForceField {
  int ntypes, vdw_type, ngp;
  double gp[64];
  Sbp sbp[RG_MAXT];
  Tbp tbp[RG_MAXT][RG_MAXT];
  Thbh thbp[RG_MAXT][RG_MAXT][RG_MAXT];
  Hbp hbp[RG_MAXT][RG_MAXT][RG_MAXT];
  Fbh fbp[RG_MAXT][RG_MAXT][RG_MAXT][RG_MAXT];
  double nve_mass[RG_MAXT];   // integrator masses (default: sbp mass)
};

// Geometry of one segment: a periodic box with edge vectors a = (lx, 0, 0),
// b = (xy, ly, 0), c = (xz, yz, lz) (LAMMPS's restricted triclinic form;
// orthogonal when the tilts are zero) and its cells.
struct SegGeom {
  double L[3];        // lx, ly, lz
  double tilt[3];     // xy, xz, yz
  int tri;            // a tilt is nonzero: fractional binning and wrap
  float Lh[3], Ll[3]; // L as an unevaluated FP32 pair (hi + lo)
  float Th[3];        // tilts in FP32 (prefilter shifts only)
  double cellw[3];    // orthogonal: cell edges (L / nc)
  float cellw_f[3];   // the same in FP32 (clipping the stencil)
  int nc[3];          // cells per dimension (fractional axes when tri)
  int S;              // stencil half-width (cells)
  int cell0;          // first global cell index of the segment
  int atom0, natoms;  // original-order atom range
};

constexpr int RG_NRED = 128;   // QEq scalar slots per segment

// Scalar controls shared by all kernels.
struct Control {
  double bo_cut, nonb_cut, nonb_low, bond_cut, hbond_cut, thb_cut, thb_cutsq;
  double list_cut2;   // squared pair-list cutoff max(nonb_cut, qeq_swb)^2
  double nonb_cut2, swb2;
  double near_cut;    // max(bond_cut, hbond_cut): "near" part of a row
  double near_cut2_lo, near_cut2_hi;   // near_cut^2 (1 -/+ 1e-12)
  float bond_cut_f, hbond_cut_f;        // FP32 copies for FP32-first tests
  double Tap[8];      // pair taper (swa = nonb_low, swb = nonb_cut)
  double qTap[8];     // QEq taper
  int enobondsflag, lgflag;
  // mixed form: the taper in factored form (1-t)^4 (1+4t+10t^2+20t^3),
  // t = r/swb, equal to the 7th-order polynomial when swa = 0; well
  // conditioned in FP32 near the cutoff where the expanded form cancels
  int tap_factored, qtap_factored;
  double inv_swb_nb, inv_swb_q;
  int nonb_all_listed;   // nonb_cut >= list cutoff: every list entry is a vdW/Coulomb pair
  int h_all_listed;      // qeq_swb >= list cutoff: every list entry has an H_ij
  // FP64 tables (tables.cpp): tab_n intervals of width tab_ds over
  // s = r^2 in [tab_s0, ...]; 0 = analytic pair functions
  int tab_n;
  double tab_s0, tab_ds, tab_inv_ds, tab_x0;   // tab_x0 = -tab_s0 / tab_ds
  float tab_s0_f;        // table or analytic form below it (either is the function)
  float tab_inv_ds_f, tab_x0_f;   // the mixed form's FP32 lookups
  float tab_inv_ds_l, tab_x0_l;   // with these: tab_inv_ds, tab_x0 as FP32 pairs
  int tab_pair[RG_MAXT][RG_MAXT];   // unordered type pair -> table index
  // FP32 copies for the prefilters (no FP64 conversions per entry; GB300
  // runs FP64 at 1/64 of the FP32 rate)
  float list_pre2_f;   // FP32 pair-list prefilter radius^2: list_cut2 (1 + 1e-5) + 0.05
  float thb_cut_f, thb_cutsq_f;
  // type triples with a valence parameter set |p_val1| > 0.001, and type
  // quadruples with a nonzero torsion set (the enumeration's table tests)
  unsigned char thb_any[RG_MAXT][RG_MAXT][RG_MAXT];
  unsigned char fb_on[RG_MAXT][RG_MAXT][RG_MAXT][RG_MAXT];
  float bo_scale_f;    // 1 + bo_cut (FP32 estimate of BO')
  float bo_half_f;     // bo_cut / 2
  // mixed form, FP32 copies used per pair (GB300 runs FP64, conversions
  // included, at 1/64 of the FP32 rate, so the FP32 kernels read no double)
  float list_cut2_f, near_cut_f, swb2_f, inv_swb_q_f, nonb_cut2_f, inv_swb_nb_f;
  float qTap_f[8], Tap_f[8], dTap_f[8];   // dTap_f[k] = k Tap[k]
  float p_vdW1_f;
  struct NbF {
    float alpha, r_vdW, D, ar, powgi, gamma, ecore, acore, rcore, lgcij, re6;
  } nb32[RG_MAXT][RG_MAXT];
  struct HbF {
    float r0_hb, p_hb1, p_hb2, p_hb3;
  } hb32[RG_MAXT][RG_MAXT][RG_MAXT];
  // log r_s, log r_pi, log r_pipi per type pair: the FP64 BO' powers as
  // exp(p (log d - log r)) with one log per bond
  double ln_r[RG_MAXT][RG_MAXT][3];
  // FP32 estimate of BO' = sum_k exp(p_k (r / r0_k)^q_k) as
  // exp2(e_k exp2(q_k (log2 r - l_k))) with e_k = p_k log2(e), l_k = log2 r0_k
  struct BoEst {
    float e[3], q[3], l[3];
    int mask;          // 1: sigma, 2: pi, 4: pi-pi bond order terms present
  } bo_est[RG_MAXT][RG_MAXT];
};

// Parse an ffield file (restates Read_Force_Field,
// reaxc_ffield_sunway.cpp:35-714).  Returns empty string or an error.
std::string rg_read_ffield(const char *path, int lgflag, ForceField *ff);
int rg_pair_index(int ti, int tj, int nt);
double rg_build_tables(const ForceField &F, const Control &C, int n, double s0, double s1,
                       std::vector<double> &nb, std::vector<double> &hq, bool check);
void rg_init_taper(double swa, double swb, double *Tap);

// ---------------------------------------------------------------------
// Device-side view of one system (sorted atom order unless noted).
struct Dev {
  int n;              // atoms
  int mixed;          // 1: FP32 arithmetic in the pair / bond kernels
  int nb_cap;         // neighbour row capacity (row-major rows)
  int nbr_tiles;      // pair-list kernel: 0 warp per atom, 1 per-cell tiles
  int nb_capN;        // the first nb_capN slots of a row hold its near
                      // entries, the remaining nb_cap - nb_capN its far ones
  int bond_cap;       // bond slots per atom (slot-major: k*n + i)
  int hb_cap;         // H-bond partner slots per H atom (row-major)
  // independent periodic systems ("segments") in one set of arrays: atoms
  // of segment k are original indices [atom0, atom0 + natoms); a single
  // system is one segment
  int nseg;
  const SegGeom *seg;    // [nseg]
  int spmv_rw;           // lanes per row in the QEq SpMVs (8, 16, 32; autotuned)
  int *seg_o;            // segment of each atom (original order)
  int *seg_s;            // segment of each atom (sorted order)
  int ncell;             // cells over all segments

  const ForceField *ff;
  const Control *ctl;
  const double *tab_nb;  // [pair][interval][16]: cubics in u of Fv, Fc, Ev, Ec (tables.cpp)
  const double *tab_h;   // [pair][interval][4]: cubic in u of H_ij
  const float *tab_nb32; // mixed form: tab_nb in FP32
  // FP64 form: tab_nb and tab_h with each coefficient as an FP32 pair
  // (float4 = two coefficients), for the orthogonal segments' pairs
  const float4 *tab_nb_fp, *tab_h_fp;

  // original order (persistent state)
  double *x_o, *v_o, *q_o, *f_o;
  int *type_o, *tag_o;
  double *s_hist, *t_hist;     // [5][n]  (k*n + i, original order)

  // binning / sort
  int *cell_o;        // cell of original atom
  int *cell_count, *cell_start, *cell_fill;
  int *perm;          // sorted -> original
  int *iperm;         // original -> sorted

  // sorted atoms
  double4 *xs;        // x, y, z, q
  float4 *xf;         // fp32 x, y, z, (type as float)
  float4 *xl;         // x - xf (FP32), so x = xf + xl to ~2^-48;
                      // w: the charge (FP32)
  float *qlo;         // q - xl.w (FP32): the charge as an FP32 pair
  int *ts, *tags;

  // full pair list (both directions), row-major rows of nb_cap: near
  // entries (d <= near_cut) in slots [0, n_near), far ones in
  // [nb_capN, nb_capN + n_far); the order within a part is the order the
  // entries were claimed in (atomically, see k_build_nbrs)
  uint32_t *nbr;      // (j << 8) | image
  float2 *hvalp;      // QEq H_ij per entry (FP64 form) as an FP32 pair (hi, lo)
  float *hval32;      // QEq H_ij per entry (mixed form)
  int *n_near, *n_far;  // entries claimed (may exceed the part's capacity
                        // until the host regrows and re-runs)

  // bonds (slot-major, slot = k*n + i)
  int *nbonds;
  uint32_t *b_nbr;
  int *b_sym;
  double *b_d, *b_dx, *b_dy, *b_dz;
  double *b_BO, *b_BOs, *b_BOpi, *b_BOpi2;
  double *b_dBOp;     // 3 * slots (xyz blocks)
  double *b_dlnpi, *b_dlnpi2;  // 3 * slots
  double *b_C;        // 11 * slots: C1dbo C2dbo C3dbo C1dbopi C2dbopi C3dbopi C4dbopi C1dbopi2 C2dbopi2 C3dbopi2 C4dbopi2
  double *b_Cdbo, *b_Cdbopi, *b_Cdbopi2;

  // H-bond partners of H atoms (row-major hb_cap), entry = nbr-row index
  int *nhb;
  uint32_t *hb_nbr;

  // per-atom bond-order workspace (sorted order)
  double *bo0;        // total (uncorrected, then corrected) bond order
  double *Deltap, *Deltap_boc, *Delta, *Delta_e, *Delta_boc, *Delta_val;
  double *exp_boc;    // 2 * n: exp(-p_boc1 Deltap), exp(-p_boc2 Deltap) per atom
  double *vlpex, *nlp, *Delta_lp, *Delta_lp_temp, *dDelta_lp, *nlp_temp;
  double *dDeltap;    // 3 * n (xyz blocks)
  double *fC;         // 4 * n: force xyz blocks + CdDelta block
  float *fC32;        // mixed form: 3 * n force xyz blocks of the FP32 pair terms
  double *vsum;       // 2 * n: per valence centre, sum of CEval5 and of CEval6
                      // (their share of Cdbopi/Cdbopi2 and Cdbo of every bond
                      // of the centre, applied in k_dbond)

  // QEq vectors (sorted order), two solves s,t interleaved as double2:
  // iterate x, right-hand side b, residual r, preconditioned residual u,
  // search direction p (qd, the SpMV's input) and its product q = H p
  double2 *qx, *qb, *qr, *qu, *qd, *qq;
  float4 *qd32;   // qd split into FP32 (hi, lo) pairs, s then t (the SpMVs' input)
  double *Hdia_inv;
  double *red;        // device scalars / reduction accumulators, RG_NRED per segment
  double *energy;     // [nseg][RG_NE]
  double *virial;     // [nseg][6]: xx yy zz xy xz yz of sum r (x) f (LAMMPS order)
  int vflag;          // accumulate the virial in this force step
  int *n_active;      // QEq: segments with an active solve (host poll)

  // valence / torsion work lists (built per force step)
  double *c_sbo;      // 10 * n per centre: SBO2, CSBO2, dSBO1, dSBO2, expval6, and in
                      // the FP64 form f9(Delta), Cf9/f9, 1/(1 + exp(p_coa2 Delta_val)),
                      // exp(-p_val10 (2 - SBO2)), -p_coa2 exp(..)/(1 + exp(..))
  double *b_et2, *b_ec2;   // per bond slot: exp(-p_tor2 BOA), exp(-p_cot2 (BOA-1.5)^2)
  double *b_vexp;     // 3 * slots (FP64 form): exp(-p_pen2 (BOA-2)^2),
                      // exp(-p_coa3 (bo0[nbr] - BOA)^2), exp(-p_coa4 (BOA-1.5)^2)
  float *b_BOf;             // per bond slot: BO in FP32, 0 where BO <= thb_cut (exact
                            // FP64 test), for the valence/torsion enumeration
  int *w_cnt_v, *w_cnt_t;  // per (centre, bond) slot counts (+1 trailing zero)
  int *w_off_v, *w_off_t;  // exclusive scans (+1: totals)
  int *w_bsum;             // scan block sums
  unsigned long long *w_val, *w_tor;   // packed items
  long long cap_val, cap_tor;
  // mixed form: near-linear angles and torsions the FP32 kernels hand to
  // an FP64 pass (fb_cnt[0] angles, fb_cnt[1] torsions)
  unsigned long long *w_fb_val, *w_fb_tor;
  int *fb_cnt;

  // RG_CHECK_FINITE=2: the first non-finite angle or torsion term is
  // recorded with its inputs (dbg_flag set, dbg[0..39])
  int debug;
  int *dbg_flag;
  double *dbg;

  // captured single-point step: QEq control on the device (qeq_ctl: 0
  // restarts, 1 loop trips, 2 trip limit reached), per-segment CG iteration
  // totals (qeq_tot[2 * nseg]), the histories saved at the step's start
  int *qeq_ctl, *qeq_tot;
  double *hist_save;     // [16][n]: s_hist, t_hist, then (MD step) x, v

  // per-atom tallies (LAMMPS eflag_atom / vflag_atom) of the nonbonded
  // pair terms, sorted order: eatom[n], vatom[6][n] (xx yy zz xy xz yz)
  int atom_tally;
  double *eatom, *vatom;

  int *status;        // [RG_NSTATUS]: 0 overflow flags, 1 max near entries, 2 max bonds,
                      // 3 max hb, 4 nonfinite, 5 pair entries, 6 bonds, 7 H-bond
                      // partners, 8 max far entries
};

// status slots
enum { ST_OVF = 0, ST_MAXNB = 1, ST_MAXB = 2, ST_MAXHB = 3, ST_NAN = 4, ST_MAXNF = 8 };
constexpr int RG_NSTATUS = 16;


enum { OVF_NBR = 1, OVF_BOND = 2, OVF_HB = 4, OVF_CELL = 8 };

#define RG_C_ELE 332.06371   // Coulomb constant, kcal A / (mol e^2) (reaxc_defs_sunway.h:59)

// x^c for the reference's truncated cube-root exponents c = 0.3333333333333
// (QEq H, fix_qeq_reax_sw64.c:885) and 0.33333333333333 (Coulomb,
// reaxc_nonbonded_sw64.c:195): cbrt(x) * x^(c - 1/3), where the tiny second
// factor is 1 + (c - 1/3) ln x to far below an ulp (ln x in FP32 suffices).
#define RG_C3_QEQ (0.3333333333333 - 1.0 / 3.0)
#define RG_C3_ELE (0.33333333333333 - 1.0 / 3.0)
#ifdef __CUDACC__

// the p-th entry of a row with nn near entries (near entries first)
inline __host__ __device__ int nbr_slot(const Dev &d, int p, int nn) {
  return p < nn ? p : d.nb_capN + (p - nn);
}
// the clipped part sizes of atom i's row
__device__ __forceinline__ int nbr_near_count(const Dev &d, int i) {
  return min(d.n_near[i], d.nb_capN);
}
__device__ __forceinline__ int nbr_far_count(const Dev &d, int i) {
  return min(d.n_far[i], d.nb_cap - d.nb_capN);
}
// Per-atom item lists (bond slots, bond candidates) of the 32 atoms of a
// warp, taken 32 items at a time: lane l brings cnt items of its atom i, and
// f(i, c) runs for every item c < cnt of every lane's atom with the warp's
// lanes on consecutive items, so a short list does not leave lanes idle.
// Every lane of the warp must call it (cnt = 0 for lanes without an atom).
template <typename Fn>
__device__ __forceinline__ void warp_items(int cnt, int i, Fn f) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  int incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(full, incl, o);
    if (lane >= o) incl += v;
  }
  const int total = __shfl_sync(full, incl, 31);
  const int excl = incl - cnt;
  for (int base = 0; base < total; base += 32) {
    const int q = base + lane;
    // the owner of item q: the first lane whose inclusive count exceeds q
    int own = 0;
#pragma unroll
    for (int step = 16; step > 0; step >>= 1)
      if (__shfl_sync(full, incl, own + step - 1) <= q) own += step;
    const int oexcl = __shfl_sync(full, excl, own);
    const int oi = __shfl_sync(full, i, own);
    if (q < total) f(oi, q - oexcl);
  }
}

// The same with every lane calling f(has, i, k) in every batch (has: the
// lane holds an item), for bodies that use warp-wide collectives.
template <typename Fn>
__device__ __forceinline__ void warp_items_all(int cnt, int i, Fn f) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  int incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(full, incl, o);
    if (lane >= o) incl += v;
  }
  const int total = __shfl_sync(full, incl, 31);
  const int excl = incl - cnt;
  for (int base = 0; base < total; base += 32) {
    const int q = base + lane;
    int own = 0;
#pragma unroll
    for (int step = 16; step > 0; step >>= 1)
      if (__shfl_sync(full, incl, own + step - 1) <= q) own += step;
    const int oexcl = __shfl_sync(full, excl, own);
    const int oi = __shfl_sync(full, i, own);
    f(q < total, oi, q - oexcl);
  }
}

// The same over a subset of each atom's slots: bit k of mask marks slot k;
// f(i, k) runs for the marked slots only.
template <typename Fn>
__device__ __forceinline__ void warp_items_mask(unsigned mask, int i, Fn f) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int cnt = __popc(mask);
  int incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(full, incl, o);
    if (lane >= o) incl += v;
  }
  const int total = __shfl_sync(full, incl, 31);
  const int excl = incl - cnt;
  for (int base = 0; base < total; base += 32) {
    const int q = base + lane;
    int own = 0;
#pragma unroll
    for (int step = 16; step > 0; step >>= 1)
      if (__shfl_sync(full, incl, own + step - 1) <= q) own += step;
    const int oexcl = __shfl_sync(full, excl, own);
    const int oi = __shfl_sync(full, i, own);
    unsigned m = __shfl_sync(full, mask, own);
    if (q < total) {
      for (int c = q - oexcl; c > 0; --c) m &= m - 1;   // drop the lower marks
      f(oi, __ffs((int)m) - 1);
    }
  }
}

// Adds v[0..K) of every thread of the block into dst[seg * stride + c],
// c = 0..K-1; seg < 0 marks a thread without values.  One FP64 atomic per
// value per block when the block's threads belong to one segment, per warp
// when a warp's do, per thread otherwise (warps that straddle two
// segments).  Every thread of the block must call it.
template <int K>
__device__ __forceinline__ void seg_block_add(const double *vin, int seg, double *dst, int stride) {
  __shared__ double sh[K][32];
  __shared__ int sw[32];
  const unsigned FULLM = 0xffffffffu;
  double v[K];
#pragma unroll
  for (int c = 0; c < K; ++c) v[c] = vin[c];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  const bool uni = __match_any_sync(FULLM, seg) == FULLM;
  if (uni) {
#pragma unroll
    for (int c = 0; c < K; ++c)
      for (int off = 16; off > 0; off >>= 1) v[c] += __shfl_down_sync(FULLM, v[c], off);
  } else if (seg >= 0) {
#pragma unroll
    for (int c = 0; c < K; ++c)
      if (v[c] != 0.0) atomicAdd(&dst[(long long)seg * stride + c], v[c]);
  }
  __syncthreads();
  if (l == 0) {
    sw[w] = uni ? seg : -1;
#pragma unroll
    for (int c = 0; c < K; ++c) sh[c][w] = uni ? v[c] : 0.0;
  }
  __syncthreads();
  if (w == 0) {
    const int nw = (int)(blockDim.x >> 5);
    const int sg = l < nw ? sw[l] : -1;
    const int s0 = __shfl_sync(FULLM, sg, 0);
    const bool one = __all_sync(FULLM, l >= nw || sg == s0) && s0 >= 0;
#pragma unroll
    for (int c = 0; c < K; ++c) {
      double x = l < nw ? sh[c][l] : 0.0;
      if (one) {
        for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(FULLM, x, off);
        if (l == 0 && x != 0.0) atomicAdd(&dst[(long long)s0 * stride + c], x);
      } else if (l < nw && sg >= 0 && x != 0.0) {
        atomicAdd(&dst[(long long)sg * stride + c], x);
      }
    }
  }
}

// virial of one term: w -= d (x) g for an atom at displacement d from the
// term's reference atom receiving the energy gradient g (forces are -g; the
// gradients of a term sum to zero, so W = sum_atoms r (x) f needs only the
// displacements within the term, never the periodic images' absolute
// positions)
__device__ __forceinline__ void vir_acc(double *w, double dx, double dy, double dz, double gx,
                                        double gy, double gz) {
  w[0] -= dx * gx;
  w[1] -= dy * gy;
  w[2] -= dz * gz;
  w[3] -= dx * gy;
  w[4] -= dx * gz;
  w[5] -= dy * gz;
}

// Lattice translation sx a + sy b + sz c of a segment, rounded per
// operation in this order (the oracle builds its periodic images the same
// way); for an orthogonal box it is (sx lx, sy ly, sz lz) exactly.
__device__ __forceinline__ void img_vec(const SegGeom &g, int sx, int sy, int sz, double &vx,
                                        double &vy, double &vz) {
  vx = __dadd_rn(__dadd_rn(__dmul_rn((double)sx, g.L[0]), __dmul_rn((double)sy, g.tilt[0])),
                 __dmul_rn((double)sz, g.tilt[1]));
  vy = __dadd_rn(__dmul_rn((double)sy, g.L[1]), __dmul_rn((double)sz, g.tilt[2]));
  vz = __dmul_rn((double)sz, g.L[2]);
}

// s in [-2, 2] as a double, from its IEEE-754 bits (integer operations
// only: a conversion would occupy the FP64 pipe like an FMA)
__device__ __forceinline__ double small_int_d(int s) {
  const int a = s < 0 ? -s : s;
  unsigned hi = a == 0 ? 0u : (a == 1 ? 0x3FF00000u : 0x40000000u);
  if (s < 0) hi |= 0x80000000u;
  return __hiloint2double((int)hi, 0);
}

// exact displacement (x_j + image) - x_i of the membership tests.  For an
// orthogonal box x_j + s L is one FMA: s L is exact for |s| <= 2, so the
// FMA rounds the same sum as the reference's add, and s = 0 gives x_j
// unchanged; no branch on the image keeps the warp's lanes together.
__device__ __forceinline__ void disp64(const SegGeom &g, const double4 &xj, const double4 &xi,
                                       int sx, int sy, int sz, double &dx, double &dy,
                                       double &dz) {
  if (!g.tri) {
    dx = __dsub_rn(__fma_rn(small_int_d(sx), g.L[0], xj.x), xi.x);
    dy = __dsub_rn(__fma_rn(small_int_d(sy), g.L[1], xj.y), xi.y);
    dz = __dsub_rn(__fma_rn(small_int_d(sz), g.L[2], xj.z), xi.z);
  } else if (sx | sy | sz) {
    double vx, vy, vz;
    img_vec(g, sx, sy, sz, vx, vy, vz);
    dx = __dsub_rn(__dadd_rn(xj.x, vx), xi.x);
    dy = __dsub_rn(__dadd_rn(xj.y, vy), xi.y);
    dz = __dsub_rn(__dadd_rn(xj.z, vz), xi.z);
  } else {
    dx = __dsub_rn(xj.x, xi.x);
    dy = __dsub_rn(xj.y, xi.y);
    dz = __dsub_rn(xj.z, xi.z);
  }
}

// FP32 image shift for the distance prefilters (which carry a margin)
__device__ __forceinline__ void img_vec32(const SegGeom &g, int sx, int sy, int sz, float &vx,
                                          float &vy, float &vz) {
  vx = (float)sx * g.Lh[0];
  vy = (float)sy * g.Lh[1];
  vz = (float)sz * g.Lh[2];
  if (g.tri) {
    vx += (float)sy * g.Th[0] + (float)sz * g.Th[1];
    vy += (float)sz * g.Th[2];
  }
}

// Mixed form: displacement x_j + s L - x_i from positions and box edges
// held as FP32 (hi, lo) pairs.  The hi parts combine first (exact or
// rounded once at the result's magnitude), so the error is a few FP32 ulps
// of the displacement itself, not of the coordinates.
__device__ __forceinline__ float df_disp(float hj, float lj, float hi, float li, int s, float Lh,
                                         float Ll) {
  const float a = __fsub_rn(__fmaf_rn((float)s, Lh, hj), hi);
  const float b = __fsub_rn(__fmaf_rn((float)s, Ll, lj), li);
  return __fadd_rn(a, b);
}

// the same with a shift given as an FP32 pair (triclinic images)
__device__ __forceinline__ float df_disp2(float hj, float lj, float hi, float li, float vh,
                                          float vl) {
  const float a = __fsub_rn(__fadd_rn(hj, vh), hi);
  const float b = __fsub_rn(__fadd_rn(lj, vl), li);
  return __fadd_rn(a, b);
}

// Unevaluated FP32 pairs (value = hi + lo) for the FP64 form's tabulated
// pair functions: positions, charges and table coefficients are exact FP32
// pairs (to ~2^-48), and the operations below keep ~2^-46 relative (of the
// operands' magnitudes) on the FP32 units, where GB300's FP64 rate is 1/64
// of FP32.  Explicitly rounded: no contraction may change them.
struct fpair {
  float hi, lo;
};

// Knuth's TwoSum: hi + lo = a + b exactly
__device__ __forceinline__ fpair fp_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

// the same for |a| >= |b| (Dekker)
__device__ __forceinline__ fpair fp_fast(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ fpair fp_add(fpair a, fpair b) {
  const fpair s = fp_two_sum(a.hi, b.hi);
  return fp_fast(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ fpair fp_mul(fpair a, fpair b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return fp_fast(p, e);
}

__device__ __forceinline__ fpair fp_sqr(fpair a) {
  const float p = __fmul_rn(a.hi, a.hi);
  float e = __fmaf_rn(a.hi, a.hi, -p);
  e = __fmaf_rn(__fadd_rn(a.hi, a.hi), a.lo, e);
  return fp_fast(p, e);
}

__device__ __forceinline__ double fp_to_double(fpair a) {
  return __dadd_rn((double)a.hi, (double)a.lo);
}

// (x_j + s L) - x_i of one coordinate from (hi, lo) positions and the box
// edge L = Lh + Ll of an orthogonal segment (s Lh and s Ll are exact for
// |s| <= 2)
__device__ __forceinline__ fpair fp_disp(float hj, float lj, float hi, float li, int s, float Lh,
                                         float Ll) {
  const float sf = (float)s;
  const fpair a = fp_two_sum(hj, __fmul_rn(sf, Lh));
  const fpair b = fp_two_sum(a.hi, -hi);
  const float lo = __fadd_rn(__fadd_rn(__fsub_rn(lj, li), __fadd_rn(a.lo, b.lo)), __fmul_rn(sf, Ll));
  return fp_fast(b.hi, lo);
}

// r^2 of a pair of an orthogonal segment as an FP32 pair
__device__ __forceinline__ fpair fp_d2(const SegGeom &g, const float4 &hj, const float4 &lj,
                                       const float4 &hi, const float4 &li, int sx, int sy, int sz) {
  const fpair dx = fp_disp(hj.x, lj.x, hi.x, li.x, sx, g.Lh[0], g.Ll[0]);
  const fpair dy = fp_disp(hj.y, lj.y, hi.y, li.y, sy, g.Lh[1], g.Ll[1]);
  const fpair dz = fp_disp(hj.z, lj.z, hi.z, li.z, sz, g.Lh[2], g.Ll[2]);
  return fp_add(fp_add(fp_sqr(dx), fp_sqr(dy)), fp_sqr(dz));
}

// table interval k and offset u in [0, 1] of s = r^2 >= tab_s0 (the FP64
// tables' intervals)
__device__ __forceinline__ void fp_interval(const Control &C, fpair s2, int &k, fpair &u) {
  const fpair x = fp_add(fp_mul(s2, {C.tab_inv_ds_f, C.tab_inv_ds_l}), {C.tab_x0_f, C.tab_x0_l});
  int kk = (int)x.hi;
  if ((float)kk == x.hi && x.lo < 0.f) --kk;
  kk = min(max(kk, 0), C.tab_n - 1);
  k = kk;
  u = fp_fast(__fsub_rn(x.hi, (float)kk), x.lo);
}

// c0 + u (c1 + u (c2 + u c3)) with the coefficients as FP32 pairs
// (c01 = c0.hi, c0.lo, c1.hi, c1.lo; c23 likewise)
__device__ __forceinline__ fpair fp_cubic(const float4 &c01, const float4 &c23, fpair u) {
  fpair h = {c23.z, c23.w};
  h = fp_add(fp_mul(h, u), {c23.x, c23.y});
  h = fp_add(fp_mul(h, u), {c01.z, c01.w});
  return fp_add(fp_mul(h, u), {c01.x, c01.y});
}

// mixed-form displacement (x_j + image) - x_i; a triclinic image is formed
// in FP64 and split into an FP32 pair
__device__ __forceinline__ void disp32(const SegGeom &g, const float4 &hj, const float4 &lj,
                                       const float4 &hi, const float4 &li, int sx, int sy,
                                       int sz, float &ex, float &ey, float &ez) {
  if (!g.tri || !(sx | sy | sz)) {
    ex = df_disp(hj.x, lj.x, hi.x, li.x, sx, g.Lh[0], g.Ll[0]);
    ey = df_disp(hj.y, lj.y, hi.y, li.y, sy, g.Lh[1], g.Ll[1]);
    ez = df_disp(hj.z, lj.z, hi.z, li.z, sz, g.Lh[2], g.Ll[2]);
  } else {
    double vx, vy, vz;
    img_vec(g, sx, sy, sz, vx, vy, vz);
    const float hx = __double2float_rn(vx), hy = __double2float_rn(vy), hz = __double2float_rn(vz);
    ex = df_disp2(hj.x, lj.x, hi.x, li.x, hx, __double2float_rn(vx - (double)hx));
    ey = df_disp2(hj.y, lj.y, hi.y, li.y, hy, __double2float_rn(vy - (double)hy));
    ez = df_disp2(hj.z, lj.z, hi.z, li.z, hz, __double2float_rn(vz - (double)hz));
  }
}

// fractional coordinates of a position in a triclinic segment by
// back-substitution (no precomputed inverse), rounded per operation
__device__ __forceinline__ void frac3(const SegGeom &g, double x, double y, double z, double &u,
                                      double &v, double &w) {
  w = __ddiv_rn(z, g.L[2]);
  v = __ddiv_rn(__dsub_rn(y, __dmul_rn(w, g.tilt[2])), g.L[1]);
  u = __ddiv_rn(__dsub_rn(__dsub_rn(x, __dmul_rn(v, g.tilt[0])), __dmul_rn(w, g.tilt[1])), g.L[0]);
}

// x^c for the exponents above: cbrt(x) (1 + (c - 1/3) ln x)
__device__ __forceinline__ double pow_third(double x, double dc) {
  return cbrt(x) * (1.0 + dc * (double)__logf((float)x));
}
// 1 / x^c for the same exponents
__device__ __forceinline__ double rpow_third(double x, double dc) {
  return rcbrt(x) * (1.0 - dc * (double)__logf((float)x));
}
#endif

// image code of a neighbour entry: sx,sy,sz in [-2,2]
__host__ __device__ inline int img_pack(int sx, int sy, int sz) {
  return (sx + 2) + 5 * (sy + 2) + 25 * (sz + 2);
}
__host__ __device__ inline void img_unpack(int c, int *sx, int *sy, int *sz) {
  *sx = c % 5 - 2;
  *sy = (c / 5) % 5 - 2;
  *sz = c / 25 - 2;
}

// kernel launchers (lists.cu, bonded.cu, nonbonded.cu, qeq.cu, nve.cu)
void launch_bin_sort(const Dev &d, cudaStream_t st);
void launch_build_nbrs(const Dev &d, cudaStream_t st);
void launch_build_bonds(const Dev &d, cudaStream_t st);
void launch_count(const Dev &d, cudaStream_t st);
void launch_bond_orders(const Dev &d, cudaStream_t st);
void launch_atom_energy(const Dev &d, cudaStream_t st, int eflag);
void launch_hbonds(const Dev &d, cudaStream_t st, int eflag);
// work-list form: prep + count (then the host reads the totals), fill + run
void launch_vt_count(const Dev &d, cudaStream_t st);
void launch_vt_run(const Dev &d, cudaStream_t st, int eflag, long long nval, long long ntor,
                   bool device_counts = false);
void launch_scan(const int *in, int *out, int n, int *bsum, cudaStream_t st);
void launch_nonbonded(const Dev &d, cudaStream_t st, int eflag);
void launch_dbond_forces(const Dev &d, cudaStream_t st);
void launch_force_out(const Dev &d, cudaStream_t st);
void launch_check_finite(const double *a, long long count, int *flag, cudaStream_t st);

// QEq
void launch_qeq_setup(const Dev &d, cudaStream_t st);
void launch_qeq_spmv(const Dev &d, cudaStream_t st, const double2 *x, double2 *y, int use_act);
void launch_qeq_cg_init(const Dev &d, cudaStream_t st, double tol, int imax);
void launch_qeq_refine_check(const Dev &d, cudaStream_t st, double tol);
void launch_qeq_cg_init_rest(const Dev &d, cudaStream_t st, double tol, int imax);
void launch_qeq_cg_A(const Dev &d, cudaStream_t st);
void launch_qeq_cg_C(const Dev &d, cudaStream_t st);
void launch_qeq_finish(const Dev &d, cudaStream_t st);
// the captured step's QEq control (qeq.cu): set_cond sets the graph
// conditions c1 (and c2 if nonzero) to "a segment is active"; loop_cond ends
// a CG loop trip: its condition stays set while a segment is active and the
// trips stay within the limit; tot adds the pass's iterations per segment
// (less the set-up iteration after the first pass); restart counts a
// refinement restart
void launch_qeq_set_cond(const Dev &d, cudaStream_t st, unsigned long long c1,
                         unsigned long long c2);
void launch_qeq_loop_cond(const Dev &d, cudaStream_t st, unsigned long long c, int limit);
void launch_qeq_tot(const Dev &d, cudaStream_t st, int pass);
void launch_qeq_restart_count(const Dev &d, cudaStream_t st);

// NVE
void launch_nve_initial(const Dev &d, cudaStream_t st, double dt);
void launch_nve_final(const Dev &d, cudaStream_t st, double dt);

// generic
void launch_zero(void *p, size_t bytes, cudaStream_t st);

// accessors used by noalloc.cu (the handle type is private to reaxgpu.cu)
struct rg_system;
void rg_set_error(rg_system *h, const std::string &msg);
void rg_noalloc_tables(const rg_system *h, const ForceField **ff, const Control **ctl,
                       int *device, double *swb, double *tol, int *imax);

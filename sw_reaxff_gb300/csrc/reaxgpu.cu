// Host side of the reaxgpu C ABI (include/reaxgpu.h): handle management,
// device memory, list capacity growth and the per-step orchestration of the
// kernels in lists.cu, bonded.cu, nonbonded.cu, qeq.cu and nve.cu.
//
// The step order follows PairReaxCSunway::compute (pair_reaxc_sunway.cpp:
// 541-793) / Compute_Forces (reaxc_forces_sunway.cpp:1297-1365): lists ->
// bond orders -> bonded terms (bond/lp/ov/un, H-bonds, valence+torsion) ->
// nonbonded -> dBond force assembly -> force copy-out; QEq
// (FixQEqReaxSunway::pre_force) runs before it on the same pair list.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/reaxgpu.h"
#include "rg_internal.h"

// Phase timer: CUDA events recorded on the handle's stream around each
// kernel group; intervals are resolved lazily (after a stream sync).
enum {
  PH_BIN = 0, PH_NBR, PH_BOND, PH_BO, PH_ATOM, PH_HB, PH_VALTOR, PH_NONB, PH_DBOND,
  PH_FOUT, PH_QSETUP, PH_QSPMV, PH_QVEC, PH_QFIN, PH_NVE, PH_N
};
static const char *kPhaseNames[PH_N] = {
    "bin_sort", "pair_list+H", "bond_list", "bond_orders", "atom_energy", "hbonds",
    "valence_torsion", "nonbonded", "dbond_forces", "force_out", "qeq_setup",
    "qeq_spmv", "qeq_vector", "qeq_finish", "nve"};

struct Prof {
  bool on = false;
  unsigned mask = ~0u;       // phases that get events (bit k: phase k)
  std::vector<cudaEvent_t> pool;
  std::vector<int> phase;   // phase of each recorded event (-1 = gap)
  size_t used = 0;
  double ms[PH_N] = {0};
  long long cnt[PH_N] = {0};
  void mark(cudaStream_t st, int ph) {
    if (!on) return;
    if (used == pool.size()) {
      if (used >= 4096) resolve();
      if (used == pool.size()) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        pool.push_back(e);
        phase.push_back(-1);
      }
    }
    cudaEventRecord(pool[used], st);
    phase[used] = ph;
    ++used;
  }
  void resolve() {
    if (used == 0) return;
    cudaEventSynchronize(pool[used - 1]);
    for (size_t k = 0; k + 1 < used; ++k) {
      if (phase[k] < 0) continue;
      float t = 0.f;
      cudaEventElapsedTime(&t, pool[k], pool[k + 1]);
      ms[phase[k]] += t;
      cnt[phase[k]] += 1;
    }
    used = 0;
  }
  void reset() {
    used = 0;
    for (int k = 0; k < PH_N; ++k) ms[k] = 0, cnt[k] = 0;
  }
  ~Prof() {
    for (auto e : pool) cudaEventDestroy(e);
  }
};

// one captured step (see rg_single_point / rg_run)
struct StepGraph {
  cudaGraphExec_t exec = nullptr;
  Dev dev{};                        // the device arrays and sizes it holds
  int flags = -1;                   // eflag | vflag << 4 | tallies << 8
  double dt = 0.0;                  // MD step: the time step (0: single point)
  long long kernels = 0;            // top-level kernel nodes of one replay
  bool failed = false;              // a capture failed: the regular path only
  Dev seen{};                       // the previous regular step's arrays,
  int seen_flags = -1;              // flags and time step: a repeat of them
  double seen_dt = -1.0;            // is captured
};

struct rg_system {
  rg_params p{};
  ForceField ff{};
  Control ctl{};
  ForceField *d_ff = nullptr;
  Control *d_ctl = nullptr;
  double *d_tab = nullptr;        // FP64 tables (nb then H)
  float *d_tab32 = nullptr;       // FP32 tables: the mixed form's nb table, or the FP64
                                  // form's nb and H tables as FP32 pairs
  double tab_err = 0.0;
  cudaStream_t st = nullptr;
  std::string err;
  int n = 0;
  bool have_box = false;
  // segments: host table, atoms per segment (-1: all atoms of a single
  // segment), allocations sized by the segment count
  std::vector<SegGeom> segs;
  std::vector<int> seg_counts;
  std::vector<void *> per_seg;
  int nseg_alloc = 0;
  int n_cap = 0;                  // atoms the per-atom arrays and lists hold
  std::vector<double> e_host;     // per-segment energies read back
  std::vector<int> seg_iters;     // last QEq: s and t iterations per segment
  Dev d{};
  std::vector<void *> per_n;    // allocations sized by n
  std::vector<void *> per_nb;   // sized by n * nb_cap
  std::vector<void *> per_b;    // sized by n * bond_cap
  std::vector<void *> per_hb;   // sized by n * hb_cap
  std::vector<void *> per_items;  // valence / torsion work items
  void *cells = nullptr;
  int ncell_alloc = 0;
  bool lists_valid = false;
  // the force step corrects the bond orders and accumulates Cdbo in the bond
  // arrays in place: a second force step on the same lists needs them built
  // again
  bool bonds_fresh = false;
  bool forces_valid = false;
  bool tallies_valid = false;   // per-atom tallies of the last force step
  // autotuned configuration: cells of cutoff/cell_div (2 or 3) and the SpMV
  // lanes per row (d.spmv_rw); tuned_n = atom count it was tuned for
  int cell_div = 2;
  int tuned_n = 0;
  bool tuning = false;
  // RG_CHECK_FINITE=1: test the force/CdDelta accumulators after every
  // force phase and name the first phase that produced a non-finite value
  bool check_finite = false;
  // the CG iterations of a poll interval as one captured CUDA graph,
  // replayed while any system's solve is active; recaptured whenever the
  // device arrays or sizes change (RG_NO_GRAPHS=1: plain launches)
  cudaGraphExec_t cg_exec = nullptr;
  Dev cg_dev{};
  bool use_graphs = true;
  // the whole single-point step (lists, QEq with device-side loops, force
  // step; rg_single_point) and the whole MD step (the same between the two
  // Verlet half-steps; rg_run) as captured graphs, recaptured when the
  // device arrays, sizes, flags or time step change; streams for the
  // conditional bodies
  StepGraph sp, md;
  int sp_trip = 4;                  // CG iterations per device-side loop trip
  cudaStream_t cap_st[8] = {nullptr};
  rg_stats stats{};
  double energy[RG_NE] = {0};
  Prof prof;
  long long launches = 0;   // kernels of this library launched so far
  long long n_val = 0, n_tor = 0;   // valence angles / torsions of the last step
};

namespace {

struct Scope {
  rg_system *h;
  bool timed;
  Scope(rg_system *hh, int ph, int kernels) : h(hh), timed((hh->prof.mask >> ph) & 1u) {
    if (timed) h->prof.mark(h->st, ph);
    h->launches += kernels;
  }
  ~Scope() {
    if (timed) h->prof.mark(h->st, -1);
  }
};

// the CG iterations run as plain launches only when their phases are timed
constexpr unsigned kCgPhases = (1u << PH_QSPMV) | (1u << PH_QVEC);

int fail(rg_system *h, int code, const std::string &msg) {
  if (h) h->err = msg;
  return code;
}

#define CK(call)                                                              \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess)                                                    \
      return fail(h, RG_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <class T>
int dalloc(rg_system *h, std::vector<void *> &bucket, T **p, size_t count) {
  void *q = nullptr;
  cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
  if (e != cudaSuccess) {
    cudaGetLastError();   // not sticky: keep it from surfacing in a later call
    return fail(h, RG_E_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  bucket.push_back(q);
  *p = (T *)q;
  return 0;
}

void free_bucket(std::vector<void *> &b) {
  for (void *p : b) cudaFree(p);
  b.clear();
}

double list_cutoff(const rg_system *h) {
  return std::max(h->ctl.nonb_cut, h->p.qeq_swb);
}

// widths of a segment's cell between opposite faces: the box edges, or for
// a triclinic cell V / |b x c|, V / |c x a|, V / |a x b|
void cell_widths(const SegGeom &g, double *w) {
  const double lx = g.L[0], ly = g.L[1], lz = g.L[2];
  const double xy = g.tilt[0], xz = g.tilt[1], yz = g.tilt[2];
  w[0] = lx; w[1] = ly; w[2] = lz;
  if (xy != 0.0 || xz != 0.0 || yz != 0.0) {
    const double V = lx * ly * lz;
    w[0] = V / std::sqrt(ly * lz * ly * lz + xy * lz * xy * lz +
                         (xy * yz - ly * xz) * (xy * yz - ly * xz));
    w[1] = ly * lz / std::sqrt(lz * lz + yz * yz);
  }
}

// cells of cutoff/3 (stencil +-3) only where every width is at least the
// cutoff: then a partner is at most one image away and the 5x5x5 image
// codes hold
bool div3_ok(const rg_system *h) {
  const double rc = list_cutoff(h);
  for (const SegGeom &g : h->segs) {
    double w[3];
    cell_widths(g, w);
    if (w[0] < rc || w[1] < rc || w[2] < rc) return false;
  }
  return true;
}

int setup_cells(rg_system *h) {
  const double rc = list_cutoff(h);
  const int S = (h->cell_div == 3 && div3_ok(h)) ? 3 : 2;
  Dev &d = h->d;
  long long ncell = 0;
  for (SegGeom &g : h->segs) {
    g.S = S;
    g.tri = (g.tilt[0] != 0.0 || g.tilt[1] != 0.0 || g.tilt[2] != 0.0);
    // cells (in fractional coordinates when triclinic) at least rc/S wide
    // across make the +-S stencil reach every partner within rc
    double w[3];
    cell_widths(g, w);
    long long nseg_cells = 1;
    for (int k = 0; k < 3; ++k) {
      g.Lh[k] = (float)g.L[k];
      g.Ll[k] = (float)(g.L[k] - (double)g.Lh[k]);
      g.Th[k] = (float)g.tilt[k];
      if (w[k] < rc / S)
        return fail(h, RG_E_ARG, "box width shorter than half the pair cutoff is not supported");
      int nc = (int)std::floor(w[k] * S / (rc * (1.0 + 1e-9)));
      nc = std::max(nc, 1);
      g.nc[k] = nc;
      g.cellw[k] = g.L[k] / nc;
      g.cellw_f[k] = (float)g.cellw[k];
      nseg_cells *= nc;
    }
    g.cell0 = (int)ncell;
    ncell += nseg_cells;
    if (ncell > (1LL << 26)) return fail(h, RG_E_ARG, "too many cells");
  }
  d.ncell = (int)ncell;
  CK(cudaMemcpyAsync((void *)d.seg, h->segs.data(), sizeof(SegGeom) * h->segs.size(),
                     cudaMemcpyHostToDevice, h->st));
  if (ncell > h->ncell_alloc) {
    if (h->cells) cudaFree(h->cells);
    const size_t nb = (ncell + 1 + 1023) / 1024 + 1;
    // count | start | fill + block sums
    CK(cudaMalloc(&h->cells, sizeof(int) * (3 * (ncell + 1) + nb)));
    h->ncell_alloc = (int)ncell;
  }
  int *c = (int *)h->cells;
  d.cell_count = c;
  d.cell_start = c + (ncell + 1);
  d.cell_fill = c + 2 * (ncell + 1);
  CK(cudaStreamSynchronize(h->st));   // the host table may change after return
  return 0;
}

// arrays sized by the segment count: geometry table, QEq scalars, energies
int alloc_segs(rg_system *h) {
  const int ns = (int)h->segs.size();
  Dev &d = h->d;
  d.nseg = ns;
  if (ns <= h->nseg_alloc) return 0;
  free_bucket(h->per_seg);
  const int cap = ns == 1 ? 1 : ns + ns / 2;
  int r = 0;
  SegGeom *sg = nullptr;
  r |= dalloc(h, h->per_seg, &sg, (size_t)cap);
  d.seg = sg;
  r |= dalloc(h, h->per_seg, &d.red, (size_t)cap * RG_NRED);
  r |= dalloc(h, h->per_seg, &d.energy, (size_t)cap * RG_NE);
  r |= dalloc(h, h->per_seg, &d.virial, (size_t)cap * 6);
  r |= dalloc(h, h->per_seg, &d.n_active, 1);
  r |= dalloc(h, h->per_seg, &d.qeq_ctl, 4);
  r |= dalloc(h, h->per_seg, &d.qeq_tot, 2 * (size_t)cap);
  if (r) return RG_E_CUDA;
  h->nseg_alloc = cap;
  return 0;
}

int alloc_bonds(rg_system *h) {
  free_bucket(h->per_b);
  Dev &d = h->d;
  const size_t S = (size_t)h->n_cap * d.bond_cap;
  int r = 0;
  r |= dalloc(h, h->per_b, &d.b_nbr, S);
  r |= dalloc(h, h->per_b, &d.b_sym, S);
  r |= dalloc(h, h->per_b, &d.b_d, S);
  r |= dalloc(h, h->per_b, &d.b_dx, S);
  r |= dalloc(h, h->per_b, &d.b_dy, S);
  r |= dalloc(h, h->per_b, &d.b_dz, S);
  r |= dalloc(h, h->per_b, &d.b_BO, S);
  r |= dalloc(h, h->per_b, &d.b_BOs, S);
  r |= dalloc(h, h->per_b, &d.b_BOpi, S);
  r |= dalloc(h, h->per_b, &d.b_BOpi2, S);
  r |= dalloc(h, h->per_b, &d.b_dBOp, 3 * S);
  r |= dalloc(h, h->per_b, &d.b_dlnpi, 3 * S);
  r |= dalloc(h, h->per_b, &d.b_dlnpi2, 3 * S);
  r |= dalloc(h, h->per_b, &d.b_C, 11 * S);
  r |= dalloc(h, h->per_b, &d.b_Cdbo, S);
  r |= dalloc(h, h->per_b, &d.b_Cdbopi, S);
  r |= dalloc(h, h->per_b, &d.b_Cdbopi2, S);
  r |= dalloc(h, h->per_b, &d.b_et2, S);
  r |= dalloc(h, h->per_b, &d.b_ec2, S);
  r |= dalloc(h, h->per_b, &d.b_vexp, 3 * S);
  r |= dalloc(h, h->per_b, &d.b_BOf, S);
  r |= dalloc(h, h->per_b, &d.w_cnt_v, S + 1);
  r |= dalloc(h, h->per_b, &d.w_cnt_t, S + 1);
  r |= dalloc(h, h->per_b, &d.w_off_v, S + 1);
  r |= dalloc(h, h->per_b, &d.w_off_t, S + 1);
  r |= dalloc(h, h->per_b, &d.w_bsum, (S + 1 + 1023) / 1024 + 1);
  return r;
}

int alloc_items(rg_system *h, long long nval, long long ntor) {
  free_bucket(h->per_items);
  Dev &d = h->d;
  d.cap_val = nval;
  d.cap_tor = ntor;
  int r = 0;
  r |= dalloc(h, h->per_items, &d.w_val, (size_t)nval);
  r |= dalloc(h, h->per_items, &d.w_tor, (size_t)ntor);
  if (d.mixed) {
    r |= dalloc(h, h->per_items, &d.w_fb_val, (size_t)nval);
    r |= dalloc(h, h->per_items, &d.w_fb_tor, (size_t)ntor);
  } else {
    d.w_fb_val = d.w_fb_tor = nullptr;
  }
  return r;
}

int alloc_nbrs(rg_system *h) {
  free_bucket(h->per_nb);
  Dev &d = h->d;
  const size_t S = (size_t)h->n_cap * d.nb_cap;
  int r = 0;
  r |= dalloc(h, h->per_nb, &d.nbr, S);
  if (d.mixed) {
    r |= dalloc(h, h->per_nb, &d.hval32, S);
    d.hvalp = nullptr;
  } else {
    r |= dalloc(h, h->per_nb, &d.hvalp, S);
    d.hval32 = nullptr;
  }
  return r;
}

int alloc_hb(rg_system *h) {
  free_bucket(h->per_hb);
  Dev &d = h->d;
  return dalloc(h, h->per_hb, &d.hb_nbr, (size_t)h->n_cap * d.hb_cap);
}

// Per-atom arrays and the lists sized for n_cap >= n atoms.  A handle whose
// atom count shrinks (or grows within its capacity) keeps its arrays: no
// cudaFree, which would wait for other streams' work, on the way.
int alloc_atoms(rg_system *h, int n) {
  Dev &d = h->d;
  if (n <= h->n_cap) {
    d.n = n;
    return 0;
  }
  free_bucket(h->per_n);
  h->n_cap = n;
  d.n = n;
  int r = 0;
  auto &B = h->per_n;
  r |= dalloc(h, B, &d.x_o, 3 * (size_t)n);
  r |= dalloc(h, B, &d.v_o, 3 * (size_t)n);
  r |= dalloc(h, B, &d.q_o, (size_t)n);
  r |= dalloc(h, B, &d.f_o, 3 * (size_t)n);
  r |= dalloc(h, B, &d.type_o, (size_t)n);
  r |= dalloc(h, B, &d.tag_o, (size_t)n);
  r |= dalloc(h, B, &d.s_hist, 5 * (size_t)n);
  r |= dalloc(h, B, &d.t_hist, 5 * (size_t)n);
  r |= dalloc(h, B, &d.cell_o, (size_t)n);
  r |= dalloc(h, B, &d.perm, (size_t)n);
  r |= dalloc(h, B, &d.iperm, (size_t)n);
  r |= dalloc(h, B, &d.hist_save, 19 * (size_t)n);
  r |= dalloc(h, B, &d.eatom, (size_t)n);
  r |= dalloc(h, B, &d.vatom, 6 * (size_t)n);
  r |= dalloc(h, B, &d.xs, (size_t)n);
  r |= dalloc(h, B, &d.xf, (size_t)n);
  r |= dalloc(h, B, &d.xl, (size_t)n);
  r |= dalloc(h, B, &d.qlo, (size_t)n);
  r |= dalloc(h, B, &d.ts, (size_t)n);
  r |= dalloc(h, B, &d.tags, (size_t)n);
  r |= dalloc(h, B, &d.n_near, (size_t)n);
  r |= dalloc(h, B, &d.n_far, (size_t)n);
  r |= dalloc(h, B, &d.nbonds, (size_t)n);
  r |= dalloc(h, B, &d.nhb, (size_t)n);
  double **pd[] = {&d.bo0, &d.Deltap, &d.Deltap_boc, &d.Delta, &d.Delta_e, &d.Delta_boc,
                   &d.Delta_val, &d.vlpex, &d.nlp, &d.Delta_lp, &d.Delta_lp_temp,
                   &d.dDelta_lp, &d.nlp_temp, &d.Hdia_inv};
  for (double **q : pd) r |= dalloc(h, B, q, (size_t)n);
  r |= dalloc(h, B, &d.dDeltap, 3 * (size_t)n);
  r |= dalloc(h, B, &d.fC, 4 * (size_t)n);
  r |= dalloc(h, B, &d.vsum, 2 * (size_t)n);
  r |= dalloc(h, B, &d.exp_boc, 2 * (size_t)n);
  r |= dalloc(h, B, &d.c_sbo, 10 * (size_t)n);
  double2 **pv[] = {&d.qx, &d.qb, &d.qr, &d.qu, &d.qd, &d.qq};
  for (double2 **q : pv) r |= dalloc(h, B, q, (size_t)n);
  r |= dalloc(h, B, &d.qd32, (size_t)n);
  if (d.mixed) r |= dalloc(h, B, &d.fC32, 3 * (size_t)n);
  else d.fC32 = nullptr;
  r |= dalloc(h, B, &d.seg_o, (size_t)n);
  r |= dalloc(h, B, &d.seg_s, (size_t)n);
  r |= dalloc(h, B, &d.status, RG_NSTATUS);
  r |= dalloc(h, B, &d.dbg_flag, 1);
  r |= dalloc(h, B, &d.dbg, 40);
  r |= dalloc(h, B, &d.fb_cnt, 2);
  if (r) return RG_E_CUDA;
  // capacity estimates from the mean density
  double vol = 0.0;
  for (const SegGeom &g : h->segs) vol += g.L[0] * g.L[1] * g.L[2];
  // (bounded: a liquid's density where no volume is known, and at most a
  // few times the densest condensed phases; the build regrows anyway)
  const double rho = vol > 0.0 ? std::min(n / vol, 0.5) : 0.12;
  const double rc = list_cutoff(h);
  const double pi = 3.14159265358979;
  // rows: near part (d <= near_cut) and far part, each 1.6x its mean count
  const double nc = std::min(std::max(h->ctl.near_cut, 1.0), rc);
  int nbN = (int)(1.6 * 4.0 / 3.0 * pi * nc * nc * nc * rho) + 32;
  int nbF = (int)(1.6 * 4.0 / 3.0 * pi * (rc * rc * rc - nc * nc * nc) * rho) + 32;
  nbN = (nbN + 31) / 32 * 32;
  nbF = (nbF + 31) / 32 * 32;
  d.nb_capN = nbN;
  d.nb_cap = nbN + nbF;
  d.bond_cap = 16;
  const double hc = std::max(h->ctl.hbond_cut, 1.0);
  d.hb_cap = (int)(1.6 * 4.0 / 3.0 * pi * hc * hc * hc * rho) + 32;
  r |= alloc_nbrs(h);
  r |= alloc_bonds(h);
  r |= alloc_hb(h);
  r |= alloc_items(h, (long long)n * 16 + 1024, (long long)n * 24 + 1024);
  return r ? RG_E_CUDA : 0;
}

int read_status(rg_system *h, int *st) {
  CK(cudaMemcpyAsync(st, h->d.status, RG_NSTATUS * sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return 0;
}

int build_lists(rg_system *h);

// The autotuner: on the system at hand, the pair-list build (bin sort +
// pair list, the FP32 candidate walk depends on the cell size) with cells
// of cutoff/2 and cutoff/3, and the QEq SpMV with 8, 16 and 32 lanes per
// row, each timed with CUDA events; the fastest stays.  Results are the
// same up to the order of floating-point sums.
int autotune(rg_system *h) {
  Dev &d = h->d;
  h->tuning = true;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  auto timed = [&](auto &&work, int reps, float &ms) -> int {
    CK(cudaEventRecord(e0, h->st));
    for (int r = 0; r < reps; ++r) work();
    CK(cudaEventRecord(e1, h->st));
    CK(cudaEventSynchronize(e1));
    CK(cudaEventElapsedTime(&ms, e0, e1));
    ms /= reps;
    return 0;
  };
  int rc = 0;
  float best = 1e30f;
  int best_div = h->p.cell_div ? h->p.cell_div : 2;
  int best_tiles = h->p.pair_kernel == 2 ? 1 : 0;
  const bool tune_div = !h->p.cell_div, tune_kernel = !h->p.pair_kernel;
  if (tune_div || tune_kernel) {
    for (int div : {2, 3}) {
      if (!tune_div && div != h->p.cell_div) continue;
      if (div == 3 && !div3_ok(h)) continue;
      h->cell_div = div;
      for (int tiles : {0, 1}) {
        if (!tune_kernel && tiles != best_tiles) continue;
        d.nbr_tiles = tiles;
        if ((rc = build_lists(h))) break;   // capacities for this configuration
        float ms = 0.f;
        if ((rc = timed([&] { launch_bin_sort(d, h->st); launch_build_nbrs(d, h->st); }, 2, ms)))
          break;
        if (ms < best) best = ms, best_div = div, best_tiles = tiles;
      }
      if (rc) break;
    }
  }
  h->cell_div = best_div;
  d.nbr_tiles = best_tiles;
  if (!rc) rc = build_lists(h);
  if (!rc && !h->p.spmv_rows) {
    // SpMV lanes per row on the list just built (a zero vector: timing only)
    CK(cudaMemsetAsync(d.qd, 0, sizeof(double2) * (size_t)d.n, h->st));
    if (d.qd32) CK(cudaMemsetAsync(d.qd32, 0, sizeof(float4) * (size_t)d.n, h->st));
    best = 1e30f;
    int best_rw = 16;
    for (int rw : {8, 16, 32}) {
      d.spmv_rw = rw;
      float ms = 0.f;
      if ((rc = timed([&] { launch_qeq_spmv(d, h->st, d.qd, d.qq, 0); }, 3, ms))) break;
      if (ms < best) best = ms, best_rw = rw;
    }
    d.spmv_rw = best_rw;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  h->tuned_n = d.n;
  h->tuning = false;
  return rc;
}

int build_lists(rg_system *h) {
  Dev &d = h->d;
  if (!d.n) return fail(h, RG_E_STATE, "no atoms set");
  if (h->p.autotune && !h->tuning &&
      (h->tuned_n == 0 || d.n > 4 * h->tuned_n || 4 * d.n < h->tuned_n)) {
    int r = autotune(h);
    if (r) return r;
    return 0;   // autotune left the lists of the chosen configuration
  }
  int rc = setup_cells(h);
  if (rc) return rc;
  CK(cudaMemsetAsync(d.status, 0, RG_NSTATUS * sizeof(int), h->st));
  {
    Scope sc(h, PH_BIN, 7);
    launch_bin_sort(d, h->st);
  }
  int st[RG_NSTATUS];
  for (int attempt = 0;; ++attempt) {
    {
      Scope sc(h, PH_NBR, 1);
      launch_build_nbrs(d, h->st);
    }
    if ((rc = read_status(h, st))) return rc;
    if (!(st[ST_OVF] & OVF_NBR)) break;
    if (attempt > 3) return fail(h, RG_E_CAPACITY, "pair list capacity");
    const int capN = std::max(d.nb_capN, (int)(st[ST_MAXNB] * 1.2) / 32 * 32 + 32);
    const int capF = std::max(d.nb_cap - d.nb_capN, (int)(st[ST_MAXNF] * 1.2) / 32 * 32 + 32);
    d.nb_capN = capN;
    d.nb_cap = capN + capF;
    h->stats.regrows++;
    if ((rc = alloc_nbrs(h))) return rc;
    CK(cudaMemsetAsync(d.status, 0, RG_NSTATUS * sizeof(int), h->st));
  }
  for (int attempt = 0;; ++attempt) {
    {
      Scope sc(h, PH_BOND, 3);
      launch_build_bonds(d, h->st);
      launch_count(d, h->st);
    }
    if ((rc = read_status(h, st))) return rc;
    if (!(st[ST_OVF] & (OVF_BOND | OVF_HB))) break;
    if (attempt > 3) return fail(h, RG_E_CAPACITY, "bond list capacity");
    if (st[ST_OVF] & OVF_BOND) {
      d.bond_cap = st[ST_MAXB] + 4;
      if ((rc = alloc_bonds(h))) return rc;
    }
    if (st[ST_OVF] & OVF_HB) {
      d.hb_cap = (int)(st[ST_MAXHB] * 1.2) + 16;
      if ((rc = alloc_hb(h))) return rc;
    }
    h->stats.regrows++;
    CK(cudaMemsetAsync(d.status, 0, RG_NSTATUS * sizeof(int), h->st));
  }
  h->stats.n_pairs = st[5];
  h->stats.n_H_entries = st[5];
  h->stats.n_bonds = st[6];
  h->stats.n_hbond_pairs = st[7];
  h->stats.max_nbrs = st[ST_MAXNB] + st[ST_MAXNF];
  h->stats.max_bonds = st[ST_MAXB];
  h->stats.max_hbonds = st[ST_MAXHB];
  h->lists_valid = true;
  h->bonds_fresh = true;
  return 0;
}

int do_compute(rg_system *h, int eflag, int vflag = 0, int atom_tally = 0, bool graph = false) {
  Dev &d = h->d;
  int rc;
  if ((!h->lists_valid || !h->bonds_fresh) && (rc = build_lists(h))) return rc;
  h->bonds_fresh = false;
  CK(cudaMemsetAsync(d.fC, 0, 4 * sizeof(double) * (size_t)d.n, h->st));
  if (d.fC32) CK(cudaMemsetAsync(d.fC32, 0, 3 * sizeof(float) * (size_t)d.n, h->st));
  CK(cudaMemsetAsync(d.vsum, 0, 2 * sizeof(double) * (size_t)d.n, h->st));
  CK(cudaMemsetAsync(d.energy, 0, (size_t)d.nseg * RG_NE * sizeof(double), h->st));
  d.vflag = vflag ? 1 : 0;
  d.atom_tally = atom_tally ? 1 : 0;
  h->tallies_valid = false;
  if (atom_tally) {
    CK(cudaMemsetAsync(d.eatom, 0, sizeof(double) * (size_t)d.n, h->st));
    CK(cudaMemsetAsync(d.vatom, 0, 6 * sizeof(double) * (size_t)d.n, h->st));
  }
  if (vflag) CK(cudaMemsetAsync(d.virial, 0, (size_t)d.nseg * 6 * sizeof(double), h->st));
  if (d.debug) CK(cudaMemsetAsync(d.dbg_flag, 0, sizeof(int), h->st));
  auto finite_after = [&](const char *phase) -> int {
    if (!h->check_finite) return 0;
    int flag = 0;
    CK(cudaMemsetAsync(d.status + ST_NAN, 0, sizeof(int), h->st));
    launch_check_finite(d.fC, 4 * (long long)d.n, d.status + ST_NAN, h->st);
    CK(cudaMemcpyAsync(&flag, d.status + ST_NAN, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    if (!flag) return 0;
    std::string msg = std::string("non-finite force after ") + phase;
    int df = 0;
    CK(cudaMemcpy(&df, d.dbg_flag, sizeof(int), cudaMemcpyDeviceToHost));
    if (df) {
      double v[40];
      CK(cudaMemcpy(v, d.dbg, sizeof v, cudaMemcpyDeviceToHost));
      msg += "; first term:";
      for (double x : v) msg += " " + std::to_string(x);
    }
    return fail(h, RG_E_NUMERIC, msg);
  };
  { Scope sc(h, PH_BO, 3); launch_bond_orders(d, h->st); }
  { Scope sc(h, PH_ATOM, 2); launch_atom_energy(d, h->st, eflag); }
  if ((rc = finite_after("atom_energy"))) return rc;
  { Scope sc(h, PH_HB, 1); launch_hbonds(d, h->st, eflag); }
  if ((rc = finite_after("hbonds"))) return rc;
  {
    Scope sc(h, PH_VALTOR, 9);
    launch_vt_count(d, h->st);
  }
  if (graph) {
    // captured: grids of the list capacities, counts read on the device
    Scope sc(h, PH_VALTOR, 1 + 2 + (d.mixed ? 1 : 0));
    launch_vt_run(d, h->st, eflag, d.cap_val, d.cap_tor, true);
  } else {
    // item totals sit after the last slot of the exclusive scans
    const long long slots = (long long)d.n * d.bond_cap;
    int tot[2];
    CK(cudaMemcpyAsync(&tot[0], d.w_off_v + slots, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CK(cudaMemcpyAsync(&tot[1], d.w_off_t + slots, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    if (tot[0] > d.cap_val || tot[1] > d.cap_tor) {
      if (alloc_items(h, std::max<long long>(d.cap_val, (long long)(tot[0] * 1.3) + 1024),
                      std::max<long long>(d.cap_tor, (long long)(tot[1] * 1.3) + 1024)))
        return RG_E_CUDA;
      h->stats.regrows++;
    }
    h->n_val = tot[0];
    h->n_tor = tot[1];
    Scope sc(h, PH_VALTOR, 1 + (tot[0] > 0) + (tot[1] > 0) + (d.mixed ? 1 : 0));
    launch_vt_run(d, h->st, eflag, tot[0], tot[1]);
  }
  if ((rc = finite_after("valence_torsion"))) return rc;
  { Scope sc(h, PH_NONB, 1); launch_nonbonded(d, h->st, eflag); }
  if ((rc = finite_after("nonbonded"))) return rc;
  { Scope sc(h, PH_DBOND, 1); launch_dbond_forces(d, h->st); }
  if ((rc = finite_after("dbond_forces"))) return rc;
  { Scope sc(h, PH_FOUT, 1); launch_force_out(d, h->st); }
  CK(cudaGetLastError());
  h->forces_valid = true;
  return 0;
}

// capture `chunk` CG iterations (A, SpMV, ctrl/C/flip) as a graph
int capture_cg(rg_system *h, int chunk) {
  Dev &d = h->d;
  if (h->cg_exec) {
    cudaGraphExecDestroy(h->cg_exec);
    h->cg_exec = nullptr;
  }
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
  for (int k = 0; k < chunk; ++k) {
    launch_qeq_cg_A(d, h->st);
    launch_qeq_spmv(d, h->st, d.qd, d.qq, 1);
    launch_qeq_cg_C(d, h->st);
  }
  cudaError_t e = cudaStreamEndCapture(h->st, &g);
  if (e == cudaSuccess) e = cudaGraphInstantiate(&h->cg_exec, g, 0);
  if (g) cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    h->cg_exec = nullptr;
    return fail(h, RG_E_CUDA, std::string("CG graph capture: ") + cudaGetErrorString(e));
  }
  h->cg_dev = d;
  return 0;
}

int do_qeq(rg_system *h, int *its, int *itt) {
  Dev &d = h->d;
  int rc;
  if (!h->lists_valid && (rc = build_lists(h))) return rc;
  const int ns = d.nseg;
  const double tol = h->p.qeq_tol;
  const int imax = h->p.qeq_imax;
  {
    Scope sc(h, PH_QSETUP, 6 + (d.mixed ? 1 : 0));
    launch_qeq_setup(d, h->st);
    launch_qeq_cg_init(d, h->st, tol, imax);
  }
  // iterate; poll the number of segments with an active solve every few
  // iterations.  The mixed form then restarts the CG from its iterate with
  // the residual recomputed with FP64 sums (iterative refinement) until that
  // residual meets the tolerance: at most RG_MAX_REFINE restarts.
  const int RG_MAX_REFINE = 3;
  const int chunk = 4;
  std::vector<double> it(2 * (size_t)ns);
  std::vector<int> tot(2 * (size_t)ns, 0);
  int refines = 0, active = 0;
  for (;;) {
    int done_iters = 0;
    for (;;) {
      CK(cudaMemcpyAsync(&active, d.n_active, sizeof(int), cudaMemcpyDeviceToHost, h->st));
      CK(cudaStreamSynchronize(h->st));
      if (active == 0) break;
      if (done_iters > imax + 8) return fail(h, RG_E_NUMERIC, "QEq iteration control lost");
      if (h->use_graphs && !(h->prof.on && (h->prof.mask & kCgPhases))) {
        // timing the CG phases needs the per-kernel event marks: plain launches
        if (!h->cg_exec || std::memcmp(&h->cg_dev, &d, sizeof(Dev)) != 0) {
          int rc2 = capture_cg(h, chunk);
          if (rc2) return rc2;
        }
        CK(cudaGraphLaunch(h->cg_exec, h->st));
        h->launches += 5 * chunk;
      } else {
        for (int k = 0; k < chunk; ++k) {
          { Scope sc(h, PH_QVEC, 1); launch_qeq_cg_A(d, h->st); }
          { Scope sc(h, PH_QSPMV, 1); launch_qeq_spmv(d, h->st, d.qd, d.qq, 1); }
          { Scope sc(h, PH_QVEC, 3); launch_qeq_cg_C(d, h->st); }
        }
      }
      done_iters += chunk;
    }
    // iterations of this pass per segment and system; the initial pass
    // counts its first (set-up) iteration like CG_v2, a restart that is not
    // needed adds nothing
    CK(cudaMemcpy2DAsync(it.data(), 2 * sizeof(double), d.red + 22, RG_NRED * sizeof(double),
                         2 * sizeof(double), ns, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    for (size_t k = 0; k < it.size(); ++k) tot[k] += std::max(0, (int)it[k] - (refines ? 1 : 0));
    if (!d.mixed || refines >= RG_MAX_REFINE) break;
    // residual with FP64 sums; the CG set-up for a restart only where it
    // is above the tolerance
    { Scope sc(h, PH_QSETUP, 6); launch_qeq_refine_check(d, h->st, tol); }
    ++refines;
    CK(cudaMemcpyAsync(&active, d.n_active, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    if (active == 0) break;
    { Scope sc(h, PH_QSETUP, 3); launch_qeq_cg_init_rest(d, h->st, tol, imax); }
    CK(cudaMemcpyAsync(&active, d.n_active, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    if (active == 0) break;
  }
  int ms = 0, mt = 0;
  for (int g = 0; g < ns; ++g) {
    ms = std::max(ms, tot[2 * g]);
    mt = std::max(mt, tot[2 * g + 1]);
  }
  h->seg_iters.swap(tot);
  h->stats.cg_iters_s = ms;
  h->stats.cg_iters_t = mt;
  h->stats.cg_system_iters += std::max(ms - 1, 0) + std::max(mt - 1, 0);
  h->stats.cg_spmv_rows_passes += std::max(std::max(ms, mt) - 1, 0);
  h->stats.qeq_restarts = refines;
  if (its) *its = ms;
  if (itt) *itt = mt;
  { Scope sc(h, PH_QFIN, 3); launch_qeq_finish(d, h->st); }
  CK(cudaGetLastError());
  return 0;
}

// ------------------------------------------------------------------
// the single-point step as one captured graph (rg_single_point)
//
// Lists, QEq and force step without a host synchronisation: the list
// kernels clip to their capacities and flag an overflow, the valence and
// torsion kernels take their counts on the device, and the QEq loops are
// conditional WHILE nodes whose condition a device kernel sets from the
// number of segments still iterating (bounded by a trip limit); the mixed
// form's refinement restarts are nested IF nodes.  The step saves the QEq
// histories first, so that the host can restore them and redo the step on
// the regular path when the replay reports an overflow.

constexpr int kMaxCapLevels = 8;

int cap_graph(rg_system *h, cudaStream_t s, cudaGraph_t *g) {
  cudaStreamCaptureStatus cs;
  CK(cudaStreamGetCaptureInfo(s, &cs, nullptr, g, nullptr, nullptr, nullptr));
  if (cs != cudaStreamCaptureStatusActive) return fail(h, RG_E_CUDA, "graph capture not active");
  return 0;
}

// a conditional node at the capture point of s; its body graph returned
int add_cond(rg_system *h, cudaStream_t s, cudaGraphConditionalNodeType type,
             cudaGraphConditionalHandle c, cudaGraph_t *body) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g;
  const cudaGraphNode_t *deps = nullptr;
  size_t nd = 0;
  CK(cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, &deps, nullptr, &nd));
  cudaGraphNodeParams np{};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = c;
  np.conditional.type = type;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  CK(cudaGraphAddNode(&node, g, deps, nullptr, nd, &np));
  *body = np.conditional.phGraph_out[0];
  CK(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  return 0;
}

// one CG pass at capture level lvl: condition from the active count (also
// into *started when given), WHILE { iteration }, then the pass's totals
int cap_cg_pass(rg_system *h, int lvl, int pass, cudaGraphConditionalHandle *started) {
  if (lvl + 1 >= kMaxCapLevels) return fail(h, RG_E_CUDA, "graph nesting too deep");
  const Dev &d = h->d;
  cudaStream_t s = h->cap_st[lvl], sb = h->cap_st[lvl + 1];
  cudaGraph_t g, body;
  int rc;
  if ((rc = cap_graph(h, s, &g))) return rc;
  cudaGraphConditionalHandle cl, cs0 = 0;
  CK(cudaGraphConditionalHandleCreate(&cl, g, 0, 0));
  if (started) {
    CK(cudaGraphConditionalHandleCreate(started, g, 0, 0));
    cs0 = *started;
  }
  launch_qeq_set_cond(d, s, cl, cs0);
  if ((rc = add_cond(h, s, cudaGraphCondTypeWhile, cl, &body))) return rc;
  CK(cudaStreamBeginCaptureToGraph(sb, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  // sp_trip CG iterations per loop trip (iterations past a system's
  // convergence skip their work, as in the host-polled loop)
  for (int k = 0; k < h->sp_trip; ++k) {
    launch_qeq_cg_A(d, sb);
    launch_qeq_spmv(d, sb, d.qd, d.qq, 1);
    launch_qeq_cg_C(d, sb);
  }
  launch_qeq_loop_cond(d, sb, cl, 4 * (h->p.qeq_imax + 8) / h->sp_trip + 4);
  cudaGraph_t out;
  CK(cudaStreamEndCapture(sb, &out));
  launch_qeq_tot(d, s, pass);
  return 0;
}

// the mixed form's refinement pass p (1..3) at level lvl: the residual
// check, then -- only where a segment needs it -- the restart and its CG
// pass, then (if that pass iterated) the next check
int cap_refine(rg_system *h, int lvl, int pass) {
  if (lvl + 2 >= kMaxCapLevels) return fail(h, RG_E_CUDA, "graph nesting too deep");
  const Dev &d = h->d;
  cudaStream_t s = h->cap_st[lvl], s1 = h->cap_st[lvl + 1], s2 = h->cap_st[lvl + 2];
  cudaGraph_t g, body;
  int rc;
  if ((rc = cap_graph(h, s, &g))) return rc;
  launch_qeq_refine_check(d, s, h->p.qeq_tol);
  launch_qeq_restart_count(d, s);
  cudaGraphConditionalHandle cb;
  CK(cudaGraphConditionalHandleCreate(&cb, g, 0, 0));
  launch_qeq_set_cond(d, s, cb, 0);
  if ((rc = add_cond(h, s, cudaGraphCondTypeIf, cb, &body))) return rc;
  CK(cudaStreamBeginCaptureToGraph(s1, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  launch_qeq_cg_init_rest(d, s1, h->p.qeq_tol, h->p.qeq_imax);
  cudaGraphConditionalHandle started = 0;
  rc = cap_cg_pass(h, lvl + 1, pass, pass < 3 ? &started : nullptr);
  if (!rc && pass < 3) {
    cudaGraph_t body2, out2;
    rc = add_cond(h, s1, cudaGraphCondTypeIf, started, &body2);
    if (!rc) {
      CK(cudaStreamBeginCaptureToGraph(s2, body2, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
      rc = cap_refine(h, lvl + 2, pass + 1);
      CK(cudaStreamEndCapture(s2, &out2));
    }
  }
  cudaGraph_t out;
  CK(cudaStreamEndCapture(s1, &out));
  return rc;
}

// the single-point step (dt = 0) or the MD step with time step dt
int capture_step(rg_system *h, StepGraph &G, int eflag, int vflag, int atom_tally, double dt) {
  Dev &d = h->d;
  if (G.exec) {
    cudaGraphExecDestroy(G.exec);
    G.exec = nullptr;
  }
  for (int k = 0; k < kMaxCapLevels; ++k)
    if (!h->cap_st[k]) CK(cudaStreamCreateWithFlags(&h->cap_st[k], cudaStreamNonBlocking));
  cudaStream_t main_st = h->st;
  h->st = h->cap_st[0];    // the launch helpers use h->st
  const long long launches0 = h->launches;
  const bool lists0 = h->lists_valid, forces0 = h->forces_valid, tallies0 = h->tallies_valid;
  const bool fresh0 = h->bonds_fresh;
  cudaGraph_t g = nullptr;
  int rc = 0;
  cudaError_t e = cudaStreamBeginCapture(h->st, cudaStreamCaptureModeRelaxed);
  if (e == cudaSuccess) {
    const size_t n = (size_t)d.n;
    cudaStream_t s = h->st;
    cudaMemcpyAsync(d.hist_save, d.s_hist, 5 * n * sizeof(double), cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(d.hist_save + 5 * n, d.t_hist, 5 * n * sizeof(double),
                    cudaMemcpyDeviceToDevice, s);
    if (dt > 0.0) {
      // an MD step also saves the positions and velocities it advances
      cudaMemcpyAsync(d.hist_save + 10 * n, d.x_o, 3 * n * sizeof(double),
                      cudaMemcpyDeviceToDevice, s);
      cudaMemcpyAsync(d.hist_save + 13 * n, d.v_o, 3 * n * sizeof(double),
                      cudaMemcpyDeviceToDevice, s);
      cudaMemcpyAsync(d.hist_save + 16 * n, d.f_o, 3 * n * sizeof(double),
                      cudaMemcpyDeviceToDevice, s);
      launch_nve_initial(d, s, dt);
    }
    cudaMemsetAsync(d.status, 0, RG_NSTATUS * sizeof(int), s);
    cudaMemsetAsync(d.qeq_ctl, 0, 4 * sizeof(int), s);
    cudaMemsetAsync(d.qeq_tot, 0, 2 * sizeof(int) * (size_t)d.nseg, s);
    launch_bin_sort(d, s);
    launch_build_nbrs(d, s);
    launch_build_bonds(d, s);
    launch_count(d, s);
    launch_qeq_setup(d, s);
    launch_qeq_cg_init(d, s, h->p.qeq_tol, h->p.qeq_imax);
    rc = cap_cg_pass(h, 0, 0, nullptr);
    if (!rc && d.mixed) rc = cap_refine(h, 0, 1);
    if (!rc) {
      launch_qeq_finish(d, s);
      h->lists_valid = true;    // built by the captured kernels above
      h->bonds_fresh = true;
      rc = do_compute(h, eflag, vflag, atom_tally, true);
      if (!rc && dt > 0.0) launch_nve_final(d, s, dt);
    }
    e = cudaStreamEndCapture(s, &g);
  }
  h->st = main_st;
  h->launches = launches0;
  h->lists_valid = lists0;
  h->bonds_fresh = fresh0;
  h->forces_valid = forces0;
  h->tallies_valid = tallies0;
  if (e == cudaSuccess && !rc) e = cudaGraphInstantiate(&G.exec, g, 0);
  if (e == cudaSuccess && !rc) {
    size_t nn = 0;
    cudaGraphGetNodes(g, nullptr, &nn);
    std::vector<cudaGraphNode_t> nodes(nn);
    cudaGraphGetNodes(g, nodes.data(), &nn);
    long long k = 0;
    for (auto nd : nodes) {
      cudaGraphNodeType t;
      if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++k;
    }
    G.kernels = k;
  }
  if (g) cudaGraphDestroy(g);
  cudaGetLastError();
  if (e != cudaSuccess || rc) {
    G.exec = nullptr;
    G.failed = true;
    return rc ? rc : fail(h, RG_E_CUDA, std::string("step graph: ") + cudaGetErrorString(e));
  }
  G.dev = d;
  G.flags = eflag | (vflag << 4) | (atom_tally << 8);
  G.dt = dt;
  return 0;
}

// whether G holds the step of the current arrays, flags and time step
bool step_matches(const rg_system *h, const StepGraph &G, int flags, double dt) {
  return G.exec && G.flags == flags && G.dt == dt &&
         std::memcmp(&G.dev, &h->d, sizeof(Dev)) == 0;
}

// after a regular step: a configuration seen twice in a row is captured
// (one-off batches and cohorts do not pay for a capture)
void maybe_capture(rg_system *h, StepGraph &G, int eflag, int vflag, int atom_tally, double dt) {
  const int flags = eflag | (vflag << 4) | (atom_tally << 8);
  const bool again = G.seen_flags == flags && G.seen_dt == dt &&
                     std::memcmp(&G.seen, &h->d, sizeof(Dev)) == 0;
  G.seen = h->d;
  G.seen_flags = flags;
  G.seen_dt = dt;
  const bool eligible = h->use_graphs && !h->prof.on && !h->check_finite && !G.failed;
  if (eligible && again && !step_matches(h, G, flags, dt))
    capture_step(h, G, eflag, vflag, atom_tally, dt);   // failures keep the regular path
}

// One replay of G and its single read-back.  Returns 1 when the step must be
// redone on the regular path (a list past its capacity, a work list past
// its capacity or a tripped CG loop limit); the saved histories (and, for
// an MD step, positions and velocities) are then restored.
int replay_step(rg_system *h, StepGraph &G, bool atom_tally) {
  Dev &d = h->d;
  CK(cudaGraphLaunch(G.exec, h->st));
  int st[RG_NSTATUS], ctl[4], items[2];
  const long long slots = (long long)d.n * d.bond_cap;
  std::vector<int> tot(2 * (size_t)d.nseg);
  CK(cudaMemcpyAsync(st, d.status, sizeof st, cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(ctl, d.qeq_ctl, sizeof ctl, cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(&items[0], d.w_off_v + slots, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(&items[1], d.w_off_t + slots, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(tot.data(), d.qeq_tot, tot.size() * sizeof(int), cudaMemcpyDeviceToHost,
                     h->st));
  CK(cudaStreamSynchronize(h->st));
  if ((st[ST_OVF] != 0) || items[0] > d.cap_val || items[1] > d.cap_tor || ctl[2]) {
    const size_t n = (size_t)d.n;
    CK(cudaMemcpyAsync(d.s_hist, d.hist_save, 5 * n * sizeof(double), cudaMemcpyDeviceToDevice,
                       h->st));
    CK(cudaMemcpyAsync(d.t_hist, d.hist_save + 5 * n, 5 * n * sizeof(double),
                       cudaMemcpyDeviceToDevice, h->st));
    if (G.dt > 0.0) {
      CK(cudaMemcpyAsync(d.x_o, d.hist_save + 10 * n, 3 * n * sizeof(double),
                         cudaMemcpyDeviceToDevice, h->st));
      CK(cudaMemcpyAsync(d.v_o, d.hist_save + 13 * n, 3 * n * sizeof(double),
                         cudaMemcpyDeviceToDevice, h->st));
      CK(cudaMemcpyAsync(d.f_o, d.hist_save + 16 * n, 3 * n * sizeof(double),
                         cudaMemcpyDeviceToDevice, h->st));
    }
    h->lists_valid = false;
    h->forces_valid = G.dt > 0.0;   // an MD step restarts from its saved forces
    h->stats.step_graph_redos++;
    return 1;
  }
  h->stats.step_graph_replays++;
  int ms = 0, mt = 0;
  for (int g = 0; g < d.nseg; ++g) {
    ms = std::max(ms, tot[2 * g]);
    mt = std::max(mt, tot[2 * g + 1]);
  }
  h->seg_iters.assign(tot.begin(), tot.end());
  h->stats.cg_iters_s = ms;
  h->stats.cg_iters_t = mt;
  h->stats.cg_system_iters += std::max(ms - 1, 0) + std::max(mt - 1, 0);
  h->stats.cg_spmv_rows_passes += std::max(std::max(ms, mt) - 1, 0);
  h->stats.qeq_restarts = ctl[0];
  h->stats.n_pairs = st[5];
  h->stats.n_H_entries = st[5];
  h->stats.n_bonds = st[6];
  h->stats.n_hbond_pairs = st[7];
  h->stats.max_nbrs = st[ST_MAXNB] + st[ST_MAXNF];
  h->stats.max_bonds = st[ST_MAXB];
  h->stats.max_hbonds = st[ST_MAXHB];
  h->n_val = items[0];
  h->n_tor = items[1];
  h->launches += G.kernels + (5LL * h->sp_trip + 1) * ctl[1];
  h->lists_valid = true;
  h->bonds_fresh = false;   // the replay's force step used them
  h->forces_valid = true;
  h->tallies_valid = atom_tally;
  if (st[ST_NAN]) return fail(h, RG_E_NUMERIC, "non-finite force");
  return 0;
}

// scalar controls from the run parameters and the force field
// (reaxc_ffield_sunway.cpp:86-88 and the pair_style defaults)
void init_control(const rg_params &p, const ForceField &ff, Control &c) {
  c.bo_cut = 0.01 * ff.gp[29];
  c.nonb_low = ff.gp[11];
  c.nonb_cut = ff.gp[12];
  c.bond_cut = p.bond_cut;
  c.hbond_cut = p.hbond_cut;
  c.thb_cut = p.thb_cut;
  c.thb_cutsq = p.thb_cutsq;
  c.enobondsflag = p.enobondsflag;
  c.lgflag = p.lgflag;
  const double lc = std::max(c.nonb_cut, p.qeq_swb);
  c.list_cut2 = lc * lc;
  c.nonb_cut2 = c.nonb_cut * c.nonb_cut;
  c.swb2 = p.qeq_swb * p.qeq_swb;
  c.near_cut = std::max(c.bond_cut, c.hbond_cut);
  c.near_cut2_lo = c.near_cut * c.near_cut * (1.0 - 1e-12);
  c.near_cut2_hi = c.near_cut * c.near_cut * (1.0 + 1e-12);
  c.bond_cut_f = (float)c.bond_cut;
  c.hbond_cut_f = (float)c.hbond_cut;
  rg_init_taper(c.nonb_low, c.nonb_cut, c.Tap);
  rg_init_taper(p.qeq_swa, p.qeq_swb, c.qTap);
  c.tap_factored = (c.nonb_low == 0.0);
  c.qtap_factored = (p.qeq_swa == 0.0);
  c.inv_swb_nb = 1.0 / c.nonb_cut;
  c.inv_swb_q = 1.0 / p.qeq_swb;
  c.nonb_all_listed = c.nonb_cut2 >= c.list_cut2;
  c.h_all_listed = c.swb2 >= c.list_cut2;
  c.list_pre2_f = (float)(c.list_cut2 * (1.0 + 1e-5) + 0.05);
  c.list_cut2_f = (float)c.list_cut2;
  c.thb_cut_f = (float)c.thb_cut;
  c.thb_cutsq_f = (float)c.thb_cutsq;
  for (int a = 0; a < RG_MAXT; ++a)
    for (int b = 0; b < RG_MAXT; ++b)
      for (int e = 0; e < RG_MAXT; ++e) {
        const Thbh &th = ff.thbp[a][b][e];
        bool any = false;
        for (int q = 0; q < th.cnt; ++q) any = any || std::fabs(th.prm[q].p_val1) > 0.001;
        c.thb_any[a][b][e] = any ? 1 : 0;
        for (int g = 0; g < RG_MAXT; ++g) {
          const Fbh &fb = ff.fbp[a][b][e][g];
          c.fb_on[a][b][e][g] = (fb.cnt && (fb.prm.V1 != 0.0 || fb.prm.V2 != 0.0 ||
                                            fb.prm.V3 != 0.0 || fb.prm.p_cot1 != 0.0)) ? 1 : 0;
        }
      }
  c.near_cut_f = (float)c.near_cut;
  c.swb2_f = (float)c.swb2;
  c.inv_swb_q_f = (float)c.inv_swb_q;
  c.nonb_cut2_f = (float)c.nonb_cut2;
  c.inv_swb_nb_f = (float)c.inv_swb_nb;
  for (int k = 0; k < 8; ++k) {
    c.qTap_f[k] = (float)c.qTap[k];
    c.Tap_f[k] = (float)c.Tap[k];
    c.dTap_f[k] = (float)(k * c.Tap[k]);
  }
  c.p_vdW1_f = (float)ff.gp[28];
  for (int a = 0; a < RG_MAXT; ++a)
    for (int b = 0; b < RG_MAXT; ++b) {
      const Tbp &tw = ff.tbp[a][b];
      Control::NbF &e = c.nb32[a][b];
      e.alpha = (float)tw.alpha;
      e.r_vdW = (float)tw.r_vdW;
      e.D = (float)tw.D;
      e.ar = (float)tw.alpha / (float)tw.r_vdW;
      e.powgi = (float)tw.powgi_vdW1;
      e.gamma = (float)tw.gamma;
      e.ecore = (float)tw.ecore;
      e.acore = (float)tw.acore;
      e.rcore = (float)tw.rcore;
      e.lgcij = (float)tw.lgcij;
      const float lg2 = (float)tw.lgre * (float)tw.lgre;
      e.re6 = lg2 * lg2 * lg2;
      for (int k = 0; k < RG_MAXT; ++k) {
        const Hbp &hp = ff.hbp[a][b][k];
        c.hb32[a][b][k] = {(float)hp.r0_hb, (float)hp.p_hb1, (float)hp.p_hb2, (float)hp.p_hb3};
      }
    }
  c.bo_scale_f = (float)(1.0 + c.bo_cut);
  c.bo_half_f = (float)(0.5 * c.bo_cut);
  for (int a = 0; a < RG_MAXT; ++a)
    for (int b = 0; b < RG_MAXT; ++b) {
      const Tbp &tw = ff.tbp[a][b];
      Control::BoEst &e = c.bo_est[a][b];
      const double pk[3] = {tw.p_bo1, tw.p_bo3, tw.p_bo5}, qk[3] = {tw.p_bo2, tw.p_bo4, tw.p_bo6};
      const double r0[3] = {tw.r_s, tw.r_p, tw.r_pp};
      for (int k = 0; k < 3; ++k) {
        e.e[k] = (float)(pk[k] * 1.4426950408889634);   // log2(e)
        e.q[k] = (float)qk[k];
        e.l[k] = r0[k] > 0.0 ? (float)std::log2(r0[k]) : 0.f;
      }
      c.ln_r[a][b][0] = tw.r_s > 0.0 ? std::log(tw.r_s) : 0.0;
      c.ln_r[a][b][1] = tw.r_p > 0.0 ? std::log(tw.r_p) : 0.0;
      c.ln_r[a][b][2] = tw.r_pp > 0.0 ? std::log(tw.r_pp) : 0.0;
      const Sbp &sa = ff.sbp[a], &sb = ff.sbp[b];
      e.mask = ((sa.r_s > 0.0 && sb.r_s > 0.0) ? 1 : 0) |
               ((sa.r_pi > 0.0 && sb.r_pi > 0.0) ? 2 : 0) |
               ((sa.r_pi_pi > 0.0 && sb.r_pi_pi > 0.0) ? 4 : 0);
    }
}

}  // namespace

extern "C" {

void rg_default_params(rg_params *p) {
  p->bond_cut = 5.0;
  p->hbond_cut = 7.5;
  p->thb_cut = 0.001;
  p->thb_cutsq = 0.00001;
  p->enobondsflag = 1;
  p->lgflag = 0;
  p->qeq_swa = 0.0;
  p->qeq_swb = 10.0;
  p->qeq_tol = 1e-6;
  p->qeq_imax = 200;
  p->precision = RG_PREC_FP64;
  p->device = 0;
  p->tabulate = 65536;
  p->tabulate_check = 0;
  p->autotune = 1;
  p->cell_div = 0;
  p->spmv_rows = 0;
  p->pair_kernel = 0;
}

int rg_create(const char *ffield_path, const rg_params *pin, rg_system **out) {
  if (!out || !ffield_path) return RG_E_ARG;
  *out = nullptr;
  rg_system *h = new rg_system();
  if (pin) h->p = *pin;
  else rg_default_params(&h->p);
  std::string e = rg_read_ffield(ffield_path, h->p.lgflag, &h->ff);
  if (!e.empty()) {
    delete h;
    return RG_E_FILE;
  }
  Control &c = h->ctl;
  init_control(h->p, h->ff, c);
  const double lc = std::sqrt(c.list_cut2);
  if (h->p.precision != RG_PREC_FP64 && h->p.precision != RG_PREC_MIXED) {
    delete h;
    return RG_E_ARG;
  }
  h->d.mixed = (h->p.precision == RG_PREC_MIXED);
  h->d.spmv_rw = 16;
  if (h->p.cell_div != 0 && h->p.cell_div != 2 && h->p.cell_div != 3) {
    delete h;
    return RG_E_ARG;
  }
  if (h->p.spmv_rows != 0 && h->p.spmv_rows != 8 && h->p.spmv_rows != 16 && h->p.spmv_rows != 32) {
    delete h;
    return RG_E_ARG;
  }
  if (h->p.cell_div) h->cell_div = h->p.cell_div;
  h->d.nbr_tiles = h->p.pair_kernel == 2 ? 1 : 0;
  if (h->p.spmv_rows) h->d.spmv_rw = h->p.spmv_rows;
  {
    const char *cf = std::getenv("RG_CHECK_FINITE");
    h->check_finite = cf && (cf[0] == '1' || cf[0] == '2');
    const char *ng = std::getenv("RG_NO_GRAPHS");
    h->use_graphs = !(ng && ng[0] == '1');
    // CG iterations per device-side loop trip of the captured step (1-8)
    const char *tr = std::getenv("RG_SP_TRIP");
    if (tr && std::atoi(tr) >= 1 && std::atoi(tr) <= 8) h->sp_trip = std::atoi(tr);
    h->d.debug = cf && cf[0] == '2';
  }
  for (int t = 0; t < RG_MAXT; ++t) h->ff.nve_mass[t] = h->ff.sbp[t].mass;
  if (c.near_cut > lc) {
    delete h;
    return RG_E_ARG;
  }
  // FP64 tables of the pair functions (tables.cpp)
  std::vector<double> tab_nb, tab_h;
  c.tab_n = 0;
  if (h->p.tabulate > 0) {
    const int nt = h->ff.ntypes;
    for (int a = 0; a < nt; ++a)
      for (int b = 0; b < nt; ++b) c.tab_pair[a][b] = rg_pair_index(a, b, nt);
    const double s0 = 0.25, s1 = c.list_cut2 * (1.0 + 1e-9);
    c.tab_n = h->p.tabulate;
    c.tab_s0 = s0;
    c.tab_s0_f = (float)s0;
    c.tab_ds = (s1 - s0) / c.tab_n;
    c.tab_inv_ds = 1.0 / c.tab_ds;
    c.tab_x0 = -s0 * c.tab_inv_ds;
    c.tab_inv_ds_f = (float)c.tab_inv_ds;
    c.tab_x0_f = (float)c.tab_x0;
    c.tab_inv_ds_l = (float)(c.tab_inv_ds - (double)c.tab_inv_ds_f);
    c.tab_x0_l = (float)(c.tab_x0 - (double)c.tab_x0_f);
    h->tab_err = rg_build_tables(h->ff, c, c.tab_n, s0, s1, tab_nb, tab_h, h->p.tabulate_check != 0);
  }
  cudaError_t ce = cudaSetDevice(h->p.device);
  if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking);
  if (ce == cudaSuccess) ce = cudaMalloc(&h->d_ff, sizeof(ForceField));
  if (ce == cudaSuccess) ce = cudaMalloc(&h->d_ctl, sizeof(Control));
  if (ce == cudaSuccess) ce = cudaMemcpy(h->d_ff, &h->ff, sizeof(ForceField), cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) ce = cudaMemcpy(h->d_ctl, &h->ctl, sizeof(Control), cudaMemcpyHostToDevice);
  if (ce == cudaSuccess && c.tab_n && h->d.mixed) {
    // the mixed form evaluates the vdW + Coulomb cubics in FP32 (its QEq H
    // values are FP32 expressions of the pair-list pass)
    std::vector<float> nb32(tab_nb.begin(), tab_nb.end());
    ce = cudaMalloc(&h->d_tab32, sizeof(float) * nb32.size());
    if (ce == cudaSuccess)
      ce = cudaMemcpy(h->d_tab32, nb32.data(), sizeof(float) * nb32.size(), cudaMemcpyHostToDevice);
  } else if (ce == cudaSuccess && c.tab_n) {
    ce = cudaMalloc(&h->d_tab, sizeof(double) * (tab_nb.size() + tab_h.size()));
    if (ce == cudaSuccess)
      ce = cudaMemcpy(h->d_tab, tab_nb.data(), sizeof(double) * tab_nb.size(), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess)
      ce = cudaMemcpy(h->d_tab + tab_nb.size(), tab_h.data(), sizeof(double) * tab_h.size(),
                      cudaMemcpyHostToDevice);
    // the same coefficients as FP32 pairs (hi, lo) for the orthogonal
    // segments' pairs
    std::vector<float> fp(2 * (tab_nb.size() + tab_h.size()));
    size_t o = 0;
    for (const std::vector<double> *t : {&tab_nb, &tab_h})
      for (double v : *t) {
        const float hi = (float)v;
        fp[o++] = hi;
        fp[o++] = (float)(v - (double)hi);
      }
    if (ce == cudaSuccess) ce = cudaMalloc(&h->d_tab32, sizeof(float) * fp.size());
    if (ce == cudaSuccess)
      ce = cudaMemcpy(h->d_tab32, fp.data(), sizeof(float) * fp.size(), cudaMemcpyHostToDevice);
  }
  if (ce != cudaSuccess) {
    if (h->d_ff) cudaFree(h->d_ff);
    if (h->d_ctl) cudaFree(h->d_ctl);
    if (h->d_tab) cudaFree(h->d_tab);
    if (h->d_tab32) cudaFree(h->d_tab32);
  if (h->cg_exec) cudaGraphExecDestroy(h->cg_exec);
    delete h;
    return RG_E_CUDA;
  }
  h->d.ff = h->d_ff;
  h->d.ctl = h->d_ctl;
  h->d.tab_nb = h->d_tab;
  h->d.tab_h = h->d_tab ? h->d_tab + tab_nb.size() : nullptr;
  if (h->d.mixed) {
    h->d.tab_nb32 = h->d_tab32;
    h->d.tab_nb_fp = h->d.tab_h_fp = nullptr;
  } else {
    h->d.tab_nb32 = nullptr;
    h->d.tab_nb_fp = reinterpret_cast<const float4 *>(h->d_tab32);
    h->d.tab_h_fp = h->d_tab32 ? reinterpret_cast<const float4 *>(h->d_tab32 + 2 * tab_nb.size())
                               : nullptr;
  }
  *out = h;
  return RG_OK;
}

int rg_set_masses(rg_system *h, const double *mass) {
  if (!h || !mass) return RG_E_ARG;
  for (int t = 0; t < h->ff.ntypes; ++t)
    if (!(mass[t] > 0.0)) return fail(h, RG_E_ARG, "masses must be positive");
  for (int t = 0; t < h->ff.ntypes; ++t) h->ff.nve_mass[t] = mass[t];
  CK(cudaSetDevice(h->p.device));
  CK(cudaMemcpyAsync(&h->d_ff->nve_mass[0], &h->ff.nve_mass[0], sizeof(h->ff.nve_mass),
                     cudaMemcpyHostToDevice, h->st));
  CK(cudaStreamSynchronize(h->st));
  return RG_OK;
}

int rg_destroy(rg_system *h) {
  if (!h) return RG_E_ARG;
  cudaSetDevice(h->p.device);
  cudaStreamSynchronize(h->st);
  free_bucket(h->per_n);
  free_bucket(h->per_nb);
  free_bucket(h->per_b);
  free_bucket(h->per_hb);
  free_bucket(h->per_items);
  free_bucket(h->per_seg);
  if (h->cells) cudaFree(h->cells);
  cudaFree(h->d_ff);
  cudaFree(h->d_ctl);
  if (h->d_tab) cudaFree(h->d_tab);
  if (h->d_tab32) cudaFree(h->d_tab32);
  if (h->cg_exec) cudaGraphExecDestroy(h->cg_exec);
  if (h->sp.exec) cudaGraphExecDestroy(h->sp.exec);
  if (h->md.exec) cudaGraphExecDestroy(h->md.exec);
  for (cudaStream_t c : h->cap_st)
    if (c) cudaStreamDestroy(c);
  cudaStreamDestroy(h->st);
  delete h;
  return RG_OK;
}

const char *rg_last_error(const rg_system *h) { return h ? h->err.c_str() : "null handle"; }

int rg_num_types(const rg_system *h) { return h ? h->ff.ntypes : 0; }

int rg_ffield_info(const char *path, int *ntypes, char *names, int len, char *msg, int msg_len) {
  if (!path || !ntypes) return RG_E_ARG;
  ForceField *ff = new ForceField();
  const std::string e = rg_read_ffield(path, 0, ff);
  if (!e.empty()) {
    if (msg && msg_len > 0) std::snprintf(msg, msg_len, "%s", e.c_str());
    delete ff;
    return RG_E_FILE;
  }
  *ntypes = ff->ntypes;
  if (names && len > 0)
    for (int t = 0; t < ff->ntypes; ++t) std::snprintf(names + (size_t)t * len, len, "%s", ff->sbp[t].name);
  delete ff;
  return RG_OK;
}

int rg_table_check(const char *ffield_path, const rg_params *pin, double *max_rel_err) {
  if (!ffield_path || !max_rel_err) return RG_E_ARG;
  rg_params p;
  if (pin) p = *pin;
  else rg_default_params(&p);
  if (p.tabulate <= 0) return RG_E_ARG;
  ForceField *ff = new ForceField();
  if (!rg_read_ffield(ffield_path, p.lgflag, ff).empty()) {
    delete ff;
    return RG_E_FILE;
  }
  Control *c = new Control();
  init_control(p, *ff, *c);
  std::vector<double> nb, hq;
  *max_rel_err = rg_build_tables(*ff, *c, p.tabulate, 0.25, c->list_cut2 * (1.0 + 1e-9), nb, hq, true);
  delete c;
  delete ff;
  return RG_OK;
}

int rg_table_info(const rg_system *h, int *intervals, double *max_rel_err) {
  if (!h) return RG_E_ARG;
  if (intervals) *intervals = h->ctl.tab_n;
  if (max_rel_err) *max_rel_err = h->tab_err;
  return RG_OK;
}

int rg_element_name(const rg_system *h, int t, char *buf, int len) {
  if (!h || t < 0 || t >= h->ff.ntypes || !buf || len < 1) return RG_E_ARG;
  std::snprintf(buf, len, "%s", h->ff.sbp[t].name);
  return RG_OK;
}

int rg_extract(const rg_system *h, const char *name, double *out) {
  if (!h || !name || !out) return RG_E_ARG;
  for (int t = 0; t < h->ff.ntypes; ++t) {
    const Sbp &s = h->ff.sbp[t];
    if (!std::strcmp(name, "chi")) out[t] = s.chi;
    else if (!std::strcmp(name, "eta")) out[t] = s.eta;
    else if (!std::strcmp(name, "gamma")) out[t] = s.gamma;
    else if (!std::strcmp(name, "mass")) out[t] = s.mass;
    else return RG_E_ARG;
  }
  return RG_OK;
}

// atom ranges of the segments from their counts and the atom count; the
// per-atom segment index goes to the device
static int sync_segments(rg_system *h) {
  const int n = h->n;
  const int ns = (int)h->segs.size();
  long long sum = 0;
  for (int g = 0; g < ns; ++g) {
    const int c = h->seg_counts[g] < 0 ? n : h->seg_counts[g];
    h->segs[g].atom0 = (int)sum;
    h->segs[g].natoms = c;
    sum += c;
  }
  if (sum != n) return fail(h, RG_E_ARG, "segment atom counts do not add up to the atom count");
  int rc = alloc_segs(h);
  if (rc) return rc;
  std::vector<int> so((size_t)n);
  for (int g = 0; g < ns; ++g)
    for (int a = 0; a < h->segs[g].natoms; ++a) so[(size_t)h->segs[g].atom0 + a] = g;
  CK(cudaMemcpyAsync(h->d.seg_o, so.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, h->st));
  CK(cudaStreamSynchronize(h->st));
  return 0;
}

// energies of the last force step summed over the segments
static int energy_sum(rg_system *h, double *out) {
  const int ns = h->d.nseg;
  h->e_host.resize((size_t)ns * RG_NE);
  CK(cudaMemcpyAsync(h->e_host.data(), h->d.energy, sizeof(double) * RG_NE * ns,
                     cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  for (int k = 0; k < RG_NE; ++k) {
    double s = 0.0;
    for (int g = 0; g < ns; ++g) s += h->e_host[(size_t)g * RG_NE + k];
    out[k] = s;
  }
  return 0;
}

int rg_set_box(rg_system *h, const double *L3) {
  if (!h || !L3) return RG_E_ARG;
  const int counts[1] = {-1};
  for (int k = 0; k < 3; ++k)
    if (!(L3[k] > 0.0) || !std::isfinite(L3[k])) return fail(h, RG_E_ARG, "box edge must be positive");
  h->segs.assign(1, SegGeom{});
  for (int k = 0; k < 3; ++k) h->segs[0].L[k] = L3[k];
  h->seg_counts.assign(counts, counts + 1);
  h->have_box = true;
  h->lists_valid = false;
  h->forces_valid = false;
  if (h->n) return sync_segments(h);
  return RG_OK;
}

int rg_set_segments(rg_system *h, int nseg, const int *counts, const double *boxes) {
  if (!h || nseg <= 0 || !counts || !boxes) return RG_E_ARG;
  for (int g = 0; g < nseg; ++g) {
    if (counts[g] <= 0) return fail(h, RG_E_ARG, "every segment needs atoms");
    for (int k = 0; k < 3; ++k)
      if (!(boxes[3 * g + k] > 0.0) || !std::isfinite(boxes[3 * g + k]))
        return fail(h, RG_E_ARG, "box edge must be positive");
  }
  h->segs.assign(nseg, SegGeom{});
  for (int g = 0; g < nseg; ++g)
    for (int k = 0; k < 3; ++k) h->segs[g].L[k] = boxes[3 * g + k];
  h->seg_counts.assign(counts, counts + nseg);
  h->have_box = true;
  h->lists_valid = false;
  h->forces_valid = false;
  long long sum = 0;
  for (int g = 0; g < nseg; ++g) sum += counts[g];
  if (h->n && sum == h->n) return sync_segments(h);
  return RG_OK;
}

int rg_set_tilt(rg_system *h, const double *tilt) {
  if (!h || !tilt) return RG_E_ARG;
  if (!h->have_box) return fail(h, RG_E_STATE, "set the box or the segments first");
  for (size_t g = 0; g < h->segs.size(); ++g)
    for (int k = 0; k < 3; ++k) {
      if (!std::isfinite(tilt[3 * g + k])) return fail(h, RG_E_ARG, "tilt must be finite");
      h->segs[g].tilt[k] = tilt[3 * g + k];
    }
  h->lists_valid = false;
  h->forces_valid = false;
  return RG_OK;
}

int rg_num_segments(const rg_system *h) { return h ? (int)h->segs.size() : RG_E_ARG; }

int rg_get_energies(rg_system *h, double *e) {
  if (!h || !e) return RG_E_ARG;
  if (!h->n) return fail(h, RG_E_STATE, "no atoms set");
  CK(cudaMemcpyAsync(e, h->d.energy, sizeof(double) * RG_NE * h->d.nseg, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return RG_OK;
}

int rg_get_virial(rg_system *h, double *v) {
  if (!h || !v) return RG_E_ARG;
  if (!h->n) return fail(h, RG_E_STATE, "no atoms set");
  CK(cudaMemcpyAsync(v, h->d.virial, sizeof(double) * 6 * h->d.nseg, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return RG_OK;
}

int rg_get_atom_tallies(rg_system *h, double *eatom, double *vatom) {
  if (!h) return RG_E_ARG;
  if (!h->tallies_valid)
    return fail(h, RG_E_STATE, "no per-atom tallies: call rg_compute with eflag & 2 or vflag & 4");
  CK(cudaSetDevice(h->p.device));
  const Dev &d = h->d;
  const size_t n = (size_t)d.n;
  std::vector<double> e(n), v(6 * n);
  std::vector<int> perm(n);
  CK(cudaMemcpyAsync(e.data(), d.eatom, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(v.data(), d.vatom, 6 * n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(perm.data(), d.perm, n * sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  for (size_t s = 0; s < n; ++s) {
    const size_t o = (size_t)perm[s];
    if (eatom) eatom[o] = e[s];
    if (vatom)
      for (int k = 0; k < 6; ++k) vatom[6 * o + k] = v[(size_t)k * n + s];
  }
  return RG_OK;
}

}  // extern "C"

// ------------------------------------------------------------------
// regrouping systems on the device (continuous batching)

namespace {

// per-atom state in the caller's order: x, v, f (3 per atom), q, type, tag,
// and the 5-deep s/t histories (history k of atom i at k * n + i)
struct StateView {
  double *x, *v, *f, *q, *sh, *th;
  int *type, *tag;
  int n;
};

struct SegMove {
  int src0, dst0, count;
};

// copy the atom ranges of moves[] from one state to another; one block per
// range
__global__ void k_gather_state(StateView dst, StateView src, const SegMove *moves) {
  const SegMove m = moves[blockIdx.x];
  for (int a = threadIdx.x; a < m.count; a += blockDim.x) {
    const long long s = m.src0 + a, t = m.dst0 + a;
    for (int c = 0; c < 3; ++c) {
      dst.x[3 * t + c] = src.x[3 * s + c];
      dst.v[3 * t + c] = src.v[3 * s + c];
      dst.f[3 * t + c] = src.f[3 * s + c];
    }
    dst.q[t] = src.q[s];
    dst.type[t] = src.type[s];
    dst.tag[t] = src.tag[s];
    for (int k = 0; k < 5; ++k) {
      dst.sh[(long long)k * dst.n + t] = src.sh[(long long)k * src.n + s];
      dst.th[(long long)k * dst.n + t] = src.th[(long long)k * src.n + s];
    }
  }
}

StateView state_of(const rg_system *h) {
  const Dev &d = h->d;
  return StateView{d.x_o, d.v_o, d.f_o, d.q_o, d.s_hist, d.t_hist, d.type_o, d.tag_o, h->n};
}

}  // namespace

extern "C" {

int rg_regroup_segments(rg_system *h, int nkeep, const int *keep, rg_system *src, int nsel,
                        const int *sel) {
  if (!h || nkeep < 0 || nsel < 0 || (nkeep && !keep) || (nsel && (!src || !sel)))
    return RG_E_ARG;
  if (nkeep + nsel == 0) return fail(h, RG_E_ARG, "rg_regroup_segments: no segment selected");
  if (nkeep && !h->n) return fail(h, RG_E_STATE, "rg_regroup_segments: no atoms set");
  if (nsel) {
    if (src == h) return fail(h, RG_E_ARG, "rg_regroup_segments: src must be another handle");
    if (!src->n) return fail(h, RG_E_STATE, "rg_regroup_segments: src holds no atoms");
    if (src->p.device != h->p.device || src->ff.ntypes != h->ff.ntypes)
      return fail(h, RG_E_ARG,
                  "rg_regroup_segments: src must be on the same device with the same force field");
  }
  const int nh = (int)h->segs.size(), ns_src = nsel ? (int)src->segs.size() : 0;
  std::vector<SegGeom> segs;
  std::vector<int> counts;
  std::vector<SegMove> own, other;
  long long n_new = 0;
  for (int k = 0; k < nkeep; ++k) {
    if (keep[k] < 0 || keep[k] >= nh)
      return fail(h, RG_E_ARG, "rg_regroup_segments: keep index out of range");
    const SegGeom &g = h->segs[keep[k]];
    own.push_back(SegMove{g.atom0, (int)n_new, g.natoms});
    segs.push_back(g);
    counts.push_back(g.natoms);
    n_new += g.natoms;
  }
  for (int k = 0; k < nsel; ++k) {
    if (sel[k] < 0 || sel[k] >= ns_src)
      return fail(h, RG_E_ARG, "rg_regroup_segments: sel index out of range");
    const SegGeom &g = src->segs[sel[k]];
    other.push_back(SegMove{g.atom0, (int)n_new, g.natoms});
    segs.push_back(g);
    counts.push_back(g.natoms);
    n_new += g.natoms;
  }
  if (n_new >= (1 << 24)) return fail(h, RG_E_ARG, "rg_regroup_segments: too many atoms");
  CK(cudaSetDevice(h->p.device));
  cudaStream_t st = h->st;
  if (nsel) {
    // the source's pending work must be complete before its state is read
    cudaEvent_t ev;
    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    CK(cudaEventRecord(ev, src->st));
    CK(cudaStreamWaitEvent(st, ev, 0));
    CK(cudaEventDestroy(ev));
  }
  // gather into stream-ordered temporaries (no device-wide synchronisation)
  const size_t N = (size_t)n_new;
  const size_t dbytes = sizeof(double) * N * 20, ibytes = sizeof(int) * N * 2;
  const size_t mbytes = sizeof(SegMove) * (own.size() + other.size());
  char *tmp = nullptr;
  CK(cudaMallocAsync((void **)&tmp, dbytes + ibytes + mbytes, st));
  double *td = (double *)tmp;
  StateView T{td, td + 3 * N, td + 6 * N, td + 9 * N, td + 10 * N, td + 15 * N,
              (int *)(tmp + dbytes), (int *)(tmp + dbytes) + N, (int)n_new};
  SegMove *dm = (SegMove *)(tmp + dbytes + ibytes);
  std::vector<SegMove> all(own);
  all.insert(all.end(), other.begin(), other.end());
  CK(cudaMemcpyAsync(dm, all.data(), mbytes, cudaMemcpyHostToDevice, st));
  if (!own.empty()) k_gather_state<<<(unsigned)own.size(), 256, 0, st>>>(T, state_of(h), dm);
  if (!other.empty())
    k_gather_state<<<(unsigned)other.size(), 256, 0, st>>>(T, state_of(src), dm + own.size());
  CK(cudaGetLastError());
  const bool forces_ok = (nkeep == 0 || h->forces_valid) && (nsel == 0 || src->forces_valid);
  // the new layout; per-atom arrays grow only when the capacity is exceeded
  CK(cudaStreamSynchronize(st));
  // the new segments first: a growing allocation estimates the list
  // capacities from their volume
  h->segs = segs;
  h->seg_counts = counts;
  h->have_box = true;
  int rc = alloc_atoms(h, (int)n_new);
  if (!rc) {
    h->n = (int)n_new;
    rc = sync_segments(h);
  }
  if (rc) {
    cudaFreeAsync(tmp, st);
    cudaStreamSynchronize(st);
    return rc;
  }
  // the temporaries hold the new layout with stride n_new: one copy each
  const Dev &d = h->d;
  CK(cudaMemcpyAsync(d.x_o, T.x, 3 * N * sizeof(double), cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(d.v_o, T.v, 3 * N * sizeof(double), cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(d.f_o, T.f, 3 * N * sizeof(double), cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(d.q_o, T.q, N * sizeof(double), cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(d.s_hist, T.sh, 5 * N * sizeof(double), cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(d.t_hist, T.th, 5 * N * sizeof(double), cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(d.type_o, T.type, N * sizeof(int), cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(d.tag_o, T.tag, N * sizeof(int), cudaMemcpyDeviceToDevice, st));
  CK(cudaFreeAsync(tmp, st));
  CK(cudaStreamSynchronize(st));
  h->lists_valid = false;
  h->forces_valid = forces_ok;
  h->tallies_valid = false;
  h->seg_iters.clear();
  return RG_OK;
}

int rg_get_segment_atoms(rg_system *h, int seg, double *x, double *v, double *q, double *f) {
  if (!h) return RG_E_ARG;
  if (seg < 0 || seg >= (int)h->segs.size()) return fail(h, RG_E_ARG, "segment index out of range");
  if (!h->n) return fail(h, RG_E_STATE, "no atoms set");
  CK(cudaSetDevice(h->p.device));
  const SegGeom &g = h->segs[seg];
  const size_t a0 = (size_t)g.atom0, c = (size_t)g.natoms;
  const Dev &d = h->d;
  if (x) CK(cudaMemcpyAsync(x, d.x_o + 3 * a0, 3 * c * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  if (v) CK(cudaMemcpyAsync(v, d.v_o + 3 * a0, 3 * c * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  if (q) CK(cudaMemcpyAsync(q, d.q_o + a0, c * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  if (f) CK(cudaMemcpyAsync(f, d.f_o + 3 * a0, 3 * c * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return RG_OK;
}

int rg_get_segment_iters(rg_system *h, int *iters) {
  if (!h || !iters) return RG_E_ARG;
  for (size_t k = 0; k < h->seg_iters.size(); ++k) iters[k] = h->seg_iters[k];
  return RG_OK;
}

static int set_atoms_impl(rg_system *h, int n, const double *x, const int *type, const int *tag,
                          const double *q, const double *v, cudaMemcpyKind kind) {
  if (!h) return RG_E_ARG;
  if (!h->have_box) return fail(h, RG_E_STATE, "rg_set_box must precede rg_set_atoms");
  if (n <= 0 || n >= (1 << 24) || !x || !type) return fail(h, RG_E_ARG, "bad atom arrays");
  CK(cudaSetDevice(h->p.device));
  if (kind == cudaMemcpyHostToDevice) {
    for (int i = 0; i < n; ++i)
      if (type[i] < 0 || type[i] >= h->ff.ntypes) return fail(h, RG_E_ARG, "atom type out of range");
    for (long long k = 0; k < 3LL * n; ++k)
      if (!std::isfinite(x[k])) return fail(h, RG_E_ARG, "non-finite position");
  }
  {
    long long sum = 0;
    for (int c : h->seg_counts) sum += c < 0 ? n : c;
    if (sum != n) return fail(h, RG_E_ARG, "segment atom counts do not add up to the atom count");
  }
  {
    int rc = alloc_atoms(h, n);
    if (rc) return rc;
  }
  h->n = n;
  {
    int rc = sync_segments(h);
    if (rc) return rc;
  }
  Dev &d = h->d;
  CK(cudaMemcpyAsync(d.x_o, x, 3 * sizeof(double) * n, kind, h->st));
  CK(cudaMemcpyAsync(d.type_o, type, sizeof(int) * n, kind, h->st));
  if (tag) {
    CK(cudaMemcpyAsync(d.tag_o, tag, sizeof(int) * n, kind, h->st));
  } else {
    std::vector<int> t(n);
    for (int i = 0; i < n; ++i) t[i] = i + 1;
    CK(cudaMemcpyAsync(d.tag_o, t.data(), sizeof(int) * n, cudaMemcpyHostToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
  }
  if (q) CK(cudaMemcpyAsync(d.q_o, q, sizeof(double) * n, kind, h->st));
  else CK(cudaMemsetAsync(d.q_o, 0, sizeof(double) * n, h->st));
  if (v) CK(cudaMemcpyAsync(d.v_o, v, 3 * sizeof(double) * n, kind, h->st));
  else CK(cudaMemsetAsync(d.v_o, 0, 3 * sizeof(double) * n, h->st));
  CK(cudaMemsetAsync(d.s_hist, 0, 5 * sizeof(double) * n, h->st));
  CK(cudaMemsetAsync(d.t_hist, 0, 5 * sizeof(double) * n, h->st));
  CK(cudaMemsetAsync(d.f_o, 0, 3 * sizeof(double) * n, h->st));
  CK(cudaStreamSynchronize(h->st));
  h->n = n;
  h->lists_valid = false;
  h->forces_valid = false;
  return RG_OK;
}

int rg_set_atoms(rg_system *h, int n, const double *x, const int *type, const int *tag,
                 const double *q, const double *v) {
  return set_atoms_impl(h, n, x, type, tag, q, v, cudaMemcpyHostToDevice);
}

int rg_set_atoms_device(rg_system *h, int n, const double *x, const int *type, const int *tag,
                        const double *q, const double *v) {
  return set_atoms_impl(h, n, x, type, tag, q, v, cudaMemcpyDeviceToDevice);
}

int rg_set_positions(rg_system *h, const double *x) {
  if (!h || !x) return RG_E_ARG;
  if (!h->n) return fail(h, RG_E_STATE, "no atoms set");
  CK(cudaMemcpyAsync(h->d.x_o, x, 3 * sizeof(double) * h->n, cudaMemcpyHostToDevice, h->st));
  h->lists_valid = false;
  h->forces_valid = false;
  return RG_OK;
}

int rg_qeq(rg_system *h, double *q_out, int *iters_s, int *iters_t) {
  if (!h) return RG_E_ARG;
  if (!h->n) return fail(h, RG_E_STATE, "no atoms set");
  CK(cudaSetDevice(h->p.device));
  int rc = do_qeq(h, iters_s, iters_t);
  if (rc) return rc;
  if (q_out) {
    CK(cudaMemcpyAsync(q_out, h->d.q_o, sizeof(double) * h->n, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
  }
  return RG_OK;
}

int rg_single_point(rg_system *h, int eflag, int vflag, double *q_out, double *f_out,
                    double *energies) {
  if (!h) return RG_E_ARG;
  if (!h->n) return fail(h, RG_E_STATE, "no atoms set");
  CK(cudaSetDevice(h->p.device));
  const int atom_tally = (eflag & 2) || (vflag & 4);
  const int ef = eflag || energies != nullptr, vf = vflag & 3;
  const int flags = ef | (vf << 4) | (atom_tally << 8);
  Dev &d = h->d;
  int rc;
  // the graph holds the device arrays, sizes and flags of its capture, and
  // the cell grid of the boxes then: the host-side grid set-up runs first
  // (a changed grid changes the arrays or sizes, so the step is recaptured)
  if (h->use_graphs && h->sp.exec && (rc = setup_cells(h))) return rc;
  d.vflag = vf ? 1 : 0;
  d.atom_tally = atom_tally ? 1 : 0;
  const bool eligible = h->use_graphs && !h->prof.on && !h->check_finite && !h->sp.failed;
  bool done = false;
  if (eligible && step_matches(h, h->sp, flags, 0.0)) {
    rc = replay_step(h, h->sp, atom_tally != 0);
    if (rc < 0) return rc;
    done = rc == 0;
  }
  if (!done) {
    if ((rc = do_qeq(h, nullptr, nullptr))) return rc;
    if ((rc = do_compute(h, ef, vf, atom_tally))) return rc;
    h->tallies_valid = atom_tally != 0;
    int st[RG_NSTATUS];
    if ((rc = read_status(h, st))) return rc;
    if (st[ST_NAN]) return fail(h, RG_E_NUMERIC, "non-finite force");
    maybe_capture(h, h->sp, ef, vf, atom_tally, 0.0);
  }
  if (q_out) CK(cudaMemcpyAsync(q_out, d.q_o, sizeof(double) * h->n, cudaMemcpyDeviceToHost, h->st));
  if (f_out) CK(cudaMemcpyAsync(f_out, d.f_o, 3 * sizeof(double) * h->n, cudaMemcpyDeviceToHost, h->st));
  if (energies && (rc = energy_sum(h, energies))) return rc;
  CK(cudaStreamSynchronize(h->st));
  return RG_OK;
}

int rg_compute(rg_system *h, int eflag, int vflag, double *f_out, double *energies) {
  if (!h) return RG_E_ARG;
  if (!h->n) return fail(h, RG_E_STATE, "no atoms set");
  CK(cudaSetDevice(h->p.device));
  // LAMMPS's flag bits: eflag 1 global energy, 2 per-atom energy; vflag 1|2
  // global virial, 4 per-atom virial
  const int atom_tally = (eflag & 2) || (vflag & 4);
  int rc = do_compute(h, eflag || energies != nullptr, vflag & 3, atom_tally);
  if (rc) return rc;
  h->tallies_valid = atom_tally != 0;
  if (f_out) CK(cudaMemcpyAsync(f_out, h->d.f_o, 3 * sizeof(double) * h->n, cudaMemcpyDeviceToHost, h->st));
  if (energies && (rc = energy_sum(h, energies))) return rc;
  int st[RG_NSTATUS];
  if ((rc = read_status(h, st))) return rc;
  if (st[ST_NAN]) return fail(h, RG_E_NUMERIC, "non-finite force");
  return RG_OK;
}

int rg_nve_initial(rg_system *h, double dt) {
  if (!h) return RG_E_ARG;
  if (!h->n) return fail(h, RG_E_STATE, "no atoms set");
  launch_nve_initial(h->d, h->st, dt);
  CK(cudaGetLastError());
  h->lists_valid = false;
  h->forces_valid = false;
  return RG_OK;
}

int rg_nve_final(rg_system *h, double dt) {
  if (!h) return RG_E_ARG;
  if (!h->n) return fail(h, RG_E_STATE, "no atoms set");
  launch_nve_final(h->d, h->st, dt);
  CK(cudaGetLastError());
  return RG_OK;
}

int rg_run(rg_system *h, int nsteps, double dt, double *energies) {
  if (!h || nsteps < 0) return RG_E_ARG;
  if (!h->n) return fail(h, RG_E_STATE, "no atoms set");
  CK(cudaSetDevice(h->p.device));
  int rc;
  if (!h->forces_valid) {  // Verlet setup: pre_force + force
    if ((rc = do_qeq(h, nullptr, nullptr))) return rc;
    if ((rc = do_compute(h, 1))) return rc;
  }
  Dev &d = h->d;
  for (int s = 0; s < nsteps; ++s) {
    const int ef = energies != nullptr && s == nsteps - 1;
    // a whole step as one replay of the captured MD step (same arrays,
    // flags and time step), else the regular launches
    bool done = false;
    const bool eligible = h->use_graphs && !h->prof.on && !h->check_finite && !h->md.failed;
    if (eligible && h->md.exec && (rc = setup_cells(h))) return rc;
    d.vflag = 0;
    d.atom_tally = 0;
    if (eligible && step_matches(h, h->md, ef, dt)) {
      rc = replay_step(h, h->md, false);
      if (rc < 0) return rc;
      done = rc == 0;
    }
    if (done) continue;
    { Scope sc(h, PH_NVE, 1); launch_nve_initial(h->d, h->st, dt); }
    h->lists_valid = false;
    h->forces_valid = false;
    if ((rc = do_qeq(h, nullptr, nullptr))) return rc;
    if ((rc = do_compute(h, ef))) return rc;
    { Scope sc(h, PH_NVE, 1); launch_nve_final(h->d, h->st, dt); }
    if (eligible) {
      // the capture sees the arrays this step settled on; it runs after the
      // step's work is queued and launches nothing
      maybe_capture(h, h->md, ef, 0, 0, dt);
    }
  }
  if (energies && (rc = energy_sum(h, energies))) return rc;
  CK(cudaStreamSynchronize(h->st));
  CK(cudaGetLastError());
  return RG_OK;
}

int rg_set_state(rg_system *h, const double *x, const double *v, const double *f) {
  if (!h || !x) return RG_E_ARG;
  if (!h->n) return fail(h, RG_E_STATE, "no atoms set");
  CK(cudaMemcpyAsync(h->d.x_o, x, 3 * sizeof(double) * h->n, cudaMemcpyHostToDevice, h->st));
  if (v) CK(cudaMemcpyAsync(h->d.v_o, v, 3 * sizeof(double) * h->n, cudaMemcpyHostToDevice, h->st));
  if (f) CK(cudaMemcpyAsync(h->d.f_o, f, 3 * sizeof(double) * h->n, cudaMemcpyHostToDevice, h->st));
  h->lists_valid = false;
  h->forces_valid = f != nullptr;
  return RG_OK;
}

int rg_get_histories(rg_system *h, double *s_hist, double *t_hist) {
  if (!h || !s_hist || !t_hist) return RG_E_ARG;
  if (!h->n) return fail(h, RG_E_STATE, "no atoms set");
  const size_t b = 5 * sizeof(double) * h->n;
  CK(cudaMemcpyAsync(s_hist, h->d.s_hist, b, cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(t_hist, h->d.t_hist, b, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return RG_OK;
}

int rg_set_histories(rg_system *h, const double *s_hist, const double *t_hist) {
  if (!h) return RG_E_ARG;
  if (!h->n) return fail(h, RG_E_STATE, "no atoms set");
  const size_t b = 5 * sizeof(double) * h->n;
  if (s_hist) CK(cudaMemcpyAsync(h->d.s_hist, s_hist, b, cudaMemcpyHostToDevice, h->st));
  else CK(cudaMemsetAsync(h->d.s_hist, 0, b, h->st));
  if (t_hist) CK(cudaMemcpyAsync(h->d.t_hist, t_hist, b, cudaMemcpyHostToDevice, h->st));
  else CK(cudaMemsetAsync(h->d.t_hist, 0, b, h->st));
  CK(cudaStreamSynchronize(h->st));
  return RG_OK;
}

void *rg_stream(rg_system *h) { return h ? (void *)h->st : nullptr; }

int rg_profile_enable(rg_system *h, int on) {
  if (!h) return RG_E_ARG;
  if (on) h->prof.reset();
  else h->prof.resolve();
  h->prof.on = on != 0;
  return RG_OK;
}

int rg_profile_phases(rg_system *h, unsigned mask) {
  if (!h) return RG_E_ARG;
  h->prof.resolve();
  h->prof.mask = mask;
  return RG_OK;
}

int rg_profile_get(rg_system *h, int max, char *names, double *ms, long long *count) {
  if (!h) return RG_E_ARG;
  h->prof.resolve();
  const int k = std::min(max, (int)PH_N);
  for (int i = 0; i < k; ++i) {
    if (names) std::snprintf(names + 32 * i, 32, "%s", kPhaseNames[i]);
    if (ms) ms[i] = h->prof.ms[i];
    if (count) count[i] = h->prof.cnt[i];
  }
  return PH_N;
}

int rg_get_atoms(rg_system *h, double *x, double *v, double *q, double *f) {
  if (!h) return RG_E_ARG;
  const int n = h->n;
  if (x) CK(cudaMemcpyAsync(x, h->d.x_o, 3 * sizeof(double) * n, cudaMemcpyDeviceToHost, h->st));
  if (v) CK(cudaMemcpyAsync(v, h->d.v_o, 3 * sizeof(double) * n, cudaMemcpyDeviceToHost, h->st));
  if (q) CK(cudaMemcpyAsync(q, h->d.q_o, sizeof(double) * n, cudaMemcpyDeviceToHost, h->st));
  if (f) CK(cudaMemcpyAsync(f, h->d.f_o, 3 * sizeof(double) * n, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return RG_OK;
}

int rg_device_arrays(rg_system *h, double **x, double **v, double **q, double **f) {
  if (!h) return RG_E_ARG;
  if (x) *x = h->d.x_o;
  if (v) *v = h->d.v_o;
  if (q) *q = h->d.q_o;
  if (f) *f = h->d.f_o;
  return RG_OK;
}

int rg_get_stats(const rg_system *h, rg_stats *s) {
  if (!h || !s) return RG_E_ARG;
  *s = h->stats;
  s->n_atoms = h->n;
  s->kernel_launches = h->launches;
  s->fp64_angles = s->fp64_torsions = 0;
  s->cell_div = h->cell_div;
  s->spmv_rows = h->d.spmv_rw;
  s->pair_kernel = h->d.nbr_tiles ? 2 : 1;
  if (h->d.mixed && h->d.fb_cnt) {
    int fb[2] = {0, 0};
    if (cudaMemcpyAsync(fb, h->d.fb_cnt, sizeof fb, cudaMemcpyDeviceToHost, h->st) == cudaSuccess &&
        cudaStreamSynchronize(h->st) == cudaSuccess) {
      s->fp64_angles = fb[0];
      s->fp64_torsions = fb[1];
    }
  }
  return RG_OK;
}

int rg_synchronize(rg_system *h) {
  if (!h) return RG_E_ARG;
  CK(cudaStreamSynchronize(h->st));
  return RG_OK;
}

}  // extern "C"

void rg_set_error(rg_system *h, const std::string &msg) {
  if (h) h->err = msg;
}

void rg_noalloc_tables(const rg_system *h, const ForceField **ff, const Control **ctl,
                       int *device, double *swb, double *tol, int *imax) {
  *ff = h->d_ff;
  *ctl = h->d_ctl;
  *device = h->p.device;
  *swb = h->p.qeq_swb;
  *tol = h->p.qeq_tol;
  *imax = h->p.qeq_imax;
}

// ------------------------------------------------------------------
// list dumps (host side, for parity checks)

namespace {

int oracle_img(int c) {
  int sx, sy, sz;
  img_unpack(c, &sx, &sy, &sz);
  return (sx + 8) | ((sy + 8) << 4) | ((sz + 8) << 8);
}

template <class T>
std::vector<T> fetch(rg_system *h, const T *p, size_t count) {
  std::vector<T> v(count);
  if (count) cudaMemcpyAsync(v.data(), p, count * sizeof(T), cudaMemcpyDeviceToHost, h->st);
  cudaStreamSynchronize(h->st);
  return v;
}

}  // namespace

extern "C" long long rg_dump_pairs(rg_system *h, int *ti, int *tj, int *img) {
  if (!h || !h->lists_valid) return -1;
  const Dev &d = h->d;
  const int n = d.n, cap = d.nb_cap;
  auto nn = fetch(h, d.n_near, n), nf = fetch(h, d.n_far, n);
  long long tot = 0;
  for (int i = 0; i < n; ++i) tot += nn[i] + nf[i];
  if (!ti) return tot;
  auto tags = fetch(h, d.tags, n);
  auto nbr = fetch(h, d.nbr, (size_t)n * cap);
  long long k = 0;
  for (int i = 0; i < n; ++i)
    for (int p = 0; p < nn[i] + nf[i]; ++p) {
      const int slot = p < nn[i] ? p : d.nb_capN + (p - nn[i]);
      const uint32_t e = nbr[(size_t)i * cap + slot];
      ti[k] = tags[i];
      tj[k] = tags[e >> 8];
      img[k] = oracle_img((int)(e & 255u));
      ++k;
    }
  return k;
}

extern "C" long long rg_dump_bonds(rg_system *h, int *ti, int *tj, int *img, double *bo) {
  if (!h || !h->forces_valid) return -1;
  const Dev &d = h->d;
  const int n = d.n;
  auto nb = fetch(h, d.nbonds, n);
  long long tot = 0;
  for (int i = 0; i < n; ++i) tot += nb[i];
  if (!ti) return tot;
  const size_t S = (size_t)n * d.bond_cap;
  auto tags = fetch(h, d.tags, n);
  auto bn = fetch(h, d.b_nbr, S);
  auto BO = fetch(h, d.b_BO, S), BOs = fetch(h, d.b_BOs, S);
  auto BOpi = fetch(h, d.b_BOpi, S), BOpi2 = fetch(h, d.b_BOpi2, S);
  long long k = 0;
  for (int i = 0; i < n; ++i)
    for (int q = 0; q < nb[i]; ++q) {
      const size_t s = (size_t)q * n + i;
      ti[k] = tags[i];
      tj[k] = tags[bn[s] >> 8];
      img[k] = oracle_img((int)(bn[s] & 255u));
      if (bo) {
        bo[4 * k + 0] = BO[s];
        bo[4 * k + 1] = BOs[s];
        bo[4 * k + 2] = BOpi[s];
        bo[4 * k + 3] = BOpi2[s];
      }
      ++k;
    }
  return k;
}

// FindBond (fix_reaxc_bonds_sunway.cpp:196-223) and PassBuffer (:226-255):
// per atom (original order) the partners with corrected BO > bo_cut, their
// bond orders, the total bond order (bo_dboc[i][0]) and the lone pairs.
extern "C" int rg_bond_table(rg_system *h, double bo_cut, int max_per_atom, int *nbond,
                             int *nbr_tag, double *bo, double *total_bo, double *nlp) {
  if (!h || max_per_atom <= 0) return RG_E_ARG;
  // bond orders belong to the positions of the last force step
  if (!h->forces_valid || !h->lists_valid)
    return fail(h, RG_E_STATE, "no force step since the last state change");
  const Dev &d = h->d;
  const int n = d.n;
  auto nb = fetch(h, d.nbonds, n);
  auto tags = fetch(h, d.tags, n);
  auto perm = fetch(h, d.perm, n);
  const size_t S = (size_t)n * d.bond_cap;
  auto bn = fetch(h, d.b_nbr, S);
  auto BO = fetch(h, d.b_BO, S);
  auto tb = fetch(h, d.bo0, n);
  auto lp = fetch(h, d.nlp, n);
  int most = 0;
  for (int i = 0; i < n; ++i) {
    const int o = perm[i];
    int c = 0;
    for (int q = 0; q < std::min(nb[i], d.bond_cap); ++q) {
      const size_t s = (size_t)q * n + i;
      if (BO[s] > bo_cut) {
        if (c < max_per_atom) {
          if (nbr_tag) nbr_tag[(size_t)o * max_per_atom + c] = tags[bn[s] >> 8];
          if (bo) bo[(size_t)o * max_per_atom + c] = BO[s];
        }
        ++c;
      }
    }
    if (nbond) nbond[o] = std::min(c, max_per_atom);
    if (total_bo) total_bo[o] = tb[i];
    if (nlp) nlp[o] = lp[i];
    most = std::max(most, c);
  }
  return most;
}

extern "C" long long rg_dump_hbonds(rg_system *h, int *ti, int *tj, int *img) {
  if (!h || !h->lists_valid) return -1;
  const Dev &d = h->d;
  const int n = d.n;
  auto nh = fetch(h, d.nhb, n);
  long long tot = 0;
  for (int i = 0; i < n; ++i) tot += nh[i];
  if (!ti) return tot;
  auto tags = fetch(h, d.tags, n);
  auto hb = fetch(h, d.hb_nbr, (size_t)n * d.hb_cap);
  long long k = 0;
  for (int i = 0; i < n; ++i)
    for (int q = 0; q < nh[i]; ++q) {
      const uint32_t e = hb[(size_t)i * d.hb_cap + q];
      ti[k] = tags[i];
      tj[k] = tags[e >> 8];
      img[k] = oracle_img((int)(e & 255u));
      ++k;
    }
  return k;
}

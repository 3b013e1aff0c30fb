/*
 * CPU oracle for the ReaxFF force step (TEST INFRASTRUCTURE ONLY).
 *
 * A plain-C, single-threaded restatement of the reference's CPU path
 * (SW_REAXFF: the `#else` host branches of the *_sw64.c files and the C++
 * host code they are called from).  Like the reference it works on an
 * extended atom array of local atoms plus periodic ghost images, builds a
 * full far-neighbour list for every atom, a full two-direction bond list
 * sorted by neighbour index and an H-bond list, and evaluates every term
 * once per local centre.  Ghost forces are folded back onto their owners at
 * the end (LAMMPS reverse communication).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
 * this code, and only as the checker or the timed CPU baseline.  The
 * product library never links it.
 */
#ifndef REAX_ORACLE_H
#define REAX_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ro_ctx ro_ctx;

/* run-time controls; ro_default_control() fills the reference defaults of
 * `pair_style reax/c NULL` (pair_reaxc_sunway.cpp:208-242) and
 * `fix qeq/reax 1 0.0 10.0 1e-6 reax/c` */
typedef struct {
  double bond_cut;      /* 5.0   */
  double hbond_cut;     /* 7.5   */
  double thb_cut;       /* 0.001 */
  double thb_cutsq;     /* 1e-5  */
  double skin;          /* 2.5: ghost cutoff = cutmax + skin */
  int enobondsflag;     /* 1 */
  int lgflag;           /* 0 */
  double qeq_swa;       /* 0.0  */
  double qeq_swb;       /* 10.0 */
  double qeq_tol;       /* 1e-6 */
  int qeq_imax;         /* 200  */
} ro_control;

void ro_default_control(ro_control *c);

/* Energy vector layout returned by ro_compute (first 14 = pvector order of
 * pair_reaxc_sunway.cpp:657-670, then tallied eng_vdwl, eng_coul, then the
 * physical (un-prefix-summed) polarisation energy). */
enum { RO_E_BOND = 0, RO_E_OVUN, RO_E_LP, RO_E_3, RO_E_ANG, RO_E_PEN,
       RO_E_COA, RO_E_HB, RO_E_TOR, RO_E_CON, RO_E_VDW, RO_E_ELE, RO_E_12,
       RO_E_POL, RO_ENG_VDWL, RO_ENG_COUL, RO_E_POL_PHYS, RO_NENERGY };

ro_ctx *ro_create(const char *ffield_path, const ro_control *ctl,
                  char *errbuf, int errlen);
void ro_destroy(ro_ctx *c);

int ro_num_types(const ro_ctx *c);
/* per-ffield-type parameter lookup: what = "mass","chi","eta","gamma" */
double ro_type_param(const ro_ctx *c, int type, const char *what);
double ro_global_param(const ro_ctx *c, int idx);

/* Set the periodic orthogonal box [0,L) and the local atoms.  type is the
 * 0-based ffield element index, tag the 1-based global id.  Positions are
 * wrapped into the box. */
/* Tilts (xy, xz, yz) of a triclinic cell for the next ro_set_system (NULL:
 * orthogonal). */
void ro_set_tilt(ro_ctx *c, const double *tilt3);
int ro_set_system(ro_ctx *c, int n, const double *box3, const double *x,
                  const int *type, const int *tag, const double *q,
                  const double *v);

/* QEq (fix qeq/reax pre_force): solves s and t, writes q (local order),
 * returns iterations of the s and t solves. */
int ro_qeq(ro_ctx *c, double *q_out, int *iters_s, int *iters_t);

/* Force step (pair reax/c compute with eflag=1, vflag=0): forces on the
 * local atoms (ghost forces folded back), energies[RO_NENERGY]. */
int ro_compute(ro_ctx *c, double *f_out, double *energies);

/* NVE velocity Verlet over nsteps (setup: qeq + compute, then per step:
 * initial_integrate, qeq, compute, final_integrate), dt in fs, real units. */
int ro_run_nve(ro_ctx *c, int nsteps, double dt, double *energies_last);
/* nsteps more NVE steps continuing from the current state (forces, charges
 * and QEq histories of the previous step; no setup evaluation) */
int ro_md_steps(ro_ctx *c, int nsteps, double dt, double *energies_last);

void ro_get_state(const ro_ctx *c, double *x, double *v, double *q,
                  double *f);

/* per-atom tallies of the last ro_compute, as LAMMPS's eatom/vatom with
 * eflag_atom/vflag_atom: only the nonbonded pair terms tally per atom in
 * the reference (ev_tally_full, reaxc_nonbonded_sw64.c:198-213): eatom[i] =
 * sum over i's full list of (E_vdW + E_ele)/2, vatom[6i..6i+5] = sum of
 * del (x) del fpair / 2 (xx yy zz xy xz yz), del = x_i - x_j */
void ro_atom_tallies(const ro_ctx *c, double *eatom, double *vatom);

/* list statistics from the last ro_compute / ro_qeq */
typedef struct {
  long long n_local, n_total, n_far_local, n_far_total, n_bonds_total,
      n_bonds_local, n_hbonds, n_H_entries;
} ro_stats;
void ro_get_stats(const ro_ctx *c, ro_stats *s);

/* List dumps for set comparison.  Each entry: (tag_i, tag_j, image code)
 * where image code = (sx+8) | (sy+8)<<4 | (sz+8)<<8 is the periodic image
 * of j relative to the local owner of i.  Returns the entry count; the
 * arrays may be NULL to query the size. */
long long ro_dump_far(const ro_ctx *c, int *ti, int *tj, int *img);
long long ro_dump_bonds(const ro_ctx *c, int *ti, int *tj, int *img,
                        double *bo /* corrected BO, 4 per entry:
                                      BO, BO_s, BO_pi, BO_pi2 */);
long long ro_dump_hbonds(const ro_ctx *c, int *ti, int *tj, int *img);

/* per-local-atom intermediate quantities after ro_compute:
 * out[n*8]: Deltap, Delta, Delta_e, Delta_boc, Delta_val, Delta_lp, nlp,
 *           CdDelta (total, after folding ghosts). */
void ro_dump_atom_terms(const ro_ctx *c, double *out);

double ro_last_time(const ro_ctx *c, int phase);

#ifdef __cplusplus
}
#endif
#endif

/*
 * reaxgpu -- GB300 (sm_103a) ReaxFF force step behind a C ABI.
 *
 * This is the seam that replaces the reference's per-kernel C entry points
 * (`extern "C" void X_C(pack*)`, reaxc_ctypes_sunway.h:915-1074) and the
 * LAMMPS plugin classes above them.  A LAMMPS `pair_style reax/c/...`,
 * `fix qeq/reax/...` and `fix nve/...` wrapper calls these functions; the
 * mapping is, per entry point:
 *
 *   rg_create        PairReaxCSunway::settings + coeff (Read_Force_Field,
 *                    pair_reaxc_sunway.cpp:202-362, reaxc_ffield_sunway.cpp:35)
 *   rg_extract       PairReaxCSunway::extract("chi"/"eta"/"gamma"),
 *                    pair_reaxc_sunway.cpp:1106-1128
 *   rg_set_box /
 *   rg_set_atoms     write_reax_atoms + the LAMMPS atom arrays x/type/tag/q/v
 *                    (pair_reaxc_sunway.cpp:797-831)
 *   rg_qeq           FixQEqReaxSunway::pre_force, fix_qeq_reax_sunway.cpp:539-600
 *   rg_compute       PairReaxCSunway::compute(eflag, vflag),
 *                    pair_reaxc_sunway.cpp:541-793
 *   rg_nve_initial   FixNVESunway::initial_integrate, fix_nve_sunway.cpp:67-100
 *   rg_nve_final     FixNVESunway::final_integrate, fix_nve_sunway.cpp:102-135
 *   rg_run           the Verlet loop those classes are driven by (LAMMPS
 *                    Verlet::run): initial_integrate -> pre_force (QEq) ->
 *                    pair compute -> final_integrate, all on the device
 *
 * All functions return 0 on success and a negative RG_E_* code on error
 * (the reference aborts through error->all / MPI_Abort instead;
 * reaxc_defs_sunway.h:148-151).  rg_last_error() gives the message.  A
 * handle owns one CUDA stream and its device memory; handles are not
 * thread-safe, distinct handles may be used from distinct threads.
 *
 * Units are LAMMPS real: Angstrom, fs, g/mol, kcal/mol, electron charge.
 */
#ifndef REAXGPU_H
#define REAXGPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rg_system rg_system;

enum {
  RG_OK = 0,
  RG_E_ARG = -1,        /* invalid argument                        */
  RG_E_FILE = -2,       /* force field unreadable / inconsistent   */
  RG_E_CUDA = -3,       /* CUDA runtime error                      */
  RG_E_CAPACITY = -4,   /* list capacity could not be grown        */
  RG_E_STATE = -5,      /* call order (e.g. no atoms set)          */
  RG_E_NUMERIC = -6     /* non-finite result detected              */
};

enum { RG_PREC_FP64 = 0, RG_PREC_MIXED = 1 };

/* Run-time controls.  rg_default_params() gives the reference defaults of
 * `pair_style reax/c NULL` (pair_reaxc_sunway.cpp:208-242) and
 * `fix qeq/reax 1 0.0 10.0 1.0e-6 reax/c`. */
typedef struct {
  double bond_cut;      /* 5.0   near-neighbour cutoff for bonds        */
  double hbond_cut;     /* 7.5   hydrogen-bond partner cutoff           */
  double thb_cut;       /* 0.001 three/four-body bond-order cutoff      */
  double thb_cutsq;     /* 1e-5                                         */
  int enobondsflag;     /* 1     e_un/e_lp also for atoms without bonds */
  int lgflag;           /* 0     low-gradient vdW correction            */
  double qeq_swa;       /* 0.0   QEq taper inner radius                 */
  double qeq_swb;       /* 10.0  QEq taper outer radius                 */
  double qeq_tol;       /* 1e-6  CG relative tolerance                  */
  int qeq_imax;         /* 200   CG iteration limit                     */
  int precision;        /* RG_PREC_FP64: FP64 accuracy throughout (list
                           decisions, bond orders, angles, accumulations
                           in FP64; the tabulated pair functions, the
                           pair forces and the QEq SpMV of orthogonal
                           boxes as FP32 pairs, ~1e-13 relative);
                           RG_PREC_MIXED: pair, H-bond, angle and SpMV
                           arithmetic in FP32 (forces ~1e-6 relative to
                           the FP64 form, charges ~5e-6 e)                */
  int device;           /* CUDA device ordinal                          */
  int tabulate;         /* vdW+Coulomb (both forms; the mixed form reads
                           an FP32 copy) and the FP64 form's QEq H from
                           cubic Hermite tables in r^2 with this many
                           intervals per type pair (the reference's control
                           "tabulate_long_range", off in its NULL control);
                           0 = analytic.  Default 65536: ~1e-10 of the
                           analytic pair functions (rg_table_check). */
  int tabulate_check;   /* 1: measure the tables' error at rg_create
                           (rg_table_info); 0 (default): skip */
  int autotune;         /* 1 (default): at the first list build of a handle
                           (and when its atom count changes by 4x) time the
                           cell division (cells of cutoff/2 or cutoff/3) and
                           the QEq SpMV's lanes per row (8, 16, 32) on the
                           system and keep the fastest; 0: cutoff/2 and 16 */
  int cell_div;         /* 0 (default): as above; 2 or 3: cells of cutoff/2
                           or cutoff/3 (3 only where every cell width is at
                           least the cutoff), not tuned */
  int spmv_rows;        /* 0 (default): as above; 8, 16 or 32: fixed */
  int pair_kernel;      /* pair-list build: 0 (default) autotuned with the
                           cell division (the warp walk when autotuning is
                           off); 1 one warp per atom; 2 per-cell tiles staged
                           in shared memory */
} rg_params;

/* Energy vector of rg_compute: entries 0..13 are the pair's pvector in the
 * reference order (pair_reaxc_sunway.cpp:657-670): e_bond, e_ov+e_un, e_lp,
 * 0, e_ang, e_pen, e_coa, e_hb, e_tor, e_con, e_vdW, e_ele, 0, e_pol; then
 * the tallied eng_vdwl and eng_coul, then the physical polarisation sum.
 * As in the reference, e_vdW and e_ele are summed over the full neighbour
 * list (twice the physical value) and e_pol is the reference's running-sum
 * value; eng_vdwl + eng_coul is the potential energy. */
enum { RG_NENERGY = 17 };

typedef struct {
  long long n_atoms, n_pairs, n_bonds, n_hbond_pairs, n_H_entries;
  int cg_iters_s, cg_iters_t;
  int max_nbrs, max_bonds, max_hbonds;
  int regrows;
  long long kernel_launches;   /* kernels launched by this handle so far */
  int qeq_restarts;            /* mixed form: residual checks of the last
                                  QEq (1 = converged at the first check) */
  int fp64_angles, fp64_torsions; /* mixed form: valence angles and torsions
                                  of the last force step evaluated by the
                                  FP64 passes (near-linear, over-coordinated) */
  int cell_div, spmv_rows;     /* the configuration in use (autotuned): cells
                                  of cutoff/cell_div, SpMV lanes per row */
  long long cg_system_iters;   /* since rg_create: CG loop iterations summed
                                  over the QEq calls and their two systems
                                  (each is one system's SpMV over the matrix;
                                  per call: (iters_s - 1) + (iters_t - 1),
                                  the slowest segment's counts) */
  long long cg_spmv_rows_passes; /* since rg_create: CG loop SpMV launches
                                  that had a system to update (per call:
                                  max(iters_s, iters_t) - 1) */
  long long step_graph_replays; /* rg_single_point calls served by one replay
                                  of the captured step */
  long long step_graph_redos;  /* replays that met a list past its capacity
                                  and redid the step on the regular path */
  int pair_kernel;             /* the pair-list build in use: 1 warp per atom,
                                  2 per-cell tiles */
} rg_stats;

void rg_default_params(rg_params *p);

/* Read the force field and create a handle on p->device. */
int rg_create(const char *ffield_path, const rg_params *p, rg_system **out);
int rg_destroy(rg_system *h);
const char *rg_last_error(const rg_system *h);

/* Element names of a force-field file, read on the host without a device
 * (what pair_coeff needs to map LAMMPS types to elements,
 * pair_reaxc_sunway.cpp:305-340): *ntypes, and if names is not NULL ntypes
 * names of len chars each (upper case).  RG_E_FILE if the file cannot be
 * read; msg (msg_len chars, may be NULL) then gets the reason. */
int rg_ffield_info(const char *path, int *ntypes, char *names, int len, char *msg,
                   int msg_len);

/* FP64 tables: intervals per type pair (0: analytic) and the largest
 * relative deviation of the interpolants from the analytic pair functions,
 * measured when the tables were built. */
int rg_table_info(const rg_system *h, int *intervals, double *max_rel_err);
/* The same check without a device: builds the tables of p->tabulate
 * intervals (p NULL: defaults) for a force field on the host. */
int rg_table_check(const char *ffield_path, const rg_params *p, double *max_rel_err);

int rg_num_types(const rg_system *h);
/* element name of ffield type t (0-based), upper case */
int rg_element_name(const rg_system *h, int t, char *buf, int len);
/* per-type "chi", "eta", "gamma" or "mass" into out[ntypes] */
int rg_extract(const rg_system *h, const char *name, double *out);

/* Per-type masses used by the integrator (g/mol, mass[ntypes] by ffield
 * type): the LAMMPS data file's Masses, which fix nve/sunway reads from
 * atom->mass (fix_nve_sunway.cpp:73-95).  Default: the force field's. */
int rg_set_masses(rg_system *h, const double *mass);

/* Orthogonal periodic box [0,L0)x[0,L1)x[0,L2). */
int rg_set_box(rg_system *h, const double *L3);

/* Triclinic boxes (LAMMPS's restricted form, the shipped TATB deck's
 * `region prism` / data-file `xy xz yz` line): edge vectors a = (lx,0,0),
 * b = (xy,ly,0), c = (xz,yz,lz) with L = (lx,ly,lz) from rg_set_box or
 * rg_set_segments and tilt[3*nseg] = (xy, xz, yz) per segment (zeros: back
 * to orthogonal).  Positions are wrapped into the cell by its fractional
 * coordinates.  Every width of the cell between opposite faces must be at
 * least half the pair cutoff.  Replaces the triclinic ghost images that
 * LAMMPS's Domain/Comm give the reference (outside its tree; the reference
 * sees them as ghost atoms, pair_reaxc_sunway.cpp:797-831), as the shipped
 * TATB deck's prism box needs (in.reaxc.lattice). */
int rg_set_tilt(rg_system *h, const double *tilt);

/* Independent systems in one handle ("segments", for batched evaluation
 * of many small systems): nseg orthogonal periodic boxes (boxes[3*nseg]),
 * segment k holding counts[k] consecutive atoms of the arrays given to
 * rg_set_atoms (whose n must be the sum).  Every call then works on all
 * segments at once: lists, QEq (each segment's own CG scalars and
 * convergence, fix_qeq_reax_sunway.cpp:983-1167 per system), forces and
 * NVE.  rg_set_box is the one-segment case.  rg_compute's energies are the
 * sums over segments; rg_get_energies gives them per segment
 * (e[nseg][RG_NENERGY]) and rg_get_segment_iters the s and t CG iterations
 * of the last QEq per segment (iters[2*nseg]). */
int rg_set_segments(rg_system *h, int nseg, const int *counts, const double *boxes);
int rg_num_segments(const rg_system *h);
int rg_get_energies(rg_system *h, double *e);
int rg_get_segment_iters(rg_system *h, int *iters);

/* Host arrays of n atoms: x[3n] (wrapped into the box), type[n] (0-based
 * ffield type), tag[n] (1-based global id; NULL -> 1..n), q[n] (NULL -> 0),
 * v[3n] (NULL -> 0).  Resets the QEq histories. */
int rg_set_atoms(rg_system *h, int n, const double *x, const int *type,
                 const int *tag, const double *q, const double *v);
/* Same, reading device pointers (no host copies). */
int rg_set_atoms_device(rg_system *h, int n, const double *x,
                        const int *type, const int *tag, const double *q,
                        const double *v);
/* Update positions only (host array), keeping histories. */
int rg_set_positions(rg_system *h, const double *x);
/* Per-step input of a host-driven MD loop (host arrays, original order):
 * positions, and optionally velocities and the forces of those positions
 * (from the previous step), keeping the QEq histories.  With f given the
 * next rg_run continues the Verlet loop without recomputing forces. */
int rg_set_state(rg_system *h, const double *x, const double *v,
                 const double *f);

/* QEq charge equilibration (pre_force).  q_out[n] host or NULL. */
int rg_qeq(rg_system *h, double *q_out, int *iters_s, int *iters_t);

/* Single point: QEq (pre_force) then the force step, as rg_qeq followed by
 * rg_compute with the same flags; q_out[n], f_out[3n], energies
 * [RG_NENERGY] host or NULL.  After a first call on a given set of arrays
 * and flags, the whole step -- binning, pair/bond/H-bond lists, the QEq with
 * its CG iterations (and the mixed form's refinement restarts) as
 * device-side loops, the force step -- replays as one captured CUDA graph,
 * with one host synchronisation at its end.  A replay that finds a list
 * past its capacity restores the QEq histories and redoes the step on the
 * regular path, which regrows.  No counterpart in the reference (it
 * launches each phase from the host); the batched evaluation of many small
 * systems (segments) is its use. */
int rg_single_point(rg_system *h, int eflag, int vflag, double *q_out, double *f_out,
                    double *energies);

/* Force step.  f_out[3n] host or NULL (forces, kcal/mol/A), energies
 * [RG_NENERGY] host or NULL; eflag = 0 skips the energy reductions;
 * vflag & 3 also accumulates the virial (rg_get_virial).  With LAMMPS's
 * per-atom bits, eflag & 2 or vflag & 4, the step also tallies per-atom
 * energy and virial (rg_get_atom_tallies). */
int rg_compute(rg_system *h, int eflag, int vflag, double *f_out,
               double *energies);
/* Virial of the last force step computed with vflag, per segment
 * (v[6*nseg]): sum over atoms of r (x) f in the order xx yy zz xy xz yz,
 * kcal/mol, the quantity LAMMPS's virial[6] holds (virial_fdotr_compute
 * over local + ghost atoms, pair_reaxc_sunway.cpp:674-763). */
int rg_get_virial(rg_system *h, double *v);

/* Per-atom energy and virial of the last rg_compute made with eflag & 2
 * (LAMMPS ENERGY_ATOM) or vflag & 4 (VIRIAL_ATOM), in the caller's atom
 * order: eatom[n] and vatom[6n] (xx yy zz xy xz yz per atom), either may be
 * NULL.  As in the reference, only the nonbonded pair terms tally per atom
 * (ev_tally_full, reaxc_inlines_sw64.h:178-222, called from
 * vdW_Coulomb_Energy_Full_C, reaxc_nonbonded_sw64.c:198-213): each pair
 * within the nonbonded cutoff gives each of its atoms half its vdW +
 * Coulomb energy and half of del (x) del fpair.  The pair style's
 * eatom/vatom (pair_reaxc_sunway.cpp, ev_setup) are filled from these.
 * RG_E_STATE if the last force step did not tally. */
int rg_get_atom_tallies(rg_system *h, double *eatom, double *vatom);

/* Velocity-Verlet halves (dt in fs). */
int rg_nve_initial(rg_system *h, double dt);
int rg_nve_final(rg_system *h, double dt);

/* nsteps of NVE MD entirely on the device: per step initial_integrate,
 * QEq, force step, final_integrate.  energies of the last step or NULL. */
int rg_run(rg_system *h, int nsteps, double dt, double *energies);

/* QEq histories (the s and t solutions of the last 5 solves that seed the
 * extrapolated initial guesses, fix_qeq_reax_sunway.cpp:618-723,1741-1752):
 * host arrays of 5*n doubles, entry k*n + i for solve k (0 = latest) of atom
 * i in the original order.  Moving a system between handles keeps its
 * trajectory with them.  rg_set_histories(h, NULL, NULL) clears them (the
 * next QEq starts from zero guesses, as after rg_set_atoms). */
int rg_get_histories(rg_system *h, double *s_hist, double *t_hist);
int rg_set_histories(rg_system *h, const double *s_hist, const double *t_hist);

/* Read back the current state (host arrays, original atom order). */
int rg_get_atoms(rg_system *h, double *x, double *v, double *q, double *f);
/* Device pointers of the state arrays (original order, 3n/n doubles). */
int rg_device_arrays(rg_system *h, double **x, double **v, double **q,
                     double **f);

int rg_get_stats(const rg_system *h, rg_stats *s);
int rg_synchronize(rg_system *h);
/* The cudaStream_t (as void*) all work of the handle is issued on. */
void *rg_stream(rg_system *h);

/* Phase timing with CUDA events on the handle's stream (the reference
 * times the same phases with GPTL regions, e.g. pair_reaxc_sunway.cpp:
 * 550-792).  rg_profile_enable(h,1) resets and starts; rg_profile_get fills
 * up to max entries of names (32 chars each), milliseconds and interval
 * counts, and returns the number of phases. */
int rg_profile_enable(rg_system *h, int on);
int rg_profile_get(rg_system *h, int max, char *names, double *ms,
                   long long *count);
/* Restrict the events to the phases in mask (bit k = phase k of
 * rg_profile_get's order; default all).  Timing one force-step phase this
 * way adds two event records per step and keeps the QEq iterations in their
 * captured CUDA graph (the QEq iteration phases are timed only with plain
 * launches). */
int rg_profile_phases(rg_system *h, unsigned mask);

/* Continuous batching: rebuild the set of systems of h on the device from
 * keep[nkeep] of its own segments (in that order) followed by sel[nsel]
 * segments of src (another handle on the same device with the same force
 * field, or NULL with nsel = 0).  Every carried system keeps its box, tilt
 * and per-atom state -- positions, velocities, forces, charges, types, tags
 * and the 5-deep s/t QEq histories -- copied device to device; no atom
 * passes through host memory.  A Verlet run (rg_run) continues from the
 * carried forces when every carried system had forces.  src's pending work
 * is waited for on the device; h and src are free again when the call
 * returns.  No counterpart in the reference (one system per LAMMPS run):
 * the segments themselves are this library's batching (rg_set_segments). */
int rg_regroup_segments(rg_system *h, int nkeep, const int *keep, rg_system *src,
                        int nsel, const int *sel);

/* One segment's atoms (host arrays of that segment's atom count; any may be
 * NULL): positions, velocities, charges and the forces of the last step. */
int rg_get_segment_atoms(rg_system *h, int seg, double *x, double *v, double *q, double *f);

/* Allocation-free QEq (no counterpart in the reference).  For callers that
 * cannot call cudaMalloc when they need charges -- code running under a host
 * application's own device-memory manager, or where an allocation would
 * synchronize or fail.  Same charges as rg_qeq's first solve after
 * rg_set_atoms (zero initial guesses), within the CG tolerance, for at most
 * RG_NOALLOC_MAX_ATOMS atoms: H is evaluated on the fly and the CG vectors
 * live in one static device array of that size, held by every GPU that loads
 * the library until exit.  Inputs and output are the caller's device arrays:
 * x[3n] (positions anywhere; wrapped into the box like rg_set_atoms),
 * type[n] (0 <= type < the force field's element count), q_out[n]; box3 is
 * a host array of orthogonal edges, each finite and at least half the QEq
 * cutoff; stream is a cudaStream_t (NULL: legacy default stream).  h only
 * supplies the force-field tables copied at rg_create.  The call runs on
 * h's device and restores the caller's current device before it returns.
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress); make it before any stream capture.  All calls share
 * the array and leave their contents in it; calls whose GPU work overlaps
 * race.  Larger n, a short or non-finite edge, a non-finite position or a
 * type outside the force field is rejected (RG_E_ARG, with a message in
 * rg_last_error) before any product is formed. */
#define RG_NOALLOC_MAX_ATOMS 8192
int rg_qeq_noalloc(rg_system *h, int n, const double *x, const int *type,
                   const double *box3, double *q_out, int *iters_s,
                   int *iters_t, void *stream);

/* Measured FP64 FMA throughput of a device (TFLOP/s): the roofline
 * denominator of the FP64 form, whose kernels are bound by the FP64 units. */
int rg_measure_fp64_peak(int device, double *tflops);

/* Bond table of the last force step (fix reax/c/bonds, FindBond,
 * fix_reaxc_bonds_sunway.cpp:196-255), per atom in the original order:
 * nbond[n] partners with corrected bond order > bo_cut (at most
 * max_per_atom listed), their tags nbr_tag[n*max_per_atom] and bond orders
 * bo[n*max_per_atom], the total bond order total_bo[n] and the lone pairs
 * nlp[n] (any array may be NULL).  Returns the largest partner count (which
 * may exceed max_per_atom) or a negative error code. */
int rg_bond_table(rg_system *h, double bo_cut, int max_per_atom, int *nbond, int *nbr_tag,
                  double *bo, double *total_bo, double *nlp);

/* List dumps for parity checks, from the last force step.  Each entry is
 * (tag_i, tag_j, image) with image = (sx+8) | (sy+8)<<4 | (sz+8)<<8 the
 * periodic image of j relative to i.  Pass NULL arrays to get the count.
 * rg_dump_bonds also returns the corrected bond orders bo[4*k] = BO, BO_s,
 * BO_pi, BO_pi2. */
long long rg_dump_pairs(rg_system *h, int *ti, int *tj, int *img);
long long rg_dump_bonds(rg_system *h, int *ti, int *tj, int *img, double *bo);
long long rg_dump_hbonds(rg_system *h, int *ti, int *tj, int *img);

#ifdef __cplusplus
}
#endif
#endif

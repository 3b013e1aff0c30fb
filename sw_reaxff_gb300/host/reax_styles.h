// Host-side C++ styles over the reaxgpu C ABI, with the interface of the
// reference's LAMMPS plugin classes for the ReaxFF time step:
//
//   PairReaxCGB300   <- pair_style reax/c/sunway   (PairReaxCSunway,
//                       pair_reaxc_sunway.h:37; settings :202-290, coeff
//                       :294-362, init_style :366-424, compute :541-793,
//                       extract :1106-1128, pvector order :657-670)
//   FixQEqReaxGB300  <- fix qeq/reax/sunway        (FixQEqReaxSunway,
//                       fix_qeq_reax_sunway.h:38; constructor :64-120, init
//                       :407-431, setup_pre_force :488, pre_force :539-600)
//   FixNVEGB300      <- fix nve/sunway             (FixNVESunway,
//                       fix_nve_sunway.h:27; init :52-58, initial_integrate
//                       :67-100, final_integrate :102-135)
//   Verlet           <- the LAMMPS Verlet setup/run order these are called in
//
// Argument lists, their meaning and the error messages are the reference's;
// where LAMMPS would call error->all (and abort), these classes throw
// reaxgb::Error with the same message.  The atom state lives on the device
// between calls (the styles call rg_nve_* / rg_qeq / rg_compute on device
// arrays); the host Atom arrays are brought up to date by Atom sync points
// (sync_host), and host edits are pushed back before the next device call
// (modified_host), like a KOKKOS dual view.
#ifndef REAX_STYLES_H
#define REAX_STYLES_H

#include <cstdio>
#include <map>
#include <stdexcept>
#include <string>
#include <array>
#include <vector>

#include "reaxgpu.h"

namespace reaxgb {

struct Error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// The part of LAMMPS's Atom and Domain the styles use: a periodic box,
// orthogonal or triclinic (edge vectors (lx,0,0), (xy,ly,0), (xz,yz,lz)).
struct Atom {
  int nlocal = 0;
  int ntypes = 0;
  int q_flag = 1;                  // atom_style charge
  int tag_enable = 1;
  std::vector<double> x, v, f, q;  // x/v/f: 3*nlocal (x0 y0 z0 x1 ...)
  std::vector<int> type, tag;      // type 1..ntypes, tag 1..natoms
  std::vector<double> mass;        // [ntypes + 1], mass[0] unused
  double boxlo[3] = {0, 0, 0}, boxhi[3] = {0, 0, 0};
  int triclinic = 0;
  double xy = 0.0, xz = 0.0, yz = 0.0;
};

struct Update {
  double dt = 1.0;                 // fs (LAMMPS real units)
  long long ntimestep = 0;
};

class PairReaxCGB300;

class FixQEqReaxGB300 {
 public:
  // fix ID group qeq/reax/gb300 nevery swa swb tol reax/c [dual]
  FixQEqReaxGB300(PairReaxCGB300 *pair, Update *update, int narg, char **arg);
  void init();
  void setup_pre_force(int vflag);
  void pre_force(int vflag);
  int nevery = 1;
  double swa = 0.0, swb = 10.0, tolerance = 1e-6;
  int imax = 200;
  int matvecs = 0, matvecs_s = 0, matvecs_t = 0;

 private:
  PairReaxCGB300 *pair_;
  Update *update_;
};

class FixNVEGB300 {
 public:
  // fix ID group nve/gb300
  FixNVEGB300(PairReaxCGB300 *pair, Update *update, int narg, char **arg);
  void init();
  void initial_integrate(int vflag);
  void final_integrate();
  void reset_dt();
  double dtv = 0.0, dtf = 0.0;

 private:
  PairReaxCGB300 *pair_;
  Update *update_;
};

// A fix called by the Verlet loop after setup and at the end of every step.
struct StepFix {
  virtual ~StepFix() = default;
  virtual void setup() = 0;
  virtual void end_of_step() = 0;
};

// fix ID group reax/c/bonds Nevery file (FixReaxCBondsSunway,
// fix_reaxc_bonds_sunway.cpp:45-330): every Nevery steps, the connection
// table with bond orders above the coarse cutoff bg_cut = 0.3, the total
// bond order, lone pairs and charge of every atom, in the reference's file
// format.
class FixReaxCBondsGB300 : public StepFix {
 public:
  FixReaxCBondsGB300(PairReaxCGB300 *pair, Atom *atom, Update *update, int narg, char **arg);
  ~FixReaxCBondsGB300() override;
  FixReaxCBondsGB300(const FixReaxCBondsGB300 &) = delete;
  FixReaxCBondsGB300 &operator=(const FixReaxCBondsGB300 &) = delete;
  void setup() override;
  void end_of_step() override;
  int nevery = 1;
  double bg_cut = 0.3;

 private:
  void output();
  PairReaxCGB300 *pair_;
  Atom *atom_;
  Update *update_;
  std::FILE *fp_ = nullptr;
};

// fix ID group reax/c/species Nevery Nrepeat Nfreq file [cutoff I J BO]
//   [element E1 .. En] [position Nposfreq file]  (FixReaxCSpeciesSunway,
// fix_reaxc_species_sunway.cpp:49-945): molecules are the connected
// components of the bonds whose bond order, averaged over Nrepeat samples
// Nevery steps apart ending at every Nfreq-th step, is above the type pair's
// cutoff (default 0.3); every Nfreq steps the species (element formulas)
// and their molecule counts are written in the reference's format, and
// with "position" each molecule's size, formula, mean charge and centre in
// fractional box coordinates.  The reference samples in post_integrate,
// where its bond orders are those of the previous step's positions; here the
// samples are taken at the end of the step, positions, charges and bond
// orders of one step together.
class FixReaxCSpeciesGB300 : public StepFix {
 public:
  FixReaxCSpeciesGB300(PairReaxCGB300 *pair, Atom *atom, Update *update, int narg, char **arg);
  ~FixReaxCSpeciesGB300() override;
  FixReaxCSpeciesGB300(const FixReaxCSpeciesGB300 &) = delete;
  FixReaxCSpeciesGB300 &operator=(const FixReaxCSpeciesGB300 &) = delete;
  void setup() override;
  void end_of_step() override;
  int nevery = 1, nrepeat = 1, nfreq = 1;
  int nmole = 0, nspec = 0;   // of the last output (the fix's vector)

 private:
  void sample();
  void output();
  void write_pos(const std::vector<int> &mol, int nmole, int nspec);
  std::string formula(const std::vector<int> &count) const;
  PairReaxCGB300 *pair_;
  Atom *atom_;
  Update *update_;
  std::FILE *fp_ = nullptr, *pos_ = nullptr;
  std::vector<std::vector<double>> bocut_;   // [ntypes+1][ntypes+1]
  std::vector<std::string> ele_;             // element name per LAMMPS type
  int posfreq_ = 0;
  std::string posfile_;
  bool multipos_ = false;
  long long nvalid_ = -1;
  int nsamples_ = 0;
  std::vector<double> xsum_, qsum_;                    // per atom (Atoms order)
  std::map<std::pair<int, int>, double> bosum_;        // (tag_i < tag_j) -> sum of BO
};

class PairReaxCGB300 {
 public:
  explicit PairReaxCGB300(Atom *atom);
  ~PairReaxCGB300();
  PairReaxCGB300(const PairReaxCGB300 &) = delete;
  PairReaxCGB300 &operator=(const PairReaxCGB300 &) = delete;

  // pair_style reax/c/gb300 NULL|control_file [checkqeq yes/no] [enobonds yes/no]
  //   [lgvdw yes/no] [safezone f] [mincap i] [maxfar i] [precision fp64/mixed]
  void settings(int narg, char **arg);
  // the reference's control file (Read_Control_File,
  // reaxc_control_sunway.cpp:33-380): its force-step keywords set the
  // cutoffs; the others are accepted and have no effect here
  void read_control_file(const char *path);
  double bg_cut = 0.3;   // bond_graph_cutoff (fix reax/c/bonds)
  // pair_coeff * * ffield.reax E1 E2 ... (one element or NULL per type)
  void coeff(int narg, char **arg);
  void init_style();
  void compute(int eflag, int vflag);
  void *extract(const char *str, int &dim);

  double pvector[14] = {0};
  double eng_vdwl = 0.0, eng_coul = 0.0;
  double virial[6] = {0};
  // per-atom tallies (LAMMPS Pair::eatom / vatom), filled by compute() when
  // eflag & 2 (ENERGY_ATOM) or vflag & 4 (VIRIAL_ATOM): local atoms only,
  // the nonbonded pair terms as in the reference
  std::vector<double> eatom;              // [nlocal]
  std::vector<std::array<double, 6>> vatom;  // [nlocal] xx yy zz xy xz yz
  int qeqflag = 1;

  // shared with the fixes
  rg_system *handle();
  void attach_qeq(FixQEqReaxGB300 *f) { fix_qeq_ = f; }
  void check(int rc, const char *what);
  void sync_device();   // push host edits of the atom arrays
  void sync_host();     // pull the device state into the host arrays
  void modified_host() { host_dirty_ = true; }
  void modified_device() { device_dirty_ = true; }
  int device() const { return params_.device; }

 private:
  void create_device();
  Atom *atom_;
  rg_params params_{};
  std::string ffield_;
  std::vector<int> map_;              // LAMMPS type -> ffield type (-1: NULL)
  std::vector<std::string> elements_;
  std::vector<double> chi_, eta_, gamma_;
  FixQEqReaxGB300 *fix_qeq_ = nullptr;
  rg_system *h_ = nullptr;
  bool uploaded_ = false, host_dirty_ = true, device_dirty_ = false;
  bool have_forces_ = false;
  friend class FixQEqReaxGB300;
  friend class FixNVEGB300;
  friend class FixReaxCBondsGB300;
  friend class FixReaxCSpeciesGB300;
};

// LAMMPS's Verlet order: setup (pre_force, force) then per step
// initial_integrate, pre_force, force, final_integrate.
class Verlet {
 public:
  Verlet(Atom *atom, Update *update, PairReaxCGB300 *pair, FixQEqReaxGB300 *qeq,
         FixNVEGB300 *nve)
      : atom_(atom), update_(update), pair_(pair), qeq_(qeq), nve_(nve) {}
  void setup();
  // thermo_every > 0: energies and a host sync on those steps (callback)
  void run(long long nsteps, int thermo_every,
           void (*thermo)(const Verlet &, void *) = nullptr, void *ctx = nullptr);
  double kinetic_energy() const;   // kcal/mol from the host velocities
  std::vector<StepFix *> end_of_step_fixes;
  Atom *atom_;
  Update *update_;
  PairReaxCGB300 *pair_;
  FixQEqReaxGB300 *qeq_;
  FixNVEGB300 *nve_;
};

}  // namespace reaxgb

#endif

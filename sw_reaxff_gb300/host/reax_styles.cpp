// Host-side C++ styles over the reaxgpu C ABI (see reax_styles.h for the
// reference classes each one mirrors).
#include "reax_styles.h"

#include <algorithm>
#include <array>
#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <strings.h>

namespace reaxgb {

namespace {

// LAMMPS force->numeric / inumeric: the whole string must be a number
double numeric(const char *s) {
  char *end = nullptr;
  errno = 0;
  const double v = std::strtod(s, &end);
  if (!s[0] || *end || errno)
    throw Error(std::string("Expected floating point parameter instead of ") + s +
                " in input script or data file");
  return v;
}

long inumeric(const char *s) {
  char *end = nullptr;
  errno = 0;
  const long v = std::strtol(s, &end, 10);
  if (!s[0] || *end || errno)
    throw Error(std::string("Expected integer parameter instead of ") + s +
                " in input script or data file");
  return v;
}

bool yes_no(const char *s, const char *illegal) {
  if (!std::strcmp(s, "yes")) return true;
  if (!std::strcmp(s, "no")) return false;
  throw Error(illegal);
}

// LAMMPS real units: ftm2v = 1 / 48.88821291^2, mvv2e = 48.88821291^2
constexpr double FTM2V = 1.0 / 48.88821291 / 48.88821291;
constexpr double MVV2E = 48.88821291 * 48.88821291;

}  // namespace

// ---------------------------------------------------------------- pair

PairReaxCGB300::PairReaxCGB300(Atom *atom) : atom_(atom) { rg_default_params(&params_); }

PairReaxCGB300::~PairReaxCGB300() {
  if (h_) rg_destroy(h_);
}

void PairReaxCGB300::settings(int narg, char **arg) {
  if (narg < 1) throw Error("Illegal pair_style command");
  // NULL: the reference's default controls (pair_reaxc_sunway.cpp:208-242);
  // else a control file (pair_reaxc_sunway.cpp:231, Read_Control_File)
  rg_default_params(&params_);
  bg_cut = 0.3;
  if (std::strcmp(arg[0], "NULL") != 0) read_control_file(arg[0]);
  qeqflag = 1;
  const char *illegal = "Illegal pair_style reax/c command";
  int iarg = 1;
  while (iarg < narg) {
    if (iarg + 2 > narg) throw Error(illegal);
    const char *key = arg[iarg], *val = arg[iarg + 1];
    if (!std::strcmp(key, "checkqeq")) {
      qeqflag = yes_no(val, illegal) ? 1 : 0;
    } else if (!std::strcmp(key, "enobonds")) {
      params_.enobondsflag = yes_no(val, illegal) ? 1 : 0;
    } else if (!std::strcmp(key, "lgvdw")) {
      params_.lgflag = yes_no(val, illegal) ? 1 : 0;
    } else if (!std::strcmp(key, "safezone")) {
      // list capacities grow on the device as needed: accepted, not used
      if (numeric(val) < 0.0) throw Error("Illegal pair_style reax/c safezone command");
    } else if (!std::strcmp(key, "mincap")) {
      if (inumeric(val) < 0) throw Error("Illegal pair_style reax/c mincap command");
    } else if (!std::strcmp(key, "maxfar")) {
      if (inumeric(val) < 0) throw Error("Illegal pair_style reax/c maxfar command");
    } else if (!std::strcmp(key, "precision")) {
      if (!std::strcmp(val, "fp64")) params_.precision = RG_PREC_FP64;
      else if (!std::strcmp(val, "mixed")) params_.precision = RG_PREC_MIXED;
      else throw Error(illegal);
    } else if (!std::strcmp(key, "device")) {
      params_.device = (int)inumeric(val);
    } else {
      throw Error(illegal);
    }
    iarg += 2;
  }
}

void PairReaxCGB300::read_control_file(const char *path) {
  std::FILE *fp = std::fopen(path, "r");
  if (!fp) throw Error(std::string("Cannot open control file ") + path);
  // keywords of Read_Control_File that do not touch the force step
  static const char *other[] = {
      "simulation_name", "ensemble_type", "nsteps", "dt", "proc_by_dim", "random_vel",
      "restart_format", "restart_freq", "reposition_atoms", "restrict_bonds", "remove_CoM_vel",
      "debug_level", "energy_update_freq", "reneighbor", "vlist_buffer", "ghost_cutoff",
      "qeq_freq", "q_err", "ilu_refactor", "ilu_droptol", "temp_init", "temp_final", "t_mass",
      "t_mode", "t_rate", "t_freq", "pressure", "p_mass", "pt_mass", "compress", "press_mode",
      "geo_format", "write_freq", "traj_compress", "traj_method", "traj_title", "atom_info",
      "atom_velocities", "atom_forces", "bond_info", "angle_info", "molecular_analysis",
      "ignore", "dipole_anal", "freq_dipole_anal", "diffusion_coef", "freq_diffusion_coef",
      "restrict_type"};
  char line[1024];
  std::string bad;
  while (std::fgets(line, sizeof line, fp)) {
    char key[256] = {0}, val[256] = {0};
    const int k = std::sscanf(line, "%255s %255s", key, val);
    if (k < 1) continue;   // blank line
    const double v = std::atof(val);
    if (!std::strcmp(key, "nbrhood_cutoff")) params_.bond_cut = v;
    else if (!std::strcmp(key, "hbond_cutoff")) params_.hbond_cut = v;
    else if (!std::strcmp(key, "thb_cutoff")) params_.thb_cut = v;
    else if (!std::strcmp(key, "thb_cutoff_sq")) params_.thb_cutsq = v;
    else if (!std::strcmp(key, "bond_graph_cutoff")) bg_cut = v;
    else if (!std::strcmp(key, "tabulate_long_range")) {
      // the reference's long-range table switch: 0 = analytic pair
      // functions; any other value selects the FP64 tables here
      if (std::atoi(val) == 0) params_.tabulate = 0;
    } else {
      bool known = false;
      for (const char *o : other) known = known || !std::strcmp(key, o);
      if (!known && bad.empty()) bad = key;
    }
  }
  std::fclose(fp);
  // the reference prints "WARNING: unknown parameter" and aborts
  if (!bad.empty()) throw Error("Unknown parameter " + bad + " in control file " + path);
}

void PairReaxCGB300::coeff(int narg, char **arg) {
  if (narg != 3 + atom_->ntypes) throw Error("Incorrect args for pair coefficients");
  if (std::strcmp(arg[0], "*") != 0 || std::strcmp(arg[1], "*") != 0)
    throw Error("Incorrect args for pair coefficients");
  int nt = 0;
  char msg[256] = {0};
  if (rg_ffield_info(arg[2], &nt, nullptr, 0, msg, sizeof msg) != RG_OK)
    throw Error(std::string("Cannot open ReaxFF potential file ") + arg[2]);
  std::vector<char> names((size_t)nt * 16);
  rg_ffield_info(arg[2], &nt, names.data(), 16, nullptr, 0);
  elements_.clear();
  for (int t = 0; t < nt; ++t) elements_.emplace_back(&names[(size_t)t * 16]);
  ffield_ = arg[2];
  // map[i] = ffield type of LAMMPS type i, -1 for NULL
  map_.assign(atom_->ntypes + 1, -1);
  int itmp = 0;
  for (int i = 3; i < narg; ++i) {
    if (!std::strcmp(arg[i], "NULL")) {
      ++itmp;
      continue;
    }
    for (int j = 0; j < nt; ++j)
      if (!strcasecmp(arg[i], elements_[j].c_str())) {
        map_[i - 2] = j;
        ++itmp;
      }
  }
  if (itmp != atom_->ntypes) throw Error("Non-existent ReaxFF type");
  int count = 0;
  for (int i = 1; i <= atom_->ntypes; ++i)
    if (map_[i] >= 0) ++count;
  if (count == 0) throw Error("Incorrect args for pair coefficients");
}

void PairReaxCGB300::init_style() {
  if (!atom_->q_flag) throw Error("Pair style reax/c requires atom attribute q");
  if (!fix_qeq_ && qeqflag == 1) throw Error("Pair reax/c requires use of fix qeq/reax");
  if (atom_->tag_enable == 0) throw Error("Pair style reax/c requires atom IDs");
  if (map_.empty()) throw Error("All pair coeffs are not set");
  for (int i = 0; i < atom_->nlocal; ++i)
    if (map_[atom_->type[i]] < 0)
      throw Error("reax/c/gb300 computes every atom: NULL-mapped types are not supported");
  // the device context is created at the first device call (setup), after
  // every style's init has checked its arguments
  if (h_) {
    rg_destroy(h_);
    h_ = nullptr;
  }
  chi_.assign(atom_->ntypes + 1, 0.0);
  eta_.assign(atom_->ntypes + 1, 0.0);
  gamma_.assign(atom_->ntypes + 1, 0.0);
  uploaded_ = false;
  host_dirty_ = true;
  device_dirty_ = false;
  have_forces_ = false;
}

void PairReaxCGB300::create_device() {
  if (fix_qeq_) {
    params_.qeq_swa = fix_qeq_->swa;
    params_.qeq_swb = fix_qeq_->swb;
    params_.qeq_tol = fix_qeq_->tolerance;
    params_.qeq_imax = fix_qeq_->imax;
  }
  if (rg_create(ffield_.c_str(), &params_, &h_) != RG_OK || !h_)
    throw Error("reax/c/gb300: cannot create the device context for " + ffield_);
  const int nt = (int)elements_.size();
  // integrator masses per ffield type from the data file's per-type masses
  std::vector<double> m(nt, 0.0);
  check(rg_extract(h_, "mass", m.data()), "rg_extract");
  std::vector<int> seen(nt, 0);
  for (int i = 1; i <= atom_->ntypes; ++i) {
    const int t = map_[i];
    if (t < 0 || (int)atom_->mass.size() <= i || !(atom_->mass[i] > 0.0)) continue;
    if (seen[t] && m[t] != atom_->mass[i])
      throw Error("reax/c/gb300: types mapped to one element need one mass");
    m[t] = atom_->mass[i];
    seen[t] = 1;
  }
  check(rg_set_masses(h_, m.data()), "rg_set_masses");
  const double L[3] = {atom_->boxhi[0] - atom_->boxlo[0], atom_->boxhi[1] - atom_->boxlo[1],
                       atom_->boxhi[2] - atom_->boxlo[2]};
  check(rg_set_box(h_, L), "rg_set_box");
  if (atom_->triclinic) {
    const double tilt[3] = {atom_->xy, atom_->xz, atom_->yz};
    check(rg_set_tilt(h_, tilt), "rg_set_tilt");
  }
}

rg_system *PairReaxCGB300::handle() {
  if (map_.empty() || chi_.empty()) throw Error("reax/c/gb300: init_style has not been called");
  if (!h_) create_device();
  return h_;
}

void PairReaxCGB300::check(int rc, const char *what) {
  if (rc != RG_OK)
    throw Error(std::string(what) + ": " + (h_ ? rg_last_error(h_) : "no device context"));
}

void PairReaxCGB300::sync_device() {
  if (!host_dirty_) return;
  if (device_dirty_)
    throw Error("reax/c/gb300: host atom arrays modified while the device copy is newer "
                "(call sync_host before editing them)");
  rg_system *h = handle();
  const int n = atom_->nlocal;
  // positions relative to the box origin, wrapped into an orthogonal box
  // (LAMMPS keeps them there between re-neighbourings); the library wraps
  // a triclinic cell's positions by their fractional coordinates itself
  std::vector<double> x(3 * (size_t)n);
  for (int i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) {
      const double lo = atom_->boxlo[c], L = atom_->boxhi[c] - atom_->boxlo[c];
      double u = atom_->x[3 * i + c] - lo;
      if (!atom_->triclinic) {
        u -= L * std::floor(u / L);
        if (u >= L) u -= L;
      }
      x[3 * i + c] = u;
    }
  if (!uploaded_) {
    std::vector<int> t(n);
    for (int i = 0; i < n; ++i) t[i] = map_[atom_->type[i]];
    check(rg_set_atoms(h, n, x.data(), t.data(), atom_->tag.data(),
                       atom_->q.empty() ? nullptr : atom_->q.data(),
                       atom_->v.empty() ? nullptr : atom_->v.data()),
          "rg_set_atoms");
    uploaded_ = true;
  } else {
    // forces of edited positions are recomputed by the next force call
    check(rg_set_state(h, x.data(), atom_->v.data(), nullptr), "rg_set_state");
    have_forces_ = false;
  }
  host_dirty_ = false;
}

void PairReaxCGB300::sync_host() {
  if (!device_dirty_) return;
  rg_system *h = handle();
  const int n = atom_->nlocal;
  atom_->x.resize(3 * (size_t)n);
  atom_->v.resize(3 * (size_t)n);
  atom_->f.resize(3 * (size_t)n);
  atom_->q.resize(n);
  check(rg_get_atoms(h, atom_->x.data(), atom_->v.data(), atom_->q.data(), atom_->f.data()),
        "rg_get_atoms");
  // back to the LAMMPS box origin
  for (int i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) atom_->x[3 * i + c] += atom_->boxlo[c];
  device_dirty_ = false;
}

void PairReaxCGB300::compute(int eflag, int vflag) {
  rg_system *h = handle();
  sync_device();
  double e[RG_NENERGY];
  check(rg_compute(h, eflag, vflag, nullptr, eflag ? e : nullptr), "rg_compute");
  have_forces_ = true;
  modified_device();
  if (eflag) {
    // pvector order of pair_reaxc_sunway.cpp:657-670 and the tallied sums
    for (int k = 0; k < 14; ++k) pvector[k] = e[k];
    eng_vdwl = e[14];
    eng_coul = e[15];
  }
  if (vflag & 3) check(rg_get_virial(h, virial), "rg_get_virial");
  if ((eflag & 2) || (vflag & 4)) {
    const int n = atom_->nlocal;
    std::vector<double> ea(n), va(6 * (size_t)n);
    check(rg_get_atom_tallies(h, ea.data(), va.data()), "rg_get_atom_tallies");
    if (eflag & 2) eatom = ea;
    if (vflag & 4) {
      vatom.resize(n);
      for (int i = 0; i < n; ++i)
        for (int k = 0; k < 6; ++k) vatom[i][k] = va[6 * (size_t)i + k];
    }
  }
}

void *PairReaxCGB300::extract(const char *str, int &dim) {
  dim = 1;
  std::vector<double> *dst = nullptr;
  if (!std::strcmp(str, "chi")) dst = &chi_;
  else if (!std::strcmp(str, "eta")) dst = &eta_;
  else if (!std::strcmp(str, "gamma")) dst = &gamma_;
  if (!dst || !h_) return nullptr;
  std::vector<double> per(elements_.size());
  check(rg_extract(h_, str, per.data()), "rg_extract");
  dst->assign(atom_->ntypes + 1, 0.0);
  for (int i = 1; i <= atom_->ntypes; ++i) (*dst)[i] = map_[i] >= 0 ? per[map_[i]] : 0.0;
  return dst->data();
}

// ---------------------------------------------------------------- fix qeq

FixQEqReaxGB300::FixQEqReaxGB300(PairReaxCGB300 *pair, Update *update, int narg, char **arg)
    : pair_(pair), update_(update) {
  const char *illegal = "Illegal fix qeq/reax command";
  if (narg < 8 || narg > 9) throw Error(illegal);
  nevery = (int)inumeric(arg[3]);
  if (nevery <= 0) throw Error(illegal);
  swa = numeric(arg[4]);
  swb = numeric(arg[5]);
  tolerance = numeric(arg[6]);
  // per-type chi/eta/gamma from the pair (extract); a parameter file is not
  // supported (fix_qeq_reax_sunway.cpp:198-247)
  if (std::strcmp(arg[7], "reax/c") != 0)
    throw Error("fix qeq/reax/gb300 takes its parameters from pair reax/c/gb300 (reax/c)");
  // the s and t systems are always solved together on the device
  if (narg == 9 && std::strcmp(arg[8], "dual") != 0) throw Error(illegal);
  if (!pair_) throw Error("No pair reax/c for fix qeq/reax");
  pair_->attach_qeq(this);
}

void FixQEqReaxGB300::init() {
  if (!pair_->atom_->q_flag) throw Error("Fix qeq/reax requires atom attribute q");
  if (pair_->atom_->nlocal == 0) throw Error("Fix qeq/reax group has no atoms");
  // init_taper (fix_qeq_reax_sunway.cpp:458-486) rejects these two
  if (swb < 0) throw Error("Fix qeq/reax has negative upper Taper radius cutoff");
  if (swa < 0) throw Error("Fix qeq/reax has negative lower Taper radius cutoff");
}

void FixQEqReaxGB300::setup_pre_force(int vflag) { pre_force(vflag); }

void FixQEqReaxGB300::pre_force(int /*vflag*/) {
  if (update_->ntimestep % nevery) return;
  rg_system *h = pair_->handle();
  pair_->sync_device();
  int its = 0, itt = 0;
  pair_->check(rg_qeq(h, nullptr, &its, &itt), "rg_qeq");
  matvecs_s = its;
  matvecs_t = itt;
  matvecs = its + itt;
  pair_->modified_device();
}

// ---------------------------------------------------------------- fix nve

FixNVEGB300::FixNVEGB300(PairReaxCGB300 *pair, Update *update, int narg, char ** /*arg*/)
    : pair_(pair), update_(update) {
  if (narg < 3) throw Error("Illegal fix nve command");
  if (!pair_) throw Error("fix nve/gb300 requires pair reax/c/gb300");
}

void FixNVEGB300::init() {
  dtv = update_->dt;
  dtf = 0.5 * update_->dt * FTM2V;
}

void FixNVEGB300::reset_dt() { init(); }

void FixNVEGB300::initial_integrate(int /*vflag*/) {
  pair_->sync_device();
  pair_->check(rg_nve_initial(pair_->handle(), dtv), "rg_nve_initial");
  pair_->modified_device();
}

void FixNVEGB300::final_integrate() {
  pair_->sync_device();
  pair_->check(rg_nve_final(pair_->handle(), dtv), "rg_nve_final");
  pair_->modified_device();
}

// ---------------------------------------------------------------- fix bonds

FixReaxCBondsGB300::FixReaxCBondsGB300(PairReaxCGB300 *pair, Atom *atom, Update *update, int narg,
                                       char **arg)
    : pair_(pair), atom_(atom), update_(update) {
  if (narg != 5) throw Error("Illegal fix reax/c/bonds command");
  nevery = (int)inumeric(arg[3]);
  if (nevery <= 0) throw Error("Illegal fix reax/c/bonds command");
  if (!pair_) throw Error("Cannot use fix reax/c/bonds without pair_style reax/c");
  fp_ = std::fopen(arg[4], "w");
  if (!fp_) throw Error(std::string("Cannot open fix reax/c/bonds file ") + arg[4]);
}

FixReaxCBondsGB300::~FixReaxCBondsGB300() {
  if (fp_) std::fclose(fp_);
}

void FixReaxCBondsGB300::setup() { output(); }

void FixReaxCBondsGB300::end_of_step() {
  if (update_->ntimestep % nevery == 0) output();
}

void FixReaxCBondsGB300::output() {
  const int n = atom_->nlocal;
  const int cap = 24;
  std::vector<int> nb(n), tags((size_t)n * cap);
  std::vector<double> bo((size_t)n * cap), tot(n), nlp(n);
  bg_cut = pair_->bg_cut;
  const int most = rg_bond_table(pair_->handle(), bg_cut, cap, nb.data(), tags.data(), bo.data(),
                                 tot.data(), nlp.data());
  pair_->check(most < 0 ? most : RG_OK, "rg_bond_table");
  pair_->sync_host();
  std::fprintf(fp_, "# Timestep %lld \n", update_->ntimestep);
  std::fprintf(fp_, "# \n");
  std::fprintf(fp_, "# Number of particles %d \n", n);
  std::fprintf(fp_, "# \n");
  std::fprintf(fp_, "# Max number of bonds per atom %d with coarse bond order cutoff %5.3f \n",
               most, bg_cut);
  std::fprintf(fp_, "# Particle connection table and bond orders \n");
  std::fprintf(fp_, "# id type nb id_1...id_nb mol bo_1...bo_nb abo nlp q \n");
  for (int i = 0; i < n; ++i) {
    std::fprintf(fp_, " %d %d %d", atom_->tag[i], atom_->type[i], nb[i]);
    for (int k = 0; k < nb[i]; ++k) std::fprintf(fp_, " %d", tags[(size_t)i * cap + k]);
    std::fprintf(fp_, " %d", 0);   // molecule id (atom_style charge has none)
    for (int k = 0; k < nb[i]; ++k) std::fprintf(fp_, "%14.3f", bo[(size_t)i * cap + k]);
    std::fprintf(fp_, "%14.3f%14.3f%14.3f\n", tot[i], nlp[i], atom_->q[i]);
  }
  std::fprintf(fp_, "# \n");
  std::fflush(fp_);
}

// ---------------------------------------------------------------- fix species

FixReaxCSpeciesGB300::FixReaxCSpeciesGB300(PairReaxCGB300 *pair, Atom *atom, Update *update,
                                           int narg, char **arg)
    : pair_(pair), atom_(atom), update_(update) {
  const char *illegal = "Illegal fix reax/c/species command";
  if (narg < 7) throw Error(illegal);
  nevery = (int)inumeric(arg[3]);
  nrepeat = (int)inumeric(arg[4]);
  nfreq = (int)inumeric(arg[5]);
  if (nevery <= 0 || nrepeat <= 0 || nfreq <= 0) throw Error(illegal);
  if (nfreq % nevery || nrepeat * nevery > nfreq) throw Error(illegal);
  if (!pair_) throw Error("Cannot use fix reax/c/species without pair_style reax/c");
  const int nt = atom_->ntypes;
  bocut_.assign(nt + 1, std::vector<double>(nt + 1, 0.30));
  static const char *dflt[] = {"C", "H", "O", "N"};
  ele_.assign(nt, "");
  for (int k = 0; k < nt && k < 4; ++k) ele_[k] = dflt[k];
  int iarg = 7;
  while (iarg < narg) {
    if (!std::strcmp(arg[iarg], "cutoff")) {
      if (iarg + 4 > narg) throw Error(illegal);
      const int it = (int)inumeric(arg[iarg + 1]), jt = (int)inumeric(arg[iarg + 2]);
      const double bo = numeric(arg[iarg + 3]);
      if (it > nt || jt > nt || it <= 0 || jt <= 0 || bo > 1.0 || bo < 0.0) throw Error(illegal);
      bocut_[it][jt] = bocut_[jt][it] = bo;
      iarg += 4;
    } else if (!std::strcmp(arg[iarg], "element")) {
      if (iarg + nt + 1 > narg) throw Error(illegal);
      for (int k = 0; k < nt; ++k) ele_[k] = arg[iarg + 1 + k];
      iarg += nt + 1;
    } else if (!std::strcmp(arg[iarg], "position")) {
      if (iarg + 3 > narg) throw Error(illegal);
      posfreq_ = (int)inumeric(arg[iarg + 1]);
      if (posfreq_ < nfreq || posfreq_ % nfreq != 0) throw Error(illegal);
      posfile_ = arg[iarg + 2];
      multipos_ = posfile_.find('*') != std::string::npos;
      if (!multipos_) {
        pos_ = std::fopen(posfile_.c_str(), "w");
        if (!pos_) throw Error("Cannot open fix reax/c/species position file");
      }
      iarg += 3;
    } else {
      throw Error(illegal);
    }
  }
  const std::string file = arg[6];
  if (file.size() > 3 && file.compare(file.size() - 3, 3, ".gz") == 0)
    throw Error("Cannot open gzipped file");
  fp_ = std::fopen(file.c_str(), "w");
  if (!fp_) throw Error("Cannot open fix reax/c/species file " + file);
}

FixReaxCSpeciesGB300::~FixReaxCSpeciesGB300() {
  if (fp_) std::fclose(fp_);
  if (pos_) std::fclose(pos_);
}

void FixReaxCSpeciesGB300::setup() {
  // first output Nfreq steps on (FixReaxCSpeciesSunway::init)
  nvalid_ = update_->ntimestep + nfreq;
  nsamples_ = 0;
  xsum_.clear();
  qsum_.clear();
  bosum_.clear();
}

void FixReaxCSpeciesGB300::end_of_step() {
  const long long t = update_->ntimestep;
  const long long first = nvalid_ - (long long)(nrepeat - 1) * nevery;
  if (t >= first && t <= nvalid_ && (nvalid_ - t) % nevery == 0) sample();
  if (t == nvalid_) {
    output();
    nvalid_ += nfreq;
    nsamples_ = 0;
    xsum_.clear();
    qsum_.clear();
    bosum_.clear();
  }
}

// one sample: positions, charges and the bond orders >= 0.10 of every pair
// (the pre-cut of PairReaxCSunway::FindBond, pair_reaxc_sunway.cpp:1170-1198)
void FixReaxCSpeciesGB300::sample() {
  const int n = atom_->nlocal;
  const int cap = 24;
  std::vector<int> nb(n), tags((size_t)n * cap);
  std::vector<double> bo((size_t)n * cap), tot(n), nlp(n);
  const int most = rg_bond_table(pair_->handle(), 0.10, cap, nb.data(), tags.data(), bo.data(),
                                 tot.data(), nlp.data());
  pair_->check(most < 0 ? most : RG_OK, "rg_bond_table");
  if (most > cap) throw Error("Increase MAXSPECBOND: an atom has more than 24 bonds");
  pair_->sync_host();
  if (xsum_.empty()) {
    xsum_.assign(3 * (size_t)n, 0.0);
    qsum_.assign(n, 0.0);
  }
  for (int i = 0; i < n; ++i) {
    for (int c = 0; c < 3; ++c) xsum_[3 * (size_t)i + c] += atom_->x[3 * (size_t)i + c];
    qsum_[i] += atom_->q[i];
  }
  // the largest order per atom pair (periodic images of one pair in small
  // boxes count once)
  std::map<std::pair<int, int>, double> s;
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < nb[i]; ++k) {
      const int a = atom_->tag[i], b = tags[(size_t)i * cap + k];
      if (a >= b) continue;
      double &v = s[{a, b}];
      v = std::max(v, bo[(size_t)i * cap + k]);
    }
  for (auto &kv : s) bosum_[kv.first] += kv.second;
  ++nsamples_;
}

std::string FixReaxCSpeciesGB300::formula(const std::vector<int> &count) const {
  std::string f;
  for (size_t j = 0; j < count.size(); ++j)
    if (count[j]) {
      f += ele_[j];
      if (count[j] != 1) f += std::to_string(count[j]);
    }
  return f;
}

void FixReaxCSpeciesGB300::output() {
  const int n = atom_->nlocal;
  const int nt = atom_->ntypes;
  if (nsamples_ == 0) sample();
  std::map<int, int> slot;   // tag -> Atoms index
  for (int i = 0; i < n; ++i) slot[atom_->tag[i]] = i;
  // union-find over the averaged bonds above their cutoff
  std::vector<int> parent(n);
  for (int i = 0; i < n; ++i) parent[i] = i;
  auto find = [&](int i) {
    while (parent[i] != i) i = parent[i] = parent[parent[i]];
    return i;
  };
  for (auto &kv : bosum_) {
    const int i = slot[kv.first.first], j = slot[kv.first.second];
    const double avg = kv.second / nsamples_;
    if (avg > bocut_[atom_->type[i]][atom_->type[j]]) parent[find(i)] = find(j);
  }
  // molecules numbered 1.. in the order of their smallest atom ID
  // (SortMolecule), species in the order of first appearance (FindSpecies)
  std::map<int, int> root_min;
  for (int i = 0; i < n; ++i) {
    const int r = find(i);
    auto it = root_min.find(r);
    if (it == root_min.end() || atom_->tag[i] < it->second) root_min[r] = atom_->tag[i];
  }
  std::vector<std::pair<int, int>> order;   // (min tag, root)
  for (auto &kv : root_min) order.push_back({kv.second, kv.first});
  std::sort(order.begin(), order.end());
  std::map<int, int> molid;
  for (size_t m = 0; m < order.size(); ++m) molid[order[m].second] = (int)m + 1;
  nmole = (int)order.size();
  std::vector<int> mol(n);
  std::vector<std::vector<int>> counts(nmole, std::vector<int>(nt, 0));
  for (int i = 0; i < n; ++i) {
    mol[i] = molid[find(i)];
    counts[mol[i] - 1][atom_->type[i] - 1]++;
  }
  std::vector<std::vector<int>> species;
  std::vector<int> nmol;
  for (int m = 0; m < nmole; ++m) {
    size_t k = 0;
    while (k < species.size() && species[k] != counts[m]) ++k;
    if (k == species.size()) {
      species.push_back(counts[m]);
      nmol.push_back(1);
    } else {
      nmol[k]++;
    }
  }
  nspec = (int)species.size();
  std::fprintf(fp_, "# Timestep     No_Moles     No_Specs     ");
  for (auto &sp : species) std::fprintf(fp_, "%s\t", formula(sp).c_str());
  std::fprintf(fp_, "\n");
  std::fprintf(fp_, "%lld", update_->ntimestep);
  std::fprintf(fp_, "%11d%11d\t", nmole, nspec);
  for (int c : nmol) std::fprintf(fp_, " %d\t", c);
  std::fprintf(fp_, "\n");
  std::fflush(fp_);
  if (posfreq_ > 0 && update_->ntimestep % posfreq_ == 0) write_pos(mol, nmole, nspec);
}

// molecule sizes, formulas, mean charges and centres (WritePos,
// fix_reaxc_species_sunway.cpp:814-935): atoms unwrapped to the half-box
// image nearest the molecule's anchor (its lexicographically smallest
// averaged position), the centre wrapped into the box and given as a
// fraction of the box edges
void FixReaxCSpeciesGB300::write_pos(const std::vector<int> &mol, int nmole_, int nspec_) {
  std::FILE *fp = pos_;
  if (multipos_) {
    std::string f = posfile_;
    f.replace(f.find('*'), 1, std::to_string(update_->ntimestep));
    fp = std::fopen(f.c_str(), "w");
    if (!fp) throw Error("Cannot open fix reax/c/species position file");
  }
  const int n = atom_->nlocal, nt = atom_->ntypes;
  const double *lo = atom_->boxlo, *hi = atom_->boxhi;
  double box[3], half[3];
  for (int c = 0; c < 3; ++c) {
    box[c] = hi[c] - lo[c];
    half[c] = box[c] / 2;
  }
  std::fprintf(fp, "Timestep %lld NMole %d  NSpec %d  xlo %f  xhi %f  ylo %f  yhi %f  zlo %f  zhi %f\n",
               update_->ntimestep, nmole_, nspec_, lo[0], hi[0], lo[1], hi[1], lo[2], hi[2]);
  std::fprintf(fp, "ID\tAtom_Count\tType\tAve_q\t\tCoM_x\t\tCoM_y\t\tCoM_z\n");
  const double w = 1.0 / nsamples_;
  std::vector<std::array<double, 3>> anchor(nmole_ + 1);
  std::vector<int> have(nmole_ + 1, 0);
  for (int i = 0; i < n; ++i) {
    const std::array<double, 3> x = {xsum_[3 * (size_t)i] * w, xsum_[3 * (size_t)i + 1] * w,
                                     xsum_[3 * (size_t)i + 2] * w};
    const int m = mol[i];
    if (!have[m] || x < anchor[m]) anchor[m] = x;
    have[m] = 1;
  }
  for (int m = 1; m <= nmole_; ++m) {
    int count = 0;
    double avq = 0.0, avx[3] = {0, 0, 0};
    std::vector<int> name(nt, 0);
    for (int i = 0; i < n; ++i) {
      if (mol[i] != m) continue;
      name[atom_->type[i] - 1]++;
      ++count;
      avq += qsum_[i] * w;
      for (int c = 0; c < 3; ++c) {
        double x = xsum_[3 * (size_t)i + c] * w;
        if (anchor[m][c] - x > half[c]) x += box[c];
        if (x - anchor[m][c] > half[c]) x -= box[c];
        avx[c] += x;
      }
    }
    std::fprintf(fp, "%d\t%d\t%s", m, count, formula(name).c_str());
    if (count > 0) {
      avq /= count;
      for (int c = 0; c < 3; ++c) {
        avx[c] /= count;
        if (avx[c] >= hi[c]) avx[c] -= box[c];
        if (avx[c] < lo[c]) avx[c] += box[c];
        avx[c] = (avx[c] - lo[c]) / box[c];
      }
      std::fprintf(fp, "\t%.8f \t%.8f \t%.8f \t%.8f", avq, avx[0], avx[1], avx[2]);
    }
    std::fprintf(fp, "\n");
  }
  if (multipos_) std::fclose(fp);
  else {
    std::fprintf(fp, "#\n");
    std::fflush(fp);
  }
}

// ---------------------------------------------------------------- Verlet

void Verlet::setup() {
  pair_->init_style();
  if (qeq_) qeq_->init();
  if (nve_) nve_->init();
  if (qeq_) qeq_->setup_pre_force(0);
  pair_->compute(1, 1);
  for (auto *f : end_of_step_fixes) f->setup();
}

void Verlet::run(long long nsteps, int thermo_every, void (*thermo)(const Verlet &, void *),
                 void *ctx) {
  for (long long s = 0; s < nsteps; ++s) {
    ++update_->ntimestep;
    const bool th = thermo_every > 0 &&
                    (update_->ntimestep % thermo_every == 0 || s == nsteps - 1);
    if (nve_) nve_->initial_integrate(0);
    if (qeq_) qeq_->pre_force(0);
    pair_->compute(th ? 1 : 0, th ? 1 : 0);   // energies and virial on thermo steps
    if (nve_) nve_->final_integrate();
    for (auto *f : end_of_step_fixes) f->end_of_step();
    if (th) {
      pair_->sync_host();
      if (thermo) thermo(*this, ctx);
    }
  }
  pair_->sync_host();
}

double Verlet::kinetic_energy() const {
  // 0.5 m v^2 in kcal/mol (LAMMPS real: mvv2e)
  double ke = 0.0;
  if ((int)atom_->mass.size() <= atom_->ntypes) throw Error("Not all per-type masses are set");
  for (int i = 0; i < atom_->nlocal; ++i) {
    const double m = atom_->mass[atom_->type[i]];
    const double *v = &atom_->v[3 * (size_t)i];
    ke += m * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  }
  return 0.5 * MVV2E * ke;
}

}  // namespace reaxgb

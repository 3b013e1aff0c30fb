// reax_md: runs a LAMMPS-style ReaxFF input deck through the GB300 styles.
//
// The reference is driven by LAMMPS input decks (in.reaxc.lattice:
// units real, atom_style charge, read_data, pair_style reax/c/sunway NULL,
// pair_coeff * * ffield.reax C H O N, fix ... qeq/reax/sunway 1 0.0 10.0
// 1.0e-6 reax/c, fix ... nve/sunway, timestep, thermo, run).  This driver
// accepts those commands, with the reference's style names (reax/c,
// reax/c/sunway, qeq/reax, qeq/reax/sunway, nve, nve/sunway) mapped to the
// GB300 styles, so the same deck runs unchanged:
//
//   units real | atom_style charge | boundary p p p | read_data FILE |
//   mass I M | pair_style ... | pair_coeff ... | fix ID all STYLE ... |
//   (STYLE: qeq/reax, nve, reax/c/bonds and their /sunway, /gb300 names)
//   timestep DT | thermo N | run N |
//   write_dump all custom FILE COLS (id type q x y z vx vy vz fx fy fz)
//   neighbor / neigh_modify / thermo_style / thermo_modify: accepted, no effect
//
// Errors print "ERROR: <message>" and exit 1, as LAMMPS does.
#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "reax_styles.h"

using reaxgb::Error;

namespace {

std::vector<std::string> split(const std::string &line) {
  std::vector<std::string> w;
  std::istringstream is(line);
  std::string s;
  while (is >> s) {
    if (s[0] == '#') break;
    w.push_back(s);
  }
  return w;
}

struct Args {
  std::vector<std::string> s;
  std::vector<char *> p;
  explicit Args(const std::vector<std::string> &w, size_t from) : s(w.begin() + from, w.end()) {
    for (auto &x : s) p.push_back(&x[0]);
  }
  int n() const { return (int)p.size(); }
  char **v() { return p.data(); }
};

bool is_style(const std::string &s, std::initializer_list<const char *> names) {
  for (const char *n : names)
    if (s == n) return true;
  return false;
}

// LAMMPS data file, atom_style charge: header counts and box, Masses,
// Atoms (id type q x y z [ix iy iz]), Velocities (id vx vy vz)
void read_data(const std::string &path, reaxgb::Atom &A) {
  std::ifstream in(path);
  if (!in) throw Error("Cannot open file " + path);
  std::string line;
  std::getline(in, line);   // title
  long long natoms = -1;
  int ntypes = -1;
  bool have_box[3] = {false, false, false};
  std::string section;
  std::vector<std::string> w;
  // header
  while (true) {

    if (!std::getline(in, line)) break;
    w = split(line);
    if (w.empty()) continue;
    if (w.size() >= 2 && w[1] == "atoms") natoms = std::stoll(w[0]);
    else if (w.size() >= 3 && w[1] == "atom" && w[2] == "types") ntypes = std::stoi(w[0]);
    else if (w.size() >= 4 && w[2] == "xlo" && w[3] == "xhi") {
      A.boxlo[0] = std::stod(w[0]); A.boxhi[0] = std::stod(w[1]); have_box[0] = true;
    } else if (w.size() >= 4 && w[2] == "ylo" && w[3] == "yhi") {
      A.boxlo[1] = std::stod(w[0]); A.boxhi[1] = std::stod(w[1]); have_box[1] = true;
    } else if (w.size() >= 6 && w[3] == "xy") {
      if (std::stod(w[0]) != 0.0 || std::stod(w[1]) != 0.0 || std::stod(w[2]) != 0.0)
        throw Error("reax_md: triclinic boxes are not supported");
    } else if (w.size() >= 4 && w[2] == "zlo" && w[3] == "zhi") {
      A.boxlo[2] = std::stod(w[0]); A.boxhi[2] = std::stod(w[1]); have_box[2] = true;
    } else if (w.size() >= 3 && (w[1] == "bonds" || w[1] == "angles" || w[1] == "dihedrals" ||
                                 w[1] == "impropers" || w[2] == "types")) {
      continue;
    } else {
      section = w[0];
      break;
    }
  }
  if (natoms <= 0 || ntypes <= 0 || !have_box[0] || !have_box[1] || !have_box[2])
    throw Error("Invalid data file header in " + path);
  if (natoms > 2147483647LL) throw Error("Too many atoms");
  const int n = (int)natoms;
  A.nlocal = n;
  A.ntypes = ntypes;
  A.x.assign(3 * (size_t)n, 0.0);
  A.v.assign(3 * (size_t)n, 0.0);
  A.f.assign(3 * (size_t)n, 0.0);
  A.q.assign(n, 0.0);
  A.type.assign(n, 0);
  A.tag.assign(n, 0);
  if (A.mass.size() < (size_t)ntypes + 1) A.mass.assign(ntypes + 1, 0.0);
  std::map<long long, int> index;   // tag -> slot (Atoms order)
  bool have_atoms = false;
  while (!section.empty()) {
    std::string next;
    std::vector<std::vector<std::string>> rows;
    while (std::getline(in, line)) {
      w = split(line);
      if (w.empty()) continue;
      if (std::isalpha((unsigned char)w[0][0])) {
        next = w[0];
        break;
      }
      rows.push_back(w);
    }
    if (section == "Masses") {
      for (auto &r : rows) {
        const int t = std::stoi(r[0]);
        if (t < 1 || t > ntypes) throw Error("Invalid type for mass set");
        A.mass[t] = std::stod(r[1]);
      }
    } else if (section == "Atoms") {
      if ((long long)rows.size() != natoms) throw Error("Unexpected end of data file");
      for (int i = 0; i < n; ++i) {
        auto &r = rows[i];
        if (r.size() < 6) throw Error("Incorrect atom format in data file");
        A.tag[i] = std::stoi(r[0]);
        A.type[i] = std::stoi(r[1]);
        if (A.type[i] < 1 || A.type[i] > ntypes) throw Error("Invalid atom type in Atoms section of data file");
        A.q[i] = std::stod(r[2]);
        for (int c = 0; c < 3; ++c) A.x[3 * i + c] = std::stod(r[3 + c]);
        if (!index.emplace(A.tag[i], i).second) throw Error("Duplicate atom IDs in data file");
      }
      have_atoms = true;
    } else if (section == "Velocities") {
      for (auto &r : rows) {
        auto it = index.find(std::stoll(r[0]));
        if (it == index.end() || r.size() < 4) throw Error("Invalid atom ID in Velocities section of data file");
        for (int c = 0; c < 3; ++c) A.v[3 * it->second + c] = std::stod(r[1 + c]);
      }
    } else {
      throw Error("Unknown identifier in data file: " + section);
    }
    section = next;
  }
  if (!have_atoms) throw Error("No Atoms section in data file");
}

void write_dump(const std::string &path, const std::vector<std::string> &cols,
                const reaxgb::Atom &A, const reaxgb::PairReaxCGB300 &pair, long long step) {
  std::FILE *fp = std::fopen(path.c_str(), "w");
  if (!fp) throw Error("Cannot open dump file " + path);
  std::fprintf(fp, "# step %lld\n# pvector", step);
  for (double e : pair.pvector) std::fprintf(fp, " %.17g", e);
  std::fprintf(fp, "\n# eng_vdwl %.17g eng_coul %.17g\n#", pair.eng_vdwl, pair.eng_coul);
  for (auto &c : cols) std::fprintf(fp, " %s", c.c_str());
  std::fprintf(fp, "\n");
  std::vector<int> order(A.nlocal);
  for (int i = 0; i < A.nlocal; ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](int a, int b) { return A.tag[a] < A.tag[b]; });
  for (int i : order) {
    for (auto &c : cols) {
      if (c == "id") std::fprintf(fp, " %d", A.tag[i]);
      else if (c == "type") std::fprintf(fp, " %d", A.type[i]);
      else if (c == "q") std::fprintf(fp, " %.17g", A.q[i]);
      else if (c == "x") std::fprintf(fp, " %.17g", A.x[3 * i]);
      else if (c == "y") std::fprintf(fp, " %.17g", A.x[3 * i + 1]);
      else if (c == "z") std::fprintf(fp, " %.17g", A.x[3 * i + 2]);
      else if (c == "vx") std::fprintf(fp, " %.17g", A.v[3 * i]);
      else if (c == "vy") std::fprintf(fp, " %.17g", A.v[3 * i + 1]);
      else if (c == "vz") std::fprintf(fp, " %.17g", A.v[3 * i + 2]);
      else if (c == "fx") std::fprintf(fp, " %.17g", A.f[3 * i]);
      else if (c == "fy") std::fprintf(fp, " %.17g", A.f[3 * i + 1]);
      else if (c == "fz") std::fprintf(fp, " %.17g", A.f[3 * i + 2]);
    }
    std::fprintf(fp, "\n");
  }
  std::fclose(fp);
}

struct Thermo {
  reaxgb::PairReaxCGB300 *pair;
  reaxgb::FixQEqReaxGB300 *qeq;
};

void print_thermo(const reaxgb::Verlet &V, void *ctx) {
  const Thermo &T = *(const Thermo *)ctx;
  const double pe = T.pair->eng_vdwl + T.pair->eng_coul;
  const double ke = V.kinetic_energy();
  std::printf("%10lld %20.10f %20.10f %20.10f %8d\n", V.update_->ntimestep, pe, ke, pe + ke,
              T.qeq ? T.qeq->matvecs : 0);
}

int run_deck(std::istream &in) {
  reaxgb::Atom atom;
  reaxgb::Update update;
  std::unique_ptr<reaxgb::PairReaxCGB300> pair;
  std::unique_ptr<reaxgb::FixQEqReaxGB300> qeq;
  std::unique_ptr<reaxgb::FixNVEGB300> nve;
  std::unique_ptr<reaxgb::Verlet> verlet;
  std::vector<std::unique_ptr<reaxgb::FixReaxCBondsGB300>> bonds;
  bool have_data = false, setup_done = false;
  int thermo_every = 0;
  std::string line;
  int lineno = 0;
  while (std::getline(in, line)) {
    ++lineno;
    const auto w = split(line);
    if (w.empty()) continue;
    const std::string &cmd = w[0];
    if (cmd == "units") {
      if (w.size() != 2 || w[1] != "real") throw Error("reax/c/gb300 requires units real");
    } else if (cmd == "atom_style") {
      if (w.size() != 2 || w[1] != "charge") throw Error("reax_md supports atom_style charge");
    } else if (cmd == "boundary") {
      if (w.size() != 4 || w[1] != "p" || w[2] != "p" || w[3] != "p")
        throw Error("reax_md supports boundary p p p");
    } else if (cmd == "read_data") {
      if (w.size() < 2) throw Error("Illegal read_data command");
      read_data(w[1], atom);
      have_data = true;
    } else if (cmd == "mass") {
      if (!have_data || w.size() != 3) throw Error("Illegal mass command");
      const int t = std::stoi(w[1]);
      if (t < 1 || t > atom.ntypes) throw Error("Invalid type for mass set");
      atom.mass[t] = std::stod(w[2]);
    } else if (cmd == "pair_style") {
      if (w.size() < 2) throw Error("Illegal pair_style command");
      if (!is_style(w[1], {"reax/c", "reax/c/sunway", "reax/c/gb300"}))
        throw Error("Unrecognized pair style " + w[1]);
      if (!have_data) throw Error("Pair_style command when no atoms have been defined");
      pair.reset(new reaxgb::PairReaxCGB300(&atom));
      Args a(w, 2);
      pair->settings(a.n(), a.v());
    } else if (cmd == "pair_coeff") {
      if (!pair) throw Error("Pair_coeff command before pair_style is defined");
      Args a(w, 1);
      pair->coeff(a.n(), a.v());
    } else if (cmd == "fix") {
      if (w.size() < 4) throw Error("Illegal fix command");
      if (w[2] != "all") throw Error("reax_md supports fixes on group all only");
      Args a(w, 1);
      if (is_style(w[3], {"qeq/reax", "qeq/reax/sunway", "qeq/reax/gb300"})) {
        qeq.reset(new reaxgb::FixQEqReaxGB300(pair.get(), &update, a.n(), a.v()));
      } else if (is_style(w[3], {"nve", "nve/sunway", "nve/gb300"})) {
        nve.reset(new reaxgb::FixNVEGB300(pair.get(), &update, a.n(), a.v()));
      } else if (is_style(w[3], {"reax/c/bonds", "reax/c/bonds/sunway", "reax/c/bonds/gb300"})) {
        bonds.emplace_back(new reaxgb::FixReaxCBondsGB300(pair.get(), &atom, &update, a.n(), a.v()));
      } else {
        throw Error("Unrecognized fix style " + w[3]);
      }
    } else if (cmd == "timestep") {
      if (w.size() != 2) throw Error("Illegal timestep command");
      update.dt = std::stod(w[1]);
      if (nve) nve->reset_dt();
    } else if (cmd == "thermo") {
      if (w.size() != 2) throw Error("Illegal thermo command");
      thermo_every = std::stoi(w[1]);
    } else if (cmd == "neighbor" || cmd == "neigh_modify" || cmd == "thermo_style" ||
               cmd == "thermo_modify") {
      // the library builds its own lists every step; thermo columns fixed
    } else if (cmd == "run") {
      if (w.size() < 2) throw Error("Illegal run command");
      if (!pair) throw Error("Run command before pair style is defined");
      const long long n = std::stoll(w[1]);
      if (!verlet) {
        verlet.reset(new reaxgb::Verlet(&atom, &update, pair.get(), qeq.get(), nve.get()));
        for (auto &b : bonds) verlet->end_of_step_fixes.push_back(b.get());
      }
      Thermo T{pair.get(), qeq.get()};
      if (!setup_done) {
        verlet->setup();
        pair->sync_host();
        std::printf("%10s %20s %20s %20s %8s\n", "Step", "PotEng", "KinEng", "TotEng", "Matvecs");
        print_thermo(*verlet, &T);
        setup_done = true;
      }
      verlet->run(n, thermo_every > 0 ? thermo_every : (int)std::max<long long>(n, 1),
                  print_thermo, &T);
    } else if (cmd == "write_dump") {
      if (w.size() < 5 || w[1] != "all" || w[2] != "custom") throw Error("Illegal write_dump command");
      if (!pair || !setup_done) throw Error("write_dump before a run");
      std::vector<std::string> cols(w.begin() + 4, w.end());
      for (auto &c : cols)
        if (!is_style(c, {"id", "type", "q", "x", "y", "z", "vx", "vy", "vz", "fx", "fy", "fz"}))
          throw Error("Invalid attribute " + c + " in dump custom command");
      pair->sync_host();
      write_dump(w[3], cols, atom, *pair, update.ntimestep);
    } else {
      throw Error("Unknown command: " + line);
    }
  }
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  try {
    if (argc > 1 && std::strcmp(argv[1], "-") != 0) {
      std::ifstream in(argv[1]);
      if (!in) throw Error(std::string("Cannot open input script ") + argv[1]);
      return run_deck(in);
    }
    return run_deck(std::cin);
  } catch (const Error &e) {
    std::fprintf(stdout, "ERROR: %s\n", e.what());
    std::fflush(stdout);
    return 1;
  } catch (const std::exception &e) {
    std::fprintf(stdout, "ERROR: %s\n", e.what());
    std::fflush(stdout);
    return 1;
  }
}

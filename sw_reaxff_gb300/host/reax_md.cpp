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
//   (STYLE: qeq/reax, nve, reax/c/bonds, reax/c/species and their
//   /sunway, /gb300 names)
//   timestep DT | thermo N | run N |
//   write_dump all custom FILE COLS (id type q x y z vx vy vz fx fy fz)
//   neighbor / neigh_modify / thermo_style / thermo_modify: accepted, no effect
//
// and what the shipped TATB deck (in.reaxc.lattice) builds its crystal
// with: variable NAME index|equal ..., $x / ${name} substitution, "&" line
// continuation, lattice custom SCALE a1 .. a2 .. a3 .. basis .., region ID
// prism|block ... [units box], create_box N REGION, create_atoms TYPE box
// [basis I T ...]; read_data also takes the "xy xz yz" tilt line.  Index
// variables can be set on the command line: reax_md -var S 2 -in deck.
//
// Errors print "ERROR: <message>" and exit 1, as LAMMPS does.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdlib>
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
      A.xy = std::stod(w[0]);
      A.xz = std::stod(w[1]);
      A.yz = std::stod(w[2]);
      A.triclinic = 1;
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

// ---------------------------------------------------------------- input
// LAMMPS input-script mechanics (input.cpp, variable.cpp): "&" joins lines,
// "#" starts a comment, $x and ${name} are replaced by the variable's value
// before the command is parsed; index variables hold a string, equal
// variables a formula evaluated when referenced.
struct Variables {
  std::map<std::string, std::pair<std::string, std::string>> v;   // name -> (style, text)
  std::map<std::string, std::string> cmdline;                      // -var NAME VALUE

  double eval(const std::string &f) const {
    size_t pos = 0;
    const double r = expr(f, pos);
    skip(f, pos);
    if (pos != f.size()) throw Error("Invalid syntax in variable formula: " + f);
    return r;
  }
  std::string value(const std::string &name) const {
    auto it = v.find(name);
    if (it == v.end()) throw Error("Substitution for illegal variable " + name);
    if (it->second.first == "index") return it->second.second;
    char buf[64];
    std::snprintf(buf, sizeof buf, "%.15g", eval(it->second.second));
    return buf;
  }
  std::string substitute(const std::string &line) const {
    std::string out;
    for (size_t i = 0; i < line.size(); ++i) {
      if (line[i] != '$' || i + 1 >= line.size()) {
        out += line[i];
        continue;
      }
      std::string name;
      if (line[i + 1] == '{') {
        const size_t e = line.find('}', i + 2);
        if (e == std::string::npos) throw Error("Invalid variable name in: " + line);
        name = line.substr(i + 2, e - i - 2);
        i = e;
      } else {
        name = line.substr(i + 1, 1);
        i += 1;
      }
      out += value(name);
    }
    return out;
  }

 private:
  static void skip(const std::string &f, size_t &p) {
    while (p < f.size() && std::isspace((unsigned char)f[p])) ++p;
  }
  double expr(const std::string &f, size_t &p) const {
    double a = term(f, p);
    for (;;) {
      skip(f, p);
      if (p < f.size() && (f[p] == '+' || f[p] == '-')) {
        const char op = f[p++];
        const double b = term(f, p);
        a = op == '+' ? a + b : a - b;
      } else {
        return a;
      }
    }
  }
  double term(const std::string &f, size_t &p) const {
    double a = power(f, p);
    for (;;) {
      skip(f, p);
      if (p < f.size() && (f[p] == '*' || f[p] == '/')) {
        const char op = f[p++];
        const double b = power(f, p);
        if (op == '/' && b == 0.0) throw Error("Divide by 0 in variable formula");
        a = op == '*' ? a * b : a / b;
      } else {
        return a;
      }
    }
  }
  double power(const std::string &f, size_t &p) const {
    const double a = unary(f, p);
    skip(f, p);
    if (p < f.size() && f[p] == '^') {
      ++p;
      return std::pow(a, power(f, p));
    }
    return a;
  }
  double unary(const std::string &f, size_t &p) const {
    skip(f, p);
    if (p < f.size() && (f[p] == '-' || f[p] == '+')) {
      const char op = f[p++];
      const double a = unary(f, p);
      return op == '-' ? -a : a;
    }
    if (p < f.size() && f[p] == '(') {
      ++p;
      const double a = expr(f, p);
      skip(f, p);
      if (p >= f.size() || f[p] != ')') throw Error("Invalid syntax in variable formula: " + f);
      ++p;
      return a;
    }
    if (f.compare(p, 2, "v_") == 0) {
      size_t e = p + 2;
      while (e < f.size() && (std::isalnum((unsigned char)f[e]) || f[e] == '_')) ++e;
      const std::string name = f.substr(p + 2, e - p - 2);
      p = e;
      return std::stod(value(name));
    }
    const char *s = f.c_str() + p;
    char *end = nullptr;
    const double a = std::strtod(s, &end);
    if (end == s) throw Error("Invalid syntax in variable formula: " + f);
    p += (size_t)(end - s);
    return a;
  }
};

// lattice custom SCALE a1 x y z a2 x y z a3 x y z basis u v w ... (lattice.cpp)
struct Lattice {
  double scale = 1.0;
  double a[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  std::vector<std::array<double, 3>> basis;
};

// region ID prism xlo xhi ylo yhi zlo zhi xy xz yz | block xlo xhi ylo yhi zlo zhi
struct Region {
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  double xy = 0, xz = 0, yz = 0;
  bool prism = false;
};

double num(const std::string &s) {
  char *end = nullptr;
  const double v = std::strtod(s.c_str(), &end);
  if (end == s.c_str()) throw Error("Expected floating point parameter instead of " + s);
  return v;
}

Lattice make_lattice(const std::vector<std::string> &w) {
  if (w.size() < 3 || w[1] != "custom") throw Error("reax_md supports lattice custom only");
  Lattice L;
  L.scale = num(w[2]);
  for (size_t k = 3; k < w.size();) {
    if ((w[k] == "a1" || w[k] == "a2" || w[k] == "a3") && k + 3 < w.size()) {
      const int r = w[k][1] - '1';
      for (int c = 0; c < 3; ++c) L.a[r][c] = num(w[k + 1 + c]);
      k += 4;
    } else if (w[k] == "basis" && k + 3 < w.size()) {
      L.basis.push_back({num(w[k + 1]), num(w[k + 2]), num(w[k + 3])});
      k += 4;
    } else {
      throw Error("Illegal lattice command");
    }
  }
  if (L.basis.empty()) throw Error("No basis atoms in lattice");
  return L;
}

Region make_region(const std::vector<std::string> &w) {
  Region R;
  if (w.size() >= 9 && w[2] == "prism") {
    for (int c = 0; c < 3; ++c) {
      R.lo[c] = num(w[3 + 2 * c]);
      R.hi[c] = num(w[4 + 2 * c]);
    }
    if (w.size() < 12) throw Error("Illegal region prism command");
    R.xy = num(w[9]);
    R.xz = num(w[10]);
    R.yz = num(w[11]);
    R.prism = true;
  } else if (w.size() >= 9 && w[2] == "block") {
    for (int c = 0; c < 3; ++c) {
      R.lo[c] = num(w[3 + 2 * c]);
      R.hi[c] = num(w[4 + 2 * c]);
    }
  } else {
    throw Error("reax_md supports region prism|block with units box");
  }
  for (size_t k = R.prism ? 12 : 9; k < w.size(); k += 2)
    if (w[k] != "units" || k + 1 >= w.size() || w[k + 1] != "box")
      throw Error("reax_md supports region ... units box only");
  return R;
}

void create_box(const std::vector<std::string> &w, const std::map<std::string, Region> &regions,
                reaxgb::Atom &A) {
  if (w.size() < 3) throw Error("Illegal create_box command");
  auto it = regions.find(w[2]);
  if (it == regions.end()) throw Error("Create_box region ID does not exist");
  const Region &R = it->second;
  A.ntypes = std::stoi(w[1]);
  if (A.ntypes <= 0) throw Error("Illegal create_box command");
  for (int c = 0; c < 3; ++c) {
    A.boxlo[c] = R.lo[c];
    A.boxhi[c] = R.hi[c];
  }
  A.triclinic = R.prism ? 1 : 0;
  A.xy = R.xy;
  A.xz = R.xz;
  A.yz = R.yz;
  A.nlocal = 0;
  A.x.clear(); A.v.clear(); A.f.clear(); A.q.clear(); A.type.clear(); A.tag.clear();
  A.mass.assign(A.ntypes + 1, 0.0);
}

// create_atoms TYPE box [basis I T ...] on a lattice (CreateAtoms::
// add_lattice in LAMMPS): lattice points i + b over the lattice-coordinate
// bounding box of the simulation box, kept when their fractional box
// coordinates lie in [-eps, 1 - 2 eps) (eps = 1e-6, the periodic-edge rule
// of one process), in k, j, i, basis order; tags continue from the last.
void create_atoms(const std::vector<std::string> &w, const Lattice *lat, reaxgb::Atom &A) {
  if (w.size() < 3 || w[2] != "box") throw Error("reax_md supports create_atoms TYPE box");
  if (!lat) throw Error("Cannot create atoms with undefined lattice");
  if (A.ntypes <= 0) throw Error("Create_atoms command before simulation box is defined");
  const int deftype = std::stoi(w[1]);
  std::vector<int> btype(lat->basis.size(), deftype);
  for (size_t k = 3; k < w.size(); k += 3) {
    if (w[k] != "basis" || k + 2 >= w.size()) throw Error("Illegal create_atoms command");
    const int b = std::stoi(w[k + 1]), t = std::stoi(w[k + 2]);
    if (b < 1 || b > (int)btype.size() || t < 1 || t > A.ntypes)
      throw Error("Illegal create_atoms command");
    btype[b - 1] = t;
  }
  if (deftype < 1 || deftype > A.ntypes) throw Error("Invalid atom type in create_atoms command");
  const double lx = A.boxhi[0] - A.boxlo[0], ly = A.boxhi[1] - A.boxlo[1],
               lz = A.boxhi[2] - A.boxlo[2];
  const double xy = A.xy, xz = A.xz, yz = A.yz;
  // lattice matrix (columns a1, a2, a3 times the scale) and its inverse
  double M[3][3];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) M[r][c] = lat->scale * lat->a[c][r];
  const double det = M[0][0] * (M[1][1] * M[2][2] - M[1][2] * M[2][1]) -
                     M[0][1] * (M[1][0] * M[2][2] - M[1][2] * M[2][0]) +
                     M[0][2] * (M[1][0] * M[2][1] - M[1][1] * M[2][0]);
  if (det == 0.0) throw Error("Degenerate lattice primitive vectors");
  double Mi[3][3];
  Mi[0][0] = (M[1][1] * M[2][2] - M[1][2] * M[2][1]) / det;
  Mi[0][1] = (M[0][2] * M[2][1] - M[0][1] * M[2][2]) / det;
  Mi[0][2] = (M[0][1] * M[1][2] - M[0][2] * M[1][1]) / det;
  Mi[1][0] = (M[1][2] * M[2][0] - M[1][0] * M[2][2]) / det;
  Mi[1][1] = (M[0][0] * M[2][2] - M[0][2] * M[2][0]) / det;
  Mi[1][2] = (M[0][2] * M[1][0] - M[0][0] * M[1][2]) / det;
  Mi[2][0] = (M[1][0] * M[2][1] - M[1][1] * M[2][0]) / det;
  Mi[2][1] = (M[0][1] * M[2][0] - M[0][0] * M[2][1]) / det;
  Mi[2][2] = (M[0][0] * M[1][1] - M[0][1] * M[1][0]) / det;
  // lattice-coordinate range of the box's eight corners
  double lmin[3] = {1e300, 1e300, 1e300}, lmax[3] = {-1e300, -1e300, -1e300};
  for (int cz = 0; cz < 2; ++cz)
    for (int cy = 0; cy < 2; ++cy)
      for (int cx = 0; cx < 2; ++cx) {
        const double p[3] = {cx * lx + cy * xy + cz * xz, cy * ly + cz * yz, cz * lz};
        for (int r = 0; r < 3; ++r) {
          const double u = Mi[r][0] * p[0] + Mi[r][1] * p[1] + Mi[r][2] * p[2];
          lmin[r] = std::min(lmin[r], u);
          lmax[r] = std::max(lmax[r], u);
        }
      }
  int lo[3], hi[3];
  for (int r = 0; r < 3; ++r) {
    lo[r] = (int)std::floor(lmin[r]) - 1;
    hi[r] = (int)std::ceil(lmax[r]) + 1;
  }
  const double eps = 1e-6;
  int next_tag = 0;
  for (int t : A.tag) next_tag = std::max(next_tag, t);
  for (int k = lo[2]; k <= hi[2]; ++k)
    for (int j = lo[1]; j <= hi[1]; ++j)
      for (int i = lo[0]; i <= hi[0]; ++i)
        for (size_t m = 0; m < lat->basis.size(); ++m) {
          const double u[3] = {i + lat->basis[m][0], j + lat->basis[m][1], k + lat->basis[m][2]};
          double p[3];
          for (int r = 0; r < 3; ++r) p[r] = M[r][0] * u[0] + M[r][1] * u[1] + M[r][2] * u[2];
          // fractional coordinates in the box (origin boxlo)
          const double fz = p[2] / lz;
          const double fy = (p[1] - fz * yz) / ly;
          const double fx = (p[0] - fy * xy - fz * xz) / lx;
          if (fx < -eps || fx >= 1.0 - 2 * eps || fy < -eps || fy >= 1.0 - 2 * eps ||
              fz < -eps || fz >= 1.0 - 2 * eps)
            continue;
          for (int r = 0; r < 3; ++r) A.x.push_back(p[r] + A.boxlo[r]);
          for (int r = 0; r < 3; ++r) A.v.push_back(0.0);
          for (int r = 0; r < 3; ++r) A.f.push_back(0.0);
          A.q.push_back(0.0);
          A.type.push_back(btype[m]);
          A.tag.push_back(++next_tag);
          ++A.nlocal;
        }
}

void write_dump(const std::string &path, const std::vector<std::string> &cols,
                const reaxgb::Atom &A, const reaxgb::PairReaxCGB300 *pair, long long step) {
  std::FILE *fp = std::fopen(path.c_str(), "w");
  if (!fp) throw Error("Cannot open dump file " + path);
  std::fprintf(fp, "# step %lld\n# pvector", step);
  for (int k = 0; k < 14; ++k) std::fprintf(fp, " %.17g", pair ? pair->pvector[k] : 0.0);
  std::fprintf(fp, "\n# eng_vdwl %.17g eng_coul %.17g\n#", pair ? pair->eng_vdwl : 0.0,
               pair ? pair->eng_coul : 0.0);
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

// thermo columns of LAMMPS's default style in real units: temperature
// from 3N - 3 degrees of freedom (compute temp), pressure in atm from the
// kinetic energy and the pair virial (compute pressure: (2 KE + W_xx +
// W_yy + W_zz) / 3V times nktv2p)
void print_thermo(const reaxgb::Verlet &V, void *ctx) {
  const Thermo &T = *(const Thermo *)ctx;
  const reaxgb::Atom &A = *V.atom_;
  const double boltz = 0.0019872067, nktv2p = 68568.415;
  const double pe = T.pair->eng_vdwl + T.pair->eng_coul;
  const double ke = V.kinetic_energy();
  const int dof = 3 * A.nlocal - 3;
  const double temp = dof > 0 ? 2.0 * ke / (dof * boltz) : 0.0;
  const double vol = (A.boxhi[0] - A.boxlo[0]) * (A.boxhi[1] - A.boxlo[1]) * (A.boxhi[2] - A.boxlo[2]);
  const double *w = T.pair->virial;
  const double press = (2.0 * ke + w[0] + w[1] + w[2]) / (3.0 * vol) * nktv2p;
  std::printf("%10lld %14.6f %20.10f %20.10f %20.10f %14.4f %8d\n", V.update_->ntimestep, temp, pe,
              ke, pe + ke, press, T.qeq ? T.qeq->matvecs : 0);
}

int run_deck(std::istream &in, const std::map<std::string, std::string> &cmdvars) {
  Variables vars;
  vars.cmdline = cmdvars;
  for (auto &kv : cmdvars) vars.v[kv.first] = {"index", kv.second};
  std::unique_ptr<Lattice> lattice;
  std::map<std::string, Region> regions;
  reaxgb::Atom atom;
  reaxgb::Update update;
  std::unique_ptr<reaxgb::PairReaxCGB300> pair;
  std::unique_ptr<reaxgb::FixQEqReaxGB300> qeq;
  std::unique_ptr<reaxgb::FixNVEGB300> nve;
  std::unique_ptr<reaxgb::Verlet> verlet;
  std::vector<std::unique_ptr<reaxgb::StepFix>> bonds;   // bond and species output
  bool have_data = false, setup_done = false;
  int thermo_every = 0;
  std::string line, raw;
  int lineno = 0;
  while (std::getline(in, raw)) {
    ++lineno;
    // "&" at the end continues the command on the next line
    line = raw;
    while (true) {
      size_t e = line.find_last_not_of(" \t\r");
      if (e == std::string::npos || line[e] != '&') break;
      line.erase(e);
      if (!std::getline(in, raw)) break;
      ++lineno;
      line += " " + raw;
    }
    const size_t hash = line.find('#');
    if (hash != std::string::npos) line.erase(hash);
    line = vars.substitute(line);
    const auto w = split(line);
    if (w.empty()) continue;
    const std::string &cmd = w[0];
    if (cmd == "variable") {
      if (w.size() < 4) throw Error("Illegal variable command");
      if (w[2] == "index") {
        // a command-line value wins (LAMMPS -var)
        if (!vars.cmdline.count(w[1])) vars.v[w[1]] = {"index", w[3]};
      } else if (w[2] == "equal") {
        std::string f;
        for (size_t k = 3; k < w.size(); ++k) f += w[k];
        vars.v[w[1]] = {"equal", f};
      } else {
        throw Error("reax_md supports index and equal variables");
      }
    } else if (cmd == "lattice") {
      lattice.reset(new Lattice(make_lattice(w)));
    } else if (cmd == "region") {
      if (w.size() < 3) throw Error("Illegal region command");
      regions[w[1]] = make_region(w);
    } else if (cmd == "create_box") {
      if (have_data) throw Error("Cannot create_box after simulation box is defined");
      create_box(w, regions, atom);
      have_data = true;
    } else if (cmd == "create_atoms") {
      create_atoms(w, lattice.get(), atom);
    } else if (cmd == "units") {
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
      } else if (is_style(w[3], {"reax/c/species", "reax/c/species/sunway",
                                 "reax/c/species/gb300"})) {
        bonds.emplace_back(new reaxgb::FixReaxCSpeciesGB300(pair.get(), &atom, &update, a.n(), a.v()));
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
        std::printf("%10s %14s %20s %20s %20s %14s %8s\n", "Step", "Temp", "PotEng", "KinEng",
                    "TotEng", "Press", "Matvecs");
        print_thermo(*verlet, &T);
        setup_done = true;
      }
      verlet->run(n, thermo_every > 0 ? thermo_every : (int)std::max<long long>(n, 1),
                  print_thermo, &T);
    } else if (cmd == "write_dump") {
      if (w.size() < 5 || w[1] != "all" || w[2] != "custom") throw Error("Illegal write_dump command");
      if (!have_data) throw Error("Write_dump command before simulation box is defined");
      std::vector<std::string> cols(w.begin() + 4, w.end());
      for (auto &c : cols)
        if (!is_style(c, {"id", "type", "q", "x", "y", "z", "vx", "vy", "vz", "fx", "fy", "fz"}))
          throw Error("Invalid attribute " + c + " in dump custom command");
      // before the first run: the host arrays (no forces, energies zero)
      if (pair && setup_done) pair->sync_host();
      write_dump(w[3], cols, atom, pair.get(), update.ntimestep);
    } else {
      throw Error("Unknown command: " + line);
    }
  }
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  try {
    // reax_md [-var NAME VALUE ...] [-in] [FILE | -]
    std::map<std::string, std::string> cmdvars;
    std::string file;
    for (int k = 1; k < argc; ++k) {
      const std::string a = argv[k];
      if ((a == "-var" || a == "-v") && k + 2 < argc) {
        cmdvars[argv[k + 1]] = argv[k + 2];
        k += 2;
      } else if ((a == "-in" || a == "-i") && k + 1 < argc) {
        file = argv[++k];
      } else {
        file = a;
      }
    }
    if (!file.empty() && file != "-") {
      std::ifstream in(file);
      if (!in) throw Error("Cannot open input script " + file);
      return run_deck(in, cmdvars);
    }
    return run_deck(std::cin, cmdvars);
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

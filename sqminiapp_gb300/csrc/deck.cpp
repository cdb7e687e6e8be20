// deck.cpp -- readers for the reference's input files.
//
// .inpt keywords and defaults follow src/lsdft_readfiles.cc:62-331 (unknown
// tokens are skipped, as the reference's fscanf scanner does), .ion follows
// :677-789 and the Troullier-Martins pseudopotential format follows :858-1101
// (V_l = value/(2r) Ry->Ha, U_l = value/r, rho = value/(4 pi r^2), r=0 row copied
// from r[1]).  Errors throw sq::DeckError instead of exit(1).
#include <cmath>
#include <fstream>
#include <functional>
#include <map>
#include <sstream>
#include <stdexcept>

#include "sq_gb300.h"
#include "sq_internal.hpp"

namespace sq {

namespace {

struct TokenStream {
  std::vector<std::string> tok;
  size_t pos = 0;
  bool done() const { return pos >= tok.size(); }
  const std::string &next(const char *what) {
    if (pos >= tok.size()) throw std::runtime_error(std::string("unexpected end of deck reading ") + what);
    return tok[pos++];
  }
  int next_int(const char *what) { return std::stoi(next(what)); }
  double next_double(const char *what) { return std::stod(next(what)); }
};

TokenStream tokenize(const std::string &path) {
  std::ifstream f(path);
  if (!f) throw std::runtime_error("cannot open " + path);
  TokenStream ts;
  std::string s;
  while (f >> s) ts.tok.push_back(s);
  return ts;
}

// Checks shared by the file readers and the in-memory description.
void check_deck(const Deck &d, const std::string &where) {
  for (int a = 0; a < 3; a++)
    if (d.grid[a] < 2 || !(d.cell_half[a] > 0))
      throw std::runtime_error(where + ": CELL and FD_GRID must be positive");
  if (d.bc < 1 || d.bc > 4) throw std::runtime_error(where + ": BOUNDARY_CONDITION must be 1..4");
  if (d.n_qp < 1 || d.n_qp > 64) throw std::runtime_error(where + ": LANCZOS_DEGREE must be 1..64");
  if (!(d.rcut > 0)) throw std::runtime_error(where + ": RADIUS_TRUNC must be positive");
}

void check_psd(const Psd &p, const std::string &where) {
  if (p.lmax < 0 || p.lmax > 3) throw std::runtime_error(where + ": lmax must be 0..3");
  if (p.lloc < 0 || p.lloc > p.lmax)
    throw std::runtime_error(where + ": PSEUDOPOTENTIAL_LOCAL out of range");
  for (int l = 0; l <= p.lmax; l++)
    if (l != p.lloc && !p.has_u[l]) throw std::runtime_error(where + ": missing wave function for l");
}

void parse_inpt(Deck &d, const std::string &path) {
  TokenStream ts = tokenize(path);
  int ntype = -1;
  const std::map<std::string, std::function<void()>> handlers = {
      {"FD_ORDER:", [&] { d.half_order = ts.next_int("FD_ORDER") / 2; }},
      {"BOUNDARY_CONDITION:", [&] { d.bc = ts.next_int("BOUNDARY_CONDITION"); }},
      {"CELL:", [&] { for (double &v : d.cell_half) v = ts.next_double("CELL"); }},
      {"FD_GRID:", [&] { for (int &v : d.grid) v = ts.next_int("FD_GRID"); }},
      {"BETA:", [&] { d.beta = ts.next_double("BETA"); }},
      {"RADIUS_TRUNC:", [&] { d.rcut = ts.next_double("RADIUS_TRUNC"); }},
      {"LANCZOS_DEGREE:", [&] { d.n_qp = ts.next_int("LANCZOS_DEGREE"); }},
      {"EXCHANGE_CORRELATION:", [&] { d.xc = ts.next("EXCHANGE_CORRELATION"); }},
      {"MIXING_PARAMETER:", [&] { d.mixing_parameter = ts.next_double("MIXING_PARAMETER"); }},
      {"MIXING_HISTORY:", [&] { d.mixing_history = ts.next_int("MIXING_HISTORY"); }},
      {"PULAY_FREQUENCY:", [&] { d.pulay_frequency = ts.next_int("PULAY_FREQUENCY"); }},
      {"TOL_SCF:", [&] { d.tol_scf = ts.next_double("TOL_SCF"); }},
      {"MAXIT_SCF:", [&] { d.maxit_scf = ts.next_int("MAXIT_SCF"); }},
      {"REFERENCE_CUTOFF:", [&] { d.reference_cutoff = ts.next_double("REFERENCE_CUTOFF"); }},
      {"NTYPE:", [&] {
         ntype = ts.next_int("NTYPE");
         if (ntype <= 0 || ntype > kMaxTypes) throw std::runtime_error("NTYPE must be 1..8");
         d.lloc.assign(ntype, 0);
         d.psd_file.assign(ntype, "");
       }},
      {"PSEUDOPOTENTIAL_LOCAL:", [&] {
         if (ntype <= 0) throw std::runtime_error("Input number of types of elements first");
         for (int &v : d.lloc) v = ts.next_int("PSEUDOPOTENTIAL_LOCAL");
       }},
      {"PSEUDOPOTENTIAL_FILE:", [&] {
         if (ntype <= 0) throw std::runtime_error("Input number of types of elements first");
         for (auto &v : d.psd_file) v = ts.next("PSEUDOPOTENTIAL_FILE");
       }},
  };
  while (!ts.done()) {
    auto it = handlers.find(ts.next("keyword"));
    if (it != handlers.end()) it->second();
  }
  if (ntype <= 0) throw std::runtime_error(path + ": NTYPE missing");
  check_deck(d, path);
}

void parse_ion(Deck &d, const std::string &path) {
  TokenStream ts = tokenize(path);
  int natoms = ts.next_int("atom count");
  while (!ts.done()) {
    d.type_name.push_back(ts.next("atom type"));
    int ne = ts.next_int("valence");
    int na = ts.next_int("atoms of type");
    d.type_valence.push_back(ne);
    int t = (int)d.type_name.size() - 1;
    for (int i = 0; i < na; i++) {
      for (int c = 0; c < 3; c++) d.atom_xyz.push_back(ts.next_double("position"));
      d.atom_type.push_back(t);
      d.n_electrons += ne;
    }
  }
  if ((int)d.type_name.size() != (int)d.lloc.size())
    throw std::runtime_error(path + ": number of blocks differs from NTYPE");
  if ((int)d.atom_type.size() != natoms)
    throw std::runtime_error(path + ": atom count differs from the positions listed");
}

std::string trim(const std::string &s) {
  size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
  return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

Psd parse_psd(const std::string &path, const std::string &type_name, int lloc) {
  std::ifstream f(path);
  if (!f) throw std::runtime_error("cannot open pseudopotential " + path);
  Psd p;
  p.lloc = lloc;
  std::string line, first;
  std::getline(f, line);
  std::istringstream(line) >> first;
  if (first != type_name)
    throw std::runtime_error(path + ": pseudopotential does not match atom type " + type_name);
  // Split the file into "... follows" sections of numbers.
  std::vector<std::pair<std::string, std::vector<double>>> sec;
  while (std::getline(f, line)) {
    std::string t = trim(line);
    if (t.find("follows") != std::string::npos) {
      sec.push_back({t, {}});
      continue;
    }
    if (sec.empty()) continue;
    std::istringstream ss(line);
    double v;
    while (ss >> v) sec.back().second.push_back(v);
  }
  const std::vector<double> *grid = nullptr;
  for (auto &s : sec)
    if (s.first == "Radial grid follows") grid = &s.second;
  if (!grid || grid->size() < 3) throw std::runtime_error(path + ": no radial grid");
  const size_t nr = grid->size();
  p.r.assign(nr + 1, 0.0);
  for (size_t i = 0; i < nr; i++) p.r[i + 1] = (*grid)[i];
  p.vloc.assign(nr + 1, 0.0);
  p.rho_atom.assign(nr + 1, 0.0);
  for (int l = 0; l < 4; l++) {
    p.V[l].assign(nr + 1, 0.0);
    p.U[l].assign(nr + 1, 0.0);
  }
  for (auto &s : sec) {
    const auto &v = s.second;
    if (s.first == "Pseudopotential follows (l on next line)") {
      int l = (int)v.at(0);
      if (l < 0 || l > 3 || v.size() < nr + 1) throw std::runtime_error(path + ": bad potential block");
      p.lmax = l;
      for (size_t i = 1; i <= nr; i++) p.V[l][i] = 0.5 * v[i] / p.r[i];
      p.V[l][0] = p.V[l][1];
    } else if (s.first == "Valence charge follows") {
      if (v.size() < nr) throw std::runtime_error(path + ": bad valence block");
      for (size_t i = 1; i <= nr; i++) p.rho_atom[i] = v[i - 1] / (4 * M_PI * p.r[i] * p.r[i]);
      p.rho_atom[0] = 0.0;
    } else if (s.first == "Pseudo-wave-function follows (l, zelect, rc)") {
      int l = (int)v.at(0);
      if (l < 0 || l > 3 || v.size() < nr + 3) throw std::runtime_error(path + ": bad wave block");
      p.rc[l] = v[2];
      p.has_u[l] = true;
      for (size_t i = 1; i <= nr; i++) p.U[l][i] = v[i + 2] / p.r[i];
      p.U[l][0] = p.U[l][1];
    }
  }
  if (p.lmax < 0) throw std::runtime_error(path + ": no pseudopotential blocks");
  if (lloc < 0 || lloc > p.lmax) throw std::runtime_error(path + ": PSEUDOPOTENTIAL_LOCAL out of range");
  p.vloc = p.V[lloc];
  for (int l = 0; l <= p.lmax; l++)
    if (l != lloc && !p.has_u[l]) throw std::runtime_error(path + ": missing wave function for l");
  return p;
}

}  // namespace

Deck deck_from_system(const ::sq_system_desc &sys) {
  const std::string where = "sq_system_desc";
  Deck d;
  if (sys.fd_order < 2 || sys.fd_order % 2 || sys.fd_order / 2 != kStencilHalf)
    throw std::runtime_error(where + ": FD_ORDER must be " + std::to_string(2 * kStencilHalf));
  d.half_order = sys.fd_order / 2;
  d.bc = sys.bc;
  for (int a = 0; a < 3; a++) {
    d.cell_half[a] = sys.cell_half[a];
    d.grid[a] = sys.grid[a];
  }
  d.beta = sys.beta;
  d.rcut = sys.rcut;
  d.n_qp = sys.n_qp;
  if (sys.mixing_parameter > 0) d.mixing_parameter = sys.mixing_parameter;
  if (sys.mixing_history > 0) d.mixing_history = sys.mixing_history;
  if (sys.pulay_frequency > 0) d.pulay_frequency = sys.pulay_frequency;
  if (sys.tol_scf > 0) d.tol_scf = sys.tol_scf;
  if (sys.maxit_scf > 0) d.maxit_scf = sys.maxit_scf;
  if (sys.reference_cutoff > 0) d.reference_cutoff = sys.reference_cutoff;
  check_deck(d, where);
  if (!(sys.beta > 0)) throw std::runtime_error(where + ": BETA must be positive");
  if (sys.n_types <= 0 || sys.n_types > kMaxTypes || !sys.psd)
    throw std::runtime_error(where + ": NTYPE must be 1..8 with a psd per type");
  if (sys.n_atoms <= 0 || !sys.atom_type || !sys.atom_xyz)
    throw std::runtime_error(where + ": atoms missing");
  for (int t = 0; t < sys.n_types; t++) {
    const sq_psd_desc &in = sys.psd[t];
    const std::string w = where + " type " + std::to_string(t);
    if (in.n_r < 3 || !in.r || in.r[0] != 0.0)
      throw std::runtime_error(w + ": radial grid of at least 3 points starting at r = 0");
    for (int i = 1; i < in.n_r; i++)
      if (!(in.r[i] > in.r[i - 1])) throw std::runtime_error(w + ": radial grid must increase");
    Psd p;
    p.name = "type" + std::to_string(t);
    p.lmax = in.lmax;
    p.lloc = in.lloc;
    p.zval = in.valence;
    p.r.assign(in.r, in.r + in.n_r);
    p.rho_atom.assign(in.n_r, 0.0);
    if (in.rho_atom) p.rho_atom.assign(in.rho_atom, in.rho_atom + in.n_r);
    for (int l = 0; l < 4; l++) {
      p.V[l].assign(in.n_r, 0.0);
      p.U[l].assign(in.n_r, 0.0);
      if (l <= in.lmax) {
        if (!in.V[l]) throw std::runtime_error(w + ": V_l missing for l <= lmax");
        p.V[l].assign(in.V[l], in.V[l] + in.n_r);
        if (l != in.lloc && in.U[l]) {
          p.U[l].assign(in.U[l], in.U[l] + in.n_r);
          p.has_u[l] = true;
          p.rc[l] = in.rc[l];
        }
      }
    }
    check_psd(p, w);
    p.vloc = p.V[p.lloc];
    d.psd.push_back(p);
    d.lloc.push_back(in.lloc);
    d.psd_file.push_back("");
    d.type_name.push_back(p.name);
    d.type_valence.push_back(in.valence);
  }
  for (int i = 0; i < sys.n_atoms; i++) {
    const int t = sys.atom_type[i];
    if (t < 0 || t >= sys.n_types) throw std::runtime_error(where + ": atom type out of range");
    d.atom_type.push_back(t);
    for (int c = 0; c < 3; c++) d.atom_xyz.push_back(sys.atom_xyz[3 * i + c]);
    d.n_electrons += sys.psd[t].valence;
  }
  return d;
}

Deck read_deck(const std::string &dir, const std::string &name) {
  Deck d;
  const std::string base = dir + "/" + name;
  parse_inpt(d, base + ".inpt");
  parse_ion(d, base + ".ion");
  // .relax only constrains ionic relaxation (src/lsdft_readfiles.cc:794-852), which the
  // SQ pass never reads; it is accepted and ignored.
  for (size_t t = 0; t < d.lloc.size(); t++) {
    d.psd.push_back(parse_psd(dir + "/pseudopotential/" + d.psd_file[t], d.type_name[t], d.lloc[t]));
    d.psd.back().name = d.type_name[t];
    d.psd.back().zval = d.type_valence[t];
  }
  return d;
}

}  // namespace sq

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
  for (int a = 0; a < 3; a++)
    if (d.grid[a] < 2 || !(d.cell_half[a] > 0))
      throw std::runtime_error(path + ": CELL and FD_GRID must be positive");
  if (d.bc < 1 || d.bc > 4) throw std::runtime_error(path + ": BOUNDARY_CONDITION must be 1..4");
  if (d.n_qp < 1 || d.n_qp > 64) throw std::runtime_error(path + ": LANCZOS_DEGREE must be 1..64");
  if (!(d.rcut > 0)) throw std::runtime_error(path + ": RADIUS_TRUNC must be positive");
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

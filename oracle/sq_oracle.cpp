// sq_oracle.cpp -- FP64 CPU oracle of the reference per-node SQ path.
//
// TEST INFRASTRUCTURE ONLY (see sq_oracle.h).  Every function below names the
// reference file:line it restates.  The reference's PETSc objects are replaced
// by plain arrays with the same arithmetic: the truncated-cube Laplacian is a
// CSR matrix with ascending column order (PETSc SeqAIJ), Vec operations are
// plain loops.  Parity against reference OUTPUTS is unpinned (the reference
// prints no lambda/weights and needs PETSc+MPI to build).
//
// Build: g++ -O2 -ffp-contract=off -fPIC -shared -pthread (oracle/Makefile).
// -ffp-contract=off keeps the arithmetic identical to the reference's x86-64
// build on every host (no fused multiply-add contraction).

#include "sq_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// spline: src/lsdft_tools.cc:75-115 (getYD_gen), :122-151 (tridiag_gen),
//         :15-68 (SplineEvaluate)
// ---------------------------------------------------------------------------
void tridiag_gen(std::vector<double> &A, std::vector<double> &B, std::vector<double> &C,
                 std::vector<double> &D, int len) {
  std::vector<double> F(len);
  double b = B[0];
  D[0] = D[0] / b;
  for (int i = 1; i < len; i++) {
    F[i] = C[i - 1] / b;
    b = B[i] - A[i] * F[i];
    if (b == 0) throw std::runtime_error("Divide by zero in tridiag_gen");
    D[i] = (D[i] - D[i - 1] * A[i]) / b;
  }
  for (int i = len - 2; i >= 0; i--) D[i] -= (D[i + 1] * F[i + 1]);
}

std::vector<double> getYD_gen(const std::vector<double> &X, const std::vector<double> &Y) {
  int len = (int)X.size();
  std::vector<double> A(len), B(len), C(len), YD(len);
  double h0 = X[1] - X[0];
  double h1 = X[2] - X[1];
  double r0 = (Y[1] - Y[0]) / h0;
  double r1 = (Y[2] - Y[1]) / h1;
  B[0] = h1 * (h0 + h1);
  C[0] = (h0 + h1) * (h0 + h1);
  YD[0] = r0 * (3 * h0 * h1 + 2 * h1 * h1) + r1 * h0 * h0;
  int i;
  for (i = 1; i < len - 1; i++) {
    h0 = X[i] - X[i - 1];
    h1 = X[i + 1] - X[i];
    r0 = (Y[i] - Y[i - 1]) / h0;
    r1 = (Y[i + 1] - Y[i]) / h1;
    A[i] = h1;
    B[i] = 2 * (h0 + h1);
    C[i] = h0;
    YD[i] = 3 * (r0 * h1 + r1 * h0);
  }
  A[i] = (h0 + h1) * (h0 + h1);
  B[i] = h0 * (h0 + h1);
  YD[i] = r0 * h1 * h1 + r1 * (3 * h0 * h1 + 2 * h0 * h0);
  tridiag_gen(A, B, C, YD, len);
  return YD;
}

// One-point SplineEvaluate.  The reference scans linearly from j=0 for every
// call; a binary search finds the same interval (largest j with X[j] <= p,
// or j where p == X[j]) and gives identical arithmetic.
double spline_eval(const std::vector<double> &X, const std::vector<double> &Y,
                   const std::vector<double> &YD, double p) {
  int len = (int)X.size();
  if (p < X[0] || p > X[len - 1]) throw std::runtime_error("out of range in spline interpolation");
  // reference: for (; j < len && p > X[j]; j++); if (p < X[j]) j--;
  int j = (int)(std::lower_bound(X.begin(), X.end(), p) - X.begin());  // first X[j] >= p
  if (j >= len) j = len - 1;
  if (p < X[j]) j--;
  double p1 = X[j];
  double dx = 1.0 / (X[j + 1] - X[j]);
  double dy = (Y[j + 1] - Y[j]) * dx;
  double A0 = Y[j];
  double A1 = YD[j];
  double A2 = dx * (3.0 * dy - 2.0 * YD[j] - YD[j + 1]);
  double A3 = dx * dx * (-2.0 * dy + YD[j] + YD[j + 1]);
  double x = p - p1;
  return ((A3 * x + A2) * x + A1) * x + A0;
}

// ---------------------------------------------------------------------------
// RealSphericalHarmonic: src/lsdft_tools.cc:156-370 (l <= 3 restated)
// ---------------------------------------------------------------------------
double real_sph_harm(double x, double y, double z, int l, int m) {
  const double C00 = 0.282094791773878;
  const double C1m1 = 0.488602511902920, C10 = 0.488602511902920, C1p1 = 0.488602511902920;
  const double C2m2 = 1.092548430592079, C2m1 = 1.092548430592079, C20 = 0.315391565252520;
  const double C2p1 = 1.092548430592079, C2p2 = 0.546274215296040;
  const double C3m3 = 0.590043589926644, C3m2 = 2.890611442640554, C3m1 = 0.457045799464466;
  const double C30 = 0.373176332590115, C3p1 = 0.457045799464466, C3p2 = 1.445305721320277;
  const double C3p3 = 0.590043589926644;
  double r = sqrt(x * x + y * y + z * z);
  double SH = 0.0;
  if (l == 0) SH = C00;
  if (r >= 1e-10) {
    if (l == 0) {
      SH = C00;
    } else if (l == 1) {
      if (m == -1) SH = C1m1 * (y / r);
      else if (m == 0) SH = C10 * (z / r);
      else if (m == 1) SH = C1p1 * (x / r);
      else throw std::runtime_error("incorrect l,m");
    } else if (l == 2) {
      if (m == -2) SH = C2m2 * (x * y) / (r * r);
      else if (m == -1) SH = C2m1 * (y * z) / (r * r);
      else if (m == 0) SH = C20 * (-x * x - y * y + 2.0 * z * z) / (r * r);
      else if (m == 1) SH = C2p1 * (z * x) / (r * r);
      else if (m == 2) SH = C2p2 * (x * x - y * y) / (r * r);
      else throw std::runtime_error("incorrect l,m");
    } else if (l == 3) {
      if (m == -3) SH = C3m3 * (3 * x * x - y * y) * y / (r * r * r);
      else if (m == -2) SH = C3m2 * (x * y * z) / (r * r * r);
      else if (m == -1) SH = C3m1 * y * (4 * z * z - x * x - y * y) / (r * r * r);
      else if (m == 0) SH = C30 * z * (2 * z * z - 3 * x * x - 3 * y * y) / (r * r * r);
      else if (m == 1) SH = C3p1 * x * (4 * z * z - x * x - y * y) / (r * r * r);
      else if (m == 2) SH = C3p2 * z * (x * x - y * y) / (r * r * r);
      else if (m == 3) SH = C3p3 * x * (x * x - 3 * y * y) / (r * r * r);
      else throw std::runtime_error("incorrect l,m");
    } else {
      throw std::runtime_error("oracle supports l <= 3");
    }
  }
  return SH;
}

// fract: src/lsdft_tools.cc:519-531
double fract(int n, int k) {
  double Nr = 1, Dr = 1;
  for (int i = n - k + 1; i <= n; i++) Nr *= i;
  for (int i = n + 1; i <= n + k; i++) Dr *= i;
  return Nr / Dr;
}

// ---------------------------------------------------------------------------
// Deck
// ---------------------------------------------------------------------------
struct Psd {
  int size = 0, lmax = -1;
  std::vector<double> r;
  std::vector<double> V[4], U[4];
  std::vector<double> Vloc, uu;
  double rc[4] = {0, 0, 0, 0};  // rc[3] is uninitialised in the reference (3-channel psd); 0 here
  bool has_U[4] = {false, false, false, false};
  // setup (src/lsdft_initObjs.cc:576-622)
  std::vector<double> UDeltaV[4], YD_UDeltaV[4], YD_U[4], YD_Vloc;
  double Gamma[4] = {0, 0, 0, 0};
};

struct Deck {
  // .inpt (src/lsdft_readfiles.cc:62-331 defaults and keywords)
  int order = 6;
  int bc = 1;
  double range[3] = {0, 0, 0};
  int npts[3] = {0, 0, 0};
  double beta = 1000;
  double rcut = 12.0;
  int n_qp = 50;
  int ntype = -1;
  std::vector<int> lloc;
  std::vector<std::string> psd_name;
  // .ion (src/lsdft_readfiles.cc:677-789)
  int natoms = 0;
  std::vector<std::string> atom_type;
  std::vector<int> noe, noa;
  std::vector<double> pos;   // 3*natoms, in .ion order
  std::vector<int> type_of;  // per atom
  int noetot = 0;
};

std::vector<std::string> tokens_of(const std::string &path) {
  std::ifstream f(path);
  if (!f) throw std::runtime_error("Couldn't open config file " + path);
  std::vector<std::string> t;
  std::string s;
  while (f >> s) t.push_back(s);
  return t;
}

void read_inpt(Deck &d, const std::string &path) {
  auto t = tokens_of(path);
  size_t i = 0;
  auto need = [&](size_t k) {
    if (i + k >= t.size() + 1) throw std::runtime_error("truncated .inpt at " + t[i - 1]);
  };
  while (i < t.size()) {
    std::string k = t[i++];
    if (k == "FD_ORDER:") { need(1); d.order = std::stoi(t[i++]) / 2; }
    else if (k == "BOUNDARY_CONDITION:") { need(1); d.bc = std::stoi(t[i++]); }
    else if (k == "CELL:") { need(3); for (int a = 0; a < 3; a++) d.range[a] = std::stod(t[i++]); }
    else if (k == "FD_GRID:") { need(3); for (int a = 0; a < 3; a++) d.npts[a] = std::stoi(t[i++]); }
    else if (k == "BETA:") { need(1); d.beta = std::stod(t[i++]); }
    else if (k == "RADIUS_TRUNC:") { need(1); d.rcut = std::stod(t[i++]); }
    else if (k == "LANCZOS_DEGREE:") { need(1); d.n_qp = std::stoi(t[i++]); }
    else if (k == "NTYPE:") {
      need(1);
      d.ntype = std::stoi(t[i++]);
      d.lloc.assign(d.ntype, 0);
      d.psd_name.assign(d.ntype, "");
    } else if (k == "PSEUDOPOTENTIAL_LOCAL:") {
      if (d.ntype <= 0) throw std::runtime_error("Input number of types of elements first");
      for (int a = 0; a < d.ntype; a++) d.lloc[a] = std::stoi(t[i++]);
    } else if (k == "PSEUDOPOTENTIAL_FILE:") {
      if (d.ntype <= 0) throw std::runtime_error("Input number of types of elements first");
      for (int a = 0; a < d.ntype; a++) d.psd_name[a] = t[i++];
    }
  }
}

void read_ion(Deck &d, const std::string &path) {
  auto t = tokens_of(path);
  size_t i = 0;
  d.natoms = std::stoi(t.at(i++));
  while (i < t.size()) {
    d.atom_type.push_back(t[i++]);
    int ne = std::stoi(t.at(i++));
    int na = std::stoi(t.at(i++));
    d.noe.push_back(ne);
    d.noa.push_back(na);
    for (int a = 0; a < na; a++) {
      for (int c = 0; c < 3; c++) d.pos.push_back(std::stod(t.at(i++)));
      d.type_of.push_back((int)d.noe.size() - 1);
      d.noetot += ne;
    }
  }
  if ((int)d.atom_type.size() != d.ntype)
    throw std::runtime_error("Number of blocks in .ion file not same as number of atom types");
}

// Read_Pseudopotential: src/lsdft_readfiles.cc:858-1101 (TM format)
void read_psd(Psd &p, const std::string &path, const std::string &atype, int lloc) {
  std::ifstream f(path);
  if (!f) throw std::runtime_error("Couldn't open pseudopotential file " + path);
  std::vector<std::string> lines;
  std::string line;
  while (std::getline(f, line)) lines.push_back(line);
  {
    std::istringstream ss(lines.at(0));
    std::string first;
    ss >> first;
    if (first != atype) throw std::runtime_error("pseudopotential file does not match atom type");
  }
  auto trim = [](std::string s) {
    size_t a = s.find_first_not_of(" \t\r"), b = s.find_last_not_of(" \t\r");
    return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
  };
  // collect blocks: header line index -> numbers until next header
  struct Block { std::string head; std::vector<double> nums; };
  std::vector<Block> blocks;
  for (size_t li = 0; li < lines.size(); li++) {
    std::string tl = trim(lines[li]);
    if (tl.find("follows") != std::string::npos) {
      blocks.push_back({tl, {}});
    } else if (!blocks.empty()) {
      std::istringstream ss(lines[li]);
      double v;
      while (ss >> v) blocks.back().nums.push_back(v);
    }
  }
  int count = -1;
  for (auto &b : blocks)
    if (b.head == "Radial grid follows") count = (int)b.nums.size();
  if (count <= 0) throw std::runtime_error("no radial grid in psd");
  p.size = count + 1;
  p.r.assign(p.size, 0.0);
  for (auto &b : blocks)
    if (b.head == "Radial grid follows")
      for (int i = 1; i <= count; i++) p.r[i] = b.nums[i - 1];
  p.Vloc.assign(p.size, 0.0);
  p.uu.assign(p.size, 0.0);
  for (int l = 0; l < 4; l++) {
    p.V[l].assign(p.size, 0.0);
    p.U[l].assign(p.size, 0.0);
  }
  for (auto &b : blocks) {
    if (b.head == "Pseudopotential follows (l on next line)") {
      int l = (int)b.nums.at(0);
      if (l < 0 || l > 3) throw std::runtime_error("bad l in psd");
      p.lmax = l;
      for (int i = 1; i <= count; i++) {
        double value = 0.5 * b.nums.at(i) / p.r[i];
        p.V[l][i] = value;
        if (lloc == l) p.Vloc[i] = value;
      }
      p.V[l][0] = p.V[l][1];
      if (lloc == l) p.Vloc[0] = p.V[l][1];
    } else if (b.head == "Valence charge follows") {
      for (int i = 1; i <= count; i++) p.uu[i] = b.nums.at(i - 1) / (4 * M_PI * p.r[i] * p.r[i]);
      p.uu[0] = 0.0;
    } else if (b.head == "Pseudo-wave-function follows (l, zelect, rc)") {
      int l = (int)b.nums.at(0);
      double rc = b.nums.at(2);
      if (l < 0 || l > 3) throw std::runtime_error("bad l in psd");
      p.rc[l] = rc;
      p.has_U[l] = true;
      for (int i = 1; i <= count; i++) p.U[l][i] = b.nums.at(i + 2) / p.r[i];
      p.U[l][0] = p.U[l][1];
    }
  }
}

// ---------------------------------------------------------------------------
// The oracle system
// ---------------------------------------------------------------------------
struct Image {
  int type, atom;          // atom = index in .ion order (reference p = xindex/3)
  double X0, Y0, Z0;       // image position
  int xs, ys, zs, xe, ye, ze;  // footprint box clipped to the extended domain (global indices)
  // chi[((lm*nz + k)*ny + j)*nx + i] over the clipped box (src/lsdft_nl.cc:141-208)
  std::vector<double> chi;
};

struct System {
  Deck d;
  std::vector<Psd> psd;
  bool faithful = true;
  double h[3] = {0, 0, 0};
  int nloc[3] = {0, 0, 0}, nh[3] = {0, 0, 0};
  double dV = 0;
  std::vector<double> cx, cy, cz;                 // FD coefficients [0..o]
  std::vector<double> cutoff;                     // pseudocharge cutoff [ntype*3]
  std::vector<int> nlm;                           // per type
  std::vector<std::vector<int>> lm_l;             // per type: l of each lm
  std::vector<Image> images;
  // CSR of the cube Laplacian (src/lsdft_initObjs.cc:393-475), ascending columns
  std::vector<int> rowptr, col;
  std::vector<double> val;
  std::vector<int> diag_pos;
  int nc = 0;
};

// Calculate_NonlocalCoefficients: src/lsdft_initObjs.cc:822-869
void nonlocal_coefficients(System &S) {
  double delta = std::max(S.h[0], std::max(S.h[1], S.h[2]));
  // reference macro max(a,b,c) = (a>b&&a>c?a:b>c?b:c)
  delta = (S.h[0] > S.h[1] && S.h[0] > S.h[2]) ? S.h[0] : (S.h[1] > S.h[2] ? S.h[1] : S.h[2]);
  const double dr = 1e-6;
  for (int at = 0; at < S.d.ntype; at++) {
    Psd &p = S.psd[at];
    for (int l = 0; l <= p.lmax; l++) {
      p.Gamma[l] = 0.0;
      if (l == S.d.lloc[at]) continue;
      double rtemp = dr, Dexact = 0.0, UlDelVl = 0, Ul = 0;
      double Rc = p.rc[l];
      while (rtemp <= (Rc + delta)) {
        UlDelVl = spline_eval(p.r, p.UDeltaV[l], p.YD_UDeltaV[l], rtemp);
        Ul = spline_eval(p.r, p.U[l], p.YD_U[l], rtemp);
        Dexact += UlDelVl * Ul * rtemp * rtemp * dr;
        rtemp = rtemp + dr;
      }
      Dexact = (Dexact - 0.5 * UlDelVl * Ul * (rtemp - dr) * (rtemp - dr) * dr) / S.dV;
      p.Gamma[l] = 1.0 / Dexact;
    }
  }
}

// Calculate_PseudochargeCutoff: src/lsdft_initObjs.cc:628-817
void pseudocharge_cutoff(System &S, double tolerance) {
  const double MaxRadius = 15.0;
  int o = S.d.order;
  int Np[3];
  for (int a = 0; a < 3; a++) Np[a] = (int)ceil(MaxRadius / S.h[a]);
  double sc[3][16];
  for (int a = 0; a < 3; a++) {
    const std::vector<double> &c = a == 0 ? S.cx : (a == 1 ? S.cy : S.cz);
    for (int p = 0; p <= o; p++) sc[a][p] = c[p] / (2.0 * M_PI);
  }
  S.cutoff.assign(3 * S.d.ntype, 0.0);
  for (int at = 0; at < S.d.ntype; at++) {
    Psd &p = S.psd[at];
    int lloc = S.d.lloc[at];
    double Rcut = p.rc[lloc];
    int Ex = Np[0] + 2 * o, Ey = Np[1] + 2 * o, Ez = Np[2] + 2 * o;
    std::vector<double> Vps((size_t)Ex * Ey * Ez);
    auto VP = [&](int k, int j, int i) -> double & { return Vps[((size_t)k * Ey + j) * Ex + i]; };
    for (int k = 0; k < Ez; k++)
      for (int j = 0; j < Ey; j++)
        for (int i = 0; i < Ex; i++) {
          double x = (i - o) * S.h[0], y = (j - o) * S.h[1], z = (k - o) * S.h[2];
          double r = sqrt(x * x + y * y + z * z);
          VP(k, j, i) = spline_eval(p.r, p.Vloc, p.YD_Vloc, r);
        }
    std::vector<double> BJ((size_t)Np[0] * Np[1] * Np[2]);
    auto BJA = [&](int k, int j, int i) -> double & {
      return BJ[((size_t)k * Np[1] + j) * Np[0] + i];
    };
    for (int k = o; k < Np[2] + o; k++)
      for (int j = o; j < Np[1] + o; j++)
        for (int i = o; i < Np[0] + o; i++) {
          double v = VP(k, j, i) * (sc[0][0] + sc[1][0] + sc[2][0]);
          for (int a = 1; a <= o; a++) {
            v += (VP(k, j, i - a) + VP(k, j, i + a)) * sc[0][a] +
                 (VP(k, j - a, i) + VP(k, j + a, i)) * sc[1][a] +
                 (VP(k - a, j, i) + VP(k + a, j, i)) * sc[2][a];
          }
          BJA(k - o, j - o, i - o) = v;
        }
    int Nc[3] = {0, 0, 0};
    double error;
    do {
      for (int a = 0; a < 3; a++) Nc[a] = (int)ceil(Rcut / S.h[a]);
      double Bint = 0.0;
      for (int k = 0; k < Nc[2]; k++)
        for (int j = 0; j < Nc[1]; j++)
          for (int i = 0; i < Nc[0]; i++) {
            double val = BJA(k, j, i);
            if (k == 0) val = 0.5 * val;
            if (k == Nc[2] - 1) val = 0.5 * val;
            if (j == 0) val = 0.5 * val;
            if (j == Nc[1] - 1) val = 0.5 * val;
            if (i == 0) val = 0.5 * val;
            if (i == Nc[0] - 1) val = 0.5 * val;
            Bint += val;
          }
      Bint = Bint * 8.0 * S.dV;
      int ne = S.d.noe[at];
      error = fabs(Bint + ne) / fabs((double)ne);
      Rcut = Rcut + 1.0;
    } while (Rcut <= 15.0 && error > tolerance);
    for (int a = 0; a < 3; a++) S.cutoff[3 * at + a] = Nc[a] * S.h[a];
  }
}

// Check_Overlap: src/lsdft_initObjs.cc:2612-2663
int check_overlap(int xcor, int ycor, int zcor, int lxdim, int lydim, int lzdim, int xs, int ys,
                  int zs, int xl, int yl, int zl, int *xstart, int *ystart, int *zstart, int *xend,
                  int *yend, int *zend) {
  *xstart = *ystart = *zstart = *xend = *yend = *zend = -1000;
  if (xs >= xcor && xs <= xcor + lxdim - 1) *xstart = xs;
  else if (xcor >= xs && xcor <= xl) *xstart = xcor;
  if (xl >= xcor && xl <= xcor + lxdim - 1) *xend = xl;
  else if (xcor + lxdim - 1 >= xs && xcor + lxdim - 1 <= xl) *xend = xcor + lxdim - 1;
  if (ys >= ycor && ys <= ycor + lydim - 1) *ystart = ys;
  else if (ycor >= ys && ycor <= yl) *ystart = ycor;
  if (yl >= ycor && yl <= ycor + lydim - 1) *yend = yl;
  else if (ycor + lydim - 1 >= ys && ycor + lydim - 1 <= yl) *yend = ycor + lydim - 1;
  if (zs >= zcor && zs <= zcor + lzdim - 1) *zstart = zs;
  else if (zcor >= zs && zcor <= zl) *zstart = zcor;
  if (zl >= zcor && zl <= zcor + lzdim - 1) *zend = zl;
  else if (zcor + lzdim - 1 >= zs && zcor + lzdim - 1 <= zl) *zend = zcor + lzdim - 1;
  return (*xstart != -1000 && *xend != -1000 && *ystart != -1000 && *yend != -1000 &&
          *zstart != -1000 && *zend != -1000)
             ? 1
             : 0;
}

// grid index of a coordinate: xi = roundf((x0 + R)/h)  (src/lsdft_initObjs.cc:1810-1812);
// the double quotient is rounded to float before roundf, as in the reference.
inline int grid_round(double x0, double R, double h) {
  return (int)roundf((float)((x0 + R + 0.0) / h));
}

// periodic image index ranges (src/lsdft_initObjs.cc:1763-1784 faithful; corrected otherwise)
void image_range(const System &S, int at, int Imin[3], int Imax[3]) {
  for (int a = 0; a < 3; a++) Imin[a] = Imax[a] = 0;
  bool per[3] = {false, false, false};
  int bc = S.d.bc;
  if (S.faithful) {
    if (bc == 1) per[0] = per[1] = per[2] = true;
    else if (bc == 3) per[0] = per[1] = true;
    else if (bc == 4) per[0] = true;
    for (int a = 0; a < 3; a++)
      if (per[a]) {
        Imax[a] = (int)ceil(S.cutoff[3 * at + a] / S.d.range[a]);
        Imin[a] = -Imax[a];
      }
  } else {
    if (bc == 1 || bc == 2) per[0] = per[1] = per[2] = true;
    else if (bc == 3) per[0] = per[1] = true;
    else if (bc == 4) per[0] = true;
    const Psd &p = S.psd[at];
    double rcmax = std::max(std::max(p.rc[0], p.rc[1]), std::max(p.rc[2], p.rc[3]));
    for (int a = 0; a < 3; a++)
      if (per[a]) {
        int off = (int)ceil(rcmax / S.h[a]);
        double reach = (S.nh[a] + off + 1) * S.h[a];
        Imax[a] = (int)ceil(reach / (2.0 * S.d.range[a])) + 1;
        Imin[a] = -Imax[a];
      }
  }
}

// GetInfluencingAtoms_Nonlocal: src/lsdft_initObjs.cc:1671-1946 (one rank: owned block is the
// whole grid, extended by ceil(Rcut/h) on every side), then CalculateNonlocalProjectors
// src/lsdft_nl.cc:141-208 for the chi values of each overlapping image.
void build_images(System &S) {
  int cor[3], dim[3];
  for (int a = 0; a < 3; a++) {
    cor[a] = -S.nh[a];
    dim[a] = S.d.npts[a] + 2 * S.nh[a];
  }
  S.images.clear();
  for (int n = 0; n < S.d.natoms; n++) {
    int at = S.d.type_of[n];
    const Psd &p = S.psd[at];
    if (p.lmax == 0) continue;
    double max1 = p.rc[0] > p.rc[1] ? p.rc[0] : p.rc[1];
    double max2 = p.rc[2] > p.rc[3] ? p.rc[2] : p.rc[3];
    double rcnl = max1 > max2 ? max1 : max2;
    int off[3];
    for (int a = 0; a < 3; a++) off[a] = (int)ceil(rcnl / S.h[a]);
    int Imin[3], Imax[3];
    image_range(S, at, Imin, Imax);
    double X0 = S.d.pos[3 * n], Y0 = S.d.pos[3 * n + 1], Z0 = S.d.pos[3 * n + 2];
    for (int PP = Imin[0]; PP <= Imax[0]; PP++)
      for (int QQ = Imin[1]; QQ <= Imax[1]; QQ++)
        for (int RR = Imin[2]; RR <= Imax[2]; RR++) {
          double x0 = X0 + PP * 2.0 * S.d.range[0];
          double y0 = Y0 + QQ * 2.0 * S.d.range[1];
          double z0 = Z0 + RR * 2.0 * S.d.range[2];
          int xi = grid_round(x0, S.d.range[0], S.h[0]);
          int yj = grid_round(y0, S.d.range[1], S.h[1]);
          int zk = grid_round(z0, S.d.range[2], S.h[2]);
          Image im;
          if (!check_overlap(cor[0], cor[1], cor[2], dim[0], dim[1], dim[2], xi - off[0],
                             yj - off[1], zk - off[2], xi + off[0], yj + off[1], zk + off[2],
                             &im.xs, &im.ys, &im.zs, &im.xe, &im.ye, &im.ze))
            continue;
          im.type = at;
          im.atom = n;
          im.X0 = x0;
          im.Y0 = y0;
          im.Z0 = z0;
          int nx = im.xe - im.xs + 1, ny = im.ye - im.ys + 1, nz = im.ze - im.zs + 1;
          int nl = S.nlm[at];
          im.chi.assign((size_t)nl * nx * ny * nz, 0.0);
          int lmc = 0;
          for (int l = 0; l <= p.lmax; l++) {
            if (l == S.d.lloc[at]) continue;
            for (int m = -l; m <= l; m++, lmc++) {
              for (int k = 0; k < nz; k++) {
                double z = S.h[2] * (k + im.zs) - S.d.range[2] - z0;
                double zz = z * z;
                for (int j = 0; j < ny; j++) {
                  double y = S.h[1] * (j + im.ys) - S.d.range[1] - y0;
                  double yy = y * y;
                  for (int i = 0; i < nx; i++) {
                    double x = S.h[0] * (i + im.xs) - S.d.range[0] - x0;
                    double r = sqrt(x * x + yy + zz);
                    double u = spline_eval(p.r, p.UDeltaV[l], p.YD_UDeltaV[l], r);
                    double sh = real_sph_harm(x, y, z, l, m);
                    im.chi[(((size_t)lmc * nz + k) * ny + j) * nx + i] = u * sh;
                  }
                }
              }
            }
          }
          S.images.push_back(std::move(im));
        }
  }
}

// Create_LaplacianLocal: src/lsdft_initObjs.cc:393-475 as a CSR matrix with ascending
// columns (PETSc SeqAIJ sorts each row); Dirichlet zero outside the cube (DM_BOUNDARY_GHOSTED).
void build_laplacian(System &S) {
  int nx = S.nloc[0], ny = S.nloc[1], nz = S.nloc[2], o = S.d.order;
  S.nc = nx * ny * nz;
  S.rowptr.assign(S.nc + 1, 0);
  S.col.clear();
  S.val.clear();
  S.diag_pos.assign(S.nc, -1);
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        int row = (k * ny + j) * nx + i;
        std::vector<std::pair<int, double>> e;
        e.push_back({row, S.cx[0] + S.cy[0] + S.cz[0]});
        for (int l = 1; l <= o; l++) {
          if (k - l >= 0) e.push_back({((k - l) * ny + j) * nx + i, S.cz[l]});
          if (k + l < nz) e.push_back({((k + l) * ny + j) * nx + i, S.cz[l]});
          if (j - l >= 0) e.push_back({(k * ny + j - l) * nx + i, S.cy[l]});
          if (j + l < ny) e.push_back({(k * ny + j + l) * nx + i, S.cy[l]});
          if (i - l >= 0) e.push_back({(k * ny + j) * nx + i - l, S.cx[l]});
          if (i + l < nx) e.push_back({(k * ny + j) * nx + i + l, S.cx[l]});
        }
        std::sort(e.begin(), e.end());
        for (auto &p : e) {
          if (p.first == row) S.diag_pos[row] = (int)S.col.size();
          S.col.push_back(p.first);
          S.val.push_back(p.second);
        }
        S.rowptr[row + 1] = (int)S.col.size();
      }
}

System *open_system(const std::string &dir, const std::string &name, bool faithful) {
  System *S = new System();
  S->faithful = faithful;
  Deck &d = S->d;
  read_inpt(d, dir + "/" + name + ".inpt");
  read_ion(d, dir + "/" + name + ".ion");
  if (d.ntype <= 0) throw std::runtime_error("NTYPE missing");
  // mesh spacing: src/lsdft_readfiles.cc:356-411
  for (int a = 0; a < 3; a++) {
    bool periodic_axis = (d.bc == 2) || (d.bc == 3 && a < 2) || (d.bc == 4 && a == 0);
    if (d.bc < 1 || d.bc > 4) throw std::runtime_error("BOUNDARY_CONDITION must be 1..4");
    S->h[a] = periodic_axis ? 2.0 * d.range[a] / d.npts[a] : 2.0 * d.range[a] / (d.npts[a] - 1);
    S->nh[a] = (int)ceil(d.rcut / S->h[a]);
    S->nloc[a] = 2 * S->nh[a] + 1;
  }
  S->dV = S->h[0] * S->h[1] * S->h[2];
  // FD coefficients: src/lsdft_readfiles.cc:453-476
  int o = d.order;
  S->cx.assign(o + 1, 0.0);
  S->cy.assign(o + 1, 0.0);
  S->cz.assign(o + 1, 0.0);
  for (int a = 1; a <= o; a++) S->cx[0] += ((double)1.0 / (a * a));
  S->cy[0] = S->cx[0];
  S->cz[0] = S->cx[0];
  S->cx[0] *= ((double)1.0 / (S->h[0] * S->h[0]));
  S->cy[0] *= ((double)1.0 / (S->h[1] * S->h[1]));
  S->cz[0] *= ((double)1.0 / (S->h[2] * S->h[2]));
  for (int p = 1; p <= o; p++) {
    S->cx[p] = (double)(-1 * pow(-1, p + 1) * fract(o, p) / (p * p * S->h[0] * S->h[0]));
    S->cy[p] = (double)(-1 * pow(-1, p + 1) * fract(o, p) / (p * p * S->h[1] * S->h[1]));
    S->cz[p] = (double)(-1 * pow(-1, p + 1) * fract(o, p) / (p * p * S->h[2] * S->h[2]));
  }
  // pseudopotentials + spline fits: src/lsdft_initObjs.cc:576-622
  S->psd.resize(d.ntype);
  S->nlm.assign(d.ntype, 0);
  S->lm_l.assign(d.ntype, {});
  for (int at = 0; at < d.ntype; at++) {
    Psd &p = S->psd[at];
    read_psd(p, dir + "/pseudopotential/" + d.psd_name[at], d.atom_type[at], d.lloc[at]);
    p.YD_Vloc = getYD_gen(p.r, p.Vloc);
    for (int l = 0; l <= p.lmax; l++) {
      p.UDeltaV[l].assign(p.size, 0.0);
      for (int i = 0; i < p.size; i++) p.UDeltaV[l][i] = p.U[l][i] * (p.V[l][i] - p.Vloc[i]);
      p.YD_UDeltaV[l] = getYD_gen(p.r, p.UDeltaV[l]);
      p.YD_U[l] = getYD_gen(p.r, p.U[l]);
    }
    // N_lm = lmax^2 + 2(lmax - lloc): src/lsdft_nl.cc:55
    S->nlm[at] = p.lmax * p.lmax + 2 * (p.lmax - d.lloc[at]);
    for (int l = 0; l <= p.lmax; l++)
      if (l != d.lloc[at])
        for (int m = -l; m <= l; m++) S->lm_l[at].push_back(l);
    if ((int)S->lm_l[at].size() != S->nlm[at]) throw std::runtime_error("lm count mismatch");
  }
  nonlocal_coefficients(*S);
  pseudocharge_cutoff(*S, 1e-6);
  build_images(*S);
  build_laplacian(*S);
  return S;
}

// ---------------------------------------------------------------------------
// per-node work (src/lsdft_scf.cc:32-164, src/lsdft_matvec.cc:25-149)
// ---------------------------------------------------------------------------
struct NodeCtx {
  std::vector<double> diag;   // Laplacian diagonal + Veff (MatCopy + MatDiagonalSet, scf.cc:73-75)
  std::vector<int> img;       // images whose box meets the cube
  std::vector<long> abase;    // IP_index[p]: first alpha slot of atom p (initObjs.cc:947-964)
  std::vector<double> alpha;  // the alpha array of Mult_NonlocalVector (matvec.cc:52)
  int Xs, Ys, Zs, Xe, Ye, Ze;
};

void node_setup(const System &S, const double *veff, double veff_const, long node, NodeCtx &c) {
  int Nx = S.d.npts[0], Ny = S.d.npts[1], Nz = S.d.npts[2];
  int I = (int)(node % Nx), J = (int)((node / Nx) % Ny), K = (int)(node / ((long)Nx * Ny));
  // truncated-cube extent in unwrapped global indices (matvec.cc:38-45)
  c.Xs = I - S.nh[0]; c.Xe = I + S.nh[0];
  c.Ys = J - S.nh[1]; c.Ye = J + S.nh[1];
  c.Zs = K - S.nh[2]; c.Ze = K + S.nh[2];
  int nx = S.nloc[0], ny = S.nloc[1], nz = S.nloc[2];
  c.diag.assign(S.nc, 0.0);
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        int row = (k * ny + j) * nx + i;
        double v = veff_const;
        if (veff) {
          int gx = ((c.Xs + i) % Nx + Nx) % Nx, gy = ((c.Ys + j) % Ny + Ny) % Ny,
              gz = ((c.Zs + k) % Nz + Nz) % Nz;
          v = veff[((long)gz * Ny + gy) * Nx + gx];
        }
        c.diag[row] = S.val[S.diag_pos[row]] + v;
      }
  c.img.clear();
  for (int q = 0; q < (int)S.images.size(); q++) {
    const Image &im = S.images[q];
    // an image with no entry inside the cube adds nothing; skipping it keeps every sum intact
    if (im.xe < c.Xs || im.xs > c.Xe || im.ye < c.Ys || im.ys > c.Ye || im.ze < c.Zs ||
        im.zs > c.Ze)
      continue;
    c.img.push_back(q);
  }
  c.abase.assign(S.d.natoms + 1, 0);
  for (int n = 0; n < S.d.natoms; n++) c.abase[n + 1] = c.abase[n] + S.nlm[S.d.type_of[n]];
  c.alpha.assign(c.abase[S.d.natoms], 0.0);
}

// MatMult (AIJ, ascending columns) followed by Mult_NonlocalVector, which adds into y.
void hamiltonian_apply(const System &S, NodeCtx &c, const double *x, double *y) {
  for (int row = 0; row < S.nc; row++) {
    double sum = 0.0;
    for (int p = S.rowptr[row]; p < S.rowptr[row + 1]; p++) {
      double a = (S.col[p] == row) ? c.diag[row] : S.val[p];
      sum += a * x[S.col[p]];
    }
    y[row] = sum;
  }
  // Faithful: every (l,m) entry of atom p accumulates into alpha[IP_index[p]] (posIdx is reset
  // per entry, matvec.cc:97-100 and :136-138).  Corrected: one slot per (atom,l,m) as the
  // legacy Mult_HamiltonianVector indexes them (matvec.cc:214-227).
  int nx = S.nloc[0], ny = S.nloc[1];
  std::fill(c.alpha.begin(), c.alpha.end(), 0.0);
  for (int pass = 0; pass < 2; pass++) {
    for (int q : c.img) {
      const Image &im = S.images[q];
      int bx = im.xe - im.xs + 1, by = im.ye - im.ys + 1, bz = im.ze - im.zs + 1;
      int nl = S.nlm[im.type];
      double *al = c.alpha.data() + c.abase[im.atom];
      const std::vector<int> &lml = S.lm_l[im.type];
      const double *G = S.psd[im.type].Gamma;
      // flattened entry order of NonlocalProjectors (nl.cc:81-123): k, j, i, then (l, m)
      int zlo = std::max(im.zs, c.Zs), zhi = std::min(im.ze, c.Ze);
      int ylo = std::max(im.ys, c.Ys), yhi = std::min(im.ye, c.Ye);
      int xlo = std::max(im.xs, c.Xs), xhi = std::min(im.xe, c.Xe);
      size_t bvol = (size_t)bz * by * bx;
      for (int k = zlo; k <= zhi; k++)
        for (int j = ylo; j <= yhi; j++)
          for (int i = xlo; i <= xhi; i++) {
            int cidx = ((k - c.Zs) * ny + (j - c.Ys)) * nx + (i - c.Xs);
            size_t bidx = ((size_t)(k - im.zs) * by + (j - im.ys)) * bx + (i - im.xs);
            for (int lm = 0; lm < nl; lm++) {
              double chi = im.chi[(size_t)lm * bvol + bidx];
              int s = S.faithful ? 0 : lm;
              if (pass == 0) al[s] += x[cidx] * chi * G[lml[lm]];
              else y[cidx] += chi * al[s];
            }
          }
    }
  }
}

double vdot(const std::vector<double> &a, const std::vector<double> &b) {
  double s = 0.0;
  for (size_t i = 0; i < a.size(); i++) s += a[i] * b[i];
  return s;
}
double vnorm(const std::vector<double> &a) { return sqrt(vdot(a, a)); }

// TridiagEigenVecSolve_NodesAndWeights: src/lsdft_tools.cc:912-1026 (NR tqli with eigenvectors)
int ql_solve(const double *diag, const double *subdiag, int n, double *lam, double *wts,
             double *lmin, double *lmax) {
  std::vector<double> d(n), e(n), z((size_t)n * n, 0.0);
  for (int i = 0; i < n; i++) {
    d[i] = diag[i];
    e[i] = subdiag[i];
    z[(size_t)i * n + i] = 1.0;
  }
  auto SIGN = [](double a, double b) { return b >= 0.0 ? fabs(a) : -fabs(a); };
  e[n - 1] = 0.0;
  int m, iter, i;
  double s, r, p, g, f, dd, c, b;
  for (int l = 0; l <= n - 1; l++) {
    iter = 0;
    do {
      for (m = l; m <= n - 2; m++) {
        dd = fabs(d[m]) + fabs(d[m + 1]);
        if ((double)(fabs(e[m]) + dd) == dd) break;
      }
      if (m != l) {
        if (iter++ == 50) return 2;  // the reference prints and exit(1)s here
        g = (d[l + 1] - d[l]) / (2.0 * e[l]);
        r = sqrt(g * g + 1.0);
        g = d[m] - d[l] + e[l] / (g + SIGN(r, g));
        s = c = 1.0;
        p = 0.0;
        for (i = m - 1; i >= l; i--) {
          f = s * e[i];
          b = c * e[i];
          e[i + 1] = (r = sqrt(g * g + f * f));
          if (r == 0.0) {
            d[i + 1] -= p;
            e[m] = 0.0;
            break;
          }
          s = f / r;
          c = g / r;
          g = d[i + 1] - p;
          r = (d[i] - g) * s + 2.0 * c * b;
          d[i + 1] = g + (p = s * r);
          g = c * r - b;
          for (int k = 0; k < n; k++) {
            f = z[(size_t)k * n + i + 1];
            z[(size_t)k * n + i + 1] = s * z[(size_t)k * n + i] + c * f;
            z[(size_t)k * n + i] = c * z[(size_t)k * n + i] - s * f;
          }
        }
        if (r == 0.0 && i >= l) continue;
        d[l] -= p;
        e[l] = g;
        e[m] = 0.0;
      }
    } while (m != l);
  }
  double emin = d[0], emax = d[0];
  for (i = 0; i < n; i++) {
    lam[i] = d[i];
    wts[i] = z[i] * z[i];  // z[0][i]^2
    if (d[i] > emax) emax = d[i];
    else if (d[i] < emin) emin = d[i];
  }
  *lmin = emin;
  *lmax = emax;
  return 0;
}

// CalculateSpectralNodesAndWeights: src/lsdft_scf.cc:87-164
int node_lanczos(const System &S, NodeCtx &c, double *a, double *b) {
  int nqp = S.d.n_qp;
  int nx = S.nloc[0], ny = S.nloc[1], nz = S.nloc[2];
  std::vector<double> Vk(S.nc, 0.0), Vkm1(S.nc, 0.0), Vkp1(S.nc, 0.0);
  // Nmid: centre of the cube in natural ordering (scf.cc:53-57)
  int Nmid = ((nz - 1) / 2) * nx * ny + ((ny - 1) / 2) * nx + (nx - 1) / 2;
  Vkm1[Nmid] = 1.0;
  hamiltonian_apply(S, c, Vkm1.data(), Vk.data());
  a[0] = vdot(Vkm1, Vk);
  for (int i = 0; i < S.nc; i++) Vk[i] += -a[0] * Vkm1[i];
  b[0] = vnorm(Vk);
  double sc = 1.0 / b[0];
  for (int i = 0; i < S.nc; i++) Vk[i] *= sc;
  for (int k = 0; k < nqp; k++) {
    hamiltonian_apply(S, c, Vk.data(), Vkp1.data());
    a[k + 1] = vdot(Vk, Vkp1);
    for (int i = 0; i < S.nc; i++) Vkp1[i] += -a[k + 1] * Vk[i];
    for (int i = 0; i < S.nc; i++) Vkp1[i] += -b[k] * Vkm1[i];
    Vkm1 = Vk;
    b[k + 1] = vnorm(Vkp1);
    Vk = Vkp1;
    sc = 1.0 / b[k + 1];
    for (int i = 0; i < S.nc; i++) Vk[i] *= sc;
  }
  return 0;
}

double fermi_dirac(double beta, double lambda, double lambda_f) {
  return 1.0 / (1.0 + exp(beta * (lambda - lambda_f)));
}

thread_local std::string g_err;

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

void *sqo_open(const char *dir, const char *name, int faithful, char *err, int errlen) {
  try {
    return open_system(dir, name, faithful != 0);
  } catch (const std::exception &e) {
    if (err && errlen > 0) {
      strncpy(err, e.what(), errlen - 1);
      err[errlen - 1] = 0;
    }
    return nullptr;
  }
}

void sqo_close(void *h) { delete (System *)h; }

int sqo_dims(void *h, int *ints, double *dbls) {
  System &S = *(System *)h;
  int v[16] = {S.d.npts[0], S.d.npts[1], S.d.npts[2], S.nloc[0], S.nloc[1], S.nloc[2],
               S.d.n_qp, S.d.npts[0] * S.d.npts[1] * S.d.npts[2], S.d.ntype, S.d.natoms,
               (int)S.images.size(), S.d.order, S.d.bc, S.nlm[0], S.d.noetot, S.faithful ? 1 : 0};
  for (int i = 0; i < 16; i++) ints[i] = v[i];
  double w[16] = {S.h[0], S.h[1], S.h[2], S.d.range[0], S.d.range[1], S.d.range[2],
                  S.d.rcut, S.d.beta, S.dV, 0.333, 0, 0, 0, 0, 0, 0};
  for (int i = 0; i < 16; i++) dbls[i] = w[i];
  return 0;
}

int sqo_fd_coeffs(void *h, double *cx, double *cy, double *cz) {
  System &S = *(System *)h;
  for (int p = 0; p <= S.d.order; p++) {
    cx[p] = S.cx[p];
    cy[p] = S.cy[p];
    cz[p] = S.cz[p];
  }
  return 0;
}

int sqo_gamma(void *h, int type, double *gamma4) {
  System &S = *(System *)h;
  if (type < 0 || type >= S.d.ntype) return 1;
  for (int l = 0; l < 4; l++) gamma4[l] = S.psd[type].Gamma[l];
  return 0;
}

int sqo_pseudocharge_cutoff(void *h, double *out) {
  System &S = *(System *)h;
  for (size_t i = 0; i < S.cutoff.size(); i++) out[i] = S.cutoff[i];
  return 0;
}

int sqo_psd_tables(void *h, int type, int *n, double *r, double *vloc, double *rho_atom,
                   double *zval) {
  System &S = *(System *)h;
  if (type < 0 || type >= S.d.ntype) return 1;
  const Psd &p = S.psd[type];
  *n = p.size;
  for (int i = 0; i < p.size; i++) {
    if (r) r[i] = p.r[i];
    if (vloc) vloc[i] = p.Vloc[i];
    if (rho_atom) rho_atom[i] = p.uu[i];
  }
  if (zval) *zval = S.d.noe[type];
  return 0;
}

int sqo_atoms(void *h, double *pos, int *types) {
  System &S = *(System *)h;
  for (int n = 0; n < S.d.natoms; n++) {
    for (int a = 0; a < 3; a++) pos[3 * n + a] = S.d.pos[3 * n + a];
    types[n] = S.d.type_of[n];
  }
  return 0;
}

// GetInfluencingAtoms_Local: src/lsdft_initObjs.cc:1409-1665
int sqo_local_overlap_count(void *h, int xcor, int ycor, int zcor, int lx, int ly, int lz,
                            const double *extra_xyz, int *count) {
  System &S = *(System *)h;
  int total = 0;
  int nat = S.d.natoms + (extra_xyz ? 1 : 0);
  for (int n = 0; n < nat; n++) {
    int at = n < S.d.natoms ? S.d.type_of[n] : 0;
    double X0, Y0, Z0;
    if (n < S.d.natoms) {
      X0 = S.d.pos[3 * n]; Y0 = S.d.pos[3 * n + 1]; Z0 = S.d.pos[3 * n + 2];
    } else {
      X0 = extra_xyz[0]; Y0 = extra_xyz[1]; Z0 = extra_xyz[2];
    }
    int off[3], Imin[3] = {0, 0, 0}, Imax[3] = {0, 0, 0};
    for (int a = 0; a < 3; a++) off[a] = (int)ceil(S.cutoff[3 * at + a] / S.h[a] + 0.5);
    bool per[3] = {S.d.bc == 1 || S.d.bc == 3 || S.d.bc == 4, S.d.bc == 1 || S.d.bc == 3,
                   S.d.bc == 1};
    for (int a = 0; a < 3; a++)
      if (per[a]) {
        Imax[a] = (int)ceil(S.cutoff[3 * at + a] / S.d.range[a]);
        Imin[a] = -Imax[a];
      }
    for (int PP = Imin[0]; PP <= Imax[0]; PP++)
      for (int QQ = Imin[1]; QQ <= Imax[1]; QQ++)
        for (int RR = Imin[2]; RR <= Imax[2]; RR++) {
          double x0 = X0 + PP * 2.0 * S.d.range[0];
          double y0 = Y0 + QQ * 2.0 * S.d.range[1];
          double z0 = Z0 + RR * 2.0 * S.d.range[2];
          int xi = grid_round(x0, S.d.range[0], S.h[0]);
          int yj = grid_round(y0, S.d.range[1], S.h[1]);
          int zk = grid_round(z0, S.d.range[2], S.h[2]);
          int a0, a1, a2, a3, a4, a5;
          total += check_overlap(xcor, ycor, zcor, lx, ly, lz, xi - off[0], yj - off[1],
                                 zk - off[2], xi + off[0], yj + off[1], zk + off[2], &a0, &a1,
                                 &a2, &a3, &a4, &a5);
        }
  }
  *count = total;
  return 0;
}

int sqo_nodes_and_weights(void *h, const double *veff, double veff_const, const long *nodes,
                          long nsel, int nthreads, double *a, double *b, double *lambda,
                          double *w, double *lmin, double *lmax) {
  System &S = *(System *)h;
  int nqp = S.d.n_qp;
  long nnodes = (long)S.d.npts[0] * S.d.npts[1] * S.d.npts[2];
  for (long t = 0; t < nsel; t++)
    if (nodes[t] < 0 || nodes[t] >= nnodes) return 1;
  if (nthreads < 1) nthreads = 1;
  std::atomic<long> next(0);
  std::atomic<int> status(0);
  auto work = [&]() {
    NodeCtx c;
    std::vector<double> aa(nqp + 1), bb(nqp + 1);
    for (;;) {
      long t = next.fetch_add(1);
      if (t >= nsel) break;
      node_setup(S, veff, veff_const, nodes[t], c);
      node_lanczos(S, c, aa.data(), bb.data());
      if (a) for (int i = 0; i <= nqp; i++) a[t * (nqp + 1) + i] = aa[i];
      if (b) for (int i = 0; i <= nqp; i++) b[t * (nqp + 1) + i] = bb[i];
      int st = ql_solve(aa.data(), bb.data(), nqp, lambda + t * nqp, w + t * nqp, lmin + t,
                        lmax + t);
      if (st) status = st;
    }
  };
  std::vector<std::thread> pool;
  for (int i = 1; i < nthreads; i++) pool.emplace_back(work);
  work();
  for (auto &th : pool) th.join();
  return status;
}

int sqo_matvec(void *h, const double *veff, double veff_const, long node, const double *x,
               double *y) {
  System &S = *(System *)h;
  NodeCtx c;
  node_setup(S, veff, veff_const, node, c);
  hamiltonian_apply(S, c, x, y);
  return 0;
}

int sqo_ql(const double *diag, const double *sub, int n, double *lambda, double *w, double *lmin,
           double *lmax) {
  return ql_solve(diag, sub, n, lambda, w, lmin, lmax);
}

// Fermi level / density / energy of the SQ method.  The reference only declares these
// (src/lsdft.h:98-102 constraint_lssgq, FermiDirac, CalculateDensity_lssgq, findRootBrent;
// :209 SystemEnergy_Calc_lssgq), so this is the published SQ quadrature restated in FP64:
// N_e(lf) = 2 sum_i sum_q w_iq f(lambda_iq - lf), bisection on [min lambda, max lambda].
int sqo_fermi_density_energy(const double *lambda, const double *w, long n_nodes, int n_qp,
                             double beta, double n_electrons, double dV, double tol, int maxit,
                             double *lambda_f, double *rho, double *e_band, double *ts,
                             int *iters) {
  long n = n_nodes * (long)n_qp;
  double lo = lambda[0], hi = lambda[0];
  for (long i = 0; i < n; i++) {
    lo = std::min(lo, lambda[i]);
    hi = std::max(hi, lambda[i]);
  }
  lo -= 1.0;
  hi += 1.0;
  int it = 0;
  double mid = 0.5 * (lo + hi);
  for (it = 0; it < maxit; it++) {
    mid = 0.5 * (lo + hi);
    double ne = 0.0;
    for (long i = 0; i < n; i++) ne += 2.0 * w[i] * fermi_dirac(beta, lambda[i], mid);
    if (ne > n_electrons) hi = mid;
    else lo = mid;
    if (hi - lo < tol) break;
  }
  double lf = 0.5 * (lo + hi);
  *lambda_f = lf;
  if (iters) *iters = it;
  double eb = 0.0, s = 0.0;
  for (long node = 0; node < n_nodes; node++) {
    double r = 0.0;
    for (int q = 0; q < n_qp; q++) {
      long i = node * n_qp + q;
      double f = fermi_dirac(beta, lambda[i], lf);
      r += w[i] * f;
      eb += 2.0 * w[i] * lambda[i] * f;
      double e = 0.0;
      if (f > 0.0 && f < 1.0) e = f * log(f) + (1.0 - f) * log(1.0 - f);
      s += 2.0 * w[i] * e;
    }
    if (rho) rho[node] = 2.0 * r / dV;
  }
  *e_band = eb;
  *ts = s / beta;
  return 0;
}

int sqo_spline(const double *x, const double *y, int n, const double *xq, double *yq, int nq) {
  try {
    std::vector<double> X(x, x + n), Y(y, y + n);
    std::vector<double> YD = getYD_gen(X, Y);
    for (int i = 0; i < nq; i++) yq[i] = spline_eval(X, Y, YD, xq[i]);
    return 0;
  } catch (...) {
    return 1;
  }
}

double sqo_ylm(double x, double y, double z, int l, int m) { return real_sph_harm(x, y, z, l, m); }

}  // extern "C"

// scf_setup.cpp -- fixed fields of the SCF closure (host, FP64).
//
// The reference declares the SCF pieces without bodies (src/lsdft.h:93 SolvePoisson, :183 mix,
// :197-204 Vxc_Calc*, :209 SystemEnergy_Calc_lssgq, :217-218 Generate_pseudocharge and
// PseudopotReference; the fields Eself, Eself_TM, Ecorrection of src/ilsdft.h:149-155).  They
// follow the real-space pseudocharge formulation that the reference's
// Calculate_PseudochargeCutoff (src/lsdft_initObjs.cc:628-817) is built for:
//   b_J    = -(1/4pi) Lap_FD V_loc,J on the box of half-width CUTOFF around atom image J, with
//            V_loc sampled at the exact atom position and the same 12th-order FD weights
//            (-(1/4pi) Lap = (1/2pi) times the -1/2 Laplacian stencil);
//   E_self = 1/2 sum_J int b_J V_J over the atoms of the cell (one image each);
//   E_c    = 1/2 int (b_ref + b) V_c + E_self - E_self,ref with V_c = sum_J (V_ref,J - V_J),
//            the overlap correction of Ghosh and Suryanarayana (SPARC) with the reference
//            potential of REFERENCE_CUTOFF (src/lsdft_readfiles.cc:80,225);
//   rho_0  = sum of the isolated-atom valence densities (the psd "Valence charge" block,
//            src/lsdft_readfiles.cc:1033-1039), scaled to the valence electron count;
//   G(k)   = 2 pi / s(k), s(k) the Fourier symbol of the FD -1/2 Laplacian on the periodic
//            grid, so phi = IFFT(G FFT(rho + b)) solves -(1/4pi) Lap_FD phi = rho + b exactly
//            for the discrete operator of Create_Laplacian (src/lsdft_initObjs.cc:308-367);
//            k = 0 is dropped (a neutralising background for the residual net charge).
#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <thread>

#include "radial_spline.hpp"
#include "scf_internal.hpp"

namespace sq {

double reference_potential(double r, double rc, double z) {
  if (r >= rc) return -z / r;
  const double R = r / rc, R2 = R * R, R5 = R2 * R2 * R;
  return -z / rc * (9.0 * R5 * R2 - 30.0 * R5 * R + 28.0 * R5 - 14.0 * R2 + 12.0) / 5.0;
}

namespace {

struct TypeFields {
  RadialSpline vloc, rho;
  double z = 0.0, rmax_rho = 0.0, rmax_table = 0.0;
  int nb[3] = {0, 0, 0};  // pseudocharge box half-width in points
  int nr[3] = {0, 0, 0};  // valence-density box half-width in points
};

struct Partial {
  std::vector<double> b, b_ref, vc, rho;
  double e_self = 0.0, e_self_ref = 0.0;
};

struct Grid {
  int N[3];
  double L[3], half[3], h[3], dV;
  int o;
  const double (*c)[kStencilHalf + 1];
  long long index(int x, int y, int z) const { return ((long long)z * N[1] + y) * N[0] + x; }
  bool inside(int x, int y, int z) const {
    return x >= 0 && x < N[0] && y >= 0 && y < N[1] && z >= 0 && z < N[2];
  }
};

double vloc_at(const TypeFields &tf, double r) {
  return r <= tf.rmax_table ? tf.vloc(r) : -tf.z / r;
}

// Every periodic image of one atom: pseudocharges, correction potential and valence density
// on the cell grid; self energies from image 0 only.
void add_atom(const Grid &g, const TypeFields &tf, double rc_ref, const double X[3], Partial &out) {
  const int o = g.o;
  int pmax[3];
  for (int a = 0; a < 3; a++)
    pmax[a] = (int)std::ceil((std::max(tf.nb[a] + o, tf.nr[a]) * g.h[a]) / g.L[a]) + 1;
  const double c0 = (g.c[0][0] + g.c[1][0] + g.c[2][0]) / (2.0 * M_PI);
  std::vector<double> V, Vr;
  for (int P = -pmax[0]; P <= pmax[0]; P++)
    for (int Q = -pmax[1]; Q <= pmax[1]; Q++)
      for (int R = -pmax[2]; R <= pmax[2]; R++) {
        const bool home = P == 0 && Q == 0 && R == 0;
        const double x0[3] = {X[0] + P * g.L[0], X[1] + Q * g.L[1], X[2] + R * g.L[2]};
        int c[3];
        bool meets_b = true, meets_r = true;
        for (int a = 0; a < 3; a++) {
          c[a] = (int)std::lround((x0[a] + g.half[a]) / g.h[a]);
          if (c[a] + tf.nb[a] < 0 || c[a] - tf.nb[a] > g.N[a] - 1) meets_b = false;
          if (c[a] + tf.nr[a] < 0 || c[a] - tf.nr[a] > g.N[a] - 1) meets_r = false;
        }
        auto coord = [&](int a, int gi) { return g.h[a] * gi - g.half[a] - x0[a]; };
        if (meets_b || home) {
          const int ex[3] = {2 * (tf.nb[0] + o) + 1, 2 * (tf.nb[1] + o) + 1, 2 * (tf.nb[2] + o) + 1};
          const size_t ne = (size_t)ex[0] * ex[1] * ex[2];
          V.resize(ne);
          Vr.resize(ne);
          for (int k = 0; k < ex[2]; k++) {
            const double z = coord(2, c[2] - tf.nb[2] - o + k);
            for (int j = 0; j < ex[1]; j++) {
              const double y = coord(1, c[1] - tf.nb[1] - o + j);
              for (int i = 0; i < ex[0]; i++) {
                const double x = coord(0, c[0] - tf.nb[0] - o + i);
                const double r = std::sqrt(x * x + y * y + z * z);
                const size_t e = ((size_t)k * ex[1] + j) * ex[0] + i;
                V[e] = vloc_at(tf, r);
                Vr[e] = reference_potential(r, rc_ref, tf.z);
              }
            }
          }
          const size_t sy = ex[0], sz = (size_t)ex[0] * ex[1];
          for (int k = o; k < ex[2] - o; k++)
            for (int j = o; j < ex[1] - o; j++)
              for (int i = o; i < ex[0] - o; i++) {
                const size_t e = k * sz + j * sy + i;
                double bv = c0 * V[e], br = c0 * Vr[e];
                for (int q = 1; q <= o; q++) {
                  const double cx = g.c[0][q] / (2.0 * M_PI), cy = g.c[1][q] / (2.0 * M_PI),
                               cz = g.c[2][q] / (2.0 * M_PI);
                  bv += cx * (V[e - q] + V[e + q]) + cy * (V[e - q * sy] + V[e + q * sy]) +
                        cz * (V[e - q * sz] + V[e + q * sz]);
                  br += cx * (Vr[e - q] + Vr[e + q]) + cy * (Vr[e - q * sy] + Vr[e + q * sy]) +
                        cz * (Vr[e - q * sz] + Vr[e + q * sz]);
                }
                if (home) {
                  out.e_self += 0.5 * bv * V[e] * g.dV;
                  out.e_self_ref += 0.5 * br * Vr[e] * g.dV;
                }
                const int gx = c[0] - tf.nb[0] + (i - o), gy = c[1] - tf.nb[1] + (j - o),
                          gz = c[2] - tf.nb[2] + (k - o);
                if (!g.inside(gx, gy, gz)) continue;
                const long long gi = g.index(gx, gy, gz);
                out.b[gi] += bv;
                out.b_ref[gi] += br;
                out.vc[gi] += Vr[e] - V[e];
              }
        }
        if (meets_r) {
          for (int gz = std::max(0, c[2] - tf.nr[2]); gz <= std::min(g.N[2] - 1, c[2] + tf.nr[2]); gz++) {
            const double z = coord(2, gz);
            for (int gy = std::max(0, c[1] - tf.nr[1]); gy <= std::min(g.N[1] - 1, c[1] + tf.nr[1]); gy++) {
              const double y = coord(1, gy);
              for (int gx = std::max(0, c[0] - tf.nr[0]); gx <= std::min(g.N[0] - 1, c[0] + tf.nr[0]); gx++) {
                const double x = coord(0, gx);
                const double r = std::sqrt(x * x + y * y + z * z);
                if (r <= tf.rmax_rho) out.rho[g.index(gx, gy, gz)] += tf.rho(r);
              }
            }
          }
        }
      }
}

}  // namespace

ScfFields build_scf_fields(const Deck &d, const Setup &s, int threads) {
  if (d.bc != 2) throw std::invalid_argument("the SCF closure needs a periodic deck (BOUNDARY_CONDITION 2)");
  Grid g;
  for (int a = 0; a < 3; a++) {
    g.N[a] = d.grid[a];
    g.L[a] = 2.0 * d.cell_half[a];
    g.half[a] = d.cell_half[a];
    g.h[a] = s.h[a];
  }
  g.dV = s.dV;
  g.o = d.half_order;
  g.c = s.c;
  const long long ng = (long long)g.N[0] * g.N[1] * g.N[2];

  const int ntype = (int)d.psd.size();
  std::vector<TypeFields> tfs(ntype);
  for (int t = 0; t < ntype; t++) {
    const Psd &p = d.psd[t];
    TypeFields &tf = tfs[t];
    tf.vloc = RadialSpline(p.r, p.vloc);
    std::vector<double> rho_tab = p.rho_atom;
    rho_tab[0] = rho_tab[1];  // the table's r = 0 row is a copy of the first radius
    tf.rho = RadialSpline(p.r, rho_tab);
    tf.z = p.zval;
    tf.rmax_table = p.r.back();
    double peak = 0.0;
    for (size_t i = 1; i < p.r.size(); i++) peak = std::max(peak, std::fabs(rho_tab[i]));
    tf.rmax_rho = 0.0;  // beyond it the valence density is below 1e-10 of its peak
    for (size_t i = 1; i < p.r.size(); i++)
      if (std::fabs(rho_tab[i]) > 1e-10 * peak) tf.rmax_rho = p.r[i];
    tf.rmax_rho = std::min(tf.rmax_rho, 20.0);
    for (int a = 0; a < 3; a++) {
      tf.nb[a] = (int)std::lround(s.pseudocharge_cutoff[3 * t + a] / s.h[a]);
      tf.nr[a] = (int)std::ceil(tf.rmax_rho / s.h[a]) + 1;
    }
  }

  const int natoms = (int)d.atom_type.size();
  int nt = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
  nt = std::max(1, std::min({nt, natoms, 16}));
  std::vector<Partial> parts(nt);
  for (auto &pt : parts) {
    pt.b.assign(ng, 0.0);
    pt.b_ref.assign(ng, 0.0);
    pt.vc.assign(ng, 0.0);
    pt.rho.assign(ng, 0.0);
  }
  auto work = [&](int tid) {
    // static atom ranges: the sums do not depend on scheduling
    const int a0 = (int)((long long)natoms * tid / nt), a1 = (int)((long long)natoms * (tid + 1) / nt);
    for (int n = a0; n < a1; n++) {
      const double X[3] = {d.atom_xyz[3 * n], d.atom_xyz[3 * n + 1], d.atom_xyz[3 * n + 2]};
      add_atom(g, tfs[d.atom_type[n]], d.reference_cutoff, X, parts[tid]);
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; t++) pool.emplace_back(work, t);
  work(0);
  for (auto &th : pool) th.join();

  ScfFields f;
  f.b = std::move(parts[0].b);
  f.b_ref = std::move(parts[0].b_ref);
  f.vc = std::move(parts[0].vc);
  f.rho0 = std::move(parts[0].rho);
  f.e_self = parts[0].e_self;
  f.e_self_ref = parts[0].e_self_ref;
  for (int t = 1; t < nt; t++) {
    for (long long i = 0; i < ng; i++) {
      f.b[i] += parts[t].b[i];
      f.b_ref[i] += parts[t].b_ref[i];
      f.vc[i] += parts[t].vc[i];
      f.rho0[i] += parts[t].rho[i];
    }
    f.e_self += parts[t].e_self;
    f.e_self_ref += parts[t].e_self_ref;
  }
  double btot = 0.0, rtot = 0.0, corr = 0.0;
  for (long long i = 0; i < ng; i++) {
    btot += f.b[i];
    rtot += f.rho0[i];
    corr += (f.b_ref[i] + f.b[i]) * f.vc[i];
  }
  f.b_total = btot * s.dV;
  f.e_corr = 0.5 * corr * s.dV + f.e_self - f.e_self_ref;
  if (!(rtot > 0.0)) throw std::runtime_error("atomic valence densities are empty");
  const double scale = d.n_electrons / (rtot * s.dV);
  for (double &v : f.rho0) v = std::max(v * scale, 0.0);

  // Poisson symbol on the R2C half grid [z][y][x <= Nx/2]
  const int hx = g.N[0] / 2 + 1;
  std::vector<double> sym[3];
  for (int a = 0; a < 3; a++) {
    sym[a].resize(g.N[a]);
    for (int m = 0; m < g.N[a]; m++) {
      double v = s.c[a][0];
      for (int q = 1; q <= g.o; q++) v += 2.0 * s.c[a][q] * std::cos(2.0 * M_PI * m * q / g.N[a]);
      sym[a][m] = v;
    }
  }
  f.green.assign((size_t)g.N[2] * g.N[1] * hx, 0.0);
  for (int kz = 0; kz < g.N[2]; kz++)
    for (int ky = 0; ky < g.N[1]; ky++)
      for (int kx = 0; kx < hx; kx++) {
        if (kx == 0 && ky == 0 && kz == 0) continue;
        f.green[((size_t)kz * g.N[1] + ky) * hx + kx] = 2.0 * M_PI / (sym[0][kx] + sym[1][ky] + sym[2][kz]);
      }
  return f;
}

}  // namespace sq

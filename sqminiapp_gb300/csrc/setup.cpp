// setup.cpp -- host setup of the device data model (FP64).
//
// What the reference builds per rank in Initialize / GetInfluencingAtoms_Nonlocal /
// CalculateNonlocalProjectors (src/lsdft_initObjs.cc:36-93,576-869,1671-1946,
// src/lsdft_nl.cc:141-208) is built here once per engine:
//   * FD weights of -1/2 Laplacian (src/lsdft_readfiles.cc:453-476);
//   * not-a-knot cubic splines of U_l (V_l - V_loc), U_l and V_loc
//     (Wolberg end conditions, src/lsdft_tools.cc:75-151);
//   * Gamma_l = dV / int U_l dV_l U_l r^2 dr, rectangle rule with dr = 1e-6
//     (src/lsdft_initObjs.cc:822-869);
//   * the pseudocharge cutoff, used by the reference for its image range
//     (src/lsdft_initObjs.cc:628-817);
//   * the atom images whose projector box meets the extended domain, with the box
//     centred on roundf((x0 + R)/h) (src/lsdft_initObjs.cc:1763-1812);
//   * radial projector tables.  The reference stores chi_lm = S_l(r) Y_lm for every
//     box point of every image (nl.cc:197-198).  Here chi_lm = T_l(r) P_lm(x,y,z) with
//     T_l = S_l(r)/r^l and P_lm the real solid harmonic (Y_lm r^l, same constants as
//     src/lsdft_tools.cc:165-187), so a table holds one value per l instead of 2l+1, and
//     images that differ by a whole number of grid periods share one table.
#include <algorithm>
#include <cmath>
#include <stdexcept>

#include "radial_spline.hpp"
#include "sq_internal.hpp"

namespace sq {

namespace {

double fd_fraction(int n, int k) {  // (n!)^2 / ((n-k)! (n+k)!)
  double num = 1, den = 1;
  for (int i = n - k + 1; i <= n; i++) num *= i;
  for (int i = n + 1; i <= n + k; i++) den *= i;
  return num / den;
}

int box_center(double x0, double R, double h) {
  // the reference rounds (x0+R)/h through float: roundf((x0 + R_x + 0*Rcut) / delta_x)
  return (int)roundf((float)((x0 + R + 0.0) / h));
}

}  // namespace

Setup build_setup(const Deck &d, bool faithful) {
  Setup s;
  const int o = d.half_order;
  if (o < 1 || o > kStencilHalf) throw std::runtime_error("FD_ORDER must be 2..12");
  for (int a = 0; a < 3; a++) {
    bool periodic_axis = d.bc == 2 || (d.bc == 3 && a < 2) || (d.bc == 4 && a == 0);
    s.h[a] = 2.0 * d.cell_half[a] / (periodic_axis ? d.grid[a] : d.grid[a] - 1);
    s.nh[a] = (int)ceil(d.rcut / s.h[a]);
    s.cube[a] = 2 * s.nh[a] + 1;
  }
  s.dV = s.h[0] * s.h[1] * s.h[2];
  double inv_sq_sum = 0;
  for (int p = 1; p <= o; p++) inv_sq_sum += 1.0 / (p * p);
  for (int a = 0; a < 3; a++) {
    for (int p = 0; p <= kStencilHalf; p++) s.c[a][p] = 0.0;
    s.c[a][0] = inv_sq_sum * (1.0 / (s.h[a] * s.h[a]));
    for (int p = 1; p <= o; p++)
      s.c[a][p] = -1 * pow(-1, p + 1) * fd_fraction(o, p) / (p * p * s.h[a] * s.h[a]);
  }

  const int ntype = (int)d.psd.size();
  s.types.resize(ntype);
  s.pseudocharge_cutoff.assign(3 * ntype, 0.0);
  std::vector<RadialSpline> proj[kMaxTypes][4];
  std::vector<double> rcnl(ntype, 0.0);
  const double hmax = (s.h[0] > s.h[1] && s.h[0] > s.h[2]) ? s.h[0] : (s.h[1] > s.h[2] ? s.h[1] : s.h[2]);

  for (int t = 0; t < ntype; t++) {
    const Psd &p = d.psd[t];
    TypeDesc &td = s.types[t];
    td.chan_mask = 0;
    int nch = 0;
    for (int l = 0; l < 4; l++) {
      td.chan_off[l] = -1;
      td.gamma[l] = 0.0;
    }
    td.support_r2_f64 = 0.0;
    td.support_r2_f32 = 0.0f;
    td.pad_ = 0;
    rcnl[t] = std::max(std::max(p.rc[0], p.rc[1]), std::max(p.rc[2], p.rc[3]));
    int off[3];
    for (int a = 0; a < 3; a++) off[a] = (int)ceil(rcnl[t] / s.h[a]);
    td.fx = 2 * off[0] + 1;
    td.fy = 2 * off[1] + 1;
    td.fz = 2 * off[2] + 1;
    if (p.lmax == 0) continue;  // no nonlocal part (src/lsdft_initObjs.cc:1833)
    for (int l = 0; l <= p.lmax; l++) {
      if (l == p.lloc) continue;
      std::vector<double> udv(p.r.size());
      for (size_t i = 0; i < p.r.size(); i++) udv[i] = p.U[l][i] * (p.V[l][i] - p.vloc[i]);
      proj[t][l].emplace_back(p.r, udv);
      RadialSpline su(p.r, p.U[l]);
      // Gamma_l: the reference's running rectangle sum, step accumulated as rtemp += dr
      const double dr = 1e-6;
      const RadialSpline &sp = proj[t][l][0];
      double rtemp = dr, acc = 0.0, last_udv = 0.0, last_u = 0.0;
      int ka = sp.interval(rtemp), kb = ka;
      const auto &knots = p.r;
      while (rtemp <= p.rc[l] + hmax) {
        while (ka + 2 < (int)knots.size() && knots[ka + 1] <= rtemp) ka++;
        kb = ka;
        last_udv = sp.eval_in(ka, rtemp);
        last_u = su.eval_in(kb, rtemp);
        acc += last_udv * last_u * rtemp * rtemp * dr;
        rtemp = rtemp + dr;
      }
      double D = (acc - 0.5 * last_udv * last_u * (rtemp - dr) * (rtemp - dr) * dr) / s.dV;
      td.gamma[l] = 1.0 / D;
      td.chan_mask |= 1 << l;
      td.chan_off[l] = nch++;
    }

    // Support radius of the projectors.  U_l (V_l - V_loc) vanishes beyond rc on the psd grid,
    // but the cubic spline rings for a few knots past the last nonzero one; scan down from the
    // box corner for the radius where every channel first exceeds the threshold.
    {
      double corner = 0.0;
      for (int a = 0; a < 3; a++) corner += (off[a] + 1) * s.h[a] * (off[a] + 1) * s.h[a];
      corner = sqrt(corner);
      double smax[4] = {0, 0, 0, 0};
      for (int l = 0; l < 4; l++)
        if (td.chan_mask & (1 << l))
          for (double r = 0.0; r <= corner; r += 1e-3) smax[l] = std::max(smax[l], fabs(proj[t][l][0](r)));
      auto radius_for = [&](double thr) {
        for (double r = corner; r > 0.0; r -= 1e-3)
          for (int l = 0; l < 4; l++)
            if ((td.chan_mask & (1 << l)) && fabs(proj[t][l][0](r)) > thr * smax[l])
              return std::min(corner, r + 0.05);
        return 0.05;
      };
      const double r64 = radius_for(1e-16), r32 = radius_for(1e-12);
      td.support_r2_f64 = r64 * r64;
      td.support_r2_f32 = (float)(r32 * r32);
    }

    // pseudocharge cutoff: b = -(1/4pi) Lap V_loc on an octant grid, radius grown by 1 bohr
    // until the integrated charge matches the valence (src/lsdft_initObjs.cc:628-817)
    {
      RadialSpline sv(p.r, p.vloc);
      const double max_radius = 15.0;
      int np[3], ex[3];
      for (int a = 0; a < 3; a++) {
        np[a] = (int)ceil(max_radius / s.h[a]);
        ex[a] = np[a] + 2 * o;
      }
      std::vector<double> vps((size_t)ex[0] * ex[1] * ex[2]);
      auto VP = [&](int k, int j, int i) { return vps[((size_t)k * ex[1] + j) * ex[0] + i]; };
      for (int k = 0; k < ex[2]; k++)
        for (int j = 0; j < ex[1]; j++)
          for (int i = 0; i < ex[0]; i++) {
            double x = (i - o) * s.h[0], y = (j - o) * s.h[1], z = (k - o) * s.h[2];
            vps[((size_t)k * ex[1] + j) * ex[0] + i] = sv(sqrt(x * x + y * y + z * z));
          }
      double sc[3][kStencilHalf + 1];
      for (int a = 0; a < 3; a++)
        for (int q = 0; q <= o; q++) sc[a][q] = s.c[a][q] / (2.0 * M_PI);
      std::vector<double> bj((size_t)np[0] * np[1] * np[2]);
      for (int k = o; k < np[2] + o; k++)
        for (int j = o; j < np[1] + o; j++)
          for (int i = o; i < np[0] + o; i++) {
            double v = VP(k, j, i) * (sc[0][0] + sc[1][0] + sc[2][0]);
            for (int q = 1; q <= o; q++)
              v += (VP(k, j, i - q) + VP(k, j, i + q)) * sc[0][q] +
                   (VP(k, j - q, i) + VP(k, j + q, i)) * sc[1][q] +
                   (VP(k - q, j, i) + VP(k + q, j, i)) * sc[2][q];
            bj[((size_t)(k - o) * np[1] + (j - o)) * np[0] + (i - o)] = v;
          }
      double radius = p.rc[p.lloc], err;
      int nc[3];
      do {
        for (int a = 0; a < 3; a++) nc[a] = (int)ceil(radius / s.h[a]);
        double bint = 0.0;
        for (int k = 0; k < nc[2]; k++)
          for (int j = 0; j < nc[1]; j++)
            for (int i = 0; i < nc[0]; i++) {
              double v = bj[((size_t)k * np[1] + j) * np[0] + i];
              if (k == 0) v *= 0.5;
              if (k == nc[2] - 1) v *= 0.5;
              if (j == 0) v *= 0.5;
              if (j == nc[1] - 1) v *= 0.5;
              if (i == 0) v *= 0.5;
              if (i == nc[0] - 1) v *= 0.5;
              bint += v;
            }
        bint *= 8.0 * s.dV;
        err = fabs(bint + p.zval) / fabs((double)p.zval);
        radius += 1.0;
      } while (radius <= 15.0 && err > 1e-6);
      for (int a = 0; a < 3; a++) s.pseudocharge_cutoff[3 * t + a] = nc[a] * s.h[a];
    }
  }

  // ---- atom images and deduplicated tables ----
  struct Key { int atom; double f[3]; int tab; };
  std::vector<Key> keys;
  const int natoms = (int)d.atom_type.size();
  for (int n = 0; n < natoms; n++) {
    const int t = d.atom_type[n];
    const TypeDesc &td = s.types[t];
    if (td.chan_mask == 0) continue;
    const Psd &p = d.psd[t];
    int off[3] = {(td.fx - 1) / 2, (td.fy - 1) / 2, (td.fz - 1) / 2};
    int fdim[3] = {td.fx, td.fy, td.fz};
    bool per[3];
    for (int a = 0; a < 3; a++) {
      bool axis_bc = (a == 0 && (d.bc == 1 || d.bc == 3 || d.bc == 4)) ||
                     (a == 1 && (d.bc == 1 || d.bc == 3)) || (a == 2 && d.bc == 1);
      per[a] = faithful ? axis_bc : (axis_bc || d.bc == 2);
    }
    int imax[3];
    for (int a = 0; a < 3; a++) {
      if (!per[a]) { imax[a] = 0; continue; }
      if (faithful) {
        imax[a] = (int)ceil(s.pseudocharge_cutoff[3 * t + a] / d.cell_half[a]);
      } else {
        double reach = (s.nh[a] + off[a] + 1) * s.h[a];
        imax[a] = (int)ceil(reach / (2.0 * d.cell_half[a])) + 1;
      }
    }
    (void)p;
    for (int P = -imax[0]; P <= imax[0]; P++)
      for (int Q = -imax[1]; Q <= imax[1]; Q++)
        for (int R = -imax[2]; R <= imax[2]; R++) {
          double x0[3] = {d.atom_xyz[3 * n] + P * 2.0 * d.cell_half[0],
                          d.atom_xyz[3 * n + 1] + Q * 2.0 * d.cell_half[1],
                          d.atom_xyz[3 * n + 2] + R * 2.0 * d.cell_half[2]};
          int lo[3];
          bool meets = true;
          double frac[3];
          for (int a = 0; a < 3; a++) {
            int c = box_center(x0[a], d.cell_half[a], s.h[a]);
            lo[a] = c - off[a];
            frac[a] = (x0[a] + d.cell_half[a]) / s.h[a] - c;
            // extended domain [-nh, N-1+nh] (src/lsdft_initObjs.cc:1699-1707, one rank)
            if (lo[a] + fdim[a] - 1 < -s.nh[a] || lo[a] > d.grid[a] - 1 + s.nh[a]) meets = false;
          }
          if (!meets) continue;
          int tab = -1;
          for (const Key &k : keys)
            if (k.atom == n && fabs(k.f[0] - frac[0]) < 1e-9 && fabs(k.f[1] - frac[1]) < 1e-9 &&
                fabs(k.f[2] - frac[2]) < 1e-9) {
              tab = k.tab;
              break;
            }
          long long base;
          if (tab < 0) {
            tab = s.n_tables++;
            keys.push_back({n, {frac[0], frac[1], frac[2]}, tab});
            base = (long long)s.tables.size();
            const int npt = td.fx * td.fy * td.fz;
            s.tables.resize(s.tables.size() + (size_t)__builtin_popcount(td.chan_mask) * npt);
            for (int l = 0; l < 4; l++) {
              if (!(td.chan_mask & (1 << l))) continue;
              const RadialSpline &sp = proj[t][l][0];
              double *dst = &s.tables[base + (size_t)td.chan_off[l] * npt];
              for (int k = 0; k < td.fz; k++) {
                double z = s.h[2] * (lo[2] + k) - d.cell_half[2] - x0[2];
                for (int j = 0; j < td.fy; j++) {
                  double y = s.h[1] * (lo[1] + j) - d.cell_half[1] - x0[1];
                  for (int i = 0; i < td.fx; i++) {
                    double x = s.h[0] * (lo[0] + i) - d.cell_half[0] - x0[0];
                    double r = sqrt(x * x + y * y + z * z);
                    double S = sp(r), T;
                    if (l == 0) T = S * 0.282094791773878;
                    else T = r >= 1e-10 ? S / pow(r, l) : 0.0;
                    dst[((size_t)k * td.fy + j) * td.fx + i] = T;
                  }
                }
              }
            }
          } else {
            base = -1;
            for (const ImageMeta &im : s.images)
              if (im.tab == tab) { base = im.tab_base; break; }
          }
          ImageMeta im{};
          im.bx = lo[0];
          im.by = lo[1];
          im.bz = lo[2];
          im.type = t;
          im.atom = n;
          im.tab = tab;
          im.tab_base = base;
          im.ox = s.h[0] * lo[0] - d.cell_half[0] - x0[0];
          im.oy = s.h[1] * lo[1] - d.cell_half[1] - x0[1];
          im.oz = s.h[2] * lo[2] - d.cell_half[2] - x0[2];
          s.images.push_back(im);
        }
  }
  // images are generated atom by atom, so equal atoms are adjacent (one alpha slot each)
  return s;
}

}  // namespace sq

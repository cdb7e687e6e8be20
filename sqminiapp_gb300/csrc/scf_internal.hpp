// scf_internal.hpp -- host-side fixed fields of the SCF closure and the device SCF state.
#pragma once

#include <vector>

#include "sq_internal.hpp"

namespace sq {

// Fields that depend on the atoms only (FP64, periodic grid, x fastest).
struct ScfFields {
  std::vector<double> b;      // pseudocharge density sum_J b_J (negative, integral ~ -N_e)
  std::vector<double> b_ref;  // reference pseudocharges of the smooth reference potential
  std::vector<double> vc;     // sum_J (V_ref,J - V_loc,J): electrostatic correction potential
  std::vector<double> rho0;   // atomic-superposition density, integral = N_e
  std::vector<double> green;  // 2 pi / s(k) on the R2C half grid [z][y][x <= Nx/2]; 0 at k = 0
  double e_self = 0.0;        // 1/2 sum_J int b_J V_J  (one image per atom)
  double e_self_ref = 0.0;    // same for the reference pseudocharges
  double e_corr = 0.0;        // 1/2 int (b_ref + b) vc + e_self - e_self_ref
  double b_total = 0.0;       // int b (should be close to -N_e)
};

// Builds every field; `threads` host threads (0 = hardware concurrency).
ScfFields build_scf_fields(const Deck &d, const Setup &s, int threads = 0);

// Reference potential of the electrostatic correction: -Z/r beyond rc, inside it the C2
// polynomial -Z/rc (9R^7 - 30R^6 + 28R^5 - 14R^2 + 12)/5, R = r/rc (Ghosh and Suryanarayana,
// Comput. Phys. Commun. 212 (2017), the SPARC reference pseudopotential).
double reference_potential(double r, double rc, double z);

}  // namespace sq

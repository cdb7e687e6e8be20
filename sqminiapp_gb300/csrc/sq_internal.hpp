// sq_internal.hpp -- data model shared by the host setup and the CUDA kernels.
//
// The reference keeps all state in one LSDFT_OBJ with jagged per-atom arrays
// (src/ilsdft.h:85-458, projector lists :20-57).  Here the state is a handful
// of flat device buffers:
//   * ImageMeta[n_images]  one record per (atom, periodic image) whose projector
//                          box meets the extended domain, sorted by atom;
//   * tables               radial projector tables T_l = S_l(r)/r^l over each box,
//                          stored once per distinct fractional atom offset;
//   * veff_ext             the effective potential padded periodically by the
//                          cube half-width so a cube window is a plain 3D slice.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

struct sq_system_desc;  // sq_gb300.h

namespace sq {

constexpr int kMaxTypes = 8;
constexpr int kMaxLm = 16;        // (l, m) slots for l <= 3, indexed l*l + l + m
constexpr int kStencilHalf = 6;   // FD_ORDER 12 (src/lsdft_readfiles.cc:150-152)

// One projector-carrying atom image.  Box = [box_lo, box_lo + box_n) in unwrapped
// global grid indices; off = coordinates (bohr) of box point (0,0,0) relative to the
// image's atom, so point (i,j,k) of the box sits at off + (hx*i, hy*j, hz*k).
struct ImageMeta {
  int bx, by, bz, type;
  int atom, tab;
  long long tab_base;     // element offset of channel 0 of this image's table
  double ox, oy, oz, pad;
};
static_assert(sizeof(ImageMeta) == 64, "ImageMeta layout");

// Per-type projector description for the kernels.
struct TypeDesc {
  int fx, fy, fz;          // box points per axis (2*ceil(rc/h)+1)
  int chan_mask;           // bit l set if channel l is nonlocal
  int chan_off[4];         // table channel index of l (only if in mask)
  double gamma[4];         // Gamma_l (src/lsdft_initObjs.cc:822-869)
  // Squared projector support radius (bohr^2): beyond it every |S_l(r)| is below 1e-16 (FP64
  // engine) or 1e-12 (FP32 engine) of its maximum, i.e. below the arithmetic's own rounding.
  double support_r2_f64;
  float support_r2_f32;
  int pad_;
};

// Everything the Lanczos kernel reads besides the buffers.
struct LanczosParams {
  int nx, ny, nz;          // cube points per axis
  int nhx, nhy, nhz;       // cube half-widths
  int Nx, Ny, Nz;          // grid nodes per axis
  int EX, EY, EZ;          // padded Veff dims (N + 2*nh)
  int pitch;               // smem row pitch of the stencil vector: nx + kStencilHalf (even
                           // in FP32), or nx with kLayoutXClamp
  int layout;              // kLayout* flags
  int upitch;              // row pitch of the elementwise vector U (nx, or nx + 1)
  int nqp;                 // Lanczos steps kept for the quadrature
  int n_images;
  int max_img;             // per-node image-list capacity
  int alpha_stride;        // coefficients per image slot (number of (l,m) of the mask union)
  int union_mask;          // bit l set if any type has a nonlocal channel l
  int lm_rank[kMaxLm];     // compact slot of (l,m) in alpha_stride, -1 if absent
  int rank_l[kMaxLm];      // l of compact slot r
  int ntype;
  int rows_per_warp;       // cube y-rows owned by one warp in the vector passes
  int zchunks;             // kLayoutQuad: z-ranges (pass A) and y-ranges (pass B) per row / plane
  int ychunks;             // kLayoutPair: y-ranges per plane of pass B (zchunks: z-ranges)
  int zsplit;              // kLayoutPair: CTA 0 of a pair owns planes [0, zsplit), CTA 1 the rest
  int vring;               // kLayoutQuad: 1 = pass A stages Veff through a per-thread shared ring
  int vq_row;              // kLayoutQuad: row length (floats) of the quad-aligned Veff copies
  long long vq_copy_stride;  // kLayoutQuad: floats per quad-aligned Veff copy
  int proj_cap;            // records of one CTA's projector list (max box points of a node)
  long long proj_bytes_per_cta;
  long long node_begin, node_end;
  double hx, hy, hz;
  float hxf, hyf, hzf;
  double cdiag;            // coeffs_x[0] + coeffs_y[0] + coeffs_z[0]
  double cx[kStencilHalf + 1], cy[kStencilHalf + 1], cz[kStencilHalf + 1];
  float cdiagf;            // FP32 copies for the FP32 engine
  float cxf[kStencilHalf + 1], cyf[kStencilHalf + 1], czf[kStencilHalf + 1];
  TypeDesc types[kMaxTypes];
};

struct Psd {
  std::string name;
  int lmax = -1, lloc = 0, zval = 0;
  std::vector<double> r, vloc, rho_atom;
  std::vector<double> V[4], U[4];
  double rc[4] = {0, 0, 0, 0};
  bool has_u[4] = {false, false, false, false};
};

// Parsed input deck (.inpt / .ion / .relax / psd), src/lsdft_readfiles.cc:21-1101.
struct Deck {
  int half_order = 6;
  int bc = 1;
  double cell_half[3] = {0, 0, 0};
  int grid[3] = {0, 0, 0};
  double beta = 1000.0;
  double rcut = 12.0;
  int n_qp = 50;
  double mixing_parameter = 0.3;
  int mixing_history = 7;
  int pulay_frequency = 1;
  double tol_scf = 1e-6;
  int maxit_scf = 100;
  double reference_cutoff = 0.5;  // src/lsdft_readfiles.cc:80
  std::string xc = "LDA";
  std::vector<int> lloc;
  std::vector<std::string> psd_file;
  std::vector<std::string> type_name;
  std::vector<int> type_valence;
  std::vector<int> atom_type;
  std::vector<double> atom_xyz;
  std::vector<Psd> psd;
  int n_electrons = 0;
};

Deck read_deck(const std::string &dir, const std::string &name);
// The same Deck from values in memory (sq_system_desc of sq_gb300.h), checked as the readers
// check the files.
Deck deck_from_system(const ::sq_system_desc &sys);

// Host setup result: everything copied to the device.
struct Setup {
  double h[3];
  int nh[3], cube[3];
  double dV;
  double c[3][kStencilHalf + 1];
  std::vector<ImageMeta> images;
  std::vector<double> tables;   // FP64 values; converted to the engine precision on upload
  int n_tables = 0;
  std::vector<TypeDesc> types;
  std::vector<double> pseudocharge_cutoff;  // [ntype][3]
};

Setup build_setup(const Deck &d, bool faithful);

}  // namespace sq

// sq_kernels.hpp -- host-side launch wrappers of the CUDA kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

#include "sq_internal.hpp"

namespace sq {

constexpr int kMaxWarpsF32 = 16;  // one CTA per SM, 16 warps: 128 registers/thread
constexpr int kMaxWarpsF64 = 16;  // FP64 register window needs up to 128 registers/thread
// cubes wider than 32 points (FP32 only): one thread per (row, x pair), up to 18 warps, so a
// 33^3 cube's 33 x 17 pairs run in one round (96 registers/thread: 5 warps share a quarter SM)
constexpr int kWideWarpsF32 = 18;

// Layout of the Lanczos vectors on chip (LanczosParams::layout, bit flags):
constexpr int kLayoutYGap = 1;    // FP32: 6 zero rows between z-planes (else y bounds-checked)
constexpr int kLayoutWide = 2;    // FP32 cubes wider than 32 points: one thread per row pair
constexpr int kLayoutXClamp = 4;  // FP64: rows without zero columns, x bounds-checked
// FP32, corrected operator: the projector list holds T_l(r) per channel and the point's box
// coordinates (12 B for s+p) instead of chi_lm and packed P|U indices (20 B); chi_lm is
// rebuilt from the solid harmonics while streaming.  For lists that would not stay in L2.
constexpr int kLayoutCompact = 8;
// FP32, corrected operator, cubes at most 32 points wide, P and U on chip: split stencil passes
// over 16-byte quads (lanczos_quad.cuh); rows of 4*ceil(nx/4) floats, no gaps.
constexpr int kLayoutQuad = 16;
constexpr int kQuadMaxThreads = 512;
// With kLayoutQuad, cubes whose P and U do not fit one CTA: a cluster of two CTAs per node,
// the cube split in z, 6 halo planes of P written by the peer through distributed shared
// memory (lanczos_quad.cuh, PairPlanes).
constexpr int kLayoutPair = 32;
constexpr int kPairThreads = 384;
// Pass A of the split-pass kernel (12-warp budget) stages Veff through a per-thread ring of
// kVRingSlots float4 in shared memory, filled by async copies kVRingSlots - 1 planes ahead.
constexpr int kVRingSlots = 4;
constexpr int kVRingThreads = 384;

// device status bits (ORed by the kernels)
constexpr int kStatusCapacity = 1;
constexpr int kStatusBreakdown = 2;
constexpr int kStatusNoConvergence = 4;
constexpr int kStatusTimeout = 8;

// channel mask the kernel is instantiated for (union mask, or 15 = generic) and its (l,m) count
int kernel_mask(int union_mask);
int mask_nlm(int mask);

size_t lanczos_smem_bytes(const LanczosParams &p, int elem_size, bool u_smem, bool faithful);

// bytes of one record of the per-node projector list (values + packed P|U index, or with
// kLayoutCompact the channel values + packed box coordinates)
size_t proj_record_bytes(int elem_size, bool faithful, int union_mask, bool compact = false);

cudaError_t launch_lanczos(const LanczosParams &p, int precision, bool faithful, bool u_smem,
                           int grid, int block, size_t smem, cudaStream_t s, const void *veff_ext,
                           const ImageMeta *images, const void *tables, void *u_scratch,
                           void *proj_scratch, double *ab, int *status);

cudaError_t launch_veff_extend(const double *veff, double vconst, void *ext, int precision,
                               const LanczosParams &p, cudaStream_t s);

// kLayoutQuad: the four quad-aligned copies of cdiag + Veff padded periodically by the cube
// half-width (copy s holds extended x index ex at row position ex + s; rows of vq_row floats).
size_t veff_quad_floats(const LanczosParams &p);
size_t lanczos_quad_smem_bytes(const LanczosParams &p);
int lanczos_quad_threads(const LanczosParams &p);
// threads to launch a single-CTA split-pass kernel with (>= lanczos_quad_threads)
int lanczos_quad_block(const LanczosParams &p);
// kLayoutPair: clusters of two CTAs that fit on the device at once (0 if none)
int lanczos_quad_pair_clusters(const LanczosParams &p, int block, size_t smem);

// Implicit QL of every node's tridiagonal; ab = [n][2][nqp] (a then b).
cudaError_t launch_quadrature(const double *ab, long long n, int nqp, double *lambda, double *w,
                              double *lmin, double *lmax, int *status, cudaStream_t s);

// Fermi level (bisection), densities, band energy and -TS.  out[0..3] = lambda_f, e_band, ts,
// iterations.  scratch: see fermi_scratch_doubles.
size_t fermi_scratch_doubles(int grid, int maxit);
cudaError_t launch_fermi(const double *lambda, const double *w, long long n_nodes, int nqp,
                         double beta, double n_electrons, double dV, double tol, int maxit,
                         double *rho, double *out, double *scratch, unsigned *barrier,
                         int *status, int grid, cudaStream_t s);

// The Fermi kernel with one CTA leaving before the first grid barrier and a short poll limit:
// the bounded wait of every other CTA runs out (kStatusTimeout); see fermi.cu.
cudaError_t launch_fermi_timeout_selftest(const double *lambda, const double *w, long long n_nodes,
                                          int nqp, double *out, double *scratch,
                                          unsigned *barrier, int *status, int grid,
                                          cudaStream_t s);

// Node densities rho = (2/dV) sum_q w f (rho may be NULL) and out[0..1] = band energy
// 2 sum w lambda f and 2 sum w [f ln f + (1-f) ln(1-f)] at a given Fermi level;
// `partial` holds 2 * grid doubles.
cudaError_t launch_density_energy(const double *lambda, const double *w, long long n_nodes, int nqp,
                                  double beta, double lf, double dV, double *rho, double *partial,
                                  int grid, double *out, cudaStream_t s);

// N_e(lf) = 2 sum w f(lambda - lf) over n_nodes*nqp entries; `partial` holds `grid` doubles.
cudaError_t launch_electron_count(const double *lambda, const double *w, long long n_nodes,
                                  int nqp, double beta, double lf, double *partial, int grid,
                                  double *out, cudaStream_t s);

// FP32 FMA throughput of `device` in TFLOP/s (register-resident FMA chains on every SM).
cudaError_t measure_fp32_peak(int device, double *tflops);

}  // namespace sq

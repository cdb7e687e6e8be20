// sq_kernels.hpp -- host-side launch wrappers of the CUDA kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

#include "sq_internal.hpp"

namespace sq {

constexpr int kBlockF32 = 1024;  // one CTA per SM, 32 warps
constexpr int kBlockF64 = 512;   // FP64 register window needs more registers per thread

// device status bits (ORed by the kernels)
constexpr int kStatusCapacity = 1;
constexpr int kStatusBreakdown = 2;
constexpr int kStatusNoConvergence = 4;
constexpr int kStatusTimeout = 8;

size_t lanczos_smem_bytes(const LanczosParams &p, int elem_size, bool u_smem, int block);

cudaError_t launch_lanczos(const LanczosParams &p, int precision, bool faithful, bool u_smem,
                           int grid, size_t smem, cudaStream_t s, const void *veff_ext,
                           const ImageMeta *images, const void *tables, void *u_scratch,
                           double *ab, int *status);

cudaError_t launch_veff_extend(const double *veff, double vconst, void *ext, int precision,
                               const LanczosParams &p, cudaStream_t s);

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

}  // namespace sq

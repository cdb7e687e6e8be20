// quadrature.cu -- Gauss quadrature nodes and weights from the Lanczos tridiagonals.
//
// Replaces TridiagEigenVecSolve_NodesAndWeights (src/lsdft_tools.cc:912-1026): implicit QL
// with Wilkinson-type shifts (Numerical Recipes tqli), lambda_q = d[q], w_q = Z[0][q]^2,
// eigenvalues left unsorted, lambda_min / lambda_max by the reference's scan.  The rows of Z
// never mix in tqli, so only row 0 is carried: O(n) storage and O(n^2) work per node with
// results identical to the full-matrix form.
//
// One thread per node, FP64.  This file is compiled with -fmad=false so every operation is
// a separately rounded IEEE multiply or add, the same arithmetic as the CPU reference.
#include <cuda_runtime.h>

#include "sq_kernels.hpp"

namespace sq {

namespace {

constexpr int kMaxQp = 64;

__global__ void quadrature_kernel(const double *__restrict__ ab, long long n, int nqp,
                                  double *__restrict__ lambda, double *__restrict__ wts,
                                  double *__restrict__ lmin, double *__restrict__ lmax,
                                  int *__restrict__ status) {
  for (long long node = blockIdx.x * (long long)blockDim.x + threadIdx.x; node < n;
       node += (long long)gridDim.x * blockDim.x) {
    double d[kMaxQp], e[kMaxQp], z[kMaxQp];
    const double *a = ab + node * 2 * nqp;
    const double *b = a + nqp;
    for (int i = 0; i < nqp; i++) {
      d[i] = a[i];
      e[i] = b[i];
      z[i] = i == 0 ? 1.0 : 0.0;
    }
    e[nqp - 1] = 0.0;
    bool failed = false;
    for (int l = 0; l <= nqp - 1 && !failed; l++) {
      int iter = 0, m;
      do {
        for (m = l; m <= nqp - 2; m++) {
          const double dd = fabs(d[m]) + fabs(d[m + 1]);
          if (fabs(e[m]) + dd == dd) break;
        }
        if (m != l) {
          if (iter++ == 50) {
            failed = true;
            break;
          }
          double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
          double r = sqrt(g * g + 1.0);
          g = d[m] - d[l] + e[l] / (g + (g >= 0.0 ? fabs(r) : -fabs(r)));
          double s = 1.0, c = 1.0, p = 0.0;
          int i;
          for (i = m - 1; i >= l; i--) {
            double f = s * e[i];
            const double bb = c * e[i];
            e[i + 1] = (r = sqrt(g * g + f * f));
            if (r == 0.0) {
              d[i + 1] -= p;
              e[m] = 0.0;
              break;
            }
            s = f / r;
            c = g / r;
            g = d[i + 1] - p;
            r = (d[i] - g) * s + 2.0 * c * bb;
            d[i + 1] = g + (p = s * r);
            g = c * r - bb;
            f = z[i + 1];
            z[i + 1] = s * z[i] + c * f;
            z[i] = c * z[i] - s * f;
          }
          if (r == 0.0 && i >= l) continue;
          d[l] -= p;
          e[l] = g;
          e[m] = 0.0;
        }
      } while (m != l);
    }
    if (failed) atomicOr(status, kStatusNoConvergence);
    double emin = d[0], emax = d[0];
    double *lo = lambda + node * nqp, *wo = wts + node * nqp;
    for (int i = 0; i < nqp; i++) {
      lo[i] = d[i];
      wo[i] = z[i] * z[i];
      if (d[i] > emax) emax = d[i];
      else if (d[i] < emin) emin = d[i];
    }
    lmin[node] = emin;
    lmax[node] = emax;
  }
}

}  // namespace

cudaError_t launch_quadrature(const double *ab, long long n, int nqp, double *lambda, double *w,
                              double *lmin, double *lmax, int *status, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int block = 128;
  const long long blocks = (n + block - 1) / block;
  const int grid = (int)(blocks < 152LL * 32 ? blocks : 152LL * 32);
  quadrature_kernel<<<grid, block, 0, s>>>(ab, n, nqp, lambda, w, lmin, lmax, status);
  return cudaGetLastError();
}

}  // namespace sq

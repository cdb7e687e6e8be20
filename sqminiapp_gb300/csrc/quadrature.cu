// quadrature.cu -- Gauss quadrature nodes and weights from the Lanczos tridiagonals.
//
// Replaces TridiagEigenVecSolve_NodesAndWeights (src/lsdft_tools.cc:912-1026): implicit QL
// with Wilkinson-type shifts (Numerical Recipes tqli), lambda_q = d[q], w_q = Z[0][q]^2,
// eigenvalues left unsorted, lambda_min / lambda_max by the reference's scan.  The rows of Z
// never mix in tqli, so only row 0 is carried: O(n) storage and O(n^2) work per node with
// results identical to the full-matrix form.
//
// One thread per node, FP64.  This file is compiled with -fmad=false so every operation is
// a separately rounded IEEE multiply or add, the same arithmetic as the CPU reference.  The
// three working arrays of a node (d, e and row 0 of Z, N_qp doubles each) live in shared
// memory, one column per thread (element i of thread t at i * blockDim + t): as local arrays
// the ~250 nodes per SM (1.5 KB each) overflow L1 and every rotation waits on L2.
#include <cuda_runtime.h>

#include "sq_kernels.hpp"

namespace sq {

namespace {

constexpr int kQuadBlock = 64;

// one thread's column of a shared array: element i at p[i * stride]
struct Col {
  double *p;
  int stride;
  __device__ __forceinline__ double &operator[](int i) const { return p[i * stride]; }
};

__global__ void __launch_bounds__(kQuadBlock)
    quadrature_kernel(const double *__restrict__ ab, long long n, int nqp,
                      double *__restrict__ lambda, double *__restrict__ wts,
                      double *__restrict__ lmin, double *__restrict__ lmax,
                      int *__restrict__ status) {
  extern __shared__ double qsm[];  // [3][nqp][blockDim]
  const Col d{qsm + threadIdx.x, (int)blockDim.x};
  const Col e{qsm + nqp * blockDim.x + threadIdx.x, (int)blockDim.x};
  const Col z{qsm + 2 * nqp * blockDim.x + threadIdx.x, (int)blockDim.x};
  for (long long node = blockIdx.x * (long long)blockDim.x + threadIdx.x; node < n;
       node += (long long)gridDim.x * blockDim.x) {
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
  if (nqp < 1 || nqp > 64) return cudaErrorInvalidValue;
  const int block = kQuadBlock;
  const size_t smem = sizeof(double) * 3 * (size_t)nqp * block;
  cudaError_t e = cudaFuncSetAttribute(quadrature_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const long long blocks = (n + block - 1) / block;
  const int grid = (int)(blocks < 152LL * 64 ? blocks : 152LL * 64);
  quadrature_kernel<<<grid, block, smem, s>>>(ab, n, nqp, lambda, w, lmin, lmax, status);
  return cudaGetLastError();
}

}  // namespace sq

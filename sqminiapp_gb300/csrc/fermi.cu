// fermi.cu -- Fermi level, node densities and band energy from the quadrature (FP64).
//
// The reference declares this closure but never defines it (src/lsdft.h:98-102
// constraint_lssgq / FermiDirac / CalculateDensity_lssgq / findRootBrent, :209
// SystemEnergy_Calc_lssgq).  With the Gauss rule of node i (lambda_iq, w_iq):
//   N_e(lf) = 2 sum_i sum_q w_iq f(lambda_iq - lf),  f(x) = 1 / (1 + exp(beta x))
// lf is found by bisection on [min lambda - 1, max lambda + 1]; then
//   rho_i = (2/dV) sum_q w_iq f,  E_band = 2 sum w lambda f,
//   -TS = (2/beta) sum w [f ln f + (1-f) ln(1-f)].
//
// One cooperative persistent launch runs every bisection step: each CTA reduces its slice
// into one partial per step, a bounded grid barrier publishes the partials, and every CTA
// sums them in the same fixed order, so all CTAs take the same branch and the result does
// not depend on scheduling.  The barrier spins a bounded number of times and then reports
// kStatusTimeout instead of waiting forever.
#include <cuda_runtime.h>

#include "sq_kernels.hpp"

namespace sq {

namespace {

constexpr int kFermiBlock = 512;
constexpr long long kSpinLimit = 1LL << 22;

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ double block_sum_d(double v, double *red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_sum_d(v);
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (warp == 0) {
    t = lane < kFermiBlock / 32 ? red[lane] : 0.0;
    t = warp_sum_d(t);
  }
  __syncthreads();
  return t;  // valid in thread 0
}

// All CTAs meet here.  Returns false (in every thread of the CTA) if the wait gave up.
__device__ bool grid_barrier(unsigned *bar, int *status, int *flag_smem) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned *gen_p = bar + 1;
    const unsigned gen = *gen_p;
    __threadfence();
    const unsigned arrived = atomicAdd(bar, 1u);
    int ok = 1;
    if (arrived == gridDim.x - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      long long spins = 0;
      while (*gen_p == gen) {
        if (++spins > kSpinLimit) {
          atomicOr(status, kStatusTimeout);
          ok = 0;
          break;
        }
        __nanosleep(100);
      }
    }
    __threadfence();
    *flag_smem = ok;
  }
  __syncthreads();
  return *flag_smem != 0;
}

__device__ __forceinline__ double fermi_dirac(double beta, double lam, double lf) {
  return 1.0 / (1.0 + exp(beta * (lam - lf)));
}

__global__ void __launch_bounds__(kFermiBlock)
    fermi_kernel(const double *__restrict__ lambda, const double *__restrict__ w,
                 long long n_nodes, int nqp, double beta, double n_electrons, double dV,
                 double tol, int maxit, double *__restrict__ rho, double *__restrict__ out,
                 double *__restrict__ scratch, unsigned *__restrict__ bar,
                 int *__restrict__ status) {
  __shared__ double red[kFermiBlock / 32];
  __shared__ double bcast[2];
  __shared__ int flag;
  const int G = gridDim.x;
  const long long n = n_nodes * nqp;
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long stride = (long long)G * blockDim.x;

  // phase 0: bracket
  double lo = 1e300, hi = -1e300;
  for (long long e = tid; e < n; e += stride) {
    lo = fmin(lo, lambda[e]);
    hi = fmax(hi, lambda[e]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = lo;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = red[0];
    for (int i = 1; i < kFermiBlock / 32; i++) m = fmin(m, red[i]);
    scratch[blockIdx.x] = m;
  }
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = hi;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = red[0];
    for (int i = 1; i < kFermiBlock / 32; i++) m = fmax(m, red[i]);
    scratch[G + blockIdx.x] = m;
  }
  if (!grid_barrier(bar, status, &flag)) return;
  if (threadIdx.x == 0) {
    double a = scratch[0], b = scratch[G];
    for (int i = 1; i < G; i++) {
      a = fmin(a, scratch[i]);
      b = fmax(b, scratch[G + i]);
    }
    bcast[0] = a - 1.0;
    bcast[1] = b + 1.0;
  }
  __syncthreads();
  lo = bcast[0];
  hi = bcast[1];

  // phase 1: bisection on the electron count
  int it;
  for (it = 0; it < maxit; it++) {
    const double mid = 0.5 * (lo + hi);
    double c = 0.0;
    for (long long e = tid; e < n; e += stride) c += 2.0 * w[e] * fermi_dirac(beta, lambda[e], mid);
    c = block_sum_d(c, red);
    if (threadIdx.x == 0) scratch[(2 + it) * (long long)G + blockIdx.x] = c;
    if (!grid_barrier(bar, status, &flag)) return;
    if (threadIdx.x == 0) {
      double ne = 0.0;
      for (int i = 0; i < G; i++) ne += scratch[(2 + it) * (long long)G + i];
      bcast[0] = ne;
    }
    __syncthreads();
    const double ne = bcast[0];
    __syncthreads();
    if (ne > n_electrons) hi = mid;
    else lo = mid;
    if (hi - lo < tol) break;
  }
  const double lf = 0.5 * (lo + hi);

  // phase 2: densities, band energy, entropy term
  double eb = 0.0, ent = 0.0;
  for (long long node = tid; node < n_nodes; node += stride) {
    double r = 0.0;
    for (int q = 0; q < nqp; q++) {
      const long long e = node * nqp + q;
      const double f = fermi_dirac(beta, lambda[e], lf);
      r += w[e] * f;
      eb += 2.0 * w[e] * lambda[e] * f;
      double s = 0.0;
      if (f > 0.0 && f < 1.0) s = f * log(f) + (1.0 - f) * log(1.0 - f);
      ent += 2.0 * w[e] * s;
    }
    if (rho) rho[node] = 2.0 * r / dV;
  }
  eb = block_sum_d(eb, red);
  ent = block_sum_d(ent, red);
  const long long rowE = (2 + (long long)maxit) * G, rowS = rowE + G;
  if (threadIdx.x == 0) {
    scratch[rowE + blockIdx.x] = eb;
    scratch[rowS + blockIdx.x] = ent;
  }
  if (!grid_barrier(bar, status, &flag)) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    double E = 0.0, S = 0.0;
    for (int i = 0; i < G; i++) {
      E += scratch[rowE + i];
      S += scratch[rowS + i];
    }
    out[0] = lf;
    out[1] = E;
    out[2] = S / beta;
    out[3] = (double)it;
  }
}

}  // namespace

size_t fermi_scratch_doubles(int grid, int maxit) { return (size_t)grid * (maxit + 4); }

cudaError_t launch_fermi(const double *lambda, const double *w, long long n_nodes, int nqp,
                         double beta, double n_electrons, double dV, double tol, int maxit,
                         double *rho, double *out, double *scratch, unsigned *barrier,
                         int *status, int grid, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(barrier, 0, 2 * sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  void *args[] = {(void *)&lambda, (void *)&w,   (void *)&n_nodes, (void *)&nqp,
                  (void *)&beta,   (void *)&n_electrons, (void *)&dV, (void *)&tol,
                  (void *)&maxit,  (void *)&rho, (void *)&out,     (void *)&scratch,
                  (void *)&barrier, (void *)&status};
  return cudaLaunchCooperativeKernel((const void *)fermi_kernel, dim3(grid), dim3(kFermiBlock),
                                     args, 0, s);
}

}  // namespace sq

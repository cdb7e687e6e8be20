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

#include <algorithm>
#include <string>

#include "sq_gb300.h"
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

// All CTAs meet here.  Returns false (in every thread of the CTA) if the wait gave up after
// spin_limit polls.
__device__ bool grid_barrier(unsigned *bar, int *status, int *flag_smem, long long spin_limit) {
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
        if (++spins > spin_limit) {
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
                 int *__restrict__ status, long long spin_limit, int skip_block) {
  __shared__ double red[kFermiBlock / 32];
  // fault injection of the timeout self-test: one CTA leaves before its first arrival, so
  // every other CTA's first barrier wait runs out
  if ((int)blockIdx.x == skip_block) return;
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
  if (!grid_barrier(bar, status, &flag, spin_limit)) return;
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
    if (!grid_barrier(bar, status, &flag, spin_limit)) return;
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
  if (!grid_barrier(bar, status, &flag, spin_limit)) return;
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

constexpr int kCountBlock = 256;

// Partial electron counts: one per CTA, in a fixed grid-stride order.
__global__ void __launch_bounds__(kCountBlock)
    count_partials_kernel(const double *__restrict__ lambda, const double *__restrict__ w,
                          long long n, double beta, double lf, double *__restrict__ partial) {
  __shared__ double red[kCountBlock / 32];
  double c = 0.0;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x)
    c += 2.0 * w[e] * fermi_dirac(beta, lambda[e], lf);
  c = warp_sum_d(c);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < kCountBlock / 32; i++) t += red[i];
    partial[blockIdx.x] = t;
  }
}

__global__ void sum_partials_kernel(const double *__restrict__ partial, int n,
                                    double *__restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < n; i++) t += partial[i];
    *out = t;
  }
}

// Node densities, band energy and entropy term of a given Fermi level (the last phase of
// fermi_kernel on its own): part[2 * block] = (2 sum w lambda f, 2 sum w s(f)) per CTA.
__global__ void __launch_bounds__(kCountBlock)
    density_energy_kernel(const double *__restrict__ lambda, const double *__restrict__ w,
                          long long n_nodes, int nqp, double beta, double lf, double dV,
                          double *__restrict__ rho, double *__restrict__ part) {
  __shared__ double red[2][kCountBlock / 32];
  double eb = 0.0, ent = 0.0;
  for (long long node = blockIdx.x * (long long)blockDim.x + threadIdx.x; node < n_nodes;
       node += (long long)gridDim.x * blockDim.x) {
    double r = 0.0;
    for (int q = 0; q < nqp; q++) {
      const long long e = node * nqp + q;
      const double f = fermi_dirac(beta, lambda[e], lf);
      r += w[e] * f;
      eb += 2.0 * w[e] * lambda[e] * f;
      double sv = 0.0;
      if (f > 0.0 && f < 1.0) sv = f * log(f) + (1.0 - f) * log(1.0 - f);
      ent += 2.0 * w[e] * sv;
    }
    if (rho) rho[node] = 2.0 * r / dV;
  }
  eb = warp_sum_d(eb);
  ent = warp_sum_d(ent);
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = eb;
    red[1][threadIdx.x >> 5] = ent;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int i = 0; i < kCountBlock / 32; i++) {
      a += red[0][i];
      b += red[1][i];
    }
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = b;
  }
}

__global__ void sum_pairs_kernel(const double *__restrict__ part, int n, double *__restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int i = 0; i < n; i++) {
      a += part[2 * i];
      b += part[2 * i + 1];
    }
    out[0] = a;
    out[1] = b;
  }
}

}  // namespace

cudaError_t launch_density_energy(const double *lambda, const double *w, long long n_nodes, int nqp,
                                  double beta, double lf, double dV, double *rho, double *partial,
                                  int grid, double *out, cudaStream_t s) {
  density_energy_kernel<<<grid, kCountBlock, 0, s>>>(lambda, w, n_nodes, nqp, beta, lf, dV, rho,
                                                     partial);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  sum_pairs_kernel<<<1, 32, 0, s>>>(partial, grid, out);
  return cudaGetLastError();
}

cudaError_t launch_electron_count(const double *lambda, const double *w, long long n_nodes,
                                  int nqp, double beta, double lf, double *partial, int grid,
                                  double *out, cudaStream_t s) {
  const long long n = n_nodes * nqp;
  count_partials_kernel<<<grid, kCountBlock, 0, s>>>(lambda, w, n, beta, lf, partial);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  sum_partials_kernel<<<1, 32, 0, s>>>(partial, grid, out);
  return cudaGetLastError();
}

// The message of sq_fermi_density_energy_noalloc failures, reported by sq_last_error_string.
void set_noalloc_error(const std::string &msg);

size_t fermi_scratch_doubles(int grid, int maxit) { return (size_t)grid * (maxit + 4); }

namespace {
cudaError_t launch_fermi_impl(const double *lambda, const double *w, long long n_nodes, int nqp,
                              double beta, double n_electrons, double dV, double tol, int maxit,
                              double *rho, double *out, double *scratch, unsigned *barrier,
                              int *status, int grid, cudaStream_t s, long long spin_limit,
                              int skip_block) {
  cudaError_t e = cudaMemsetAsync(barrier, 0, 2 * sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  void *args[] = {(void *)&lambda, (void *)&w,   (void *)&n_nodes, (void *)&nqp,
                  (void *)&beta,   (void *)&n_electrons, (void *)&dV, (void *)&tol,
                  (void *)&maxit,  (void *)&rho, (void *)&out,     (void *)&scratch,
                  (void *)&barrier, (void *)&status, (void *)&spin_limit, (void *)&skip_block};
  return cudaLaunchCooperativeKernel((const void *)fermi_kernel, dim3(grid), dim3(kFermiBlock),
                                     args, 0, s);
}
}  // namespace

cudaError_t launch_fermi(const double *lambda, const double *w, long long n_nodes, int nqp,
                         double beta, double n_electrons, double dV, double tol, int maxit,
                         double *rho, double *out, double *scratch, unsigned *barrier,
                         int *status, int grid, cudaStream_t s) {
  return launch_fermi_impl(lambda, w, n_nodes, nqp, beta, n_electrons, dV, tol, maxit, rho, out,
                           scratch, barrier, status, grid, s, kSpinLimit, -1);
}

// Fault-injection self-test of the grid barrier's bounded wait: the same cooperative launch
// with one CTA leaving before its first arrival and a short poll limit (about 4096 polls of
// 100 ns), so the other CTAs give up, record kStatusTimeout and return.  Nothing faults or
// hangs: the kernel ends and the context stays usable.
cudaError_t launch_fermi_timeout_selftest(const double *lambda, const double *w, long long n_nodes,
                                          int nqp, double *out, double *scratch,
                                          unsigned *barrier, int *status, int grid,
                                          cudaStream_t s) {
  return launch_fermi_impl(lambda, w, n_nodes, nqp, 30.0, 1.0, 1.0, 1e-12, 10, nullptr, out,
                           scratch, barrier, status, grid, s, 1LL << 12, 0);
}

// ---------------------------------------------------------------------------------------
// Allocation-free entry point.
//
// Some callers cannot call cudaMalloc: code running inside a host framework that owns the
// device allocator and forbids side allocations, plugin hosts that run with a fixed memory
// budget, and stream-ordered pipelines that must not hit the allocator's implicit device
// synchronisation between steps.  For them the Fermi-level kernel can run on a file-scope
// scratch array that is part of the loaded module instead of on handle-owned buffers.
//
// Scratch capacity: kNoallocMaxBlocks CTA partials for each of kNoallocMaxIters bisection
// steps plus four rows for the bracket and energy sums (about 410 KiB of doubles), the grid
// barrier, the four scalar results and a status word.  Every GPU that loads the library
// holds this array until the process exits.  All calls share it and it keeps the contents
// of the last call: the barrier and the status word are cleared at the start of each call,
// everything else is written before it is read.  Two calls whose work overlaps on the GPU
// (on different streams, or from different host threads) race on the array and give wrong
// results; calls must be ordered.
//
// The array's device address belongs to the CUDA context that is current when it is looked
// up, so every call looks it up again with cudaGetSymbolAddress (no allocation): a context
// that was destroyed and made again, or another context made current by the caller, never
// sees a stale address.
// ---------------------------------------------------------------------------------------
namespace {
constexpr int kNoallocMaxBlocks = 256;
constexpr int kNoallocMaxIters = 200;
constexpr size_t kNoallocPartials = (size_t)kNoallocMaxBlocks * (kNoallocMaxIters + 4);

struct NoallocScratch {
  double partials[kNoallocPartials];
  double out[4];
  unsigned barrier[2];
  int status;
  int pad;
};

static __device__ __align__(256) NoallocScratch g_noalloc_scratch;
}  // namespace

extern "C" sq_status sq_fermi_density_energy_noalloc(const double *d_lambda,
                                                     const double *d_weights, long n_nodes,
                                                     int n_qp, double beta, double n_electrons,
                                                     double dV, double tol, int maxit,
                                                     double *d_rho, double *out, void *stream) {
  if (!d_lambda || !d_weights || !out) {
    set_noalloc_error("null argument");
    return SQ_BAD_INPUT;
  }
  if (n_nodes <= 0 || n_qp <= 0 || !(beta > 0) || !(dV > 0) || !(tol > 0)) {
    set_noalloc_error("n_nodes, n_qp, beta, dV and tol must be positive");
    return SQ_BAD_INPUT;
  }
  if (maxit < 1 || maxit > kNoallocMaxIters) {
    set_noalloc_error("maxit must be 1.." + std::to_string(kNoallocMaxIters) +
                      " (capacity of the static scratch array)");
    return SQ_CAPACITY;
  }
  cudaStream_t s = (cudaStream_t)stream;
  // the call ends with a device-to-host copy and a stream synchronisation, neither of which a
  // stream capture allows: refuse before touching the stream
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(s, &cap);
  if (e != cudaSuccess) {
    set_noalloc_error(std::string("cudaStreamIsCapturing: ") + cudaGetErrorString(e));
    return SQ_CUDA_ERROR;
  }
  if (cap != cudaStreamCaptureStatusNone) {
    set_noalloc_error("the stream is being captured; this call synchronises it and cannot be "
                      "captured");
    return SQ_BAD_INPUT;
  }
  int dev = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) {
    set_noalloc_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    return SQ_CUDA_ERROR;
  }
  // the array's address in the current context (looked up on every call, see above)
  void *ptr = nullptr;
  if ((e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch)) != cudaSuccess) {
    set_noalloc_error(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    return SQ_CUDA_ERROR;
  }
  NoallocScratch *scr = reinterpret_cast<NoallocScratch *>(ptr);
  int sms = 0, per_sm = 0;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess ||
      (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fermi_kernel, kFermiBlock, 0)) !=
          cudaSuccess) {
    set_noalloc_error(std::string("device query: ") + cudaGetErrorString(e));
    return SQ_CUDA_ERROR;
  }
  if (per_sm < 1) {
    set_noalloc_error("the Fermi kernel cannot be resident on this device");
    return SQ_CUDA_ERROR;
  }
  // one CTA per SM (co-resident for the cooperative launch), as the handle-based path uses
  const int grid = std::min(sms, kNoallocMaxBlocks);
  if ((e = cudaMemsetAsync(&scr->status, 0, sizeof(int), s)) != cudaSuccess ||
      (e = launch_fermi(d_lambda, d_weights, n_nodes, n_qp, beta, n_electrons, dV, tol, maxit,
                        d_rho, scr->out, scr->partials, scr->barrier, &scr->status, grid, s)) !=
          cudaSuccess) {
    set_noalloc_error(std::string("fermi kernel: ") + cudaGetErrorString(e));
    return SQ_CUDA_ERROR;
  }
  double res[4];
  int st = 0;
  if ((e = cudaMemcpyAsync(res, scr->out, sizeof(res), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaMemcpyAsync(&st, &scr->status, sizeof(int), cudaMemcpyDeviceToHost, s)) !=
          cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess) {
    set_noalloc_error(std::string("result copy: ") + cudaGetErrorString(e));
    return SQ_CUDA_ERROR;
  }
  if (st & kStatusTimeout) {
    set_noalloc_error("a device-side wait gave up");
    return SQ_DEVICE_TIMEOUT;
  }
  out[0] = res[0];
  out[1] = res[1];
  out[2] = res[2];
  // res[3] = bisection steps taken; the kernel leaves the loop early once hi - lo < tol, so
  // reaching maxit means the bracket never got that narrow
  if (res[3] >= (double)maxit) {
    set_noalloc_error("Fermi bisection did not reach tol in maxit steps (outputs hold the last "
                      "midpoint)");
    return SQ_NO_CONVERGENCE;
  }
  return SQ_OK;
}

}  // namespace sq

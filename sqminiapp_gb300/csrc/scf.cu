// scf.cu -- the SCF closure on the GPU (FP64 fields) around the per-node SQ pass.
//
// The reference declares the SCF driver and its pieces without bodies (SCF_LSSGQ,
// src/lsdft.h:153; SolvePoisson :93; mix :183; Vxc_Calc_CA_PW / Exc_Calc_CA_PW :201-202;
// SystemEnergy_Calc_lssgq :209) and reads their parameters (MIXING_PARAMETER,
// MIXING_HISTORY, PULAY_FREQUENCY, TOL_SCF, MAXIT_SCF; src/lsdft_readfiles.cc:219-241;
// EXCHANGE_CORRELATION LDA_PW, test/Mg1.inpt:6).  One iteration k, on density x_k = rho_in:
//   phi   = IFFT(G FFT(rho_in + b))              periodic Poisson of the FD Laplacian
//   Vxc   = LDA: Slater exchange + Perdew-Wang 1992 correlation (unpolarised)
//   Veff  = phi + Vxc  ->  per-node Lanczos + Gauss quadrature  ->  Fermi bisection
//   rho_out, E_band, -TS from the quadrature (fermi.cu)
//   F     = E_band + E_xc[rho_in] - int rho_in Vxc + 1/2 int (b - rho_in) phi - E_self + E_c - TS
//           (the Harris-Foulkes form of the free energy used with density mixing)
//   err   = ||rho_out - rho_in|| / ||rho_out||; converged when err < TOL_SCF
//   mix   = Periodic Pulay (Banerjee, Suryanarayana, Pask, Chem. Phys. Lett. 647 (2016) 31):
//           f_k = rho_out - rho_in; x_{k+1} = xbar + beta P fbar, xbar = x_k - dX gamma,
//           fbar = f_k - dF gamma with (dF^T dF) gamma = dF^T f_k over the last
//           MIXING_HISTORY differences when (k+1) % PULAY_FREQUENCY == 0 (gamma = 0, plain
//           mixing, otherwise); P = Kerker k^2/(k^2 + k_TF^2) (the reference's default
//           preconditioned mixing, precond = 1, src/lsdft_readfiles.cc:102, with its
//           Helmholtz preconditioner declared at src/lsdft.h:231-235), applied exactly with
//           the FD symbol; negatives are cut and the density is scaled back to N_e.
// Every reduction is two-stage with a fixed block count and fixed summation order, so a run
// is bitwise repeatable.
#include <cufft.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <string>
#include <vector>

#include "handle.hpp"
#include "scf_internal.hpp"
#include "sq_gb300.h"
#include "sq_kernels.hpp"

namespace sq {

namespace {

constexpr int kBlock = 256;
constexpr int kRedBlocks = 128;  // partial sums per reduction
constexpr int kMaxHistory = 16;
constexpr int kMaxSums = (kMaxHistory + 1) * (kMaxHistory + 2) / 2;
// FP32 Lanczos vectors leave a noise floor of about 1e-5 in the relative density residual
// (measured on 4-atom Mg cells at h = 0.5 and 0.85); the FP32 engine never asks for less.
// At that residual its free energy is within 1e-6 Ha/atom of the FP64 engine's.
constexpr double kFp32ResidualFloor = 3e-5;
// Default Kerker wave vector (1/bohr).  Larger cells converge faster with stronger damping of
// their long wavelengths (k_TF 2 with mixing 0.5 on 32 and 108 Mg atoms), the 4-atom cell
// with less (k_TF 1, mixing 0.3); callers choose per cell through sq_scf_options.
constexpr double kKerkerKtf = 1.0;

void ckfft(cufftResult r, const char *what) {
  if (r != CUFFT_SUCCESS) throw CudaError(std::string(what) + ": cuFFT error " + std::to_string((int)r));
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Writes the block's sum of v into part[k * gridDim.x + blockIdx.x].
__device__ void block_partial(double v, double *part, int k) {
  __shared__ double red[kBlock / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kBlock / 32; w++) t += red[w];
    part[(size_t)k * gridDim.x + blockIdx.x] = t;
  }
}

// sums[k] = sum over b of part[k * nb + b], k < nsum, in block order.
__global__ void finish_sums(const double *__restrict__ part, int nb, int nsum, double *__restrict__ sums) {
  for (int k = threadIdx.x; k < nsum; k += blockDim.x) {
    double t = 0.0;
    for (int b = 0; b < nb; b++) t += part[(size_t)k * nb + b];
    sums[k] = t;
  }
}

__global__ void add_kernel(const double *__restrict__ a, const double *__restrict__ b,
                           double *__restrict__ out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = a[i] + b[i];
}

__global__ void green_kernel(cufftDoubleComplex *__restrict__ spec, const double *__restrict__ green,
                             long long n, double scale) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double g = green[i] * scale;
    spec[i].x *= g;
    spec[i].y *= g;
  }
}

}  // namespace

// LDA exchange-correlation energy density per electron and potential, unpolarised:
// Slater exchange eps_x = -(3/4)(3 rho/pi)^(1/3), v_x = (4/3) eps_x; Perdew-Wang 1992
// correlation (Phys. Rev. B 45, 13244, Table I, zeta = 0 column: A = 0.031091,
// alpha1 = 0.21370, beta1..4 = 7.5957, 3.5876, 1.6382, 0.49294, p = 1),
// v_c = eps_c - (rs/3) d eps_c / d rs.  rho <= 0 gives zeros.
__host__ __device__ inline void lda_pw92(double rho, double &eps, double &v) {
  if (!(rho > 0.0)) {
    eps = 0.0;
    v = 0.0;
    return;
  }
  const double A = 0.031091, a1 = 0.21370, b1 = 7.5957, b2 = 3.5876, b3 = 1.6382, b4 = 0.49294;
  const double c3pi = 0.98474502184269654;   // (3/pi)^(1/3)
  const double c34pi = 0.62035049089940001;  // (3/(4 pi))^(1/3)
  const double r13 = cbrt(rho);
  const double ex = -0.75 * c3pi * r13;
  const double rs = c34pi / r13;
  const double srs = sqrt(rs);
  const double q0 = -2.0 * A * (1.0 + a1 * rs);
  const double q1 = 2.0 * A * (b1 * srs + b2 * rs + b3 * rs * srs + b4 * rs * rs);
  const double q1p = A * (b1 / srs + 2.0 * b2 + 3.0 * b3 * srs + 4.0 * b4 * rs);
  const double lg = log1p(1.0 / q1);
  const double ec = q0 * lg;
  const double dec = -2.0 * A * a1 * lg - q0 * q1p / (q1 * q1 + q1);
  eps = ex + ec;
  v = (4.0 / 3.0) * ex + ec - rs / 3.0 * dec;
}

namespace {

// vxc, veff = phi + vxc and the partial sums of rho eps_xc, rho vxc and (b - rho) phi.
__global__ void __launch_bounds__(kBlock)
    potential_kernel(const double *__restrict__ rho, const double *__restrict__ phi,
                     const double *__restrict__ b, double *__restrict__ vxc,
                     double *__restrict__ veff, long long n, double *__restrict__ part) {
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double e, v;
    const double r = rho[i];
    lda_pw92(r, e, v);
    vxc[i] = v;
    veff[i] = phi[i] + v;
    s0 += r * e;
    s1 += r * v;
    s2 += (b[i] - r) * phi[i];
  }
  block_partial(s0, part, 0);
  block_partial(s1, part, 1);
  block_partial(s2, part, 2);
}

// f = rho_out - rho_in into `f`; partial sums of f^2 and rho_out^2.
__global__ void __launch_bounds__(kBlock)
    residual_kernel(const double *__restrict__ rin, const double *__restrict__ rout,
                    double *__restrict__ f, long long n, double *__restrict__ part) {
  double s0 = 0.0, s1 = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double d = rout[i] - rin[i];
    f[i] = d;
    s0 += d * d;
    s1 += rout[i] * rout[i];
  }
  block_partial(s0, part, 0);
  block_partial(s1, part, 1);
}

// history slot: dx = x - xprev, df = f - fprev; then xprev = x, fprev = f.
__global__ void history_kernel(const double *__restrict__ x, const double *__restrict__ f,
                               double *__restrict__ xprev, double *__restrict__ fprev,
                               double *__restrict__ dx, double *__restrict__ df, long long n,
                               int have_prev) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    if (have_prev) {
      dx[i] = x[i] - xprev[i];
      df[i] = f[i] - fprev[i];
    }
    xprev[i] = x[i];
    fprev[i] = f[i];
  }
}

// Gram entries: blockIdx.y enumerates pairs (i <= j) of the vectors v_0..v_{c-1} = df slots,
// v_c = f.  Pair p -> partial sums in part[p][gridDim.x].
__global__ void __launch_bounds__(kBlock)
    gram_kernel(const double *__restrict__ df, const double *__restrict__ f, int count,
                long long n, double *__restrict__ part) {
  int p = blockIdx.y, i = 0;
  while (p > count - i) {  // row i holds pairs (i, i..count)
    p -= count - i + 1;
    i++;
  }
  const int j = i + p;
  const double *u = i < count ? df + (size_t)i * n : f;
  const double *v = j < count ? df + (size_t)j * n : f;
  double s = 0.0;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x)
    s += u[e] * v[e];
  block_partial(s, part, blockIdx.y);
}

// xbar = x - sum_j g_j dx_j (in place), fbar = f - sum_j g_j df_j.
__global__ void __launch_bounds__(kBlock)
    pulay_combine_kernel(double *__restrict__ x, const double *__restrict__ f,
                         const double *__restrict__ dx, const double *__restrict__ df,
                         const double *__restrict__ g, int count, double *__restrict__ fbar,
                         long long n) {
  __shared__ double gs[kMaxHistory];
  if (threadIdx.x < count) gs[threadIdx.x] = g[threadIdx.x];
  __syncthreads();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double xv = x[i], fv = f[i];
    for (int j = 0; j < count; j++) {
      xv -= gs[j] * dx[(size_t)j * n + i];
      fv -= gs[j] * df[(size_t)j * n + i];
    }
    x[i] = xv;
    fbar[i] = fv;
  }
}

// Kerker preconditioner k^2 / (k^2 + k_TF^2) with the FD symbol: k^2 -> 2 s(k) = 4 pi / G(k);
// 0 at k = 0.  `scale` folds in the 1/N of the inverse transform.
__global__ void kerker_kernel(cufftDoubleComplex *__restrict__ spec, const double *__restrict__ green,
                              long long n, double ktf2, double scale) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double pk = i == 0 ? 0.0 : 4.0 * M_PI / (4.0 * M_PI + ktf2 * green[i]) * scale;
    spec[i].x *= pk;
    spec[i].y *= pk;
  }
}

__global__ void sub_kernel(const double *__restrict__ a, const double *__restrict__ b,
                           double *__restrict__ out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = a[i] - b[i];
}

// x = max(0, x + beta w) (w may alias nothing else); partial sums of the new x.
__global__ void __launch_bounds__(kBlock)
    mix_kernel(double *__restrict__ x, const double *__restrict__ w, double beta, long long n,
               double *__restrict__ part) {
  double s = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double v = x[i] + beta * w[i];
    v = v > 0.0 ? v : 0.0;
    x[i] = v;
    s += v;
  }
  block_partial(s, part, 0);
}

// x *= n_electrons / (sum * dV)
__global__ void scale_kernel(double *__restrict__ x, const double *__restrict__ sum, double target,
                             long long n) {
  const double sc = target / sum[0];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    x[i] *= sc;
}

}  // namespace

struct ScfState {
  ScfFields fields;
  int N[3] = {0, 0, 0};
  long long ng = 0, nspec = 0;
  double *d_b = nullptr, *d_rho0 = nullptr, *d_green = nullptr;
  double *d_rho_in = nullptr, *d_rho_out = nullptr, *d_phi = nullptr, *d_vxc = nullptr;
  double *d_veff = nullptr, *d_work = nullptr, *d_f = nullptr;
  double *d_dx = nullptr, *d_df = nullptr, *d_xprev = nullptr, *d_fprev = nullptr;
  double *d_part = nullptr, *d_sums = nullptr, *d_gamma = nullptr;
  cufftDoubleComplex *d_spec = nullptr;
  cufftHandle plan_f = 0, plan_i = 0;
  bool plans = false;
  // options in force
  double tol = 1e-6, mix = 0.3, fermi_tol = 1e-12, kerker_ktf = kKerkerKtf;
  int maxit = 100, history = 7, pulay_every = 2;
  // progress
  int iter = 0, have_prev = 0, hist_count = 0;
  bool converged = false;
  std::vector<double> hist_F, hist_err;
  sq_scf_result last{};
  // a sharded iteration in progress (sq_scf_shard_*): this rank's node range, its start time
  long long shard_b = 0, shard_e = 0;
  std::chrono::steady_clock::time_point shard_t0;
  // CUDA graph of an iteration's device part (Poisson, potential, SQ pass)
  bool use_graph = false;
  cudaGraphExec_t graph_exec = nullptr;
  const double *graph_lambda = nullptr;  // the quadrature buffer the graph writes

  ~ScfState() {
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    if (plans) {
      cufftDestroy(plan_f);
      cufftDestroy(plan_i);
    }
    for (double **p : {&d_b, &d_rho0, &d_green, &d_rho_in, &d_rho_out, &d_phi, &d_vxc, &d_veff,
                       &d_work, &d_f, &d_dx, &d_df, &d_xprev, &d_fprev, &d_part, &d_sums, &d_gamma})
      dev_free(*p);
    dev_free(d_spec);
  }
};

void scf_destroy(ScfState *s) { delete s; }

namespace {

int grid_for(long long n) { return (int)std::min<long long>(4096, std::max<long long>(1, (n + kBlock - 1) / kBlock)); }

ScfState &scf_state(sq_handle *h) {
  if (h->scf) return *h->scf;
  if (h->deck.bc != 2) throw std::invalid_argument("the SCF closure needs a periodic deck (BOUNDARY_CONDITION 2)");
  auto *s = new ScfState();
  h->scf = s;
  s->fields = build_scf_fields(h->deck, h->setup);
  for (int a = 0; a < 3; a++) s->N[a] = h->deck.grid[a];
  s->ng = (long long)s->N[0] * s->N[1] * s->N[2];
  s->nspec = (long long)s->N[2] * s->N[1] * (s->N[0] / 2 + 1);
  const size_t nb = sizeof(double) * (size_t)s->ng;
  dev_alloc(&s->d_b, nb, "scf b");
  dev_alloc(&s->d_rho0, nb, "scf rho0");
  dev_alloc(&s->d_green, sizeof(double) * (size_t)s->nspec, "scf green");
  dev_alloc(&s->d_rho_in, nb, "scf rho_in");
  dev_alloc(&s->d_rho_out, nb, "scf rho_out");
  dev_alloc(&s->d_phi, nb, "scf phi");
  dev_alloc(&s->d_vxc, nb, "scf vxc");
  dev_alloc(&s->d_veff, nb, "scf veff");
  dev_alloc(&s->d_work, nb, "scf work");
  dev_alloc(&s->d_f, nb, "scf residual");
  dev_alloc(&s->d_xprev, nb, "scf xprev");
  dev_alloc(&s->d_fprev, nb, "scf fprev");
  dev_alloc(&s->d_dx, nb * kMaxHistory, "scf dx history");
  dev_alloc(&s->d_df, nb * kMaxHistory, "scf df history");
  dev_alloc(&s->d_part, sizeof(double) * (size_t)kMaxSums * kRedBlocks, "scf partials");
  dev_alloc(&s->d_sums, sizeof(double) * kMaxSums, "scf sums");
  dev_alloc(&s->d_gamma, sizeof(double) * kMaxHistory, "scf gamma");
  dev_alloc(&s->d_spec, sizeof(cufftDoubleComplex) * (size_t)s->nspec, "scf spectrum");
  ck(cudaMemcpy(s->d_b, s->fields.b.data(), nb, cudaMemcpyHostToDevice), "b H2D");
  ck(cudaMemcpy(s->d_rho0, s->fields.rho0.data(), nb, cudaMemcpyHostToDevice), "rho0 H2D");
  ck(cudaMemcpy(s->d_green, s->fields.green.data(), sizeof(double) * s->nspec, cudaMemcpyHostToDevice),
     "green H2D");
  // [z][y][x] row-major, x fastest: cufftPlan3d takes the slowest dimension first
  ckfft(cufftPlan3d(&s->plan_f, s->N[2], s->N[1], s->N[0], CUFFT_D2Z), "plan D2Z");
  ckfft(cufftPlan3d(&s->plan_i, s->N[2], s->N[1], s->N[0], CUFFT_Z2D), "plan Z2D");
  s->plans = true;
  return *s;
}

// Sums k < nsum of the last reduction, to host memory (synchronises the stream).
void read_sums(ScfState &s, int nsum, double *out, cudaStream_t st) {
  finish_sums<<<1, 256, 0, st>>>(s.d_part, kRedBlocks, nsum, s.d_sums);
  ck(cudaGetLastError(), "finish sums");
  ck(cudaMemcpyAsync(out, s.d_sums, sizeof(double) * nsum, cudaMemcpyDeviceToHost, st), "sums D2H");
  ck(cudaStreamSynchronize(st), "sync");
}

void poisson(ScfState &s, const double *rho, double *phi, cudaStream_t st) {
  add_kernel<<<grid_for(s.ng), kBlock, 0, st>>>(rho, s.d_b, s.d_work, s.ng);
  ck(cudaGetLastError(), "rho + b");
  ckfft(cufftSetStream(s.plan_f, st), "fft stream");
  ckfft(cufftSetStream(s.plan_i, st), "fft stream");
  ckfft(cufftExecD2Z(s.plan_f, s.d_work, s.d_spec), "D2Z");
  green_kernel<<<grid_for(s.nspec), kBlock, 0, st>>>(s.d_spec, s.d_green, s.nspec, 1.0 / (double)s.ng);
  ck(cudaGetLastError(), "green");
  ckfft(cufftExecZ2D(s.plan_i, s.d_spec, phi), "Z2D");
}

// Small dense solve A g = r (n <= kMaxHistory) by Gaussian elimination with partial
// pivoting, after symmetric Jacobi scaling; false when a pivot is negligible.
bool solve_small(std::vector<double> A, std::vector<double> r, int n, std::vector<double> &g) {
  std::vector<double> d(n);
  for (int i = 0; i < n; i++) {
    if (!(A[i * n + i] > 0.0)) return false;
    d[i] = 1.0 / std::sqrt(A[i * n + i]);
  }
  for (int i = 0; i < n; i++) {
    r[i] *= d[i];
    for (int j = 0; j < n; j++) A[i * n + j] *= d[i] * d[j];
  }
  for (int c = 0; c < n; c++) {
    int piv = c;
    for (int i = c + 1; i < n; i++)
      if (std::fabs(A[i * n + c]) > std::fabs(A[piv * n + c])) piv = i;
    if (std::fabs(A[piv * n + c]) < 1e-13) return false;
    if (piv != c) {
      for (int j = 0; j < n; j++) std::swap(A[c * n + j], A[piv * n + j]);
      std::swap(r[c], r[piv]);
    }
    for (int i = c + 1; i < n; i++) {
      const double m = A[i * n + c] / A[c * n + c];
      for (int j = c; j < n; j++) A[i * n + j] -= m * A[c * n + j];
      r[i] -= m * r[c];
    }
  }
  g.assign(n, 0.0);
  for (int i = n - 1; i >= 0; i--) {
    double v = r[i];
    for (int j = i + 1; j < n; j++) v -= A[i * n + j] * g[j];
    g[i] = v / A[i * n + i];
  }
  for (int i = 0; i < n; i++) g[i] *= d[i];
  return true;
}

void begin(sq_handle *h, const sq_scf_options *o, const double *rho_init, bool rho_on_device,
           cudaStream_t st) {
  ScfState &s = scf_state(h);
  const Deck &d = h->deck;
  s.tol = (o && o->tol > 0) ? o->tol : d.tol_scf;
  if (h->opt.precision == 32) s.tol = std::max(s.tol, kFp32ResidualFloor);
  s.maxit = (o && o->maxit > 0) ? o->maxit : d.maxit_scf;
  s.mix = (o && o->mixing_parameter > 0) ? o->mixing_parameter : d.mixing_parameter;
  s.history = (o && o->mixing_history > 0) ? o->mixing_history : d.mixing_history;
  s.pulay_every = (o && o->pulay_frequency > 0) ? o->pulay_frequency : d.pulay_frequency;
  s.fermi_tol = (o && o->fermi_tol > 0) ? o->fermi_tol : 1e-12;
  // the reference preconditions its mixing by default (precond = 1, src/lsdft_readfiles.cc:102)
  s.kerker_ktf = (o && o->kerker_ktf != 0.0) ? o->kerker_ktf : kKerkerKtf;
  if (s.history > kMaxHistory)
    throw std::invalid_argument("MIXING_HISTORY above " + std::to_string(kMaxHistory) + " is not supported");
  if (s.pulay_every < 1) s.pulay_every = 1;
  s.use_graph = o && o->cuda_graph != 0;
  if (s.graph_exec) {  // captured anew at the second iteration of this run
    cudaGraphExecDestroy(s.graph_exec);
    s.graph_exec = nullptr;
  }
  s.graph_lambda = nullptr;
  s.iter = 0;
  s.have_prev = 0;
  s.hist_count = 0;
  s.converged = false;
  s.hist_F.clear();
  s.hist_err.clear();
  s.last = sq_scf_result{};
  s.last.tol = s.tol;
  const size_t nb = sizeof(double) * (size_t)s.ng;
  if (rho_init) {
    ck(cudaMemcpyAsync(s.d_rho_in, rho_init, nb,
                       rho_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st),
       "rho_init copy");
    // a caller's guess is cut at zero and scaled to the electron count like a mixed density
    const double zero = 0.0;
    ck(cudaMemcpyAsync(s.d_gamma, &zero, sizeof(double), cudaMemcpyHostToDevice, st), "zero");
    mix_kernel<<<kRedBlocks, kBlock, 0, st>>>(s.d_rho_in, s.d_rho0, 0.0, s.ng, s.d_part);
    ck(cudaGetLastError(), "clip");
    finish_sums<<<1, 256, 0, st>>>(s.d_part, kRedBlocks, 1, s.d_sums);
    scale_kernel<<<grid_for(s.ng), kBlock, 0, st>>>(s.d_rho_in, s.d_sums,
                                                    d.n_electrons / h->setup.dV, s.ng);
    ck(cudaGetLastError(), "scale");
  } else {
    ck(cudaMemcpyAsync(s.d_rho_in, s.d_rho0, nb, cudaMemcpyDeviceToDevice, st), "rho0 copy");
  }
  ck(cudaStreamSynchronize(st), "sync");
}

sq_status finish(sq_handle *h, sq_scf_result *res, cudaStream_t st, double lambda_f,
                 double e_band, double ts, std::chrono::steady_clock::time_point t0);

sq_status step(sq_handle *h, sq_scf_result *res, cudaStream_t st) {
  ScfState &s = *h->scf;
  const Deck &d = h->deck;
  const double dV = h->setup.dV;
  const auto t0 = std::chrono::steady_clock::now();
  // potential of rho_in, then the SQ pass: direct launches, or (cuda_graph) the first
  // iteration direct and every later one a replay of one captured graph of the same launches
  // (its buffers are fixed from sq_scf_begin on)
  ensure_quadrature_buffers(h, s.ng);
  auto device_part = [&](cudaStream_t q) -> sq_status {
    poisson(s, s.d_rho_in, s.d_phi, q);
    potential_kernel<<<kRedBlocks, kBlock, 0, q>>>(s.d_rho_in, s.d_phi, s.d_b, s.d_vxc, s.d_veff,
                                                   s.ng, s.d_part);
    ck(cudaGetLastError(), "potential");
    finish_sums<<<1, 256, 0, q>>>(s.d_part, kRedBlocks, 3, s.d_sums + kMaxSums - 3);
    ck(cudaGetLastError(), "finish sums");
    return run_device(h, s.d_veff, 0.0, 0, s.ng, h->d_lambda, h->d_w, h->d_lmin, h->d_lmax, q);
  };
  sq_status rs = SQ_OK;
  if (s.use_graph && s.graph_lambda != h->d_lambda && s.iter > 0) {
    if (s.graph_exec) {
      cudaGraphExecDestroy(s.graph_exec);
      s.graph_exec = nullptr;
    }
    cudaGraph_t g = nullptr;
    ck(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
    rs = device_part(st);  // recorded, not run
    const cudaError_t ec = cudaStreamEndCapture(st, &g);
    if (rs != SQ_OK) {
      if (g) cudaGraphDestroy(g);
      return rs;
    }
    ck(ec, "end capture");
    ck(cudaGraphInstantiate(&s.graph_exec, g, 0), "graph instantiate");
    cudaGraphDestroy(g);
    s.graph_lambda = h->d_lambda;
  }
  if (s.use_graph && s.graph_exec && s.graph_lambda == h->d_lambda) {
    // the handle's timing events bracket the whole graph (potential + SQ pass)
    ck(cudaEventRecord(h->ev[0], st), "event");
    ck(cudaGraphLaunch(s.graph_exec, st), "graph launch");
    ck(cudaEventRecord(h->ev[1], st), "event");
    ck(cudaEventRecord(h->ev[2], st), "event");
    h->ev_valid = true;
    h->last_n = s.ng;
  } else {
    rs = device_part(st);
  }
  if (rs != SQ_OK) return rs;
  // the Lanczos status bits stay set: device_status below reports them with the Fermi ones
  ck(launch_fermi(h->d_lambda, h->d_w, s.ng, h->lp.nqp, h->info.beta, d.n_electrons, dV,
                  s.fermi_tol, h->fermi_maxit, s.d_rho_out, h->d_fermi_out, h->d_fermi_scratch,
                  h->d_bar, h->d_status, h->fermi_grid, st),
     "fermi");
  double fo[4];
  ck(cudaMemcpyAsync(fo, h->d_fermi_out, sizeof(fo), cudaMemcpyDeviceToHost, st), "fermi D2H");
  rs = device_status(h, st);
  if (rs != SQ_OK) return rs;
  return finish(h, res, st, fo[0], fo[1], fo[2], t0);
}

// Everything of an iteration after rho_out, lambda_f, e_band and -TS are known (rho_out in
// s.d_rho_out, the exchange-correlation sums of the potential in the last three sums): the
// residual, the free energy, the history and the Periodic-Pulay update of rho_in.
sq_status finish(sq_handle *h, sq_scf_result *res, cudaStream_t st, double lambda_f,
                 double e_band, double ts, std::chrono::steady_clock::time_point t0) {
  ScfState &s = *h->scf;
  const Deck &d = h->deck;
  const double dV = h->setup.dV;
  const double fo[3] = {lambda_f, e_band, ts};
  double es[3];
  ck(cudaMemcpyAsync(es, s.d_sums + kMaxSums - 3, sizeof(es), cudaMemcpyDeviceToHost, st), "sums D2H");
  ck(cudaStreamSynchronize(st), "sync");
  double kt[2] = {0, 0};
  if (h->ev_valid) {
    float a = 0, b = 0;
    ck(cudaEventElapsedTime(&a, h->ev[0], h->ev[1]), "elapsed");
    ck(cudaEventElapsedTime(&b, h->ev[1], h->ev[2]), "elapsed");
    kt[0] = a;
    kt[1] = b;
  }
  // residual
  residual_kernel<<<kRedBlocks, kBlock, 0, st>>>(s.d_rho_in, s.d_rho_out, s.d_f, s.ng, s.d_part);
  ck(cudaGetLastError(), "residual");
  double rr[2];
  read_sums(s, 2, rr, st);
  const double err = std::sqrt(rr[0] / rr[1]);

  sq_scf_result &r = s.last;
  r.iterations = s.iter + 1;
  r.lambda_f = fo[0];
  r.e_band = fo[1];
  r.ts = fo[2];
  r.e_xc = es[0] * dV;
  r.e_xc_dc = es[1] * dV;
  r.e_electrostatic = 0.5 * es[2] * dV;
  r.e_self = s.fields.e_self;
  r.e_corr = s.fields.e_corr;
  r.free_energy = r.e_band + r.e_xc - r.e_xc_dc + r.e_electrostatic - r.e_self + r.e_corr + r.ts;
  r.free_energy_per_atom = r.free_energy / std::max<size_t>(1, d.atom_type.size());
  r.residual = err;
  r.sq_ms += kt[0] + kt[1];
  s.hist_F.push_back(r.free_energy);
  s.hist_err.push_back(err);
  s.converged = err < s.tol;
  r.converged = s.converged ? 1 : 0;

  if (!s.converged) {
    // Periodic Pulay mixing of rho_in
    const int slot = s.have_prev ? (s.iter - 1) % s.history : 0;
    history_kernel<<<grid_for(s.ng), kBlock, 0, st>>>(
        s.d_rho_in, s.d_f, s.d_xprev, s.d_fprev, s.d_dx + (size_t)slot * s.ng,
        s.d_df + (size_t)slot * s.ng, s.ng, s.have_prev);
    ck(cudaGetLastError(), "history");
    if (s.have_prev) s.hist_count = std::min(s.hist_count + 1, s.history);
    s.have_prev = 1;
    int count = 0;
    std::vector<double> g;
    if ((s.iter + 1) % s.pulay_every == 0 && s.hist_count > 0) {
      const int c = s.hist_count, npair = (c + 1) * (c + 2) / 2;
      gram_kernel<<<dim3(kRedBlocks, npair), kBlock, 0, st>>>(s.d_df, s.d_f, c, s.ng, s.d_part);
      ck(cudaGetLastError(), "gram");
      std::vector<double> pr(npair);
      read_sums(s, npair, pr.data(), st);
      std::vector<double> A((size_t)c * c), rhs(c);
      int p = 0;
      for (int i = 0; i <= c; i++)
        for (int j = i; j <= c; j++, p++) {
          if (j < c) {
            A[i * c + j] = pr[p];
            A[j * c + i] = pr[p];
          } else if (i < c) {
            rhs[i] = pr[p];
          }
        }
      if (solve_small(A, rhs, c, g)) count = c;
    }
    if (count > 0)
      ck(cudaMemcpyAsync(s.d_gamma, g.data(), sizeof(double) * count, cudaMemcpyHostToDevice, st), "gamma H2D");
    // xbar, fbar (= x, f when there is no Pulay step); w = P fbar
    pulay_combine_kernel<<<grid_for(s.ng), kBlock, 0, st>>>(s.d_rho_in, s.d_f, s.d_dx, s.d_df,
                                                            s.d_gamma, count, s.d_work, s.ng);
    ck(cudaGetLastError(), "pulay combine");
    if (s.kerker_ktf > 0.0) {
      ckfft(cufftExecD2Z(s.plan_f, s.d_work, s.d_spec), "D2Z");
      kerker_kernel<<<grid_for(s.nspec), kBlock, 0, st>>>(s.d_spec, s.d_green, s.nspec,
                                                          s.kerker_ktf * s.kerker_ktf, 1.0 / (double)s.ng);
      ck(cudaGetLastError(), "kerker");
      ckfft(cufftExecZ2D(s.plan_i, s.d_spec, s.d_work), "Z2D");
    }
    mix_kernel<<<kRedBlocks, kBlock, 0, st>>>(s.d_rho_in, s.d_work, s.mix, s.ng, s.d_part);
    ck(cudaGetLastError(), "mix");
    finish_sums<<<1, 256, 0, st>>>(s.d_part, kRedBlocks, 1, s.d_sums);
    scale_kernel<<<grid_for(s.ng), kBlock, 0, st>>>(s.d_rho_in, s.d_sums, d.n_electrons / dV, s.ng);
    ck(cudaGetLastError(), "scale");
    ck(cudaStreamSynchronize(st), "sync");
  }
  s.iter++;
  r.seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (res) *res = r;
  return SQ_OK;
}

}  // namespace

double *scf_rho0_device(sq_handle *h) { return scf_state(h).d_rho0; }
double *scf_rho_out_device(sq_handle *h) { return scf_state(h).d_rho_out; }
void scf_begin_device_density(sq_handle *h, const sq_scf_options *o, const double *d_rho) {
  begin(h, o, d_rho, true, h->own_stream);
}

// After a learned start: keep of its correction to the atomic superposition only the short
// wavelengths, rho_in = max(0, rho0 + P (rho_in - rho0)) with the Kerker symbol
// P = k^2 / (k^2 + k0^2), scaled to the electron count.  A local model's error at long
// wavelengths is the part a metal's density response amplifies (as 1/k^2).
void scf_highpass_start(sq_handle *h, double k0) {
  ScfState &s = *h->scf;
  const cudaStream_t st = h->own_stream;
  sub_kernel<<<grid_for(s.ng), kBlock, 0, st>>>(s.d_rho_in, s.d_rho0, s.d_work, s.ng);
  ck(cudaGetLastError(), "correction");
  ckfft(cufftSetStream(s.plan_f, st), "fft stream");
  ckfft(cufftSetStream(s.plan_i, st), "fft stream");
  ckfft(cufftExecD2Z(s.plan_f, s.d_work, s.d_spec), "D2Z");
  kerker_kernel<<<grid_for(s.nspec), kBlock, 0, st>>>(s.d_spec, s.d_green, s.nspec, k0 * k0,
                                                      1.0 / (double)s.ng);
  ck(cudaGetLastError(), "high-pass");
  ckfft(cufftExecZ2D(s.plan_i, s.d_spec, s.d_work), "Z2D");
  ck(cudaMemcpyAsync(s.d_rho_in, s.d_rho0, sizeof(double) * (size_t)s.ng,
                     cudaMemcpyDeviceToDevice, st), "rho0 copy");
  mix_kernel<<<kRedBlocks, kBlock, 0, st>>>(s.d_rho_in, s.d_work, 1.0, s.ng, s.d_part);
  ck(cudaGetLastError(), "start");
  finish_sums<<<1, 256, 0, st>>>(s.d_part, kRedBlocks, 1, s.d_sums);
  scale_kernel<<<grid_for(s.ng), kBlock, 0, st>>>(s.d_rho_in, s.d_sums,
                                                  h->deck.n_electrons / h->setup.dV, s.ng);
  ck(cudaGetLastError(), "scale");
  ck(cudaStreamSynchronize(st), "sync");
}

}  // namespace sq

using namespace sq;

extern "C" {

sq_status sq_scf_begin(sq_handle *h, const sq_scf_options *opt, const double *rho_init) {
  if (!h) return fail(SQ_BAD_INPUT, "null argument");
  return guarded([&] {
    ck(cudaSetDevice(h->opt.device), "cudaSetDevice");
    begin(h, opt, rho_init, false, h->own_stream);
    return SQ_OK;
  });
}

sq_status sq_scf_begin_device(sq_handle *h, const sq_scf_options *opt, const double *d_rho_init) {
  if (!h || !d_rho_init) return fail(SQ_BAD_INPUT, "null argument");
  return guarded([&] {
    ck(cudaSetDevice(h->opt.device), "cudaSetDevice");
    begin(h, opt, d_rho_init, true, h->own_stream);
    return SQ_OK;
  });
}

sq_status sq_scf_step(sq_handle *h, sq_scf_result *result) {
  if (!h) return fail(SQ_BAD_INPUT, "null argument");
  if (!h->scf) return fail(SQ_BAD_INPUT, "sq_scf_begin has not been called");
  return guarded([&] {
    ck(cudaSetDevice(h->opt.device), "cudaSetDevice");
    return step(h, result, h->own_stream);
  });
}

// ---- one SCF iteration with the nodes sharded over ranks (see sq_gb300.h) ----
sq_status sq_scf_shard_sq(sq_handle *h, long node_begin, long node_end, double *minmax) {
  if (!h || !minmax) return fail(SQ_BAD_INPUT, "null argument");
  if (!h->scf) return fail(SQ_BAD_INPUT, "sq_scf_begin has not been called");
  return guarded([&] {
    ScfState &s = *h->scf;
    if (node_begin < 0 || node_end > s.ng || node_end <= node_begin)
      return fail(SQ_BAD_INPUT, "node range outside the grid");
    ck(cudaSetDevice(h->opt.device), "cudaSetDevice");
    cudaStream_t st = h->own_stream;
    s.shard_t0 = std::chrono::steady_clock::now();
    const long long n = node_end - node_begin;
    ensure_quadrature_buffers(h, n);
    poisson(s, s.d_rho_in, s.d_phi, st);
    potential_kernel<<<kRedBlocks, kBlock, 0, st>>>(s.d_rho_in, s.d_phi, s.d_b, s.d_vxc, s.d_veff,
                                                    s.ng, s.d_part);
    ck(cudaGetLastError(), "potential");
    finish_sums<<<1, 256, 0, st>>>(s.d_part, kRedBlocks, 3, s.d_sums + kMaxSums - 3);
    ck(cudaGetLastError(), "finish sums");
    sq_status rs = run_device(h, s.d_veff, 0.0, node_begin, node_end, h->d_lambda, h->d_w,
                              h->d_lmin, h->d_lmax, st);
    if (rs != SQ_OK) return rs;
    rs = device_status(h, st);
    if (rs != SQ_OK) return rs;
    std::vector<double> lo(n), hi(n);
    ck(cudaMemcpy(lo.data(), h->d_lmin, sizeof(double) * n, cudaMemcpyDeviceToHost), "D2H");
    ck(cudaMemcpy(hi.data(), h->d_lmax, sizeof(double) * n, cudaMemcpyDeviceToHost), "D2H");
    minmax[0] = *std::min_element(lo.begin(), lo.end());
    minmax[1] = *std::max_element(hi.begin(), hi.end());
    s.shard_b = node_begin;
    s.shard_e = node_end;
    return SQ_OK;
  });
}

sq_status sq_scf_shard_counts(sq_handle *h, int k, const double *lambda_f, double *counts) {
  if (!h || !lambda_f || !counts || k <= 0) return fail(SQ_BAD_INPUT, "null argument or k <= 0");
  if (!h->scf || h->scf->shard_e <= h->scf->shard_b)
    return fail(SQ_BAD_INPUT, "sq_scf_shard_sq has not been called");
  return guarded([&] {
    ScfState &s = *h->scf;
    ck(cudaSetDevice(h->opt.device), "cudaSetDevice");
    cudaStream_t st = h->own_stream;
    const int grid = 4 * h->num_sms;
    for (int i = 0; i < k; i++) {
      ck(launch_electron_count(h->d_lambda, h->d_w, s.shard_e - s.shard_b, h->lp.nqp,
                               h->info.beta, lambda_f[i], h->d_fermi_scratch, grid,
                               h->d_fermi_out, st),
         "electron count");
      ck(cudaMemcpyAsync(counts + i, h->d_fermi_out, sizeof(double), cudaMemcpyDeviceToHost, st),
         "D2H");
    }
    ck(cudaStreamSynchronize(st), "sync");
    return SQ_OK;
  });
}

sq_status sq_scf_shard_density(sq_handle *h, double lambda_f, double *rho_local, double *sums) {
  if (!h || !rho_local || !sums) return fail(SQ_BAD_INPUT, "null argument");
  if (!h->scf || h->scf->shard_e <= h->scf->shard_b)
    return fail(SQ_BAD_INPUT, "sq_scf_shard_sq has not been called");
  return guarded([&] {
    ScfState &s = *h->scf;
    ck(cudaSetDevice(h->opt.device), "cudaSetDevice");
    cudaStream_t st = h->own_stream;
    const long long n = s.shard_e - s.shard_b;
    const int grid = 2 * h->num_sms;
    ck(launch_density_energy(h->d_lambda, h->d_w, n, h->lp.nqp, h->info.beta, lambda_f,
                             h->setup.dV, s.d_rho_out + s.shard_b, h->d_fermi_scratch, grid,
                             h->d_fermi_out, st),
       "density");
    ck(cudaMemcpyAsync(rho_local, s.d_rho_out + s.shard_b, sizeof(double) * n,
                       cudaMemcpyDeviceToHost, st), "D2H");
    ck(cudaMemcpyAsync(sums, h->d_fermi_out, 2 * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H");
    ck(cudaStreamSynchronize(st), "sync");
    return SQ_OK;
  });
}

sq_status sq_scf_shard_finish(sq_handle *h, const double *rho_out, double lambda_f, double e_band,
                              double ts, sq_scf_result *result) {
  if (!h || !rho_out) return fail(SQ_BAD_INPUT, "null argument");
  if (!h->scf || h->scf->shard_e <= h->scf->shard_b)
    return fail(SQ_BAD_INPUT, "sq_scf_shard_sq has not been called");
  return guarded([&] {
    ScfState &s = *h->scf;
    ck(cudaSetDevice(h->opt.device), "cudaSetDevice");
    cudaStream_t st = h->own_stream;
    ck(cudaMemcpyAsync(s.d_rho_out, rho_out, sizeof(double) * s.ng, cudaMemcpyHostToDevice, st),
       "rho_out H2D");
    s.shard_b = s.shard_e = 0;
    return finish(h, result, st, lambda_f, e_band, ts, s.shard_t0);
  });
}

sq_status sq_scf_run(sq_handle *h, const sq_scf_options *opt, const double *rho_init,
                     sq_scf_result *result) {
  sq_status st = sq_scf_begin(h, opt, rho_init);
  if (st != SQ_OK) return st;
  for (int k = 0; k < h->scf->maxit; k++) {
    st = sq_scf_step(h, result);
    if (st != SQ_OK) return st;
    if (h->scf->converged) return SQ_OK;
  }
  return fail(SQ_NO_CONVERGENCE, "SCF did not reach TOL_SCF within MAXIT_SCF iterations");
}

sq_status sq_scf_get_density(sq_handle *h, double *rho_out, double *rho_in) {
  if (!h || !h->scf) return fail(SQ_BAD_INPUT, "no SCF state");
  return guarded([&] {
    ScfState &s = *h->scf;
    ck(cudaStreamSynchronize(h->own_stream), "sync");
    if (rho_out)
      ck(cudaMemcpy(rho_out, s.d_rho_out, sizeof(double) * s.ng, cudaMemcpyDeviceToHost), "rho D2H");
    if (rho_in)
      ck(cudaMemcpy(rho_in, s.d_rho_in, sizeof(double) * s.ng, cudaMemcpyDeviceToHost), "rho D2H");
    return SQ_OK;
  });
}

sq_status sq_scf_get_fields(sq_handle *h, double *b, double *rho0, double *phi, double *vxc,
                            double *scalars) {
  if (!h) return fail(SQ_BAD_INPUT, "null argument");
  return guarded([&] {
    ck(cudaSetDevice(h->opt.device), "cudaSetDevice");
    ScfState &s = scf_state(h);
    const size_t nb = sizeof(double) * (size_t)s.ng;
    ck(cudaStreamSynchronize(h->own_stream), "sync");
    if (b) std::copy(s.fields.b.begin(), s.fields.b.end(), b);
    if (rho0) std::copy(s.fields.rho0.begin(), s.fields.rho0.end(), rho0);
    if (phi) ck(cudaMemcpy(phi, s.d_phi, nb, cudaMemcpyDeviceToHost), "phi D2H");
    if (vxc) ck(cudaMemcpy(vxc, s.d_vxc, nb, cudaMemcpyDeviceToHost), "vxc D2H");
    if (scalars) {
      scalars[0] = s.fields.e_self;
      scalars[1] = s.fields.e_self_ref;
      scalars[2] = s.fields.e_corr;
      scalars[3] = s.fields.b_total;
    }
    return SQ_OK;
  });
}

sq_status sq_scf_history(sq_handle *h, int cap, double *free_energy, double *residual, int *count) {
  if (!h || !count) return fail(SQ_BAD_INPUT, "null argument");
  if (!h->scf) {
    *count = 0;
    return SQ_OK;
  }
  const ScfState &s = *h->scf;
  *count = (int)s.hist_F.size();
  for (int i = 0; i < std::min(cap, *count); i++) {
    if (free_energy) free_energy[i] = s.hist_F[i];
    if (residual) residual[i] = s.hist_err[i];
  }
  return SQ_OK;
}

sq_status sq_lda_pw92(const double *rho, long n, double *eps, double *v) {
  if ((!rho && n > 0) || n < 0) return fail(SQ_BAD_INPUT, "null argument");
  for (long i = 0; i < n; i++) {
    double e, p;
    sq::lda_pw92(rho[i], e, p);
    if (eps) eps[i] = e;
    if (v) v[i] = p;
  }
  return SQ_OK;
}

}  // extern "C"

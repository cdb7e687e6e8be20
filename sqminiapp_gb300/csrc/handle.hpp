// handle.hpp -- the engine handle behind the C ABI and the helpers shared by its entry points.
#pragma once

#include <cuda_runtime.h>

#include <stdexcept>
#include <string>

#include "sq_gb300.h"
#include "sq_internal.hpp"

namespace sq {

struct ScfState;  // scf.cu
void scf_destroy(ScfState *s);

struct CudaError : std::runtime_error {
  explicit CudaError(const std::string &m) : std::runtime_error(m) {}
};

// Records the message for sq_last_error_string and returns s.
sq_status fail(sq_status s, const std::string &msg);
const std::string &last_error();
// Throws CudaError when e is not cudaSuccess.
void ck(cudaError_t e, const char *what);

template <typename P> void dev_alloc(P **ptr, size_t bytes, const char *what) {
  *ptr = nullptr;
  if (bytes == 0) bytes = 16;
  ck(cudaMalloc((void **)ptr, bytes), what);
}

template <typename P> void dev_free(P *&ptr) {
  if (ptr) cudaFree((void *)ptr);
  ptr = nullptr;
}

// Device buffer owned by a scope: freed on every exit path, exceptions included.
template <typename P> struct DevBuf {
  P *p = nullptr;
  DevBuf(size_t bytes, const char *what) { dev_alloc(&p, bytes, what); }
  ~DevBuf() { dev_free(p); }
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  P *get() const { return p; }
};

// Grows a device array of doubles to at least `need` elements (contents are not kept).
void ensure_capacity(double *&ptr, long long &cap, long long need, const char *what);

// Exceptions of the body become status codes.
template <typename F> sq_status guarded(F &&f) {
  try {
    return f();
  } catch (const CudaError &e) {
    return fail(SQ_CUDA_ERROR, e.what());
  } catch (const std::exception &e) {
    return fail(SQ_BAD_INPUT, e.what());
  }
}

}  // namespace sq

struct sq_handle {
  sq::Deck deck;
  sq::Setup setup;
  sq_options opt{};
  sq_info info{};
  sq::LanczosParams lp{};
  int num_sms = 0;
  bool u_smem = false;
  bool quad = false;    // the split-pass FP32 kernel (kLayoutQuad)
  bool tuned = false;   // its tile has been chosen (sq_options.tile, or timed on a first call)
  size_t smem = 0;
  int grid = 0;
  int block = 0;
  int fermi_grid = 0;
  size_t elem = 4;
  // device buffers owned by the handle
  sq::ImageMeta *d_images = nullptr;
  void *d_tables = nullptr;
  void *d_veff_ext = nullptr;
  double *d_veff_in = nullptr;
  void *d_u = nullptr;
  void *d_proj = nullptr;
  int *d_status = nullptr;
  double *d_ab = nullptr;
  long long ab_cap = 0;
  long long last_n = 0;
  double *d_lambda = nullptr, *d_w = nullptr, *d_lmin = nullptr, *d_lmax = nullptr;
  long long out_cap = 0;
  double *d_rho = nullptr;
  long long rho_cap = 0;
  double *d_fermi_scratch = nullptr;
  unsigned *d_bar = nullptr;
  double *d_fermi_out = nullptr;
  int fermi_maxit = 400;
  cudaStream_t own_stream = nullptr;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  bool ev_valid = false;
  sq::ScfState *scf = nullptr;  // SCF closure state, created by the first SCF call
  // measured cost of one node on one SM (ms), from the events of the last Lanczos launch;
  // mixed-cell batches split the SMs by it
  double node_sm_ms = 0.0;
  int cost_grid = 0;
  long long cost_nodes = 0;

  ~sq_handle();
};

namespace sq {

// Per-node Lanczos + quadrature of nodes [nb, ne) on stream s (device buffers).
// grid_limit > 0 caps the persistent grid (CTAs = SMs used), else one CTA per SM.
sq_status run_device(sq_handle *h, const double *d_veff, double veff_const, long long nb,
                     long long ne, double *d_lambda, double *d_w, double *d_lmin, double *d_lmax,
                     cudaStream_t s, int grid_limit = 0);
// Folds the timing of the last Lanczos launch, once its events have completed, into
// node_sm_ms (non-blocking).
void update_node_cost(sq_handle *h);
// Synchronises s and turns the device status bits into a status code.
sq_status device_status(sq_handle *h, cudaStream_t s);
// Grows the handle's lambda / weight / lambda_min / lambda_max arrays to n nodes.
void ensure_quadrature_buffers(sq_handle *h, long long n);

}  // namespace sq

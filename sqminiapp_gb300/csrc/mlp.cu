// mlp.cu -- learned warm start: node descriptors, a BF16 MLP on the 5th-generation tensor
// cores (inference and training kernels), Adam, and the SCF start from its prediction.
//
// The reference starts every SCF from the atomic superposition (SuperposAtRho,
// src/ilsdft.h:269) and has no learned part.  Here a 64-128-128-1 MLP with SiLU activations
// maps 64 rotation-invariant neighbour descriptors of a grid point to the correction
// rho_SCF - rho_0 of the converged density over the superposition; rho_0 + prediction, cut at
// zero and scaled to N_e, starts the SCF.  A zero network is exactly the superposition start.
//
// Descriptors (per grid point x, over atom images J within R_CUT = 8 bohr):
//   g_n(r) = exp(-(r - mu_n)^2 / (2 sigma^2)) (cos(pi r / R_CUT) + 1)/2, mu_n = 8n/15, sigma = 0.5
//   c_{n,lm} = sum_J g_n(r_J) Y_lm(x - X_J)  (real harmonics l <= 3, reference constants)
//   feature[4n + l] = sqrt(sum_m c_{n,lm}^2)
// Network (standardised features, standardised target): BF16 operands, FP32 accumulation in
// TMEM.  One CTA works on 128-row tiles: GEMM1 X[128x64] W1 -> Z1, SiLU -> H1 (BF16, shared),
// GEMM2 H1 W2 -> Z2, SiLU, dot with w3 on the CUDA cores.  Training adds the backward pass on
// the same tile: dZ2 (BF16), GEMM3 dH1 = dZ2 W2^T, GEMM4 dW2 += H1^T dZ2, dZ1 = dH1 SiLU'(Z1)
// (BF16), GEMM5 dW1^T += dZ1^T X; the weight gradients accumulate in TMEM over the CTA's tiles.
// Every operand is K-major without swizzle (tc5.cuh); the transposed operands are written as
// separate K-major copies, so no MMA needs a transposed descriptor.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "handle.hpp"
#include "sq_gb300.h"
#include "sq_kernels.hpp"
#include "tc5.cuh"

namespace sq {

// SCF entry points of scf.cu used here
double *scf_rho0_device(sq_handle *h);
double *scf_rho_out_device(sq_handle *h);
void scf_begin_device_density(sq_handle *h, const sq_scf_options *o, const double *d_rho);
void scf_highpass_start(sq_handle *h, double k0);

namespace {

using bf16 = __nv_bfloat16;
constexpr int kFeat = 64, kHid = 128, kTile = 128;
constexpr float kRcut = 8.0f, kSigma = 0.5f;
constexpr int oW1 = 0, ob1 = oW1 + kFeat * kHid, oW2 = ob1 + kHid, ob2 = oW2 + kHid * kHid,
              ow3 = ob2 + kHid, ob3 = ow3 + kHid, kParams = ob3 + 1;
constexpr int kPartial = kParams + 1;  // + loss
static_assert(kParams == SQ_MLP_N_PARAMS, "parameter count of the header");
constexpr uint32_t kXTileBytes = kTile * kFeat * 2;  // 16 KiB
constexpr long long kWaitLimit = 1LL << 22;
constexpr int kStatusTimeoutBit = 8;

__device__ __forceinline__ float silu(float z) { return z / (1.0f + expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
  const float s = 1.0f / (1.0f + expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

__device__ __forceinline__ void st_bf16(uint8_t *base, uint32_t off, float v) {
  *reinterpret_cast<bf16 *>(base + off) = __float2bfloat16_rn(v);
}

// Warp reduce-scatter of v[32] over the lanes: lane L ends with sum over lanes of v[L].
__device__ __forceinline__ float transpose_reduce(float (&v)[32]) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int s = 16; s >= 1; s >>= 1) {
    const bool upper = lane & s;
#pragma unroll
    for (int i = 0; i < s; i++) {
      const float send = upper ? v[i] : v[i + s];
      const float keep = upper ? v[i + s] : v[i];
      v[i] = keep + __shfl_xor_sync(full, send, s);
    }
  }
  return v[0];
}

// ---------------------------------------------------------------------------------------------
// descriptors: one warp per grid point; lane L handles radial n = L/2 and harmonics
// [8 (L&1), 8 (L&1) + 8).
__global__ void descriptor_kernel(const float4 *__restrict__ img, int n_img, int Nx, int Ny,
                                  float hx, float hy, float hz, float Rx, float Ry, float Rz,
                                  long long n_nodes, float *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  const int n = lane >> 1, half = lane & 1;
  const float mu = n * (kRcut / 15.0f);
  const float inv2s2 = 1.0f / (2.0f * kSigma * kSigma);
  for (long long node = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); node < n_nodes;
       node += warps) {
    const int i = (int)(node % Nx), j = (int)((node / Nx) % Ny), k = (int)(node / ((long long)Nx * Ny));
    const float px = i * hx - Rx, py = j * hy - Ry, pz = k * hz - Rz;
    float c[8];
#pragma unroll
    for (int m = 0; m < 8; m++) c[m] = 0.f;
    for (int J = 0; J < n_img; J++) {
      const float4 a = img[J];
      const float dx = px - a.x, dy = py - a.y, dz = pz - a.z;
      const float r2 = dx * dx + dy * dy + dz * dz;
      if (r2 >= kRcut * kRcut) continue;
      const float r = sqrtf(r2);
      const float fc = 0.5f * (cospif(r / kRcut) + 1.0f);
      const float g = expf(-(r - mu) * (r - mu) * inv2s2) * fc;
      const bool on = r > 1e-6f;
      const float inv = on ? 1.0f / r : 0.0f;
      const float x = dx * inv, y = dy * inv, z = dz * inv;
      float Y[8];
      if (half == 0) {
        Y[0] = 0.282094791773878f;
        Y[1] = 0.488602511902920f * y;
        Y[2] = 0.488602511902920f * z;
        Y[3] = 0.488602511902920f * x;
        Y[4] = 1.092548430592079f * x * y;
        Y[5] = 1.092548430592079f * y * z;
        Y[6] = 0.315391565252520f * (2.f * z * z - x * x - y * y);
        Y[7] = 1.092548430592079f * z * x;
      } else {
        Y[0] = 0.546274215296040f * (x * x - y * y);
        Y[1] = 0.590043589926644f * (3.f * x * x - y * y) * y;
        Y[2] = 2.890611442640554f * x * y * z;
        Y[3] = 0.457045799464466f * y * (4.f * z * z - x * x - y * y);
        Y[4] = 0.373176332590115f * z * (2.f * z * z - 3.f * x * x - 3.f * y * y);
        Y[5] = 0.457045799464466f * x * (4.f * z * z - x * x - y * y);
        Y[6] = 1.445305721320277f * z * (x * x - y * y);
        Y[7] = 0.590043589926644f * x * (x * x - 3.f * y * y);
      }
#pragma unroll
      for (int m = 0; m < 8; m++) c[m] += g * Y[m];
    }
    float p0, p1, p2, p3;
    if (half == 0) {
      p0 = c[0] * c[0];
      p1 = c[1] * c[1] + c[2] * c[2] + c[3] * c[3];
      p2 = c[4] * c[4] + c[5] * c[5] + c[6] * c[6] + c[7] * c[7];
      p3 = 0.f;
    } else {
      p0 = p1 = 0.f;
      p2 = c[0] * c[0];
      p3 = 0.f;
#pragma unroll
      for (int m = 1; m < 8; m++) p3 += c[m] * c[m];
    }
    p2 += __shfl_xor_sync(0xffffffffu, p2, 1);
    float *o = out + node * kFeat + 4 * n;
    if (half == 0) {
      o[0] = sqrtf(p0);
      o[1] = sqrtf(p1);
      o[2] = sqrtf(p2);
    } else {
      o[3] = sqrtf(p3);
    }
  }
}

// standardised BF16 features in the tile layouts: xa = A operand [128 rows][64] per tile,
// xt = K-major copy of its transpose [64][128 rows] per tile (may be null); rows >= n are 0.
__global__ void pack_features_kernel(const float *__restrict__ raw, long long n, long long n_pad,
                                     const float *__restrict__ mean, const float *__restrict__ inv_std,
                                     uint8_t *__restrict__ xa, uint8_t *__restrict__ xt) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n_pad * kFeat;
       e += (long long)gridDim.x * blockDim.x) {
    const long long row = e / kFeat;
    const int f = (int)(e % kFeat);
    const float v = row < n ? (raw[e] - mean[f]) * inv_std[f] : 0.f;
    const long long t = row / kTile;
    const uint32_t r = (uint32_t)(row % kTile);
    st_bf16(xa + t * kXTileBytes, tc5::tile_offset(r, f, kFeat), v);
    if (xt) st_bf16(xt + t * kXTileBytes, tc5::tile_offset(f, r, kTile), v);
  }
}

// BF16 B operands from the FP32 master weights: w1p [hid][in] (K = 64), w2p [out][in]
// (K = 128) for the forward products, w2tp [in][out] (K = 128) for dH1 = dZ2 W2^T.
__global__ void pack_weights_kernel(const float *__restrict__ p, uint8_t *__restrict__ w1p,
                                    uint8_t *__restrict__ w2p, uint8_t *__restrict__ w2tp) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < kFeat * kHid + kHid * kHid;
       e += gridDim.x * blockDim.x) {
    if (e < kFeat * kHid) {
      const int in = e / kHid, hid = e % kHid;
      st_bf16(w1p, tc5::tile_offset(hid, in, kFeat), p[oW1 + e]);
    } else {
      const int q = e - kFeat * kHid, in = q / kHid, out = q % kHid;
      st_bf16(w2p, tc5::tile_offset(out, in, kHid), p[oW2 + q]);
      st_bf16(w2tp, tc5::tile_offset(in, out, kHid), p[oW2 + q]);
    }
  }
}

__device__ __forceinline__ float bf16_round(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

// shared-memory map of the forward kernel
constexpr uint32_t kFwdXs = 0, kFwdW1 = 16384, kFwdW2 = 32768, kFwdH1 = 65536, kFwdB1 = 98304,
                   kFwdB2 = kFwdB1 + 512, kFwdW3 = kFwdB2 + 512, kFwdBar = kFwdW3 + 512,
                   kFwdSmem = kFwdBar + 64;

// y[row] = network output (standardised units) for every row of xa (ntiles tiles).
__global__ void __launch_bounds__(128) mlp_forward_kernel(const uint8_t *__restrict__ xa, long long ntiles,
                                                          long long n_rows, const uint8_t *__restrict__ w1p,
                                                          const uint8_t *__restrict__ w2p,
                                                          const float *__restrict__ params,
                                                          float *__restrict__ y, int *status) {
  extern __shared__ __align__(1024) uint8_t sm[];
  float *b1 = reinterpret_cast<float *>(sm + kFwdB1);
  float *b2 = reinterpret_cast<float *>(sm + kFwdB2);
  float *w3 = reinterpret_cast<float *>(sm + kFwdW3);
  uint64_t *bar_tma = reinterpret_cast<uint64_t *>(sm + kFwdBar);
  uint64_t *bar_mma = bar_tma + 1;
  uint32_t *slot = reinterpret_cast<uint32_t *>(bar_tma + 2);
  const int tid = threadIdx.x, warp = tid >> 5;
  if (tid == 0) {
    tc5::mbar_init(bar_tma, 1);
    tc5::mbar_init(bar_mma, 1);
    tc5::fence_async_smem();
  }
  if (warp == 0) tc5::tmem_alloc(slot, 256);
  b1[tid] = params[ob1 + tid];
  b2[tid] = params[ob2 + tid];
  w3[tid] = bf16_round(params[ow3 + tid]);
  const float b3 = params[ob3];
  tc5::fence_before_sync();
  __syncthreads();
  tc5::fence_after_sync();
  const uint32_t tmem = *slot;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  uint32_t tma_phase = 0, mma_phase = 0;
  bool ok = true;
  if (tid == 0) {
    tc5::mbar_expect_tx(bar_tma, 16384 + 32768);
    tc5::bulk_g2s(sm + kFwdW1, w1p, 16384, bar_tma);
    tc5::bulk_g2s(sm + kFwdW2, w2p, 32768, bar_tma);
  }
  ok = tc5::mbar_wait(bar_tma, tma_phase, kWaitLimit);
  ok = __syncthreads_and(ok);
  tma_phase ^= 1;
  constexpr uint32_t id1 = tc5::idesc_bf16(128, 128);
  for (long long t = blockIdx.x; ok && t < ntiles; t += gridDim.x) {
    if (tid == 0) {
      tc5::mbar_expect_tx(bar_tma, kXTileBytes);
      tc5::bulk_g2s(sm + kFwdXs, xa + t * kXTileBytes, kXTileBytes, bar_tma);
    }
    ok = __syncthreads_and(tc5::mbar_wait(bar_tma, tma_phase, kWaitLimit));
    tma_phase ^= 1;
    if (!ok) break;
    if (tid == 0) {
      tc5::fence_after_sync();
      const uint32_t xs = tc5::smem_u32(sm + kFwdXs), w1 = tc5::smem_u32(sm + kFwdW1);
#pragma unroll
      for (int kk = 0; kk < kFeat / 16; kk++)
        tc5::mma_bf16(tmem, tc5::desc_kmajor(xs + kk * 256, kFeat), tc5::desc_kmajor(w1 + kk * 256, kFeat),
                      id1, kk > 0);
      tc5::mma_commit(bar_mma);
    }
    ok = __syncthreads_and(tc5::mbar_wait(bar_mma, mma_phase, kWaitLimit));
    mma_phase ^= 1;
    if (!ok) break;
    tc5::fence_after_sync();
    const uint32_t row = tid;
#pragma unroll 1
    for (int c0 = 0; c0 < kHid; c0 += 32) {
      float v[32];
      tc5::tmem_ld32(tmem + lane_base + c0, v);
#pragma unroll
      for (int i = 0; i < 32; i++) st_bf16(sm + kFwdH1, tc5::tile_offset(row, c0 + i, kHid), silu(v[i] + b1[c0 + i]));
    }
    tc5::fence_async_smem();
    tc5::fence_before_sync();
    __syncthreads();
    if (tid == 0) {
      tc5::fence_after_sync();
      const uint32_t h1 = tc5::smem_u32(sm + kFwdH1), w2 = tc5::smem_u32(sm + kFwdW2);
#pragma unroll
      for (int kk = 0; kk < kHid / 16; kk++)
        tc5::mma_bf16(tmem + 128, tc5::desc_kmajor(h1 + kk * 256, kHid), tc5::desc_kmajor(w2 + kk * 256, kHid),
                      id1, kk > 0);
      tc5::mma_commit(bar_mma);
    }
    ok = __syncthreads_and(tc5::mbar_wait(bar_mma, mma_phase, kWaitLimit));
    mma_phase ^= 1;
    if (!ok) break;
    tc5::fence_after_sync();
    float acc = b3;
#pragma unroll 1
    for (int c0 = 0; c0 < kHid; c0 += 32) {
      float v[32];
      tc5::tmem_ld32(tmem + lane_base + 128 + c0, v);
#pragma unroll
      for (int i = 0; i < 32; i++) acc += silu(v[i] + b2[c0 + i]) * w3[c0 + i];
    }
    if (t * kTile + row < n_rows) y[t * kTile + row] = acc;
    tc5::fence_before_sync();
    __syncthreads();
  }
  if (!ok && tid == 0) atomicOr(status, kStatusTimeoutBit);
  tc5::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc5::fence_after_sync();
    tc5::tmem_dealloc(tmem, 256);
  }
}

// shared-memory map of the training kernel
constexpr uint32_t kTrXs = 0, kTrXt = 16384, kTrW1 = 32768, kTrW2 = 49152, kTrW2t = 81920,
                   kTrA = 114688, kTrB = 147456, kTrC = 180224, kTrF = 212992;  // floats after
constexpr uint32_t kTrB1 = kTrF, kTrB2 = kTrB1 + 512, kTrW3 = kTrB2 + 512, kTrDb1 = kTrW3 + 512,
                   kTrDb2 = kTrDb1 + 512, kTrDw3 = kTrDb2 + 512, kTrRed = kTrDw3 + 512,
                   kTrBar = kTrRed + 64, kTrSmem = kTrBar + 64;

// Forward + backward of the tiles tiles[blockIdx.x * per_cta ...]; per-CTA partial gradients
// (and sum of squared residuals) into partial[blockIdx.x][kPartial].  TMEM columns: Z1 [0,128),
// Z2 / dH1 [128,256), dW2 [256,384), dW1^T [384,448).
__global__ void __launch_bounds__(128, 1)
    mlp_train_kernel(const uint8_t *__restrict__ xa, const uint8_t *__restrict__ xt,
                     const float *__restrict__ tgt, const float *__restrict__ mask,
                     const int *__restrict__ tiles, int per_cta, const uint8_t *__restrict__ w1p,
                     const uint8_t *__restrict__ w2p, const uint8_t *__restrict__ w2tp,
                     const float *__restrict__ params, float inv_count, float *__restrict__ partial,
                     int *status) {
  extern __shared__ __align__(1024) uint8_t sm[];
  float *b1 = reinterpret_cast<float *>(sm + kTrB1);
  float *b2 = reinterpret_cast<float *>(sm + kTrB2);
  float *w3 = reinterpret_cast<float *>(sm + kTrW3);
  float *db1 = reinterpret_cast<float *>(sm + kTrDb1);
  float *db2 = reinterpret_cast<float *>(sm + kTrDb2);
  float *dw3 = reinterpret_cast<float *>(sm + kTrDw3);
  float *red = reinterpret_cast<float *>(sm + kTrRed);
  uint64_t *bar_tma = reinterpret_cast<uint64_t *>(sm + kTrBar);
  uint64_t *bar_mma = bar_tma + 1;
  uint32_t *slot = reinterpret_cast<uint32_t *>(bar_tma + 2);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    tc5::mbar_init(bar_tma, 1);
    tc5::mbar_init(bar_mma, 1);
    tc5::fence_async_smem();
  }
  if (warp == 0) tc5::tmem_alloc(slot, 512);
  b1[tid] = params[ob1 + tid];
  b2[tid] = params[ob2 + tid];
  w3[tid] = bf16_round(params[ow3 + tid]);
  db1[tid] = db2[tid] = dw3[tid] = 0.f;
  const float b3 = params[ob3];
  tc5::fence_before_sync();
  __syncthreads();
  tc5::fence_after_sync();
  const uint32_t tmem = *slot;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  uint32_t tma_phase = 0, mma_phase = 0;
  if (tid == 0) {
    tc5::mbar_expect_tx(bar_tma, 16384 + 32768 + 32768);
    tc5::bulk_g2s(sm + kTrW1, w1p, 16384, bar_tma);
    tc5::bulk_g2s(sm + kTrW2, w2p, 32768, bar_tma);
    tc5::bulk_g2s(sm + kTrW2t, w2tp, 32768, bar_tma);
  }
  bool ok = __syncthreads_and(tc5::mbar_wait(bar_tma, tma_phase, kWaitLimit));
  tma_phase ^= 1;
  float loss = 0.f, db3 = 0.f;
  constexpr uint32_t id128 = tc5::idesc_bf16(128, 128), id64 = tc5::idesc_bf16(128, 64);
  const uint32_t sXs = tc5::smem_u32(sm + kTrXs), sXt = tc5::smem_u32(sm + kTrXt),
                 sW1 = tc5::smem_u32(sm + kTrW1), sW2 = tc5::smem_u32(sm + kTrW2),
                 sW2t = tc5::smem_u32(sm + kTrW2t), sA = tc5::smem_u32(sm + kTrA),
                 sB = tc5::smem_u32(sm + kTrB), sC = tc5::smem_u32(sm + kTrC);
  const uint32_t row = tid;
  for (int it = 0; ok && it < per_cta; it++) {
    const long long t = tiles[(long long)blockIdx.x * per_cta + it];
    if (tid == 0) {
      tc5::mbar_expect_tx(bar_tma, 2 * kXTileBytes);
      tc5::bulk_g2s(sm + kTrXs, xa + t * kXTileBytes, kXTileBytes, bar_tma);
      tc5::bulk_g2s(sm + kTrXt, xt + t * kXTileBytes, kXTileBytes, bar_tma);
    }
    const float target = tgt[t * kTile + row], m = mask[t * kTile + row];
    ok = __syncthreads_and(tc5::mbar_wait(bar_tma, tma_phase, kWaitLimit));
    tma_phase ^= 1;
    if (!ok) break;
    // GEMM1: Z1 = X W1
    if (tid == 0) {
      tc5::fence_after_sync();
#pragma unroll
      for (int kk = 0; kk < kFeat / 16; kk++)
        tc5::mma_bf16(tmem, tc5::desc_kmajor(sXs + kk * 256, kFeat), tc5::desc_kmajor(sW1 + kk * 256, kFeat),
                      id128, kk > 0);
      tc5::mma_commit(bar_mma);
    }
    ok = __syncthreads_and(tc5::mbar_wait(bar_mma, mma_phase, kWaitLimit));
    mma_phase ^= 1;
    if (!ok) break;
    tc5::fence_after_sync();
    // epilogue 1: H1 = SiLU(Z1 + b1) -> A copy (rows, K = hid) and transposed copy (hid, K = rows)
#pragma unroll 1
    for (int c0 = 0; c0 < kHid; c0 += 32) {
      float v[32];
      tc5::tmem_ld32(tmem + lane_base + c0, v);
#pragma unroll
      for (int i = 0; i < 32; i++) {
        const float h = silu(v[i] + b1[c0 + i]);
        st_bf16(sm + kTrA, tc5::tile_offset(row, c0 + i, kHid), h);
        st_bf16(sm + kTrB, tc5::tile_offset(c0 + i, row, kTile), h);
      }
    }
    tc5::fence_async_smem();
    tc5::fence_before_sync();
    __syncthreads();
    // GEMM2: Z2 = H1 W2
    if (tid == 0) {
      tc5::fence_after_sync();
#pragma unroll
      for (int kk = 0; kk < kHid / 16; kk++)
        tc5::mma_bf16(tmem + 128, tc5::desc_kmajor(sA + kk * 256, kHid), tc5::desc_kmajor(sW2 + kk * 256, kHid),
                      id128, kk > 0);
      tc5::mma_commit(bar_mma);
    }
    ok = __syncthreads_and(tc5::mbar_wait(bar_mma, mma_phase, kWaitLimit));
    mma_phase ^= 1;
    if (!ok) break;
    tc5::fence_after_sync();
    // epilogue 2: y, residual, dz2 = dy w3 SiLU'(Z2 + b2); dw3, db2 partial sums
    float y = b3;
#pragma unroll 1
    for (int c0 = 0; c0 < kHid; c0 += 32) {
      float v[32];
      tc5::tmem_ld32(tmem + lane_base + 128 + c0, v);
#pragma unroll
      for (int i = 0; i < 32; i++) y += silu(v[i] + b2[c0 + i]) * w3[c0 + i];
    }
    const float r = (y - target) * m;
    loss += r * r;
    const float dy = 2.0f * r * inv_count;
    db3 += dy;
#pragma unroll 1
    for (int c0 = 0; c0 < kHid; c0 += 32) {
      float v[32], g3[32], g2[32];
      tc5::tmem_ld32(tmem + lane_base + 128 + c0, v);
#pragma unroll
      for (int i = 0; i < 32; i++) {
        const float z = v[i] + b2[c0 + i];
        g3[i] = dy * silu(z);
        const float dz = dy * w3[c0 + i] * dsilu(z);
        g2[i] = dz;
        st_bf16(sm + kTrA, tc5::tile_offset(row, c0 + i, kHid), dz);
        st_bf16(sm + kTrC, tc5::tile_offset(c0 + i, row, kTile), dz);
      }
      const float s3 = transpose_reduce(g3);
      const float s2 = transpose_reduce(g2);
      atomicAdd(&dw3[c0 + lane], s3);
      atomicAdd(&db2[c0 + lane], s2);
    }
    tc5::fence_async_smem();
    tc5::fence_before_sync();
    __syncthreads();
    // GEMM3: dH1 = dZ2 W2^T (into the Z2 columns); GEMM4: dW2 += H1^T dZ2
    if (tid == 0) {
      tc5::fence_after_sync();
#pragma unroll
      for (int kk = 0; kk < kHid / 16; kk++)
        tc5::mma_bf16(tmem + 128, tc5::desc_kmajor(sA + kk * 256, kHid), tc5::desc_kmajor(sW2t + kk * 256, kHid),
                      id128, kk > 0);
#pragma unroll
      for (int kk = 0; kk < kTile / 16; kk++)
        tc5::mma_bf16(tmem + 256, tc5::desc_kmajor(sB + kk * 256, kTile), tc5::desc_kmajor(sC + kk * 256, kTile),
                      id128, (it > 0 || kk > 0) ? 1u : 0u);
      tc5::mma_commit(bar_mma);
    }
    ok = __syncthreads_and(tc5::mbar_wait(bar_mma, mma_phase, kWaitLimit));
    mma_phase ^= 1;
    if (!ok) break;
    tc5::fence_after_sync();
    // epilogue 3: dz1 = dH1 SiLU'(Z1 + b1) -> transposed copy (hid, K = rows); db1
#pragma unroll 1
    for (int c0 = 0; c0 < kHid; c0 += 32) {
      float dh[32], z[32];
      tc5::tmem_ld32(tmem + lane_base + 128 + c0, dh);
      tc5::tmem_ld32(tmem + lane_base + c0, z);
#pragma unroll
      for (int i = 0; i < 32; i++) {
        const float dz = dh[i] * dsilu(z[i] + b1[c0 + i]);
        dh[i] = dz;
        st_bf16(sm + kTrB, tc5::tile_offset(c0 + i, row, kTile), dz);
      }
      const float s1 = transpose_reduce(dh);
      atomicAdd(&db1[c0 + lane], s1);
    }
    tc5::fence_async_smem();
    tc5::fence_before_sync();
    __syncthreads();
    // GEMM5: dW1^T += dZ1^T X
    if (tid == 0) {
      tc5::fence_after_sync();
#pragma unroll
      for (int kk = 0; kk < kTile / 16; kk++)
        tc5::mma_bf16(tmem + 384, tc5::desc_kmajor(sB + kk * 256, kTile), tc5::desc_kmajor(sXt + kk * 256, kTile),
                      id64, (it > 0 || kk > 0) ? 1u : 0u);
      tc5::mma_commit(bar_mma);
    }
    ok = __syncthreads_and(tc5::mbar_wait(bar_mma, mma_phase, kWaitLimit));
    mma_phase ^= 1;
    tc5::fence_after_sync();
  }
  float *out = partial + (size_t)blockIdx.x * kPartial;
  if (ok && per_cta > 0) {
    // dW2[in = lane row][out = column]; dW1[in = column][hid = lane row]
#pragma unroll 1
    for (int c0 = 0; c0 < kHid; c0 += 32) {
      float v[32];
      tc5::tmem_ld32(tmem + lane_base + 256 + c0, v);
#pragma unroll
      for (int i = 0; i < 32; i++) out[oW2 + row * kHid + c0 + i] = v[i];
    }
#pragma unroll 1
    for (int c0 = 0; c0 < kFeat; c0 += 32) {
      float v[32];
      tc5::tmem_ld32(tmem + lane_base + 384 + c0, v);
#pragma unroll
      for (int i = 0; i < 32; i++) out[oW1 + (c0 + i) * kHid + row] = v[i];
    }
  }
  // loss and db3: block sums
  float l = loss, d = db3;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    l += __shfl_xor_sync(0xffffffffu, l, o);
    d += __shfl_xor_sync(0xffffffffu, d, o);
  }
  if (lane == 0) {
    red[warp] = l;
    red[4 + warp] = d;
  }
  tc5::fence_before_sync();
  __syncthreads();
  if (ok && per_cta > 0) {
    out[ob1 + tid] = db1[tid];
    out[ob2 + tid] = db2[tid];
    out[ow3 + tid] = dw3[tid];
    if (tid == 0) {
      out[ob3] = red[4] + red[5] + red[6] + red[7];
      out[kParams] = red[0] + red[1] + red[2] + red[3];
    }
  } else if (per_cta > 0) {
    for (int e = tid; e < kPartial; e += blockDim.x) out[e] = 0.f;
    if (tid == 0) atomicOr(status, kStatusTimeoutBit);
  }
  if (warp == 0) {
    tc5::fence_after_sync();
    tc5::tmem_dealloc(tmem, 512);
  }
}

// grad[p] = sum over CTAs of partial[cta][p] (fixed order); grad[kParams] = loss sum.
__global__ void reduce_partials_kernel(const float *__restrict__ partial, int G, float *__restrict__ grad) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < kPartial; p += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int b = 0; b < G; b++) s += partial[(size_t)b * kPartial + p];
    grad[p] = s;
  }
}

__global__ void adam_kernel(float *__restrict__ p, float *__restrict__ m, float *__restrict__ v,
                            const float *__restrict__ g, float lr, float c1, float c2) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < kParams; e += gridDim.x * blockDim.x) {
    const float gi = g[e];
    const float mi = b1 * m[e] + (1.f - b1) * gi;
    const float vi = b2 * v[e] + (1.f - b2) * gi * gi;
    m[e] = mi;
    v[e] = vi;
    p[e] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  }
}

// rho = rho0 + (y * t_std + t_mean)
__global__ void correction_kernel(const double *__restrict__ rho0, const float *__restrict__ y, double t_mean,
                                  double t_std, long long n, double *__restrict__ rho) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    rho[i] = rho0[i] + ((double)y[i] * t_std + t_mean);
}

// targets: t = (rho_out - rho0) as FP32
__global__ void target_kernel(const double *__restrict__ rho_out, const double *__restrict__ rho0, long long n,
                              float *__restrict__ t) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    t[i] = (float)(rho_out[i] - rho0[i]);
}

// standardised targets and row masks of the packed set
__global__ void pack_targets_kernel(const float *__restrict__ t, long long n, long long n_pad, float mean,
                                    float inv_std, float *__restrict__ tp, float *__restrict__ mask) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_pad; i += (long long)gridDim.x * blockDim.x) {
    tp[i] = i < n ? (t[i] - mean) * inv_std : 0.f;
    mask[i] = i < n ? 1.f : 0.f;
  }
}

void ck_launch(const char *what) { ck(cudaGetLastError(), what); }

int grid_of(long long n, int block = 256) {
  return (int)std::max<long long>(1, std::min<long long>(8192, (n + block - 1) / block));
}

}  // namespace
}  // namespace sq

using namespace sq;

struct sq_mlp {
  int device = 0;
  int num_sms = 0;
  float *d_params = nullptr, *d_m = nullptr, *d_v = nullptr, *d_grad = nullptr, *d_partial = nullptr;
  uint8_t *d_w1p = nullptr, *d_w2p = nullptr, *d_w2tp = nullptr;
  float *d_mean = nullptr, *d_istd = nullptr;
  int *d_status = nullptr, *d_tiles = nullptr;
  int tiles_cap = 0;
  // standardisation
  float mean[kFeat], inv_std[kFeat];
  double t_mean = 0.0, t_std = 1.0;
  bool standardised = false;
  // training set: raw features and targets (device)
  float *d_raw = nullptr, *d_tgt_raw = nullptr;
  long long n_samples = 0, cap = 0;
  // packed training tiles
  uint8_t *d_xa = nullptr, *d_xt = nullptr;
  float *d_t = nullptr, *d_mask = nullptr;
  long long ntiles = 0, packed_samples = -1;
  long long adam_step = 0;
  int partial_rows = 0;
  std::mt19937_64 rng{12345};

  ~sq_mlp() {
    for (float **p : {&d_params, &d_m, &d_v, &d_grad, &d_partial, &d_mean, &d_istd, &d_raw, &d_tgt_raw, &d_t,
                      &d_mask})
      dev_free(*p);
    for (uint8_t **p : {&d_w1p, &d_w2p, &d_w2tp, &d_xa, &d_xt}) dev_free(*p);
    dev_free(d_status);
    dev_free(d_tiles);
  }
};

namespace {

void mlp_alloc(sq_mlp *m) {
  ck(cudaSetDevice(m->device), "cudaSetDevice");
  ck(cudaDeviceGetAttribute(&m->num_sms, cudaDevAttrMultiProcessorCount, m->device), "sm count");
  dev_alloc(&m->d_params, sizeof(float) * kParams, "mlp params");
  dev_alloc(&m->d_m, sizeof(float) * kParams, "adam m");
  dev_alloc(&m->d_v, sizeof(float) * kParams, "adam v");
  dev_alloc(&m->d_grad, sizeof(float) * kPartial, "grad");
  dev_alloc(&m->d_w1p, 16384, "w1 packed");
  dev_alloc(&m->d_w2p, 32768, "w2 packed");
  dev_alloc(&m->d_w2tp, 32768, "w2t packed");
  dev_alloc(&m->d_mean, sizeof(float) * kFeat, "mean");
  dev_alloc(&m->d_istd, sizeof(float) * kFeat, "istd");
  dev_alloc(&m->d_status, sizeof(int) * 2, "status");
  ck(cudaMemset(m->d_m, 0, sizeof(float) * kParams), "memset");
  ck(cudaMemset(m->d_v, 0, sizeof(float) * kParams), "memset");
  ck(cudaMemset(m->d_status, 0, sizeof(int) * 2), "memset");
  for (int f = 0; f < kFeat; f++) {
    m->mean[f] = 0.f;
    m->inv_std[f] = 1.f;
  }
  ck(cudaFuncSetAttribute(mlp_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFwdSmem),
     "forward smem");
  ck(cudaFuncSetAttribute(mlp_train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrSmem),
     "train smem");
}

void upload_standardisation(sq_mlp *m) {
  ck(cudaMemcpy(m->d_mean, m->mean, sizeof(m->mean), cudaMemcpyHostToDevice), "mean H2D");
  ck(cudaMemcpy(m->d_istd, m->inv_std, sizeof(m->inv_std), cudaMemcpyHostToDevice), "istd H2D");
}

void pack_weights(sq_mlp *m, cudaStream_t s) {
  pack_weights_kernel<<<96, 256, 0, s>>>(m->d_params, m->d_w1p, m->d_w2p, m->d_w2tp);
  ck_launch("pack weights");
}

sq_status mlp_status(sq_mlp *m) {
  int st = 0;
  ck(cudaMemcpy(&st, m->d_status, sizeof(int), cudaMemcpyDeviceToHost), "status D2H");
  if (st) {
    ck(cudaMemset(m->d_status, 0, sizeof(int)), "status reset");
    return fail(SQ_DEVICE_TIMEOUT, "a tensor-core wait of the MLP kernels gave up");
  }
  return SQ_OK;
}

// Atom images within R_CUT of the cell (positions of the grid frame, FP32).
std::vector<float4> neighbour_images(const Deck &d) {
  std::vector<float4> img;
  double L[3];
  for (int a = 0; a < 3; a++) L[a] = 2.0 * d.cell_half[a];
  int rep[3];
  for (int a = 0; a < 3; a++) rep[a] = (int)std::ceil(kRcut / L[a]) + 1;
  for (size_t n = 0; n < d.atom_type.size(); n++)
    for (int P = -rep[0]; P <= rep[0]; P++)
      for (int Q = -rep[1]; Q <= rep[1]; Q++)
        for (int R = -rep[2]; R <= rep[2]; R++) {
          const double x = d.atom_xyz[3 * n] + P * L[0], y = d.atom_xyz[3 * n + 1] + Q * L[1],
                       z = d.atom_xyz[3 * n + 2] + R * L[2];
          const double p[3] = {x, y, z};
          bool near = true;
          for (int a = 0; a < 3; a++)
            if (p[a] < -d.cell_half[a] - kRcut - 1.0 || p[a] > d.cell_half[a] + kRcut + 1.0) near = false;
          if (near) img.push_back(make_float4((float)x, (float)y, (float)z, 0.f));
        }
  return img;
}

// raw descriptors of the handle's cell into d_out [n_nodes][64] (device)
void compute_descriptors(sq_handle *h, float *d_out, cudaStream_t s) {
  const Deck &d = h->deck;
  std::vector<float4> img = neighbour_images(d);
  DevBuf<float4> buf(sizeof(float4) * std::max<size_t>(1, img.size()), "images");
  float4 *d_img = buf.get();
  ck(cudaMemcpyAsync(d_img, img.data(), sizeof(float4) * img.size(), cudaMemcpyHostToDevice, s), "images H2D");
  const long long n = h->info.n_nodes;
  descriptor_kernel<<<grid_of(n * 32, 256), 256, 0, s>>>(
      d_img, (int)img.size(), d.grid[0], d.grid[1], (float)h->setup.h[0], (float)h->setup.h[1],
      (float)h->setup.h[2], (float)d.cell_half[0], (float)d.cell_half[1], (float)d.cell_half[2], n, d_out);
  ck_launch("descriptors");
  ck(cudaStreamSynchronize(s), "sync");
}

// standardisation from the stored raw samples (means and standard deviations per feature)
void fit_standardisation(sq_mlp *m) {
  const long long n = m->n_samples;
  std::vector<float> raw((size_t)n * kFeat), t(n);
  ck(cudaMemcpy(raw.data(), m->d_raw, sizeof(float) * raw.size(), cudaMemcpyDeviceToHost), "raw D2H");
  ck(cudaMemcpy(t.data(), m->d_tgt_raw, sizeof(float) * n, cudaMemcpyDeviceToHost), "t D2H");
  for (int f = 0; f < kFeat; f++) {
    double s = 0, s2 = 0;
    for (long long i = 0; i < n; i++) {
      const double v = raw[(size_t)i * kFeat + f];
      s += v;
      s2 += v * v;
    }
    const double mu = s / n, var = std::max(0.0, s2 / n - mu * mu);
    m->mean[f] = (float)mu;
    m->inv_std[f] = (float)(var > 1e-12 ? 1.0 / std::sqrt(var) : 1.0);
  }
  double s = 0, s2 = 0;
  for (long long i = 0; i < n; i++) {
    s += t[i];
    s2 += (double)t[i] * t[i];
  }
  m->t_mean = s / n;
  const double var = std::max(0.0, s2 / n - m->t_mean * m->t_mean);
  m->t_std = var > 1e-30 ? std::sqrt(var) : 1.0;
  m->standardised = true;
  upload_standardisation(m);
}

void pack_training_set(sq_mlp *m, cudaStream_t s) {
  if (m->packed_samples == m->n_samples) return;
  const long long n = m->n_samples, nt = (n + kTile - 1) / kTile, np = nt * kTile;
  dev_free(m->d_xa);
  dev_free(m->d_xt);
  dev_free(m->d_t);
  dev_free(m->d_mask);
  dev_alloc(&m->d_xa, (size_t)nt * kXTileBytes, "train xa");
  dev_alloc(&m->d_xt, (size_t)nt * kXTileBytes, "train xt");
  dev_alloc(&m->d_t, sizeof(float) * np, "train t");
  dev_alloc(&m->d_mask, sizeof(float) * np, "train mask");
  pack_features_kernel<<<grid_of(np * kFeat), 256, 0, s>>>(m->d_raw, n, np, m->d_mean, m->d_istd, m->d_xa, m->d_xt);
  ck_launch("pack features");
  pack_targets_kernel<<<grid_of(np), 256, 0, s>>>(m->d_tgt_raw, n, np, (float)m->t_mean,
                                                  (float)(1.0 / m->t_std), m->d_t, m->d_mask);
  ck_launch("pack targets");
  m->ntiles = nt;
  m->packed_samples = n;
}

// Packed samples a training kernel reads: feature tiles in both layouts, targets, row masks.
struct TileSet {
  const uint8_t *xa, *xt;
  const float *t, *mask;
};

// One forward+backward over the given tiles (host list) of `set`; gradients into d_grad.
void run_train_kernel(sq_mlp *m, const TileSet &set, const std::vector<int> &tiles, int per_cta,
                      float inv_count, cudaStream_t s) {
  const int G = (int)(tiles.size() / per_cta);
  if ((int)tiles.size() > m->tiles_cap) {
    dev_free(m->d_tiles);
    dev_alloc(&m->d_tiles, sizeof(int) * tiles.size(), "tiles");
    m->tiles_cap = (int)tiles.size();
  }
  if (G > m->partial_rows) {
    dev_free(m->d_partial);
    dev_alloc(&m->d_partial, sizeof(float) * (size_t)G * kPartial, "partials");
    m->partial_rows = G;
  }
  ck(cudaMemcpyAsync(m->d_tiles, tiles.data(), sizeof(int) * tiles.size(), cudaMemcpyHostToDevice, s), "tiles H2D");
  mlp_train_kernel<<<G, 128, kTrSmem, s>>>(set.xa, set.xt, set.t, set.mask, m->d_tiles, per_cta, m->d_w1p,
                                           m->d_w2p, m->d_w2tp, m->d_params, inv_count, m->d_partial,
                                           m->d_status);
  ck_launch("mlp train");
  reduce_partials_kernel<<<(kPartial + 255) / 256, 256, 0, s>>>(m->d_partial, G, m->d_grad);
  ck_launch("reduce partials");
}

// network output for every node of the handle's cell -> d_y (n_nodes floats)
void predict_y(sq_mlp *m, sq_handle *h, float *d_y, cudaStream_t s) {
  const long long n = h->info.n_nodes, nt = (n + kTile - 1) / kTile, np = nt * kTile;
  DevBuf<float> raw(sizeof(float) * (size_t)n * kFeat, "descriptors");
  DevBuf<uint8_t> xa(sizeof(uint8_t) * (size_t)nt * kXTileBytes, "tiles");
  float *d_raw = raw.get();
  uint8_t *d_xa = xa.get();
  compute_descriptors(h, d_raw, s);
  pack_features_kernel<<<grid_of(np * kFeat), 256, 0, s>>>(d_raw, n, np, m->d_mean, m->d_istd, d_xa, nullptr);
  ck_launch("pack features");
  pack_weights(m, s);
  const int grid = (int)std::min<long long>(nt, 2LL * m->num_sms);
  mlp_forward_kernel<<<grid, 128, kFwdSmem, s>>>(d_xa, nt, n, m->d_w1p, m->d_w2p, m->d_params, d_y, m->d_status);
  ck_launch("mlp forward");
  ck(cudaStreamSynchronize(s), "sync");
}

}  // namespace

extern "C" {

sq_status sq_mlp_create(int device, unsigned long long seed, sq_mlp **out) {
  if (!out) return fail(SQ_BAD_INPUT, "null argument");
  *out = nullptr;
  sq_mlp *m = new sq_mlp();
  sq_status st = guarded([&] {
    m->device = device;
    mlp_alloc(m);
    // He-style initialisation (normal, std sqrt(2 / fan_in)), zero biases, small output layer
    std::mt19937_64 g(seed);
    std::normal_distribution<float> nd(0.f, 1.f);
    std::vector<float> p(kParams, 0.f);
    for (int e = 0; e < kFeat * kHid; e++) p[oW1 + e] = nd(g) * std::sqrt(2.f / kFeat);
    for (int e = 0; e < kHid * kHid; e++) p[oW2 + e] = nd(g) * std::sqrt(2.f / kHid);
    for (int e = 0; e < kHid; e++) p[ow3 + e] = nd(g) * std::sqrt(1.f / kHid);
    ck(cudaMemcpy(m->d_params, p.data(), sizeof(float) * kParams, cudaMemcpyHostToDevice), "params H2D");
    upload_standardisation(m);
    m->rng.seed(seed ^ 0x9e3779b97f4a7c15ULL);
    return SQ_OK;
  });
  if (st != SQ_OK) {
    delete m;
    return st;
  }
  *out = m;
  return SQ_OK;
}

void sq_mlp_destroy(sq_mlp *m) { delete m; }

sq_status sq_mlp_set_params(sq_mlp *m, const float *params, const float *feat_mean, const float *feat_inv_std,
                            double t_mean, double t_std) {
  if (!m || !params) return fail(SQ_BAD_INPUT, "null argument");
  return guarded([&] {
    ck(cudaSetDevice(m->device), "cudaSetDevice");
    ck(cudaMemcpy(m->d_params, params, sizeof(float) * kParams, cudaMemcpyHostToDevice), "params H2D");
    if (feat_mean && feat_inv_std) {
      std::memcpy(m->mean, feat_mean, sizeof(m->mean));
      std::memcpy(m->inv_std, feat_inv_std, sizeof(m->inv_std));
      m->standardised = true;
      upload_standardisation(m);
    }
    m->t_mean = t_mean;
    m->t_std = t_std;
    m->packed_samples = -1;
    return SQ_OK;
  });
}

sq_status sq_mlp_get_params(const sq_mlp *m, float *params, float *feat_mean, float *feat_inv_std, double *t_mean,
                            double *t_std) {
  if (!m) return fail(SQ_BAD_INPUT, "null argument");
  return guarded([&] {
    ck(cudaSetDevice(m->device), "cudaSetDevice");
    if (params) ck(cudaMemcpy(params, m->d_params, sizeof(float) * kParams, cudaMemcpyDeviceToHost), "params D2H");
    if (feat_mean) std::memcpy(feat_mean, m->mean, sizeof(m->mean));
    if (feat_inv_std) std::memcpy(feat_inv_std, m->inv_std, sizeof(m->inv_std));
    if (t_mean) *t_mean = m->t_mean;
    if (t_std) *t_std = m->t_std;
    return SQ_OK;
  });
}

sq_status sq_mlp_save(const sq_mlp *m, const char *path) {
  if (!m || !path) return fail(SQ_BAD_INPUT, "null argument");
  return guarded([&] {
    std::vector<float> p(kParams);
    ck(cudaSetDevice(m->device), "cudaSetDevice");
    ck(cudaMemcpy(p.data(), m->d_params, sizeof(float) * kParams, cudaMemcpyDeviceToHost), "params D2H");
    FILE *f = std::fopen(path, "wb");
    if (!f) return fail(SQ_BAD_INPUT, std::string("cannot write ") + path);
    const char magic[8] = {'S', 'Q', 'M', 'L', 'P', '0', '0', '1'};
    const int dims[4] = {kFeat, kHid, kHid, 1};
    bool ok = std::fwrite(magic, 1, 8, f) == 8 && std::fwrite(dims, sizeof(int), 4, f) == 4 &&
              std::fwrite(m->mean, sizeof(float), kFeat, f) == (size_t)kFeat &&
              std::fwrite(m->inv_std, sizeof(float), kFeat, f) == (size_t)kFeat &&
              std::fwrite(&m->t_mean, sizeof(double), 1, f) == 1 && std::fwrite(&m->t_std, sizeof(double), 1, f) == 1 &&
              std::fwrite(p.data(), sizeof(float), kParams, f) == (size_t)kParams;
    std::fclose(f);
    return ok ? SQ_OK : fail(SQ_BAD_INPUT, std::string("write error on ") + path);
  });
}

sq_status sq_mlp_load(const char *path, int device, sq_mlp **out) {
  if (!path || !out) return fail(SQ_BAD_INPUT, "null argument");
  *out = nullptr;
  FILE *f = std::fopen(path, "rb");
  if (!f) return fail(SQ_BAD_INPUT, std::string("cannot read ") + path);
  char magic[8];
  int dims[4];
  float mean[kFeat], istd[kFeat];
  double tm, ts;
  std::vector<float> p(kParams);
  bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "SQMLP001", 8) == 0 &&
            std::fread(dims, sizeof(int), 4, f) == 4 && dims[0] == kFeat && dims[1] == kHid && dims[2] == kHid &&
            dims[3] == 1 && std::fread(mean, sizeof(float), kFeat, f) == (size_t)kFeat &&
            std::fread(istd, sizeof(float), kFeat, f) == (size_t)kFeat && std::fread(&tm, sizeof(double), 1, f) == 1 &&
            std::fread(&ts, sizeof(double), 1, f) == 1 && std::fread(p.data(), sizeof(float), kParams, f) == (size_t)kParams;
  std::fclose(f);
  if (!ok) return fail(SQ_BAD_INPUT, std::string("not a 64-128-128-1 model file: ") + path);
  sq_mlp *m = nullptr;
  sq_status st = sq_mlp_create(device, 1, &m);
  if (st != SQ_OK) return st;
  st = sq_mlp_set_params(m, p.data(), mean, istd, tm, ts);
  if (st != SQ_OK) {
    delete m;
    return st;
  }
  *out = m;
  return SQ_OK;
}

sq_status sq_descriptors(sq_handle *h, float *desc) {
  if (!h || !desc) return fail(SQ_BAD_INPUT, "null argument");
  return guarded([&] {
    ck(cudaSetDevice(h->opt.device), "cudaSetDevice");
    const long long n = h->info.n_nodes;
    DevBuf<float> d(sizeof(float) * (size_t)n * kFeat, "descriptors");
    compute_descriptors(h, d.get(), h->own_stream);
    ck(cudaMemcpy(desc, d.get(), sizeof(float) * (size_t)n * kFeat, cudaMemcpyDeviceToHost), "descriptors D2H");
    return SQ_OK;
  });
}

sq_status sq_mlp_add_training_cell(sq_mlp *m, sq_handle *h) {
  if (!m || !h) return fail(SQ_BAD_INPUT, "null argument");
  if (!h->scf) return fail(SQ_BAD_INPUT, "run an SCF on the handle first");
  if (h->opt.device != m->device) return fail(SQ_BAD_INPUT, "model and engine on different devices");
  return guarded([&] {
    ck(cudaSetDevice(m->device), "cudaSetDevice");
    cudaStream_t s = h->own_stream;
    const long long n = h->info.n_nodes, need = m->n_samples + n;
    if (need > m->cap) {
      const long long cap = std::max(need, 2 * m->cap);
      float *raw = nullptr, *t = nullptr;
      dev_alloc(&raw, sizeof(float) * (size_t)cap * kFeat, "training features");
      dev_alloc(&t, sizeof(float) * (size_t)cap, "training targets");
      if (m->n_samples) {
        ck(cudaMemcpy(raw, m->d_raw, sizeof(float) * (size_t)m->n_samples * kFeat, cudaMemcpyDeviceToDevice), "copy");
        ck(cudaMemcpy(t, m->d_tgt_raw, sizeof(float) * (size_t)m->n_samples, cudaMemcpyDeviceToDevice), "copy");
      }
      dev_free(m->d_raw);
      dev_free(m->d_tgt_raw);
      m->d_raw = raw;
      m->d_tgt_raw = t;
      m->cap = cap;
    }
    compute_descriptors(h, m->d_raw + (size_t)m->n_samples * kFeat, s);
    target_kernel<<<grid_of(n), 256, 0, s>>>(scf_rho_out_device(h), scf_rho0_device(h), n,
                                             m->d_tgt_raw + m->n_samples);
    ck_launch("targets");
    ck(cudaStreamSynchronize(s), "sync");
    m->n_samples = need;
    return SQ_OK;
  });
}

sq_status sq_mlp_train(sq_mlp *m, int steps, int tiles_per_step, double lr, double *final_loss) {
  if (!m || steps < 0 || tiles_per_step <= 0) return fail(SQ_BAD_INPUT, "bad argument");
  if (m->n_samples == 0) return fail(SQ_BAD_INPUT, "no training samples");
  return guarded([&] {
    ck(cudaSetDevice(m->device), "cudaSetDevice");
    cudaStream_t s = 0;
    if (!m->standardised) fit_standardisation(m);
    pack_training_set(m, s);
    // tiles_per_step tiles per step over at most one CTA per SM
    const int G = std::min(tiles_per_step, m->num_sms);
    const int per_cta = (tiles_per_step + G - 1) / G;
    std::vector<int> tiles((size_t)G * per_cta);
    std::uniform_int_distribution<long long> pick(0, m->ntiles - 1);
    const float inv_count = 1.0f / (float)(G * per_cta * kTile);
    double loss = 0.0;
    for (int it = 0; it < steps; it++) {
      for (int &t : tiles) t = (int)pick(m->rng);
      pack_weights(m, s);
      run_train_kernel(m, TileSet{m->d_xa, m->d_xt, m->d_t, m->d_mask}, tiles, per_cta, inv_count, s);
      m->adam_step++;
      const double c1 = 1.0 / (1.0 - std::pow(0.9, (double)m->adam_step));
      const double c2 = 1.0 / (1.0 - std::pow(0.999, (double)m->adam_step));
      adam_kernel<<<(kParams + 255) / 256, 256, 0, s>>>(m->d_params, m->d_m, m->d_v, m->d_grad, (float)lr,
                                                        (float)c1, (float)c2);
      ck_launch("adam");
      if (it == steps - 1) {
        float lsum = 0.f;
        ck(cudaMemcpyAsync(&lsum, m->d_grad + kParams, sizeof(float), cudaMemcpyDeviceToHost, s), "loss D2H");
        ck(cudaStreamSynchronize(s), "sync");
        loss = lsum * inv_count;
      }
    }
    ck(cudaStreamSynchronize(s), "sync");
    sq_status st = mlp_status(m);
    if (st != SQ_OK) return st;
    if (final_loss) *final_loss = loss;
    return SQ_OK;
  });
}

sq_status sq_mlp_gradients(sq_mlp *m, const float *x, const float *t, long n, double *loss, float *grads) {
  if (!m || !x || !t || n <= 0 || !grads) return fail(SQ_BAD_INPUT, "bad argument");
  return guarded([&] {
    ck(cudaSetDevice(m->device), "cudaSetDevice");
    cudaStream_t s = 0;
    const long long nt = (n + kTile - 1) / kTile, np = nt * kTile;
    DevBuf<float> x_d(sizeof(float) * (size_t)n * kFeat, "x"), t_d(sizeof(float) * n, "t"),
        tp_d(sizeof(float) * np, "t"), mask_d(sizeof(float) * np, "mask"),
        zero_d(sizeof(float) * kFeat, "zero"), one_d(sizeof(float) * kFeat, "one");
    DevBuf<uint8_t> xa_d((size_t)nt * kXTileBytes, "xa"), xt_d((size_t)nt * kXTileBytes, "xt");
    std::vector<float> z(kFeat, 0.f), o(kFeat, 1.f);
    ck(cudaMemcpy(zero_d.get(), z.data(), sizeof(float) * kFeat, cudaMemcpyHostToDevice), "H2D");
    ck(cudaMemcpy(one_d.get(), o.data(), sizeof(float) * kFeat, cudaMemcpyHostToDevice), "H2D");
    ck(cudaMemcpy(x_d.get(), x, sizeof(float) * (size_t)n * kFeat, cudaMemcpyHostToDevice), "x H2D");
    ck(cudaMemcpy(t_d.get(), t, sizeof(float) * n, cudaMemcpyHostToDevice), "t H2D");
    pack_features_kernel<<<grid_of(np * kFeat), 256, 0, s>>>(x_d.get(), n, np, zero_d.get(), one_d.get(),
                                                             xa_d.get(), xt_d.get());
    pack_targets_kernel<<<grid_of(np), 256, 0, s>>>(t_d.get(), n, np, 0.f, 1.f, tp_d.get(), mask_d.get());
    ck_launch("pack");
    // every tile once, one tile per CTA
    std::vector<int> tiles((size_t)nt);
    for (long long i = 0; i < nt; i++) tiles[i] = (int)i;
    pack_weights(m, s);
    run_train_kernel(m, TileSet{xa_d.get(), xt_d.get(), tp_d.get(), mask_d.get()}, tiles, 1,
                     1.0f / (float)n, s);
    std::vector<float> g(kPartial);
    ck(cudaMemcpy(g.data(), m->d_grad, sizeof(float) * kPartial, cudaMemcpyDeviceToHost), "grad D2H");
    sq_status st = mlp_status(m);
    if (st != SQ_OK) return st;
    std::memcpy(grads, g.data(), sizeof(float) * kParams);
    if (loss) *loss = g[kParams] / (double)n;
    return SQ_OK;
  });
}

sq_status sq_mlp_forward(sq_mlp *m, const float *x, long n, float *y) {
  if (!m || !x || !y || n <= 0) return fail(SQ_BAD_INPUT, "bad argument");
  return guarded([&] {
    ck(cudaSetDevice(m->device), "cudaSetDevice");
    cudaStream_t s = 0;
    const long long nt = (n + kTile - 1) / kTile, np = nt * kTile;
    DevBuf<float> x_d(sizeof(float) * (size_t)n * kFeat, "x"), y_d(sizeof(float) * n, "y"),
        zero_d(sizeof(float) * kFeat, "zero"), one_d(sizeof(float) * kFeat, "one");
    DevBuf<uint8_t> xa_d((size_t)nt * kXTileBytes, "xa");
    std::vector<float> z(kFeat, 0.f), o(kFeat, 1.f);
    ck(cudaMemcpy(zero_d.get(), z.data(), sizeof(float) * kFeat, cudaMemcpyHostToDevice), "H2D");
    ck(cudaMemcpy(one_d.get(), o.data(), sizeof(float) * kFeat, cudaMemcpyHostToDevice), "H2D");
    ck(cudaMemcpy(x_d.get(), x, sizeof(float) * (size_t)n * kFeat, cudaMemcpyHostToDevice), "x H2D");
    pack_features_kernel<<<grid_of(np * kFeat), 256, 0, s>>>(x_d.get(), n, np, zero_d.get(), one_d.get(),
                                                             xa_d.get(), nullptr);
    ck_launch("pack");
    pack_weights(m, s);
    const int grid = (int)std::min<long long>(nt, 2LL * m->num_sms);
    mlp_forward_kernel<<<grid, 128, kFwdSmem, s>>>(xa_d.get(), nt, n, m->d_w1p, m->d_w2p, m->d_params,
                                                   y_d.get(), m->d_status);
    ck_launch("mlp forward");
    ck(cudaMemcpy(y, y_d.get(), sizeof(float) * n, cudaMemcpyDeviceToHost), "y D2H");
    return mlp_status(m);
  });
}

sq_status sq_mlp_predict_density(sq_mlp *m, sq_handle *h, double *rho) {
  if (!m || !h || !rho) return fail(SQ_BAD_INPUT, "null argument");
  return guarded([&] {
    ck(cudaSetDevice(h->opt.device), "cudaSetDevice");
    const long long n = h->info.n_nodes;
    DevBuf<float> y_d(sizeof(float) * n, "y");
    DevBuf<double> rho_d(sizeof(double) * n, "rho");
    predict_y(m, h, y_d.get(), h->own_stream);
    correction_kernel<<<grid_of(n), 256, 0, h->own_stream>>>(scf_rho0_device(h), y_d.get(), m->t_mean,
                                                             m->t_std, n, rho_d.get());
    ck_launch("correction");
    ck(cudaMemcpyAsync(rho, rho_d.get(), sizeof(double) * n, cudaMemcpyDeviceToHost, h->own_stream), "rho D2H");
    ck(cudaStreamSynchronize(h->own_stream), "sync");
    return mlp_status(m);
  });
}

sq_status sq_scf_begin_learned(sq_handle *h, const sq_scf_options *opt, sq_mlp *m) {
  if (!h || !m) return fail(SQ_BAD_INPUT, "null argument");
  return guarded([&] {
    ck(cudaSetDevice(h->opt.device), "cudaSetDevice");
    const long long n = h->info.n_nodes;
    DevBuf<float> y_d(sizeof(float) * n, "y");
    DevBuf<double> rho_d(sizeof(double) * n, "rho");
    predict_y(m, h, y_d.get(), h->own_stream);
    correction_kernel<<<grid_of(n), 256, 0, h->own_stream>>>(scf_rho0_device(h), y_d.get(), m->t_mean,
                                                             m->t_std, n, rho_d.get());
    ck_launch("correction");
    sq_status st = mlp_status(m);
    if (st == SQ_OK) {
      scf_begin_device_density(h, opt, rho_d.get());  // copies rho; synchronises
      if (opt && opt->learned_highpass > 0.0) scf_highpass_start(h, opt->learned_highpass);
    }
    return st;
  });
}

}  // extern "C"

// lanczos.cu -- batched per-node Lanczos on the truncated-cube Hamiltonian (sm_103a).
//
// Replaces the hot loop of NodesAndWeights_LSSGQ / CalculateSpectralNodesAndWeights
// (src/lsdft_scf.cc:60-150): for every FD node, n_qp Lanczos steps from the unit vector at
// the cube centre on H = -1/2 Lap (12th-order FD, Dirichlet cube, src/lsdft_initObjs.cc:393-475)
// + diag(Veff) + the Kleinman-Bylander projectors of the atom images that meet the cube
// (src/lsdft_matvec.cc:25-149).
//
// Layout.  A persistent CTA owns one node at a time and keeps both Lanczos vectors on chip:
//   P  the stencil source, FP32/FP64, rows padded by 6 zeros in x (pitch = nx + 6) so the
//      x-neighbours of a row need no bounds checks;
//   U  the elementwise vector (v_{k-1}, then the new residual), unpadded; in shared memory
//      when both fit, else in a per-CTA slice of global scratch.
// A warp owns one y-row of the cube and walks z with a 13-value register window, so each
// output costs 12 x-loads + 12 y-loads + 1 z-load from shared memory.
// The nonlocal term uses per-node image lists built on chip: one warp per atom gathers
// c_lm = <chi_lm, v> with lane-strided loads and a shuffle reduction, then one warp per image
// scatters chi_lm alpha_lm back with shared-memory atomics.  chi_lm is rebuilt on the fly as
// T_l(r) * P_lm(x,y,z) from the per-atom radial tables (L2 resident).
//
// Recurrence (reference scf.cc:119-147, same quantities, fused passes):
//   P = b_{k-1} v_k (unnormalised), U = v_{k-1};
//   pass 1:  h = H P / b_{k-1};  a_k = <v_k, h>;  U <- h - b_{k-1} U
//   pass 2:  w = U - a_k v_k;    b_k = ||w||;     P <- w;  U <- v_k
// a_k and b_k are accumulated per thread in the vector precision and summed across the CTA
// in FP64.
#include <cuda_runtime.h>

#include <cstdint>

#include "sq_internal.hpp"
#include "sq_kernels.hpp"

namespace sq {

namespace {

constexpr int O = kStencilHalf;
constexpr int W = 2 * O + 1;

template <typename T> struct Coef;
template <> struct Coef<float> {
  static __device__ __forceinline__ float x(const LanczosParams &p, int d) { return p.cxf[d]; }
  static __device__ __forceinline__ float y(const LanczosParams &p, int d) { return p.cyf[d]; }
  static __device__ __forceinline__ float z(const LanczosParams &p, int d) { return p.czf[d]; }
  static __device__ __forceinline__ float diag(const LanczosParams &p) { return p.cdiagf; }
};
template <> struct Coef<double> {
  static __device__ __forceinline__ double x(const LanczosParams &p, int d) { return p.cx[d]; }
  static __device__ __forceinline__ double y(const LanczosParams &p, int d) { return p.cy[d]; }
  static __device__ __forceinline__ double z(const LanczosParams &p, int d) { return p.cz[d]; }
  static __device__ __forceinline__ double diag(const LanczosParams &p) { return p.cdiag; }
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
template <typename T> __device__ __forceinline__ T warp_sum_t(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum of one double per thread over the CTA; `red` holds NW+1 doubles.  Contains two barriers.
template <int NW> __device__ __forceinline__ double block_sum(double v, double *red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_sum(v);
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    double t = lane < NW ? red[lane] : 0.0;
    t = warp_sum(t);
    if (lane == 0) red[NW] = t;
  }
  __syncthreads();
  return red[NW];
}

// Real solid harmonics r^l Y_lm with the reference's constants (src/lsdft_tools.cc:165-187),
// slot index l*l + l + m.  For l = 0 the constant is folded into the table.
// FN(slot, value) is called for every (l,m) of channel l.
template <typename T, typename FN>
__device__ __forceinline__ void solid_harmonics(int l, T x, T y, T z, FN &&fn) {
  if (l == 0) {
    fn(0, T(1));
  } else if (l == 1) {
    const T c = T(0.488602511902920);
    fn(1, c * y);
    fn(2, c * z);
    fn(3, c * x);
  } else if (l == 2) {
    fn(4, T(1.092548430592079) * (x * y));
    fn(5, T(1.092548430592079) * (y * z));
    fn(6, T(0.315391565252520) * (-x * x - y * y + T(2) * z * z));
    fn(7, T(1.092548430592079) * (z * x));
    fn(8, T(0.546274215296040) * (x * x - y * y));
  } else {
    fn(9, T(0.590043589926644) * (T(3) * x * x - y * y) * y);
    fn(10, T(2.890611442640554) * (x * y * z));
    fn(11, T(0.457045799464466) * y * (T(4) * z * z - x * x - y * y));
    fn(12, T(0.373176332590115) * z * (T(2) * z * z - T(3) * x * x - T(3) * y * y));
    fn(13, T(0.457045799464466) * x * (T(4) * z * z - x * x - y * y));
    fn(14, T(1.445305721320277) * z * (x * x - y * y));
    fn(15, T(0.590043589926644) * x * (x * x - T(3) * y * y));
  }
}

// Decode point t of an ex*ey*ez box (x fastest) without integer division.
__device__ __forceinline__ void box_point(int t, int ex, int ey, float inv_ex, float inv_ey,
                                          int &lx, int &ly, int &lz) {
  int row = __float2int_rz((float(t) + 0.5f) * inv_ex);
  lx = t - row * ex;
  lz = __float2int_rz((float(row) + 0.5f) * inv_ey);
  ly = row - lz * ey;
}

struct Isect {
  int x0, y0, z0, ex, ey, ez;  // intersection start (global) and extents
};

__device__ __forceinline__ Isect intersect(const ImageMeta &m, const TypeDesc &td, int Xs, int Ys,
                                           int Zs, int nx, int ny, int nz) {
  Isect s;
  s.x0 = max(m.bx, Xs);
  s.y0 = max(m.by, Ys);
  s.z0 = max(m.bz, Zs);
  s.ex = min(m.bx + td.fx, Xs + nx) - s.x0;
  s.ey = min(m.by + td.fy, Ys + ny) - s.y0;
  s.ez = min(m.bz + td.fz, Zs + nz) - s.z0;
  return s;
}

template <typename T, bool FAITHFUL, bool U_SMEM, int BLOCK>
__global__ void __launch_bounds__(BLOCK, 1)
    lanczos_kernel(const __grid_constant__ LanczosParams p, const T *__restrict__ veff_ext,
                   const ImageMeta *__restrict__ images, const T *__restrict__ tables,
                   T *__restrict__ u_global, double *__restrict__ ab_out, int *__restrict__ status) {
  constexpr int NW = BLOCK / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nx = p.nx, ny = p.ny, nz = p.nz, pitch = p.pitch;
  const int PS = ny * pitch;       // P plane stride
  const int US = ny * nx;          // U plane stride
  const int nc = nz * ny * nx;
  const int psize = ((O + nz * PS) + 3) & ~3;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *P = reinterpret_cast<T *>(smem_raw);
  T *U;
  unsigned char *cur = smem_raw + sizeof(T) * psize;
  if constexpr (U_SMEM) {
    U = reinterpret_cast<T *>(cur);
    cur += sizeof(T) * ((nc + 3) & ~3);
  } else {
    U = u_global + (size_t)blockIdx.x * (size_t)((nc + 3) & ~3);
  }
  double *red = reinterpret_cast<double *>(cur);       // 2 x (NW+1)
  cur += sizeof(double) * 2 * (NW + 1);
  double *sab = reinterpret_cast<double *>(cur);       // a[64], b[64]
  cur += sizeof(double) * 128;
  T *alpha = reinterpret_cast<T *>(cur);
  cur += sizeof(T) * p.max_img * p.alpha_stride;
  int *list = reinterpret_cast<int *>(cur);
  cur += sizeof(int) * p.max_img;
  int *slot = reinterpret_cast<int *>(cur);
  cur += sizeof(int) * p.max_img;
  int *gstart = reinterpret_cast<int *>(cur);
  cur += sizeof(int) * (p.max_img + 1);
  int *cnt = reinterpret_cast<int *>(cur);             // [0] images, [1] groups, [2] overflow

  const int x = lane;
  const bool xin = x < nx;
  const int xc = xin ? x : nx - 1;

  for (long long node = p.node_begin + blockIdx.x; node < p.node_end; node += gridDim.x) {
    const int I = (int)(node % p.Nx);
    const int J = (int)((node / p.Nx) % p.Ny);
    const int K = (int)(node / ((long long)p.Nx * p.Ny));
    const int Xs = I - p.nhx, Ys = J - p.nhy, Zs = K - p.nhz;

    // ---- per-node image list (warp 0) while the other warps clear the vectors ----
    if (warp == 0) {
      int count = 0;
      for (int base = 0; base < p.n_images; base += 32) {
        const int i = base + lane;
        bool ok = false;
        if (i < p.n_images) {
          const int4 b = *reinterpret_cast<const int4 *>(&images[i]);
          const TypeDesc &td = p.types[b.w];
          ok = b.x <= Xs + nx - 1 && b.x + td.fx - 1 >= Xs && b.y <= Ys + ny - 1 &&
               b.y + td.fy - 1 >= Ys && b.z <= Zs + nz - 1 && b.z + td.fz - 1 >= Zs;
        }
        const unsigned m = __ballot_sync(0xffffffffu, ok);
        const int pos = count + __popc(m & ((1u << lane) - 1u));
        if (ok && pos < p.max_img) list[pos] = i;
        count += __popc(m);
      }
      const int n = min(count, p.max_img);
      int groups = 0;
      for (int base = 0; base < n; base += 32) {
        const int k = base + lane;
        bool start = false;
        if (k < n) start = (k == 0) || images[list[k]].atom != images[list[k - 1]].atom;
        const unsigned m = __ballot_sync(0xffffffffu, start);
        const int g = groups + __popc(m & ((1u << lane) - 1u)) + (start ? 0 : -1);
        if (k < n) {
          slot[k] = g;
          if (start) gstart[g] = k;
        }
        groups += __popc(m);
      }
      if (lane == 0) {
        gstart[groups] = n;
        cnt[0] = n;
        cnt[1] = groups;
        cnt[2] = count > p.max_img;
      }
    } else {
      for (int e = threadIdx.x - 32; e < psize; e += BLOCK - 32) P[e] = T(0);
      for (int e = threadIdx.x - 32; e < nc; e += BLOCK - 32) U[e] = T(0);
    }
    __syncthreads();
    const int n_img = cnt[0], n_grp = cnt[1];
    if (cnt[2]) {  // capacity exceeded: report and leave NaN coefficients for this node
      if (threadIdx.x == 0) atomicOr(status, kStatusCapacity);
      for (int j = threadIdx.x; j < 2 * p.nqp; j += BLOCK)
        ab_out[(node - p.node_begin) * 2 * p.nqp + j] = __longlong_as_double(0x7ff8000000000000ll);
      __syncthreads();
      continue;
    }
    if (threadIdx.x == 0) P[O + ((nz - 1) / 2 * ny + (ny - 1) / 2) * pitch + (nx - 1) / 2] = T(1);
    __syncthreads();

    double beta = 1.0;
    bool broke = false;
    for (int j = 0; j < p.nqp; j++) {
      const T inv = T(1.0 / beta);
      const T tbeta = T(beta);
      double anl = 0.0;  // <v_k, V_nl v_k>, lane 0 of each warp

      // ---- nonlocal gather: one warp per atom (all its images in the cube) ----
      for (int g = warp; g < n_grp; g += NW) {
        T acc[kMaxLm];
#pragma unroll
        for (int s = 0; s < kMaxLm; s++) acc[s] = T(0);
        T acc_s = T(0);
        int type = 0;
        for (int k = gstart[g]; k < gstart[g + 1]; k++) {
          const ImageMeta m = images[list[k]];
          type = m.type;
          const TypeDesc &td = p.types[m.type];
          const Isect q = intersect(m, td, Xs, Ys, Zs, nx, ny, nz);
          const int npts = q.ex * q.ey * q.ez;
          const float iex = 1.0f / q.ex, iey = 1.0f / q.ey;
          const int fvol = td.fx * td.fy * td.fz;
          const T ox = T(m.ox), oy = T(m.oy), oz = T(m.oz);
          const T hx = T(p.hx), hy = T(p.hy), hz = T(p.hz);
          T gam[4];
#pragma unroll
          for (int l = 0; l < 4; l++) gam[l] = T(td.gamma[l]);
          for (int t = lane; t < npts; t += 32) {
            int lx, ly, lz;
            box_point(t, q.ex, q.ey, iex, iey, lx, ly, lz);
            const int gx = q.x0 + lx, gy = q.y0 + ly, gz = q.z0 + lz;
            const int tx = gx - m.bx, ty = gy - m.by, tz = gz - m.bz;
            const T v = P[O + ((gz - Zs) * ny + (gy - Ys)) * pitch + (gx - Xs)];
            const T dx = ox + hx * T(tx), dy = oy + hy * T(ty), dz = oz + hz * T(tz);
            const T *tb = tables + m.tab_base + (tz * td.fy + ty) * td.fx + tx;
#pragma unroll
            for (int l = 0; l < 4; l++) {
              if (!(td.chan_mask & (1 << l))) continue;
              const T tv = tb[td.chan_off[l] * fvol] * v;
              if constexpr (FAITHFUL) {
                const T gl = gam[l];
                solid_harmonics<T>(l, dx, dy, dz, [&](int s, T ylm) {
                  acc[0] += gl * ylm * tv;
                  acc_s += ylm * tv;
                });
              } else {
                solid_harmonics<T>(l, dx, dy, dz, [&](int s, T ylm) { acc[s] += ylm * tv; });
              }
            }
          }
        }
        const TypeDesc &td = p.types[type];
        if constexpr (FAITHFUL) {
          const double cg = (double)warp_sum_t(acc[0]) * (double)inv;
          const double cs = (double)warp_sum_t(acc_s) * (double)inv;
          if (lane == 0) {
            alpha[g * p.alpha_stride] = T(cg);
            anl += cs * cg;
          }
        } else {
#pragma unroll
          for (int s = 0; s < kMaxLm; s++) {
            const int l = s < 1 ? 0 : (s < 4 ? 1 : (s < 9 ? 2 : 3));
            if (!(p.union_mask & (1 << l))) continue;
            const double c = (double)warp_sum_t(acc[s]) * (double)inv;
            if (lane == 0) {
              const double gl = (td.chan_mask & (1 << l)) ? td.gamma[l] : 0.0;
              alpha[g * p.alpha_stride + p.lm_rank[s]] = T(gl * c);
              anl += gl * c * c;
            }
          }
        }
      }
      __syncthreads();

      // ---- pass 1: stencil + Veff, U <- H v_k - b_{k-1} U, a_k partial ----
      T a_acc = T(0);
      for (int y = warp; y < ny; y += NW) {
        const int rowP = O + y * pitch + xc;
        const int rowU = y * nx + xc;
        const T *vrow = veff_ext + ((size_t)K * p.EY + (J + y)) * p.EX + (I + xc);
        const size_t VS = (size_t)p.EY * p.EX;
        T win[W];
#pragma unroll
        for (int q = -O; q < O; q++) win[q + O] = (q >= 0 && q < nz) ? P[rowP + min(q, nz - 1) * PS] : T(0);
        for (int z0 = 0; z0 < nz; z0 += W) {
#pragma unroll
          for (int s = 0; s < W; s++) {
            const int z = z0 + s;
            if (z >= nz) break;
            const int qn = z + O;
            win[(s + 2 * O) % W] = (qn < nz) ? P[rowP + min(qn, nz - 1) * PS] : T(0);
            const int i = rowP + z * PS;
            const T vc = win[(s + O) % W];
            T h = (Coef<T>::diag(p) + vrow[z * VS]) * vc;
#pragma unroll
            for (int d = 1; d <= O; d++) {
              h += Coef<T>::z(p, d) * (win[(s + O - d + W) % W] + win[(s + O + d) % W]);
              h += Coef<T>::x(p, d) * (P[i - d] + P[i + d]);
              const T ym = P[y - d >= 0 ? i - d * pitch : i];
              const T yp = P[y + d < ny ? i + d * pitch : i];
              h += Coef<T>::y(p, d) * ((y - d >= 0 ? ym : T(0)) + (y + d < ny ? yp : T(0)));
            }
            h *= inv;
            if (xin) {
              const int u = rowU + z * US;
              a_acc += (vc * inv) * h;
              U[u] = h - tbeta * U[u];
            }
          }
        }
      }
      __syncthreads();

      // ---- nonlocal scatter: one warp per image, U += sum_lm chi_lm alpha_lm ----
      for (int k = warp; k < n_img; k += NW) {
        const ImageMeta m = images[list[k]];
        const TypeDesc &td = p.types[m.type];
        const Isect q = intersect(m, td, Xs, Ys, Zs, nx, ny, nz);
        const int npts = q.ex * q.ey * q.ez;
        const float iex = 1.0f / q.ex, iey = 1.0f / q.ey;
        const int fvol = td.fx * td.fy * td.fz;
        const T *al = alpha + slot[k] * p.alpha_stride;
        const T ox = T(m.ox), oy = T(m.oy), oz = T(m.oz);
        const T hx = T(p.hx), hy = T(p.hy), hz = T(p.hz);
        for (int t = lane; t < npts; t += 32) {
          int lx, ly, lz;
          box_point(t, q.ex, q.ey, iex, iey, lx, ly, lz);
          const int gx = q.x0 + lx, gy = q.y0 + ly, gz = q.z0 + lz;
          const int tx = gx - m.bx, ty = gy - m.by, tz = gz - m.bz;
          const T dx = ox + hx * T(tx), dy = oy + hy * T(ty), dz = oz + hz * T(tz);
          const T *tb = tables + m.tab_base + (tz * td.fy + ty) * td.fx + tx;
          T val = T(0);
#pragma unroll
          for (int l = 0; l < 4; l++) {
            if (!(td.chan_mask & (1 << l))) continue;
            const T tv = tb[td.chan_off[l] * fvol];
            T sum = T(0);
            if constexpr (FAITHFUL) {
              solid_harmonics<T>(l, dx, dy, dz, [&](int s, T ylm) { sum += ylm; });
              val += tv * sum * al[0];
            } else {
              solid_harmonics<T>(l, dx, dy, dz, [&](int s, T ylm) { sum += ylm * al[p.lm_rank[s]]; });
              val += tv * sum;
            }
          }
          atomicAdd(&U[((gz - Zs) * ny + (gy - Ys)) * nx + (gx - Xs)], val);
        }
      }
      const double a = block_sum<NW>((double)a_acc + (lane == 0 ? anl : 0.0), red);

      // ---- pass 2: w = U - a_k v_k, P <- w, U <- v_k, b_k = ||w|| ----
      const T ta = T(a);
      T b_acc = T(0);
      for (int y = warp; y < ny; y += NW) {
        const int rowP = O + y * pitch + xc;
        const int rowU = y * nx + xc;
        if (xin) {
          for (int z = 0; z < nz; z++) {
            const T pv = P[rowP + z * PS];
            const T vk = pv * inv;
            const T w = U[rowU + z * US] - ta * vk;
            P[rowP + z * PS] = w;
            U[rowU + z * US] = vk;
            b_acc += w * w;
          }
        }
      }
      const double b2 = block_sum<NW>((double)b_acc, red + NW + 1);
      const double b = sqrt(b2);
      if (threadIdx.x == 0) {
        sab[j] = a;
        sab[64 + j] = b;
      }
      if (!(b > 0.0) || !isfinite(b)) {  // breakdown: the Krylov space is invariant
        broke = true;
        if (threadIdx.x == 0) {
          atomicOr(status, kStatusBreakdown);
          for (int r = j + 1; r < p.nqp; r++) {
            sab[r] = 0.0;
            sab[64 + r] = 0.0;
          }
        }
        break;
      }
      beta = b;
    }
    (void)broke;
    __syncthreads();
    for (int r = threadIdx.x; r < p.nqp; r += BLOCK) {
      double *o = ab_out + (node - p.node_begin) * 2 * p.nqp;
      o[r] = sab[r];
      o[p.nqp + r] = sab[64 + r];
    }
    __syncthreads();
  }
}

template <typename T>
__global__ void veff_extend_kernel(const double *__restrict__ veff, double vconst,
                                   T *__restrict__ ext, int Nx, int Ny, int Nz, int nhx, int nhy,
                                   int nhz, int EX, int EY, int EZ) {
  const long long total = (long long)EX * EY * EZ;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int ex = (int)(e % EX), ey = (int)((e / EX) % EY), ez = (int)(e / ((long long)EX * EY));
    const int gx = ((ex - nhx) % Nx + Nx) % Nx;
    const int gy = ((ey - nhy) % Ny + Ny) % Ny;
    const int gz = ((ez - nhz) % Nz + Nz) % Nz;
    ext[e] = T(veff ? veff[((long long)gz * Ny + gy) * Nx + gx] : vconst);
  }
}

}  // namespace

size_t lanczos_smem_bytes(const LanczosParams &p, int elem_size, bool u_smem, int block) {
  const int nw = block / 32;
  const size_t psize = (size_t)((O + p.nz * p.ny * p.pitch) + 3) & ~size_t(3);
  const size_t nc = (size_t)p.nx * p.ny * p.nz;
  size_t b = elem_size * psize;
  if (u_smem) b += elem_size * ((nc + 3) & ~size_t(3));
  b += sizeof(double) * 2 * (nw + 1) + sizeof(double) * 128;
  b += (size_t)elem_size * p.max_img * p.alpha_stride;
  b += sizeof(int) * (3 * (size_t)p.max_img + 1) + sizeof(int) * 4;
  return b;
}

template <typename T, bool FAITHFUL, bool U_SMEM, int BLOCK>
static cudaError_t launch_one(const LanczosParams &p, int grid, size_t smem, cudaStream_t s,
                              const void *veff_ext, const ImageMeta *images, const void *tables,
                              void *u_scratch, double *ab, int *status) {
  auto k = lanczos_kernel<T, FAITHFUL, U_SMEM, BLOCK>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k<<<grid, BLOCK, smem, s>>>(p, (const T *)veff_ext, images, (const T *)tables, (T *)u_scratch,
                              ab, status);
  return cudaGetLastError();
}

cudaError_t launch_lanczos(const LanczosParams &p, int precision, bool faithful, bool u_smem,
                           int grid, size_t smem, cudaStream_t s, const void *veff_ext,
                           const ImageMeta *images, const void *tables, void *u_scratch,
                           double *ab, int *status) {
  if (precision == 32) {
    if (faithful)
      return u_smem ? launch_one<float, true, true, kBlockF32>(p, grid, smem, s, veff_ext, images, tables, u_scratch, ab, status)
                    : launch_one<float, true, false, kBlockF32>(p, grid, smem, s, veff_ext, images, tables, u_scratch, ab, status);
    return u_smem ? launch_one<float, false, true, kBlockF32>(p, grid, smem, s, veff_ext, images, tables, u_scratch, ab, status)
                  : launch_one<float, false, false, kBlockF32>(p, grid, smem, s, veff_ext, images, tables, u_scratch, ab, status);
  }
  if (faithful)
    return launch_one<double, true, false, kBlockF64>(p, grid, smem, s, veff_ext, images, tables, u_scratch, ab, status);
  return launch_one<double, false, false, kBlockF64>(p, grid, smem, s, veff_ext, images, tables, u_scratch, ab, status);
}

cudaError_t launch_veff_extend(const double *veff, double vconst, void *ext, int precision,
                               const LanczosParams &p, cudaStream_t s) {
  const long long total = (long long)p.EX * p.EY * p.EZ;
  const int block = 256;
  const int grid = (int)std::min<long long>((total + block - 1) / block, 152LL * 16);
  if (precision == 32)
    veff_extend_kernel<float><<<grid, block, 0, s>>>(veff, vconst, (float *)ext, p.Nx, p.Ny, p.Nz,
                                                     p.nhx, p.nhy, p.nhz, p.EX, p.EY, p.EZ);
  else
    veff_extend_kernel<double><<<grid, block, 0, s>>>(veff, vconst, (double *)ext, p.Nx, p.Ny, p.Nz,
                                                      p.nhx, p.nhy, p.nhz, p.EX, p.EY, p.EZ);
  return cudaGetLastError();
}

}  // namespace sq

// lanczos_kernel.cuh -- the batched per-node Lanczos kernel (template, sm_103a).
//
// Replaces the hot loop of NodesAndWeights_LSSGQ / CalculateSpectralNodesAndWeights
// (src/lsdft_scf.cc:60-150): for every FD node, n_qp Lanczos steps from the unit vector at
// the cube centre on H = -1/2 Lap (12th-order FD, Dirichlet cube, src/lsdft_initObjs.cc:393-475)
// + diag(Veff) + the Kleinman-Bylander projectors of the atom images that meet the cube
// (src/lsdft_matvec.cc:25-149).
//
// Layout.  A persistent CTA (one per SM) owns one node at a time and keeps both Lanczos
// vectors on chip:
//   P  the stencil source, with 6 zero columns between rows (x; FP64 cubes too large for
//      them drop the columns and bounds-check x instead) and, in FP32, 6 zero rows
//      between consecutive z-planes and before the first (y): row -d of a plane is a zero
//      row of the gap before it, row ny-1+d one of the gap after it, so no neighbour load
//      needs a bounds check;
//   U  the elementwise vector (v_{k-1}, then the new residual); in shared memory when both
//      fit, else in a per-CTA slice of global scratch.
// Vector passes (FP32): a half-warp owns one y-row and a z-range; each lane computes the x
// pair (x, x+1) from 64-bit shared loads, forming neighbour sums with Blackwell's packed
// add.rn.f32x2, and walks z with a 13-plane register ring, so one output costs ~10 shared
// loads.  Cubes wider than 32 points (WIDE) give each thread one (row, x pair) over all of
// z instead, consecutive threads on consecutive pairs.  FP64 uses one warp per row with
// scalar loads.
// Nonlocal term: when a node starts, its projector matrix restricted to the cube (support
// points only) is written once to a per-CTA list in global scratch: per point the packed
// P/U indices and chi_lm (chi_lm = T_l(r) P_lm(x,y,z), from the per-atom radial tables and
// the real solid harmonics).  Every Lanczos step then streams that list twice, cut into
// equal per-warp ranges: the gather accumulates c_lm = <chi_lm, P> per lane and adds the
// shuffle-reduced sums into the atom's slot with shared atomics when a range leaves an
// image; the scatter adds sum_lm chi_lm alpha_lm into U with shared atomics.  Compact lists
// (kLayoutCompact) store T_l(r) per channel and the point's box coordinates instead, and the
// stream rebuilds chi_lm and the P/U indices from per-image data kept in shared memory.
//
// Recurrence (reference scf.cc:119-147, same quantities, fused passes):
//   P = b_{k-1} v_k (unnormalised), U = v_{k-1};
//   pass 1:  h = H P / b_{k-1};  a_k = <v_k, h>;  U <- h - b_{k-1} U
//   pass 2:  w = U - a_k v_k;    b_k = ||w||;     P <- w;  U <- v_k
// a_k and b_k are accumulated per thread in the vector precision and summed across the CTA
// in FP64.
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

#include "sq_internal.hpp"
#include "sq_kernels.hpp"

namespace sq {
namespace lk {

constexpr int O = kStencilHalf;
constexpr int W = 2 * O + 1;
constexpr int kMaxWarps = 32;

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

// (l,m) bookkeeping of a channel mask (bit l = nonlocal channel l), slot s = l*l + l + m.
template <int MASK> struct Lm {
  static constexpr int nlm = ((MASK & 1) ? 1 : 0) + ((MASK & 2) ? 3 : 0) + ((MASK & 4) ? 5 : 0) +
                             ((MASK & 8) ? 7 : 0);
  static __host__ __device__ constexpr int l_of(int s) { return s < 1 ? 0 : (s < 4 ? 1 : (s < 9 ? 2 : 3)); }
  static __host__ __device__ constexpr int rank(int s) {
    int base = 0;
    for (int q = 0; q < l_of(s); q++)
      if (MASK & (1 << q)) base += 2 * q + 1;
    return base + (s - l_of(s) * l_of(s));
  }
};

template <typename T> __device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum of one double per thread over the CTA (nw warps); red holds kMaxWarps+1 doubles.
__device__ __forceinline__ double block_sum(double v, double *red, int nw) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_sum(v);
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    double t = lane < nw ? red[lane] : 0.0;
    t = warp_sum(t);
    if (lane == 0) red[kMaxWarps] = t;
  }
  __syncthreads();
  return red[kMaxWarps];
}

// Real solid harmonics r^l Y_lm with the reference's constants (src/lsdft_tools.cc:165-187);
// FN(slot, value) for every m of channel l.  For l = 0 the constant is folded into the table.
template <int L, typename T, typename FN>
__device__ __forceinline__ void solid_harmonics(T x, T y, T z, FN &&fn) {
  if constexpr (L == 0) {
    fn(0, T(1));
  } else if constexpr (L == 1) {
    const T c = T(0.488602511902920);
    fn(1, c * y);
    fn(2, c * z);
    fn(3, c * x);
  } else if constexpr (L == 2) {
    fn(4, T(1.092548430592079) * (x * y));
    fn(5, T(1.092548430592079) * (y * z));
    fn(6, T(0.315391565252520) * (T(2) * z * z - x * x - y * y));
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

// Blackwell packed FP32: two adds in one instruction (PTX add.rn.f32x2, sm_100+).
__device__ __forceinline__ float2 add2(float2 a, float2 b) {
  unsigned long long ra = *reinterpret_cast<unsigned long long *>(&a);
  unsigned long long rb = *reinterpret_cast<unsigned long long *>(&b);
  unsigned long long rd;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(rd) : "l"(ra), "l"(rb));
  return *reinterpret_cast<float2 *>(&rd);
}
__device__ __forceinline__ void fma2s(float2 &h, float c, float2 s) {
  h.x = fmaf(c, s.x, h.x);
  h.y = fmaf(c, s.y, h.y);
}

template <typename T> __device__ __forceinline__ T hx_of(const LanczosParams &p);
template <> __device__ __forceinline__ float hx_of<float>(const LanczosParams &p) { return p.hxf; }
template <> __device__ __forceinline__ double hx_of<double>(const LanczosParams &p) { return p.hx; }
template <typename T> __device__ __forceinline__ T hy_of(const LanczosParams &p);
template <> __device__ __forceinline__ float hy_of<float>(const LanczosParams &p) { return p.hyf; }
template <> __device__ __forceinline__ double hy_of<double>(const LanczosParams &p) { return p.hy; }
template <typename T> __device__ __forceinline__ T hz_of(const LanczosParams &p);
template <> __device__ __forceinline__ float hz_of<float>(const LanczosParams &p) { return p.hzf; }
template <> __device__ __forceinline__ double hz_of<double>(const LanczosParams &p) { return p.hz; }

template <typename T> __device__ __forceinline__ T support_r2(const TypeDesc &td);
template <> __device__ __forceinline__ float support_r2<float>(const TypeDesc &td) { return td.support_r2_f32; }
template <> __device__ __forceinline__ double support_r2<double>(const TypeDesc &td) { return td.support_r2_f64; }

// One record of the per-node projector list: N values of T (chi_lm, or for the reference's
// shared-slot operator sum_lm Gamma_l chi_lm and sum_lm chi_lm), padded to whole 16-byte
// vectors so a warp streams the list with 128-bit loads.
template <typename T, int N> struct ProjRec {
  static constexpr int n = N;
  static constexpr int per_vec = 16 / (int)sizeof(T);
  static constexpr int nvec = (N + per_vec - 1) / per_vec;
  using vec_t = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
  static __device__ __forceinline__ void store(vec_t *rec, int e, const T *v) {
    T tmp[nvec * per_vec];
#pragma unroll
    for (int s = 0; s < nvec * per_vec; s++) tmp[s] = s < N ? v[s] : T(0);
#pragma unroll
    for (int j = 0; j < nvec; j++) {
      vec_t x;
      if constexpr (sizeof(T) == 4) {
        x.x = tmp[4 * j]; x.y = tmp[4 * j + 1]; x.z = tmp[4 * j + 2]; x.w = tmp[4 * j + 3];
      } else {
        x.x = tmp[2 * j]; x.y = tmp[2 * j + 1];
      }
      rec[(size_t)e * nvec + j] = x;
    }
  }
  static __device__ __forceinline__ void load(const vec_t *rec, int e, T *c) {
#pragma unroll
    for (int j = 0; j < nvec; j++) {
      const vec_t x = rec[(size_t)e * nvec + j];
      T t[per_vec];
      if constexpr (sizeof(T) == 4) {
        t[0] = x.x; t[1] = x.y; t[2] = x.z; t[3] = x.w;
      } else {
        t[0] = x.x; t[1] = x.y;
      }
#pragma unroll
      for (int s = 0; s < per_vec; s++)
        if (j * per_vec + s < N) c[j * per_vec + s] = t[s];
    }
  }
};

// One record of the compact projector list (kLayoutCompact): the radial values T_l of the N
// channels of the kernel's mask, in one 8-byte word when they fit, else in 16-byte vectors.
template <typename T, int N> struct ChanRec {
  static constexpr int n = N;
  static constexpr bool word = N * (int)sizeof(T) <= 8;
  using vec_t = typename std::conditional<
      word, typename std::conditional<sizeof(T) == 4, float2, double>::type,
      typename std::conditional<sizeof(T) == 4, float4, double2>::type>::type;
  static constexpr int per_vec = (int)(sizeof(vec_t) / sizeof(T));
  static constexpr int nvec = (N + per_vec - 1) / per_vec;
  union Cast {
    vec_t v;
    T t[per_vec];
  };
  static __device__ __forceinline__ void store(vec_t *rec, int e, const T *v) {
#pragma unroll
    for (int j = 0; j < nvec; j++) {
      Cast x;
#pragma unroll
      for (int s = 0; s < per_vec; s++) x.t[s] = j * per_vec + s < N ? v[j * per_vec + s] : T(0);
      rec[(size_t)e * nvec + j] = x.v;
    }
  }
  static __device__ __forceinline__ void load(const vec_t *rec, int e, T *c) {
#pragma unroll
    for (int j = 0; j < nvec; j++) {
      Cast x;
      x.v = rec[(size_t)e * nvec + j];
#pragma unroll
      for (int s = 0; s < per_vec; s++)
        if (j * per_vec + s < N) c[j * per_vec + s] = x.t[s];
    }
  }
};

// Points per lane per batch of the projector-list streaming loops: 8 for records of up to
// 16 bytes, fewer for wider records so the batch stays in registers.
template <int BYTES> __host__ __device__ constexpr int stream_batch() { return BYTES <= 16 ? 8 : (BYTES <= 32 ? 4 : 2); }

template <typename T, bool FAITHFUL, int MASK> constexpr int rec_values() {
  return FAITHFUL ? 2 : Lm<MASK>::nlm;
}

// Per-image data of the current node, decoded once when a warp range enters an image.
// Point (lx,ly,lz) of box ∩ cube sits at P[pbase + lz*PS + ly*pitch + lx],
// U[ubase + (lz*ny + ly)*nx + lx], table entry tab[(lz*fy + ly)*fx + lx], and at
// coordinates (ox + hx*lx, oy + hy*ly, oz + hz*lz) relative to the image's atom.
template <typename T> struct ImgView {
  int pbase, ubase;
  int ex, ey;
  float iex, iey;
  int fx, fxy, fvol;
  int chan_mask;
  const T *tab;
  T ox, oy, oz;
  T r2max;  // projector support radius squared
};

template <typename T>
__device__ __forceinline__ ImgView<T> load_view(const LanczosParams &p, const ImageMeta *images,
                                                const T *tables, int gidx, int blo, int bext,
                                                int Xs, int Ys, int Zs, int OFF, int PS) {
  ImgView<T> v;
  const ImageMeta m = images[gidx];
  const TypeDesc &td = p.types[m.type];
  const int cx0 = blo & 1023, cy0 = (blo >> 10) & 1023, cz0 = blo >> 20;
  v.ex = bext & 1023;
  v.ey = (bext >> 10) & 1023;
  v.iex = 1.0f / v.ex;
  v.iey = 1.0f / v.ey;
  v.pbase = OFF + cz0 * PS + cy0 * p.pitch + cx0;
  v.ubase = (cz0 * p.ny + cy0) * p.upitch + cx0;
  const int tx0 = Xs + cx0 - m.bx, ty0 = Ys + cy0 - m.by, tz0 = Zs + cz0 - m.bz;
  v.fx = td.fx;
  v.fxy = td.fx * td.fy;
  v.fvol = v.fxy * td.fz;
  v.chan_mask = td.chan_mask;
  v.tab = tables + m.tab_base + (tz0 * v.fxy + ty0 * v.fx + tx0);
  v.ox = T(m.ox + p.hx * tx0);
  v.oy = T(m.oy + p.hy * ty0);
  v.oz = T(m.oz + p.hz * tz0);
  v.r2max = support_r2<T>(td);
  return v;
}

// Decode point t of the intersection box (x fastest) without integer division.
template <typename T>
__device__ __forceinline__ void decode(const ImgView<T> &v, int t, int &lx, int &ly, int &lz) {
  const int row = __float2int_rz((float(t) + 0.5f) * v.iex);
  lx = t - row * v.ex;
  lz = __float2int_rz((float(row) + 0.5f) * v.iey);
  ly = row - lz * v.ey;
}

template <typename T, bool FAITHFUL, bool U_SMEM, int MASK, int LAYOUT>
__global__ void __launch_bounds__((LAYOUT & kLayoutWide) ? 32 * kWideWarpsF32 : 512, 1)
    lanczos_kernel(const __grid_constant__ LanczosParams p, const T *__restrict__ veff_ext,
                   const ImageMeta *__restrict__ images, const T *__restrict__ tables,
                   T *__restrict__ u_global, unsigned char *proj_scratch,
                   double *__restrict__ ab_out, int *__restrict__ status) {
  constexpr int NLM = Lm<MASK>::nlm;
  constexpr bool COMPACT = LAYOUT & kLayoutCompact;
  static_assert(!COMPACT || !FAITHFUL, "compact records carry the corrected operator's channels");
  constexpr int NCH = (MASK & 1) + ((MASK >> 1) & 1) + ((MASK >> 2) & 1) + ((MASK >> 3) & 1);
  using Rec = typename std::conditional<COMPACT, ChanRec<T, NCH>,
                                        ProjRec<T, FAITHFUL ? 2 : NLM>>::type;
  constexpr int kStream = stream_batch<Rec::nvec * (int)sizeof(typename Rec::vec_t)>();
  constexpr int CSTRIDE = FAITHFUL ? 2 : NLM;  // gather accumulators per atom slot
  constexpr int ASTRIDE = FAITHFUL ? 1 : NLM;  // projector coefficients per atom slot
  const int nw = blockDim.x >> 5;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr bool YPAD = LAYOUT & kLayoutYGap, WIDE = LAYOUT & kLayoutWide,
                 XCLAMP = LAYOUT & kLayoutXClamp;
  const int nx = p.nx, ny = p.ny, nz = p.nz, pitch = p.pitch;
  // P index of (x,y,z) = OFF + z*PS + y*pitch + x.  YPAD: O zero rows precede every z-plane
  // and follow the last, so y-neighbours need no bounds checks either.
  const int PS = (YPAD ? ny + O : ny) * pitch;
  const int OFF = YPAD ? O * pitch : O;
  const int upitch = p.upitch;  // U row pitch (nx, or nx+1 to keep FP32 pairs aligned)
  const int US = ny * upitch;   // U plane stride
  const int nc = nz * US;       // U elements including the row padding
  const int psize = ((OFF + nz * PS) + 3) & ~3;
  const int maxi = p.max_img;

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
  double *red = reinterpret_cast<double *>(cur);  // 2 x (kMaxWarps+1)
  cur += sizeof(double) * 2 * (kMaxWarps + 1);
  double *sab = reinterpret_cast<double *>(cur);  // a[64], b[64]
  cur += sizeof(double) * 128;
  T *cacc = reinterpret_cast<T *>(cur);
  cur += sizeof(T) * maxi * CSTRIDE;
  T *alpha = reinterpret_cast<T *>(cur);
  cur += sizeof(T) * maxi * ASTRIDE;
  // compact records: per image of the node, its atom offset and P / U bases
  T *cox = reinterpret_cast<T *>(cur), *coy = cox + maxi, *coz = coy + maxi;
  int *cpb = reinterpret_cast<int *>(coz + maxi), *cub = cpb + maxi;
  if constexpr (COMPACT) cur += (3 * sizeof(T) + 2 * sizeof(int)) * maxi;
  int *img = reinterpret_cast<int *>(cur);
  cur += sizeof(int) * maxi;
  int *slot = reinterpret_cast<int *>(cur);
  cur += sizeof(int) * maxi;
  int *slot_type = reinterpret_cast<int *>(cur);
  cur += sizeof(int) * maxi;
  int *blo = reinterpret_cast<int *>(cur);
  cur += sizeof(int) * maxi;
  int *bext = reinterpret_cast<int *>(cur);
  cur += sizeof(int) * maxi;
  int *pref = reinterpret_cast<int *>(cur);
  cur += sizeof(int) * (maxi + 1);
  int *kept = reinterpret_cast<int *>(cur);
  cur += sizeof(int) * maxi;
  int *koff = reinterpret_cast<int *>(cur);
  cur += sizeof(int) * (maxi + 1);
  int *cnt = reinterpret_cast<int *>(cur);  // [0] images, [1] slots, [2] overflow

  // this CTA's slice of the per-node projector list (records, then packed P|U indices)
  typename Rec::vec_t *rec = reinterpret_cast<typename Rec::vec_t *>(
      proj_scratch + (size_t)blockIdx.x * p.proj_bytes_per_cta);
  unsigned *ridx = reinterpret_cast<unsigned *>(
      reinterpret_cast<unsigned char *>(rec) + (size_t)p.proj_cap * sizeof(typename Rec::vec_t) * Rec::nvec);

  const int x = lane;
  const bool xin = x < nx;
  const int xc = xin ? x : nx - 1;
  const int y_begin = warp * p.rows_per_warp;
  const int y_end = min(ny, y_begin + p.rows_per_warp);
  // FP32 vector passes: half-warp hw owns row py and a z-chunk [zb, ze); lane hl owns the x
  // pair (px, px+1) with px even.  pact = the pair has a cube point, phi = so does px+1.
  constexpr bool PAIRED = sizeof(T) == 4;
  const int hw = threadIdx.x >> 4, hl = threadIdx.x & 15;
  const int nzs = max(1, (2 * nw) / ny);
  const int py = hw / nzs, zc = hw - (hw / nzs) * nzs;
  const int zlen = (nz + nzs - 1) / nzs;
  const int zb = zc * zlen, ze = min(nz, zb + zlen);
  const int px = 2 * hl;
  const bool pact = PAIRED && !WIDE && py < ny && px < nx && zb < ze;
  const int phi = (px + 1 < nx) ? 1 : 0;
  const int pxc = px < nx ? px : ((nx - 1) & ~1);
  // WIDE: task t = (row t / npairs, pair t % npairs), all of z
  const int npairs = (nx + 1) >> 1, ntask = ny * npairs;

  // compact records: chi_lm = P_lm(dx,dy,dz) T_l at a point, from the record's channel values
  // tv (the same products the full list build stores); fn(rank of (l,m), chi_lm)
  auto for_chi = [&](T dx, T dy, T dz, const T *tv, auto &&fn) {
    int c = 0;
    auto ch = [&](auto Lc) {
      constexpr int L = decltype(Lc)::value;
      if constexpr ((MASK >> L) & 1) {
        const T t = tv[c++];
        solid_harmonics<L, T>(dx, dy, dz, [&](int s, T ylm) { fn(Lm<MASK>::rank(s), ylm * t); });
      }
    };
    ch(std::integral_constant<int, 0>{});
    ch(std::integral_constant<int, 1>{});
    ch(std::integral_constant<int, 2>{});
    ch(std::integral_constant<int, 3>{});
  };

  for (long long node = p.node_begin + blockIdx.x; node < p.node_end; node += gridDim.x) {
    const int I = (int)(node % p.Nx);
    const int J = (int)((node / p.Nx) % p.Ny);
    const int K = (int)(node / ((long long)p.Nx * p.Ny));
    const int Xs = I - p.nhx, Ys = J - p.nhy, Zs = K - p.nhz;

    // ---- per-node image list, slots and point offsets (warp 0); others clear ----
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
        if (ok && pos < maxi) img[pos] = i;
        count += __popc(m);
      }
      __syncwarp();
      const int n = min(count, maxi);
      int slots = 0, offset = 0;
      for (int base = 0; base < n; base += 32) {
        const int k = base + lane;
        bool start = false;
        int npts = 0, lo = 0, ext = 0, atom = -1, type = 0;
        if (k < n) {
          const ImageMeta m = images[img[k]];
          atom = m.atom;
          type = m.type;
          start = (k == 0) || images[img[k - 1]].atom != atom;
          const TypeDesc &td = p.types[m.type];
          const int x0 = max(m.bx, Xs), y0 = max(m.by, Ys), z0 = max(m.bz, Zs);
          const int ex = min(m.bx + td.fx, Xs + nx) - x0;
          const int ey = min(m.by + td.fy, Ys + ny) - y0;
          const int ez = min(m.bz + td.fz, Zs + nz) - z0;
          npts = ex * ey * ez;
          lo = (x0 - Xs) | ((y0 - Ys) << 10) | ((z0 - Zs) << 20);
          ext = ex | (ey << 10) | (ez << 20);
        }
        const unsigned m = __ballot_sync(0xffffffffu, start);
        const int g = slots + __popc(m & ((1u << lane) - 1u)) + (start ? 0 : -1);
        int incl = npts;  // inclusive scan of npts
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int t = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += t;
        }
        if (k < n) {
          slot[k] = g;
          if (start) slot_type[g] = type;
          blo[k] = lo;
          bext[k] = ext;
          pref[k] = offset + incl - npts;
        }
        slots += __popc(m);
        offset += __shfl_sync(0xffffffffu, incl, 31);
      }
      if (lane == 0) {
        pref[n] = offset;
        cnt[0] = n;
        cnt[1] = slots;
        cnt[2] = count > maxi;
      }
    } else {
      for (int e = threadIdx.x - 32; e < psize; e += blockDim.x - 32) P[e] = T(0);
      for (int e = threadIdx.x - 32; e < nc; e += blockDim.x - 32) U[e] = T(0);
      for (int e = threadIdx.x - 32; e < maxi * CSTRIDE; e += blockDim.x - 32) cacc[e] = T(0);
    }
    __syncthreads();
    const int n_img = cnt[0], n_slot = cnt[1];
    if (cnt[2]) {  // capacity exceeded: report and leave NaN coefficients for this node
      if (threadIdx.x == 0) atomicOr(status, kStatusCapacity);
      for (int j = threadIdx.x; j < 2 * p.nqp; j += blockDim.x)
        ab_out[(node - p.node_begin) * 2 * p.nqp + j] = __longlong_as_double(0x7ff8000000000000ll);
      __syncthreads();
      continue;
    }
    if (threadIdx.x == 0) P[OFF + (nz - 1) / 2 * PS + (ny - 1) / 2 * pitch + (nx - 1) / 2] = T(1);
    if (pref[n_img] > p.proj_cap) {  // cannot happen with the host's capacity; guard anyway
      if (threadIdx.x == 0) atomicOr(status, kStatusCapacity);
      for (int j = threadIdx.x; j < 2 * p.nqp; j += blockDim.x)
        ab_out[(node - p.node_begin) * 2 * p.nqp + j] = __longlong_as_double(0x7ff8000000000000ll);
      __syncthreads();
      continue;
    }

    // ---- build this node's projector list: one warp per image, support points only ----
    // Record e of image k sits at e = pref[k] + (rank among the image's kept points) and holds
    // chi_lm (or, faithful, sum_lm Gamma_l chi_lm and sum_lm chi_lm) and the packed P|U index.
    for (int kk = warp; kk < n_img; kk += nw) {
      const ImgView<T> v = load_view<T>(p, images, tables, img[kk], blo[kk], bext[kk], Xs, Ys, Zs, OFF, PS);
      if constexpr (COMPACT) {
        if (lane == 0) {
          cox[kk] = v.ox;
          coy[kk] = v.oy;
          coz[kk] = v.oz;
          cpb[kk] = v.pbase;
          cub[kk] = v.ubase;
        }
      }
      T gam[4];
      {
        const TypeDesc &td = p.types[slot_type[slot[kk]]];
#pragma unroll
        for (int l = 0; l < 4; l++) gam[l] = T(td.gamma[l]);
      }
      const int npts = pref[kk + 1] - pref[kk];
      int kept_n = 0;
      for (int q0 = 0; q0 < npts; q0 += 32) {
        const int q = q0 + lane;
        int lx, ly, lz;
        decode(v, min(q, npts - 1), lx, ly, lz);
        const T dx = v.ox + hx_of<T>(p) * T(lx), dy = v.oy + hy_of<T>(p) * T(ly),
                dz = v.oz + hz_of<T>(p) * T(lz);
        const bool ok = q < npts && dx * dx + dy * dy + dz * dz <= v.r2max;
        const unsigned m = __ballot_sync(0xffffffffu, ok);
        if constexpr (COMPACT) {
          if (ok) {  // T_l of the mask's channels (0 where the type has none), box coordinates
            const T *tb = v.tab + lz * v.fxy + ly * v.fx + lx;
            T out[Rec::n];
            int chan = 0, c = 0;
#pragma unroll
            for (int l = 0; l < 4; l++)
              if (MASK & (1 << l)) out[c++] = (v.chan_mask & (1 << l)) ? tb[(chan++) * v.fvol] : T(0);
            const int e = pref[kk] + kept_n + __popc(m & ((1u << lane) - 1u));
            Rec::store(rec, e, out);
            ridx[e] = (unsigned)lx | ((unsigned)ly << 8) | ((unsigned)lz << 16);
          }
        } else if (ok) {
          const T *tb = v.tab + lz * v.fxy + ly * v.fx + lx;
          T out[Rec::n];
#pragma unroll
          for (int s = 0; s < Rec::n; s++) out[s] = T(0);
          int chan = 0;
          auto channel = [&](auto Lc) {
            constexpr int L = decltype(Lc)::value;
            if constexpr (MASK & (1 << L)) {
              if (v.chan_mask & (1 << L)) {
                const T t = tb[(chan++) * v.fvol];
                if constexpr (FAITHFUL) {
                  T ssum = T(0);
                  solid_harmonics<L, T>(dx, dy, dz, [&](int s, T ylm) { ssum += ylm; });
                  out[0] += gam[L] * ssum * t;
                  out[1] += ssum * t;
                } else {
                  solid_harmonics<L, T>(dx, dy, dz, [&](int s, T ylm) {
                    out[Lm<MASK>::rank(s)] = ylm * t;
                  });
                }
              }
            }
          };
          channel(std::integral_constant<int, 0>{});
          channel(std::integral_constant<int, 1>{});
          channel(std::integral_constant<int, 2>{});
          channel(std::integral_constant<int, 3>{});
          const int e = pref[kk] + kept_n + __popc(m & ((1u << lane) - 1u));
          Rec::store(rec, e, out);
          const int pi = v.pbase + lz * PS + ly * pitch + lx;
          const int ui = v.ubase + (lz * ny + ly) * upitch + lx;
          ridx[e] = (unsigned)pi | ((unsigned)ui << 16);
        }
        kept_n += __popc(m);
      }
      if (lane == 0) kept[kk] = kept_n;
    }
    __syncthreads();
    if (warp == 0) {  // exclusive scan of kept -> koff
      int offset = 0;
      for (int base = 0; base < n_img; base += 32) {
        const int kk = base + lane;
        const int c = kk < n_img ? kept[kk] : 0;
        int incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int t = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += t;
        }
        if (kk < n_img) koff[kk] = offset + incl - c;
        offset += __shfl_sync(0xffffffffu, incl, 31);
      }
      if (lane == 0) koff[n_img] = offset;
    }
    __syncthreads();
    const int total = koff[n_img];
    const int per = (total + nw - 1) / nw;
    const int r_begin = min(total, warp * per), r_end = min(total, r_begin + per);
    int k_first = 0;  // image holding kept point r_begin: largest k with koff[k] <= r_begin
    {
      int lo = 0, hi = n_img;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (koff[mid] <= r_begin) lo = mid;
        else hi = mid - 1;
      }
      k_first = min(lo, max(n_img - 1, 0));
    }
    __syncthreads();

    double beta = 1.0;
    for (int j = 0; j < p.nqp; j++) {
      const T inv = T(1.0 / beta);
      const T tbeta = T(beta);

      // ---- nonlocal gather: stream this warp's range of the projector list ----
      {
        int pos = r_begin, k = k_first;
        while (pos < r_end) {
          const int kend = min(r_end, koff[k + 1]);
          const int shift = pref[k] - koff[k];  // list position of kept point i is i + shift
          T acc[CSTRIDE];
#pragma unroll
          for (int s = 0; s < CSTRIDE; s++) acc[s] = T(0);
          int pb = 0;
          T ox = T(0), oy = T(0), oz = T(0);
          if constexpr (COMPACT) {
            pb = cpb[k];
            ox = cox[k];
            oy = coy[k];
            oz = coz[k];
          }
          // batches of kStream points per lane: all list loads of a batch are issued before
          // any is used (addresses clamped into the segment), so each warp keeps
          // 2*kStream L2 requests in flight
          for (int i0 = pos + lane; i0 < kend; i0 += 32 * kStream) {
            T c[kStream][Rec::n];
            unsigned ix[kStream];
#pragma unroll
            for (int u = 0; u < kStream; u++) {
              const int e = min(i0 + 32 * u, kend - 1) + shift;
              ix[u] = ridx[e];
              Rec::load(rec, e, c[u]);
            }
#pragma unroll
            for (int u = 0; u < kStream; u++) {
              if constexpr (COMPACT) {
                const int lx = ix[u] & 255u, ly = (ix[u] >> 8) & 255u, lz = ix[u] >> 16;
                const T val = (i0 + 32 * u < kend) ? P[pb + lz * PS + ly * pitch + lx] : T(0);
                for_chi(ox + hx_of<T>(p) * T(lx), oy + hy_of<T>(p) * T(ly),
                        oz + hz_of<T>(p) * T(lz), c[u], [&](int r, T chi) { acc[r] += chi * val; });
              } else {
                const T val = (i0 + 32 * u < kend) ? P[ix[u] & 0xffffu] : T(0);
#pragma unroll
                for (int s = 0; s < Rec::n; s++) acc[s] += c[u][s] * val;
              }
            }
          }
          const int sl = slot[k];
#pragma unroll
          for (int s = 0; s < CSTRIDE; s++) {
            const T r = warp_sum(acc[s]);
            if (lane == 0) atomicAdd(&cacc[sl * CSTRIDE + s], r);
          }
          pos = kend;
          k++;
        }
      }

      // ---- pass 1: stencil + Veff, U <- H v_k - b_{k-1} U, a_k partial ----
      T a_acc = T(0);
      if constexpr (PAIRED) {
        // half-warp item (row py, z-chunk); lane pair x = px, px+1 (px even)
        const float2 *P2 = reinterpret_cast<const float2 *>(P);
        float2 *U2 = reinterpret_cast<float2 *>(U);
        const int PS2 = PS >> 1, pitch2 = pitch >> 1, US2 = US >> 1;
        const int VS = p.EY * p.EX;
        // one (row ry, pair rx..rx+1, z-range [rzb, rze)) item; rphi = pair has a second point
        auto pair_pass1 = [&](const int ry, const int rx, const int rphi, const int rzb,
                              const int rze) {
          const int rowP2 = (OFF + ry * pitch + rx) >> 1;
          const int rowU2 = (ry * upitch + rx) >> 1;
          const float *vrow = veff_ext + ((size_t)K * p.EY + (J + ry)) * p.EX + (I + rx);
          const float2 zero2 = make_float2(0.f, 0.f);
          float2 win[W];
#pragma unroll
          for (int q = -O; q < O; q++) {
            const int zq = rzb + q;
            win[q + O + 1] = (zq >= 0 && zq < nz) ? P2[rowP2 + min(max(zq, 0), nz - 1) * PS2] : zero2;
          }
          // ring window: plane z + d lives in win[(z - rzb + d + O + 1) % W]; the 13-step
          // unroll keeps every index static so the window never moves between registers
          for (int z0 = rzb; z0 < rze; z0 += W) {
#pragma unroll
            for (int s = 0; s < W; s++) {
              const int z = z0 + s;
              if (z >= rze) break;
              const int qn = z + O;
              win[s] = (qn < nz) ? P2[rowP2 + min(qn, nz - 1) * PS2] : zero2;
#define WIN(dd) win[(s + (dd) + O + 1) % W]
              const int i2 = rowP2 + z * PS2;
              float2 L[7];  // x-6 .. x+7
  #pragma unroll
              for (int jx = 0; jx < 7; jx++) L[jx] = P2[i2 - 3 + jx];
              const float2 vc = WIN(0);
              float2 hz, hx, hy;
              hz.x = (p.cdiagf + vrow[z * VS]) * vc.x;
              hz.y = (p.cdiagf + vrow[z * VS + rphi]) * vc.y;
              hx = zero2;
              hy = zero2;
  #pragma unroll
              for (int d = 1; d <= O; d++) {
                fma2s(hz, p.czf[d], add2(WIN(-d), WIN(d)));
                if constexpr (YPAD) {
                  fma2s(hy, p.cyf[d], add2(P2[i2 - d * pitch2], P2[i2 + d * pitch2]));
                } else {  // rows outside the cube are zero: clamp the index, then drop the value
                  const float2 ym = P2[ry - d >= 0 ? i2 - d * pitch2 : i2];
                  const float2 yp = P2[ry + d < ny ? i2 + d * pitch2 : i2];
                  fma2s(hy, p.cyf[d], add2(ry - d >= 0 ? ym : zero2, ry + d < ny ? yp : zero2));
                }
                if (d % 2 == 0) {
                  fma2s(hx, p.cxf[d], add2(L[3 - d / 2], L[3 + d / 2]));
                } else {
                  const float2 s = make_float2(L[(5 - d) / 2].y + L[(5 + d) / 2].y,
                                               L[(7 - d) / 2].x + L[(7 + d) / 2].x);
                  fma2s(hx, p.cxf[d], s);
                }
              }
              float2 h = add2(add2(hz, hx), hy);
              h.x *= inv;
              h.y *= inv;
              const int u2 = rowU2 + z * US2;
              const float2 uo = U2[u2];
              a_acc += (vc.x * inv) * h.x;
              float2 un;
              un.x = h.x - tbeta * uo.x;
              un.y = 0.f;
              if (rphi) {
                a_acc += (vc.y * inv) * h.y;
                un.y = h.y - tbeta * uo.y;
              }
              U2[u2] = un;

#undef WIN
            }
          }
        };
        if constexpr (WIDE) {
          for (int t = threadIdx.x; t < ntask; t += blockDim.x) {
            const int ty = t / npairs, tx = 2 * (t - ty * npairs);
            pair_pass1(ty, tx, tx + 1 < nx ? 1 : 0, 0, nz);
          }
        } else if (pact) {
          pair_pass1(py, pxc, phi, zb, ze);
        }
      } else {
        for (int y = y_begin; y < y_end; y++) {
          const int rowP = OFF + y * pitch + xc;
          const int rowU = y * upitch + xc;
          const T *vrow = veff_ext + ((size_t)K * p.EY + (J + y)) * p.EX + (I + xc);
          const size_t VS = (size_t)p.EY * p.EX;
          T win[W];
  #pragma unroll
          for (int q = -O; q < O; q++)
            win[q + O + 1] = (q >= 0 && q < nz) ? P[rowP + min(max(q, 0), nz - 1) * PS] : T(0);
  #pragma unroll 1
          for (int z = 0; z < nz; z++) {
  #pragma unroll
            for (int t = 0; t < W - 1; t++) win[t] = win[t + 1];
            const int qn = z + O;
            win[W - 1] = (qn < nz) ? P[rowP + min(qn, nz - 1) * PS] : T(0);
            const int i = rowP + z * PS;
            const T vc = win[O];
            T h = (Coef<T>::diag(p) + vrow[z * VS]) * vc;
  #pragma unroll
            for (int d = 1; d <= O; d++) {
              h += Coef<T>::z(p, d) * (win[O - d] + win[O + d]);
              if constexpr (XCLAMP) {  // no zero columns between rows: clamp, then drop
                const T xm = P[xc - d >= 0 ? i - d : i];
                const T xp = P[xc + d < nx ? i + d : i];
                h += Coef<T>::x(p, d) * ((xc - d >= 0 ? xm : T(0)) + (xc + d < nx ? xp : T(0)));
              } else {
                h += Coef<T>::x(p, d) * (P[i - d] + P[i + d]);
              }
              if constexpr (YPAD) {
                h += Coef<T>::y(p, d) * (P[i - d * pitch] + P[i + d * pitch]);
              } else {  // rows outside the cube are zero: clamp the index, then drop the value
                const T ym = P[y - d >= 0 ? i - d * pitch : i];
                const T yp = P[y + d < ny ? i + d * pitch : i];
                h += Coef<T>::y(p, d) * ((y - d >= 0 ? ym : T(0)) + (y + d < ny ? yp : T(0)));
              }
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
      // the gather above and the stencil touch disjoint outputs (atom slots, U), so warps move
      // from one to the other without waiting; one barrier then covers both
      __syncthreads();

      // ---- projector coefficients alpha from the gathered c, plus <v, V_nl v> ----
      double a_part = 0.0;
      for (int e = threadIdx.x; e < n_slot * ASTRIDE; e += blockDim.x) {
        if constexpr (FAITHFUL) {
          const double cg = (double)cacc[2 * e] * (double)inv;
          const double cs = (double)cacc[2 * e + 1] * (double)inv;
          cacc[2 * e] = T(0);
          cacc[2 * e + 1] = T(0);
          alpha[e] = T(cg);
          a_part += cs * cg;
        } else {
          const int sl = e / NLM, r = e - sl * NLM;
          const TypeDesc &td = p.types[slot_type[sl]];
          const int l = p.rank_l[r];
          const double c = (double)cacc[e] * (double)inv;
          cacc[e] = T(0);
          const double gl = (td.chan_mask & (1 << l)) ? td.gamma[l] : 0.0;
          alpha[e] = T(gl * c);
          a_part += gl * c * c;
        }
      }

      __syncthreads();

      // ---- nonlocal scatter: U += sum_lm chi_lm alpha_lm over this warp's range ----
      {
        int pos = r_begin, k = k_first;
        while (pos < r_end) {
          const int kend = min(r_end, koff[k + 1]);
          const int shift = pref[k] - koff[k];
          const T *al = alpha + slot[k] * ASTRIDE;
          T coef[ASTRIDE];
#pragma unroll
          for (int s = 0; s < ASTRIDE; s++) coef[s] = al[s];
          int ub = 0;
          T ox = T(0), oy = T(0), oz = T(0);
          if constexpr (COMPACT) {
            ub = cub[k];
            ox = cox[k];
            oy = coy[k];
            oz = coz[k];
          }
          for (int i0 = pos + lane; i0 < kend; i0 += 32 * kStream) {
            T c[kStream][Rec::n];
            unsigned ix[kStream];
#pragma unroll
            for (int u = 0; u < kStream; u++) {
              const int e = min(i0 + 32 * u, kend - 1) + shift;
              ix[u] = ridx[e];
              Rec::load(rec, e, c[u]);
            }
#pragma unroll
            for (int u = 0; u < kStream; u++) {
              T val;
              int ui;
              if constexpr (COMPACT) {
                const int lx = ix[u] & 255u, ly = (ix[u] >> 8) & 255u, lz = ix[u] >> 16;
                ui = ub + (lz * ny + ly) * upitch + lx;
                val = T(0);
                for_chi(ox + hx_of<T>(p) * T(lx), oy + hy_of<T>(p) * T(ly),
                        oz + hz_of<T>(p) * T(lz), c[u], [&](int r, T chi) { val += chi * coef[r]; });
              } else if constexpr (FAITHFUL) {
                ui = ix[u] >> 16;
                val = c[u][1] * coef[0];
              } else {
                ui = ix[u] >> 16;
                val = T(0);
#pragma unroll
                for (int s = 0; s < Rec::n; s++) val += c[u][s] * coef[s];
              }
              if (i0 + 32 * u < kend) atomicAdd(&U[ui], val);
            }
          }
          pos = kend;
          k++;
        }
      }
      const double a = block_sum((double)a_acc + a_part, red, nw);

      // ---- pass 2: w = U - a_k v_k, P <- w, U <- v_k, b_k = ||w|| ----
      const T ta = T(a);
      T b_acc = T(0);
      if constexpr (PAIRED) {
        float2 *P2 = reinterpret_cast<float2 *>(P);
        float2 *U2 = reinterpret_cast<float2 *>(U);
        const int PS2 = PS >> 1, US2 = US >> 1;
        auto pair_pass2 = [&](const int ry, const int rx, const int rphi, const int rzb,
                              const int rze) {
          const int rowP2 = (OFF + ry * pitch + rx) >> 1;
          const int rowU2 = (ry * upitch + rx) >> 1;
          for (int z = rzb; z < rze; z++) {
            const float2 pv = P2[rowP2 + z * PS2];
            const float2 uv = U2[rowU2 + z * US2];
            float2 vk, w;
            vk.x = pv.x * inv;
            vk.y = rphi ? pv.y * inv : 0.f;
            w.x = uv.x - ta * vk.x;
            w.y = rphi ? uv.y - ta * vk.y : 0.f;
            P2[rowP2 + z * PS2] = w;
            U2[rowU2 + z * US2] = vk;
            b_acc += w.x * w.x + w.y * w.y;
          }
        };
        if constexpr (WIDE) {
          for (int t = threadIdx.x; t < ntask; t += blockDim.x) {
            const int ty = t / npairs, tx = 2 * (t - ty * npairs);
            pair_pass2(ty, tx, tx + 1 < nx ? 1 : 0, 0, nz);
          }
        } else if (pact) {
          pair_pass2(py, pxc, phi, zb, ze);
        }
      } else if (xin) {
        for (int y = y_begin; y < y_end; y++) {
          const int rowP = OFF + y * pitch + x;
          const int rowU = y * upitch + x;
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
      const double b = sqrt(block_sum((double)b_acc, red + kMaxWarps + 1, nw));
      if (threadIdx.x == 0) {
        sab[j] = a;
        sab[64 + j] = b;
      }
      if (!(b > 0.0) || !isfinite(b)) {  // breakdown: the Krylov space is invariant
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
    __syncthreads();
    for (int r = threadIdx.x; r < p.nqp; r += blockDim.x) {
      double *o = ab_out + (node - p.node_begin) * 2 * p.nqp;
      o[r] = sab[r];
      o[p.nqp + r] = sab[64 + r];
    }
    __syncthreads();
  }
}

template <typename T, bool FAITHFUL, bool U_SMEM, int MASK, int LAYOUT>
cudaError_t launch_variant(const LanczosParams &p, int grid, int block, size_t smem,
                           cudaStream_t s, const void *veff_ext, const ImageMeta *images,
                           const void *tables, void *u_scratch, void *proj_scratch, double *ab,
                           int *status) {
  static_assert(!(LAYOUT & kLayoutWide) || (sizeof(T) == 4 && (LAYOUT & kLayoutYGap) && !U_SMEM),
                "cubes wider than 32 points: FP32 pair passes, y gaps, U in global scratch");
  static_assert(!(LAYOUT & kLayoutXClamp) || sizeof(T) == 8, "x-clamped rows are an FP64 layout");
  static_assert(!(LAYOUT & kLayoutYGap) || sizeof(T) == 4, "y gaps are an FP32 layout");
  auto k = lanczos_kernel<T, FAITHFUL, U_SMEM, MASK, LAYOUT>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k<<<grid, block, smem, s>>>(p, (const T *)veff_ext, images, (const T *)tables, (T *)u_scratch,
                              (unsigned char *)proj_scratch, ab, status);
  return cudaGetLastError();
}

template <typename T, bool FAITHFUL, bool U_SMEM, int LAYOUT>
cudaError_t launch_mask(int mask, const LanczosParams &p, int grid, int block, size_t smem,
                        cudaStream_t s, const void *veff_ext, const ImageMeta *images,
                        const void *tables, void *u_scratch, void *proj_scratch, double *ab,
                        int *status) {
  switch (mask) {
    case 3: return launch_variant<T, FAITHFUL, U_SMEM, 3, LAYOUT>(p, grid, block, smem, s, veff_ext, images, tables, u_scratch, proj_scratch, ab, status);
    case 5: return launch_variant<T, FAITHFUL, U_SMEM, 5, LAYOUT>(p, grid, block, smem, s, veff_ext, images, tables, u_scratch, proj_scratch, ab, status);
    case 6: return launch_variant<T, FAITHFUL, U_SMEM, 6, LAYOUT>(p, grid, block, smem, s, veff_ext, images, tables, u_scratch, proj_scratch, ab, status);
    case 7: return launch_variant<T, FAITHFUL, U_SMEM, 7, LAYOUT>(p, grid, block, smem, s, veff_ext, images, tables, u_scratch, proj_scratch, ab, status);
    default: return launch_variant<T, FAITHFUL, U_SMEM, 15, LAYOUT>(p, grid, block, smem, s, veff_ext, images, tables, u_scratch, proj_scratch, ab, status);
  }
}

}  // namespace lk
}  // namespace sq

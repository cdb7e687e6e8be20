// lanczos_quad.cuh -- FP32 Lanczos kernel with split stencil passes over aligned quads.
//
// Same recurrence and operator as lanczos_kernel.cuh (src/lsdft_scf.cc:119-147 with
// H = -1/2 Lap (12th-order FD, Dirichlet cube, src/lsdft_initObjs.cc:393-475) + diag(Veff)
// + the Kleinman-Bylander projectors of the atom images that meet the cube,
// src/lsdft_matvec.cc:25-149); FP32 vectors, corrected operator, full projector records.
//
// Layout.  P and U are both [nz][ny][pitch] floats in shared memory, pitch = 4*ceil(nx/4),
// planes padded to a bank-friendly stride (quad_plane_floats): every row starts on a 16-byte
// boundary and holds whole float4 quads; the pad columns [nx, pitch) and plane pads stay zero.  There are no zero rows or columns between rows: neighbours outside
// the cube are never loaded (x: the quad loads are predicated off at the row ends; y and z:
// the register rings start and end with zeros).  A point's P and U indices are the same,
// z*PS + y*pitch + x.
//
// Stencil, split by axis so that two of the three axes come from registers:
//   pass A  a thread owns one quad (x..x+3) of row y over a z-range and walks z with a
//           13-plane register ring (one float4 load per plane); the x neighbours of the quad
//           are four aligned float4 loads of the same row; it adds the diagonal (cdiag + Veff,
//           read as one aligned float4 from a quad-aligned copy of the padded potential) and
//           forms U <- (diag + Dz + Dx) v - b U;
//   pass B  a thread owns one quad of plane z over a y-range and walks y with a 13-row
//           register ring: U += Dy v.
// Eight consecutive threads own the quads of one row (pass A) or one plane (pass B), so a
// quarter-warp's float4 accesses cover one contiguous row: no bank conflicts.
//
// Projector list: as in lanczos_kernel.cuh (chi_lm of the node's support points, built once
// per node into the CTA's slice of global scratch), with one index per point (P and U share
// it); consecutive lanes stream consecutive points, so every record load of a warp is one
// contiguous 512-byte run.
//
// Per Lanczos step (P = b v_k unnormalised, U = v_{k-1}), four CTA barriers:
//   1  projector gather c = chi^T P (per-warp ranges of the node's list, one partial per
//      warp and image, no atomics)  ||  pass A
//   2  pass B  ||  alpha = Gamma c / b (and <v, V_nl v>)  -> per-warp partials of a_k
//   3  projector scatter U += chi alpha  ||  every warp reduces the a_k partials
//   4  w = U - a_k v, P <- w, U <- v  -> per-warp partials of b_k^2
// After barrier 4 every warp reduces the b partials itself (the same tree in every warp, so
// every thread sees the same b_k and takes the same branch).  a_k and b_k^2 are summed per
// thread in FP32 with Kahan compensation, then across threads as double-float pairs (an FP32
// head and tail added with error-free transformations, about 48 bits of significand): GB300's
// FP64 pipe runs at a small fraction of its FP32 rate, so the step loop keeps FP64 out of its
// critical path and converts to double only to store a_k and b_k.
//
// Memory traffic.  In the 12-warp budget pass A reads Veff through a per-thread ring of four
// float4 in shared memory, filled by cp.async three planes ahead (slot-major: each warp access
// is 512 contiguous bytes).  The list's stores and loads carry an L2 evict-last policy.  Nodes
// after the first round come from a device-side queue.
//
// CTA pair (PAIR, lanczos_quad_pair_kernel): one node per cluster of two CTAs for cubes whose
// P and U do not fit one CTA.  The cube is split in z (PairPlanes); each CTA owns its planes of
// U and of the list and holds P on its planes plus the 6 the z stencil reads from the peer's
// side, which the peer stores there in its update phase (distributed shared memory).  Barriers
// 2 and 4 become cluster barriers; c is exchanged per slot after phase 2 and a_k, b_k are
// summed from both CTAs' partials in rank order, so both CTAs take every branch together.
#pragma once

#include <cooperative_groups.h>

#include "lanczos_kernel.cuh"

namespace sq {
namespace lq {

using lk::O;
using lk::W;
using lk::kMaxWarps;

// Blackwell packed FP32 (PTX .f32x2, sm_100+): two lanes of float2 per instruction.
__device__ __forceinline__ unsigned long long as_u64(float2 a) {
  return *reinterpret_cast<unsigned long long *>(&a);
}
__device__ __forceinline__ float2 as_f2(unsigned long long r) {
  return *reinterpret_cast<float2 *>(&r);
}
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {  // a*b + c
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(as_u64(a)), "l"(as_u64(b)), "l"(as_u64(c)));
  return as_f2(d);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) {
  unsigned long long d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(as_u64(a)), "l"(as_u64(b)));
  return as_f2(d);
}
__device__ __forceinline__ float2 add2(float2 a, float2 b) {
  unsigned long long d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(as_u64(a)), "l"(as_u64(b)));
  return as_f2(d);
}
__device__ __forceinline__ float2 lo(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi(float4 v) { return make_float2(v.z, v.w); }
__device__ __forceinline__ float2 splat(float c) { return make_float2(c, c); }

// Kahan-compensated FP32 running sum.
struct Kahan {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
};

// Double-float value hi + lo (|lo| <= ulp(hi)/2) and its sum (Knuth's TwoSum, then a
// renormalising FastTwoSum).
struct DF {
  float hi, lo;
};
__device__ __forceinline__ DF df_add(DF x, DF y) {
  const float s = x.hi + y.hi;
  const float bb = s - x.hi;
  float e = (x.hi - (s - bb)) + (y.hi - bb);
  e += x.lo + y.lo;
  const float h = s + e;
  return DF{h, e - (h - s)};
}
__device__ __forceinline__ DF df_of(const Kahan &k) {  // s - c, renormalised
  const float h = k.s - k.c;
  return DF{h, -k.c - (h - k.s)};
}
__device__ __forceinline__ DF df_warp_sum(DF v) {  // the same butterfly in every lane
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    DF w;
    w.hi = __shfl_xor_sync(0xffffffffu, v.hi, o);
    w.lo = __shfl_xor_sync(0xffffffffu, v.lo, o);
    v = df_add(v, w);
  }
  return v;
}
// Sum of nw per-warp partials red[0..nw), the same tree in every lane of every warp, so every
// thread gets the bit-identical total.
__device__ __forceinline__ DF df_all_reduce(const float2 *red, int nw) {
  const int lane = threadIdx.x & 31;
  const float2 r = lane < nw ? red[lane] : make_float2(0.f, 0.f);
  return df_warp_sum(DF{r.x, r.y});
}

// Floats per z-plane of P and U: ny rows of pitch, plus a pad that makes the plane stride
// congruent to one row (4 * pitch/4 floats) modulo the 32 banks.  The y pass has nq = pitch/4
// consecutive threads per plane and consecutive planes on consecutive thread groups, so its
// float4 accesses then fall on consecutive banks across the whole warp (without the pad two
// planes of a quarter-warp can share banks, e.g. 27 rows of 28 floats: offset 20 banks).
__host__ __device__ constexpr int quad_plane_floats(int ny, int pitch) {
  return ny * pitch + ((pitch - ny * pitch) % 32 + 32) % 32;
}

// CTA pair (cube split in z at zsplit): CTA r owns planes [zo0, zo1) of P and U and keeps
// P's planes [pz0, pz1) = its own plus O halo planes on the peer's side, which the peer writes.
struct PairPlanes {
  int zo0, zo1, pz0, pz1;
};
__host__ __device__ constexpr PairPlanes pair_planes(int nz, int zsplit, int rank) {
  return rank == 0 ? PairPlanes{0, zsplit, 0, zsplit + O < nz ? zsplit + O : nz}
                   : PairPlanes{zsplit, nz, zsplit - O > 0 ? zsplit - O : 0, nz};
}
// planes of P and of U to allocate: the larger of the two CTAs'
__host__ __device__ constexpr int pair_p_planes(int nz, int zsplit) {
  return (pair_planes(nz, zsplit, 0).pz1 - pair_planes(nz, zsplit, 0).pz0) >
                 (pair_planes(nz, zsplit, 1).pz1 - pair_planes(nz, zsplit, 1).pz0)
             ? pair_planes(nz, zsplit, 0).pz1 - pair_planes(nz, zsplit, 0).pz0
             : pair_planes(nz, zsplit, 1).pz1 - pair_planes(nz, zsplit, 1).pz0;
}
__host__ __device__ constexpr int pair_u_planes(int nz, int zsplit) {
  return zsplit > nz - zsplit ? zsplit : nz - zsplit;
}

// The per-node projector list (records and point indices) is written once per node and read
// twice per Lanczos step from L2: its stores and loads carry an L2 evict-last cache policy so
// that other traffic does not push it out between the steps.
__device__ __forceinline__ unsigned long long l2_keep_policy() {
  unsigned long long pol;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
__device__ __forceinline__ void st_keep(float4 *p, float4 v, unsigned long long pol) {
  asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(p), "f"(v.x),
               "f"(v.y), "f"(v.z), "f"(v.w), "l"(pol)
               : "memory");
}
__device__ __forceinline__ void st_keep(unsigned *p, unsigned v, unsigned long long pol) {
  asm volatile("st.global.L2::cache_hint.u32 [%0], %1, %2;" ::"l"(p), "r"(v), "l"(pol) : "memory");
}
__device__ __forceinline__ float4 ld_keep(const float4 *p, unsigned long long pol) {
  float4 v;
  asm volatile("ld.global.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ unsigned ld_keep(const unsigned *p, unsigned long long pol) {
  unsigned v;
  asm volatile("ld.global.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
  return v;
}
// one list record (N values of chi_lm, zero-padded to whole float4) with the policy above
template <int N>
__device__ __forceinline__ void rec_store_keep(float4 *rec, int e, const float *v,
                                               unsigned long long pol) {
  constexpr int nv = (N + 3) / 4;
#pragma unroll
  for (int j = 0; j < nv; j++) {
    float t[4];
#pragma unroll
    for (int q = 0; q < 4; q++) t[q] = 4 * j + q < N ? v[4 * j + q] : 0.f;
    st_keep(rec + (size_t)e * nv + j, make_float4(t[0], t[1], t[2], t[3]), pol);
  }
}
template <int N>
__device__ __forceinline__ void rec_load_keep(const float4 *rec, int e, float *c,
                                              unsigned long long pol) {
  constexpr int nv = (N + 3) / 4;
#pragma unroll
  for (int j = 0; j < nv; j++) {
    const float4 x = ld_keep(rec + (size_t)e * nv + j, pol);
    const float t[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
    for (int q = 0; q < 4; q++)
      if (4 * j + q < N) c[4 * j + q] = t[q];
  }
}

// PAIR: one node per cluster of two CTAs (the cube split in z, see PairPlanes); else one node
// per CTA.
template <int MASK, int MAXT, bool ISO, bool PAIR>
__device__ __forceinline__ void quad_body(const LanczosParams &p, const float *__restrict__ veffq,
                                          const ImageMeta *__restrict__ images,
                                          const float *__restrict__ tables,
                                          unsigned char *proj_scratch, double *__restrict__ ab_out,
                                          int *__restrict__ status) {
  constexpr int NLM = lk::Lm<MASK>::nlm;
  using Rec = lk::ProjRec<float, NLM>;
  // points per lane per batch of the gather and of the scatter (all loads of a batch are in
  // flight together; larger batches waste more lanes at the end of each image's range)
  constexpr int kRecBytes = Rec::nvec * (int)sizeof(typename Rec::vec_t);
  constexpr int kStreamG = kRecBytes <= 16 ? 6 : lk::stream_batch<kRecBytes>();
  constexpr int kStreamS = kRecBytes <= 16 ? 8 : lk::stream_batch<kRecBytes>();
  const int nw = blockDim.x >> 5;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nx = p.nx, ny = p.ny, nz = p.nz, pitch = p.pitch;
  const int nq = pitch >> 2;        // quads per row
  const int PS = quad_plane_floats(ny, pitch);  // plane stride (floats)
  const int PS4 = PS >> 2;                       // plane stride (quads)
  const int maxi = p.max_img;
  // planes owned ([zo0, zo1): U and the list) and held of P ([pz0, pz1)); P plane z sits at
  // local plane z - pz0, U plane z at z - zo0
  int cr = 0;  // rank in the CTA pair
  if constexpr (PAIR) cr = (int)cooperative_groups::this_cluster().block_rank();
  const PairPlanes pp = PAIR ? pair_planes(nz, p.zsplit, cr) : PairPlanes{0, nz, 0, nz};
  const int zo0 = pp.zo0, zo1 = pp.zo1, pz0 = pp.pz0, pz1 = pp.pz1, nzo = zo1 - zo0;
  const int ncp = (PAIR ? pair_p_planes(nz, p.zsplit) : nz) * PS;  // floats of P
  const int ncu = (PAIR ? pair_u_planes(nz, p.zsplit) : nz) * PS;  // floats of U
  const int pofs4 = -pz0 * PS4, uofs4 = -zo0 * PS4;  // quad index shifts of planes
  const int udelta = (zo0 - pz0) * PS;  // U index of a list point = its P index - udelta

  extern __shared__ __align__(16) unsigned char smem_raw[];
  float *P = reinterpret_cast<float *>(smem_raw);
  float *U = P + ncp;
  unsigned char *cur = reinterpret_cast<unsigned char *>(U + ncu);
  double *sab = reinterpret_cast<double *>(cur);  // a[64], b[64]
  float2 *red_a = reinterpret_cast<float2 *>(sab + 128);  // per-warp double-float partials
  float2 *red_b = red_a + kMaxWarps;
  cur += sizeof(double) * (2 * kMaxWarps + 128);
  // gathered c per (warp, image): warp w's range covers images k_first(w).. so k + w is
  // unique for every pair it visits; plain stores, summed per slot in a fixed order
  float *part = reinterpret_cast<float *>(cur);
  cur += sizeof(float) * (maxi + kMaxWarps) * NLM;
  float *alpha = reinterpret_cast<float *>(cur);
  cur += sizeof(float) * maxi * NLM;
  // PAIR: the two CTAs' gathered c per (slot, lm), [rank][slot * NLM + lm] (each CTA writes
  // its row into both), the per-warp partials of the projector part of a_k and the two
  // CTAs' capacity flags
  float *cx = reinterpret_cast<float *>(cur);
  float2 *red_n = reinterpret_cast<float2 *>(cur);
  int *xflag = reinterpret_cast<int *>(cur);
  if constexpr (PAIR) {
    cur += sizeof(float) * 2 * maxi * NLM;
    cur += (8 - (reinterpret_cast<uintptr_t>(cur) & 7)) & 7;
    red_n = reinterpret_cast<float2 *>(cur);
    cur += sizeof(float2) * kMaxWarps;
    xflag = reinterpret_cast<int *>(cur);
    cur += sizeof(int) * 4;
  }
  int *img = reinterpret_cast<int *>(cur);
  int *slot = img + maxi;
  int *slot_type = slot + maxi;
  int *blo = slot_type + maxi;
  int *bext = blo + maxi;
  int *pref = bext + maxi;      // maxi + 1
  int *kept = pref + maxi + 1;
  int *koff = kept + maxi;      // maxi + 1
  int *slot_first = koff + maxi + 1;  // first image of every slot (images sorted by atom)
  int *cnt = slot_first + maxi;  // [0] images, [1] slots, [2] overflow, [3] next node
  // Veff rings of pass A (p.vring): slot s of thread t at s * kVRingThreads + t, so a warp's
  // accesses to one slot are 512 contiguous bytes (no bank conflicts); 16-byte aligned
  float4 *vring = reinterpret_cast<float4 *>(
      (reinterpret_cast<uintptr_t>(cnt + 4) + 15) & ~static_cast<uintptr_t>(15));

  typename Rec::vec_t *rec = reinterpret_cast<typename Rec::vec_t *>(
      proj_scratch + (size_t)blockIdx.x * p.proj_bytes_per_cta);
  unsigned *ridx = reinterpret_cast<unsigned *>(
      reinterpret_cast<unsigned char *>(rec) + (size_t)p.proj_cap * sizeof(typename Rec::vec_t) * Rec::nvec);

  const float4 *P4c = reinterpret_cast<const float4 *>(P);
  float4 *P4 = reinterpret_cast<float4 *>(P);
  float4 *U4 = reinterpret_cast<float4 *>(U);
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  const unsigned long long kpol = l2_keep_policy();
  static_assert(std::is_same<typename Rec::vec_t, float4>::value, "FP32 records of float4");

  // thread -> quad of a row (pass A) / of a plane (pass B): nq consecutive threads own the
  // quads of one row or plane, so consecutive threads touch consecutive 16-byte quads
  const int grp = threadIdx.x / nq, ql = threadIdx.x - grp * nq;
  const int nch = p.zchunks, nchB = PAIR ? p.ychunks : p.zchunks;
  // pass A: row yA, z-range [zbA, zeA) of the owned planes
  const int yA = grp % ny, zcA = grp / ny;
  const int zlen = (nzo + nch - 1) / nch;
  const int zbA = zo0 + min(nzo, zcA * zlen), zeA = min(zo1, zbA + zlen);
  const bool actA = zcA < nch && zbA < zeA;
  // pass B: owned plane zB, y-range [ybB, yeB)
  const int zB = zo0 + grp % nzo, ycB = grp / nzo;
  const int ylen = (ny + nchB - 1) / nchB;
  const int ybB = min(ny, ycB * ylen), yeB = min(ny, ybB + ylen);
  const bool actB = ycB < nchB && ybB < yeB;
  // x neighbours of the quad inside the row; lanes of the last quad zero its pad points
  const bool hm1 = ql >= 1, hm2 = ql >= 2, hp1 = ql + 1 < nq, hp2 = ql + 2 < nq;
  const int x0 = 4 * ql;
  const bool in1 = x0 + 1 < nx, in2 = x0 + 2 < nx, in3 = x0 + 3 < nx;  // x0 < nx always

  // nodes: the first round one per CTA, then a queue (status[1], zeroed before the launch):
  // per-node cost varies with the atoms near the node, so CTAs take nodes as they finish.
  // PAIR: node i of the cluster sequence, both CTAs alike (no queue).
  const long long n_units = PAIR ? gridDim.x / 2 : gridDim.x;
  const long long unit = PAIR ? blockIdx.x / 2 : blockIdx.x;
  for (long long node = p.node_begin + unit; node < p.node_end;
       node = PAIR ? node + n_units : p.node_begin + n_units + cnt[3]) {
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
          const int xa = max(m.bx, Xs), ya = max(m.by, Ys), za = max(m.bz, Zs + zo0);
          const int ex = min(m.bx + td.fx, Xs + nx) - xa;
          const int ey = min(m.by + td.fy, Ys + ny) - ya;
          const int ez = max(0, min(m.bz + td.fz, Zs + zo1) - za);  // owned planes only
          npts = ex * ey * ez;
          lo = (xa - Xs) | ((ya - Ys) << 10) | ((za - Zs) << 20);
          ext = ex | (ey << 10) | (ez << 20);
        }
        const unsigned m = __ballot_sync(0xffffffffu, start);
        const int g = slots + __popc(m & ((1u << lane) - 1u)) + (start ? 0 : -1);
        int incl = npts;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int t = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += t;
        }
        if (k < n) {
          slot[k] = g;
          if (start) {
            slot_type[g] = type;
            slot_first[g] = k;
          }
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
      for (int e = threadIdx.x - 32; e < (ncp >> 2); e += blockDim.x - 32) P4[e] = zero4;
      for (int e = threadIdx.x - 32; e < (ncu >> 2); e += blockDim.x - 32) U4[e] = zero4;
    }
    __syncthreads();
    const int n_img = cnt[0], n_slot = cnt[1];
    bool overflow = cnt[2] || pref[n_img] > p.proj_cap;
    if constexpr (PAIR) {  // both CTAs take the capacity branch together
      if (threadIdx.x == 0) {
        xflag[cr] = overflow;
        *cooperative_groups::this_cluster().map_shared_rank(xflag + cr, cr ^ 1) = overflow;
      }
      cooperative_groups::this_cluster().sync();
      overflow = xflag[0] || xflag[1];
    } else {
      // the next node, read by every thread after this node's last barrier (the previous
      // value was read before the barrier above)
      if (threadIdx.x == 0) cnt[3] = atomicAdd(status + 1, 1);
    }
    if (overflow) {  // capacity exceeded: report, NaN coefficients
      if (threadIdx.x == 0) atomicOr(status, kStatusCapacity);
      if (cr == 0)
        for (int j = threadIdx.x; j < 2 * p.nqp; j += blockDim.x)
          ab_out[(node - p.node_begin) * 2 * p.nqp + j] = __longlong_as_double(0x7ff8000000000000ll);
      if constexpr (PAIR) cooperative_groups::this_cluster().sync();  // flags read by both
      else __syncthreads();
      continue;
    }
    {  // v_0: the unit vector at the cube centre, in every CTA that holds that plane of P
      const int zc = (nz - 1) / 2;
      if (threadIdx.x == 0 && zc >= pz0 && zc < pz1)
        P[(zc - pz0) * PS + (ny - 1) / 2 * pitch + (nx - 1) / 2] = 1.f;
    }

    // ---- this node's projector list: one warp per image, support points only ----
    for (int kk = warp; kk < n_img; kk += nw) {
      const lk::ImgView<float> v =
          lk::load_view<float>(p, images, tables, img[kk], blo[kk], bext[kk], Xs, Ys, Zs, pofs4 * 4, PS);
      const int npts = pref[kk + 1] - pref[kk];
      int kept_n = 0;
      for (int q0 = 0; q0 < npts; q0 += 32) {
        const int q = q0 + lane;
        int lx, ly, lz;
        lk::decode(v, min(q, npts - 1), lx, ly, lz);
        const float dx = v.ox + p.hxf * float(lx), dy = v.oy + p.hyf * float(ly),
                    dz = v.oz + p.hzf * float(lz);
        const bool ok = q < npts && dx * dx + dy * dy + dz * dz <= v.r2max;
        const unsigned m = __ballot_sync(0xffffffffu, ok);
        if (ok) {
          const float *tb = v.tab + lz * v.fxy + ly * v.fx + lx;
          float out[Rec::n];
#pragma unroll
          for (int s = 0; s < Rec::n; s++) out[s] = 0.f;
          int chan = 0;
          auto channel = [&](auto Lc) {
            constexpr int L = decltype(Lc)::value;
            if constexpr (MASK & (1 << L)) {
              if (v.chan_mask & (1 << L)) {
                const float t = tb[(chan++) * v.fvol];
                lk::solid_harmonics<L, float>(dx, dy, dz, [&](int s, float ylm) {
                  out[lk::Lm<MASK>::rank(s)] = ylm * t;
                });
              }
            }
          };
          channel(std::integral_constant<int, 0>{});
          channel(std::integral_constant<int, 1>{});
          channel(std::integral_constant<int, 2>{});
          channel(std::integral_constant<int, 3>{});
          const int e = pref[kk] + kept_n + __popc(m & ((1u << lane) - 1u));
          rec_store_keep<NLM>(rec, e, out, kpol);
          st_keep(ridx + e, (unsigned)(v.pbase + lz * PS + ly * pitch + lx), kpol);
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

    // quad-aligned copy of the padded Veff + cdiag for this node (copy s: I + s = 0 mod 4)
    const int sh = (4 - (I & 3)) & 3;
    const float4 *vq = reinterpret_cast<const float4 *>(veffq + (size_t)sh * p.vq_copy_stride) +
                       (size_t)((I + sh) >> 2);
    const size_t VPS4 = (size_t)p.EY * (p.vq_row >> 2);  // plane stride in quads
    const size_t VRS4 = (size_t)(p.vq_row >> 2);         // row stride in quads

    float tb = 1.f;  // b_{k-1}
    for (int j = 0; j < p.nqp; j++) {
      const float inv = 1.f / tb;
      const float2 inv2 = splat(inv), ntb2 = splat(-tb);

      // ---- phase 1: projector gather  ||  pass A ----
      {
        int pos = r_begin, k = k_first;
        while (pos < r_end) {
          const int kend = min(r_end, koff[k + 1]);
          const int shift = pref[k] - koff[k];
          float acc[NLM];
#pragma unroll
          for (int s = 0; s < NLM; s++) acc[s] = 0.f;
          for (int i0 = pos + lane; i0 < kend; i0 += 32 * kStreamG) {
            float c[kStreamG][NLM];
            unsigned ix[kStreamG];
#pragma unroll
            for (int u = 0; u < kStreamG; u++) {
              const int e = min(i0 + 32 * u, kend - 1) + shift;
              ix[u] = ld_keep(ridx + e, kpol);
              rec_load_keep<NLM>(rec, e, c[u], kpol);
            }
#pragma unroll
            for (int u = 0; u < kStreamG; u++) {
              const float val = (i0 + 32 * u < kend) ? P[ix[u]] : 0.f;
#pragma unroll
              for (int s = 0; s < NLM; s++) acc[s] = fmaf(c[u][s], val, acc[s]);
            }
          }
#pragma unroll
          for (int s = 0; s < NLM; s++) {
            const float r = lk::warp_sum(acc[s]);
            if (lane == 0) part[(k + warp) * NLM + s] = r;
          }
          pos = kend;
          k++;
        }
      }
      Kahan ka;
      if (actA) {
        // stencil weights scaled by 1/b_{k-1} (live in registers during this pass only)
        float2 czs[O + 1], cxs[O + 1];
#pragma unroll
        for (int d = 1; d <= O; d++) {
          czs[d] = splat(p.czf[d] * inv);
          cxs[d] = ISO ? czs[d] : splat(p.cxf[d] * inv);
        }
        const int row4 = yA * nq + ql;  // quad index of (x0, yA) in a plane
        const float4 *vrow = vq + (size_t)(K * p.EY + J + yA) * VRS4 + ql;
        float4 ring[W];
#pragma unroll
        for (int q = -O; q < O; q++) {
          const int zq = zbA + q;
          ring[q + O + 1] = (zq >= 0 && zq < nz) ? P4c[row4 + zq * PS4 + pofs4] : zero4;
        }
        // x neighbours: the upper half of quad q-2, quads q-1 and q+1, the lower half of q+2
        float2 xm2 = make_float2(0.f, 0.f), xp2 = make_float2(0.f, 0.f);
        float4 xm1 = zero4, xp1 = zero4;
        const float2 *P2c = reinterpret_cast<const float2 *>(P);
        // U of plane z+1 loads while plane z is computed, and Veff (from L2) kVRingSlots - 1
        // planes ahead through the thread's ring of async copies (p.vring; else one plane
        // ahead in registers).  The 16-warp budget has no registers to spare for either.
        constexpr bool kPrefetch = MAXT <= 384;
        constexpr int kAhead = kVRingSlots - 1;
        const bool use_ring = kPrefetch && p.vring;
        const unsigned vr0 = (unsigned)__cvta_generic_to_shared(vring + threadIdx.x);
        auto vcopy = [&](int zc, int slot) {  // Veff quad of plane zc into ring slot
          if (zc < zeA)
            asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(
                             vr0 + 16u * (unsigned)(slot * kVRingThreads)),
                         "l"(__cvta_generic_to_global(vrow + (size_t)zc * VPS4))
                         : "memory");
          asm volatile("cp.async.commit_group;" ::: "memory");  // one group per plane, even empty
        };
        float4 nuo = zero4, ndv = zero4;
        if constexpr (kPrefetch) {
          nuo = U4[row4 + zbA * PS4 + uofs4];
          if (use_ring) {
            for (int d = 0; d < kAhead; d++) vcopy(zbA + d, d);
          } else {
            ndv = __ldg(vrow + (size_t)zbA * VPS4);
          }
        }
        for (int z0 = zbA; z0 < zeA; z0 += W) {
#pragma unroll
          for (int s = 0; s < W; s++) {
            const int z = z0 + s;
            if (z >= zeA) break;
            const int qn = z + O;
            ring[s] = qn < nz ? P4c[row4 + qn * PS4 + pofs4] : zero4;
#define RING(dd) ring[(s + (dd) + O + 1) % W]
            const int i4 = row4 + z * PS4 + pofs4, iu4 = row4 + z * PS4 + uofs4;
            if (hm2) xm2 = P2c[2 * i4 - 3];
            if (hm1) xm1 = P4c[i4 - 1];
            if (hp1) xp1 = P4c[i4 + 1];
            if (hp2) xp2 = P2c[2 * i4 + 4];
            const float4 c = RING(0);
            float4 dv, uo;
            if constexpr (kPrefetch) {
              if (use_ring) {
                // plane z's copy is done once at most kAhead - 1 later groups are pending; the
                // copy of plane z + kAhead then goes to the slot read one plane earlier
                asm volatile("cp.async.wait_group %0;" ::"n"(kAhead - 1) : "memory");
                const int i = z - zbA;
                dv = vring[(i & (kVRingSlots - 1)) * kVRingThreads + threadIdx.x];
                vcopy(z + kAhead, (i + kAhead) & (kVRingSlots - 1));
              } else {
                dv = ndv;
                if (z + 1 < zeA) ndv = __ldg(vrow + (size_t)(z + 1) * VPS4);
              }
              uo = nuo;
              if (z + 1 < zeA) nuo = U4[iu4 + PS4];
            } else {
              dv = __ldg(vrow + (size_t)z * VPS4);
              uo = U4[iu4];
            }
            const float2 vs01 = mul2(lo(c), inv2), vs23 = mul2(hi(c), inv2);  // v_k
            float2 h01 = mul2(lo(dv), vs01), h23 = mul2(hi(dv), vs23);
#pragma unroll
            for (int d = 1; d <= O; d++) {
              h01 = fma2(czs[d], add2(lo(RING(-d)), lo(RING(d))), h01);
              h23 = fma2(czs[d], add2(hi(RING(-d)), hi(RING(d))), h23);
            }
#undef RING
            // x neighbours: e[i] = P[x0 - 6 + i], i = 0..15
            const float e[16] = {xm2.x, xm2.y, xm1.x, xm1.y, xm1.z, xm1.w, c.x,   c.y,
                                 c.z,   c.w,   xp1.x, xp1.y, xp1.z, xp1.w, xp2.x, xp2.y};
#pragma unroll
            for (int d = 1; d <= O; d++) {
              if (d % 2 == 0) {
                h01 = fma2(cxs[d], add2(make_float2(e[6 - d], e[7 - d]), make_float2(e[6 + d], e[7 + d])), h01);
                h23 = fma2(cxs[d], add2(make_float2(e[8 - d], e[9 - d]), make_float2(e[8 + d], e[9 + d])), h23);
              } else {
                h01 = fma2(cxs[d], make_float2(e[6 - d] + e[6 + d], e[7 - d] + e[7 + d]), h01);
                h23 = fma2(cxs[d], make_float2(e[8 - d] + e[8 + d], e[9 - d] + e[9 + d]), h23);
              }
            }
            // zero the pad points, U <- h - b_{k-1} U, a_k partial <v_k, h>
            h01.y = in1 ? h01.y : 0.f;
            h23.x = in2 ? h23.x : 0.f;
            h23.y = in3 ? h23.y : 0.f;
            const float2 n01 = fma2(ntb2, lo(uo), h01), n23 = fma2(ntb2, hi(uo), h23);
            U4[iu4] = make_float4(n01.x, n01.y, n23.x, n23.y);
            const float2 pa = fma2(vs01, h01, mul2(vs23, h23));
            ka.add(pa.x + pa.y);
          }
        }
      }
      __syncthreads();

      // ---- phase 2: pass B  ||  alpha = Gamma c / b ----
      if (actB) {
        float2 cys[O + 1];
#pragma unroll
        for (int d = 1; d <= O; d++) cys[d] = splat((ISO ? p.czf[d] : p.cyf[d]) * inv);
        // quad index of (x0, y = 0) in plane zB of P and of U
        const int pl4 = zB * PS4 + ql + pofs4, pl4u = zB * PS4 + ql + uofs4;
        // ring[j] holds row ybB - 6 + j; row y+7 and U of row y+1 load while row y computes
        float4 ring[W];
#pragma unroll
        for (int j = 0; j < W; j++) {
          const int yq = ybB - O + j;
          ring[j] = (yq >= 0 && yq < ny) ? P4c[pl4 + yq * nq] : zero4;
        }
        float4 nuo = U4[pl4u + ybB * nq];
        for (int y0 = ybB; y0 < yeB; y0 += W) {
#pragma unroll
          for (int s = 0; s < W; s++) {
            const int y = y0 + s;
            if (y >= yeB) break;
            const int u4 = pl4 + y * nq, uu4 = pl4u + y * nq;
            const float4 uo = nuo;
            const float4 nring = y + O + 1 < ny ? P4c[u4 + (O + 1) * nq] : zero4;
            if (y + 1 < yeB) nuo = U4[uu4 + nq];
#define RING(dd) ring[(s + (dd) + O) % W]
            float2 h01 = make_float2(0.f, 0.f), h23 = make_float2(0.f, 0.f);
#pragma unroll
            for (int d = 1; d <= O; d++) {
              h01 = fma2(cys[d], add2(lo(RING(-d)), lo(RING(d))), h01);
              h23 = fma2(cys[d], add2(hi(RING(-d)), hi(RING(d))), h23);
            }
            const float4 c = RING(0);
#undef RING
            const float2 n01 = add2(lo(uo), h01), n23 = add2(hi(uo), h23);
            U4[uu4] = make_float4(n01.x, n01.y, n23.x, n23.y);
            const float2 pa = fma2(mul2(lo(c), inv2), h01, mul2(mul2(hi(c), inv2), h23));
            ka.add(pa.x + pa.y);
            ring[s] = nring;  // row y-6 leaves, row y+7 joins
          }
        }
      }
      // alpha = Gamma_l c, with c = <chi, v_k>; <v_k, V_nl v_k> = sum Gamma_l c^2 joins a_k
      for (int e = threadIdx.x; e < n_slot * NLM; e += blockDim.x) {
        const int sl = e / NLM, r = e - sl * NLM;
        const TypeDesc &td = p.types[slot_type[sl]];
        const int l = p.rank_l[r];
        // c of the slot: its images' partials from every warp whose range meets them, in a
        // fixed order (no atomics: shared-memory float atomics on a few hot addresses stall)
        float csum = 0.f;
        for (int k = slot_first[sl]; k < n_img && slot[k] == sl; k++) {
          if (koff[k + 1] == koff[k]) continue;
          const int w1 = (koff[k + 1] - 1) / per;
          for (int w = koff[k] / per; w <= w1; w++) csum += part[(k + w) * NLM + r];
        }
        if constexpr (PAIR) {  // this CTA's part of c, into both CTAs' row cr of cx
          cx[cr * maxi * NLM + e] = csum;
          *cooperative_groups::this_cluster().map_shared_rank(cx + cr * maxi * NLM + e, cr ^ 1) = csum;
        } else {
          const float cv = csum * inv;
          const float gl = (td.chan_mask & (1 << l)) ? float(td.gamma[l]) : 0.f;
          const float al = gl * cv;
          alpha[e] = al;
          ka.add(al * cv);
        }
      }
      {
        const DF ap = df_warp_sum(df_of(ka));
        if (lane == 0) red_a[warp] = make_float2(ap.hi, ap.lo);
      }
      if constexpr (PAIR) cooperative_groups::this_cluster().sync();
      else __syncthreads();

      // ---- phase 3: projector scatter U += chi alpha  ||  a_k ----
      {
        int pos = r_begin, k = k_first;
        while (pos < r_end) {
          const int kend = min(r_end, koff[k + 1]);
          const int shift = pref[k] - koff[k];
          float coef[NLM];
          if constexpr (PAIR) {  // alpha = Gamma_l (c_0 + c_1) / b from the two CTAs' rows
            const int sl = slot[k];
            const TypeDesc &td = p.types[slot_type[sl]];
#pragma unroll
            for (int s = 0; s < NLM; s++) {
              const int l = p.rank_l[s];
              const float gl = (td.chan_mask & (1 << l)) ? float(td.gamma[l]) : 0.f;
              coef[s] = gl * ((cx[sl * NLM + s] + cx[maxi * NLM + sl * NLM + s]) * inv);
            }
          } else {
            const float *al = alpha + slot[k] * NLM;
#pragma unroll
            for (int s = 0; s < NLM; s++) coef[s] = al[s];
          }
          for (int i0 = pos + lane; i0 < kend; i0 += 32 * kStreamS) {
            float c[kStreamS][NLM];
            unsigned ix[kStreamS];
#pragma unroll
            for (int u = 0; u < kStreamS; u++) {
              const int e = min(i0 + 32 * u, kend - 1) + shift;
              ix[u] = ld_keep(ridx + e, kpol);
              rec_load_keep<NLM>(rec, e, c[u], kpol);
            }
#pragma unroll
            for (int u = 0; u < kStreamS; u++) {
              float val = 0.f;
#pragma unroll
              for (int s = 0; s < NLM; s++) val = fmaf(c[u][s], coef[s], val);
              // fire-and-forget shared atomics: a plain read-add-write waits on the read
              if (i0 + 32 * u < kend) atomicAdd(&U[ix[u] - udelta], val);
            }
          }
          pos = kend;
          k++;
        }
      }
      DF adf;
      if constexpr (PAIR) {
        // <v, V_nl v> = sum Gamma_l c^2 over the slots, the same sum in both CTAs
        Kahan kn;
        for (int e = threadIdx.x; e < n_slot * NLM; e += blockDim.x) {
          const int sl = e / NLM, r = e - sl * NLM;
          const TypeDesc &td = p.types[slot_type[sl]];
          const int l = p.rank_l[r];
          const float gl = (td.chan_mask & (1 << l)) ? float(td.gamma[l]) : 0.f;
          const float cv = (cx[e] + cx[maxi * NLM + e]) * inv;
          kn.add(gl * cv * cv);
        }
        const DF np = df_warp_sum(df_of(kn));
        if (lane == 0) red_n[warp] = make_float2(np.hi, np.lo);
        __syncthreads();
        // a_k: CTA 0's stencil partials, CTA 1's, then the projector part (fixed order)
        auto cl = cooperative_groups::this_cluster();
        const float2 *ra0 = cr == 0 ? red_a : cl.map_shared_rank(red_a, 0);
        const float2 *ra1 = cr == 1 ? red_a : cl.map_shared_rank(red_a, 1);
        adf = df_add(df_add(df_all_reduce(ra0, nw), df_all_reduce(ra1, nw)), df_all_reduce(red_n, nw));
      } else {
        adf = df_all_reduce(red_a, nw);
        __syncthreads();
      }

      // ---- phase 4: w = U - a_k v, P <- w, U <- v, b_k^2 partial ----
      {
        const float2 na2 = splat(-(adf.hi + adf.lo));
        Kahan kb;
        // owned planes: P's at quad e + udelta/4, U's at e.  PAIR: quads [h0, h1) are the
        // peer's halo planes and also go to its P at e + dpeer.
        const int nown = nzo * PS4;
        float4 *P4o = P4 + (udelta >> 2);
        int h0 = 0, h1 = 0, dpeer = 0;
        float4 *P4peer = P4;
        if constexpr (PAIR) {
          const PairPlanes pq = pair_planes(nz, p.zsplit, cr ^ 1);
          h0 = (max(zo0, pq.pz0) - zo0) * PS4;
          h1 = (min(zo1, pq.pz1) - zo0) * PS4;
          dpeer = (zo0 - pq.pz0) * PS4;
          P4peer = cooperative_groups::this_cluster().map_shared_rank(P4, cr ^ 1);
        }
        // the next quad's P and U are read before this quad's are written
        float4 npv = zero4, nuv = zero4;
        if (threadIdx.x < nown) {
          npv = P4o[threadIdx.x];
          nuv = U4[threadIdx.x];
        }
        for (int e = threadIdx.x; e < nown; e += blockDim.x) {
          const float4 pv = npv, uv = nuv;
          if (e + (int)blockDim.x < nown) {
            npv = P4o[e + blockDim.x];
            nuv = U4[e + blockDim.x];
          }
          const float2 v01 = mul2(lo(pv), inv2), v23 = mul2(hi(pv), inv2);
          const float2 w01 = fma2(na2, v01, lo(uv)), w23 = fma2(na2, v23, hi(uv));
          const float4 w4 = make_float4(w01.x, w01.y, w23.x, w23.y);
          P4o[e] = w4;
          if constexpr (PAIR) {
            if (e >= h0 && e < h1) P4peer[e + dpeer] = w4;
          }
          U4[e] = make_float4(v01.x, v01.y, v23.x, v23.y);
          const float2 q = fma2(w01, w01, mul2(w23, w23));
          kb.add(q.x + q.y);
        }
        const DF bp = df_warp_sum(df_of(kb));
        if (lane == 0) red_b[warp] = make_float2(bp.hi, bp.lo);
        if (threadIdx.x == 0) sab[j] = (double)adf.hi + (double)adf.lo;
      }
      DF b2;
      if constexpr (PAIR) {  // the halo planes and both CTAs' b partials are in place
        auto cl = cooperative_groups::this_cluster();
        cl.sync();
        const float2 *rb0 = cr == 0 ? red_b : cl.map_shared_rank(red_b, 0);
        const float2 *rb1 = cr == 1 ? red_b : cl.map_shared_rank(red_b, 1);
        b2 = df_add(df_all_reduce(rb0, nw), df_all_reduce(rb1, nw));
      } else {
        __syncthreads();
        b2 = df_all_reduce(red_b, nw);
      }
      const float bf = sqrtf(b2.hi + b2.lo);
      if (threadIdx.x == 0) sab[64 + j] = sqrt((double)b2.hi + (double)b2.lo);
      if (!(bf > 0.f) || !isfinite(bf)) {  // breakdown: the Krylov space is invariant
        if (threadIdx.x == 0) {
          atomicOr(status, kStatusBreakdown);
          for (int r = j + 1; r < p.nqp; r++) {
            sab[r] = 0.0;
            sab[64 + r] = 0.0;
          }
        }
        break;
      }
      tb = bf;
    }
    __syncthreads();
    if (cr == 0)
      for (int r = threadIdx.x; r < p.nqp; r += blockDim.x) {
        double *o = ab_out + (node - p.node_begin) * 2 * p.nqp;
        o[r] = sab[r];
        o[p.nqp + r] = sab[64 + r];
      }
    __syncthreads();
  }
  // no CTA of a pair leaves while its peer may still read its shared memory
  if constexpr (PAIR) cooperative_groups::this_cluster().sync();
}

template <int MASK, int MAXT, bool ISO>
__global__ void __launch_bounds__(MAXT, 1)
    lanczos_quad_kernel(const __grid_constant__ LanczosParams p, const float *__restrict__ veffq,
                        const ImageMeta *__restrict__ images, const float *__restrict__ tables,
                        unsigned char *proj_scratch, double *__restrict__ ab_out,
                        int *__restrict__ status) {
  quad_body<MASK, MAXT, ISO, false>(p, veffq, images, tables, proj_scratch, ab_out, status);
}

// One node per cluster of two CTAs (cubes whose P and U do not fit one CTA).
template <int MASK, bool ISO>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(384, 1)
    lanczos_quad_pair_kernel(const __grid_constant__ LanczosParams p,
                             const float *__restrict__ veffq, const ImageMeta *__restrict__ images,
                             const float *__restrict__ tables, unsigned char *proj_scratch,
                             double *__restrict__ ab_out, int *__restrict__ status) {
  quad_body<MASK, 384, ISO, true>(p, veffq, images, tables, proj_scratch, ab_out, status);
}

template <int MASK, int MAXT, bool ISO>
cudaError_t launch_quad_variant(const LanczosParams &p, int grid, int block, size_t smem,
                                cudaStream_t s, const void *veffq, const ImageMeta *images,
                                const void *tables, void *proj_scratch, double *ab, int *status) {
  if (block > MAXT) return cudaErrorInvalidConfiguration;
  auto k = lanczos_quad_kernel<MASK, MAXT, ISO>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k<<<grid, block, smem, s>>>(p, (const float *)veffq, images, (const float *)tables,
                              (unsigned char *)proj_scratch, ab, status);
  return cudaGetLastError();
}

template <int MASK, bool ISO>
cudaError_t launch_quad_pair_variant(const LanczosParams &p, int grid, int block, size_t smem,
                                     cudaStream_t s, const void *veffq, const ImageMeta *images,
                                     const void *tables, void *proj_scratch, double *ab,
                                     int *status) {
  if (block > 384 || grid % 2 != 0) return cudaErrorInvalidConfiguration;
  auto k = lanczos_quad_pair_kernel<MASK, ISO>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k<<<grid, block, smem, s>>>(p, (const float *)veffq, images, (const float *)tables,
                              (unsigned char *)proj_scratch, ab, status);
  return cudaGetLastError();
}

// Clusters of two that can be resident at once for this block and shared-memory size.
template <int MASK, bool ISO>
cudaError_t pair_max_clusters(int block, size_t smem, int *clusters) {
  auto k = lanczos_quad_pair_kernel<MASK, ISO>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(2, 1, 1);
  cfg.blockDim = dim3(block, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr;
  attr.id = cudaLaunchAttributeClusterDimension;
  attr.val.clusterDim.x = 2;
  attr.val.clusterDim.y = 1;
  attr.val.clusterDim.z = 1;
  cfg.attrs = &attr;
  cfg.numAttrs = 1;
  return cudaOccupancyMaxActiveClusters(clusters, (void *)k, &cfg);
}

}  // namespace lq
}  // namespace sq

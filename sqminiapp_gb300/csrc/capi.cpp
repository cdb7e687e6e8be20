// capi.cpp -- the C ABI of include/sq_gb300.h.
//
// A handle owns the parsed deck, the host setup and the device buffers.  Every entry point
// returns sq_status; fatal paths of the reference (exit(1)) become SQ_BAD_INPUT,
// SQ_NO_CONVERGENCE, ... and sq_last_error_string() gives the message.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "handle.hpp"
#include "sq_gb300.h"
#include "scf_internal.hpp"
#include "sq_internal.hpp"
#include "sq_kernels.hpp"

namespace sq {

namespace {
thread_local std::string g_last_error;
}  // namespace

sq_status fail(sq_status s, const std::string &msg) {
  g_last_error = msg;
  return s;
}

void set_noalloc_error(const std::string &msg) { g_last_error = msg; }

const std::string &last_error() { return g_last_error; }

void ck(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

void ensure_capacity(double *&ptr, long long &cap, long long need, const char *what) {
  if (need <= cap) return;
  dev_free(ptr);
  dev_alloc(&ptr, sizeof(double) * (size_t)need, what);
  cap = need;
}

}  // namespace sq

using namespace sq;

sq_handle::~sq_handle() {
  sq::scf_destroy(scf);
  dev_free(d_images);
  dev_free(d_tables);
  dev_free(d_veff_ext);
  dev_free(d_veff_in);
  dev_free(d_u);
  dev_free(d_proj);
  dev_free(d_status);
  dev_free(d_ab);
  dev_free(d_lambda);
  dev_free(d_w);
  dev_free(d_lmin);
  dev_free(d_lmax);
  dev_free(d_rho);
  dev_free(d_fermi_scratch);
  dev_free(d_bar);
  dev_free(d_fermi_out);
  for (auto &e : ev)
    if (e) cudaEventDestroy(e);
  if (own_stream) cudaStreamDestroy(own_stream);
}

namespace {

// Largest number of images that meet one node's cube, by a 3D difference array over the
// node grid: image box [b, b+f) meets the cube of node I iff I in [b - nh, b + f - 1 + nh].
int max_images_per_node(const sq::Setup &s, const sq::Deck &d) {
  const int N[3] = {d.grid[0], d.grid[1], d.grid[2]};
  const int M[3] = {N[0] + 1, N[1] + 1, N[2] + 1};
  std::vector<int> diff((size_t)M[0] * M[1] * M[2], 0);
  auto at = [&](int x, int y, int z) -> int & { return diff[((size_t)z * M[1] + y) * M[0] + x]; };
  for (const sq::ImageMeta &im : s.images) {
    const sq::TypeDesc &td = s.types[im.type];
    const int b[3] = {im.bx, im.by, im.bz}, f[3] = {td.fx, td.fy, td.fz};
    int lo[3], hi[3];
    bool empty = false;
    for (int a = 0; a < 3; a++) {
      lo[a] = std::max(0, b[a] - s.nh[a]);
      hi[a] = std::min(N[a] - 1, b[a] + f[a] - 1 + s.nh[a]);
      if (lo[a] > hi[a]) empty = true;
    }
    if (empty) continue;
    for (int c = 0; c < 8; c++) {
      const int x = (c & 1) ? hi[0] + 1 : lo[0];
      const int y = (c & 2) ? hi[1] + 1 : lo[1];
      const int z = (c & 4) ? hi[2] + 1 : lo[2];
      at(x, y, z) += (__builtin_popcount(c) & 1) ? -1 : 1;
    }
  }
  int best = 0;
  for (int z = 0; z < M[2]; z++)
    for (int y = 0; y < M[1]; y++)
      for (int x = 0; x < M[0]; x++) {
        int v = at(x, y, z);
        if (x > 0) v += at(x - 1, y, z);
        if (y > 0) v += at(x, y - 1, z);
        if (z > 0) v += at(x, y, z - 1);
        if (x > 0 && y > 0) v -= at(x - 1, y - 1, z);
        if (x > 0 && z > 0) v -= at(x - 1, y, z - 1);
        if (y > 0 && z > 0) v -= at(x, y - 1, z - 1);
        if (x > 0 && y > 0 && z > 0) v += at(x - 1, y - 1, z - 1);
        at(x, y, z) = v;
        if (x < N[0] && y < N[1] && z < N[2]) best = std::max(best, v);
      }
  return best;
}

// Largest number of (image, box point) pairs inside one node's cube.  The overlap of an image
// box with the cube of node (I,J,K) is a product of three 1D overlaps, so every image adds
// ov_x(I) ov_y(J) ov_z(K) over the nodes whose cubes it meets.
long long max_box_points_per_node(const sq::Setup &s, const sq::Deck &d) {
  const int N[3] = {d.grid[0], d.grid[1], d.grid[2]};
  std::vector<long long> acc((size_t)N[0] * N[1] * N[2], 0);
  for (const sq::ImageMeta &im : s.images) {
    const sq::TypeDesc &td = s.types[im.type];
    const int b[3] = {im.bx, im.by, im.bz}, f[3] = {td.fx, td.fy, td.fz};
    std::vector<int> ov[3];
    int lo[3];
    bool empty = false;
    for (int a = 0; a < 3; a++) {
      lo[a] = std::max(0, b[a] - s.nh[a]);
      const int hi = std::min(N[a] - 1, b[a] + f[a] - 1 + s.nh[a]);
      if (hi < lo[a]) empty = true;
      for (int I = lo[a]; I <= hi; I++)
        ov[a].push_back(std::min(b[a] + f[a] - 1, I + s.nh[a]) - std::max(b[a], I - s.nh[a]) + 1);
    }
    if (empty) continue;
    for (size_t kz = 0; kz < ov[2].size(); kz++)
      for (size_t jy = 0; jy < ov[1].size(); jy++) {
        const long long yz = (long long)ov[1][jy] * ov[2][kz];
        long long *row = &acc[((size_t)(lo[2] + kz) * N[1] + (lo[1] + jy)) * N[0] + lo[0]];
        for (size_t ix = 0; ix < ov[0].size(); ix++) row[ix] += yz * ov[0][ix];
      }
  }
  long long best = 0;
  for (long long v : acc) best = std::max(best, v);
  return best;
}

// Mean over all nodes of sum_images |box ∩ cube|.  The overlap of a box with the cube of
// node (I,J,K) factorises over the axes, so the sum over the node grid is a product of
// three 1D sums per image.
double projector_points_per_node(const sq::Setup &s, const sq::Deck &d) {
  double total = 0.0;
  for (const sq::ImageMeta &im : s.images) {
    const sq::TypeDesc &td = s.types[im.type];
    const int b[3] = {im.bx, im.by, im.bz}, f[3] = {td.fx, td.fy, td.fz};
    double prod = 1.0;
    for (int a = 0; a < 3; a++) {
      long long sum = 0;
      for (int I = 0; I < d.grid[a]; I++) {
        const int lo = std::max(b[a], I - s.nh[a]), hi = std::min(b[a] + f[a] - 1, I + s.nh[a]);
        if (hi >= lo) sum += hi - lo + 1;
      }
      prod *= (double)sum;
    }
    total += prod;
  }
  return total / ((double)d.grid[0] * d.grid[1] * d.grid[2]);
}

// Fraction of projector box points inside the FP32 support sphere, over all images: the
// share of box points a per-node list keeps.
double kept_fraction(const sq::Setup &s) {
  double kept = 0.0, total = 0.0;
  for (const sq::ImageMeta &im : s.images) {
    const sq::TypeDesc &td = s.types[im.type];
    const double r2 = td.support_r2_f32;
    long long k = 0;
    for (int z = 0; z < td.fz; z++) {
      const double dz = im.oz + s.h[2] * z;
      for (int y = 0; y < td.fy; y++) {
        const double dy = im.oy + s.h[1] * y, ryz = dy * dy + dz * dz;
        for (int x = 0; x < td.fx; x++) {
          const double dx = im.ox + s.h[0] * x;
          if (dx * dx + ryz <= r2) k++;
        }
      }
    }
    kept += (double)k;
    total += (double)td.fx * td.fy * td.fz;
  }
  return total > 0.0 ? kept / total : 1.0;
}

void fill_info(sq_info &in, const sq::Deck &d, const sq::Setup &s, int max_img,
               const sq_options &opt) {
  int mask = 0;
  for (const sq::TypeDesc &t : s.types) mask |= t.chan_mask;
  in.n_lm = 0;
  for (int l = 0; l < 4; l++)
    if (mask & (1 << l)) in.n_lm += 2 * l + 1;
  in.proj_points_per_node = projector_points_per_node(s, d);
  in.kernel_layout = in.kernel_u_on_chip = in.kernel_threads = in.kernel_smem_bytes = 0;
  for (int a = 0; a < 3; a++) {
    in.grid[a] = d.grid[a];
    in.cube[a] = s.cube[a];
    in.h[a] = s.h[a];
    in.cell_half[a] = d.cell_half[a];
  }
  in.n_qp = d.n_qp;
  in.fd_half_order = d.half_order;
  in.bc = d.bc;
  in.n_atoms = (int)d.atom_type.size();
  in.n_types = (int)d.psd.size();
  in.n_images = (int)s.images.size();
  in.n_tables = s.n_tables;
  in.max_images_per_node = max_img;
  in.precision = opt.precision;
  in.faithful = opt.faithful;
  in.n_nodes = (long)d.grid[0] * d.grid[1] * d.grid[2];
  in.rcut = d.rcut;
  in.beta = d.beta;
  in.dV = s.dV;
  in.n_electrons = d.n_electrons;
}

// Host part of the engine setup: the Lanczos kernel's parameters, on-chip layout, projector
// list format, block and shared memory for a device with h->num_sms SMs, smem_optin bytes of
// opt-in shared memory per block and l2_bytes of L2.  Touches no GPU.
void plan_engine(sq_handle *h, int smem_optin, int l2_bytes) {
  const sq::Deck &d = h->deck;
  const sq::Setup &s = h->setup;
  sq::LanczosParams &p = h->lp;
  p.nx = s.cube[0];
  p.ny = s.cube[1];
  p.nz = s.cube[2];
  p.nhx = s.nh[0];
  p.nhy = s.nh[1];
  p.nhz = s.nh[2];
  p.Nx = d.grid[0];
  p.Ny = d.grid[1];
  p.Nz = d.grid[2];
  p.EX = p.Nx + 2 * p.nhx;
  p.EY = p.Ny + 2 * p.nhy;
  p.EZ = p.Nz + 2 * p.nhz;
  // FP32 vector passes work on aligned x pairs: even row pitches for P and U
  p.pitch = p.nx + sq::kStencilHalf;
  p.upitch = p.nx;
  if (h->opt.precision == 32) {
    p.pitch += p.pitch & 1;
    p.upitch += p.upitch & 1;
  }
  p.nqp = d.n_qp;
  p.n_images = (int)s.images.size();
  p.ntype = (int)s.types.size();
  p.hx = s.h[0];
  p.hy = s.h[1];
  p.hz = s.h[2];
  p.hxf = (float)p.hx;
  p.hyf = (float)p.hy;
  p.hzf = (float)p.hz;
  p.cdiag = s.c[0][0] + s.c[1][0] + s.c[2][0];
  p.cdiagf = (float)p.cdiag;
  for (int q = 0; q <= sq::kStencilHalf; q++) {
    p.cx[q] = s.c[0][q];
    p.cy[q] = s.c[1][q];
    p.cz[q] = s.c[2][q];
    p.cxf[q] = (float)p.cx[q];
    p.cyf[q] = (float)p.cy[q];
    p.czf[q] = (float)p.cz[q];
  }
  p.union_mask = 0;
  for (size_t t = 0; t < s.types.size(); t++) {
    p.types[t] = s.types[t];
    p.union_mask |= s.types[t].chan_mask;
  }
  // (l,m) ranks in the order of the instantiated channel mask (sq::lk::Lm<MASK>::rank)
  const int kmask = sq::kernel_mask(p.union_mask);
  int rank = 0;
  for (int l = 0; l < 4; l++)
    for (int m = -l; m <= l; m++) {
      const int s = l * l + l + m;
      p.lm_rank[s] = (kmask & (1 << l)) ? rank : -1;
      if (kmask & (1 << l)) p.rank_l[rank++] = l;
    }
  for (int r = rank; r < sq::kMaxLm; r++) p.rank_l[r] = 0;
  p.alpha_stride = h->opt.faithful ? 1 : rank;

  const bool wide = p.nx > 32;
  if (wide && h->opt.precision != 32)
    throw std::invalid_argument("cubes wider than 32 points in x need FP32 vectors");
  if (d.n_qp > 64) throw std::invalid_argument("LANCZOS_DEGREE above 64 is not supported");

  const int need_img = std::max(1, max_images_per_node(s, d));
  p.max_img = need_img;
  h->elem = h->opt.precision == 32 ? 4 : 8;
  const int maxw = h->opt.precision == 32 ? sq::kMaxWarpsF32 : sq::kMaxWarpsF64;
  p.rows_per_warp = (p.ny + maxw - 1) / maxw;
  h->block = 32 * ((p.ny + p.rows_per_warp - 1) / p.rows_per_warp);
  if (wide) {  // one thread per (row, x pair)
    const int tasks = p.ny * ((p.nx + 1) / 2);
    h->block = 32 * std::min(sq::kWideWarpsF32, (tasks + 31) / 32);
  }
  const bool faithful = h->opt.faithful != 0;
  h->u_smem = false;
  p.layout = 0;
  p.zchunks = 1;
  p.ychunks = 1;
  p.zsplit = 0;
  p.vring = 0;
  p.vq_row = 4 * ((p.EX + 6 + 3) / 4);  // the row of a quad-aligned Veff copy (see below)
  p.vq_copy_stride = (long long)p.vq_row * p.EY * p.EZ;
  h->quad = false;
  if (h->opt.kernel < 0 || h->opt.kernel > 2 || h->opt.tile < 0)
    throw std::invalid_argument("sq_options.kernel must be 0, 1 or 2 and tile >= 0");
  if (h->opt.precision == 32 && !faithful && h->opt.kernel != 1 && h->opt.list_format != 2) {
    // split-pass kernel over 16-byte quads: P and U on chip as [nz][ny][4 ceil(nx/4)], full
    // projector records, which must stay in L2 together (152 CTAs' lists)
    sq::LanczosParams q = p;
    q.layout = sq::kLayoutQuad;
    q.pitch = q.upitch = 4 * ((p.nx + 3) / 4);
    q.zchunks = h->opt.tile > 0 ? h->opt.tile : 2;
    const int threads = sq::lanczos_quad_threads(q);
    const double list_bytes = (double)h->num_sms * projector_points_per_node(s, d) *
                              kept_fraction(s) *
                              (double)sq::proj_record_bytes(4, false, p.union_mask, false);
    if (!wide && threads <= sq::kQuadMaxThreads &&
        sq::lanczos_quad_smem_bytes(q) <= (size_t)smem_optin &&
        (h->opt.list_format == 1 || list_bytes <= 0.75 * (double)l2_bytes)) {
      p = q;
      h->quad = true;
      h->u_smem = true;
      h->block = sq::lanczos_quad_block(q);
      p.vring = 1;  // pass A's Veff rings, where they fit (12-warp budget only)
      if (h->block > sq::kVRingThreads || sq::lanczos_quad_smem_bytes(p) > (size_t)smem_optin)
        p.vring = 0;
    } else if (h->opt.tile == 0 && p.nz >= 2 * sq::kStencilHalf + 2) {
      // the same kernel on a pair of CTAs per node, the cube split in z: each holds its half
      // of U and its half of P plus 6 halo planes; each streams its half of the list
      q.layout = sq::kLayoutQuad | sq::kLayoutPair;
      q.zsplit = (p.nz + 1) / 2;
      q.zchunks = 1;
      q.ychunks = 2;
      int pt = sq::lanczos_quad_threads(q);
      if (pt > sq::kPairThreads) {
        q.ychunks = 1;
        pt = sq::lanczos_quad_threads(q);
      }
      if (pt <= sq::kPairThreads && sq::lanczos_quad_smem_bytes(q) <= (size_t)smem_optin &&
          (h->opt.list_format == 1 || 0.5 * list_bytes <= 0.75 * (double)l2_bytes)) {
        p = q;
        p.vring = 1;
        if (sq::lanczos_quad_smem_bytes(p) > (size_t)smem_optin) p.vring = 0;
        h->quad = true;
        h->u_smem = true;
        // all 12 warps of the register budget: the stencil passes use pt threads, the list
        // streams and the update all of them (fewer, longer warp ranges are slower)
        h->block = sq::kPairThreads;
        h->tuned = true;  // one tile
      }
    }
  }
  if (h->opt.kernel == 2 && !h->quad)
    throw std::invalid_argument("the split-pass FP32 kernel does not apply to this cell and options "
                                "(FP32, corrected operator, P and U on one or two CTAs, lists in L2)");
  if (h->quad) {
    // nothing else to choose: layout, threads and lists are fixed above
  } else if (h->opt.precision == 32) {
    // first choice: y gaps and U on chip; then U on chip without the gaps (y bounds-checked);
    // then y gaps with U in global scratch
    const size_t optin = (size_t)smem_optin;
    p.layout = sq::kLayoutYGap | (wide ? sq::kLayoutWide : 0);
    if (!wide) {
      if (sq::lanczos_smem_bytes(p, 4, true, faithful) <= optin) {
        h->u_smem = true;
      } else {
        p.layout = 0;
        if (sq::lanczos_smem_bytes(p, 4, true, faithful) <= optin) h->u_smem = true;
        else p.layout = sq::kLayoutYGap;
      }
    }
  }
  if (!h->quad && h->opt.precision == 32 && !faithful && h->opt.list_format != 1) {
    // compact records when the full lists of all SMs (plus U slices in global scratch) would
    // take more than 3/4 of the L2, or on request; only if the extra per-image data fits
    bool compact = h->opt.list_format == 2;
    if (!compact) {
      const double kept = projector_points_per_node(s, d) * kept_fraction(s);
      double bytes = (double)h->num_sms * kept *
                     (double)sq::proj_record_bytes(4, false, p.union_mask, false);
      if (!h->u_smem) bytes += (double)h->num_sms * 4.0 * p.upitch * p.ny * p.nz;
      compact = bytes > 0.75 * (double)l2_bytes;
    }
    if (compact) {
      sq::LanczosParams q = p;
      q.layout |= sq::kLayoutCompact;
      if (sq::lanczos_smem_bytes(q, 4, h->u_smem, faithful) <= (size_t)smem_optin) p = q;
    }
  }
  h->smem = h->quad ? sq::lanczos_quad_smem_bytes(p)
                    : sq::lanczos_smem_bytes(p, (int)h->elem, h->u_smem, faithful);
  if (h->smem > (size_t)smem_optin && h->opt.precision == 64) {
    p.pitch = p.nx;  // rows without zero columns; the kernel bounds-checks x instead
    p.layout = sq::kLayoutXClamp;
    h->smem = sq::lanczos_smem_bytes(p, (int)h->elem, h->u_smem, faithful);
  }
  if (h->smem > (size_t)smem_optin)
    throw std::invalid_argument("cube of " + std::to_string(p.nx) + "x" + std::to_string(p.ny) +
                                "x" + std::to_string(p.nz) +
                                " does not fit in shared memory at this precision");
  h->grid = h->num_sms;
  if (!h->quad) {  // projector records pack the P and U indices of a cube point into 16 bits each
    const long long pitch_rows = (p.layout & sq::kLayoutYGap) ? p.ny + sq::kStencilHalf : p.ny;
    const long long psize = (long long)sq::kStencilHalf * p.pitch + (long long)p.nz * pitch_rows * p.pitch;
    if (psize >= 65536 || (long long)p.upitch * p.ny * p.nz >= 65536)
      throw std::invalid_argument("truncated cube too large for 16-bit point indices");
  }
  const long long cap = std::max(1LL, max_box_points_per_node(s, d));
  if (cap > (1LL << 31) - 1) throw std::invalid_argument("projector list too large");
  p.proj_cap = (int)cap;
  p.proj_bytes_per_cta =
      (long long)((cap * sq::proj_record_bytes((int)h->elem, faithful, p.union_mask,
                                               (p.layout & sq::kLayoutCompact) != 0) +
                   255) & ~255LL);
  fill_info(h->info, d, s, p.max_img, h->opt);
  h->info.kernel_layout = p.layout;
  h->info.kernel_u_on_chip = h->u_smem ? 1 : 0;
  h->info.kernel_threads = h->block;
  h->info.kernel_smem_bytes = (int)h->smem;
}

void build_engine(sq_handle *h) {
  ck(cudaSetDevice(h->opt.device), "cudaSetDevice");
  ck(cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->opt.device), "sm count");
  int smem_optin = 0, l2 = 0;
  ck(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->opt.device),
     "smem optin");
  ck(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, h->opt.device), "L2 size");
  plan_engine(h, smem_optin, l2);
  if (h->lp.layout & sq::kLayoutPair) {  // no more pairs than fit on the device at once
    const int pairs = sq::lanczos_quad_pair_clusters(h->lp, h->block, h->smem);
    if (pairs < 1) throw std::runtime_error("no cluster of two CTAs fits this kernel on the device");
    h->grid = std::min(h->grid / 2, pairs) * 2;
  }
  ck(cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking), "stream");
  for (auto &e : h->ev) ck(cudaEventCreate(&e), "event");
  const sq::Setup &s = h->setup;
  const sq::LanczosParams &p = h->lp;

  // device buffers
  dev_alloc(&h->d_images, sizeof(sq::ImageMeta) * s.images.size(), "images");
  ck(cudaMemcpy(h->d_images, s.images.data(), sizeof(sq::ImageMeta) * s.images.size(),
                cudaMemcpyHostToDevice), "images H2D");
  dev_alloc(&h->d_tables, h->elem * s.tables.size(), "tables");
  if (h->opt.precision == 32) {
    std::vector<float> t32(s.tables.begin(), s.tables.end());
    ck(cudaMemcpy(h->d_tables, t32.data(), 4 * t32.size(), cudaMemcpyHostToDevice), "tables H2D");
  } else {
    ck(cudaMemcpy(h->d_tables, s.tables.data(), 8 * s.tables.size(), cudaMemcpyHostToDevice),
       "tables H2D");
  }
  dev_alloc(&h->d_veff_ext,
            h->quad ? sizeof(float) * sq::veff_quad_floats(p) : h->elem * (size_t)p.EX * p.EY * p.EZ,
            "veff_ext");
  dev_alloc(&h->d_veff_in, sizeof(double) * (size_t)p.Nx * p.Ny * p.Nz, "veff");
  if (!h->u_smem) {
    const size_t nc4 = ((size_t)p.upitch * p.ny * p.nz + 3) & ~size_t(3);
    dev_alloc(&h->d_u, h->elem * nc4 * h->grid, "U scratch");
  }
  dev_alloc(&h->d_proj, (size_t)p.proj_bytes_per_cta * h->grid, "projector list scratch");
  dev_alloc(&h->d_status, sizeof(int) * 4, "status");
  ck(cudaMemset(h->d_status, 0, sizeof(int) * 4), "status memset");
  h->fermi_grid = h->num_sms;
  dev_alloc(&h->d_fermi_scratch, sizeof(double) * sq::fermi_scratch_doubles(h->fermi_grid, h->fermi_maxit),
            "fermi scratch");
  dev_alloc(&h->d_bar, sizeof(unsigned) * 2, "barrier");
  dev_alloc(&h->d_fermi_out, sizeof(double) * 4, "fermi out");
}

}  // namespace

namespace sq {

sq_status device_status(sq_handle *h, cudaStream_t s) {
  int st = 0;
  ck(cudaMemcpyAsync(&st, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, s), "status D2H");
  ck(cudaStreamSynchronize(s), "sync");
  // the upstream cause first: a Lanczos breakdown (b_k zero or not finite) also leaves a
  // tridiagonal that QL may not converge on
  if (st & sq::kStatusTimeout) return fail(SQ_DEVICE_TIMEOUT, "a device-side wait gave up");
  if (st & sq::kStatusCapacity) return fail(SQ_CAPACITY, "per-node image list overflow");
  if (st & sq::kStatusBreakdown)
    return fail(SQ_LANCZOS_BREAKDOWN, "Lanczos breakdown (b_k zero or not finite)");
  if (st & sq::kStatusNoConvergence)
    return fail(SQ_NO_CONVERGENCE, "Too many iterations in Tridiagonal solver");
  return SQ_OK;
}

void ensure_quadrature_buffers(sq_handle *h, long long n) {
  const long long nq = n * h->lp.nqp;
  long long cap = h->out_cap;
  ensure_capacity(h->d_lambda, cap, nq, "lambda");
  cap = h->out_cap;
  ensure_capacity(h->d_w, cap, nq, "weights");
  cap = h->out_cap;
  ensure_capacity(h->d_lmin, cap, std::max(nq, n), "lambda_min");
  cap = h->out_cap;
  ensure_capacity(h->d_lmax, cap, std::max(nq, n), "lambda_max");
  h->out_cap = std::max(h->out_cap, nq);
}

void update_node_cost(sq_handle *h) {
  if (!h->ev_valid || h->cost_nodes <= 0) return;
  if (cudaEventQuery(h->ev[1]) != cudaSuccess) {
    cudaGetLastError();  // a pending event is not an error
    return;
  }
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]) == cudaSuccess && ms > 0.f)
    h->node_sm_ms = (double)ms * h->cost_grid / (double)h->cost_nodes;
  cudaGetLastError();
  h->cost_nodes = 0;
}

sq_status run_device(sq_handle *h, const double *d_veff, double veff_const, long long nb,
                     long long ne, double *d_lambda, double *d_w, double *d_lmin, double *d_lmax,
                     cudaStream_t s, int grid_limit) {
  const long long n = ne - nb;
  if (nb < 0 || ne > h->info.n_nodes || n <= 0)
    return fail(SQ_BAD_INPUT, "node range outside the grid");
  ensure_capacity(h->d_ab, h->ab_cap, 2 * (long long)h->lp.nqp * n, "lanczos coefficients");
  sq::LanczosParams p = h->lp;
  p.node_begin = nb;
  p.node_end = ne;
  ck(cudaMemsetAsync(h->d_status, 0, sizeof(int), s), "status reset");
  ck(sq::launch_veff_extend(d_veff, veff_const, h->d_veff_ext, h->opt.precision, p, s), "veff");
  int grid = (int)std::min<long long>(grid_limit > 0 ? std::min(grid_limit, h->grid) : h->grid, n);
  if (p.layout & sq::kLayoutPair)  // two CTAs per node: an even grid, one pair per node at most
    grid = 2 * (int)std::max<long long>(
                   1, std::min<long long>((grid_limit > 0 ? std::min(grid_limit, h->grid) : h->grid) / 2, n));
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  ck(cudaStreamIsCapturing(s, &cap), "capture status");
  const bool timed = cap == cudaStreamCaptureStatusNone;  // no timing events inside a graph
  if (h->quad && !h->tuned && h->opt.tile == 0 && timed && n >= 2LL * grid) {
    // autotune the split-pass kernel's tile (z- / y-ranges per row / plane) on this call's
    // first nodes, one node per CTA per candidate, and keep the fastest for the handle
    cudaEvent_t t0, t1;
    ck(cudaEventCreate(&t0), "event");
    ck(cudaEventCreate(&t1), "event");
    float best = 1e30f;
    int best_tile = p.zchunks;
    for (int tile = 1; tile <= 4; tile++) {
      sq::LanczosParams q = p;
      q.zchunks = tile;
      q.node_end = nb + grid;
      const int threads = sq::lanczos_quad_threads(q);
      if (threads > sq::kQuadMaxThreads) break;
      float ms = 0.f;
      for (int rep = 0; rep < 2; rep++) {  // the first launch of a tile loads its code
        ck(cudaEventRecord(t0, s), "event");
        ck(sq::launch_lanczos(q, 32, false, true, grid, sq::lanczos_quad_block(q), h->smem, s,
                              h->d_veff_ext,
                              h->d_images, h->d_tables, h->d_u, h->d_proj, h->d_ab, h->d_status),
           "lanczos (tile probe)");
        ck(cudaEventRecord(t1, s), "event");
        ck(cudaEventSynchronize(t1), "event");
        ck(cudaEventElapsedTime(&ms, t0, t1), "event");
      }
      if (ms < best) {
        best = ms;
        best_tile = tile;
      }
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    h->lp.zchunks = p.zchunks = best_tile;
    h->block = sq::lanczos_quad_block(p);
    h->info.kernel_threads = h->block;
    h->tuned = true;
  }
  if (timed) {
    update_node_cost(h);
    h->cost_grid = grid;
    h->cost_nodes = n;
    ck(cudaEventRecord(h->ev[0], s), "event");
  }
  ck(sq::launch_lanczos(p, h->opt.precision, h->opt.faithful != 0, h->u_smem, grid, h->block, h->smem, s,
                        h->d_veff_ext, h->d_images, h->d_tables, h->d_u, h->d_proj, h->d_ab,
                        h->d_status),
     "lanczos");
  if (timed) ck(cudaEventRecord(h->ev[1], s), "event");
  ck(sq::launch_quadrature(h->d_ab, n, p.nqp, d_lambda, d_w, d_lmin, d_lmax, h->d_status, s),
     "quadrature");
  if (timed) ck(cudaEventRecord(h->ev[2], s), "event");
  h->ev_valid = timed;
  h->last_n = n;
  return SQ_OK;
}


}  // namespace sq

namespace {
sq_status describe(const sq::Deck &d, int faithful, sq_info *info, double *gamma, double *cutoff) {
  sq::Setup s = sq::build_setup(d, faithful != 0);
  sq_options opt{faithful, 0, 0, 0, 0, 0};
  *info = sq_info{};
  fill_info(*info, d, s, max_images_per_node(s, d), opt);
  for (size_t t = 0; t < s.types.size(); t++) {
    if (gamma)
      for (int l = 0; l < 4; l++) gamma[4 * t + l] = s.types[t].gamma[l];
    if (cutoff)
      for (int a = 0; a < 3; a++) cutoff[3 * t + a] = s.pseudocharge_cutoff[3 * t + a];
  }
  return SQ_OK;
}

// sq_create_from_deck and sq_create share everything after the deck is in memory.
sq_status create_from(const std::function<sq::Deck()> &deck, const sq_options *opt,
                      sq_handle **out) {
  *out = nullptr;
  sq_handle *h = new sq_handle();
  sq_status st = guarded([&] {
    h->opt = opt ? *opt : sq_options{0, 32, 0, 0, 0, 0};
    if (h->opt.precision != 32 && h->opt.precision != 64)
      return fail(SQ_BAD_INPUT, "precision must be 32 or 64");
    if (h->opt.list_format < 0 || h->opt.list_format > 2)
      return fail(SQ_BAD_INPUT, "list_format must be 0, 1 or 2");
    h->deck = deck();
    h->setup = sq::build_setup(h->deck, h->opt.faithful != 0);
    build_engine(h);
    return SQ_OK;
  });
  if (st != SQ_OK) {
    delete h;
    return st;
  }
  *out = h;
  return SQ_OK;
}
}  // namespace

extern "C" {

sq_status sq_create_from_deck(const char *deck_dir, const char *name, const sq_options *opt,
                              sq_handle **out) {
  if (!out || !deck_dir || !name) return fail(SQ_BAD_INPUT, "null argument");
  const std::string dir(deck_dir), nm(name);
  return create_from([&] { return sq::read_deck(dir, nm); }, opt, out);
}

void sq_destroy(sq_handle *h) { delete h; }


sq_status sq_create(const sq_system_desc *sys, const sq_options *opt, sq_handle **out) {
  if (!out || !sys) return fail(SQ_BAD_INPUT, "null argument");
  return create_from([&] { return sq::deck_from_system(*sys); }, opt, out);
}

sq_status sq_describe_system(const sq_system_desc *sys, int faithful, sq_info *info,
                             double *gamma, double *cutoff) {
  if (!sys || !info) return fail(SQ_BAD_INPUT, "null argument");
  return guarded([&] { return describe(sq::deck_from_system(*sys), faithful, info, gamma, cutoff); });
}

sq_status sq_describe_deck(const char *deck_dir, const char *name, int faithful, sq_info *info,
                           double *gamma, double *cutoff) {
  if (!deck_dir || !name || !info) return fail(SQ_BAD_INPUT, "null argument");
  return guarded([&] {
    sq::Deck d = sq::read_deck(deck_dir, name);
    return describe(d, faithful, info, gamma, cutoff);
  });
}

sq_status sq_plan_kernel(const char *deck_dir, const char *name, const sq_options *opt,
                         int num_sms, int smem_optin, int l2_bytes, sq_info *info) {
  if (!deck_dir || !name || !opt || !info) return fail(SQ_BAD_INPUT, "null argument");
  if (num_sms <= 0 || smem_optin <= 0 || l2_bytes <= 0)
    return fail(SQ_BAD_INPUT, "device properties must be positive");
  if (opt->precision != 32 && opt->precision != 64)
    return fail(SQ_BAD_INPUT, "precision must be 32 or 64");
  if (opt->list_format < 0 || opt->list_format > 2)
    return fail(SQ_BAD_INPUT, "list_format must be 0, 1 or 2");
  sq_handle h;  // host fields only: no device buffer, stream or event is created
  return guarded([&] {
    h.opt = *opt;
    h.deck = sq::read_deck(deck_dir, name);
    h.setup = sq::build_setup(h.deck, opt->faithful != 0);
    h.num_sms = num_sms;
    plan_engine(&h, smem_optin, l2_bytes);
    *info = h.info;
    return SQ_OK;
  });
}

sq_status sq_describe_scf_fields(const char *deck_dir, const char *name, double *b, double *rho0,
                                 double *green, double *scalars) {
  if (!deck_dir || !name) return fail(SQ_BAD_INPUT, "null argument");
  return guarded([&] {
    sq::Deck d = sq::read_deck(deck_dir, name);
    sq::Setup s = sq::build_setup(d, false);
    sq::ScfFields f = sq::build_scf_fields(d, s);
    if (b) std::copy(f.b.begin(), f.b.end(), b);
    if (rho0) std::copy(f.rho0.begin(), f.rho0.end(), rho0);
    if (green) std::copy(f.green.begin(), f.green.end(), green);
    if (scalars) {
      scalars[0] = f.e_self;
      scalars[1] = f.e_self_ref;
      scalars[2] = f.e_corr;
      scalars[3] = f.b_total;
    }
    return SQ_OK;
  });
}

sq_status sq_get_info(const sq_handle *h, sq_info *info) {
  if (!h || !info) return fail(SQ_BAD_INPUT, "null argument");
  *info = h->info;
  return SQ_OK;
}

sq_status sq_nodes_and_weights_device(sq_handle *h, const double *d_veff, double veff_const,
                                      long node_begin, long node_end, double *d_lambda,
                                      double *d_weights, double *d_lambda_min,
                                      double *d_lambda_max, void *stream) {
  if (!h || !d_lambda || !d_weights || !d_lambda_min || !d_lambda_max)
    return fail(SQ_BAD_INPUT, "null argument");
  return guarded([&] {
    ck(cudaSetDevice(h->opt.device), "cudaSetDevice");
    return run_device(h, d_veff, veff_const, node_begin, node_end, d_lambda, d_weights,
                      d_lambda_min, d_lambda_max, (cudaStream_t)stream);
  });
}

sq_status sq_sync_status(sq_handle *h, void *stream) {
  if (!h) return fail(SQ_BAD_INPUT, "null argument");
  return guarded([&] { return device_status(h, (cudaStream_t)stream); });
}

sq_status sq_nodes_and_weights(sq_handle *h, const double *veff, double veff_const,
                               long node_begin, long node_end, double *lambda, double *weights,
                               double *lambda_min, double *lambda_max) {
  if (!h || !lambda || !weights || !lambda_min || !lambda_max)
    return fail(SQ_BAD_INPUT, "null argument");
  return guarded([&] {
    ck(cudaSetDevice(h->opt.device), "cudaSetDevice");
    cudaStream_t s = h->own_stream;
    const long long n = (long long)node_end - node_begin;
    if (n <= 0 || node_begin < 0 || node_end > h->info.n_nodes)
      return fail(SQ_BAD_INPUT, "node range outside the grid");
    const long long q = h->lp.nqp;
    ensure_quadrature_buffers(h, n);
    const double *dv = nullptr;
    if (veff) {
      ck(cudaMemcpyAsync(h->d_veff_in, veff, sizeof(double) * h->info.n_nodes,
                         cudaMemcpyHostToDevice, s), "veff H2D");
      dv = h->d_veff_in;
    }
    sq_status st = run_device(h, dv, veff_const, node_begin, node_end, h->d_lambda, h->d_w,
                              h->d_lmin, h->d_lmax, s);
    if (st != SQ_OK) return st;
    ck(cudaMemcpyAsync(lambda, h->d_lambda, sizeof(double) * n * q, cudaMemcpyDeviceToHost, s), "D2H");
    ck(cudaMemcpyAsync(weights, h->d_w, sizeof(double) * n * q, cudaMemcpyDeviceToHost, s), "D2H");
    ck(cudaMemcpyAsync(lambda_min, h->d_lmin, sizeof(double) * n, cudaMemcpyDeviceToHost, s), "D2H");
    ck(cudaMemcpyAsync(lambda_max, h->d_lmax, sizeof(double) * n, cudaMemcpyDeviceToHost, s), "D2H");
    return device_status(h, s);
  });
}

sq_status sq_copy_lanczos_coefficients(sq_handle *h, double *a, double *b, long n) {
  if (!h || !a || !b) return fail(SQ_BAD_INPUT, "null argument");
  return guarded([&] {
    if (n > h->last_n) return fail(SQ_BAD_INPUT, "more nodes requested than the last call computed");
    const int q = h->lp.nqp;
    std::vector<double> ab((size_t)2 * q * n);
    ck(cudaStreamSynchronize(h->own_stream), "sync");
    ck(cudaDeviceSynchronize(), "sync");
    ck(cudaMemcpy(ab.data(), h->d_ab, sizeof(double) * ab.size(), cudaMemcpyDeviceToHost), "ab D2H");
    for (long i = 0; i < n; i++)
      for (int k = 0; k < q; k++) {
        a[i * q + k] = ab[(size_t)i * 2 * q + k];
        b[i * q + k] = ab[(size_t)i * 2 * q + q + k];
      }
    return SQ_OK;
  });
}

sq_status sq_fermi_density_energy_device(sq_handle *h, const double *d_lambda,
                                         const double *d_weights, long n_nodes,
                                         double n_electrons, double tol, double *lambda_f,
                                         double *d_rho, double *e_band, double *ts,
                                         void *stream) {
  if (!h || !d_lambda || !d_weights || !lambda_f || !e_band || !ts)
    return fail(SQ_BAD_INPUT, "null argument");
  return guarded([&] {
    if (n_nodes <= 0) return fail(SQ_BAD_INPUT, "n_nodes must be positive");
    ck(cudaSetDevice(h->opt.device), "cudaSetDevice");
    cudaStream_t s = (cudaStream_t)stream;
    ck(cudaMemsetAsync(h->d_status, 0, sizeof(int), s), "status reset");
    ck(sq::launch_fermi(d_lambda, d_weights, n_nodes, h->lp.nqp, h->info.beta, n_electrons,
                        h->info.dV, tol, h->fermi_maxit, d_rho, h->d_fermi_out,
                        h->d_fermi_scratch, h->d_bar, h->d_status, h->fermi_grid, s),
       "fermi");
    double outv[4];
    ck(cudaMemcpyAsync(outv, h->d_fermi_out, sizeof(outv), cudaMemcpyDeviceToHost, s), "D2H");
    sq_status st = device_status(h, s);
    if (st != SQ_OK) return st;
    *lambda_f = outv[0];
    *e_band = outv[1];
    *ts = outv[2];
    return SQ_OK;
  });
}

sq_status sq_fermi_density_energy(sq_handle *h, const double *lambda, const double *weights,
                                  long n_nodes, double n_electrons, double tol, double *lambda_f,
                                  double *rho, double *e_band, double *ts) {
  if (!h || !lambda || !weights || !lambda_f || !e_band || !ts)
    return fail(SQ_BAD_INPUT, "null argument");
  return guarded([&] {
    if (n_nodes <= 0) return fail(SQ_BAD_INPUT, "n_nodes must be positive");
    ck(cudaSetDevice(h->opt.device), "cudaSetDevice");
    cudaStream_t s = h->own_stream;
    const long long nq = (long long)n_nodes * h->lp.nqp;
    ensure_quadrature_buffers(h, n_nodes);
    ensure_capacity(h->d_rho, h->rho_cap, n_nodes, "rho");
    ck(cudaMemcpyAsync(h->d_lambda, lambda, sizeof(double) * nq, cudaMemcpyHostToDevice, s), "H2D");
    ck(cudaMemcpyAsync(h->d_w, weights, sizeof(double) * nq, cudaMemcpyHostToDevice, s), "H2D");
    sq_status st = sq_fermi_density_energy_device(h, h->d_lambda, h->d_w, n_nodes, n_electrons,
                                                  tol, lambda_f, h->d_rho, e_band, ts, s);
    if (st != SQ_OK) return st;
    if (rho) {
      ck(cudaMemcpyAsync(rho, h->d_rho, sizeof(double) * n_nodes, cudaMemcpyDeviceToHost, s), "D2H");
      ck(cudaStreamSynchronize(s), "sync");
    }
    return SQ_OK;
  });
}

sq_status sq_electron_count_device(sq_handle *h, const double *d_lambda, const double *d_weights,
                                   long n_nodes, double lambda_f, double *count, void *stream) {
  if (!h || !d_lambda || !d_weights || !count) return fail(SQ_BAD_INPUT, "null argument");
  return guarded([&] {
    if (n_nodes <= 0) return fail(SQ_BAD_INPUT, "n_nodes must be positive");
    ck(cudaSetDevice(h->opt.device), "cudaSetDevice");
    cudaStream_t s = (cudaStream_t)stream;
    const int grid = 4 * h->num_sms;  // <= fermi scratch rows (maxit + 4) * fermi_grid
    double *partial = h->d_fermi_scratch, *out = h->d_fermi_out;
    ck(sq::launch_electron_count(d_lambda, d_weights, n_nodes, h->lp.nqp, h->info.beta, lambda_f,
                                 partial, grid, out, s),
       "electron count");
    ck(cudaMemcpyAsync(count, out, sizeof(double), cudaMemcpyDeviceToHost, s), "D2H");
    ck(cudaStreamSynchronize(s), "sync");
    return SQ_OK;
  });
}

sq_status sq_last_kernel_times(sq_handle *h, double *ms) {
  if (!h || !ms) return fail(SQ_BAD_INPUT, "null argument");
  return guarded([&] {
    if (!h->ev_valid) return fail(SQ_BAD_INPUT, "no nodes_and_weights call yet");
    ck(cudaEventSynchronize(h->ev[2]), "event sync");
    float a = 0, b = 0;
    ck(cudaEventElapsedTime(&a, h->ev[0], h->ev[1]), "elapsed");
    ck(cudaEventElapsedTime(&b, h->ev[1], h->ev[2]), "elapsed");
    ms[0] = a;
    ms[1] = b;
    return SQ_OK;
  });
}

sq_status sq_measure_fp32_peak(int device, double *tflops) {
  if (!tflops) return fail(SQ_BAD_INPUT, "null argument");
  return guarded([&] {
    ck(cudaSetDevice(device), "cudaSetDevice");
    ck(sq::measure_fp32_peak(device, tflops), "fp32 probe");
    return SQ_OK;
  });
}

sq_status sq_batch_nodes_and_weights(sq_handle *const *cells, int n_cells, const double *const *d_veff,
                                     const double *veff_const, double *const *d_lambda,
                                     double *const *d_weights, double *const *d_lambda_min,
                                     double *const *d_lambda_max, void *stream) {
  if (!cells || n_cells <= 0 || !d_lambda || !d_weights || !d_lambda_min || !d_lambda_max)
    return fail(SQ_BAD_INPUT, "null argument");
  return guarded([&] {
    for (int c = 0; c < n_cells; c++) {
      if (!cells[c] || !d_lambda[c] || !d_weights[c] || !d_lambda_min[c] || !d_lambda_max[c])
        return fail(SQ_BAD_INPUT, "null cell argument");
      if (cells[c]->opt.device != cells[0]->opt.device)
        return fail(SQ_BAD_INPUT, "all cells of a batch on one device");
      for (int o = 0; o < c; o++)
        if (cells[o] == cells[c]) return fail(SQ_BAD_INPUT, "a handle appears twice in the batch");
    }
    ck(cudaSetDevice(cells[0]->opt.device), "cudaSetDevice");
    const int sms = cells[0]->num_sms;
    if (n_cells > sms) return fail(SQ_BAD_INPUT, "more cells than SMs in one batch");
    // Work per cell: nodes x the measured cost of a node on one SM when every cell has run
    // before (the split then follows the kernels' real speeds), else nodes x per-node FLOPs.
    bool measured = true;
    for (int c = 0; c < n_cells; c++) {
      update_node_cost(cells[c]);
      if (!(cells[c]->node_sm_ms > 0.0)) measured = false;
    }
    std::vector<double> per_node(n_cells);
    for (int c = 0; c < n_cells; c++) {
      const sq_info &in = cells[c]->info;
      const double nc = (double)in.cube[0] * in.cube[1] * in.cube[2];
      per_node[c] = measured ? cells[c]->node_sm_ms
                             : in.n_qp * ((2.0 * (6 * in.fd_half_order + 1) + 9.0) * nc +
                                          4.0 * in.n_lm * in.proj_points_per_node);
    }
    // one SM each, then every further SM to the cell that would finish last; a cell's finish
    // time counts whole rounds of nodes, ceil(nodes / SMs) x cost per node
    std::vector<int> share(n_cells, 1);
    auto finish = [&](int c, int sh) {
      return std::ceil((double)cells[c]->info.n_nodes / sh) * per_node[c];
    };
    for (int left = sms - n_cells; left > 0; left--) {
      int worst = 0;
      for (int c = 1; c < n_cells; c++)
        if (finish(c, share[c]) > finish(worst, share[worst])) worst = c;
      if (share[worst] >= cells[worst]->info.n_nodes) break;  // more SMs would idle
      share[worst]++;
    }
    // fork: every cell's stream waits for the caller's stream and runs its cell on its SM
    // share; the caller's stream waits for all of them
    cudaStream_t s = (cudaStream_t)stream;
    cudaEvent_t fork = nullptr;
    ck(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming), "event");
    std::vector<cudaEvent_t> join(n_cells, nullptr);
    sq_status st = SQ_OK;
    ck(cudaEventRecord(fork, s), "event");
    for (int c = 0; c < n_cells && st == SQ_OK; c++) {
      sq_handle *h = cells[c];
      ck(cudaStreamWaitEvent(h->own_stream, fork, 0), "wait");
      st = run_device(h, d_veff ? d_veff[c] : nullptr, veff_const ? veff_const[c] : 0.0, 0,
                      h->info.n_nodes, d_lambda[c], d_weights[c], d_lambda_min[c],
                      d_lambda_max[c], h->own_stream, share[c]);
      ck(cudaEventCreateWithFlags(&join[c], cudaEventDisableTiming), "event");
      ck(cudaEventRecord(join[c], h->own_stream), "event");
      ck(cudaStreamWaitEvent(s, join[c], 0), "wait");
    }
    cudaEventDestroy(fork);
    for (cudaEvent_t e : join)
      if (e) cudaEventDestroy(e);
    if (st != SQ_OK) return st;
    for (int c = 0; c < n_cells; c++) {
      st = device_status(cells[c], cells[c]->own_stream);
      if (st != SQ_OK) return st;
    }
    return SQ_OK;
  });
}

sq_status sq_tridiag_nodes_and_weights(const double *a, const double *b, long n_nodes, int n_qp,
                                       double *lambda, double *weights, double *lambda_min,
                                       double *lambda_max, int device) {
  if (!a || !b || !lambda || !weights || !lambda_min || !lambda_max)
    return fail(SQ_BAD_INPUT, "null argument");
  if (n_nodes <= 0 || n_qp <= 0 || n_qp > 64)
    return fail(SQ_BAD_INPUT, "n_nodes must be positive and n_qp in 1..64");
  return guarded([&] {
    ck(cudaSetDevice(device), "cudaSetDevice");
    const size_t nq = (size_t)n_nodes * n_qp;
    std::vector<double> ab(2 * nq);  // the kernel's [node][a | b] rows
    for (long i = 0; i < n_nodes; i++) {
      std::memcpy(&ab[(size_t)i * 2 * n_qp], a + (size_t)i * n_qp, sizeof(double) * n_qp);
      std::memcpy(&ab[(size_t)i * 2 * n_qp + n_qp], b + (size_t)i * n_qp, sizeof(double) * n_qp);
    }
    sq::DevBuf<double> d_ab(sizeof(double) * ab.size(), "ab");
    sq::DevBuf<double> d_out(sizeof(double) * (2 * nq + 2 * (size_t)n_nodes), "quadrature");
    sq::DevBuf<int> d_st(sizeof(int), "status");
    double *dl = d_out.get(), *dw = dl + nq, *dmin = dw + nq, *dmax = dmin + n_nodes;
    ck(cudaMemcpy(d_ab.get(), ab.data(), sizeof(double) * ab.size(), cudaMemcpyHostToDevice), "H2D");
    ck(cudaMemset(d_st.get(), 0, sizeof(int)), "status reset");
    ck(sq::launch_quadrature(d_ab.get(), n_nodes, n_qp, dl, dw, dmin, dmax, d_st.get(), 0),
       "quadrature");
    int st = 0;
    ck(cudaMemcpy(&st, d_st.get(), sizeof(int), cudaMemcpyDeviceToHost), "D2H");
    ck(cudaMemcpy(lambda, dl, sizeof(double) * nq, cudaMemcpyDeviceToHost), "D2H");
    ck(cudaMemcpy(weights, dw, sizeof(double) * nq, cudaMemcpyDeviceToHost), "D2H");
    ck(cudaMemcpy(lambda_min, dmin, sizeof(double) * n_nodes, cudaMemcpyDeviceToHost), "D2H");
    ck(cudaMemcpy(lambda_max, dmax, sizeof(double) * n_nodes, cudaMemcpyDeviceToHost), "D2H");
    if (st & sq::kStatusNoConvergence)
      return fail(SQ_NO_CONVERGENCE, "Too many iterations in Tridiagonal solver");
    return SQ_OK;
  });
}

sq_status sq_fermi_timeout_selftest(int device) {
  return guarded([&] {
    ck(cudaSetDevice(device), "cudaSetDevice");
    int sms = 0;
    ck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "sm count");
    const int grid = std::max(2, std::min(sms, 64));
    const long long n = 4096, nqp = 4;
    std::vector<double> lam(n * nqp), w(n * nqp, 1.0 / nqp);
    for (size_t i = 0; i < lam.size(); i++) lam[i] = -1.0 + 2.0 * (double)i / (double)lam.size();
    sq::DevBuf<double> d_in(sizeof(double) * 2 * lam.size(), "inputs");
    sq::DevBuf<double> d_scr(sizeof(double) * ((size_t)grid * 16 + 4), "scratch");
    sq::DevBuf<unsigned> d_bar(sizeof(unsigned) * 2, "barrier");
    sq::DevBuf<int> d_st(sizeof(int), "status");
    ck(cudaMemcpy(d_in.get(), lam.data(), sizeof(double) * lam.size(), cudaMemcpyHostToDevice), "H2D");
    ck(cudaMemcpy(d_in.get() + lam.size(), w.data(), sizeof(double) * w.size(),
                  cudaMemcpyHostToDevice), "H2D");
    ck(cudaMemset(d_st.get(), 0, sizeof(int)), "status reset");
    ck(sq::launch_fermi_timeout_selftest(d_in.get(), d_in.get() + lam.size(), n, (int)nqp,
                                         d_scr.get() + (size_t)grid * 16, d_scr.get(), d_bar.get(),
                                         d_st.get(), grid, 0),
       "fermi (timeout self-test)");
    ck(cudaDeviceSynchronize(), "sync");
    int st = 0;
    ck(cudaMemcpy(&st, d_st.get(), sizeof(int), cudaMemcpyDeviceToHost), "D2H");
    if (st & sq::kStatusTimeout) return fail(SQ_DEVICE_TIMEOUT, "a device-side wait gave up");
    return SQ_OK;
  });
}

const char *sq_last_error_string(void) { return sq::last_error().c_str(); }

}  // extern "C"

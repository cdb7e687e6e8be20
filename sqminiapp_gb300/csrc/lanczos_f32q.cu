// lanczos_f32q.cu -- instantiations of the split-pass FP32 Lanczos kernel (kLayoutQuad) and its
// host-side sizes.
#include "lanczos_quad.cuh"

namespace sq {

int lanczos_quad_threads(const LanczosParams &p) {
  // pitch/4 threads per row (pass A) or plane (pass B), zchunks ranges each (a pair: rows
  // over the owned planes, zchunks z-ranges; owned planes, ychunks y-ranges)
  // at least two warps: warp 0 builds the per-node image list while the others clear P and U
  const int groups = (p.layout & kLayoutPair)
                         ? std::max(p.ny * p.zchunks, lq::pair_u_planes(p.nz, p.zsplit) * p.ychunks)
                         : std::max(p.ny, p.nz) * p.zchunks;
  return std::max(64, 32 * (((p.pitch / 4) * groups + 31) / 32));
}

int lanczos_quad_block(const LanczosParams &p) {
  // every warp of the register budget (12 warps at up to 384 threads, 16 above): the passes
  // use lanczos_quad_threads of them, the list streams and the update all
  const int t = lanczos_quad_threads(p);
  if (t <= 256) return t;
  return t <= 384 ? 384 : kQuadMaxThreads;
}

size_t lanczos_quad_smem_bytes(const LanczosParams &p) {
  const bool pair = (p.layout & kLayoutPair) != 0;
  const size_t ps = lq::quad_plane_floats(p.ny, p.pitch);
  const int nlm = mask_nlm(kernel_mask(p.union_mask));
  size_t b = pair ? sizeof(float) * ps * (lq::pair_p_planes(p.nz, p.zsplit) +
                                          lq::pair_u_planes(p.nz, p.zsplit))
                  : sizeof(float) * 2 * ps * p.nz;           // P, U
  b += sizeof(double) * (2 * lk::kMaxWarps + 128);           // a_k / b_k partials, a[], b[]
  b += sizeof(float) * (2 * (size_t)p.max_img + lk::kMaxWarps) * nlm;  // c partials, alpha
  if (pair)  // both CTAs' c, an 8-byte alignment, projector a_k partials, capacity flags
    b += sizeof(float) * 2 * (size_t)p.max_img * nlm + 8 + sizeof(float) * 2 * lk::kMaxWarps +
         sizeof(int) * 4;
  b += sizeof(int) * (9 * (size_t)p.max_img + 2) + sizeof(int) * 4;    // per-node image lists
  if (p.vring) b += 16 + sizeof(float) * 4 * kVRingSlots * kVRingThreads;  // Veff rings
  return b;
}

size_t veff_quad_floats(const LanczosParams &p) { return 4 * (size_t)p.vq_copy_stride; }

namespace {
template <int MAXT, bool ISO>
cudaError_t launch_quad_mask(int mask, const LanczosParams &p, int grid, int block, size_t smem,
                             cudaStream_t s, const void *veffq, const ImageMeta *images,
                             const void *tables, void *proj_scratch, double *ab, int *status) {
  switch (mask) {
    case 3: return lq::launch_quad_variant<3, MAXT, ISO>(p, grid, block, smem, s, veffq, images, tables, proj_scratch, ab, status);
    case 5: return lq::launch_quad_variant<5, MAXT, ISO>(p, grid, block, smem, s, veffq, images, tables, proj_scratch, ab, status);
    case 6: return lq::launch_quad_variant<6, MAXT, ISO>(p, grid, block, smem, s, veffq, images, tables, proj_scratch, ab, status);
    case 7: return lq::launch_quad_variant<7, MAXT, ISO>(p, grid, block, smem, s, veffq, images, tables, proj_scratch, ab, status);
    default: return lq::launch_quad_variant<15, MAXT, ISO>(p, grid, block, smem, s, veffq, images, tables, proj_scratch, ab, status);
  }
}
}  // namespace

// Two register budgets: up to 12 warps (3 per SM sub-partition: 168 registers a thread) and up
// to 16 warps (128).  Isotropic meshes (hx = hy = hz) share one set of stencil weights.
cudaError_t launch_lanczos_f32_quad(int mask, const LanczosParams &p, int grid, int block,
                                    size_t smem, cudaStream_t s, const void *veffq,
                                    const ImageMeta *images, const void *tables,
                                    void *proj_scratch, double *ab, int *status) {
  bool iso = true;
  for (int d = 0; d <= kStencilHalf; d++)
    iso = iso && p.cxf[d] == p.czf[d] && p.cyf[d] == p.czf[d];
  if (block <= 384)
    return iso ? launch_quad_mask<384, true>(mask, p, grid, block, smem, s, veffq, images, tables, proj_scratch, ab, status)
               : launch_quad_mask<384, false>(mask, p, grid, block, smem, s, veffq, images, tables, proj_scratch, ab, status);
  return iso ? launch_quad_mask<kQuadMaxThreads, true>(mask, p, grid, block, smem, s, veffq, images, tables, proj_scratch, ab, status)
             : launch_quad_mask<kQuadMaxThreads, false>(mask, p, grid, block, smem, s, veffq, images, tables, proj_scratch, ab, status);
}

}  // namespace sq

// lanczos_f32p.cu -- instantiations of the split-pass FP32 Lanczos kernel on CTA pairs
// (kLayoutQuad | kLayoutPair): one node per cluster of two CTAs, for cubes whose P and U do
// not fit one CTA's shared memory.
#include "lanczos_quad.cuh"

namespace sq {

namespace {
template <bool ISO>
cudaError_t launch_pair_mask(int mask, const LanczosParams &p, int grid, int block, size_t smem,
                             cudaStream_t s, const void *veffq, const ImageMeta *images,
                             const void *tables, void *proj_scratch, double *ab, int *status) {
  switch (mask) {
    case 3: return lq::launch_quad_pair_variant<3, ISO>(p, grid, block, smem, s, veffq, images, tables, proj_scratch, ab, status);
    case 5: return lq::launch_quad_pair_variant<5, ISO>(p, grid, block, smem, s, veffq, images, tables, proj_scratch, ab, status);
    case 6: return lq::launch_quad_pair_variant<6, ISO>(p, grid, block, smem, s, veffq, images, tables, proj_scratch, ab, status);
    case 7: return lq::launch_quad_pair_variant<7, ISO>(p, grid, block, smem, s, veffq, images, tables, proj_scratch, ab, status);
    default: return lq::launch_quad_pair_variant<15, ISO>(p, grid, block, smem, s, veffq, images, tables, proj_scratch, ab, status);
  }
}

template <bool ISO>
cudaError_t clusters_mask(int mask, int block, size_t smem, int *n) {
  switch (mask) {
    case 3: return lq::pair_max_clusters<3, ISO>(block, smem, n);
    case 5: return lq::pair_max_clusters<5, ISO>(block, smem, n);
    case 6: return lq::pair_max_clusters<6, ISO>(block, smem, n);
    case 7: return lq::pair_max_clusters<7, ISO>(block, smem, n);
    default: return lq::pair_max_clusters<15, ISO>(block, smem, n);
  }
}

bool isotropic(const LanczosParams &p) {
  bool iso = true;
  for (int d = 0; d <= kStencilHalf; d++)
    iso = iso && p.cxf[d] == p.czf[d] && p.cyf[d] == p.czf[d];
  return iso;
}
}  // namespace

cudaError_t launch_lanczos_f32_pair(int mask, const LanczosParams &p, int grid, int block,
                                    size_t smem, cudaStream_t s, const void *veffq,
                                    const ImageMeta *images, const void *tables,
                                    void *proj_scratch, double *ab, int *status) {
  return isotropic(p) ? launch_pair_mask<true>(mask, p, grid, block, smem, s, veffq, images, tables, proj_scratch, ab, status)
                      : launch_pair_mask<false>(mask, p, grid, block, smem, s, veffq, images, tables, proj_scratch, ab, status);
}

int lanczos_quad_pair_clusters(const LanczosParams &p, int block, size_t smem) {
  int n = 0;
  const int mask = kernel_mask(p.union_mask);
  const cudaError_t e = isotropic(p) ? clusters_mask<true>(mask, block, smem, &n)
                                     : clusters_mask<false>(mask, block, smem, &n);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  return n;
}

}  // namespace sq

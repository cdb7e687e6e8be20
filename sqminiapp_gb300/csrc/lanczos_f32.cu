// lanczos_f32.cu -- FP32-vector instantiations of the Lanczos kernel, y-gapped layout.
#include "lanczos_kernel.cuh"

namespace sq {

cudaError_t launch_lanczos_f32(int mask, bool faithful, bool u_smem, const LanczosParams &p,
                               int grid, int block, size_t smem, cudaStream_t s,
                               const void *veff_ext, const ImageMeta *images, const void *tables,
                               void *u_scratch, void *proj_scratch, double *ab, int *status) {
  constexpr int L = kLayoutYGap;
  if (faithful)
    return u_smem ? lk::launch_mask<float, true, true, L>(mask, p, grid, block, smem, s, veff_ext, images, tables, u_scratch, proj_scratch, ab, status)
                  : lk::launch_mask<float, true, false, L>(mask, p, grid, block, smem, s, veff_ext, images, tables, u_scratch, proj_scratch, ab, status);
  return u_smem ? lk::launch_mask<float, false, true, L>(mask, p, grid, block, smem, s, veff_ext, images, tables, u_scratch, proj_scratch, ab, status)
                : lk::launch_mask<float, false, false, L>(mask, p, grid, block, smem, s, veff_ext, images, tables, u_scratch, proj_scratch, ab, status);
}

}  // namespace sq

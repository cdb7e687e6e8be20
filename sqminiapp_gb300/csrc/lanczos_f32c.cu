// lanczos_f32c.cu -- FP32 instantiations with the compact projector list (corrected operator):
// every on-chip layout of the FP32 kernel, for cells whose full lists would not stay in L2.
#include "lanczos_kernel.cuh"

namespace sq {

cudaError_t launch_lanczos_f32_compact(int mask, bool u_smem, const LanczosParams &p, int grid,
                                       int block, size_t smem, cudaStream_t s,
                                       const void *veff_ext, const ImageMeta *images,
                                       const void *tables, void *u_scratch, void *proj_scratch,
                                       double *ab, int *status) {
  constexpr int C = kLayoutCompact;
  const int base = p.layout & ~C;
  if (base == (kLayoutYGap | kLayoutWide) && !u_smem)
    return lk::launch_mask<float, false, false, C | kLayoutYGap | kLayoutWide>(mask, p, grid, block, smem, s, veff_ext, images, tables, u_scratch, proj_scratch, ab, status);
  if (base == kLayoutYGap)
    return u_smem ? lk::launch_mask<float, false, true, C | kLayoutYGap>(mask, p, grid, block, smem, s, veff_ext, images, tables, u_scratch, proj_scratch, ab, status)
                  : lk::launch_mask<float, false, false, C | kLayoutYGap>(mask, p, grid, block, smem, s, veff_ext, images, tables, u_scratch, proj_scratch, ab, status);
  if (base == 0 && u_smem)
    return lk::launch_mask<float, false, true, C>(mask, p, grid, block, smem, s, veff_ext, images, tables, u_scratch, proj_scratch, ab, status);
  return cudaErrorInvalidValue;
}

}  // namespace sq

// lanczos_f32w.cu -- FP32 instantiations for cubes wider than 32 points in x (U in global
// scratch: such a cube's padded P alone takes most of the 227 KB of shared memory).
#include "lanczos_kernel.cuh"

namespace sq {

cudaError_t launch_lanczos_f32_wide(int mask, bool faithful, const LanczosParams &p, int grid,
                                    int block, size_t smem, cudaStream_t s, const void *veff_ext,
                                    const ImageMeta *images, const void *tables, void *u_scratch,
                                    void *proj_scratch, double *ab, int *status) {
  if (faithful)
    return lk::launch_mask<float, true, false, kLayoutYGap | kLayoutWide>(mask, p, grid, block, smem, s, veff_ext, images, tables, u_scratch, proj_scratch, ab, status);
  return lk::launch_mask<float, false, false, kLayoutYGap | kLayoutWide>(mask, p, grid, block, smem, s, veff_ext, images, tables, u_scratch, proj_scratch, ab, status);
}

}  // namespace sq

// lanczos_f64.cu -- FP64-vector instantiations of the Lanczos kernel (U in global scratch).
#include "lanczos_kernel.cuh"

namespace sq {

cudaError_t launch_lanczos_f64_xclamp(int mask, bool faithful, const LanczosParams &p, int grid,
                                      int block, size_t smem, cudaStream_t s,
                                      const void *veff_ext, const ImageMeta *images,
                                      const void *tables, void *u_scratch, void *proj_scratch,
                                      double *ab, int *status);

cudaError_t launch_lanczos_f64(int mask, bool faithful, const LanczosParams &p, int grid,
                               int block, size_t smem, cudaStream_t s, const void *veff_ext,
                               const ImageMeta *images, const void *tables, void *u_scratch,
                               void *proj_scratch, double *ab, int *status) {
  if (p.layout & kLayoutXClamp)  // rows without zero columns (cubes of 29^3 and up)
    return launch_lanczos_f64_xclamp(mask, faithful, p, grid, block, smem, s, veff_ext, images,
                                     tables, u_scratch, proj_scratch, ab, status);
  if (faithful)
    return lk::launch_mask<double, true, false, 0>(mask, p, grid, block, smem, s, veff_ext, images, tables, u_scratch, proj_scratch, ab, status);
  return lk::launch_mask<double, false, false, 0>(mask, p, grid, block, smem, s, veff_ext, images, tables, u_scratch, proj_scratch, ab, status);
}

}  // namespace sq

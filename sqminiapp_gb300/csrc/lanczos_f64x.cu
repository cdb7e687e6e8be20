// lanczos_f64x.cu -- FP64 instantiations for cubes whose x-padded rows do not fit in shared
// memory: rows of exactly nx points, x-neighbours bounds-checked.
#include "lanczos_kernel.cuh"

namespace sq {

cudaError_t launch_lanczos_f64_xclamp(int mask, bool faithful, const LanczosParams &p, int grid,
                                      int block, size_t smem, cudaStream_t s,
                                      const void *veff_ext, const ImageMeta *images,
                                      const void *tables, void *u_scratch, void *proj_scratch,
                                      double *ab, int *status) {
  if (faithful)
    return lk::launch_mask<double, true, false, kLayoutXClamp>(mask, p, grid, block, smem, s, veff_ext, images, tables, u_scratch, proj_scratch, ab, status);
  return lk::launch_mask<double, false, false, kLayoutXClamp>(mask, p, grid, block, smem, s, veff_ext, images, tables, u_scratch, proj_scratch, ab, status);
}

}  // namespace sq

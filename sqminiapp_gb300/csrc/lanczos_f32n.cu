// lanczos_f32n.cu -- FP32 instantiations without the zero rows between z-planes (y-neighbours
// bounds-checked), for cubes whose P and U fit in shared memory together only that way
// (29^3: 121 KB + 101 KB).
#include "lanczos_kernel.cuh"

namespace sq {

cudaError_t launch_lanczos_f32_nogap(int mask, bool faithful, const LanczosParams &p, int grid,
                                     int block, size_t smem, cudaStream_t s,
                                     const void *veff_ext, const ImageMeta *images,
                                     const void *tables, void *u_scratch, void *proj_scratch,
                                     double *ab, int *status) {
  if (faithful)
    return lk::launch_mask<float, true, true, 0>(mask, p, grid, block, smem, s, veff_ext, images, tables, u_scratch, proj_scratch, ab, status);
  return lk::launch_mask<float, false, true, 0>(mask, p, grid, block, smem, s, veff_ext, images, tables, u_scratch, proj_scratch, ab, status);
}

}  // namespace sq

// lanczos.cu -- host dispatch of the batched Lanczos kernel and the Veff padding kernel.
#include <cuda_runtime.h>

#include <algorithm>

#include "lanczos_kernel.cuh"
#include "sq_internal.hpp"
#include "sq_kernels.hpp"

namespace sq {

namespace {

template <typename T>
__global__ void veff_extend_kernel(const double *__restrict__ veff, double vconst,
                                   T *__restrict__ ext, int Nx, int Ny, int Nz, int nhx, int nhy,
                                   int nhz, int EX, int EY, int EZ) {
  const long long total = (long long)EX * EY * EZ;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int ex = (int)(e % EX), ey = (int)((e / EX) % EY), ez = (int)(e / ((long long)EX * EY));
    const int gx = ((ex - nhx) % Nx + Nx) % Nx;
    const int gy = ((ey - nhy) % Ny + Ny) % Ny;
    const int gz = ((ez - nhz) % Nz + Nz) % Nz;
    ext[e] = T(veff ? veff[((long long)gz * Ny + gy) * Nx + gx] : vconst);
  }
}

// Quad-aligned copies of cdiag + Veff for the split-pass kernel: copy c holds extended x index
// ex at row position ex + c, so a node at grid x = I reads its cube row from copy (4 - I%4)%4
// at a 16-byte boundary; positions outside [c, c + EX) hold 0.
__global__ void veff_quad_kernel(const double *__restrict__ veff, double vconst, double cdiag,
                                 float *__restrict__ out, int Nx, int Ny, int Nz, int nhx, int nhy,
                                 int nhz, int EX, int EY, int EZ, int row) {
  const long long per_copy = (long long)row * EY * EZ;
  const long long total = 4 * per_copy;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(e / per_copy);
    const long long r = e - c * per_copy;
    const int pos = (int)(r % row);
    const long long rr = r / row;
    const int ey = (int)(rr % EY), ez = (int)(rr / EY);
    const int ex = pos - c;
    float v = 0.f;
    if (ex >= 0 && ex < EX) {
      const int gx = ((ex - nhx) % Nx + Nx) % Nx;
      const int gy = ((ey - nhy) % Ny + Ny) % Ny;
      const int gz = ((ez - nhz) % Nz + Nz) % Nz;
      v = float(cdiag + (veff ? veff[((long long)gz * Ny + gy) * Nx + gx] : vconst));
    }
    out[e] = v;
  }
}

}  // namespace

int kernel_mask(int union_mask) {
  return (union_mask == 3 || union_mask == 5 || union_mask == 6 || union_mask == 7) ? union_mask : 15;
}

size_t proj_record_bytes(int elem_size, bool faithful, int union_mask, bool compact) {
  if (compact) {  // lk::ChanRec: channel values in one 8-byte word or whole 16-byte vectors
    int nch = 0;
    for (int l = 0; l < 4; l++)
      if (kernel_mask(union_mask) & (1 << l)) nch++;
    const size_t vb = (size_t)nch * elem_size;
    return (vb <= 8 ? 8 : 16 * ((vb + 15) / 16)) + sizeof(unsigned);
  }
  const int n = faithful ? 2 : mask_nlm(kernel_mask(union_mask));
  const int per_vec = 16 / elem_size;
  return (size_t)16 * ((n + per_vec - 1) / per_vec) + sizeof(unsigned);
}

int mask_nlm(int mask) {
  int n = 0;
  for (int l = 0; l < 4; l++)
    if (mask & (1 << l)) n += 2 * l + 1;
  return n;
}

size_t lanczos_smem_bytes(const LanczosParams &p, int elem_size, bool u_smem, bool faithful) {
  const bool ypad = (p.layout & kLayoutYGap) != 0;
  const size_t ps = (size_t)(ypad ? p.ny + lk::O : p.ny) * p.pitch;
  const size_t off = ypad ? (size_t)lk::O * p.pitch : lk::O;
  const size_t psize = (off + p.nz * ps + 3) & ~size_t(3);
  const size_t nc = (size_t)p.upitch * p.ny * p.nz;
  const int nlm = mask_nlm(kernel_mask(p.union_mask));
  const size_t cstride = faithful ? 2 : nlm, astride = faithful ? 1 : nlm;
  size_t b = elem_size * psize;
  if (u_smem) b += elem_size * ((nc + 3) & ~size_t(3));
  b += sizeof(double) * 2 * (lk::kMaxWarps + 1) + sizeof(double) * 128;
  b += (size_t)elem_size * p.max_img * (cstride + astride);
  b += sizeof(int) * (8 * (size_t)p.max_img + 2) + sizeof(int) * 4;
  if (p.layout & kLayoutCompact) b += (2 * sizeof(int) + 3 * (size_t)elem_size) * p.max_img;
  return b;
}

cudaError_t launch_lanczos_f32(int mask, bool faithful, bool u_smem, const LanczosParams &p,
                               int grid, int block, size_t smem, cudaStream_t s,
                               const void *veff_ext, const ImageMeta *images, const void *tables,
                               void *u_scratch, void *proj_scratch, double *ab, int *status);
cudaError_t launch_lanczos_f64(int mask, bool faithful, const LanczosParams &p, int grid,
                               int block, size_t smem, cudaStream_t s, const void *veff_ext,
                               const ImageMeta *images, const void *tables, void *u_scratch,
                               void *proj_scratch, double *ab, int *status);
cudaError_t launch_lanczos_f32_nogap(int mask, bool faithful, const LanczosParams &p, int grid,
                                     int block, size_t smem, cudaStream_t s,
                                     const void *veff_ext, const ImageMeta *images,
                                     const void *tables, void *u_scratch, void *proj_scratch,
                                     double *ab, int *status);
cudaError_t launch_lanczos_f32_compact(int mask, bool u_smem, const LanczosParams &p, int grid,
                                       int block, size_t smem, cudaStream_t s,
                                       const void *veff_ext, const ImageMeta *images,
                                       const void *tables, void *u_scratch, void *proj_scratch,
                                       double *ab, int *status);
cudaError_t launch_lanczos_f32_wide(int mask, bool faithful, const LanczosParams &p, int grid,
                                    int block, size_t smem, cudaStream_t s, const void *veff_ext,
                                    const ImageMeta *images, const void *tables, void *u_scratch,
                                    void *proj_scratch, double *ab, int *status);

cudaError_t launch_lanczos_f32_quad(int mask, const LanczosParams &p, int grid, int block,
                                    size_t smem, cudaStream_t s, const void *veffq,
                                    const ImageMeta *images, const void *tables,
                                    void *proj_scratch, double *ab, int *status);
cudaError_t launch_lanczos_f32_pair(int mask, const LanczosParams &p, int grid, int block,
                                    size_t smem, cudaStream_t s, const void *veffq,
                                    const ImageMeta *images, const void *tables,
                                    void *proj_scratch, double *ab, int *status);

cudaError_t launch_lanczos(const LanczosParams &p, int precision, bool faithful, bool u_smem,
                           int grid, int block, size_t smem, cudaStream_t s, const void *veff_ext,
                           const ImageMeta *images, const void *tables, void *u_scratch,
                           void *proj_scratch, double *ab, int *status) {
  const int mask = kernel_mask(p.union_mask);
  const bool gap = (p.layout & kLayoutYGap) != 0;
  if (precision == 32) {
    if (p.layout & kLayoutQuad) {  // corrected operator, full records, P and U on chip
      if (faithful || !u_smem || (p.layout & ~(kLayoutQuad | kLayoutPair)))
        return cudaErrorInvalidValue;
      if (p.layout & kLayoutPair)
        return launch_lanczos_f32_pair(mask, p, grid, block, smem, s, veff_ext, images, tables,
                                       proj_scratch, ab, status);
      // status[1]: the kernel's node queue (nodes past the first round go to whichever CTA
      // finishes first)
      const cudaError_t e = cudaMemsetAsync(status + 1, 0, sizeof(int), s);
      if (e != cudaSuccess) return e;
      return launch_lanczos_f32_quad(mask, p, grid, block, smem, s, veff_ext, images, tables,
                                     proj_scratch, ab, status);
    }
    if (p.layout & kLayoutCompact) {  // corrected operator only
      if (faithful) return cudaErrorInvalidValue;
      return launch_lanczos_f32_compact(mask, u_smem, p, grid, block, smem, s, veff_ext, images,
                                        tables, u_scratch, proj_scratch, ab, status);
    }
    if (p.layout & kLayoutWide) {  // U in global scratch
      if (!gap || u_smem) return cudaErrorInvalidValue;
      return launch_lanczos_f32_wide(mask, faithful, p, grid, block, smem, s, veff_ext, images,
                                     tables, u_scratch, proj_scratch, ab, status);
    }
    if (!gap) {  // U in shared memory
      if (!u_smem) return cudaErrorInvalidValue;
      return launch_lanczos_f32_nogap(mask, faithful, p, grid, block, smem, s, veff_ext, images,
                                      tables, u_scratch, proj_scratch, ab, status);
    }
    return launch_lanczos_f32(mask, faithful, u_smem, p, grid, block, smem, s, veff_ext, images,
                              tables, u_scratch, proj_scratch, ab, status);
  }
  if (gap || (p.layout & (kLayoutWide | kLayoutCompact)) || u_smem) return cudaErrorInvalidValue;
  return launch_lanczos_f64(mask, faithful, p, grid, block, smem, s, veff_ext, images, tables,
                            u_scratch, proj_scratch, ab, status);
}

cudaError_t launch_veff_extend(const double *veff, double vconst, void *ext, int precision,
                               const LanczosParams &p, cudaStream_t s) {
  if (p.layout & kLayoutQuad) {
    const long long total = (long long)veff_quad_floats(p);
    const int block = 256;
    const int grid = (int)std::min<long long>((total + block - 1) / block, 152LL * 16);
    veff_quad_kernel<<<grid, block, 0, s>>>(veff, vconst, p.cdiag, (float *)ext, p.Nx, p.Ny, p.Nz,
                                            p.nhx, p.nhy, p.nhz, p.EX, p.EY, p.EZ, p.vq_row);
    return cudaGetLastError();
  }
  const long long total = (long long)p.EX * p.EY * p.EZ;
  const int block = 256;
  const int grid = (int)std::min<long long>((total + block - 1) / block, 152LL * 16);
  if (precision == 32)
    veff_extend_kernel<float><<<grid, block, 0, s>>>(veff, vconst, (float *)ext, p.Nx, p.Ny, p.Nz,
                                                     p.nhx, p.nhy, p.nhz, p.EX, p.EY, p.EZ);
  else
    veff_extend_kernel<double><<<grid, block, 0, s>>>(veff, vconst, (double *)ext, p.Nx, p.Ny,
                                                      p.Nz, p.nhx, p.nhy, p.nhz, p.EX, p.EY, p.EZ);
  return cudaGetLastError();
}

}  // namespace sq

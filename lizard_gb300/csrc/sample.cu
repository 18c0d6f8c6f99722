// Row (a) of the hot path on sm_103a: the picture sampler, when the grid itself is asked for (the transform's column
// pass otherwise samples as it loads). Every sample of the n x n picture grid is read from the captured luma frame
// through the registration: the homography H (module -> image) plus the bilinear blend of the node mesh's
// displacements, then a bilinear luma read at gamma 1. By the receiver's read: the reference decoder's integer read
// (ob_sample_grid_pic's x86-64 form, liblizard/src/acquire.c:5302-5440, in strips of 64 columns as
// liblizard/src/lizard_phy.c:1634 calls it) or the exact walk (ob_sample_grid, acquire.c:5121-5196 with
// internal.h:11-23 sample()), each restated operation for operation (sample_dev.cuh), so either gives the reference's
// values bit for bit.
//
// One thread a sample, a 32 x 8 tile of samples a CTA: a warp reads a row run of 32 samples, whose luma reads are
// neighbouring pixels of one or two image rows.
#include <cuda_runtime.h>
#include <stdint.h>
#include "lizg_internal.h"
#include "sample_dev.cuh"

namespace lizg {

__global__ void __launch_bounds__(256) sample_kernel(SampleDev sd, const uint8_t *luma, int w, int h, int pitch, int64_t fstride,
                                                     const float *reg, int regstride, float *grid) {
  const int f = blockIdx.z, x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  const int n = sd.n;
  if (x >= n || y >= n) return;
  const float *H = reg + (int64_t)f * regstride;
  grid[(int64_t)f * n * n + (int64_t)y * n + x] = sample_xy(sd, luma + f * fstride, w, h, pitch, H, H + 9, x, sd.colt[x], sd.rowt[y]);
}

__global__ void sample_tables_kernel(SampleDev sd, float4 *colt, float4 *rowt) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < sd.n) { colt[t] = sample_col(sd, t); rowt[t] = sample_row(sd, t); }
}

cudaError_t sample_tables_launch(SampleDev sd, float4 *colt, float4 *rowt, cudaStream_t st) {
  sample_tables_kernel<<<(sd.n + 255) / 256, 256, 0, st>>>(sd, colt, rowt);
  return cudaGetLastError();
}

cudaError_t sample_launch(const SampleDev &sd, int frames, const uint8_t *luma, int w, int h, int pitch, int64_t fstride,
                          const float *reg, int regstride, float *grid, cudaStream_t st) {
  const dim3 g((sd.n + 31) / 32, (sd.n + 7) / 8, frames);
  sample_kernel<<<g, 256, 0, st>>>(sd, luma, w, h, pitch, fstride, reg, regstride, grid);
  return cudaGetLastError();
}

}  // namespace lizg

// Row (a) of the hot path on sm_103a: the picture sampler. Every sample of the n x n picture grid is read from the
// captured luma frame through the registration: the homography H (module -> image) plus the bilinear blend of the
// node mesh's displacements, then a bilinear luma read at gamma 1 (grey / 255), the frame edge clamped. This is the
// reference's exact walk, liblizard/src/acquire.c:5121-5196 ob_sample_grid with internal.h:11-23 sample(), restated
// operation for operation in float and compiled with -fmad=false, so it gives that walk's values bit for bit. (The
// reference's decoder runs a faster integer read of the same map, ob_sample_grid_pic, which its own test holds
// within 1/200 of grey of this walk: liblizard/test/sample_grid.c.)
//
// One thread a sample, a 32 x 8 tile of samples a CTA: a warp reads a row run of 32 samples, whose luma reads are
// neighbouring pixels of one or two image rows.
#include <cuda_runtime.h>
#include <stdint.h>
#include "lizg_internal.h"

namespace lizg {

// The mesh cell along one axis: the last k in [0, nn - 2] with m >= node[k], else 0 (liblizard/src/acquire.c:5089-5094).
__device__ __forceinline__ int node_cell(const float *node, int nn, float m) {
  int k = 0;
  for (int q = 1; q <= nn - 2; q++) if (m >= node[q]) k = q;
  return k;
}

__global__ void __launch_bounds__(256) sample_kernel(SampleDev sd, const uint8_t *luma, int w, int h, int pitch, int64_t fstride,
                                                     const float *reg, int regstride, float *grid) {
  const int f = blockIdx.z, x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  const int n = sd.n;
  if (x >= n || y >= n) return;
  const uint8_t *px = luma + f * fstride;
  const float *H = reg + (int64_t)f * regstride, *nodes = H + 9;
  const float mx = sd.g0 + (float)x * sd.step, my = sd.g0 + (float)y * sd.step;
  const int j = node_cell(sd.node_y, sd.ny, my), i = node_cell(sd.node_x, sd.nx, mx);
  const float v = (my - sd.node_y[j]) / (sd.node_y[j + 1] - sd.node_y[j]);
  const float *n00 = nodes + 2 * (j * sd.nx + i), *n10 = n00 + 2, *n01 = n00 + 2 * sd.nx, *n11 = n01 + 2;
  const float inv = 1.0f / (sd.node_x[i + 1] - sd.node_x[i]);
  const float ex = ((n10[0] - n00[0]) * (1 - v) + (n11[0] - n01[0]) * v) * inv, cx = n00[0] * (1 - v) + n01[0] * v - ex * sd.node_x[i];
  const float ey = ((n10[1] - n00[1]) * (1 - v) + (n11[1] - n01[1]) * v) * inv, cy = n00[1] * (1 - v) + n01[1] * v - ey * sd.node_x[i];
  const float kw = H[7] * my + 1, ku = H[1] * my + H[2], kv = H[4] * my + H[5];
  const float rw = 1 / (H[6] * mx + kw);
  const float pu = (H[0] * mx + ku) * rw, pv = (H[3] * mx + kv) * rw;
  const float dx = cx + ex * mx, dy = cy + ey * mx;
  // sample(): the pixel centres at half-integers, clamped to the frame; a NaN coordinate reads pixel 0
  float sx = pu + dx - 0.5f, sy = pv + dy - 0.5f;
  if (sx < 0) sx = 0; else if (sx > w - 1.001f) sx = w - 1.001f;
  if (sy < 0) sy = 0; else if (sy > h - 1.001f) sy = h - 1.001f;
  const int xi = sx >= 0 ? (int)sx : 0, yi = sy >= 0 ? (int)sy : 0;
  const float fx = sx - xi, fy = sy - yi;
  const uint8_t *p = px + (int64_t)yi * pitch + xi;
  const float a = p[0] / 255.0f, b = p[1] / 255.0f, c = p[pitch] / 255.0f, d = p[pitch + 1] / 255.0f;
  grid[(int64_t)f * n * n + (int64_t)y * n + x] = (a + (b - a) * fx) * (1 - fy) + (c + (d - c) * fx) * fy;
}

cudaError_t sample_launch(const SampleDev &sd, int frames, const uint8_t *luma, int w, int h, int pitch, int64_t fstride,
                          const float *reg, int regstride, float *grid, cudaStream_t st) {
  const dim3 g((sd.n + 31) / 32, (sd.n + 7) / 8, frames);
  sample_kernel<<<g, 256, 0, st>>>(sd, luma, w, h, pitch, fstride, reg, regstride, grid);
  return cudaGetLastError();
}

}  // namespace lizg

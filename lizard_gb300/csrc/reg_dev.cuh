// The registration's device arithmetic shared by the anchor search and the border nodes, each in the reference's
// float and double order (translation units that include it are compiled with -fmad=false): the homography, the lens
// model's displacement, the bilinear grey read.
#ifndef LIZG_REG_DEV_CUH
#define LIZG_REG_DEV_CUH
#include <stdint.h>
#include "sample_dev.cuh"

namespace lizg {

constexpr int kLensP = 11, kLensStride = 4 + kLensP;   // a lens model: K, ax, ay, R, then kLensP coefficients

__device__ __forceinline__ void project(const float *h, float x, float y, float *u, float *v) {
  const float w = h[6] * x + h[7] * y + 1;
  *u = (h[0] * x + h[1] * y + h[2]) / w;
  *v = (h[3] * x + h[4] * y + h[5]) / w;
}

// The lens model's displacement at (u, v) (liblizard/src/acquire.c:1506-1512, 1615-1620): lens = K, ax, ay, R, t[11].
__device__ __forceinline__ void lens_at(const double *lens, double u, double v, float *dx, float *dy) {
  const int K = (int)lens[0];
  const double x = (u - lens[1]) / lens[3], y = (v - lens[2]) / lens[3];
  double fx = 0, fy = 0;
  fx += lens[4] * x; fy += lens[4] * 0.0;
  fx += lens[5] * y; fy += lens[5] * 0.0;
  fx += lens[6] * 0.0; fy += lens[6] * x;
  fx += lens[7] * 0.0; fy += lens[7] * y;
  fx += lens[8] * 1.0; fy += lens[8] * 0.0;
  fx += lens[9] * 0.0; fy += lens[9] * 1.0;
  fx += lens[10] * (-x * x); fy += lens[10] * (-x * y);
  fx += lens[11] * (-x * y); fy += lens[11] * (-y * y);
  const double s = x * x + y * y;
  double sk = s;
  for (int k = 0; k < K; k++, sk *= s) { fx += lens[12 + k] * (sk * x); fy += lens[12 + k] * (sk * y); }
  *dx = (float)fx; *dy = (float)fy;
}

// The bilinear grey read at gamma 1 (liblizard/src/internal.h:11-23), rows w apart; a grey level k reads k / 255.
__device__ __forceinline__ float sample(const uint8_t *px, int w, int h, float x, float y) {
  x -= 0.5f; y -= 0.5f;
  const float xm = (float)w - 1.001f, ym = (float)h - 1.001f;
  if (x < 0) x = 0; else if (x > xm) x = xm;
  if (y < 0) y = 0; else if (y > ym) y = ym;
  const int xi = x >= 0 ? (int)x : 0, yi = y >= 0 ? (int)y : 0;
  const float fx = x - (float)xi, fy = y - (float)yi;
  const uint8_t *p = px + (int64_t)yi * w + xi;
  const float a = grey_of(p[0]), b = grey_of(p[1]), c = grey_of(p[w]), d = grey_of(p[w + 1]);
  return (a + (b - a) * fx) * (1 - fy) + (c + (d - c) * fx) * fy;
}

}  // namespace lizg
#endif

// The anchor search on sm_103a: the registration's 7 x 7 anchors found in a batch of captured frames, the step of the
// reference's front half that the refinement of the registration starts from (liblizard/src/acquire.c:1876-2036
// anchor_find, restated from its portable build, the scalar twin of its SIMD paths). Compiled with -fmad=false: every
// float and double operation rounds once, in the reference's order, so the results are that build's bit for bit.
//
// One CTA an anchor of a frame: the window of W x W samples a template step (a / 16 modules) apart about the anchor's
// place, read through H and the lens model; its integral images of the greys and of their squares in double (each
// row's running sums by one thread a row, then each column accumulated down by one thread a column, the additions
// the reference makes); the normalised correlation with the anchor's pattern (two concentric squares) at every
// offset within three modules, from four box sums an offset; the first largest in scan order; a parabola each way.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string>
#include "lizard_gb300.h"
#include "lizg_internal.h"
#include "reg_dev.cuh"

namespace lizg {

constexpr int kAnchK = 7, kAnchTs = 16, kAnchReach = 3, kMarginM = 15;
constexpr float kAnchPeak = 0.6f;

// The window's geometry for a ring span (a = span / 64 modules a side, r steps of reach, W samples across, O offsets).
struct AnchGeom {
  int a, r, W, O;
  float hs;
};
static AnchGeom anch_geom(int span) {
  AnchGeom g;
  g.a = span / 64;
  g.hs = (float)g.a / kAnchTs;
  g.r = (int)ceilf((float)kAnchReach / g.hs);
  g.W = kAnchTs + 2 * g.r;
  g.O = 2 * g.r + 1;
  return g;
}

__device__ __forceinline__ void anchor_map(const float *h, const double *lens, float X, float Y, float *u, float *v) {
  project(h, X, Y, u, v);
  if (lens) { float dx, dy; lens_at(lens, *u, *v, &dx, &dy); *u += dx; *v += dy; }
}

struct AnchArgs {
  int span, w, h, frames, hstride;
  int64_t fstride;
  AnchGeom g;
  int m0[kAnchK];
  const uint8_t *luma, *skip;
  const float *H;
  const double *lens;
  const int *lens_on;       // frames: 0 where frame f searches through H alone (NULL: every frame through lens)
  const uint8_t *active;    // frames: 0 where frame f is not searched at all (NULL: every frame)
  lizg_anchor_out out;
};

__device__ __forceinline__ double abox(const double *I, int W1, int x, int y, int s) {
  return I[(y + s) * W1 + x + s] - I[y * W1 + x + s] - I[(y + s) * W1 + x] + I[y * W1 + x];
}

__global__ void __launch_bounds__(256) anchor_find_kernel(AnchArgs a) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int f = blockIdx.x / (kAnchK * kAnchK), k = blockIdx.x % (kAnchK * kAnchK), i = k % kAnchK, j = k / kAnchK;
  const int64_t o = (int64_t)f * kAnchK * kAnchK + k;
  if (a.skip && a.skip[o]) return;   // found before: left as it is
  if (a.active && !a.active[f]) return;
  const AnchGeom g = a.g;
  const int r = g.r, W = g.W, O = g.O, W1 = W + 1, tid = threadIdx.x;
  const float hs = g.hs, ah = (float)g.a * 0.5f;
  double *I1 = reinterpret_cast<double *>(sm), *I2 = I1 + W1 * W1;
  float *win = reinterpret_cast<float *>(I2 + W1 * W1), *C = win + W * W;
  __shared__ float s_h[9], s_tm, s_tn, s_bv[256];
  __shared__ double s_lens[kLensStride];
  __shared__ int s_r25[2], s_r6[2], s_bi[256];
  if (tid < 9) s_h[tid] = a.H[(int64_t)f * a.hstride + tid];
  const bool use_lens = a.lens && (!a.lens_on || a.lens_on[f]);
  if (use_lens && tid < kLensStride) s_lens[tid] = a.lens[(int64_t)f * kLensStride + tid];
  if (tid == 0) {
    // the pattern's mean and norm in the reference's order, and its squares' ranges along an axis
    float tm = 0, tn = 0;
    for (int y = 0; y < kAnchTs; y++)
      for (int x = 0; x < kAnchTs; x++) {
        const float u = ((float)x + 0.5f) * hs - ah, v = ((float)y + 0.5f) * hs - ah, dc = fmaxf(fabsf(u), fabsf(v)) / ah;
        tm += dc < 0.25f || dc >= 0.6f ? 1.0f : -1.0f;
      }
    tm /= (float)(kAnchTs * kAnchTs);
    for (int y = 0; y < kAnchTs; y++)
      for (int x = 0; x < kAnchTs; x++) {
        const float u = ((float)x + 0.5f) * hs - ah, v = ((float)y + 0.5f) * hs - ah, dc = fmaxf(fabsf(u), fabsf(v)) / ah;
        const float t = (dc < 0.25f || dc >= 0.6f ? 1.0f : -1.0f) - tm;
        tn += t * t;
      }
    s_tm = tm;
    s_tn = sqrtf(tn);
    int i25 = kAnchTs, j25 = -1, i6 = kAnchTs, j6 = -1;
    for (int x = 0; x < kAnchTs; x++) {
      const float d = fabsf(((float)x + 0.5f) * hs - ah) / ah;
      if (d < 0.25f) { if (x < i25) i25 = x; j25 = x; }
      if (d < 0.6f) { if (x < i6) i6 = x; j6 = x; }
    }
    s_r25[0] = i25; s_r25[1] = j25; s_r6[0] = i6; s_r6[1] = j6;
  }
  __syncthreads();
  const double *lens = use_lens ? s_lens : nullptr;
  const float x0 = (float)a.m0[i], y0 = (float)a.m0[j], X = x0 + ah, Y = y0 + ah;
  const uint8_t *px = a.luma + (int64_t)f * a.fstride;
  // the window
  for (int t = tid; t < W * W; t += blockDim.x) {
    const int wx = t % W, wy = t / W;
    float u, v;
    anchor_map(s_h, lens, x0 + ((float)(wx - r) + 0.5f) * hs, y0 + ((float)(wy - r) + 0.5f) * hs, &u, &v);
    win[t] = sample(px, a.w, a.h, u, v);
  }
  for (int t = tid; t < W1; t += blockDim.x) { I1[t] = 0; I2[t] = 0; I1[t * W1] = 0; I2[t * W1] = 0; }
  __syncthreads();
  // each row's running sums (left to right), then each column accumulated down the rows
  if (tid < W) {
    double s = 0, q = 0;
    for (int wx = 0; wx < W; wx++) {
      const double vv = win[tid * W + wx];
      s += vv; q += vv * vv;
      I1[(tid + 1) * W1 + wx + 1] = s; I2[(tid + 1) * W1 + wx + 1] = q;
    }
  }
  __syncthreads();
  if (tid < W) {
    for (int wy = 0; wy < W; wy++) {
      I1[(wy + 1) * W1 + tid + 1] = I1[wy * W1 + tid + 1] + I1[(wy + 1) * W1 + tid + 1];
      I2[(wy + 1) * W1 + tid + 1] = I2[wy * W1 + tid + 1] + I2[(wy + 1) * W1 + tid + 1];
    }
  }
  __syncthreads();
  // the correlation at every offset; each thread keeps its first largest in scan order
  const int i25 = s_r25[0], j25 = s_r25[1], i6 = s_r6[0], j6 = s_r6[1];
  const double tmd = (double)s_tm, tnd = (double)s_tn;
  float bv = -2;
  int bi = O * O;
  for (int t = tid; t < O * O; t += blockDim.x) {
    const int qx = t % O, qy = t / O;
    const double s1 = abox(I1, W1, qx, qy, kAnchTs), s2 = abox(I2, W1, qx, qy, kAnchTs), var = s2 - s1 * s1 / (double)(kAnchTs * kAnchTs);
    const double s25 = j25 >= i25 ? abox(I1, W1, qx + i25, qy + i25, j25 - i25 + 1) : 0;
    const double s6 = j6 >= i6 ? abox(I1, W1, qx + i6, qy + i6, j6 - i6 + 1) : 0;
    const double st = 2 * (s25 - s6) + s1 * (1 - tmd);
    const float c = var > 1e-12 ? (float)(st / (sqrt(var) * tnd)) : 0.0f;
    C[t] = c;
    if (c > bv) { bv = c; bi = t; }
  }
  s_bv[tid] = bv; s_bi[tid] = bi;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (tid < s) {
      const float ov = s_bv[tid + s];
      const int oi = s_bi[tid + s];
      if (ov > s_bv[tid] || (ov == s_bv[tid] && oi < s_bi[tid])) { s_bv[tid] = ov; s_bi[tid] = oi; }
    }
    __syncthreads();
  }
  if (tid != 0) return;
  const float best = s_bv[0];
  const int bx = s_bi[0] % O - r, by = s_bi[0] / O - r;
  float sx = 0, sy = 0;
  if (bx > -r && bx < r) {
    const float l = C[(by + r) * O + bx + r - 1], c = best, rr = C[(by + r) * O + bx + r + 1], d = l - 2 * c + rr;
    if (d < 0) sx = 0.5f * (l - rr) / d;
  }
  if (by > -r && by < r) {
    const float l = C[(by + r - 1) * O + bx + r], c = best, rr = C[(by + r + 1) * O + bx + r], d = l - 2 * c + rr;
    if (d < 0) sy = 0.5f * (l - rr) / d;
  }
  float u, v, hu, hv;
  anchor_map(s_h, lens, X + ((float)bx + sx) * hs, Y + ((float)by + sy) * hs, &u, &v);
  project(s_h, X, Y, &hu, &hv);
  a.out.peak[o] = best; a.out.dx[o] = u - hu; a.out.dy[o] = v - hv; a.out.u[o] = u; a.out.v[o] = v;
  a.out.ok[o] = best >= kAnchPeak && bx > -r && bx < r && by > -r && by < r;
}

// Queues the search for a batch of frames (arguments as lizg_anchor_find_dev's, already checked).
cudaError_t anchor_find_launch(int span, const uint8_t *d_luma, int w, int h, int64_t frame_stride, const float *d_H, int h_stride,
                               const double *d_lens, const uint8_t *d_skip, int frames, const lizg_anchor_out &out, cudaStream_t st,
                               const int *d_lens_on, const uint8_t *d_active) {
  AnchArgs a{};
  a.lens_on = d_lens_on; a.active = d_active;
  a.span = span; a.w = w; a.h = h; a.frames = frames; a.hstride = h_stride; a.fstride = frame_stride;
  a.g = anch_geom(span);
  for (int i = 0; i < kAnchK; i++) a.m0[i] = (int)floor(kMarginM + (double)span * (i + 0.5) / kAnchK - a.g.a / 2.0 + 0.5);
  a.luma = d_luma; a.skip = d_skip; a.H = d_H; a.lens = d_lens; a.out = out;
  const int W1 = a.g.W + 1;
  const size_t smem = 2 * sizeof(double) * W1 * W1 + sizeof(float) * ((size_t)a.g.W * a.g.W + (size_t)a.g.O * a.g.O);
  static SmemOptIn opt;
  cudaError_t e;
  if ((e = opt.set(reinterpret_cast<const void *>(anchor_find_kernel), 120 * 1024)) != cudaSuccess) return e;
  anchor_find_kernel<<<frames * kAnchK * kAnchK, 256, smem, st>>>(a);
  return cudaGetLastError();
}

}  // namespace lizg

extern "C" int lizg_anchor_find_dev(int span, const uint8_t *d_luma, int w, int h, int64_t frame_stride, const float *d_H, int h_stride,
                                    const double *d_lens, const uint8_t *d_skip, int frames, const lizg_anchor_out *out, void *stream) {
  using namespace lizg;
  if (span != 128 && span != 256 && span != 512) return record_error(LIZG_E_ARG, "lizg_anchor_find_dev: span must be 128, 256 or 512");
  if (!d_luma || !d_H || !out || !out->ok || !out->peak || !out->dx || !out->dy || !out->u || !out->v)
    return record_error(LIZG_E_ARG, "lizg_anchor_find_dev: NULL argument");
  if (w < 2 || h < 2 || frames < 1 || frame_stride < (int64_t)w * h || h_stride < 9)
    return record_error(LIZG_E_ARG, "lizg_anchor_find_dev: bad frame geometry, H stride or frame count");
  int sms = 0;
  if (int rc = device_ready(&sms)) return rc;
  const cudaError_t e = anchor_find_launch(span, d_luma, w, h, frame_stride, d_H, h_stride, d_lens, d_skip, frames, *out, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return record_error(LIZG_E_CUDA, (std::string("lizg_anchor_find_dev: ") + cudaGetErrorString(e)).c_str());
  return 0;
}

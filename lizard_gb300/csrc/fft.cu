// Row (b) of the hot path on sm_103a: the anchors' erase, the detrend projections and the 2D mixed-radix FFT of the
// n x n picture grid, restated from the reference's decode (liblizard/src/lizard_phy.c:1596-1716) for the GPU.
//
// Three kernels a batch:
//   hole_fit_kernel   one CTA a frame: the shading surface's right-hand side over every eighth sample outside the
//                     anchors' squares, times the inverse normal matrix: beta (6 doubles a frame);
//   fft_cols_kernel   a CTA takes 8 picture columns of a frame (4 complex lines: column x0 + j real, x0 + 4 + j
//                     imaginary), erases the anchors' squares as it loads them (beta's surface), sums each column's
//                     detrend moments, transforms the 4 lines along y in shared memory and separates the two real
//                     columns of each, writing Y[v][x] for the kept rows v (the used coefficients' v < vrows);
//   fft_rows_kernel   a CTA takes 4 kept rows v of a frame, reduces the columns' moments to the five projections,
//                     transforms along x and subtracts the surface's spectrum (the xy term everywhere, the x terms
//                     on v = 0, the y terms on u = 0), writing T[v][u].
// The transforms are Stockham autosort passes of radix 4, 2, 3 and 5 (every ladder size is 2^a 3^b 5^c) over
// shared-memory ping-pong buffers, twiddles from a table computed in double. FP32 throughout, as the reference's.
#include <cuda_runtime.h>
#include <stdint.h>
#include "lizg_internal.h"
#include "sample_dev.cuh"

namespace lizg {

__device__ __forceinline__ float2 cmul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }

// Forward DFTs (e^{-i}) of 2, 3, 4 and 5 points in place.
__device__ __forceinline__ void dft2(float2 *v) { const float2 a = v[0], b = v[1]; v[0] = cadd(a, b); v[1] = csub(a, b); }
__device__ __forceinline__ void dft4(float2 *v) {
  const float2 s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]), s13 = cadd(v[1], v[3]), d13 = csub(v[1], v[3]);
  v[0] = cadd(s02, s13); v[2] = csub(s02, s13);
  v[1] = make_float2(d02.x + d13.y, d02.y - d13.x);   // d02 - i d13
  v[3] = make_float2(d02.x - d13.y, d02.y + d13.x);   // d02 + i d13
}
__device__ __forceinline__ void dft3(float2 *v) {
  const float s3 = 0.86602540378443864676f;
  const float2 a = v[0], t = cadd(v[1], v[2]), d = csub(v[1], v[2]);
  const float2 m = make_float2(a.x - 0.5f * t.x, a.y - 0.5f * t.y);
  v[0] = cadd(a, t);
  v[1] = make_float2(m.x + s3 * d.y, m.y - s3 * d.x);   // m - i s3 d
  v[2] = make_float2(m.x - s3 * d.y, m.y + s3 * d.x);   // m + i s3 d
}
__device__ __forceinline__ void dft5(float2 *v) {
  const float c1 = 0.30901699437494742410f, c2 = -0.80901699437494742410f;   // cos 2pi/5, cos 4pi/5
  const float s1 = 0.95105651629515357212f, s2 = 0.58778525229247312917f;    // sin 2pi/5, sin 4pi/5
  const float2 a = v[0], p1 = cadd(v[1], v[4]), m1 = csub(v[1], v[4]), p2 = cadd(v[2], v[3]), m2 = csub(v[2], v[3]);
  const float2 r1 = make_float2(a.x + c1 * p1.x + c2 * p2.x, a.y + c1 * p1.y + c2 * p2.y);
  const float2 r2 = make_float2(a.x + c2 * p1.x + c1 * p2.x, a.y + c2 * p1.y + c1 * p2.y);
  const float2 q1 = make_float2(s1 * m1.x + s2 * m2.x, s1 * m1.y + s2 * m2.y);   // times -i below
  const float2 q2 = make_float2(s2 * m1.x - s1 * m2.x, s2 * m1.y - s1 * m2.y);
  v[0] = make_float2(a.x + p1.x + p2.x, a.y + p1.y + p2.y);
  v[1] = make_float2(r1.x + q1.y, r1.y - q1.x);
  v[4] = make_float2(r1.x - q1.y, r1.y + q1.x);
  v[2] = make_float2(r2.x + q2.y, r2.y - q2.x);
  v[3] = make_float2(r2.x - q2.y, r2.y + q2.x);
}

// L lines of n points (line l at a + l n) transformed along their length; b is as large as a. The passes alternate
// between the two; the result's buffer is returned. Every thread of the CTA takes part.
// n / d for n < 2^16 by the pass's precomputed reciprocal m = ceil(2^32 / d) (m = 0: d = 1).
__device__ __forceinline__ int fdiv(int n, uint32_t m) { return m ? (int)__umulhi((uint32_t)n, m) : n; }

__device__ float2 *fft_lines(float2 *a, float2 *b, int L, const FftDev &xd) {
  const int N = xd.n, tid = threadIdx.x, nth = blockDim.x;
  for (int s = 0; s < xd.nstages; s++) {
    const int R = xd.radix[s], NR = xd.nr[s], Ns = xd.ns[s], step = N / (Ns * R);
    const uint32_t mnr = xd.mnr[s], mns = xd.mns[s];
    for (int t = tid; t < L * NR; t += nth) {
      const int l = fdiv(t, mnr), j = t - l * NR, jq = fdiv(j, mns), k = j - jq * Ns;
      const float2 *in = a + l * N;
      float2 *out = b + l * N;
      float2 v[5];
      v[0] = in[j];
      for (int r = 1; r < R; r++) v[r] = cmul(in[j + r * NR], xd.tw[r * k * step]);
      if (R == 4) dft4(v); else if (R == 2) dft2(v); else if (R == 3) dft3(v); else dft5(v);
      const int base = jq * Ns * R + k;
      for (int r = 0; r < R; r++) out[base + r * Ns] = v[r];
    }
    __syncthreads();
    float2 *x = a; a = b; b = x;
  }
  return a;
}

// A frame's picture sample (x, y): read from a supplied grid, or sampled straight from the captured frame through
// its registration (the sampler fused into the pass that reads it).
__device__ __forceinline__ float src_at(const SrcDev &s, int f, int x, int y) {
  if (s.grid) return s.grid[f * s.gstride + (int64_t)y * s.sd.n + x];
  const float *H = s.reg + (int64_t)f * s.regstride;
  return sample_xy(s.sd, s.luma + f * s.fstride, s.w, s.h, s.pitch, H, H + 9, s.sd.colt[x], s.sd.rowt[y]);
}

__device__ __forceinline__ bool in_square(const FftDev &xd, int t) {
  bool in = false;
#pragma unroll
  for (int i = 0; i < 7; i++) in |= t >= xd.elo[i] && t <= xd.ehi[i];
  return in;
}

// The shading basis 1, c(x), q(x), c(y), q(y), c(x) c(y) at sample (x, y) (liblizard/src/lizard_phy.c:336-340).
__device__ __forceinline__ void hole_basis(const FftDev &xd, int x, int y, double b[6]) {
  const double cx = xd.cx[x], cy = xd.cx[y];
  b[0] = 1; b[1] = cx; b[2] = xd.qx[x]; b[3] = cy; b[4] = xd.qx[y]; b[5] = cx * cy;
}

__global__ void __launch_bounds__(256) hole_fit_kernel(FftDev xd, SrcDev src, double *beta) {
  const int f = blockIdx.x, n = xd.n, c = n / 8;
  double rhs[6] = {0, 0, 0, 0, 0, 0};
  for (int k = threadIdx.x; k < c * c; k += blockDim.x) {
    const int x = 8 * (k % c), y = 8 * (k / c);
    if (in_square(xd, x) && in_square(xd, y)) continue;
    const double v = src_at(src, f, x, y);
    double b[6];
    hole_basis(xd, x, y, b);
    for (int r = 0; r < 6; r++) rhs[r] += b[r] * v;
  }
  __shared__ double red[6][256];
  for (int r = 0; r < 6; r++) red[r][threadIdx.x] = rhs[r];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) for (int r = 0; r < 6; r++) red[r][threadIdx.x] += red[r][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x < 6) {
    double acc = 0;
    for (int k = 0; k < 6; k++) acc += xd.hole_inv[threadIdx.x * 6 + k] * red[k][0];
    beta[f * 6 + threadIdx.x] = acc;
  }
}

constexpr int kColTile = 8;          // picture columns a column-pass CTA takes (kColTile / 2 complex lines)
constexpr int kRowTile = 4;          // kept rows a row-pass CTA takes

__global__ void __launch_bounds__(256) fft_cols_kernel(FftDev xd, SrcDev src, const double *beta, double *colsum, float2 *Y) {
  extern __shared__ float2 sm[];
  const int n = xd.n, tiles = n / kColTile, f = blockIdx.x / tiles, x0 = (blockIdx.x % tiles) * kColTile;
  constexpr int L = kColTile / 2;
  float2 *a = sm, *b = sm + L * n;
  double bt[6];
  for (int r = 0; r < 6; r++) bt[r] = beta[f * 6 + r];
  // load: thread t takes column j = t % 8 at rows y = t / 8, t / 8 + 32, ...; the anchors' squares are erased to
  // the shading surface as they are read; each column's z, z c(y), z q(y) summed on the way.
  const int j = threadIdx.x % kColTile, x = x0 + j;
  const bool xin = in_square(xd, x);
  float s0 = 0, s1 = 0, s2 = 0;
  for (int y = threadIdx.x / kColTile; y < n; y += blockDim.x / kColTile) {
    float v;
    if (xin && in_square(xd, y)) {
      double bb[6], h = 0;
      hole_basis(xd, x, y, bb);
      for (int r = 0; r < 6; r++) h += bt[r] * bb[r];
      v = (float)h;
    } else {
      v = src_at(src, f, x, y);
    }
    s0 += v; s1 += v * xd.cx[y]; s2 += v * xd.qx[y];
    float2 *dst = a + (j % L) * n + y;
    if (j < L) dst->x = v; else dst->y = v;
  }
  __shared__ double red[3][256];
  red[0][threadIdx.x] = s0; red[1][threadIdx.x] = s1; red[2][threadIdx.x] = s2;
  __syncthreads();
  if (threadIdx.x < kColTile) {
    double t0 = 0, t1 = 0, t2 = 0;
    for (int k = threadIdx.x; k < (int)blockDim.x; k += kColTile) { t0 += red[0][k]; t1 += red[1][k]; t2 += red[2][k]; }
    double *cs = colsum + ((int64_t)f * n + x0 + threadIdx.x) * 3;
    cs[0] = t0; cs[1] = t1; cs[2] = t2;
  }
  float2 *z = fft_lines(a, b, L, xd);
  // separate the two real columns of each line: A(v) = (Z(v) + conj Z(n - v)) / 2, B(v) = -i (Z(v) - conj Z(n - v)) / 2
  float2 *Yf = Y + (int64_t)f * xd.vrows * n;
  for (int t = threadIdx.x; t < xd.vrows * kColTile; t += blockDim.x) {
    const int v = t / kColTile, jj = t % kColTile, l = jj % L;
    const float2 zv = z[l * n + v], zm = z[l * n + (n - v) % n];
    float2 o;
    if (jj < L) o = make_float2(0.5f * (zv.x + zm.x), 0.5f * (zv.y - zm.y));
    else o = make_float2(0.5f * (zv.y + zm.y), -0.5f * (zv.x - zm.x));
    Yf[(int64_t)v * n + x0 + jj] = o;
  }
}

// The five projections of each frame from its columns' moments, normalised (liblizard/src/lizard_phy.c:1584-1591,
// 1718): px, py, pxy, pxx, pyy.
__global__ void __launch_bounds__(256) proj_kernel(FftDev xd, const double *colsum, double *proj) {
  const int f = blockIdx.x, n = xd.n;
  const double *cs = colsum + (int64_t)f * n * 3;
  double p[5] = {0, 0, 0, 0, 0};
  for (int xx = threadIdx.x; xx < n; xx += blockDim.x) {
    const double c = xd.cx[xx], q = xd.qx[xx], S0 = cs[3 * xx], S1 = cs[3 * xx + 1], S2 = cs[3 * xx + 2];
    p[0] += c * S0; p[1] += S1; p[2] += c * S1; p[3] += q * S0; p[4] += S2;
  }
  __shared__ double red[5][256];
  for (int r = 0; r < 5; r++) red[r][threadIdx.x] = p[r];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) for (int r = 0; r < 5; r++) red[r][threadIdx.x] += red[r][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double *o = proj + 5 * f;
    o[0] = red[0][0] / (n * xd.sx2); o[1] = red[1][0] / (n * xd.sx2); o[2] = red[2][0] / (xd.sx2 * xd.sx2);
    o[3] = red[3][0] / (n * xd.sq2); o[4] = red[4][0] / (n * xd.sq2);
  }
}

__global__ void __launch_bounds__(256) fft_rows_kernel(FftDev xd, const double *proj, const float2 *Y, float2 *T) {
  extern __shared__ float2 sm[];
  const int n = xd.n, tiles = (xd.vrows + kRowTile - 1) / kRowTile, f = blockIdx.x / tiles, v0 = (blockIdx.x % tiles) * kRowTile;
  const int L = min(kRowTile, xd.vrows - v0);
  float2 *a = sm, *b = sm + kRowTile * n;
  const float2 *Yf = Y + (int64_t)f * xd.vrows * n;
  for (int t = threadIdx.x; t < L * n; t += blockDim.x) a[t] = Yf[(int64_t)v0 * n + t];
  __syncthreads();
  float2 *z = fft_lines(a, b, L, xd);
  float2 *Tf = T + (int64_t)f * xd.vrows * n;
  const double *pj = proj + 5 * f;
  const double px = pj[0], py = pj[1], pxy = pj[2], pxx = pj[3], pyy = pj[4];
  // the surface's spectrum off (liblizard/src/lizard_phy.c:1697-1716): the xy term's column factor pxy X1[u] worked
  // out once a u for the CTA's rows, then the x terms on v = 0 and the y terms on u = 0
  for (int u = threadIdx.x; u < n; u += blockDim.x) {
    const float2 x1u = xd.x1[u];
    const float ar = (float)(pxy * x1u.x), ai = (float)(pxy * x1u.y);
    float2 c0 = make_float2(0, 0);
    if (v0 == 0) {
      const float2 x2u = xd.x2[u];
      c0 = make_float2((float)(n * (px * x1u.x + pxx * x2u.x)), (float)(n * (px * x1u.y + pxx * x2u.y)));
    }
    for (int l = 0; l < L; l++) {
      const int v = v0 + l;
      float2 o = z[l * n + u];
      const float2 x1v = xd.x1[v];
      o.x -= ar * x1v.x - ai * x1v.y;
      o.y -= ar * x1v.y + ai * x1v.x;
      if (v == 0) { o.x -= c0.x; o.y -= c0.y; }
      if (u == 0) {
        const float2 x2v = xd.x2[v];
        o.x -= (float)(n * (py * x1v.x + pyy * x2v.x));
        o.y -= (float)(n * (py * x1v.y + pyy * x2v.y));
      }
      Tf[(int64_t)v * n + u] = o;
    }
  }
}

// coef[f][i] = T[f][tix[i]]: the used coefficients in pos order (for a caller that wants the spectrum itself).
__global__ void gather_coef_kernel(const float2 *T, int64_t tstride, const int32_t *tix, int need, int frames, float2 *coef) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= (int64_t)frames * need) return;
  const int f = (int)(g / need), i = (int)(g % need);
  coef[g] = T[f * tstride + tix[i]];
}

static bool g_attr[2] = {false, false};

cudaError_t fft_launch(const FftDev &xd, int frames, const SrcDev &src, double *beta, double *colsum, double *proj,
                       float2 *Y, float2 *T, cudaStream_t st) {
  const int smc = 2 * (kColTile / 2) * xd.n * (int)sizeof(float2), smr = 2 * kRowTile * xd.n * (int)sizeof(float2);
  cudaError_t e;
  if (!g_attr[0]) {
    if ((e = cudaFuncSetAttribute(fft_cols_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * 4 * 1536 * 8)) != cudaSuccess) return e;
    if ((e = cudaFuncSetAttribute(fft_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * kRowTile * 1536 * 8)) != cudaSuccess) return e;
    g_attr[0] = true;
  }
  hole_fit_kernel<<<frames, 256, 0, st>>>(xd, src, beta);
  fft_cols_kernel<<<frames * (xd.n / kColTile), 256, smc, st>>>(xd, src, beta, colsum, Y);
  proj_kernel<<<frames, 256, 0, st>>>(xd, colsum, proj);
  fft_rows_kernel<<<frames * ((xd.vrows + kRowTile - 1) / kRowTile), 256, smr, st>>>(xd, proj, Y, T);
  return cudaGetLastError();
}

cudaError_t gather_coef_launch(const float2 *T, int64_t tstride, const int32_t *tix, int need, int frames, float2 *coef, cudaStream_t st) {
  const int64_t tot = (int64_t)frames * need;
  gather_coef_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(T, tstride, tix, need, frames, coef);
  return cudaGetLastError();
}

}  // namespace lizg

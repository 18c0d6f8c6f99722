// The registration's refinement from the anchors on sm_103a (include/lizard_gb300.h lizg_refine_*): for a batch of
// frames registered by a homography alone (a finder's corners), rounds of the anchor search (anchor.cu) and of the
// lens model the found anchors give about H, then the model written into the registration's node mesh, so the
// receiver samples through H and the lens. Compiled with -fmad=false: the fit's sums, its solves and the model's
// values round as the reference's do.
//
// The fit restates the reference's anchor_model with lensm_fit's first round (liblizard/src/acquire.c:2038-2055,
// 1630-1669; lens_rows 1506-1512, solve_lens 1491-1504): the four corner nodes (no displacement) and the anchors found
// (their displacement about H), x and y about the frame's centre over its half-diagonal; the normal equations of the
// 8 + 3 term model summed once in the points' order; each model of 0..3 radial terms solved by Gauss-Jordan; the one
// of least AICc kept. One warp a frame: lane l sums entries l, l + 32, l + 64 of the 77 (upper triangle and right
// side) over the points in order; lane 0 solves.
#include <cuda_runtime.h>
#include <math.h>
#include <cmath>
#include <stdint.h>
#include <new>
#include <string>
#include "lizard_gb300.h"
#include "lizg_internal.h"

namespace lizg {

constexpr int kNA = 49, kLP = 11, kLStride = 15, kMaxPts = kNA + 4, kMargin15 = 15;

__device__ __forceinline__ void project_f(const float *h, float x, float y, float *u, float *v) {
  const float w = h[6] * x + h[7] * y + 1;
  *u = (h[0] * x + h[1] * y + h[2]) / w;
  *v = (h[3] * x + h[4] * y + h[5]) / w;
}

__device__ __forceinline__ void rows_of(double x, double y, double *rx, double *ry) {
  rx[0] = x; rx[1] = y; rx[2] = 0; rx[3] = 0; rx[4] = 1; rx[5] = 0; rx[6] = -x * x; rx[7] = -x * y;
  ry[0] = 0; ry[1] = 0; ry[2] = x; ry[3] = y; ry[4] = 0; ry[5] = 1; ry[6] = -x * y; ry[7] = -y * y;
  const double s = x * x + y * y;
  double sk = s;
  for (int k = 0; k < 3; k++, sk *= s) { rx[8 + k] = sk * x; ry[8 + k] = sk * y; }
}

struct FitArgs {
  int span, iw, ih, hstride, nn, a;
  double ax, ay, R;                // the model's axis (the frame's centre) and scale (its half-diagonal), host libm
  float node_lo, node_hi;          // the corner nodes' module coordinates (first and last of the lattice)
  int m0[7];
  const float *reg;                // frames x hstride: H first
  const uint8_t *ok;
  const float *dx, *dy;
  double *lens;                    // frames x 15
  int *have;
};

__global__ void __launch_bounds__(32) lens_fit_kernel(FitArgs a) {
  const int f = blockIdx.x, lane = threadIdx.x;
  __shared__ double s_rx[kMaxPts][kLP], s_ry[kMaxPts][kLP], s_d[kMaxPts][2], s_A[kLP][kLP + 1], A[kLP][kLP + 1];
  __shared__ int s_np;
  __shared__ float s_h[9];
  if (lane < 9) s_h[lane] = a.reg[(int64_t)f * a.hstride + lane];
  __syncwarp();
  const double ax = a.ax, ay = a.ay, R = a.R;
  if (lane == 0) {
    // the points in the reference's order: the four corner nodes, then the anchors found in row-major order
    int np = 0;
    for (int c = 0; c < 4; c++) {
      float u, v;
      project_f(s_h, (c == 1 || c == 2) ? a.node_hi : a.node_lo, c >= 2 ? a.node_hi : a.node_lo, &u, &v);
      rows_of((u - ax) / R, (v - ay) / R, s_rx[np], s_ry[np]);
      s_d[np][0] = 0; s_d[np][1] = 0; np++;
    }
    const float ah = a.a * 0.5f;
    for (int k = 0; k < kNA; k++) {
      const int64_t o = (int64_t)f * kNA + k;
      if (!a.ok[o]) continue;
      const float X = (float)a.m0[k % 7] + ah, Y = (float)a.m0[k / 7] + ah;
      float u, v;
      project_f(s_h, X, Y, &u, &v);
      rows_of((u - ax) / R, (v - ay) / R, s_rx[np], s_ry[np]);
      s_d[np][0] = a.dx[o]; s_d[np][1] = a.dy[o]; np++;
    }
    s_np = np;
  }
  __syncwarp();
  const int np = s_np;
  // the normal equations' upper triangle and right side, each entry summed over the points in order
  for (int e = lane; e < 77; e += 32) {
    int p, q;
    if (e < 66) { p = 0; int r = e; while (r >= kLP - p) { r -= kLP - p; p++; } q = p + r; }
    else { p = e - 66; q = kLP; }
    double acc = 0;
    for (int i = 0; i < np; i++)
      acc += q < kLP ? s_rx[i][p] * s_rx[i][q] + s_ry[i][p] * s_ry[i][q] : s_rx[i][p] * s_d[i][0] + s_ry[i][p] * s_d[i][1];
    s_A[p][q] = acc;
  }
  __syncwarp();
  if (lane != 0) return;
  for (int p = 1; p < kLP; p++) for (int q = 0; q < p; q++) s_A[p][q] = s_A[q][p];
  double best = INFINITY, tb[kLP];
  for (int c = 0; c < kLP; c++) tb[c] = 0;
  int K = -1;
  for (int k = 0; k <= 3; k++) {
    const int p = 8 + k;
    for (int r = 0; r < kLP; r++) for (int c = 0; c <= kLP; c++) A[r][c] = s_A[r][c];
    for (int c = 0; c < p; c++) A[c][c] += 1e-12;
    if (2 * np - p - 1 <= 0) continue;
    bool solved = true;
    for (int c = 0; c < p && solved; c++) {
      int pv = c;
      for (int r = c + 1; r < p; r++) if (fabs(A[r][c]) > fabs(A[pv][c])) pv = r;
      if (fabs(A[pv][c]) < 1e-14) { solved = false; break; }
      for (int kk = 0; kk <= kLP; kk++) { const double t = A[c][kk]; A[c][kk] = A[pv][kk]; A[pv][kk] = t; }
      for (int r = 0; r < p; r++) {
        if (r == c) continue;
        const double fr = A[r][c] / A[c][c];
        for (int kk = c; kk <= kLP; kk++) A[r][kk] -= fr * A[c][kk];
      }
    }
    if (!solved) continue;
    double t[kLP], rss = 0;
    for (int c = 0; c < kLP; c++) t[c] = 0;
    for (int c = 0; c < p; c++) t[c] = A[c][kLP] / A[c][c];
    for (int i = 0; i < np; i++) {
      double fx = 0, fy = 0;
      for (int c = 0; c < p; c++) { fx += t[c] * s_rx[i][c]; fy += t[c] * s_ry[i][c]; }
      rss += (s_d[i][0] - fx) * (s_d[i][0] - fx) + (s_d[i][1] - fy) * (s_d[i][1] - fy);
    }
    const double n2 = 2.0 * np, aicc = n2 * log(rss / n2 + 1e-30) + 2.0 * p + 2.0 * p * (p + 1) / (n2 - p - 1);
    if (aicc < best) { best = aicc; K = k; for (int c = 0; c < kLP; c++) tb[c] = t[c]; }
  }
  double *L = a.lens + (int64_t)f * kLStride;
  if (K < 0) {   // no model: no displacement
    L[0] = 0; L[1] = ax; L[2] = ay; L[3] = R;
    for (int c = 0; c < kLP; c++) L[4 + c] = 0;
    a.have[f] = 0;
    return;
  }
  L[0] = K; L[1] = ax; L[2] = ay; L[3] = R;
  for (int c = 0; c < kLP; c++) L[4 + c] = tb[c];
  a.have[f] = 1;
}

// The lens model's displacement at every node (through H) into the registration's mesh: reg[f][9 + 2 k] = dx, dy;
// zeros where no model fitted.
__global__ void __launch_bounds__(256) mesh_kernel(const double *lens, const int *have, const float *node, int nn, float *reg, int hstride) {
  const int f = blockIdx.x;
  float *rg = reg + (int64_t)f * hstride;
  const double *L = lens + (int64_t)f * kLStride;
  const bool on = have[f] != 0;
  for (int k = threadIdx.x; k < nn * nn; k += blockDim.x) {
    float dx = 0, dy = 0;
    if (on) {
      float u, v;
      project_f(rg, node[k % nn], node[k / nn], &u, &v);
      const int K = (int)L[0];
      const double x = (u - L[1]) / L[3], y = (v - L[2]) / L[3];
      double rx[kLP], ry[kLP];
      rows_of(x, y, rx, ry);
      double fx = 0, fy = 0;
      for (int c = 0; c < 8 + K; c++) { fx += L[4 + c] * rx[c]; fy += L[4 + c] * ry[c]; }
      dx = (float)fx; dy = (float)fy;
    }
    rg[9 + 2 * k] = dx; rg[10 + 2 * k] = dy;
  }
}

// The anchors found a frame.
__global__ void count_found_kernel(const uint8_t *ok, int32_t *found) {
  const int f = blockIdx.x;
  int c = threadIdx.x < kNA ? ok[(int64_t)f * kNA + threadIdx.x] : 0;
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  __shared__ int s[2];
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) found[f] = s[0] + s[1];
}

}  // namespace lizg

struct lizg_refiner {
  int span = 0, max_frames = 0, nn = 0;
  float *node = nullptr;
  uint8_t *ok = nullptr;
  float *peak = nullptr, *dx = nullptr, *dy = nullptr, *u = nullptr, *v = nullptr;
  double *lens = nullptr;
  int *have = nullptr;
};

extern "C" {

void lizg_refiner_free(lizg_refiner *r) {
  if (!r) return;
  void *ps[] = {r->node, r->ok, r->peak, r->dx, r->dy, r->u, r->v, r->lens, r->have};
  for (void *p : ps) if (p) cudaFree(p);
  delete r;
}

lizg_refiner *lizg_refiner_new(int span, int max_frames) {
  if (span != 128 && span != 256 && span != 512) { lizg::record_error(LIZG_E_ARG, "lizg_refiner_new: span must be 128, 256 or 512"); return nullptr; }
  if (max_frames < 1 || max_frames > 4096) { lizg::record_error(LIZG_E_ARG, "lizg_refiner_new: max_frames must be 1..4096"); return nullptr; }
  int sms = 0;
  if (lizg::device_ready(&sms)) return nullptr;
  lizg_refiner *r = new (std::nothrow) lizg_refiner;
  if (!r) { lizg::record_error(LIZG_E_NOMEM, "lizg_refiner_new: out of host memory"); return nullptr; }
  r->span = span; r->max_frames = max_frames;
  float nodes[40];
  r->nn = lizg::layout_nodes(span + 2 * lizg::kMargin15, nodes);
  const size_t F = (size_t)max_frames, A = F * lizg::kNA;
  cudaError_t e = cudaSuccess;
  auto al = [&](void **p, size_t b) { if (e == cudaSuccess) e = cudaMalloc(p, b); };
  al((void **)&r->node, sizeof(float) * r->nn);
  al((void **)&r->ok, A); al((void **)&r->peak, 4 * A); al((void **)&r->dx, 4 * A); al((void **)&r->dy, 4 * A);
  al((void **)&r->u, 4 * A); al((void **)&r->v, 4 * A);
  al((void **)&r->lens, sizeof(double) * F * lizg::kLStride); al((void **)&r->have, sizeof(int) * F);
  if (e == cudaSuccess) e = cudaMemcpy(r->node, nodes, sizeof(float) * r->nn, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    lizg::record_error(LIZG_E_CUDA, (std::string("lizg_refiner_new: ") + cudaGetErrorString(e)).c_str());
    lizg_refiner_free(r);
    return nullptr;
  }
  return r;
}

int lizg_refine_dev(lizg_refiner *r, const uint8_t *d_luma, int w, int h, int64_t frame_stride, float *d_reg, int frames, int rounds,
                    int32_t *d_found, double *d_lens, void *stream) {
  using namespace lizg;
  if (!r || !d_luma || !d_reg) return record_error(LIZG_E_ARG, "lizg_refine_dev: NULL argument");
  if (frames < 1 || frames > r->max_frames || rounds < 1 || rounds > 8 || w < 2 || h < 2 || frame_stride < (int64_t)w * h)
    return record_error(LIZG_E_ARG, "lizg_refine_dev: frames, rounds or frame geometry out of range");
  int sms = 0;
  if (int rc = device_ready(&sms)) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int hstride = 9 + 2 * r->nn * r->nn;
  const lizg_anchor_out out{r->ok, r->peak, r->dx, r->dy, r->u, r->v};
  FitArgs fa{};
  fa.span = r->span; fa.iw = w; fa.ih = h; fa.hstride = hstride; fa.nn = r->nn; fa.a = r->span / 64;
  // the axis and scale as the reference's lensm_axis takes them (liblizard/src/acquire.c:1622-1628), no axis set
  fa.ax = (double)(w * 0.5f); fa.ay = (double)(h * 0.5f); fa.R = 0;
  for (int c = 0; c < 4; c++) { const double d = std::hypot((c & 1 ? w : 0) - fa.ax, (c & 2 ? h : 0) - fa.ay); if (d > fa.R) fa.R = d; }
  if (!(fa.R > 0)) fa.R = 1;
  {
    float nodes[40];
    layout_nodes(r->span + 2 * kMargin15, nodes);
    fa.node_lo = nodes[0]; fa.node_hi = nodes[r->nn - 1];
  }
  for (int i = 0; i < 7; i++) fa.m0[i] = (int)floor(kMargin15 + (double)r->span * (i + 0.5) / 7 - fa.a / 2.0 + 0.5);
  fa.reg = d_reg; fa.ok = r->ok; fa.dx = r->dx; fa.dy = r->dy; fa.lens = r->lens; fa.have = r->have;
  cudaError_t e = cudaMemsetAsync(r->ok, 0, (size_t)frames * kNA, st);
  for (int round = 0; round < rounds && e == cudaSuccess; round++) {
    // anchors not yet found, through H and (from the second round) the lens model so far; then the model again
    if ((e = anchor_find_launch(r->span, d_luma, w, h, frame_stride, d_reg, hstride, round ? r->lens : nullptr, r->ok, frames, out, st)) != cudaSuccess) break;
    lens_fit_kernel<<<frames, 32, 0, st>>>(fa);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    mesh_kernel<<<frames, 256, 0, st>>>(r->lens, r->have, r->node, r->nn, d_reg, hstride);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && d_lens) e = cudaMemcpyAsync(d_lens, r->lens, sizeof(double) * frames * kLStride, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && d_found) {
    count_found_kernel<<<frames, 64, 0, st>>>(r->ok, d_found);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return record_error(LIZG_E_CUDA, (std::string("lizg_refine_dev: ") + cudaGetErrorString(e)).c_str());
  return 0;
}

}  // extern "C"

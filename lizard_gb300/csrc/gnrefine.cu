// The registration refined from the known pilots: Gauss-Newton on the 8 homography parameters, the mismatch measured
// where the receiver measures it. The picture is sampled through the registration (H, then the node mesh) and the
// receiver's own front (the anchors' erase, the shading fit's subtraction, the 2D transform) takes it to the
// spectrum; every block tail's coefficients are pilots whose symbols the receiver knows up to a sign a block parity
// (liblizard/src/lizard_phy.c:280-329, 451-472). The front is linear in the picture, so the Jacobian of the pilots'
// coefficients in H is that same front applied to eight tangent pictures (the image's gradient at each sample times
// the warp's derivative in each parameter), exact to the bilinear read, with the warp recomputed from H and the mesh
// at every sample rather than stored. Forward mode: Gauss-Newton needs J^T J, which eight tangents give whole.
//
// The mismatch: each pilot against its symbol times a real gain fitted a radius band and block parity (the blur's
// response is real and radial; a gain a block would absorb the phase ramps that carry the registration's error).
// Each step's normal equations are summed in double in a fixed order (the result is reproducible) and solved with
// the columns scaled. A step is kept only where the mismatch falls; otherwise it is halved from the best registration
// so far. The plain registration is the baseline and the fallback: a frame whose mismatch never falls keeps it.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <algorithm>
#include <cmath>
#include <new>
#include <string>
#include <vector>
#include "format.h"
#include "lizard_codes.h"
#include "lizard_gb300.h"
#include "lizg_internal.h"
#include "reg_dev.cuh"

namespace lizg {

constexpr int kGnThreads = 256, kGnParams = 8, kGnBins = 8, kGnGroups = 2 * kGnBins, kGnPics = 1 + kGnParams;
constexpr int kGnSums = kGnParams * (kGnParams + 1) / 2 + kGnParams + 1;   // N's upper triangle, J^T r, the loss

struct GnArgs {
  int n, nn, w, h, reg_stride, npilot, need;
  int64_t fstride;
  float g0, step;
  float pos[40];
  const uint8_t *luma;
  const float *reg;        // the frames' registrations (the mesh is read from here)
  const int32_t *pilot;    // pos index of each pilot coefficient
  const float2 *shat;      // its symbol for a count bit of 0
  const uint8_t *group;    // parity * kGnBins + radius band
};

struct GnState {
  float Hc[9], Hbest[9];
  double loss_best, dbest[kGnParams];
  float scale;
  int evals, improved;
};

// The picture sample (x, y) and its eight tangents in h0..h7: the module point, H, the mesh's bilinear displacement
// (acquire.c:5095-5105), the bilinear read at gamma 1 and its gradient.
__global__ void __launch_bounds__(kGnThreads) gn_tangent_kernel(GnArgs a, const GnState *st, float *grids) {
  const int f = blockIdx.x / a.n, y = blockIdx.x % a.n;
  const float *h = st[f].Hc;
  const float *reg = a.reg + (int64_t)f * a.reg_stride;
  const uint8_t *px = a.luma + f * a.fstride;
  const int64_t n2 = (int64_t)a.n * a.n;
  float *g0 = grids + (int64_t)f * kGnPics * n2 + (int64_t)y * a.n;
  const float my = a.g0 + (float)y * a.step;
  int j = 0;
  { int hi = a.nn - 2; while (j < hi) { const int mid = (j + hi + 1) >> 1; if (my >= a.pos[mid]) j = mid; else hi = mid - 1; } }
  const float vv = (my - a.pos[j]) / (a.pos[j + 1] - a.pos[j]);
  for (int x = threadIdx.x; x < a.n; x += blockDim.x) {
    const float mx = a.g0 + (float)x * a.step;
    int i = 0;
    { int hi = a.nn - 2; while (i < hi) { const int mid = (i + hi + 1) >> 1; if (mx >= a.pos[mid]) i = mid; else hi = mid - 1; } }
    const float uu = (mx - a.pos[i]) / (a.pos[i + 1] - a.pos[i]);
    const float *n00 = reg + 9 + 2 * (j * a.nn + i), *n10 = n00 + 2, *n01 = n00 + 2 * a.nn, *n11 = n01 + 2;
    const float mdx = (n00[0] * (1 - uu) + n10[0] * uu) * (1 - vv) + (n01[0] * (1 - uu) + n11[0] * uu) * vv;
    const float mdy = (n00[1] * (1 - uu) + n10[1] * uu) * (1 - vv) + (n01[1] * (1 - uu) + n11[1] * uu) * vv;
    const float wd = h[6] * mx + h[7] * my + 1;
    const float U = (h[0] * mx + h[1] * my + h[2]) / wd, V = (h[3] * mx + h[4] * my + h[5]) / wd;
    float sx = U + mdx - 0.5f, sy = V + mdy - 0.5f;
    const float xm = (float)a.w - 1.001f, ym = (float)a.h - 1.001f;
    if (sx < 0) sx = 0; else if (sx > xm) sx = xm;
    if (sy < 0) sy = 0; else if (sy > ym) sy = ym;
    const int xi = sx >= 0 ? (int)sx : 0, yi = sy >= 0 ? (int)sy : 0;
    const float fx = sx - (float)xi, fy = sy - (float)yi;
    const uint8_t *p = px + (int64_t)yi * a.w + xi;
    const float A = grey_of(p[0]), B = grey_of(p[1]), C = grey_of(p[a.w]), D = grey_of(p[a.w + 1]);
    g0[x] = (A + (B - A) * fx) * (1 - fy) + (C + (D - C) * fx) * fy;
    const float Iu = (B - A) * (1 - fy) + (D - C) * fy, Iv = (C - A) * (1 - fx) + (D - B) * fx;
    const float iw = 1.0f / wd;
    const float du[kGnParams] = {mx * iw, my * iw, iw, 0.0f, 0.0f, 0.0f, -U * mx * iw, -U * my * iw};
    const float dv[kGnParams] = {0.0f, 0.0f, 0.0f, mx * iw, my * iw, iw, -V * mx * iw, -V * my * iw};
#pragma unroll
    for (int q = 0; q < kGnParams; q++) g0[(int64_t)(q + 1) * n2 + x] = Iu * du[q] + Iv * dv[q];
  }
}

// Sums a double over the CTA in a fixed order (a warp's tree, then the warps in turn).
__device__ double block_sum(double v, double *red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0;
  for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
  return t;
}

// A frame's pilots: the gains, the mismatch, the normal equations and the step; then the step kept or not.
__global__ void __launch_bounds__(kGnThreads) gn_step_kernel(GnArgs a, const float2 *coef, GnState *st, int last) {
  __shared__ double red[kGnThreads / 32], gain[kGnGroups], sums[kGnSums];
  const int f = blockIdx.x, tid = threadIdx.x;
  const float2 *C0 = coef + (int64_t)f * kGnPics * a.need;
  // the gains: sum Re(conj(s) C) / sum |s|^2 a group
  for (int g = 0; g < kGnGroups; g++) {
    double num = 0, den = 0;
    for (int k = tid; k < a.npilot; k += blockDim.x) {
      if (a.group[k] != g) continue;
      const float2 s = a.shat[k], c = C0[a.pilot[k]];
      num += (double)s.x * c.x + (double)s.y * c.y;
      den += (double)s.x * s.x + (double)s.y * s.y;
    }
    num = block_sum(num, red);
    den = block_sum(den, red);
    if (tid == 0) gain[g] = den > 0 ? num / den : 0.0;
  }
  __syncthreads();
  // the mismatch r = C - gain s, J^T J, J^T r and the loss, a thread's pilots then the CTA
  double acc[kGnSums];
#pragma unroll
  for (int q = 0; q < kGnSums; q++) acc[q] = 0;
  for (int k = tid; k < a.npilot; k += blockDim.x) {
    const int64_t pk = a.pilot[k];
    const float2 s = a.shat[k], c = C0[pk];
    const double gk = gain[a.group[k]];
    const double rx = c.x - gk * s.x, ry = c.y - gk * s.y;
    double jx[kGnParams], jy[kGnParams];
#pragma unroll
    for (int q = 0; q < kGnParams; q++) { const float2 jq = C0[(int64_t)(q + 1) * a.need + pk]; jx[q] = jq.x; jy[q] = jq.y; }
    int o = 0;
#pragma unroll
    for (int p = 0; p < kGnParams; p++)
#pragma unroll
      for (int q = p; q < kGnParams; q++) acc[o++] += jx[p] * jx[q] + jy[p] * jy[q];
#pragma unroll
    for (int p = 0; p < kGnParams; p++) acc[o++] += jx[p] * rx + jy[p] * ry;
    acc[o] += rx * rx + ry * ry;
  }
  for (int q = 0; q < kGnSums; q++) {
    const double t = block_sum(acc[q], red);
    if (tid == 0) sums[q] = t;
  }
  __syncthreads();
  if (tid != 0) return;
  GnState &S = st[f];
  const double loss = sums[kGnSums - 1];
  // the step at the current registration: columns scaled to unit norm, a little ridge, Gauss-Jordan with pivoting
  double N[kGnParams][kGnParams + 1], sc[kGnParams];
  int o = 0;
  for (int p = 0; p < kGnParams; p++)
    for (int q = p; q < kGnParams; q++) { N[p][q] = sums[o]; N[q][p] = sums[o]; o++; }
  for (int p = 0; p < kGnParams; p++) sc[p] = N[p][p] > 0 ? sqrt(N[p][p]) : 1.0;
  for (int p = 0; p < kGnParams; p++) {
    for (int q = 0; q < kGnParams; q++) N[p][q] /= sc[p] * sc[q];
    N[p][p] += 1e-9;
    N[p][kGnParams] = -sums[o + p] / sc[p];
  }
  bool ok = true;
  for (int c = 0; c < kGnParams && ok; c++) {
    int piv = c;
    for (int r = c + 1; r < kGnParams; r++) if (fabs(N[r][c]) > fabs(N[piv][c])) piv = r;
    if (!(fabs(N[piv][c]) > 1e-300)) { ok = false; break; }
    if (piv != c) for (int q = 0; q <= kGnParams; q++) { const double t = N[c][q]; N[c][q] = N[piv][q]; N[piv][q] = t; }
    const double d = N[c][c];
    for (int q = c; q <= kGnParams; q++) N[c][q] /= d;
    for (int r = 0; r < kGnParams; r++) {
      if (r == c) continue;
      const double m = N[r][c];
      if (m != 0) for (int q = c; q <= kGnParams; q++) N[r][q] -= m * N[c][q];
    }
  }
  double delta[kGnParams];
  for (int p = 0; p < kGnParams; p++) delta[p] = ok && isfinite(N[p][kGnParams]) ? N[p][kGnParams] / sc[p] : 0.0;
  // keep the registration if the mismatch fell (the first is the baseline), else halve the last step from the best
  if (S.evals == 0 || loss < S.loss_best) {
    if (S.evals > 0) S.improved = 1;
    S.loss_best = loss;
    for (int q = 0; q < 9; q++) S.Hbest[q] = S.Hc[q];
    for (int p = 0; p < kGnParams; p++) S.dbest[p] = delta[p];
    S.scale = 1.0f;
  } else {
    S.scale *= 0.5f;
  }
  S.evals++;
  for (int q = 0; q < 9; q++) S.Hc[q] = S.Hbest[q];
  if (!last) for (int p = 0; p < kGnParams; p++) S.Hc[p] = (float)((double)S.Hbest[p] + S.scale * S.dbest[p]);
}

__global__ void gn_load_kernel(const float *reg, int reg_stride, int frames, GnState *st) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= frames) return;
  GnState &S = st[f];
  for (int q = 0; q < 9; q++) S.Hc[q] = S.Hbest[q] = reg[(int64_t)f * reg_stride + q];
  S.loss_best = 0; S.scale = 1.0f; S.evals = 0; S.improved = 0;
  for (int p = 0; p < kGnParams; p++) S.dbest[p] = 0;
}

__global__ void gn_store_kernel(const GnState *st, int frames, float *reg, int reg_stride, float *loss_out, int32_t *improved_out) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= frames) return;
  for (int q = 0; q < 9; q++) reg[(int64_t)f * reg_stride + q] = st[f].Hbest[q];
  if (loss_out) loss_out[f] = (float)st[f].loss_best;
  if (improved_out) improved_out[f] = st[f].improved;
}

}  // namespace lizg

struct lizg_gn {
  lizg::Format f;
  lizg::GnArgs a{};
  lizg_rx *rx = nullptr;
  int chunk = 0;
  float *grids = nullptr;
  float2 *coef = nullptr;
  lizg::GnState *state = nullptr;
  std::vector<void *> owned;
};

extern "C" {

lizg_gn *lizg_gn_new(int n, int subch, int span, int chunk) {
  using namespace lizg;
  if (chunk < 1 || chunk > 64) { record_error(LIZG_E_ARG, "lizg_gn_new: chunk must be 1..64"); return nullptr; }
  int sms = 0;
  if (device_ready(&sms)) return nullptr;
  lizg_gn *g = new (std::nothrow) lizg_gn();
  if (!g) { record_error(LIZG_E_NOMEM, "lizg_gn_new: out of host memory"); return nullptr; }
  if (format_build(n, subch, span, g->f)) { delete g; record_error(LIZG_E_ARG, "lizg_gn_new: no such format"); return nullptr; }
  const Format &f = g->f;
  // the pilots: their symbols (count bit 0) and groups (block parity, radius band by quantile)
  std::vector<int32_t> pk;
  std::vector<float2> shat;
  std::vector<int> par;
  std::vector<double> rho;
  const float qa = 0.70710678f;
  for (int b = 0; b < f.blocks; b++) {
    const Tier &tr = f.tier[f.block_tier[b]];
    const int first = f.block_slot[b] / 2;
    for (int s = tr.nt / 2; s < tr.slots / 2; s++) {
      const int k = first + s;
      pk.push_back(k);
      shat.push_back(make_float2(f.white[2 * k] ? -qa : qa, f.white[2 * k + 1] ? -qa : qa));
      par.push_back(b & 1);
      rho.push_back(std::hypot((double)f.uv[2 * k], (double)f.uv[2 * k + 1]));
    }
  }
  const int np = (int)pk.size();
  std::vector<double> sorted = rho;
  std::sort(sorted.begin(), sorted.end());
  std::vector<uint8_t> grp(np);
  for (int k = 0; k < np; k++) {
    int bin = 0;
    for (int q = 1; q < kGnBins; q++) if (np && rho[k] > sorted[(size_t)((double)q * (np - 1) / kGnBins)]) bin = q;
    grp[k] = (uint8_t)(par[k] * kGnBins + bin);
  }
  GnArgs &a = g->a;
  a.n = n; a.npilot = np; a.need = subch * kSub;
  a.g0 = kMargin + 0.5f / f.scale; a.step = 1.0f / f.scale;
  a.nn = layout_nodes(span + 2 * kMargin, a.pos);
  a.reg_stride = 9 + 2 * a.nn * a.nn;
  g->chunk = chunk;
  auto up = [&](const void *src, size_t bytes, void **dst) -> bool {
    if (cudaMalloc(dst, std::max<size_t>(bytes, 1)) != cudaSuccess) return false;
    g->owned.push_back(*dst);
    return !src || !bytes || cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice) == cudaSuccess;   // no source: scratch
  };
  void *p1 = nullptr, *p2 = nullptr, *p3 = nullptr, *p4 = nullptr, *p5 = nullptr, *p6 = nullptr;
  bool ok = np >= 16 && up(pk.data(), pk.size() * 4, &p1) && up(shat.data(), shat.size() * sizeof(float2), &p2) && up(grp.data(), grp.size(), &p3);
  ok = ok && up(nullptr, sizeof(float) * (size_t)chunk * kGnPics * n * n, &p4) && up(nullptr, sizeof(float2) * (size_t)chunk * kGnPics * a.need, &p5) &&
       up(nullptr, sizeof(GnState) * (size_t)chunk, &p6);
  if (ok) {
    a.pilot = static_cast<int32_t *>(p1); a.shat = static_cast<float2 *>(p2); a.group = static_cast<uint8_t *>(p3);
    g->grids = static_cast<float *>(p4); g->coef = static_cast<float2 *>(p5); g->state = static_cast<GnState *>(p6);
    g->rx = lizg_rx_new(n, subch, span, chunk * kGnPics);
    ok = g->rx != nullptr;
  }
  if (!ok) {
    lizg_gn_free(g);
    record_error(LIZG_E_NOMEM, np < 16 ? "lizg_gn_new: the format has too few pilots" : "lizg_gn_new: device allocation failed");
    return nullptr;
  }
  return g;
}

void lizg_gn_free(lizg_gn *g) {
  if (!g) return;
  if (g->rx) lizg_rx_free(g->rx);
  for (void *p : g->owned) cudaFree(p);
  delete g;
}

int lizg_gn_pictures_dev(lizg_gn *g, const uint8_t *d_luma, int w, int h, int64_t frame_stride, const float *d_reg, int frames, float *d_pics,
                         void *stream) {
  using namespace lizg;
  if (!g || !d_luma || !d_reg || !d_pics || frames < 1 || frames > g->chunk || w < 2 || h < 2 || (frames > 1 && frame_stride < (int64_t)w * h))
    return record_error(LIZG_E_ARG, "lizg_gn_pictures_dev: NULL argument, frames outside 1..chunk or frame under 2 x 2");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  GnArgs a = g->a;
  a.w = w; a.h = h; a.fstride = frame_stride; a.luma = d_luma; a.reg = d_reg;
  gn_load_kernel<<<(frames + 127) / 128, 128, 0, st>>>(d_reg, a.reg_stride, frames, g->state);
  gn_tangent_kernel<<<frames * a.n, kGnThreads, 0, st>>>(a, g->state, d_pics);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : record_error(LIZG_E_CUDA, (std::string("lizg_gn_pictures_dev: ") + cudaGetErrorString(e)).c_str());
}

int lizg_gn_refine_dev(lizg_gn *g, const uint8_t *d_luma, int w, int h, int64_t frame_stride, float *d_reg, int frames, int steps, float *d_loss,
                       int32_t *d_improved, void *stream) {
  using namespace lizg;
  if (!g || !d_luma || !d_reg || frames < 1 || steps < 0 || steps > 16 || w < 2 || h < 2 || (frames > 1 && frame_stride < (int64_t)w * h))
    return record_error(LIZG_E_ARG, "lizg_gn_refine_dev: NULL argument, empty batch, steps outside 0..16 or frame under 2 x 2");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  for (int f0 = 0; f0 < frames; f0 += g->chunk) {
    const int fc = std::min(g->chunk, frames - f0);
    GnArgs a = g->a;
    a.w = w; a.h = h; a.fstride = frame_stride;
    a.luma = d_luma + (int64_t)f0 * frame_stride;
    a.reg = d_reg + (int64_t)f0 * a.reg_stride;
    gn_load_kernel<<<(fc + 127) / 128, 128, 0, st>>>(a.reg, a.reg_stride, fc, g->state);
    for (int e = 0; e <= steps; e++) {   // steps + 1 evaluations: the baseline, then each step's
      gn_tangent_kernel<<<fc * a.n, kGnThreads, 0, st>>>(a, g->state, g->grids);
      if (cudaGetLastError() != cudaSuccess) return record_error(LIZG_E_CUDA, "lizg_gn_refine_dev: tangent launch failed");
      if (int rc = lizg_rx_spectrum_grid_dev(g->rx, g->grids, fc * kGnPics, reinterpret_cast<float *>(g->coef), stream)) return rc;
      gn_step_kernel<<<fc, kGnThreads, 0, st>>>(a, g->coef, g->state, e == steps);
    }
    gn_store_kernel<<<(fc + 127) / 128, 128, 0, st>>>(g->state, fc, d_reg + (int64_t)f0 * a.reg_stride, a.reg_stride, d_loss ? d_loss + f0 : nullptr,
                                                      d_improved ? d_improved + f0 : nullptr);
  }
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : record_error(LIZG_E_CUDA, (std::string("lizg_gn_refine_dev: ") + cudaGetErrorString(e)).c_str());
}

}  // extern "C"

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
#include <cstddef>
#include <math.h>
#include <cmath>
#include <stdint.h>
#include <new>
#include <string>
#include "lizard_gb300.h"
#include "lizg_internal.h"
#include "reg_dev.cuh"

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
  const int *gate;                 // frames, may be NULL: 0 where no model is fitted (have 0)
};

// Gauss-Jordan with partial pivoting on the first p rows of A (the right-hand side in column kLP) across a warp, the
// reference's solve_lens (liblizard/src/acquire.c:1491-1504) operation for operation: lane 0 finds the pivot (the
// first largest magnitude), the lanes swap the two rows, take each row's factor from its pivot-column entry, then
// update every (row, column) entry, each with the product and subtraction the serial loop makes. Returns (on every
// lane) 0 where a pivot falls under thresh.
__device__ bool warp_gj(double (*A)[kLP + 1], int p, double thresh, double *s_f, int *s_piv) {
  const int lane = threadIdx.x & 31;
  for (int c = 0; c < p; c++) {
    if (lane == 0) {
      int pv = c;
      for (int r = c + 1; r < p; r++) if (fabs(A[r][c]) > fabs(A[pv][c])) pv = r;
      s_piv[0] = pv;
      s_piv[1] = fabs(A[pv][c]) < thresh;
    }
    __syncwarp();
    if (s_piv[1]) return false;
    const int pv = s_piv[0];
    if (pv != c)
      for (int k = lane; k <= kLP; k += 32) { const double t = A[c][k]; A[c][k] = A[pv][k]; A[pv][k] = t; }
    __syncwarp();
    for (int r = lane; r < p; r += 32) s_f[r] = r == c ? 0.0 : A[r][c] / A[c][c];
    __syncwarp();
    const int ncol = kLP + 1 - c;
    for (int e = lane; e < p * ncol; e += 32) {
      const int r = e / ncol, k = c + (e - r * ncol);
      if (r != c) A[r][k] -= s_f[r] * A[c][k];
    }
    __syncwarp();
  }
  return true;
}

// A fitting block: 4 warps, one a model of K = 0..3 radial terms.
constexpr int kFitThreads = 128;
struct FitScratch {
  double A[4][kLP][kLP + 1];
  double f[4][kLP], t[4][kLP], term[4][kMaxPts], aicc[4], tb[kLP];
  int ok[4], piv[4][2], K;
};

// lensm_fit's models over the points (liblizard/src/acquire.c:1651-1668) from its summed normal equations sA (upper
// triangle and right side; n of the np points not dropped), on a block of kFitThreads: warp k solves the system of
// 8 + k unknowns (warp_gj), its lanes each point's residual term, its lane 0 their sum over the points in order and
// AICc; thread 0 keeps the least in the order k = 0..3. Out: F.tb, F.K (-1 where none solved).
__device__ void block_models(int np, int n, double (*rx)[kLP], double (*ry)[kLP], double (*d)[2], const uint8_t *drop, double (*sA)[kLP + 1],
                             FitScratch &F) {
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  for (int e = tid; e < kLP * kLP; e += blockDim.x) {
    const int p = e / kLP, q = e - p * kLP;
    if (p > q) sA[p][q] = sA[q][p];
  }
  __syncthreads();
  if (w < 4) {
    const int k = w, p = 8 + k;
    double (*A)[kLP + 1] = F.A[k];
    for (int e = lane; e < kLP * (kLP + 1); e += 32) {
      const int r = e / (kLP + 1), c = e - r * (kLP + 1);
      A[r][c] = sA[r][c] + (r == c && c < p ? 1e-12 : 0.0);
    }
    __syncwarp();
    const bool ok = 2 * n - p - 1 > 0 && warp_gj(A, p, 1e-14, F.f[k], F.piv[k]);
    if (ok) {
      for (int c = lane; c < kLP; c += 32) F.t[k][c] = c < p ? A[c][kLP] / A[c][c] : 0.0;
      __syncwarp();
      for (int i = lane; i < np; i += 32) {
        if (drop && drop[i]) continue;
        double fx = 0, fy = 0;
        for (int c = 0; c < p; c++) { fx += F.t[k][c] * rx[i][c]; fy += F.t[k][c] * ry[i][c]; }
        F.term[k][i] = (d[i][0] - fx) * (d[i][0] - fx) + (d[i][1] - fy) * (d[i][1] - fy);
      }
      __syncwarp();
      if (lane == 0) {
        double rss = 0;
        for (int i = 0; i < np; i++)
          if (!(drop && drop[i])) rss += F.term[k][i];
        const double n2 = 2.0 * n;
        F.aicc[k] = n2 * log(rss / n2 + 1e-30) + 2.0 * p + 2.0 * p * (p + 1) / (n2 - p - 1);
      }
    }
    if (lane == 0) F.ok[k] = ok;
  }
  __syncthreads();
  if (tid == 0) {
    double best = INFINITY;
    F.K = -1;
    for (int c = 0; c < kLP; c++) F.tb[c] = 0;
    for (int k = 0; k <= 3; k++)
      if (F.ok[k] && F.aicc[k] < best) { best = F.aicc[k]; F.K = k; for (int c = 0; c < kLP; c++) F.tb[c] = F.t[k][c]; }
  }
  __syncthreads();
}

// The normal equations' upper triangle and right side over the points not dropped (drop NULL: all), an entry a thread,
// each summed over the points in their order.
__device__ void block_normal(int np, double (*rx)[kLP], double (*ry)[kLP], double (*d)[2], const uint8_t *drop, double (*sA)[kLP + 1]) {
  for (int e = threadIdx.x; e < 77; e += blockDim.x) {
    int p, q;
    if (e < 66) { p = 0; int r = e; while (r >= kLP - p) { r -= kLP - p; p++; } q = p + r; }
    else { p = e - 66; q = kLP; }
    double acc = 0;
    for (int i = 0; i < np; i++)
      if (!(drop && drop[i])) acc += q < kLP ? rx[i][p] * rx[i][q] + ry[i][p] * ry[i][q] : rx[i][p] * d[i][0] + ry[i][p] * d[i][1];
    sA[p][q] = acc;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kFitThreads) lens_fit_kernel(FitArgs a) {
  const int f = blockIdx.x, tid = threadIdx.x;
  if (a.gate && !a.gate[f]) {
    if (tid == 0) a.have[f] = 0;
    return;
  }
  __shared__ double s_rx[kMaxPts][kLP], s_ry[kMaxPts][kLP], s_d[kMaxPts][2], s_A[kLP][kLP + 1];
  __shared__ FitScratch F;
  __shared__ int s_np, s_at[kNA];
  __shared__ float s_h[9];
  if (tid < 9) s_h[tid] = a.reg[(int64_t)f * a.hstride + tid];
  if (tid == 0) {
    // the points in the reference's order: the four corner nodes, then the anchors found in row-major order
    int np = 4;
    for (int k = 0; k < kNA; k++) s_at[k] = a.ok[(int64_t)f * kNA + k] ? np++ : -1;
    s_np = np;
  }
  __syncthreads();
  const double ax = a.ax, ay = a.ay, R = a.R;
  const float ah = a.a * 0.5f;
  for (int t = tid; t < 4 + kNA; t += blockDim.x) {
    float u, v;
    if (t < 4) {
      project_f(s_h, (t == 1 || t == 2) ? a.node_hi : a.node_lo, t >= 2 ? a.node_hi : a.node_lo, &u, &v);
      rows_of((u - ax) / R, (v - ay) / R, s_rx[t], s_ry[t]);
      s_d[t][0] = 0; s_d[t][1] = 0;
    } else {
      const int k = t - 4, i = s_at[k];
      if (i < 0) continue;
      const int64_t o = (int64_t)f * kNA + k;
      project_f(s_h, (float)a.m0[k % 7] + ah, (float)a.m0[k / 7] + ah, &u, &v);
      rows_of((u - ax) / R, (v - ay) / R, s_rx[i], s_ry[i]);
      s_d[i][0] = a.dx[o]; s_d[i][1] = a.dy[o];
    }
  }
  __syncthreads();
  const int np = s_np;
  block_normal(np, s_rx, s_ry, s_d, nullptr, s_A);
  block_models(np, np, s_rx, s_ry, s_d, nullptr, s_A, F);
  if (tid != 0) return;
  double *L = a.lens + (int64_t)f * kLStride;
  if (F.K < 0) {   // no model: no displacement
    L[0] = 0; L[1] = ax; L[2] = ay; L[3] = R;
    for (int c = 0; c < kLP; c++) L[4 + c] = 0;
    a.have[f] = 0;
    return;
  }
  L[0] = F.K; L[1] = ax; L[2] = ay; L[3] = R;
  for (int c = 0; c < kLP; c++) L[4 + c] = F.tb[c];
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


// ---------------------------------------------------------------- the anchors' registration (acquire.c:2039-2197)
//
// The reference's anchor_register for a batch of frames: rounds of the anchor search through the homography the
// anchors found so far say (anchor_homo) and the lens model they say about it, held to the robust rule
// (anchor_model_free with lensm_fit's rounds); then each corner judged by that map and, where it disagrees by more
// than 3 modules, searched again (the border node search on the corner, through the corners' H and the joint model
// of the anchors and the kept corners) and H made again from the four corners; then the anchors' model about H.
// The serial parts run on one warp a frame: lanes sum the normal equations' entries (each entry over the points in
// order), lane 0 solves, judges and sorts, in double as the reference does.

constexpr int kRounds = 6, kAnchMin = 12, kCornerMod = 3;

// A frame's registration state between the kernels.
struct RegState {
  float H0[9], Ha[9], quad[8], hu[4], hv[4];
  float mpx;
  int have, nf, active, held, mc_on, moved;
  uint8_t redo[4];
};

struct RegArgs {
  int span, iw, ih, hstride, nn, a;
  double ax, ay, R;
  float node_lo, node_hi;
  int m0[7];
  float *reg;                      // frames x hstride: H first (in the corners', out the registration's)
  const float *quad_in;            // frames x 8, may be NULL (the corners through H)
  RegState *st;
  uint8_t *ok;
  float *dx, *dy, *u, *v;
  double *mf, *mc;                 // frames x 15: the anchors' own model (about Ha) and the joint one (about H)
  int *have_mf, *on_mc;            // frames: where each model holds (the anchor search and the corner search read them)
  const float *nodes;              // frames x nn^2 x 4: the corners' second search
};

// lensm_fit (liblizard/src/acquire.c:1630-1694) over np points whose rows (lens_rows at K = 3) are rx, ry, residuals
// d, places qx, qy, on a block of kFitThreads: the normal equations over the points not dropped (block_normal), the
// models (block_models); with robust, every point's distance from the model on its own thread, their median by
// ranks (each thread places its distances in the sorted order), the verdicts on thread 0, and round again while a
// verdict changes (at most four rounds). lens (shared, 15) receives the model (K, ax, ay, R, coefficients). Returns
// (on every thread) 1 where a model fitted.
__device__ int block_lensm_fit(int np, double (*rx)[kLP], double (*ry)[kLP], double (*d)[2], const double *qx, const double *qy, uint8_t *drop,
                               bool robust, double tau_floor, double ax, double ay, double R, double *lens, double (*sA)[kLP + 1],
                               FitScratch &F, double *res, double *srt, int *s_flag) {
  const int tid = threadIdx.x;
  int ok = 0;
  for (int round = 0; round < 4; round++) {
    int n = 0;
    for (int i = 0; i < np; i++) n += !drop[i];
    block_normal(np, rx, ry, d, drop, sA);
    block_models(np, n, rx, ry, d, drop, sA, F);
    if (F.K < 0) break;
    if (tid == 0) {
      lens[0] = F.K; lens[1] = ax; lens[2] = ay; lens[3] = R;
      for (int c = 0; c < kLP; c++) lens[4 + c] = F.tb[c];
    }
    ok = 1;
    __syncthreads();
    if (!robust || round == 3) break;
    // the robust rule: every point's distance from the model, tau from their median, the verdicts again
    for (int i = tid; i < np; i += blockDim.x) {
      float fx, fy;
      lens_at(lens, qx[i] * R + ax, qy[i] * R + ay, &fx, &fy);
      res[i] = hypot(d[i][0] - fx, d[i][1] - fy);
    }
    __syncthreads();
    for (int i = tid; i < np; i += blockDim.x) {   // the ascending order, ties by index: the sort's array
      int rank = 0;
      for (int j = 0; j < np; j++) rank += res[j] < res[i] || (res[j] == res[i] && j < i);
      srt[rank] = res[i];
    }
    __syncthreads();
    if (tid == 0) {
      const double tau = fmax(tau_floor, 3 * 1.4826 * srt[np / 2]);
      int changed = 0;
      for (int i = 0; i < np; i++) {
        const uint8_t bad = res[i] > tau;
        if (bad != drop[i]) { drop[i] = bad; changed++; }
      }
      s_flag[1] = changed > 0;
    }
    __syncthreads();
    if (!s_flag[1]) break;
  }
  return ok;
}

__global__ void reg_init_kernel(RegArgs a, int frames) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= frames) return;
  RegState &S = a.st[f];
  const float *h = a.reg + (int64_t)f * a.hstride;
  for (int k = 0; k < 9; k++) { S.H0[k] = h[k]; S.Ha[k] = h[k]; }
  const float lo = a.node_lo, hi = a.node_hi, src[8] = {lo, lo, hi, lo, hi, hi, lo, hi};
  for (int c = 0; c < 4; c++) {
    if (a.quad_in) { S.quad[2 * c] = a.quad_in[(int64_t)f * 8 + 2 * c]; S.quad[2 * c + 1] = a.quad_in[(int64_t)f * 8 + 2 * c + 1]; }
    else project_f(h, src[2 * c], src[2 * c + 1], &S.quad[2 * c], &S.quad[2 * c + 1]);
  }
  // pixels a module: the quad's sides over the lattice's, as the reference's acquisition measures it
  float mpx = 0;
  for (int k = 0; k < 4; k++) {
    const int k1 = (k + 1) & 3;
    mpx += hypotf(S.quad[2 * k1] - S.quad[2 * k], S.quad[2 * k1 + 1] - S.quad[2 * k + 1]) / hypotf(src[2 * k1] - src[2 * k], src[2 * k1 + 1] - src[2 * k + 1]) / 4;
  }
  S.mpx = mpx;
  S.have = 0; S.nf = 0; S.active = 1; S.held = 0; S.mc_on = 0; S.moved = 0;
  for (int c = 0; c < 4; c++) S.redo[c] = 0;
  a.have_mf[f] = 0; a.on_mc[f] = 0;
  for (int k = 0; k < kNA; k++) a.ok[(int64_t)f * kNA + k] = 0;
}

// One round's bookkeeping after the search: the anchors found, the homography they say, the robust model about it,
// the anchors it drops no longer found (acquire.c:2133-2143). A block of kFitThreads a frame.
__global__ void __launch_bounds__(kFitThreads) reg_round_kernel(RegArgs a, uint8_t *active) {
  const int f = blockIdx.x, tid = threadIdx.x;
  RegState &S = a.st[f];
  if (!S.active) return;
  __shared__ double s_rx[kNA][kLP], s_ry[kNA][kLP], s_d[kNA][2], s_qx[kNA], s_qy[kNA], s_A[kLP][kLP + 1], s_res[kNA], s_srt[kNA];
  __shared__ double s_M[kLP][kLP + 1], s_mean[6], s_lens[kLensStride], s_gf[kLP];
  __shared__ FitScratch F;
  __shared__ float s_X[kNA], s_Y[kNA], s_u[kNA], s_v[kNA];
  __shared__ uint8_t s_ok[kNA], s_drop[kNA];
  __shared__ int s_at[kNA], s_pos[kNA], s_np, s_flag[2], s_go, s_piv[2];
  const float ah = a.a * 0.5f;
  for (int k = tid; k < kNA; k += blockDim.x) {
    const int64_t o = (int64_t)f * kNA + k;
    s_ok[k] = a.ok[o]; s_u[k] = a.u[o]; s_v[k] = a.v[o];
    s_X[k] = (float)a.m0[k % 7] + ah; s_Y[k] = (float)a.m0[k / 7] + ah;
  }
  __syncthreads();
  if (tid == 0) {
    int now = 0;
    for (int k = 0; k < kNA; k++) now += s_ok[k];
    s_go = 1;
    if (now == S.nf || now < 4) { S.active = 0; active[f] = 0; s_go = 0; }
    else {
      S.nf = now;
      // anchor_homo (acquire.c:2062-2094): centres and scales, in the anchors' order
      int n = 0, rows = 0, cols = 0, rm = 0, cm = 0;
      double mx = 0, my = 0, mu = 0, mv = 0;
      for (int k = 0; k < kNA; k++) if (s_ok[k]) { n++; mx += s_X[k]; my += s_Y[k]; mu += s_u[k]; mv += s_v[k]; rm |= 1 << (k / 7); cm |= 1 << (k % 7); }
      for (int b = 0; b < 7; b++) { rows += (rm >> b) & 1; cols += (cm >> b) & 1; }
      double sx = 0, su = 0;
      int fit = n >= 8 && rows >= 3 && cols >= 3;
      if (fit) {
        mx /= n; my /= n; mu /= n; mv /= n;
        for (int k = 0; k < kNA; k++) if (s_ok[k]) { sx += hypot(s_X[k] - mx, s_Y[k] - my); su += hypot(s_u[k] - mu, s_v[k] - mv); }
        sx = sx / n / 1.4142135623730951; su = su / n / 1.4142135623730951;
        fit = sx > 0 && su > 0;
      }
      s_mean[0] = mx; s_mean[1] = my; s_mean[2] = mu; s_mean[3] = mv; s_mean[4] = sx; s_mean[5] = su;
      s_flag[0] = fit;
    }
  }
  __syncthreads();
  if (!s_go) return;
  if (s_flag[0]) {
    const double mx = s_mean[0], my = s_mean[1], mu = s_mean[2], mv = s_mean[3], sx = s_mean[4], su = s_mean[5];
    // the 8 x 8 normal equations and right side, an entry a thread, each over the anchors in order; the rest zero
    for (int e = tid; e < kLP * (kLP + 1); e += blockDim.x) {
      const int p = e / (kLP + 1), q = e - p * (kLP + 1);
      if (p >= 8 || (q >= 8 && q < kLP)) { s_M[p][q] = 0; continue; }
      double acc = 0;
      for (int k = 0; k < kNA; k++) {
        if (!s_ok[k]) continue;
        const double x = (s_X[k] - mx) / sx, y = (s_Y[k] - my) / sx, uu = (s_u[k] - mu) / su, vv = (s_v[k] - mv) / su;
        const double r0[8] = {x, y, 1, 0, 0, 0, -uu * x, -uu * y}, r1[8] = {0, 0, 0, x, y, 1, -vv * x, -vv * y};
        acc += q < kLP ? r0[p] * r0[q] + r1[p] * r1[q] : r0[p] * uu + r1[p] * vv;
      }
      s_M[p][q] = acc;
    }
    __syncthreads();
    if (tid < 32) {   // solve_lens(M, 8) on warp 0, then H through the centring
      const bool solved = warp_gj(s_M, 8, 1e-14, s_gf, s_piv);
      if (solved && tid == 0) {
        double g[9];
        for (int p = 0; p < 8; p++) g[p] = s_M[p][kLP] / s_M[p][p];
        g[8] = 1;
        const double tx[9] = {1 / sx, 0, -mx / sx, 0, 1 / sx, -my / sx, 0, 0, 1}, ti[9] = {su, 0, mu, 0, su, mv, 0, 0, 1};
        double gt[9], h[9];
        for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) { gt[3 * r + c] = 0; for (int k = 0; k < 3; k++) gt[3 * r + c] += g[3 * r + k] * tx[3 * k + c]; }
        for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) { h[3 * r + c] = 0; for (int k = 0; k < 3; k++) h[3 * r + c] += ti[3 * r + k] * gt[3 * k + c]; }
        if (fabs(h[8]) > 1e-12) for (int k = 0; k < 9; k++) S.Ha[k] = (float)(h[k] / h[8]);
      }
    }
    __syncthreads();
  }
  // anchor_model_free (acquire.c:2101-2118): the anchors' displacements about Ha, the robust rule at half a module
  if (tid == 0) {
    int np = 0;
    for (int k = 0; k < kNA; k++) s_pos[k] = s_ok[k] ? np++ : -1;
    s_np = np;
  }
  __syncthreads();
  for (int k = tid; k < kNA; k += blockDim.x) {
    const int i = s_pos[k];
    if (i < 0) continue;
    float hu, hv;
    project_f(S.Ha, s_X[k], s_Y[k], &hu, &hv);
    const float ddx = s_u[k] - hu, ddy = s_v[k] - hv;
    a.dx[(int64_t)f * kNA + k] = ddx; a.dy[(int64_t)f * kNA + k] = ddy;
    s_qx[i] = (hu - a.ax) / a.R; s_qy[i] = (hv - a.ay) / a.R;
    rows_of(s_qx[i], s_qy[i], s_rx[i], s_ry[i]);
    s_d[i][0] = ddx; s_d[i][1] = ddy; s_drop[i] = 0; s_at[i] = k;
  }
  __syncthreads();
  const int np = s_np;
  const int have = np >= 4 && block_lensm_fit(np, s_rx, s_ry, s_d, s_qx, s_qy, s_drop, true, 0.5 * (double)S.mpx, a.ax, a.ay, a.R, s_lens,
                                              s_A, F, s_res, s_srt, s_flag);
  if (tid == 0) {
    S.have = have;
    a.have_mf[f] = have;
    if (have) {
      for (int c = 0; c < kLensStride; c++) a.mf[(int64_t)f * kLensStride + c] = s_lens[c];
      for (int i = 0; i < np; i++) if (s_drop[i]) a.ok[(int64_t)f * kNA + s_at[i]] = 0;
      int nf = 0;
      for (int k = 0; k < kNA; k++) nf += a.ok[(int64_t)f * kNA + k];
      S.nf = nf;
    } else {
      S.active = 0; active[f] = 0;
    }
  }
}

// After the rounds: each corner judged by the anchors' own map (Ha, mf), the joint model of the anchors and the kept
// corners about the corners' H (acquire.c:2144-2173); the corners to search again. A block of kFitThreads a frame.
__global__ void __launch_bounds__(kFitThreads) reg_corners_kernel(RegArgs a) {
  const int f = blockIdx.x, tid = threadIdx.x;
  RegState &S = a.st[f];
  __shared__ double s_rx[kMaxPts][kLP], s_ry[kMaxPts][kLP], s_d[kMaxPts][2], s_qx[kMaxPts], s_qy[kMaxPts], s_A[kLP][kLP + 1];
  __shared__ double s_res[kMaxPts], s_srt[kMaxPts], s_lens[kLensStride];
  __shared__ FitScratch F;
  __shared__ uint8_t s_drop[kMaxPts];
  __shared__ int s_pos[kNA], s_np, s_flag[2], s_go;
  if (tid == 0) {
    s_go = S.have && S.nf >= kAnchMin;
    S.held = s_go;
    int np = 4;
    for (int k = 0; k < kNA; k++) s_pos[k] = a.ok[(int64_t)f * kNA + k] ? np++ : -1;
    s_np = np;
  }
  __syncthreads();
  if (!s_go) {
    if (tid == 0) { a.on_mc[f] = 0; for (int c = 0; c < 4; c++) S.redo[c] = 0; }
    return;
  }
  const float ah = a.a * 0.5f, lo = a.node_lo, hi = a.node_hi;
  for (int t = tid; t < 4 + kNA; t += blockDim.x) {
    if (t < 4) {   // the corner nodes about H (no displacement), and each judged by the anchors' own map
      float u, v, pu, pv, mu, mv;
      project_f(S.H0, (t == 1 || t == 2) ? hi : lo, t >= 2 ? hi : lo, &u, &v);
      S.hu[t] = u; S.hv[t] = v;
      s_qx[t] = (u - a.ax) / a.R; s_qy[t] = (v - a.ay) / a.R;
      rows_of(s_qx[t], s_qy[t], s_rx[t], s_ry[t]);
      s_d[t][0] = 0; s_d[t][1] = 0;
      project_f(S.Ha, (t == 1 || t == 2) ? hi : lo, t >= 2 ? hi : lo, &pu, &pv);
      lens_at(a.mf + (int64_t)f * kLensStride, pu, pv, &mu, &mv);
      s_drop[t] = hypotf(pu + mu - S.quad[2 * t], pv + mv - S.quad[2 * t + 1]) > kCornerMod * S.mpx;
    } else {
      const int k = t - 4, i = s_pos[k];
      if (i < 0) continue;
      const int64_t o = (int64_t)f * kNA + k;
      float hu, hv;
      project_f(S.H0, (float)a.m0[k % 7] + ah, (float)a.m0[k / 7] + ah, &hu, &hv);
      s_qx[i] = (hu - a.ax) / a.R; s_qy[i] = (hv - a.ay) / a.R;
      rows_of(s_qx[i], s_qy[i], s_rx[i], s_ry[i]);
      s_d[i][0] = a.u[o] - hu; s_d[i][1] = a.v[o] - hv; s_drop[i] = 0;
    }
  }
  __syncthreads();
  const int fit = block_lensm_fit(s_np, s_rx, s_ry, s_d, s_qx, s_qy, s_drop, false, 0, a.ax, a.ay, a.R, s_lens, s_A, F, s_res, s_srt, s_flag);
  if (tid == 0) {
    S.mc_on = fit;
    a.on_mc[f] = fit;
    for (int c = 0; c < kLensStride; c++) a.mc[(int64_t)f * kLensStride + c] = s_lens[c];
    for (int c = 0; c < 4; c++) S.redo[c] = fit && s_drop[c];
  }
}

// The redo flags where the border node search reads them.
__global__ void reg_redo_kernel(const RegState *st, int frames, uint8_t *redo) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < 4 * frames) redo[t] = st[t / 4].redo[t % 4];
}

// The corners searched again replace the measured ones (score 0.35 or more: the search's place, else the joint
// model's), H made again from the four (acquire.c:2174-2195, homography 611-654), the anchors' displacements about H.
// A thread a frame.
__global__ void reg_finish_kernel(RegArgs a, int frames, float *quad_out) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= frames) return;
  RegState &S = a.st[f];
  float *h = a.reg + (int64_t)f * a.hstride;
  if (S.held) {
    const int nn = a.nn;
    int moved = 0;
    for (int c = 0; c < 4; c++) {
      if (!S.redo[c]) continue;
      const int i = (c == 1 || c == 2) ? nn - 1 : 0, j = c >= 2 ? nn - 1 : 0;
      const float *nd = a.nodes + ((int64_t)f * nn * nn + j * nn + i) * 4;
      float mu, mv;
      lens_at(a.mc + (int64_t)f * kLensStride, S.hu[c], S.hv[c], &mu, &mv);
      if (nd[2] >= 0.35f) { S.quad[2 * c] = S.hu[c] + nd[0]; S.quad[2 * c + 1] = S.hv[c] + nd[1]; }
      else { S.quad[2 * c] = S.hu[c] + mu; S.quad[2 * c + 1] = S.hv[c] + mv; }
      moved++;
    }
    S.moved = moved;
    if (moved) {
      const float lo = a.node_lo, hi = a.node_hi, src[8] = {lo, lo, hi, lo, hi, hi, lo, hi};
      double M[8][9];
      for (int i = 0; i < 4; i++) {
        const double x = src[2 * i], y = src[2 * i + 1], u = S.quad[2 * i], v = S.quad[2 * i + 1];
        const double r0[9] = {x, y, 1, 0, 0, 0, -u * x, -u * y, u}, r1[9] = {0, 0, 0, x, y, 1, -v * x, -v * y, v};
        for (int k = 0; k < 9; k++) { M[2 * i][k] = r0[k]; M[2 * i + 1][k] = r1[k]; }
      }
      bool solved = true;
      for (int c = 0; c < 8 && solved; c++) {
        int p = c;
        for (int r = c + 1; r < 8; r++) if (fabs(M[r][c]) > fabs(M[p][c])) p = r;
        if (fabs(M[p][c]) < 1e-12) { solved = false; break; }
        for (int k = 0; k < 9; k++) { const double t = M[c][k]; M[c][k] = M[p][k]; M[p][k] = t; }
        for (int r = 0; r < 8; r++) {
          if (r == c) continue;
          const double fr = M[r][c] / M[c][c];
          for (int k = c; k < 9; k++) M[r][k] -= fr * M[c][k];
        }
      }
      if (solved) {
        for (int k = 0; k < 8; k++) h[k] = (float)(M[k][8] / M[k][k]);
        h[8] = 1;
      }
    }
    const float ah = a.a * 0.5f;
    for (int k = 0; k < kNA; k++) {
      const int64_t o = (int64_t)f * kNA + k;
      if (!a.ok[o]) continue;
      float hu, hv;
      project_f(h, (float)a.m0[k % 7] + ah, (float)a.m0[k / 7] + ah, &hu, &hv);
      a.dx[o] = a.u[o] - hu; a.dy[o] = a.v[o] - hv;
    }
  }
  if (quad_out) for (int k = 0; k < 8; k++) quad_out[(int64_t)f * 8 + k] = S.quad[k];
}

__global__ void reg_held_kernel(const RegState *st, int frames, int *held) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f < frames) held[f] = st[f].held;
}

}  // namespace lizg

struct lizg_refiner {
  int span = 0, max_frames = 0, nn = 0;
  float *node = nullptr;
  uint8_t *ok = nullptr;
  float *peak = nullptr, *dx = nullptr, *dy = nullptr, *u = nullptr, *v = nullptr;
  double *lens = nullptr;
  int *have = nullptr;
  // the anchors' registration (lizg_anchor_register_dev): per frame its state, the anchors' own model and the joint
  // one with their flags, the frames still searching, the corners to search again and the corner search's nodes
  lizg::RegState *st = nullptr;
  double *mf = nullptr, *mc = nullptr;
  int *have_mf = nullptr, *on_mc = nullptr, *held = nullptr;
  uint8_t *active = nullptr, *redo = nullptr;
  float *nodes = nullptr;
};

extern "C" {

void lizg_refiner_free(lizg_refiner *r) {
  if (!r) return;
  void *ps[] = {r->node, r->ok, r->peak, r->dx, r->dy, r->u, r->v, r->lens, r->have, r->st, r->mf, r->mc, r->have_mf, r->on_mc,
                r->held, r->active, r->redo, r->nodes};
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
  al((void **)&r->st, sizeof(lizg::RegState) * F);
  al((void **)&r->mf, sizeof(double) * F * lizg::kLStride); al((void **)&r->mc, sizeof(double) * F * lizg::kLStride);
  al((void **)&r->have_mf, sizeof(int) * F); al((void **)&r->on_mc, sizeof(int) * F); al((void **)&r->held, sizeof(int) * F);
  al((void **)&r->active, F); al((void **)&r->redo, 4 * F);
  al((void **)&r->nodes, sizeof(float) * 4 * F * r->nn * r->nn);
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
    lens_fit_kernel<<<frames, kFitThreads, 0, st>>>(fa);
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

int lizg_anchor_register_dev(lizg_refiner *r, const uint8_t *d_luma, const uint8_t *d_rim, int w, int h, int64_t frame_stride, float *d_reg,
                             float *d_quad, int frames, int32_t *d_held, double *d_lens, const lizg_anchor_out *anchors, void *stream) {
  using namespace lizg;
  if (!r || !d_luma || !d_reg) return record_error(LIZG_E_ARG, "lizg_anchor_register_dev: NULL argument");
  if (frames < 1 || frames > r->max_frames || w < 2 || h < 2 || frame_stride < (int64_t)w * h)
    return record_error(LIZG_E_ARG, "lizg_anchor_register_dev: frames or frame geometry out of range");
  if (anchors && (!anchors->ok || !anchors->peak || !anchors->dx || !anchors->dy || !anchors->u || !anchors->v))
    return record_error(LIZG_E_ARG, "lizg_anchor_register_dev: anchors without all six outputs");
  int sms = 0;
  if (int rc = device_ready(&sms)) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int hstride = 9 + 2 * r->nn * r->nn;
  RegArgs a{};
  a.span = r->span; a.iw = w; a.ih = h; a.hstride = hstride; a.nn = r->nn; a.a = r->span / 64;
  // the axis and scale as lensm_axis takes them (liblizard/src/acquire.c:1622-1628), no axis set
  a.ax = (double)(w * 0.5f); a.ay = (double)(h * 0.5f); a.R = 0;
  for (int c = 0; c < 4; c++) { const double d = std::hypot((c & 1 ? w : 0) - a.ax, (c & 2 ? h : 0) - a.ay); if (d > a.R) a.R = d; }
  if (!(a.R > 0)) a.R = 1;
  {
    float nodes[40];
    layout_nodes(r->span + 2 * kMargin15, nodes);
    a.node_lo = nodes[0]; a.node_hi = nodes[r->nn - 1];
  }
  for (int i = 0; i < 7; i++) a.m0[i] = (int)floor(kMargin15 + (double)r->span * (i + 0.5) / 7 - a.a / 2.0 + 0.5);
  a.reg = d_reg; a.quad_in = d_quad; a.st = r->st; a.ok = r->ok; a.dx = r->dx; a.dy = r->dy; a.u = r->u; a.v = r->v;
  a.mf = r->mf; a.mc = r->mc; a.have_mf = r->have_mf; a.on_mc = r->on_mc; a.nodes = r->nodes;
  const lizg_anchor_out out{r->ok, r->peak, r->dx, r->dy, r->u, r->v};
  // the search's homography is each frame's Ha, inside its state
  const float *d_Ha = reinterpret_cast<const float *>(reinterpret_cast<const char *>(r->st) + offsetof(RegState, Ha));
  static_assert(sizeof(RegState) % sizeof(float) == 0, "the states' stride in floats");
  const int st_stride = (int)(sizeof(RegState) / sizeof(float));
  cudaError_t e = cudaMemsetAsync(r->active, 1, frames, st);
  if (e == cudaSuccess) { reg_init_kernel<<<(frames + 127) / 128, 128, 0, st>>>(a, frames); e = cudaGetLastError(); }
  for (int round = 0; round < kRounds && e == cudaSuccess; round++) {
    if ((e = anchor_find_launch(r->span, d_luma, w, h, frame_stride, d_Ha, st_stride, r->mf, r->ok, frames, out, st, r->have_mf, r->active)) != cudaSuccess) break;
    reg_round_kernel<<<frames, kFitThreads, 0, st>>>(a, r->active);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) { reg_corners_kernel<<<frames, kFitThreads, 0, st>>>(a); e = cudaGetLastError(); }
  if (e == cudaSuccess) { reg_redo_kernel<<<(4 * frames + 255) / 256, 256, 0, st>>>(r->st, frames, r->redo); e = cudaGetLastError(); }
  if (e == cudaSuccess) {
    const float *d_H0 = reinterpret_cast<const float *>(reinterpret_cast<const char *>(r->st) + offsetof(RegState, H0));
    e = border_corners_launch(r->span, d_rim ? d_rim : d_luma, w, h, frame_stride, d_H0, st_stride, r->mc, r->on_mc, r->redo, frames, r->nodes, st);
  }
  if (e == cudaSuccess) { reg_finish_kernel<<<(frames + 127) / 128, 128, 0, st>>>(a, frames, d_quad); e = cudaGetLastError(); }
  if (e == cudaSuccess) { reg_held_kernel<<<(frames + 127) / 128, 128, 0, st>>>(r->st, frames, r->held); e = cudaGetLastError(); }
  if (e == cudaSuccess) {
    // the anchors' model about H (anchor_model) where the registration held, then the mesh
    FitArgs fa{};
    fa.span = r->span; fa.iw = w; fa.ih = h; fa.hstride = hstride; fa.nn = r->nn; fa.a = r->span / 64;
    fa.ax = a.ax; fa.ay = a.ay; fa.R = a.R; fa.node_lo = a.node_lo; fa.node_hi = a.node_hi;
    for (int i = 0; i < 7; i++) fa.m0[i] = a.m0[i];
    fa.reg = d_reg; fa.ok = r->ok; fa.dx = r->dx; fa.dy = r->dy; fa.lens = r->lens; fa.have = r->have; fa.gate = r->held;
    lens_fit_kernel<<<frames, kFitThreads, 0, st>>>(fa);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) { mesh_kernel<<<frames, 256, 0, st>>>(r->lens, r->have, r->node, r->nn, d_reg, hstride); e = cudaGetLastError(); }
  if (e == cudaSuccess && d_held) e = cudaMemcpyAsync(d_held, r->held, sizeof(int) * frames, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && d_lens) e = cudaMemcpyAsync(d_lens, r->lens, sizeof(double) * frames * kLStride, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && anchors) {
    const size_t n = (size_t)frames * kNA;
    if ((e = cudaMemcpyAsync(anchors->ok, r->ok, n, cudaMemcpyDeviceToDevice, st)) == cudaSuccess &&
        (e = cudaMemcpyAsync(anchors->peak, r->peak, 4 * n, cudaMemcpyDeviceToDevice, st)) == cudaSuccess &&
        (e = cudaMemcpyAsync(anchors->dx, r->dx, 4 * n, cudaMemcpyDeviceToDevice, st)) == cudaSuccess &&
        (e = cudaMemcpyAsync(anchors->dy, r->dy, 4 * n, cudaMemcpyDeviceToDevice, st)) == cudaSuccess &&
        (e = cudaMemcpyAsync(anchors->u, r->u, 4 * n, cudaMemcpyDeviceToDevice, st)) == cudaSuccess)
      e = cudaMemcpyAsync(anchors->v, r->v, 4 * n, cudaMemcpyDeviceToDevice, st);
  }
  if (e != cudaSuccess) return record_error(LIZG_E_CUDA, (std::string("lizg_anchor_register_dev: ") + cudaGetErrorString(e)).c_str());
  return 0;
}

}  // extern "C"

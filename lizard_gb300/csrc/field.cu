// The registration refined by its adjoint on sm_103a (include/lizard_gb300.h lizg_field_*): Gauss-Newton over the
// 8 homography parameters and a 7 x 7 field of anchor displacements, against the known pilots, the timing track and
// the anchors' measured centres. No reference counterpart: a refinement of the held registration before the soft
// stage.
//
// The parameters. H[0..7] (H[8] = 1), and a displacement (x, y, pixels) at each of the 7 x 7 anchors' centres. The
// field reaches the mesh as the reference's interior fill carries its anchors' readings inward
// (liblizard/src/acquire.c:2199-2217 anch_herm4, 2335-2385): knots on each axis at the node lattice's two ends (held
// at zero: the border holds the map there) and at the 7 anchors' centres between; each node's displacement gains
// the 4 x 4 cubic Hermite blend of its knots, on top of the registration's own mesh. The sampler then blends the
// nodes bilinearly, so every sample's position is affine in the field.
//
// The mismatch, three terms:
//  - pilots: every block tail's coefficients measured by the receiver's own front (sampling through the registration
//    by the exact walk, the anchors' erase, the detrend, the 2D transform), each against its known symbol times a
//    real gain a radius band and block parity (the gains fitted afresh at every evaluation);
//  - the timing track: the border's track cells (2 x 2 modules, dark or light by the layout's track bits) sampled at
//    their centres, each against the frame's dark or light level;
//  - the anchors' centres: where the registration maps each anchor's centre against where the anchor search found it.
// Each term is weighted to unit mean square at the starting registration, and the field has a Gaussian prior of
// 0.25 pixels a knot (so its 98 knots do not follow the residuals' noise).
//
// The adjoint (reverse mode). The pilots' residuals r are scattered into a half-plane spectrum and one inverse
// transform (the sender's, enc_fft_launch) gives the mismatch's gradient in every picture sample,
// g(x, y) = 2 Re sum_p r_p e^{+2 pi i (u_p x + v_p y) / n}, less the detrend's share (the surface's projections, taken
// exactly; the anchors' erased squares are held constant). One pass over the samples recomputes the warp (H, the mesh
// with the field in it) and the bilinear read's gradient at every sample, and sums g times each parameter's tangent:
// the mismatch's full gradient J^T r in the 106 parameters. Gauss-Newton needs J^T J as well, which the adjoint
// does not give; this one uses, for the pilots, the tangent pictures' own Gram matrix (over H, exact) and their
// energies (over the field, the diagonal) scaled by the share of the picture's energy the pilots carry (Parseval: a
// tangent picture's spectrum takes the picture's shape), plus the track's and the anchors' exact J^T J. Each step is
// solved in double (the columns scaled, a Levenberg damping), kept where the weighted mismatch falls, halved from the
// best registration otherwise. The registration the caller gave is the baseline and the fallback.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>
#include "format.h"
#include "lizard_gb300.h"
#include "lizg_internal.h"
#include "sample_dev.cuh"

namespace lizg {

constexpr int kFK = 9;                          // knots an axis: the two ends and the 7 anchors
constexpr int kFP = LIZG_FIELD_PARAMS;          // 8 + 2 x 49
constexpr int kFThreads = 256, kFRows = 8;      // the gradient pass: a warp a picture row, 8 rows a CTA
constexpr int kFBins = 8, kFGroups = 2 * kFBins;
constexpr int kFHs = 8 + 36 + 2;                // a CTA's H sums: g t (8), the tangents' Gram (36), sum z, sum z^2
constexpr int kFFs = 2 * kFK * kFK * 2;         // and the field's: g t and t^2 at each knot, two components
constexpr int kFPart = kFHs + kFFs;
constexpr int kFMaxTrack = 1024;
constexpr double kFieldSigma = 0.25;            // the field's prior, pixels a knot

struct FieldArgs {
  int n, nn, w, h, reg_stride, npilot, need, vrows, ntrack;
  int64_t fstride;
  float g0, step;
  float pos[40];
  float anc[7];                    // the anchors' centres along an axis (module coordinates)
  int elo[7], ehi[7];
  double sx2, sq2;
  const uint8_t *luma;
  const float *cx, *qx;            // the detrend basis, n each
  const float2 *x1, *x2;           // its DFTs
  const float *wk;                 // nn x kFK: node i's Hermite weight on knot a
  const int32_t *pilot;            // pos index of each pilot
  const int16_t *puv;              // its (u, v)
  const float2 *shat;              // its symbol for a count bit of 0
  const uint8_t *group;            // parity * kFBins + radius band
  const float4 *track;             // a track cell's centre (mx, my) and 1 where dark
};

struct FieldState {
  float theta[kFP];                // the evaluation in hand
  float best[kFP];
  float delta[kFP];                // the step from best
  double loss_best, wp, wa, wt;
  float scale;
  int evals, improved;
};

// Per frame and evaluation, from the pilots' pass: the pilots' loss, the detrend's adjoint constants K1..K5, the
// pilots' energy.
struct PilotTerms {
  double loss, k[5], energy;
};

// The warp at module point (mx, my): H, then the mesh's bilinear displacement from the frame's registration reg;
// the node cell (i, j) and the place (uu, vv) in it.
struct WarpAt {
  float u, v, wd, iw, U, V;
  int i, j;
  float uu, vv;
};
__device__ __forceinline__ int cell_of(const float *pos, int nn, float m) {
  int lo = 0, hi = nn - 2;
  while (lo < hi) { const int mid = (lo + hi + 1) >> 1; if (m >= pos[mid]) lo = mid; else hi = mid - 1; }
  return lo;
}
// The warp at (mx, my) in node cell (i, j) at place (uu, vv).
__device__ __forceinline__ WarpAt warp_in(const FieldArgs &a, const float *reg, float mx, float my, int i, int j, float uu, float vv) {
  WarpAt o;
  o.i = i; o.j = j; o.uu = uu; o.vv = vv;
  const float *n00 = reg + 9 + 2 * (o.j * a.nn + o.i), *n10 = n00 + 2, *n01 = n00 + 2 * a.nn, *n11 = n01 + 2;
  const float mdx = (n00[0] * (1 - o.uu) + n10[0] * o.uu) * (1 - o.vv) + (n01[0] * (1 - o.uu) + n11[0] * o.uu) * o.vv;
  const float mdy = (n00[1] * (1 - o.uu) + n10[1] * o.uu) * (1 - o.vv) + (n01[1] * (1 - o.uu) + n11[1] * o.uu) * o.vv;
  const float *h = reg;
  o.wd = h[6] * mx + h[7] * my + 1;
  o.iw = 1.0f / o.wd;
  o.U = (h[0] * mx + h[1] * my + h[2]) * o.iw;
  o.V = (h[3] * mx + h[4] * my + h[5]) * o.iw;
  o.u = o.U + mdx;
  o.v = o.V + mdy;
  return o;
}
// pos, inv: the node positions (a.pos) and each cell's 1 / width, in the caller's CTA's shared memory (lanes search
// them at different places, which a kernel parameter would serve one address at a time).
__device__ __forceinline__ WarpAt warp_at(const FieldArgs &a, const float *pos, const float *inv, const float *reg, float mx, float my) {
  const int i = cell_of(pos, a.nn, mx), j = cell_of(pos, a.nn, my);
  return warp_in(a, reg, mx, my, i, j, (mx - pos[i]) * inv[i], (my - pos[j]) * inv[j]);
}
// The bilinear read at gamma 1 at pixel point (u, v) (sample()'s clamp) and its gradient in u and v (zero along an
// axis the clamp holds: past the frame's edge the read no longer moves with the point).
__device__ __forceinline__ float read_grad(const uint8_t *px, int w, int h, float u, float v, float *Iu, float *Iv) {
  float sx = u - 0.5f, sy = v - 0.5f;
  const float xm = (float)w - 1.001f, ym = (float)h - 1.001f;
  const bool hx = !(sx >= 0 && sx <= xm), hy = !(sy >= 0 && sy <= ym);
  if (sx < 0) sx = 0; else if (sx > xm) sx = xm;
  if (sy < 0) sy = 0; else if (sy > ym) sy = ym;
  const int xi = sx >= 0 ? (int)sx : 0, yi = sy >= 0 ? (int)sy : 0;
  const float fx = sx - (float)xi, fy = sy - (float)yi;
  const uint8_t *p = px + (int64_t)yi * w + xi;
  const float A = grey_of(p[0]), B = grey_of(p[1]), C = grey_of(p[w]), D = grey_of(p[w + 1]);
  *Iu = hx ? 0.0f : (B - A) * (1 - fy) + (D - C) * fy;
  *Iv = hy ? 0.0f : (C - A) * (1 - fx) + (D - B) * fx;
  return (A + (B - A) * fx) * (1 - fy) + (C + (D - C) * fx) * fy;
}
// The warp's derivative in h0..h7 at (mx, my): du[q], dv[q].
__device__ __forceinline__ void dwarp_dh(const WarpAt &o, float mx, float my, float du[8], float dv[8]) {
  const float iw = o.iw;
  du[0] = mx * iw; du[1] = my * iw; du[2] = iw; du[3] = 0; du[4] = 0; du[5] = 0; du[6] = -o.U * mx * iw; du[7] = -o.U * my * iw;
  dv[0] = 0; dv[1] = 0; dv[2] = 0; dv[3] = mx * iw; dv[4] = my * iw; dv[5] = iw; dv[6] = -o.V * mx * iw; dv[7] = -o.V * my * iw;
}
// A point's weight on knot a along one axis: the bilinear blend of its cell's two nodes' Hermite weights.
// wk: the knot weights (a.wk) in shared memory.
__device__ __forceinline__ float knot_w(const float *wk, int i, float uu, int k) {
  return (1 - uu) * wk[i * kFK + k] + uu * wk[(i + 1) * kFK + k];
}
// The node positions and knot weights a CTA reads at every point, staged in its shared memory.
struct FieldShared {
  float pos[40], inv[40];
  float wk[40 * kFK];
};
__device__ __forceinline__ void stage_shared(const FieldArgs &a, FieldShared &s) {
  for (int t = threadIdx.x; t < a.nn; t += blockDim.x) {
    s.pos[t] = a.pos[t];
    s.inv[t] = t + 1 < a.nn ? 1.0f / (a.pos[t + 1] - a.pos[t]) : 0.0f;
  }
  for (int t = threadIdx.x; t < a.nn * kFK; t += blockDim.x) s.wk[t] = a.wk[t];
  __syncthreads();
}
__device__ __forceinline__ bool in_sq(const FieldArgs &a, int t) {
  bool in = false;
#pragma unroll
  for (int q = 0; q < 7; q++) in |= t >= a.elo[q] && t <= a.ehi[q];
  return in;
}

// The registration the parameters give: H from theta, the base registration's mesh plus the field's Hermite blend
// at every node. A CTA a frame.
__global__ void __launch_bounds__(256) field_mesh_kernel(FieldArgs a, const FieldState *st, int use_best, const float *base, float *out) {
  const int f = blockIdx.x;
  const float *th = use_best ? st[f].best : st[f].theta;
  const float *b = base + (int64_t)f * a.reg_stride;
  float *o = out + (int64_t)f * a.reg_stride;
  if (threadIdx.x < 9) o[threadIdx.x] = threadIdx.x < 8 ? th[threadIdx.x] : 1.0f;
  for (int t = threadIdx.x; t < a.nn * a.nn; t += blockDim.x) {
    const int j = t / a.nn, i = t - j * a.nn;
    float dx = b[9 + 2 * t], dy = b[10 + 2 * t];
    for (int kb = 1; kb < kFK - 1; kb++) {
      const float wy = a.wk[j * kFK + kb];
      if (wy == 0) continue;
      for (int ka = 1; ka < kFK - 1; ka++) {
        const float ww = wy * a.wk[i * kFK + ka];
        const int q = 8 + 2 * ((kb - 1) * 7 + (ka - 1));
        dx += ww * th[q];
        dy += ww * th[q + 1];
      }
    }
    o[9 + 2 * t] = dx;
    o[10 + 2 * t] = dy;
  }
}

// Sums a double over the CTA in a fixed order (a warp's tree, then the warps in turn).
__device__ double fblock_sum(double v, double *red) {
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

// The pilots: the gains, the residuals (into the half-plane spectrum R, pilots only, R zero elsewhere), the loss, the
// detrend's adjoint constants and the pilots' energy. A CTA a frame.
__global__ void __launch_bounds__(kFThreads) field_pilot_kernel(FieldArgs a, const float2 *coef, const uint8_t *skip, float2 *R, PilotTerms *pt) {
  __shared__ double red[kFThreads / 32], gain[kFGroups];
  __shared__ float s_acc[kFGroups * 2][kFThreads];   // each thread's own column: its pilots' sums by group
  const int f = blockIdx.x, tid = threadIdx.x, n = a.n;
  if (skip && skip[f]) return;
  const float2 *C = coef + (int64_t)f * a.need;
  // the gains: each group's sum s.c over s.s, a thread's pilots summed in float in its own slots, then the slots in
  // thread order in double (FP64 is a narrow pipe on this part: the per-pilot work stays in float)
  for (int q = 0; q < 2 * kFGroups; q++) s_acc[q][tid] = 0.0f;
  for (int k = tid; k < a.npilot; k += blockDim.x) {
    const float2 s = a.shat[k], c = C[a.pilot[k]];
    const int g = a.group[k];
    s_acc[2 * g][tid] += s.x * c.x + s.y * c.y;
    s_acc[2 * g + 1][tid] += s.x * s.x + s.y * s.y;
  }
  __syncthreads();
  if (tid < kFGroups) {
    double num = 0, den = 0;
    for (int t = 0; t < (int)blockDim.x; t++) { num += s_acc[2 * tid][t]; den += s_acc[2 * tid + 1][t]; }
    gain[tid] = den > 0 ? num / den : 0.0;
  }
  __syncthreads();
  float loss = 0, en = 0, k1 = 0, k2 = 0, k3 = 0, k4 = 0, k5 = 0;
  float2 *Rf = R + (int64_t)f * a.vrows * n;
  for (int k = tid; k < a.npilot; k += blockDim.x) {
    const float2 s = a.shat[k], c = C[a.pilot[k]];
    const float gk = (float)gain[a.group[k]];
    const float rx = c.x - gk * s.x, ry = c.y - gk * s.y;
    loss += rx * rx + ry * ry;
    en += c.x * c.x + c.y * c.y;
    const int u = a.puv[2 * k], v = a.puv[2 * k + 1], um = (u + n) % n;
    Rf[(int64_t)v * n + um] = make_float2(rx, ry);
    // Re(conj(r) z) = rx zx + ry zy
    const float2 xu = a.x1[um], xv = a.x1[v];
    const float pr = xu.x * xv.x - xu.y * xv.y, pi = xu.x * xv.y + xu.y * xv.x;
    k1 += rx * pr + ry * pi;
    if (v == 0) { const float2 yu = a.x2[um]; k2 += rx * xu.x + ry * xu.y; k3 += rx * yu.x + ry * yu.y; }
    if (u == 0) { const float2 yv = a.x2[v]; k4 += rx * xv.x + ry * xv.y; k5 += rx * yv.x + ry * yv.y; }
  }
  const double lossd = fblock_sum(loss, red), end = fblock_sum(en, red);
  const double k1d = fblock_sum(k1, red), k2d = fblock_sum(k2, red), k3d = fblock_sum(k3, red), k4d = fblock_sum(k4, red), k5d = fblock_sum(k5, red);
  if (tid == 0) {
    PilotTerms &p = pt[f];
    p.loss = lossd; p.energy = end;
    p.k[0] = 2 * k1d / (a.sx2 * a.sx2); p.k[1] = 2 * k2d / a.sx2; p.k[2] = 2 * k3d / a.sq2; p.k[3] = 2 * k4d / a.sx2; p.k[4] = 2 * k5d / a.sq2;
  }
}

// The adjoint pass over the samples. A CTA takes kFRows picture rows of a frame, a warp a row, each lane a run of n / 32
// consecutive columns. G: the mismatch's gradient at every sample (the residuals' inverse transform); g = G - 0.5 - the
// detrend's adjoint terms; t = the image gradient times the warp's derivative. Out: per CTA, in part[f][blk], the H
// sums g t (8), the tangents' Gram (36, upper triangle row by row), sum z and sum z^2 of the samples read, then for
// each knot pair (b, a) and component the field's g t (kFK^2 x 2) and t^2 (kFK^2 x 2).
// The row's my is fixed, so every H tangent is one of a = Iu / w, b = Iv / w, c = -(Iu U + Iv V) / w times 1, mx or
// my: the lane sums g a, g b, g c and g times each against mx, and each product of two of a, b, c against 1, mx and
// mx^2 (24 sums), and the 44 H sums are made from them at the row's end. A sample's weight on knot k along x is the
// blend (1 - uu) W_i[k] + uu W_{i+1}[k] of its cell's two nodes, so the lane sums g Iu, g Iv and the squares' terms
// against (1 - uu), uu and their products over the samples of one cell (10 sums), and adds them into its knot sums (in
// shared memory, a slot a lane) each time its run leaves a cell.
constexpr int kCellSums = 10;
__global__ void __launch_bounds__(kFThreads, 2) field_grad_kernel(FieldArgs a, const float *regs, const float *G, const PilotTerms *pt,
                                                               const uint8_t *skip, float *part) {
  const int blocks = a.n / kFRows, f = blockIdx.x / blocks, blk = blockIdx.x - f * blocks;
  if (skip && skip[f]) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, y = blk * kFRows + warp, n = a.n;
  const float *reg = regs + (int64_t)f * a.reg_stride;
  const uint8_t *px = a.luma + f * a.fstride;
  const float *Gf = G + (int64_t)f * n * n + (int64_t)y * n;
  __shared__ FieldShared fs;
  stage_shared(a, fs);
  __shared__ float s_kn[kFRows][kFK * 4][32];   // each lane's knot sums: g tx, g ty, tx^2, ty^2 at each knot a
  __shared__ float s_pq[kFRows][kFK][4];        // a row's field sums over its lanes
  __shared__ float s_wy[kFRows][kFK];
  __shared__ float s_h[kFThreads / 32][kFHs];
  float (*kn)[32] = s_kn[warp];
  for (int e = 0; e < kFK * 4; e++) kn[e][lane] = 0;
  // the detrend's adjoint constants in float: the gradient's share of them needs no more (FP64 is a narrow pipe here)
  const float K0 = (float)pt[f].k[0], K1 = (float)pt[f].k[1], K2 = (float)pt[f].k[2], K3 = (float)pt[f].k[3], K4 = (float)pt[f].k[4];
  const float my = a.g0 + (float)y * a.step;
  const float cy = a.cx[y], qy = a.qx[y];
  const bool ysq = in_sq(a, y);
  // the lane's sums: g a, g a mx, g b, g b mx, g c, g c mx; aa, ab, ac, bb, bc, cc against 1, mx, mx^2; z, z^2
  float ga[6] = {0, 0, 0, 0, 0, 0}, gm[18], zs = 0, zz = 0;
#pragma unroll
  for (int q = 0; q < 18; q++) gm[q] = 0;
  float cs[kCellSums];
#pragma unroll
  for (int q = 0; q < kCellSums; q++) cs[q] = 0;
  const int jrow = cell_of(fs.pos, a.nn, my);
  const float vrow = (my - fs.pos[jrow]) * fs.inv[jrow];
  const int per = n / 32, x0 = lane * per;
  int icell = cell_of(fs.pos, a.nn, a.g0 + (float)x0 * a.step), ccell = icell;
  // the cell sums of cell ic into the lane's knot sums
  auto flush = [&](int ic) {
#pragma unroll
    for (int k = 0; k < kFK; k++) {
      const float w0 = fs.wk[ic * kFK + k], w1 = fs.wk[(ic + 1) * kFK + k];
      if (w0 == 0.0f && w1 == 0.0f) continue;
      kn[4 * k + 0][lane] += w0 * cs[0] + w1 * cs[1];
      kn[4 * k + 1][lane] += w0 * cs[2] + w1 * cs[3];
      kn[4 * k + 2][lane] += w0 * w0 * cs[4] + 2.0f * w0 * w1 * cs[5] + w1 * w1 * cs[6];
      kn[4 * k + 3][lane] += w0 * w0 * cs[7] + 2.0f * w0 * w1 * cs[8] + w1 * w1 * cs[9];
    }
#pragma unroll
    for (int q = 0; q < kCellSums; q++) cs[q] = 0;
  };
  for (int x = x0; x < x0 + per; x++) {
    const float mx = a.g0 + (float)x * a.step;
    while (icell < a.nn - 2 && mx >= fs.pos[icell + 1]) icell++;
    if (icell != ccell) { flush(ccell); ccell = icell; }
    const float uu = (mx - fs.pos[icell]) * fs.inv[icell];
    const WarpAt o = warp_in(a, reg, mx, my, icell, jrow, uu, vrow);
    float Iu, Iv;
    const float z = read_grad(px, a.w, a.h, o.u, o.v, &Iu, &Iv);
    zs += z; zz += z * z;
    if (ysq && in_sq(a, x)) continue;   // erased: the shading surface, held constant
    const float cxx = a.cx[x], qxx = a.qx[x];
    const float g = Gf[x] - 0.5f - (K0 * cxx * cy + K1 * cxx + K2 * qxx + K3 * cy + K4 * qy);
    const float ta = o.iw * Iu, tb = o.iw * Iv, tc = -o.iw * (Iu * o.U + Iv * o.V), m2 = mx * mx;
    const float gta = g * ta, gtb = g * tb, gtc = g * tc;
    ga[0] += gta; ga[1] += gta * mx; ga[2] += gtb; ga[3] += gtb * mx; ga[4] += gtc; ga[5] += gtc * mx;
    const float pr[6] = {ta * ta, ta * tb, ta * tc, tb * tb, tb * tc, tc * tc};
#pragma unroll
    for (int q = 0; q < 6; q++) { gm[3 * q] += pr[q]; gm[3 * q + 1] += pr[q] * mx; gm[3 * q + 2] += pr[q] * m2; }
    const float v1 = uu, v0 = 1.0f - uu, gu = g * Iu, gv = g * Iv, uu2 = Iu * Iu, vv2 = Iv * Iv;
    cs[0] += gu * v0; cs[1] += gu * v1; cs[2] += gv * v0; cs[3] += gv * v1;
    cs[4] += uu2 * v0 * v0; cs[5] += uu2 * v0 * v1; cs[6] += uu2 * v1 * v1;
    cs[7] += vv2 * v0 * v0; cs[8] += vv2 * v0 * v1; cs[9] += vv2 * v1 * v1;
  }
  flush(ccell);
  // the 44 H sums from the lane's 24: t = (a mx, a my, a, b mx, b my, b, c mx, c my), each a (abc) x (mx, my, 1) term
  float hs[kFHs];
  {
    const int which[8] = {0, 0, 0, 1, 1, 1, 2, 2}, mono[8] = {1, 2, 0, 1, 2, 0, 1, 2};   // mono: 0 = 1, 1 = mx, 2 = my
    const float my2 = my * my;
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const float s0 = ga[2 * which[q]], s1 = ga[2 * which[q] + 1];
      hs[q] = mono[q] == 1 ? s1 : mono[q] == 2 ? my * s0 : s0;
    }
    int e = 8;
#pragma unroll
    for (int p = 0; p < 8; p++)
#pragma unroll
      for (int q = p; q < 8; q++) {
        const int u = min(which[p], which[q]), v = max(which[p], which[q]);
        const int pi = u == 0 ? v : u == 1 ? 2 + v : 5;   // the pair's index in aa, ab, ac, bb, bc, cc
        const int nx = (mono[p] == 1) + (mono[q] == 1), ny = (mono[p] == 2) + (mono[q] == 2);
        const float fy = ny == 0 ? 1.0f : ny == 1 ? my : my2;
        hs[e++] = fy * gm[3 * pi + nx];
      }
    hs[44] = zs; hs[45] = zz;
  }
  // the row's field sums over the warp's lanes, then weighted by the row's knot weights across the CTA's rows in order
  __syncwarp();
  for (int e = lane; e < kFK * 4; e += 32) {
    float v = 0;
    for (int l = 0; l < 32; l++) v += kn[e][l];
    s_pq[warp][e >> 2][e & 3] = v;
  }
  if (lane < kFK) s_wy[warp][lane] = knot_w(fs.wk, jrow, vrow, lane);
#pragma unroll
  for (int q = 0; q < kFHs; q++) {
    float v = hs[q];
#pragma unroll
    for (int s2 = 16; s2 > 0; s2 >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s2);
    if (lane == 0) s_h[warp][q] = v;
  }
  __syncthreads();
  float *out = part + ((int64_t)f * blocks + blk) * kFPart;
  for (int q = threadIdx.x; q < kFHs; q += blockDim.x) {
    float acc = 0;
    for (int r = 0; r < kFRows; r++) acc += s_h[r][q];
    out[q] = acc;
  }
  for (int e = threadIdx.x; e < kFK * kFK * 2; e += blockDim.x) {   // (b, a, c): g t and t^2
    const int c = e & 1, ka = (e >> 1) % kFK, kb = (e >> 1) / kFK;
    float gt = 0, tt = 0;
    for (int r = 0; r < kFRows; r++) {
      const float wy = s_wy[r][kb];
      gt += wy * s_pq[r][ka][c];
      tt += wy * wy * s_pq[r][ka][2 + c];
    }
    out[kFHs + e] = gt;
    out[kFHs + kFK * kFK * 2 + e] = tt;
  }
}

// A point's Jacobian row in one image axis (0: u, 1: v) for module point (mx, my), written into a dense row of kFPad
// floats the caller zeroed: H's 8 (du or dv), then the field's knots around it (that axis's component); with axis < 0,
// a sample's row: the image gradient (scale_u, scale_v) times the warp's derivative, both components of each knot.
constexpr int kFPad = (kFP + 3) / 4 * 4;   // a staged row's stride, floats: whole 16-byte groups
__device__ __forceinline__ void point_row(const FieldShared &fs, const WarpAt &o, float mx, float my, int axis, float scale_u,
                                          float scale_v, float *row) {
  float du[8], dv[8];
  dwarp_dh(o, mx, my, du, dv);
  for (int q = 0; q < 8; q++) row[q] = scale_u * du[q] + scale_v * dv[q];
  for (int kb = 1; kb < kFK - 1; kb++) {
    const float wy = knot_w(fs.wk, o.j, o.vv, kb);
    if (wy == 0) continue;
    for (int ka = 1; ka < kFK - 1; ka++) {
      const float ww = wy * knot_w(fs.wk, o.i, o.uu, ka);
      if (ww == 0) continue;
      const int q = 8 + 2 * ((kb - 1) * 7 + (ka - 1));
      if (axis < 0) {
        row[q] = scale_u * ww;
        row[q + 1] = scale_v * ww;
      } else {
        row[q + axis] = ww;
      }
    }
  }
}

// The normal equations of the three terms at the evaluation in hand, the loss, and the step (kept or halved). A CTA a
// frame; A (kFP x kFP doubles) in dynamic shared memory, then the staged rows. The track's and the anchors' residual
// rows are staged kRowBatch at a time as dense rows (a thread a row); each thread then sums a 4 x 4 tile of the upper
// triangle of J^T W J over the batch in float and adds it into A (double), and the terms' J^T r a parameter a thread,
// so every sum runs in a fixed order. With terms set (the checks' call), the three terms' raw losses and gradients
// are written there instead (frames x 3 x (1 + kFP)) and no step is taken.
constexpr int kRowBatch = 128;
constexpr int kFTiles = kFPad / 4, kFTileCount = kFTiles * (kFTiles + 1) / 2;
constexpr size_t kSolveSmem = sizeof(double) * kFP * kFP + sizeof(float) * kRowBatch * kFPad;
static_assert((sizeof(double) * kFP * kFP) % 16 == 0, "the staged rows start on a 16-byte boundary");
__global__ void __launch_bounds__(256, 1) field_solve_kernel(FieldArgs a, const float *regs, const float *part, const PilotTerms *pt,
                                                          const float *anc_u, const float *anc_v, const uint8_t *anc_ok,
                                                          const uint8_t *skip, FieldState *st, int last, double *terms) {
  extern __shared__ __align__(16) double smA[];
  float *Jd = reinterpret_cast<float *>(smA + kFP * kFP);   // kRowBatch x kFPad
  __shared__ double bv[3][kFP], red[8], s_sum[kFPart], s_lvl[2], s_loss[3], s_cnt[3];
  __shared__ double x[kFP], sc[kFP], isc[kFP], s_inv[kFP];
  __shared__ float r_w[kRowBatch], r_r[kRowBatch];
  __shared__ int r_term[kRowBatch];
  __shared__ FieldShared fs;
  const int f = blockIdx.x, tid = threadIdx.x, blocks = a.n / kFRows;
  if (skip && skip[f]) return;
  stage_shared(a, fs);
  const float *reg = regs + (int64_t)f * a.reg_stride;
  const uint8_t *px = a.luma + f * a.fstride;
  FieldState &S = st[f];
  // the last evaluation of a refinement only weighs its point against the best so far: no gradient, no system
  const bool only_loss = last && !terms;
  // the adjoint pass's partial sums, in block order within each of 8 interleaved sums (8 loads in flight a thread),
  // the 8 then added pairwise (blocks is a multiple of 8 for every picture size; any rest is summed after)
  for (int q = tid; q < (only_loss ? 0 : kFPart); q += blockDim.x) {
    const float *p = part + (int64_t)f * blocks * kFPart + q;
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int b = 0;
    for (; b + 8 <= blocks; b += 8) {
#pragma unroll
      for (int u = 0; u < 8; u++) acc[u] += p[(int64_t)(b + u) * kFPart];
    }
    double tail = 0;
    for (; b < blocks; b++) tail += p[(int64_t)b * kFPart];
    s_sum[q] = ((acc[0] + acc[1]) + (acc[2] + acc[3])) + ((acc[4] + acc[5]) + (acc[6] + acc[7])) + tail;
  }
  for (int q = tid; q < (only_loss ? 0 : 3 * kFP); q += blockDim.x) bv[q / kFP][q % kFP] = 0;
  for (int q = tid; q < (only_loss ? 0 : kFP * kFP); q += blockDim.x) smA[q] = 0;
  __syncthreads();
  // the track's levels: the dark cells' and the light cells' mean sample
  double ld = 0, ll = 0, nd = 0, nl = 0;
  for (int t = tid; t < a.ntrack; t += blockDim.x) {
    const float4 c = a.track[t];
    const WarpAt o = warp_at(a, fs.pos, fs.inv, reg, c.x, c.y);
    float Iu, Iv;
    const float z = read_grad(px, a.w, a.h, o.u, o.v, &Iu, &Iv);
    if (c.z > 0) { ld += z; nd += 1; } else { ll += z; nl += 1; }
  }
  ld = fblock_sum(ld, red); ll = fblock_sum(ll, red); nd = fblock_sum(nd, red); nl = fblock_sum(nl, red);
  if (tid == 0) { s_lvl[0] = nd > 0 ? ld / nd : 0; s_lvl[1] = nl > 0 ? ll / nl : 0; }
  __syncthreads();
  // the track's and the anchors' losses
  double lt = 0, la = 0, na = 0;
  for (int t = tid; t < a.ntrack; t += blockDim.x) {
    const float4 c = a.track[t];
    const WarpAt o = warp_at(a, fs.pos, fs.inv, reg, c.x, c.y);
    float Iu, Iv;
    const float z = read_grad(px, a.w, a.h, o.u, o.v, &Iu, &Iv);
    const double r = z - (c.z > 0 ? s_lvl[0] : s_lvl[1]);
    lt += r * r;
  }
  if (anc_ok)
    for (int k = tid; k < 49; k += blockDim.x) {
      if (!anc_ok[f * 49 + k]) continue;
      const WarpAt o = warp_at(a, fs.pos, fs.inv, reg, a.anc[k % 7], a.anc[k / 7]);
      const double ru = o.u - anc_u[f * 49 + k], rv = o.v - anc_v[f * 49 + k];
      la += ru * ru + rv * rv;
      na += 1;
    }
  lt = fblock_sum(lt, red); la = fblock_sum(la, red); na = fblock_sum(na, red);
  if (tid == 0) {
    s_loss[0] = pt[f].loss; s_loss[1] = lt; s_loss[2] = la; s_cnt[0] = a.npilot; s_cnt[1] = a.ntrack; s_cnt[2] = na;
    // the terms' weights, fixed at the first evaluation: each term's residuals at unit mean square there (an anchor's
    // reading under blur is far noisier than its 0.15 px on a sharp capture, so its spread is measured, not assumed)
    if (!terms && S.evals == 0) {
      S.wp = s_loss[0] > 0 ? s_cnt[0] / s_loss[0] : 0;
      S.wt = s_loss[1] > 0 ? s_cnt[1] / s_loss[1] : 0;
      S.wa = s_loss[2] > 0 ? 2 * s_cnt[2] / s_loss[2] : 0;
    }
  }
  __syncthreads();
  if (only_loss) {
    // the loss as below, then the better of this point and the best so far kept as the result
    double fprior = 0;
    for (int q = 8 + tid; q < kFP; q += blockDim.x) fprior += (double)S.theta[q] * S.theta[q];
    fprior = fblock_sum(fprior, red) / (kFieldSigma * kFieldSigma);
    if (tid != 0) return;
    const double loss = S.wp * s_loss[0] + S.wt * s_loss[1] + S.wa * s_loss[2] + fprior;
    if (S.evals == 0 || loss < S.loss_best) {
      if (S.evals > 0) S.improved = 1;
      S.loss_best = loss;
      for (int q = 0; q < kFP; q++) S.best[q] = S.theta[q];
    }
    S.evals++;
    for (int q = 0; q < kFP; q++) S.theta[q] = S.best[q];
    return;
  }
  const double wt = terms ? 0.0 : S.wt, wa = terms ? 0.0 : S.wa;
  const bool need_a = wt != 0 || wa != 0;
  // the track's rows (term 1), then the anchors' two rows each (term 2)
  const int rows = a.ntrack + (anc_ok ? 98 : 0);
  for (int base = 0; base < rows; base += kRowBatch) {
    const int nrow = min(kRowBatch, rows - base);
    for (int e = tid; e < kRowBatch * kFPad / 4; e += blockDim.x) reinterpret_cast<float4 *>(Jd)[e] = make_float4(0, 0, 0, 0);
    __syncthreads();
    if (tid < nrow) {
      const int t = base + tid;
      float *row = Jd + tid * kFPad;
      int term = 1;
      float r = 0;
      if (t < a.ntrack) {
        const float4 c = a.track[t];
        const WarpAt o = warp_at(a, fs.pos, fs.inv, reg, c.x, c.y);
        float Iu, Iv;
        const float z = read_grad(px, a.w, a.h, o.u, o.v, &Iu, &Iv);
        r = (float)(z - (c.z > 0 ? s_lvl[0] : s_lvl[1]));
        point_row(fs, o, c.x, c.y, -1, Iu, Iv, row);
      } else {
        const int k = (t - a.ntrack) >> 1, ax = (t - a.ntrack) & 1;
        term = 2;
        if (anc_ok[f * 49 + k]) {
          const float X = a.anc[k % 7], Y = a.anc[k / 7];
          const WarpAt o = warp_at(a, fs.pos, fs.inv, reg, X, Y);
          r = ax == 0 ? o.u - anc_u[f * 49 + k] : o.v - anc_v[f * 49 + k];
          point_row(fs, o, X, Y, ax, ax == 0 ? 1.0f : 0.0f, ax == 1 ? 1.0f : 0.0f, row);
        }
      }
      r_term[tid] = term; r_r[tid] = r; r_w[tid] = (float)(term == 1 ? wt : wa);
    }
    __syncthreads();
    if (need_a)
      for (int t = tid; t < kFTileCount; t += blockDim.x) {
        int ti = 0, rem = t;   // tile row ti holds the tiles tj = ti .. kFTiles - 1
        while (rem >= kFTiles - ti) { rem -= kFTiles - ti; ti++; }
        const int tj = ti + rem;
        float acc[4][4];
#pragma unroll
        for (int p = 0; p < 4; p++)
#pragma unroll
          for (int q = 0; q < 4; q++) acc[p][q] = 0;
        for (int r = 0; r < nrow; r++) {
          const float w = r_w[r];
          const float4 va = *reinterpret_cast<const float4 *>(Jd + r * kFPad + 4 * ti);
          const float4 vb = *reinterpret_cast<const float4 *>(Jd + r * kFPad + 4 * tj);
          const float pa[4] = {w * va.x, w * va.y, w * va.z, w * va.w}, pb[4] = {vb.x, vb.y, vb.z, vb.w};
#pragma unroll
          for (int p = 0; p < 4; p++)
#pragma unroll
            for (int q = 0; q < 4; q++) acc[p][q] += pa[p] * pb[q];
        }
#pragma unroll
        for (int p = 0; p < 4; p++)
#pragma unroll
          for (int q = 0; q < 4; q++) {
            const int i = 4 * ti + p, j = 4 * tj + q;
            if (i < kFP && j < kFP) smA[i * kFP + j] += acc[p][q];
          }
      }
    for (int i = tid; i < kFP; i += blockDim.x) {
      float g1 = 0, g2 = 0;
      for (int r = 0; r < nrow; r++) {
        const float v = Jd[r * kFPad + i] * r_r[r];
        if (r_term[r] == 1) g1 += v; else g2 += v;
      }
      bv[1][i] += g1;
      bv[2][i] += g2;
    }
    __syncthreads();
  }
  // the upper triangle mirrored into the lower
  for (int e = tid; e < kFP * kFP; e += blockDim.x) {
    const int p = e / kFP, q = e - p * kFP;
    if (p > q) smA[e] = smA[q * kFP + p];
  }
  // the pilots' gradient: the adjoint pass's g t is d(loss)/d(theta), twice J^T r
  for (int q = tid; q < kFP; q += blockDim.x) {
    if (q < 8) bv[0][q] = 0.5 * s_sum[q];
    else {
      const int e = (q - 8) >> 1, c = (q - 8) & 1, kb = e / 7 + 1, ka = e % 7 + 1;
      bv[0][q] = 0.5 * s_sum[kFHs + (kb * kFK + ka) * 2 + c];
    }
  }
  __syncthreads();
  if (terms) {   // the checks: raw losses and gradients (2 J^T r) of the three terms
    double *o = terms + (int64_t)f * 3 * (1 + kFP);
    for (int q = tid; q < 3 * (1 + kFP); q += blockDim.x) {
      const int term = q / (1 + kFP), e = q % (1 + kFP);
      o[q] = e == 0 ? s_loss[term] : 2.0 * bv[term][e - 1];
    }
    return;
  }
  const double wp = S.wp;
  // the field's prior: each knot's displacement a zero-mean Gaussian of kFieldSigma pixels (the field carries what
  // the registration's own mesh left, which is small where the anchors and the lens model already fit), so 98 knots
  // cannot follow the residuals' noise
  double fprior = 0;
  for (int q = 8 + tid; q < kFP; q += blockDim.x) fprior += (double)S.theta[q] * S.theta[q];
  fprior = fblock_sum(fprior, red) / (kFieldSigma * kFieldSigma);
  // the pilots' J^T J: the tangents' Gram over H, their energies on the field's diagonal, times the pilots' share of
  // the picture's energy; the prior's diagonal
  const double npx = (double)a.n * a.n, mean = s_sum[44] / npx, ez = s_sum[45] - npx * mean * mean;
  const double rho = ez > 0 ? pt[f].energy / ez : 0;
  for (int e = tid; e < 64; e += blockDim.x) {
    const int p = e >> 3, q = e & 7, lo = min(p, q), hi = max(p, q);
    const int g = 8 + lo * 8 - lo * (lo - 1) / 2 + (hi - lo);   // (lo, hi) in the upper triangle, row by row
    smA[p * kFP + q] += wp * rho * s_sum[g];
  }
  for (int q = 8 + tid; q < kFP; q += blockDim.x) {
    const int e = (q - 8) >> 1, c = (q - 8) & 1, kb = e / 7 + 1, ka = e % 7 + 1;
    smA[q * kFP + q] += wp * rho * s_sum[kFHs + kFK * kFK * 2 + (kb * kFK + ka) * 2 + c] + 1.0 / (kFieldSigma * kFieldSigma);
  }
  __syncthreads();
  const double loss = wp * s_loss[0] + wt * s_loss[1] + wa * s_loss[2] + fprior;
  // the right-hand side, the columns scaled, a Levenberg damping
  for (int q = tid; q < kFP; q += blockDim.x) {
    const double d = smA[q * kFP + q];
    sc[q] = d > 0 ? sqrt(d) : 1.0;
    isc[q] = 1.0 / sc[q];
    x[q] = -(wp * bv[0][q] + wt * bv[1][q] + wa * bv[2][q] + (q >= 8 ? S.theta[q] / (kFieldSigma * kFieldSigma) : 0.0));
  }
  __syncthreads();
  for (int e = tid; e < kFP * kFP; e += blockDim.x) {
    const int p = e / kFP, q = e % kFP;
    smA[e] *= isc[p] * isc[q];
    if (p == q) smA[e] = smA[e] * 1.001 + 1e-9;
  }
  for (int q = tid; q < kFP; q += blockDim.x) x[q] *= isc[q];
  __syncthreads();
  if (tid == 0) s_inv[0] = 1.0 / smA[0];
  __syncthreads();
  // L D L^T (the system is symmetric positive definite: J^T J, the prior and the damping) in the lower triangle, in
  // place, a column a step across the CTA (16 x 16 threads over the trailing rows and columns); a column's entries
  // become L's one step later, once nothing reads them. Every thread reads the same pivot, so all stop together; the
  // thread that finishes the next pivot takes its reciprocal (one double division a column).
  const int tx = tid & 15, ty = tid >> 4;
  bool ok = true;
  for (int c = 0; c < kFP; c++) {
    const double d = smA[c * kFP + c];
    if (!(d > 1e-300)) { ok = false; break; }
    if (c > 0) {
      const double ip = s_inv[c - 1];
      for (int r = c + tid; r < kFP; r += blockDim.x) smA[r * kFP + c - 1] *= ip;
    }
    const double id = s_inv[c];
    for (int r = c + 1 + ty; r < kFP; r += 16) {
      const double lr = smA[r * kFP + c] * id;
      for (int q = c + 1 + tx; q <= r; q += 16) smA[r * kFP + q] -= lr * smA[q * kFP + c];
    }
    if (tid == 0 && c + 1 < kFP) s_inv[c + 1] = 1.0 / smA[(c + 1) * kFP + c + 1];   // this thread's own last update
    __syncthreads();
  }
  // L y = b, D z = y, L^T w = z: one warp, a column a step
  if (ok && tid < 32) {
    for (int c = 0; c < kFP; c++) {
      __syncwarp();
      const double yc = x[c];
      for (int r = c + 1 + tid; r < kFP; r += 32) x[r] -= smA[r * kFP + c] * yc;
    }
    __syncwarp();
    for (int q = tid; q < kFP; q += 32) x[q] *= s_inv[q];
    for (int c = kFP - 1; c >= 0; c--) {
      __syncwarp();
      const double zc = x[c];
      for (int r = tid; r < c; r += 32) x[r] -= smA[c * kFP + r] * zc;
    }
  }
  __syncthreads();
  if (tid != 0) return;
  const bool s_ok = ok;
  float delta[kFP];
  for (int q = 0; q < kFP; q++) delta[q] = s_ok && isfinite(x[q] * isc[q]) ? (float)(x[q] * isc[q]) : 0.0f;
  if (S.evals == 0 || loss < S.loss_best) {
    if (S.evals > 0) S.improved = 1;
    S.loss_best = loss;
    for (int q = 0; q < kFP; q++) { S.best[q] = S.theta[q]; S.delta[q] = delta[q]; }
    S.scale = 1.0f;
  } else {
    S.scale *= 0.5f;
  }
  S.evals++;
  for (int q = 0; q < kFP; q++) S.theta[q] = last ? S.best[q] : S.best[q] + S.scale * S.delta[q];
}

__global__ void field_load_kernel(const float *reg, int reg_stride, const float *theta, int frames, FieldState *st) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= frames) return;
  FieldState &S = st[f];
  for (int q = 0; q < kFP; q++) {
    const float v = theta ? theta[(int64_t)f * kFP + q] : (q < 8 ? reg[(int64_t)f * reg_stride + q] : 0.0f);
    S.theta[q] = S.best[q] = v;
    S.delta[q] = 0;
  }
  S.loss_best = 0; S.wp = S.wa = S.wt = 0; S.scale = 1.0f; S.evals = 0; S.improved = 0;
}

__global__ void field_store_kernel(const FieldState *st, const uint8_t *skip, int frames, float *loss_out, int32_t *improved_out) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= frames) return;
  const bool s = skip && skip[f];
  if (loss_out) loss_out[f] = s ? 0.0f : (float)st[f].loss_best;
  if (improved_out) improved_out[f] = s ? 0 : st[f].improved;
}

// The refined registration written back: the best parameters' H and mesh, frames the gate skips untouched.
__global__ void field_copy_kernel(const float *src, const uint8_t *skip, int frames, int reg_stride, float *dst) {
  const int f = blockIdx.y;
  if (f >= frames || (skip && skip[f])) return;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < reg_stride; t += gridDim.x * blockDim.x) dst[(int64_t)f * reg_stride + t] = src[(int64_t)f * reg_stride + t];
}

}  // namespace lizg

struct lizg_field {
  lizg::Format f;
  lizg::FieldArgs a{};
  lizg_rx *rx = nullptr;
  int chunk = 0;
  lizg::EncFft enc{};
  float *eff = nullptr, *G = nullptr, *part = nullptr, *base = nullptr;
  float2 *coef = nullptr, *R = nullptr;
  lizg::FieldState *state = nullptr;
  lizg::PilotTerms *pt = nullptr;
  uint8_t *skip = nullptr;
  std::vector<void *> owned;
};

namespace {

// A cubic Hermite's weights on its knots at x (the knots' slopes from their neighbours, one-sided at the ends): the
// value is sum w[q] v[b + q], q = 0..3 (liblizard/src/acquire.c:2199-2217, the interior fill's mesh).
void herm4(const double *t, int n, double x, int *b, double w[4]) {
  int i = 0;
  while (i < n - 2 && x >= t[i + 1]) i++;
  const double hc = t[i + 1] - t[i], s = (x - t[i]) / hc, s2 = s * s, s3 = s2 * s;
  const double h00 = 2 * s3 - 3 * s2 + 1, h01 = -2 * s3 + 3 * s2, A = (s3 - 2 * s2 + s) * hc, Bc = (s3 - s2) * hc;
  w[0] = w[3] = 0; w[1] = h00; w[2] = h01;
  if (i > 0) { const double d = t[i + 1] - t[i - 1]; w[0] -= A / d; w[2] += A / d; } else { w[1] -= A / hc; w[2] += A / hc; }
  if (i + 2 < n) { const double d = t[i + 2] - t[i]; w[1] -= Bc / d; w[3] += Bc / d; } else { w[1] -= Bc / hc; w[2] += Bc / hc; }
  *b = i - 1;
}

int track_bit(int side, int j) {   // liblizard/src/layout.c:57-61
  uint32_t v = (uint32_t)(side * 4099 + (j >> 1)) * 2654435761u + 40503u;
  v ^= v >> 15;
  v *= 2246822519u;
  v ^= v >> 13;
  return (int)((v ^ (uint32_t)j) & 1);
}

}  // namespace

extern "C" {

lizg_field *lizg_field_new(int n, int subch, int span, int chunk) {
  using namespace lizg;
  if (chunk < 1 || chunk > 256) { record_error(LIZG_E_ARG, "lizg_field_new: chunk must be 1..256"); return nullptr; }
  int sms = 0;
  if (device_ready(&sms)) return nullptr;
  lizg_field *g = new (std::nothrow) lizg_field();
  if (!g) { record_error(LIZG_E_NOMEM, "lizg_field_new: out of host memory"); return nullptr; }
  if (format_build(n, subch, span, g->f)) { delete g; record_error(LIZG_E_ARG, "lizg_field_new: no such format"); return nullptr; }
  const Format &f = g->f;
  FieldArgs &a = g->a;
  a.n = n; a.need = subch * kSub;
  a.g0 = kMargin + 0.5f / f.scale; a.step = 1.0f / f.scale;
  a.nn = layout_nodes(span + 2 * kMargin, a.pos);
  a.reg_stride = 9 + 2 * a.nn * a.nn;
  a.sx2 = f.sx2; a.sq2 = f.sq2;
  for (int i = 0; i < 7; i++) { a.elo[i] = f.elo[i]; a.ehi[i] = f.ehi[i]; }
  const int aside = span / 64;
  for (int i = 0; i < 7; i++) a.anc[i] = (float)((int)std::floor(kMargin + (double)span * (i + 0.5) / 7 - aside / 2.0 + 0.5) + aside / 2.0);
  // the pilots: their symbols (count bit 0), groups (block parity, radius band by quantile), (u, v)
  std::vector<int32_t> pk;
  std::vector<int16_t> puv;
  std::vector<float2> shat;
  std::vector<int> par;
  std::vector<double> rho;
  const float qa = 0.70710678f;
  int vmax = 0;
  for (size_t k = 0; k < f.uv.size() / 2; k++) vmax = std::max<int>(vmax, f.uv[2 * k + 1]);
  for (int b = 0; b < f.blocks; b++) {
    const Tier &tr = f.tier[f.block_tier[b]];
    const int first = f.block_slot[b] / 2;
    for (int s = tr.nt / 2; s < tr.slots / 2; s++) {
      const int k = first + s;
      pk.push_back(k);
      puv.push_back(f.uv[2 * k]); puv.push_back(f.uv[2 * k + 1]);
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
    for (int q = 1; q < kFBins; q++) if (np && rho[k] > sorted[(size_t)((double)q * (np - 1) / kFBins)]) bin = q;
    grp[k] = (uint8_t)(par[k] * kFBins + bin);
  }
  a.npilot = np;
  a.vrows = vmax + 1;
  // the Hermite weights of every node on the knots (the lattice's ends and the anchors' centres)
  double kn[kFK];
  const double X0 = a.pos[0], SX = a.pos[a.nn - 1] - a.pos[0];
  kn[0] = 0; kn[kFK - 1] = 1;
  for (int i = 0; i < 7; i++) kn[i + 1] = (a.anc[i] - X0) / SX;
  std::vector<float> wk((size_t)a.nn * kFK, 0.0f);
  for (int i = 0; i < a.nn; i++) {
    int b;
    double w[4];
    herm4(kn, kFK, (a.pos[i] - X0) / SX, &b, w);
    for (int q = 0; q < 4; q++) if (b + q >= 0 && b + q < kFK) wk[(size_t)i * kFK + b + q] += (float)w[q];
  }
  // the timing track's cells: 2 x 2 modules at depth 5..6 on every side, the even runs of 4 (layout.c:57-61, 69-141)
  std::vector<float4> track;
  {
    const int side = span + 2 * kMargin, reserve = 15;
    for (int sd = 0; sd < 4; sd++)
      for (int cell = 0; reserve + 2 * cell + 1 < side - reserve; cell++) {
        if ((cell / 4) & 1) continue;
        const float along = (float)(reserve + 2 * cell + 1), depth = 6.0f;
        const float dark = (float)track_bit(sd, cell / 4 / 2 * 4 + cell % 4);
        float mx, my;
        if (sd == 0) { mx = along; my = depth; }
        else if (sd == 2) { mx = along; my = (float)side - depth; }
        else if (sd == 3) { mx = depth; my = along; }
        else { mx = (float)side - depth; my = along; }
        if ((int)track.size() < kFMaxTrack) track.push_back(make_float4(mx, my, dark, 0.0f));
      }
  }
  a.ntrack = (int)track.size();
  // the detrend basis and its DFTs, the sender's transform's twiddles
  std::vector<float2> x1(n), x2(n);
  for (int t = 0; t < n; t++) { x1[t] = make_float2(f.x1r[t], f.x1i[t]); x2[t] = make_float2(f.x2r[t], f.x2i[t]); }
  int rad[3], lines;
  if (fft_plan(n, rad, &lines)) { delete g; record_error(LIZG_E_ARG, "lizg_field_new: no transform plan"); return nullptr; }
  std::vector<float2> tws(n);
  for (int s = 0, ns = 1; s < 3; ns *= rad[s], s++)
    for (int q = 1; q < rad[s]; q++)
      for (int k = 0; k < ns; k++) {
        const double th = -2.0 * 3.14159265358979323846 * q * k / ((double)ns * rad[s]);
        tws[ns + (q - 1) * ns + k] = make_float2((float)std::cos(th), (float)std::sin(th));
      }
  g->chunk = chunk;
  bool ok = np >= 16;
  auto up = [&](const void *src, size_t bytes) -> void * {
    void *d = nullptr;
    if (!ok || cudaMalloc(&d, std::max<size_t>(bytes, 1)) != cudaSuccess) { ok = false; return nullptr; }
    g->owned.push_back(d);
    if (src && bytes && cudaMemcpy(d, src, bytes, cudaMemcpyHostToDevice) != cudaSuccess) ok = false;
    return d;
  };
  a.pilot = static_cast<int32_t *>(up(pk.data(), pk.size() * 4));
  a.puv = static_cast<int16_t *>(up(puv.data(), puv.size() * 2));
  a.shat = static_cast<float2 *>(up(shat.data(), shat.size() * sizeof(float2)));
  a.group = static_cast<uint8_t *>(up(grp.data(), grp.size()));
  a.wk = static_cast<float *>(up(wk.data(), wk.size() * 4));
  a.track = static_cast<float4 *>(up(track.data(), track.size() * sizeof(float4)));
  a.cx = static_cast<float *>(up(f.cx.data(), f.cx.size() * 4));
  a.qx = static_cast<float *>(up(f.qx.data(), f.qx.size() * 4));
  a.x1 = static_cast<float2 *>(up(x1.data(), x1.size() * sizeof(float2)));
  a.x2 = static_cast<float2 *>(up(x2.data(), x2.size() * sizeof(float2)));
  g->enc.n = n; g->enc.vrows = a.vrows; g->enc.lim = 3.0e38f; g->enc.sc = 1.0f;
  g->enc.tws = static_cast<float2 *>(up(tws.data(), tws.size() * sizeof(float2)));
  const size_t C = (size_t)chunk;
  g->eff = static_cast<float *>(up(nullptr, C * a.reg_stride * 4));
  g->base = static_cast<float *>(up(nullptr, C * a.reg_stride * 4));
  g->G = static_cast<float *>(up(nullptr, C * n * n * 4));
  g->part = static_cast<float *>(up(nullptr, C * (n / kFRows) * kFPart * 4));
  g->coef = static_cast<float2 *>(up(nullptr, C * a.need * sizeof(float2)));
  g->R = static_cast<float2 *>(up(nullptr, C * a.vrows * n * sizeof(float2)));
  g->state = static_cast<FieldState *>(up(nullptr, C * sizeof(FieldState)));
  g->pt = static_cast<PilotTerms *>(up(nullptr, C * sizeof(PilotTerms)));
  g->skip = static_cast<uint8_t *>(up(nullptr, C));
  if (ok) {
    g->rx = lizg_rx_new(n, subch, span, chunk);
    ok = g->rx != nullptr;
    if (ok) lizg_rx_set_read(g->rx, LIZG_READ_EXACT);   // the refinement's forward model: the float walk it differentiates
  }
  if (!ok) {
    lizg_field_free(g);
    record_error(LIZG_E_NOMEM, np < 16 ? "lizg_field_new: the format has too few pilots" : "lizg_field_new: device allocation failed");
    return nullptr;
  }
  static SmemOptIn opt;
  if (opt.set(reinterpret_cast<const void *>(field_solve_kernel), (int)kSolveSmem) != cudaSuccess) {
    lizg_field_free(g);
    record_error(LIZG_E_CUDA, "lizg_field_new: shared memory opt-in");
    return nullptr;
  }
  return g;
}

void lizg_field_free(lizg_field *g) {
  if (!g) return;
  if (g->rx) lizg_rx_free(g->rx);
  for (void *p : g->owned) cudaFree(p);
  delete g;
}

}  // extern "C"

namespace {

// One evaluation of a chunk of fc frames (luma and base registrations at frame f0 of the call): the registration the
// parameters give, the spectrum, the pilots, the adjoint transform and pass, then the step (or, with terms, the raw
// terms).
int field_eval(lizg_field *g, const lizg::FieldArgs &a, const float *base, int fc, const lizg_anchor_out *anchors, int f0, int last,
               double *terms, cudaStream_t st) {
  using namespace lizg;
  field_mesh_kernel<<<fc, 256, 0, st>>>(a, g->state, 0, base, g->eff);
  if (int rc = rx_spectrum_luma(g->rx, a.luma, a.w, a.h, a.w, a.fstride, g->eff, fc, reinterpret_cast<float *>(g->coef), st)) return rc;
  // the last evaluation of a refinement (last, no terms asked for) needs the pilots' loss alone: no adjoint
  const bool adjoint = !last || terms;
  if (adjoint) cudaMemsetAsync(g->R, 0, sizeof(float2) * (size_t)fc * a.vrows * a.n, st);
  field_pilot_kernel<<<fc, kFThreads, 0, st>>>(a, g->coef, g->skip, g->R, g->pt);
  if (adjoint) {
    if (enc_fft_launch(g->enc, fc, g->R, g->G, st) != cudaSuccess) return record_error(LIZG_E_CUDA, "lizg_field: adjoint transform launch");
    field_grad_kernel<<<fc * (a.n / kFRows), kFThreads, 0, st>>>(a, g->eff, g->G, g->pt, g->skip, g->part);
  }
  const float *au = anchors ? anchors->u + (int64_t)f0 * 49 : nullptr, *av = anchors ? anchors->v + (int64_t)f0 * 49 : nullptr;
  const uint8_t *ao = anchors ? anchors->ok + (int64_t)f0 * 49 : nullptr;
  field_solve_kernel<<<fc, 256, kSolveSmem, st>>>(a, g->eff, g->part, g->pt, au, av, ao, g->skip, g->state, last, terms);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : record_error(LIZG_E_CUDA, (std::string("lizg_field: ") + cudaGetErrorString(e)).c_str());
}

int check_frames(const lizg_field *g, const uint8_t *d_luma, int w, int h, int64_t frame_stride, const void *d_reg, int frames, const char *who) {
  if (!g || !d_luma || !d_reg || frames < 1 || w < 2 || h < 2 || (frames > 1 && frame_stride < (int64_t)w * h))
    return lizg::record_error(LIZG_E_ARG, (std::string(who) + ": NULL argument, empty batch or frame under 2 x 2").c_str());
  return 0;
}

}  // namespace

extern "C" {

int lizg_field_refine_dev(lizg_field *g, const uint8_t *d_luma, int w, int h, int64_t frame_stride, float *d_reg, int frames, int steps,
                          const lizg_anchor_out *anchors, const uint8_t *d_gate, float *d_loss, int32_t *d_improved, void *stream) {
  using namespace lizg;
  if (int rc = check_frames(g, d_luma, w, h, frame_stride, d_reg, frames, "lizg_field_refine_dev")) return rc;
  if (steps < 0 || steps > 16) return record_error(LIZG_E_ARG, "lizg_field_refine_dev: steps outside 0..16");
  if (anchors && (!anchors->ok || !anchors->u || !anchors->v)) return record_error(LIZG_E_ARG, "lizg_field_refine_dev: anchors without ok, u, v");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the gate on the host: only runs of frames it lets through are worked on
  std::vector<uint8_t> gate(frames, 1);
  if (d_gate && (cudaMemcpyAsync(gate.data(), d_gate, frames, cudaMemcpyDeviceToHost, st) != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess))
    return record_error(LIZG_E_CUDA, "lizg_field_refine_dev: reading the gate");
  for (int f0 = 0; f0 < frames;) {
    if (!gate[f0]) { f0++; continue; }
    int fc = 0;
    while (f0 + fc < frames && fc < g->chunk && gate[f0 + fc]) fc++;
    FieldArgs a = g->a;
    a.w = w; a.h = h; a.fstride = frame_stride;
    a.luma = d_luma + (int64_t)f0 * frame_stride;
    float *reg = d_reg + (int64_t)f0 * a.reg_stride;
    cudaMemsetAsync(g->skip, 0, fc, st);
    cudaMemcpyAsync(g->base, reg, sizeof(float) * fc * a.reg_stride, cudaMemcpyDeviceToDevice, st);
    field_load_kernel<<<(fc + 127) / 128, 128, 0, st>>>(g->base, a.reg_stride, nullptr, fc, g->state);
    for (int e = 0; e <= steps; e++)   // steps + 1 evaluations: the baseline, then each step's
      if (int rc = field_eval(g, a, g->base, fc, anchors, f0, e == steps, nullptr, st)) return rc;
    field_mesh_kernel<<<fc, 256, 0, st>>>(a, g->state, 1, g->base, g->eff);
    field_copy_kernel<<<dim3(1, fc), 256, 0, st>>>(g->eff, g->skip, fc, a.reg_stride, reg);
    field_store_kernel<<<(fc + 127) / 128, 128, 0, st>>>(g->state, g->skip, fc, d_loss ? d_loss + f0 : nullptr, d_improved ? d_improved + f0 : nullptr);
    f0 += fc;
  }
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : record_error(LIZG_E_CUDA, (std::string("lizg_field_refine_dev: ") + cudaGetErrorString(e)).c_str());
}

int lizg_field_terms_dev(lizg_field *g, const uint8_t *d_luma, int w, int h, int64_t frame_stride, const float *d_reg, const float *d_theta,
                         int frames, const lizg_anchor_out *anchors, double *d_terms, void *stream) {
  using namespace lizg;
  if (int rc = check_frames(g, d_luma, w, h, frame_stride, d_reg, frames, "lizg_field_terms_dev")) return rc;
  if (!d_theta || !d_terms || frames > g->chunk) return record_error(LIZG_E_ARG, "lizg_field_terms_dev: NULL theta or terms, or frames over the chunk");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  FieldArgs a = g->a;
  a.w = w; a.h = h; a.fstride = frame_stride; a.luma = d_luma;
  cudaMemsetAsync(g->skip, 0, frames, st);
  cudaMemcpyAsync(g->base, d_reg, sizeof(float) * frames * a.reg_stride, cudaMemcpyDeviceToDevice, st);
  field_load_kernel<<<(frames + 127) / 128, 128, 0, st>>>(g->base, a.reg_stride, d_theta, frames, g->state);
  return field_eval(g, a, g->base, frames, anchors, 0, 0, d_terms, st);
}

}  // extern "C"

// The picture sampler's arithmetic for one sample (row a), shared by the standalone sampler and the column pass that
// reads samples straight from the captured frame, in the receiver's two reads: the exact walk (liblizard/src/
// acquire.c:5121-5196 and internal.h:11-23, what the reference's portable build decodes with) and the decode's integer
// read (below, what its x86-64 build decodes with). Every float operation is an explicit round-to-nearest intrinsic
// in the reference's order, so no compiler contraction can change a value: the results are the reference's bit for
// bit, whatever the file's -fmad setting.
#ifndef LIZG_SAMPLE_DEV_CUH
#define LIZG_SAMPLE_DEV_CUH
#include "lizg_internal.h"

namespace lizg {

// The mesh cell along one axis: the last k in [0, nn - 2] with m >= node[k], else 0 (liblizard/src/acquire.c:5089).
__device__ __forceinline__ int node_cell(const float *node, int nn, float m) {
  int k = 0;
  for (int q = 1; q <= nn - 2; q++) if (m >= node[q]) k = q;
  return k;
}

// The format's per-column and per-row quantities of the walk (liblizard/src/acquire.c:5131-5140, 5160-5166).
__device__ __forceinline__ float4 sample_col(const SampleDev &sd, int x) {
  const float mx = __fadd_rn(sd.g0, __fmul_rn((float)x, sd.step));
  const int i = node_cell(sd.node_x, sd.nx, mx);
  return make_float4(mx, __int_as_float(i), __fdiv_rn(1.0f, __fsub_rn(sd.node_x[i + 1], sd.node_x[i])), 0.0f);
}
__device__ __forceinline__ float4 sample_row(const SampleDev &sd, int y) {
  const float my = __fadd_rn(sd.g0, __fmul_rn((float)y, sd.step));
  const int j = node_cell(sd.node_y, sd.ny, my);
  return make_float4(my, __int_as_float(j), __fdiv_rn(__fsub_rn(my, sd.node_y[j]), __fsub_rn(sd.node_y[j + 1], sd.node_y[j])), 0.0f);
}

// k / 255 rounded to nearest for a grey level k (0..255), with no division and no table: q = k r, r the float
// nearest 1 / 255, then one correction from the exact remainder k - 255 q (Markstein's method). It equals the
// correctly rounded quotient, the reference's i / 255.0f, for every k (checked exhaustively in exact arithmetic).
__device__ __forceinline__ float grey_of(unsigned k) {
  const float r = 0.003921568859368563f, kf = (float)k, q = __fmul_rn(kf, r);
  return __fmaf_rn(__fmaf_rn(-q, 255.0f, kf), r, q);
}

// The walk's quantities of one picture row: the row's place in its mesh cell and the homography's row terms.
struct RowTerms {
  float my, v, omv, kw, ku, kv;
  int j;
};
__device__ __forceinline__ RowTerms row_terms(const float *H, float4 rt) {
  RowTerms r;
  r.my = rt.x; r.v = rt.z; r.omv = __fsub_rn(1.0f, r.v); r.j = __float_as_int(rt.y);
  r.kw = __fadd_rn(__fmul_rn(H[7], r.my), 1.0f); r.ku = __fadd_rn(__fmul_rn(H[1], r.my), H[2]); r.kv = __fadd_rn(__fmul_rn(H[4], r.my), H[5]);
  return r;
}

// The mesh displacement's line along a row within cell (i, j): d = c + e mx, each axis.
struct CellTerms {
  float ex, cx, ey, cy;
};
__device__ __forceinline__ CellTerms cell_terms(const SampleDev &sd, const float *nodes, int i, float inv, const RowTerms &r) {
  const float *n00 = nodes + 2 * (r.j * sd.nx + i), *n10 = n00 + 2, *n01 = n00 + 2 * sd.nx, *n11 = n01 + 2;
  const float nxi = sd.node_x[i], v = r.v, omv = r.omv;
  CellTerms c;
  c.ex = __fmul_rn(__fadd_rn(__fmul_rn(__fsub_rn(n10[0], n00[0]), omv), __fmul_rn(__fsub_rn(n11[0], n01[0]), v)), inv);
  c.cx = __fsub_rn(__fadd_rn(__fmul_rn(n00[0], omv), __fmul_rn(n01[0], v)), __fmul_rn(c.ex, nxi));
  c.ey = __fmul_rn(__fadd_rn(__fmul_rn(__fsub_rn(n10[1], n00[1]), omv), __fmul_rn(__fsub_rn(n11[1], n01[1]), v)), inv);
  c.cy = __fsub_rn(__fadd_rn(__fmul_rn(n00[1], omv), __fmul_rn(n01[1], v)), __fmul_rn(c.ey, nxi));
  return c;
}

// The sample at module column mx of a row: h6 = H[6] mx, h0 = H[0] mx, h3 = H[3] mx (the column's products), then the
// projection, the mesh's displacement, the frame-edge clamp and the bilinear grey read.
__device__ __forceinline__ float sample_at(const uint8_t *px, int w, int h, int pitch, float mx, float h6, float h0, float h3,
                                           const RowTerms &r, const CellTerms &c) {
  const float rw = __fdiv_rn(1.0f, __fadd_rn(h6, r.kw));
  const float pu = __fmul_rn(__fadd_rn(h0, r.ku), rw), pv = __fmul_rn(__fadd_rn(h3, r.kv), rw);
  const float dx = __fadd_rn(c.cx, __fmul_rn(c.ex, mx)), dy = __fadd_rn(c.cy, __fmul_rn(c.ey, mx));
  float sx = __fsub_rn(__fadd_rn(pu, dx), 0.5f), sy = __fsub_rn(__fadd_rn(pv, dy), 0.5f);
  const float xm = __fsub_rn((float)w, 1.001f), ym = __fsub_rn((float)h, 1.001f);
  if (sx < 0) sx = 0; else if (sx > xm) sx = xm;
  if (sy < 0) sy = 0; else if (sy > ym) sy = ym;
  const int xi = sx >= 0 ? (int)sx : 0, yi = sy >= 0 ? (int)sy : 0;   // a NaN coordinate reads pixel 0
  const float fx = __fsub_rn(sx, (float)xi), fy = __fsub_rn(sy, (float)yi);
  const uint8_t *p = px + (int64_t)yi * pitch + xi;
  const float a = grey_of(p[0]), b = grey_of(p[1]), cc = grey_of(p[pitch]), d = grey_of(p[pitch + 1]);
  return __fadd_rn(__fmul_rn(__fadd_rn(a, __fmul_rn(__fsub_rn(b, a), fx)), __fsub_rn(1.0f, fy)),
                   __fmul_rn(__fadd_rn(cc, __fmul_rn(__fsub_rn(d, cc), fx)), fy));
}

// Sample (x, y) of the picture grid from frame px (w x h, rows pitch apart) through H (9 floats) and the node mesh,
// given the column's and the row's table entries.
__device__ __forceinline__ float sample_xy_exact(const SampleDev &sd, const uint8_t *px, int w, int h, int pitch, const float *H,
                                                 const float *nodes, float4 ct, float4 rt) {
  const RowTerms r = row_terms(H, rt);
  const CellTerms c = cell_terms(sd, nodes, __float_as_int(ct.y), ct.z, r);
  const float mx = ct.x;
  return sample_at(px, w, h, pitch, mx, __fmul_rn(H[6], mx), __fmul_rn(H[0], mx), __fmul_rn(H[3], mx), r, c);
}

// ---------------------------------------------------------------- the decode's read (LIZG_READ_DECODE)
//
// The reference decoder's own picture read on x86-64 (liblizard/src/acquire.c:5302-5440 sample_grid_lin, reached through
// ob_sample_grid_pic :5465-5480, with lin_pts / lin_grey / lin_get :723-779), which lizard_finish calls a strip of 64
// columns at a time (liblizard/src/lizard_phy.c:1634) and once for the shading fit's every-eighth samples (:1611).
// The same map as the exact walk with other roundings: each column's displacement as D + v E (D, E lines in the
// column's place u within its mesh cell, worked out once a mesh row), the homography's numerators and denominator
// as four-column lanes stepped four columns at a time from the call's first column (lane l starts at
// l (h step) + (h m0 + the row's terms); each step adds 4 (h step)), one reciprocal of the denominator, and the
// point (less half a pixel, x a 512th of a pixel on) read in integers: 16.16 coordinates, 8-bit x and 15-bit y
// fractions, a two-stage integer blend giving 128 times the grey, times 257 / 2^23. Every float operation here is an
// explicit round-to-nearest intrinsic in the reference's order, so the values are its bit for bit.

// A column's displacement terms at mesh row j: D = (dx, dy) and E = (ex, ey), the point's offset being D + v E plus
// the homography's part (liblizard/src/acquire.c:5330-5346 with tu :5310-5316). x's entry of the column table gives
// its module coordinate mx, mesh cell i and 1 / the cell's width.
__device__ __forceinline__ float4 lin_cell(const SampleDev &sd, const float *nodes, float4 ct, int j) {
  const int i = __float_as_int(ct.y);
  const float U = __fmul_rn(__fsub_rn(ct.x, sd.node_x[i]), ct.z);
  const float *a = nodes + 2 * (j * sd.nx + i), *b = a + 2 * sd.nx;
  const float ax = __fsub_rn(a[2], a[0]), ay = __fsub_rn(a[3], a[1]);
  const float dx = __fadd_rn(__fsub_rn(a[0], 0.498046875f), __fmul_rn(ax, U));   // 0.5 - 1 / 512
  const float ex = __fadd_rn(__fsub_rn(b[0], a[0]), __fmul_rn(__fsub_rn(__fsub_rn(b[2], b[0]), ax), U));
  const float dy = __fadd_rn(__fsub_rn(a[1], 0.5f), __fmul_rn(ay, U));
  const float ey = __fadd_rn(__fsub_rn(b[1], a[1]), __fmul_rn(__fsub_rn(__fsub_rn(b[3], b[1]), ay), U));
  return make_float4(dx, ex, dy, ey);
}

// A column's lanes of the homography walk within its call: lane l = the column's place mod 4, g = the four-column
// steps from the call's first column to it, the lanes' starts l (h step) and the step 4 (h step) for h = H[6], H[0],
// H[3], and h m0 (m0 the call's first column's module coordinate).
struct LinCol {
  float bw, bu, bv, cw, cu, cv, w0, u0, v0;
  int g;
};
// k: the column's place in its call; m0: the call's first column's module coordinate; st: the call's step.
__device__ __forceinline__ LinCol lin_col(const float *H, int k, float m0, float st) {
  LinCol c;
  const float hw = __fmul_rn(H[6], st), hu = __fmul_rn(H[0], st), hv = __fmul_rn(H[3], st), lane = (float)(k & 3);
  c.bw = __fmul_rn(lane, hw); c.bu = __fmul_rn(lane, hu); c.bv = __fmul_rn(lane, hv);
  c.cw = __fmul_rn(4.0f, hw); c.cu = __fmul_rn(4.0f, hu); c.cv = __fmul_rn(4.0f, hv);
  c.w0 = __fmul_rn(H[6], m0); c.u0 = __fmul_rn(H[0], m0); c.v0 = __fmul_rn(H[3], m0);
  c.g = k >> 2;   // the calls here span at most 256 columns: one chunk of the walk
  return c;
}
// The grid's column x: its call is the strip of 64 columns holding it (liblizard/src/lizard_phy.c:1634).
__device__ __forceinline__ LinCol lin_col_grid(const SampleDev &sd, const float *H, int x) {
  const int xs = x & ~63;
  return lin_col(H, x - xs, __fadd_rn(sd.g0, __fmul_rn((float)xs, sd.step)), sd.step);
}
// The shading fit's column kx (every eighth picture column): one call from column 0 at eight steps (:1611).
__device__ __forceinline__ LinCol lin_col_shade(const SampleDev &sd, const float *H, int kx) {
  return lin_col(H, kx, sd.g0, __fmul_rn(8.0f, sd.step));
}

// The lanes' numerators and denominator at a row (row terms kw, ku, kv as row_terms gives them), g steps on.
struct LinNum {
  float w, u, v;
};
__device__ __forceinline__ LinNum lin_start(const LinCol &c, float kw, float ku, float kv) {
  LinNum s;
  s.w = __fadd_rn(c.bw, __fadd_rn(c.w0, kw)); s.u = __fadd_rn(c.bu, __fadd_rn(c.u0, ku)); s.v = __fadd_rn(c.bv, __fadd_rn(c.v0, kv));
  return s;
}
__device__ __forceinline__ void lin_steps(const LinCol &c, LinNum &s, int steps) {
  for (int q = 0; q < steps; q++) { s.w = __fadd_rn(s.w, c.cw); s.u = __fadd_rn(s.u, c.cu); s.v = __fadd_rn(s.v, c.cv); }
}

// 16.16 from a coordinate: below 0 (and NaN) 0, held under 2^15 pixels, truncated (the product is exact).
__device__ __forceinline__ int lin_q16(float v) {
  v = v > 0.0f ? v : 0.0f;
  v = v < 32767.0f ? v : 32767.0f;
  return (int)__fmul_rn(v, 65536.0f);
}
// The point at (X, Y) (pixel coordinates less the half pixel, X a 512th on) read in integers: the integer parts
// clamped to w - 2 and h - 2 (every read inside the frame), each row's pair blended as 256 a + (b - a) fx, the
// rows' halved difference (floored) times fy rounded at bit 15, plus the top row's half; 128 times the grey (0 to
// 32640, -1 where the halves round so), times 257 / 2^23 (exact).
__device__ __forceinline__ float lin_read(const uint8_t *px, int w, int h, int pitch, float X, float Y) {
  const int xq = lin_q16(X), yq = lin_q16(Y);
  const int xi = min(xq >> 16, w - 2), yi = min(yq >> 16, h - 2);
  const int fx = (xq >> 8) & 0xff, fy = (yq & 0xffff) >> 1;
  const uint8_t *p = px + (int64_t)yi * pitch + xi;
  const int a = p[0], b = p[1], c = p[pitch], d = p[pitch + 1];
  const int top = 256 * a + (b - a) * fx, bot = 256 * c + (d - c) * fx;
  const int r = ((((bot - top) >> 1) * fy + (1 << 14)) >> 15) + (top >> 1);
  return __fmul_rn((float)r, 257.0f / 8388608.0f);
}
// The point of lanes s (at the column's step) with the column's displacement terms T at the row's place vv.
__device__ __forceinline__ float lin_point(const uint8_t *px, int w, int h, int pitch, const LinNum &s, float4 T, float vv) {
  const float rw = __fdiv_rn(1.0f, s.w);
  const float X = __fadd_rn(__fadd_rn(T.x, __fmul_rn(T.y, vv)), __fmul_rn(s.u, rw));
  const float Y = __fadd_rn(__fadd_rn(T.z, __fmul_rn(T.w, vv)), __fmul_rn(s.v, rw));
  return lin_read(px, w, h, pitch, X, Y);
}

// Sample (x, y) of the picture grid by the decode's read, everything worked out from H and the mesh.
__device__ __forceinline__ float sample_xy_decode(const SampleDev &sd, const uint8_t *px, int w, int h, int pitch, const float *H,
                                                  const float *nodes, int x, float4 ct, float4 rt) {
  const RowTerms r = row_terms(H, rt);
  const LinCol c = lin_col_grid(sd, H, x);
  LinNum s = lin_start(c, r.kw, r.ku, r.kv);
  lin_steps(c, s, c.g);
  return lin_point(px, w, h, pitch, s, lin_cell(sd, nodes, ct, r.j), r.v);
}

// Sample (x, y) by the receiver's read: the decode's (sd.read = LIZG_READ_DECODE) or the exact walk.
__device__ __forceinline__ float sample_xy(const SampleDev &sd, const uint8_t *px, int w, int h, int pitch, const float *H,
                                           const float *nodes, int x, float4 ct, float4 rt) {
  return sd.read == LIZG_READ_DECODE ? sample_xy_decode(sd, px, w, h, pitch, H, nodes, x, ct, rt)
                                     : sample_xy_exact(sd, px, w, h, pitch, H, nodes, ct, rt);
}

}  // namespace lizg
#endif

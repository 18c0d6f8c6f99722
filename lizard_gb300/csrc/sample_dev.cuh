// The picture sampler's arithmetic for one sample (row a), shared by the standalone sampler and the column pass that
// reads samples straight from the captured frame. Every float operation is an explicit round-to-nearest intrinsic
// in the reference's order (liblizard/src/acquire.c:5121-5196 and internal.h:11-23), so no compiler contraction can
// change a value: the result is the reference's exact walk bit for bit, whatever the file's -fmad setting.
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
__device__ __forceinline__ float sample_xy(const SampleDev &sd, const uint8_t *px, int w, int h, int pitch, const float *H,
                                           const float *nodes, float4 ct, float4 rt) {
  const RowTerms r = row_terms(H, rt);
  const CellTerms c = cell_terms(sd, nodes, __float_as_int(ct.y), ct.z, r);
  const float mx = ct.x;
  return sample_at(px, w, h, pitch, mx, __fmul_rn(H[6], mx), __fmul_rn(H[0], mx), __fmul_rn(H[3], mx), r, c);
}

}  // namespace lizg
#endif

// Oracle (test infrastructure only): the anchor search of the registration's front half, restated in plain C from the
// reference's portable build (liblizard/src/acquire.c:1876-2036 anchor_find, its #else branch: the scalar twin of the
// SIMD paths), to hold the GPU's anchor search to. Compiled with -ffp-contract=off: every float and double operation
// rounds once, in the reference's order. Pinned against the reference's own portable build (oracle/_ref/
// libref_scalar.so) by the CPU tests and against fixtures it made (tests/golden/anchor_ref.npz).
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "oracle.h"

enum { ANK = 7, ANTS = 16, ANREACH = 3, LENSP = 11, MARGIN = 15 };
static const float ANPEAK = 0.6f;

// The layout's anchor lattice (liblizard/src/acquire.c:41-45): side a = span / 64 modules, anchor i's low edge m0.
static int anchor_m0(int span, int i) {
  const int a = span / 64;
  return (int)floor(MARGIN + (double)span * (i + 0.5) / ANK - a / 2.0 + 0.5);
}

// H: module -> image (liblizard/src/internal.h:107-112).
static void project(const float *h, float x, float y, float *u, float *v) {
  const float w = h[6] * x + h[7] * y + 1;
  *u = (h[0] * x + h[1] * y + h[2]) / w;
  *v = (h[3] * x + h[4] * y + h[5]) / w;
}

// The lens model's displacement at image point (u, v) (liblizard/src/acquire.c:1506-1512 lens_rows, 1615-1620
// lensm_at): lens = K, ax, ay, R, t[LENSP].
static void lens_at(const double *lens, double u, double v, float *dx, float *dy) {
  const int K = (int)lens[0];
  const double x = (u - lens[1]) / lens[3], y = (v - lens[2]) / lens[3];
  double rx[LENSP], ry[LENSP];
  const double ex[8] = {x, y, 0, 0, 1, 0, -x * x, -x * y}, ey[8] = {0, 0, x, y, 0, 1, -x * y, -y * y};
  for (int a = 0; a < 8; a++) { rx[a] = ex[a]; ry[a] = ey[a]; }
  const double s = x * x + y * y;
  double sk = s;
  for (int k = 0; k < K; k++, sk *= s) { rx[8 + k] = sk * x; ry[8 + k] = sk * y; }
  double fx = 0, fy = 0;
  for (int a = 0; a < 8 + K; a++) { fx += lens[4 + a] * rx[a]; fy += lens[4 + a] * ry[a]; }
  *dx = (float)fx; *dy = (float)fy;
}

// Module point -> image point through H and the lens model when given (liblizard/src/acquire.c:1699-1702).
static void anchor_map(const float *h, const double *lens, float X, float Y, float *u, float *v) {
  project(h, X, Y, u, v);
  if (lens) { float dx, dy; lens_at(lens, *u, *v, &dx, &dy); *u += dx; *v += dy; }
}

// The bilinear grey read at gamma 1 (liblizard/src/internal.h:11-23), rows w apart.
static float sample(const uint8_t *px, int w, int h, float x, float y) {
  x -= 0.5f; y -= 0.5f;
  if (x < 0) x = 0; else if (x > w - 1.001f) x = w - 1.001f;
  if (y < 0) y = 0; else if (y > h - 1.001f) y = h - 1.001f;
  const int xi = x >= 0 ? (int)x : 0, yi = y >= 0 ? (int)y : 0;
  const float fx = x - xi, fy = y - yi;
  const uint8_t *p = px + yi * w + xi;
  const float a = p[0] / 255.0f, b = p[1] / 255.0f, c = p[w] / 255.0f, d = p[w + 1] / 255.0f;
  return (a + (b - a) * fx) * (1 - fy) + (c + (d - c) * fx) * fy;
}

#define ABOX(I, x, y, s) ((I)[((y) + (s)) * W1 + (x) + (s)] - (I)[(y) * W1 + (x) + (s)] - (I)[((y) + (s)) * W1 + (x)] + (I)[(y) * W1 + (x)])

int orc_anchor_find(int span, const uint8_t *px, int w, int h, const float *H, const double *lens, const uint8_t *ok_in,
                    uint8_t *ok, float *peak, float *dxo, float *dyo, float *uo, float *vo) {
  const int a = span / 64;
  if (a < 1) return 0;
  const float hs = (float)a / ANTS;
  const int r = (int)ceilf((float)ANREACH / hs), W = ANTS + 2 * r, O = 2 * r + 1, W1 = W + 1;
  // the template: concentric squares, +1 inside a quarter and outside six tenths of the half side, -1 between
  float T[ANTS * ANTS], tm = 0, tn = 0;
  for (int y = 0; y < ANTS; y++)
    for (int x = 0; x < ANTS; x++) {
      const float u = (x + 0.5f) * hs - a * 0.5f, v = (y + 0.5f) * hs - a * 0.5f, dc = fmaxf(fabsf(u), fabsf(v)) / (a * 0.5f);
      T[y * ANTS + x] = dc < 0.25f || dc >= 0.6f ? 1.0f : -1.0f;
      tm += T[y * ANTS + x];
    }
  tm /= (float)(ANTS * ANTS);
  for (int k = 0; k < ANTS * ANTS; k++) { T[k] -= tm; tn += T[k] * T[k]; }
  tn = sqrtf(tn);
  int i25 = ANTS, j25 = -1, i6 = ANTS, j6 = -1;
  for (int x = 0; x < ANTS; x++) {
    const float d = fabsf((x + 0.5f) * hs - a * 0.5f) / (a * 0.5f);
    if (d < 0.25f) { if (x < i25) i25 = x; j25 = x; }
    if (d < 0.6f) { if (x < i6) i6 = x; j6 = x; }
  }
  float *win = malloc(sizeof(float) * W * W), *C = malloc(sizeof(float) * O * O);
  double *I1 = malloc(sizeof(double) * W1 * W1), *I2 = malloc(sizeof(double) * W1 * W1);
  int found = 0;
  for (int j = 0; j < ANK; j++)
    for (int i = 0; i < ANK; i++) {
      const int k = j * ANK + i;
      ok[k] = 0; peak[k] = 0; dxo[k] = dyo[k] = uo[k] = vo[k] = 0;
      if (ok_in && ok_in[k]) { ok[k] = 1; found++; continue; }
      const float x0 = (float)anchor_m0(span, i), y0 = (float)anchor_m0(span, j), X = x0 + a * 0.5f, Y = y0 + a * 0.5f;
      // the window: W x W samples a template step apart about the anchor's place
      for (int wy = 0; wy < W; wy++)
        for (int wx = 0; wx < W; wx++) {
          float u, v;
          anchor_map(H, lens, x0 + (wx - r + 0.5f) * hs, y0 + (wy - r + 0.5f) * hs, &u, &v);
          win[wy * W + wx] = sample(px, w, h, u, v);
        }
      // its integral images of the greys and their squares, in double, row by row
      for (int x = 0; x < W1; x++) I1[x] = I2[x] = 0;
      for (int wy = 0; wy < W; wy++) {
        double s = 0, q = 0;
        I1[(wy + 1) * W1] = I2[(wy + 1) * W1] = 0;
        for (int wx = 0; wx < W; wx++) {
          const double vv = win[wy * W + wx];
          s += vv; q += vv * vv;
          I1[(wy + 1) * W1 + wx + 1] = I1[wy * W1 + wx + 1] + s;
          I2[(wy + 1) * W1 + wx + 1] = I2[wy * W1 + wx + 1] + q;
        }
      }
      // the normalised correlation at every offset from box sums; the first largest in scan order
      float best = -2;
      int bx = 0, by = 0;
      for (int oy = -r; oy <= r; oy++)
        for (int ox = -r; ox <= r; ox++) {
          const int qx = r + ox, qy = r + oy;
          const double s1 = ABOX(I1, qx, qy, ANTS), s2 = ABOX(I2, qx, qy, ANTS), var = s2 - s1 * s1 / (ANTS * ANTS);
          const double s25 = j25 >= i25 ? ABOX(I1, qx + i25, qy + i25, j25 - i25 + 1) : 0;
          const double s6 = j6 >= i6 ? ABOX(I1, qx + i6, qy + i6, j6 - i6 + 1) : 0;
          const double st = 2 * (s25 - s6) + s1 * (1 - (double)tm);
          const float c = var > 1e-12 ? (float)(st / (sqrt(var) * tn)) : 0;
          C[(oy + r) * O + ox + r] = c;
          if (c > best) { best = c; bx = ox; by = oy; }
        }
      // a parabola through the peak and its neighbours, each way
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
      anchor_map(H, lens, X + (bx + sx) * hs, Y + (by + sy) * hs, &u, &v);
      project(H, X, Y, &hu, &hv);
      peak[k] = best; dxo[k] = u - hu; dyo[k] = v - hv; uo[k] = u; vo[k] = v;
      ok[k] = best >= ANPEAK && bx > -r && bx < r && by > -r && by < r;
      found += ok[k];
    }
  free(win); free(C); free(I1); free(I2);
  return found;
}

// ---------------------------------------------------------------- the lens model from the anchors

// Gauss-Jordan with partial pivoting on the first n rows of the normal equations, right-hand side in column LENSP
// (liblizard/src/acquire.c:1491-1504 solve_lens).
static int solve_lens(double A[LENSP][LENSP + 1], int n) {
  for (int c = 0; c < n; c++) {
    int p = c;
    for (int r = c + 1; r < n; r++) if (fabs(A[r][c]) > fabs(A[p][c])) p = r;
    if (fabs(A[p][c]) < 1e-14) return 0;
    for (int k = 0; k <= LENSP; k++) { const double t = A[c][k]; A[c][k] = A[p][k]; A[p][k] = t; }
    for (int r = 0; r < n; r++) {
      if (r == c) continue;
      const double f = A[r][c] / A[c][c];
      for (int k = c; k <= LENSP; k++) A[r][k] -= f * A[c][k];
    }
  }
  return 1;
}

static void lens_rows(double x, double y, int K, double *rx, double *ry) {
  const double ex[8] = {x, y, 0, 0, 1, 0, -x * x, -x * y}, ey[8] = {0, 0, x, y, 0, 1, -x * y, -y * y};
  for (int a = 0; a < 8; a++) { rx[a] = ex[a]; ry[a] = ey[a]; }
  const double s = x * x + y * y;
  double sk = s;
  for (int k = 0; k < K; k++, sk *= s) { rx[8 + k] = sk * x; ry[8 + k] = sk * y; }
}

// The lens model the anchors and the four corner nodes give about H (liblizard/src/acquire.c:2043-2061 anchor_model,
// with lensm_fit's first round, 1630-1669: the normal equations summed once in the points' order, every model of
// 0..3 radial terms solved, the one of least AICc kept). The axis is the frame's centre and R its half-diagonal
// (lensm_axis, 1622-1628, with no axis set). nodes: the layout's node lattice (nn a side). lens out: K, ax, ay, R,
// then the 11 coefficients. Returns 1 where a model fits, else 0.
int orc_lens_fit(int span, int iw, int ih, const float *H, const uint8_t *ok, const float *adx, const float *ady, double *lens) {
  const int a = span / 64;
  float nodes[40];
  const int nn = orc_layout_nodes(span + 2 * MARGIN, nodes);
  const double ax = iw * 0.5f, ay = ih * 0.5f;
  double R = 0;
  for (int c = 0; c < 4; c++) { const double d = hypot((c & 1 ? iw : 0) - ax, (c & 2 ? ih : 0) - ay); if (d > R) R = d; }
  if (!(R > 0)) R = 1;
  double qx[ANK * ANK + 4], qy[ANK * ANK + 4], dx[ANK * ANK + 4], dy[ANK * ANK + 4];
  int np = 0;
  for (int c = 0; c < 4; c++) {
    float u, v;
    project(H, nodes[(c == 1 || c == 2) ? nn - 1 : 0], nodes[c >= 2 ? nn - 1 : 0], &u, &v);
    qx[np] = (u - ax) / R; qy[np] = (v - ay) / R; dx[np] = 0; dy[np] = 0; np++;
  }
  for (int k = 0; k < ANK * ANK; k++) {
    if (!ok[k]) continue;
    const float X = (float)anchor_m0(span, k % ANK) + a * 0.5f, Y = (float)anchor_m0(span, k / ANK) + a * 0.5f;
    float u, v;
    project(H, X, Y, &u, &v);
    qx[np] = (u - ax) / R; qy[np] = (v - ay) / R; dx[np] = adx[k]; dy[np] = ady[k]; np++;
  }
  double A3[LENSP][LENSP + 1], rx[LENSP], ry[LENSP];
  memset(A3, 0, sizeof A3);
  for (int i = 0; i < np; i++) {
    lens_rows(qx[i], qy[i], 3, rx, ry);
    for (int p = 0; p < LENSP; p++) {
      for (int q = p; q < LENSP; q++) A3[p][q] += rx[p] * rx[q] + ry[p] * ry[q];
      A3[p][LENSP] += rx[p] * dx[i] + ry[p] * dy[i];
    }
  }
  for (int p = 1; p < LENSP; p++) for (int q = 0; q < p; q++) A3[p][q] = A3[q][p];
  double best = INFINITY, tb[LENSP] = {0};
  int K = -1;
  for (int k = 0; k <= 3; k++) {
    const int p = 8 + k;
    double A[LENSP][LENSP + 1];
    memcpy(A, A3, sizeof A);
    for (int c = 0; c < p; c++) A[c][c] += 1e-12;
    if (2 * np - p - 1 <= 0 || !solve_lens(A, p)) continue;
    double t[LENSP] = {0}, rss = 0;
    for (int c = 0; c < p; c++) t[c] = A[c][LENSP] / A[c][c];
    for (int i = 0; i < np; i++) {
      lens_rows(qx[i], qy[i], k, rx, ry);
      double fx = 0, fy = 0;
      for (int c = 0; c < p; c++) { fx += t[c] * rx[c]; fy += t[c] * ry[c]; }
      rss += (dx[i] - fx) * (dx[i] - fx) + (dy[i] - fy) * (dy[i] - fy);
    }
    const double n2 = 2.0 * np, aicc = n2 * log(rss / n2 + 1e-30) + 2.0 * p + 2.0 * p * (p + 1) / (n2 - p - 1);
    if (aicc < best) { best = aicc; K = k; memcpy(tb, t, sizeof tb); }
  }
  if (K < 0) return 0;
  lens[0] = K; lens[1] = ax; lens[2] = ay; lens[3] = R;
  for (int c = 0; c < LENSP; c++) lens[4 + c] = tb[c];
  return 1;
}

// ---------------------------------------------------------------- the border nodes (acquire.c:839-859, 1205-1374)

enum { NCORNER = 12, NRESERVE = 15, FB = 18, NMAXN = 40 };
static const float NODE_NONE = -2.0f;

// The layout's cell kinds with the format word's cells flagged (liblizard/src/layout.c:69-141): 2 dark, 1 light, 0
// the picture's, | 8 on a word cell.
static void mesh_kind(int span, unsigned char *kind) {
  const int side = span + 2 * MARGIN;
  for (int y = 0; y < side; y++)
    for (int x = 0; x < side; x++) {
      const int dx = x < side - 1 - x ? x : side - 1 - x, dy = y < side - 1 - y ? y : side - 1 - y, d = dx < dy ? dx : dy;
      unsigned char k;
      if (dx < NCORNER && dy < NCORNER) {
        const int in = dx >= 1 && dx <= NCORNER - 2 && dy >= 1 && dy <= NCORNER - 2, cd = dx < dy ? dx : dy;
        k = in && !(cd >= 3 && cd < 5) ? 2 : 1;
      } else {
        int dark = d >= 1 && d <= 2;
        if (d >= 5 && d < 7) {
          const int along = dy <= dx ? x : y, sd = dy <= dx ? (y < side / 2 ? 0 : 2) : (x < side / 2 ? 3 : 1);
          const int cell = (along - NRESERVE) / 2, run = cell / 4;
          if (along >= NRESERVE && along < side - NRESERVE && !(run & 1)) dark = orc_thin_track(sd, run / 2 * 4 + cell % 4);
        }
        k = d >= MARGIN - 3 ? 0 : dark ? 2 : 1;
      }
      kind[y * side + x] = k;
    }
  const int cells = orc_fmt_side_cells(side, NRESERVE);
  for (int sd = 0; sd < 4; sd++)
    for (int i = 0; i < cells; i++) {
      const int off = ((i / 4) * 8 + i % 4 + 4) * 2;
      for (int j = 0; j < 2; j++)
        for (int e = 0; e < 2; e++) {
          const int t = NRESERVE + off + j, dd = 5 + e;
          const int x = sd == 0 || sd == 2 ? t : sd == 3 ? dd : side - 1 - dd, y = sd == 0 ? dd : sd == 2 ? side - 1 - dd : t;
          kind[y * side + x] = 1 | 8;   // the word painted blank: only the flag matters to the templates
        }
    }
}

static int in_capture(int w, int h, float u, float v) { return u >= 0.5f && u <= w - 0.5f && v >= 0.5f && v <= h - 0.5f; }

static int node_inside(int w, int h, const float *H, int cx0, int cy0, const int *r, float pdx, float pdy, float ax, float bx, float ay, float by) {
  const float x0 = cx0 + r[0] + 0.5f + ax, x1 = cx0 + r[1] - 0.5f + bx, y0 = cy0 + r[2] + 0.5f + ay, y1 = cy0 + r[3] - 0.5f + by;
  for (int c = 0; c < 4; c++) {
    const float x = c & 1 ? x1 : x0, y = c & 2 ? y1 : y0;
    float u, v;
    if (!(H[6] * x + H[7] * y + 1 > 0)) return 0;
    project(H, x, y, &u, &v);
    if (!(u + pdx >= 1.5f && u + pdx <= w - 1.5f && v + pdy >= 1.5f && v + pdy <= h - 1.5f)) return 0;
  }
  return 1;
}

typedef struct { float dx, dy, score; int done; } onode_t;
typedef struct { const unsigned char *kind; int side, nn; const float *pos; } omesh_t;

// The template's correlation with the node shifted (ox, oy) modules (acquire.c:1205-1238, the scalar build).
static float node_ncc(const omesh_t *M, const uint8_t *px, int w, int h, int cx0, int cy0, const int *r, const float *H, float pdx, float pdy,
                      float ox, float oy, int edge, int nmin) {
  float st = 0, ss = 0, stt = 0, sss = 0, sts = 0;
  int n = 0, nin = 0;
  const int lo = r[0], hi = r[1], ylo = r[2], yhi = r[3], side = hi - lo;
  float S[FB * FB];
  for (int dy = ylo; dy < yhi; dy++) {
    const float my = cy0 + dy + 0.5f + oy;
    for (int dx = lo; dx < hi; dx++) {
      const float mx = cx0 + dx + 0.5f + ox;
      float u, v;
      project(H, mx, my, &u, &v);
      S[(dy - ylo) * side + dx - lo] = sample(px, w, h, u + pdx, v + pdy);
    }
  }
  for (int dy = ylo; dy < yhi; dy++)
    for (int dx = lo; dx < hi; dx++) {
      const int kind = M->kind[(cy0 + dy) * M->side + cx0 + dx];
      if (kind == 0 || (kind & 8)) continue;
      if (edge) {
        float u, v;
        project(H, cx0 + dx + 0.5f + ox, cy0 + dy + 0.5f + oy, &u, &v);
        nin += in_capture(w, h, u + pdx, v + pdy);
      }
      const float t = (kind & 3) == 2 ? -1.0f : 1.0f, s = S[(dy - ylo) * side + dx - lo];
      st += t; ss += s; stt += t * t; sss += s * s; sts += t * s; n++;
    }
  if (edge && nin < nmin) return NODE_NONE;
  const float vt = stt - st * st / n, vs = sss - ss * ss / n;
  if (vt <= 0 || vs <= 1e-9f) return 0;
  return (sts - st * ss / n) / sqrtf(vt * vs);
}

// One node's refinement (acquire.c:1242-1374 refine_node, the scalar build): the prior from the measured neighbours
// (less the lens model's part, then the model's at the node), a coarse search over 7 x 7 half-module offsets read off
// one grid of samples, then two passes of 3 x 3 searches at a quarter and an eighth of a module, a parabola each way.
static void refine_node(const omesh_t *M, const uint8_t *px, int w, int h, const float *H, int i, int j, onode_t *nodes, const double *lens) {
  const int nn = M->nn, cx0 = (int)M->pos[i], cy0 = (int)M->pos[j];
  const float mcx = cx0 + 0.5f, mcy = cy0 + 0.5f;
  int rect[4];
  {
    int ex = (j == 0 || j == nn - 1) ? 6 : 2, ey = (i == 0 || i == nn - 1) ? 6 : 2;
    if (ex == 6 && ey == 6) { ex = NCORNER - 1 < FB - 3 ? NCORNER - 1 : FB - 3; ey = ex; }
    rect[0] = -ex < -cx0 ? -cx0 : -ex; rect[1] = ex + 1 > M->side - cx0 ? M->side - cx0 : ex + 1;
    rect[2] = -ey < -cy0 ? -cy0 : -ey; rect[3] = ey + 1 > M->side - cy0 ? M->side - cy0 : ey + 1;
  }
  float pdx = 0, pdy = 0;
  int pn = 0;
  for (int dj = -1; dj <= 1; dj++)
    for (int di = -1; di <= 1; di++) {
      const int ii = i + di, jj = j + dj;
      if (ii < 0 || jj < 0 || ii >= nn || jj >= nn || !nodes[jj * nn + ii].done) continue;
      float rx = nodes[jj * nn + ii].dx, ry = nodes[jj * nn + ii].dy;
      if (lens) { float u, v, mx, my; project(H, M->pos[ii], M->pos[jj], &u, &v); lens_at(lens, u, v, &mx, &my); rx -= mx; ry -= my; }
      pdx += rx; pdy += ry; pn++;
    }
  if (pn) { pdx /= pn; pdy /= pn; }
  if (lens) { float u, v, mx, my; project(H, M->pos[i], M->pos[j], &u, &v); lens_at(lens, u, v, &mx, &my); pdx += mx; pdy += my; }
  const int edge = !node_inside(w, h, H, cx0, cy0, rect, pdx, pdy, -1.5f, 1.5f, -1.5f, 1.5f);
  float ppx, ppy, ax, ay, bx, by;
  project(H, mcx, mcy, &ppx, &ppy); project(H, mcx + 1, mcy, &ax, &ay); project(H, mcx, mcy + 1, &bx, &by);
  const float jxx = ax - ppx, jxy = ay - ppy, jyx = bx - ppx, jyy = by - ppy;
  enum { GMAX = 2 * FB + 5 };
  float G[GMAX * GMAX + 8], GM[GMAX * GMAX + 8], tv[FB * FB];
  int at[FB * FB], cells = 0;
  const int lo = rect[0], ylo = rect[2], side = rect[1] - rect[0], tall = rect[3] - rect[2], GW = 2 * side + 5, GH = 2 * tall + 5;
  for (int gy = 0; gy < GH; gy++) {
    const float my = (float)(2 * (cy0 + ylo) + gy - 2) * 0.5f;
    for (int gx = 0; gx < GW; gx++) {
      const float mx = (float)(2 * (cx0 + lo) + gx - 2) * 0.5f;
      float u, v;
      project(H, mx, my, &u, &v);
      G[gy * GW + gx] = sample(px, w, h, u + pdx, v + pdy);
      GM[gy * GW + gx] = !edge || in_capture(w, h, u + pdx, v + pdy) ? 1.0f : 0;
    }
  }
  float st = 0, stt = 0;
  for (int dy = 0; dy < tall; dy++)
    for (int dx = 0; dx < side; dx++) {
      const int kind = M->kind[(cy0 + ylo + dy) * M->side + cx0 + lo + dx];
      if (kind == 0 || (kind & 8)) continue;
      tv[cells] = (kind & 3) == 2 ? -1.0f : 1.0f;
      at[cells] = (2 * dy + 3) * GW + 2 * dx + 3;
      st += tv[cells]; stt += tv[cells] * tv[cells]; cells++;
    }
  const float vt = stt - st * st / cells;
  const int nmin = (cells + 1) / 2;
  float best = NODE_NONE, box = 0, boy = 0;
  for (int k = 0; k < 4; k++) G[GW * GH + k] = GM[GW * GH + k] = 0;
  for (int b = -3; b <= 3; b++)
    for (int a = -3; a <= 3; a++) {
      const float *g0 = G + b * GW + a, *m0 = GM + b * GW + a;
      float ss = 0, sss = 0, sts = 0, sn = 0;
      for (int k = 0; k < cells; k++) { const float v = g0[at[k]]; ss += v; sss += v * v; sts += tv[k] * v; }
      if (edge) for (int k = 0; k < cells; k++) sn += m0[at[k]];
      const float vs = sss - ss * ss / cells;
      const float sc = edge && sn < nmin ? NODE_NONE : vt <= 0 || vs <= 1e-9f ? 0 : (sts - st * ss / cells) / sqrtf(vt * vs);
      if (sc > best) { best = sc; box = a * 0.5f; boy = b * 0.5f; }
    }
  float g[3][3], step = 0.25f;
  int have[3][3] = {{0}}, ma = 1, mb = 1;
  g[1][1] = best; have[1][1] = 1;
  for (int pass = 0; pass < 2; pass++, step *= 0.5f) {
    for (int move = 0; move < 8; move++) {
      if (ma != 1 || mb != 1) {
        float ng[3][3];
        int nh[3][3];
        for (int b2 = 0; b2 < 3; b2++)
          for (int a2 = 0; a2 < 3; a2++) {
            const int sb = b2 + mb - 1, sa = a2 + ma - 1, in = sb >= 0 && sb < 3 && sa >= 0 && sa < 3;
            nh[b2][a2] = in && have[sb][sa];
            ng[b2][a2] = in ? g[sb][sa] : 0;
          }
        memcpy(g, ng, sizeof g); memcpy(have, nh, sizeof have); ma = mb = 1;
      }
      const int ce = !node_inside(w, h, H, cx0, cy0, rect, pdx, pdy, box - step, box + step, boy - step, boy + step);
      for (int b2 = -1; b2 <= 1; b2++)
        for (int a2 = -1; a2 <= 1; a2++)
          if (!have[b2 + 1][a2 + 1]) {
            g[b2 + 1][a2 + 1] = node_ncc(M, px, w, h, cx0, cy0, rect, H, pdx, pdy, box + a2 * step, boy + b2 * step, ce, nmin);
            have[b2 + 1][a2 + 1] = 1;
          }
      int ba = 1, bb = 1;
      for (int b2 = 0; b2 < 3; b2++) for (int a2 = 0; a2 < 3; a2++) if (g[b2][a2] > g[bb][ba]) { ba = a2; bb = b2; }
      if (ba == 1 && bb == 1) break;
      box += (ba - 1) * step; boy += (bb - 1) * step; ma = ba; mb = bb;
    }
    if (pass == 0) {
      const float c = g[mb][ma];
      memset(have, 0, sizeof have); g[1][1] = c; have[1][1] = 1; ma = mb = 1;
    }
  }
  best = g[1][1];
  const float dxx = g[1][0] - 2 * g[1][1] + g[1][2], dyy = g[0][1] - 2 * g[1][1] + g[2][1];
  if (dxx < -1e-6f && g[1][0] > NODE_NONE && g[1][2] > NODE_NONE) box += 0.125f * 0.5f * (g[1][0] - g[1][2]) / dxx;
  if (dyy < -1e-6f && g[0][1] > NODE_NONE && g[2][1] > NODE_NONE) boy += 0.125f * 0.5f * (g[0][1] - g[2][1]) / dyy;
  onode_t *nd = &nodes[j * nn + i];
  nd->done = 1; nd->score = best;
  if (best < 0.35f) { nd->dx = pdx; nd->dy = pdy; return; }
  nd->dx = pdx + box * jxx + boy * jyx;
  nd->dy = pdy + box * jxy + boy * jyy;
}

// The border nodes of a frame through H (and the lens model, or NULL): corners as measured, the marked nodes in rings
// outward from the corners (acquire.c:5044-5058). nodes_out: nn * nn x (dx, dy, score, done). Returns nn.
int orc_border_nodes(int span, const uint8_t *px, int w, int h, const float *H, const double *lens, float *nodes_out) {
  const int side = span + 2 * MARGIN;
  unsigned char *kind = malloc((size_t)side * side);
  float pos[NMAXN];
  const int nn = orc_layout_nodes(side, pos);
  onode_t *nodes = calloc((size_t)nn * nn, sizeof(onode_t));
  if (!kind || !nodes) { free(kind); free(nodes); return -1; }
  mesh_kind(span, kind);
  const omesh_t M = {kind, side, nn, pos};
  for (int c = 0; c < 4; c++) nodes[((c >= 2) ? nn - 1 : 0) * nn + ((c == 1 || c == 2) ? nn - 1 : 0)].done = 1;
  int order[4 * NMAXN], no = 0;
  for (int ring = 0; ring <= nn; ring++)   // ring by ring, rows within a ring
    for (int j = 0; j < nn; j++)
      for (int i = 0; i < nn; i++) {
        const int ex = i == 0 || i == nn - 1, ey = j == 0 || j == nn - 1;
        if (!((ex || ey) && !(ex && ey))) continue;
        const int r = (i < nn - 1 - i ? i : nn - 1 - i) + (j < nn - 1 - j ? j : nn - 1 - j);
        if (r == ring) order[no++] = j * nn + i;
      }
  for (int k = 0; k < no; k++) {
    if (nodes[order[k]].done) continue;
    refine_node(&M, px, w, h, H, order[k] % nn, order[k] / nn, nodes, lens);
  }
  for (int k = 0; k < nn * nn; k++) {
    nodes_out[4 * k] = nodes[k].dx; nodes_out[4 * k + 1] = nodes[k].dy; nodes_out[4 * k + 2] = nodes[k].score; nodes_out[4 * k + 3] = (float)nodes[k].done;
  }
  free(kind); free(nodes);
  return nn;
}

// ---------------------------------------------------------------- the anchors' registration (acquire.c:2039-2197)

// lensm_fit (liblizard/src/acquire.c:1630-1694) about the axis (ax, ay) and scale R: the normal equations over the
// points not dropped, summed once in the points' order; every model of 0..3 radial terms solved, the least AICc
// kept. With isb (the points the robust rule judges), up to three more rounds: each judged point's distance from the
// model, tau = max(tau_floor, 3 x 1.4826 x their median), a point further than tau dropped, the model fitted again
// until no verdict changes. lens out as lens_at takes it. Returns 1 where a model fitted.
static int cmp_dbl(const void *a, const void *b) { const double x = *(const double *)a, y = *(const double *)b; return (x > y) - (x < y); }
static int lensm_fit_o(int np, const double *qx, const double *qy, const double *dx, const double *dy, const unsigned char *isb,
                       unsigned char *drop, double tau_floor, double ax, double ay, double R, double *lens) {
  int ok = 0;
  lens[1] = ax; lens[2] = ay; lens[3] = R;
  for (int round = 0; round < 4; round++) {
    double A3[LENSP][LENSP + 1], rx[LENSP], ry[LENSP], best = INFINITY, tb[LENSP] = {0};
    memset(A3, 0, sizeof A3);
    int n = 0, K = -1;
    for (int i = 0; i < np; i++) {
      if (drop[i]) continue;
      n++;
      lens_rows(qx[i], qy[i], 3, rx, ry);
      for (int p = 0; p < LENSP; p++) {
        for (int q = p; q < LENSP; q++) A3[p][q] += rx[p] * rx[q] + ry[p] * ry[q];
        A3[p][LENSP] += rx[p] * dx[i] + ry[p] * dy[i];
      }
    }
    for (int p = 1; p < LENSP; p++) for (int q = 0; q < p; q++) A3[p][q] = A3[q][p];
    for (int k = 0; k <= 3; k++) {
      const int p = 8 + k;
      double A[LENSP][LENSP + 1];
      memcpy(A, A3, sizeof A);
      for (int c = 0; c < p; c++) A[c][c] += 1e-12;
      if (2 * n - p - 1 <= 0 || !solve_lens(A, p)) continue;
      double t[LENSP] = {0}, rss = 0;
      for (int c = 0; c < p; c++) t[c] = A[c][LENSP] / A[c][c];
      for (int i = 0; i < np; i++) {
        if (drop[i]) continue;
        lens_rows(qx[i], qy[i], k, rx, ry);
        double fx = 0, fy = 0;
        for (int c = 0; c < p; c++) { fx += t[c] * rx[c]; fy += t[c] * ry[c]; }
        rss += (dx[i] - fx) * (dx[i] - fx) + (dy[i] - fy) * (dy[i] - fy);
      }
      const double n2 = 2.0 * n, aicc = n2 * log(rss / n2 + 1e-30) + 2.0 * p + 2.0 * p * (p + 1) / (n2 - p - 1);
      if (aicc < best) { best = aicc; K = k; memcpy(tb, t, sizeof tb); }
    }
    if (K < 0) break;
    lens[0] = K;
    for (int c = 0; c < LENSP; c++) lens[4 + c] = tb[c];
    ok = 1;
    if (!isb || round == 3) break;
    double res[ANK * ANK + 4], srt[ANK * ANK + 4];
    int nb = 0, changed = 0;
    for (int i = 0; i < np; i++) {
      if (!isb[i]) continue;
      float fx, fy;
      lens_at(lens, qx[i] * R + ax, qy[i] * R + ay, &fx, &fy);
      res[nb++] = hypot(dx[i] - fx, dy[i] - fy);
    }
    if (!nb) break;
    memcpy(srt, res, (size_t)nb * sizeof(double));
    qsort(srt, (size_t)nb, sizeof(double), cmp_dbl);
    const double tau = fmax(tau_floor, 3 * 1.4826 * srt[nb / 2]);
    for (int i = 0, b = 0; i < np; i++) {
      if (!isb[i]) continue;
      const unsigned char bad = res[b++] > tau;
      if (bad != drop[i]) { drop[i] = bad; changed++; }
    }
    if (!changed) break;
  }
  return ok;
}

// The homography through the anchors found (liblizard/src/acquire.c:2062-2094 anchor_homo): least squares with
// h33 = 1 on coordinates centred and scaled by their mean distance over sqrt 2; 0 where fewer than eight anchors or
// fewer than three of the grid's rows or columns hold them.
static int anchor_homo_o(int span, const uint8_t *ok, const float *u, const float *v, float *H) {
  const int a = span / 64;
  int n = 0, rows = 0, cols = 0, rm = 0, cm = 0;
  double mx = 0, my = 0, mu = 0, mv = 0;
  float X[ANK * ANK], Y[ANK * ANK];
  for (int k = 0; k < ANK * ANK; k++) {
    X[k] = (float)anchor_m0(span, k % ANK) + a * 0.5f; Y[k] = (float)anchor_m0(span, k / ANK) + a * 0.5f;
    if (ok[k]) { n++; mx += X[k]; my += Y[k]; mu += u[k]; mv += v[k]; rm |= 1 << (k / ANK); cm |= 1 << (k % ANK); }
  }
  for (int b = 0; b < ANK; b++) { rows += (rm >> b) & 1; cols += (cm >> b) & 1; }
  if (n < 8 || rows < 3 || cols < 3) return 0;
  mx /= n; my /= n; mu /= n; mv /= n;
  double sx = 0, su = 0;
  for (int k = 0; k < ANK * ANK; k++) if (ok[k]) { sx += hypot(X[k] - mx, Y[k] - my); su += hypot(u[k] - mu, v[k] - mv); }
  sx = sx / n / 1.4142135623730951; su = su / n / 1.4142135623730951;
  if (!(sx > 0) || !(su > 0)) return 0;
  double M[LENSP][LENSP + 1];
  memset(M, 0, sizeof M);
  for (int k = 0; k < ANK * ANK; k++) {
    if (!ok[k]) continue;
    const double x = (X[k] - mx) / sx, y = (Y[k] - my) / sx, uu = (u[k] - mu) / su, vv = (v[k] - mv) / su;
    const double r0[8] = {x, y, 1, 0, 0, 0, -uu * x, -uu * y}, r1[8] = {0, 0, 0, x, y, 1, -vv * x, -vv * y};
    for (int p = 0; p < 8; p++) { for (int q = 0; q < 8; q++) M[p][q] += r0[p] * r0[q] + r1[p] * r1[q]; M[p][LENSP] += r0[p] * uu + r1[p] * vv; }
  }
  if (!solve_lens(M, 8)) return 0;
  double g[9];
  for (int p = 0; p < 8; p++) g[p] = M[p][LENSP] / M[p][p];
  g[8] = 1;
  const double tx[9] = {1 / sx, 0, -mx / sx, 0, 1 / sx, -my / sx, 0, 0, 1}, ti[9] = {su, 0, mu, 0, su, mv, 0, 0, 1};
  double gt[9], h[9];
  for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) { gt[3 * r + c] = 0; for (int k = 0; k < 3; k++) gt[3 * r + c] += g[3 * r + k] * tx[3 * k + c]; }
  for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) { h[3 * r + c] = 0; for (int k = 0; k < 3; k++) h[3 * r + c] += ti[3 * r + k] * gt[3 * k + c]; }
  if (!(fabs(h[8]) > 1e-12)) return 0;
  for (int k = 0; k < 9; k++) H[k] = (float)(h[k] / h[8]);
  return 1;
}

// The homography through four point pairs (liblizard/src/acquire.c:611-654 solve8 / homography, the portable form).
static int homography_o(const float *src, const float *dst, float *H) {
  double A[8][9];
  for (int i = 0; i < 4; i++) {
    const double x = src[2 * i], y = src[2 * i + 1], u = dst[2 * i], v = dst[2 * i + 1];
    const double r0[9] = {x, y, 1, 0, 0, 0, -u * x, -u * y, u}, r1[9] = {0, 0, 0, x, y, 1, -v * x, -v * y, v};
    memcpy(A[2 * i], r0, sizeof r0); memcpy(A[2 * i + 1], r1, sizeof r1);
  }
  for (int c = 0; c < 8; c++) {
    int p = c;
    for (int r = c + 1; r < 8; r++) if (fabs(A[r][c]) > fabs(A[p][c])) p = r;
    if (fabs(A[p][c]) < 1e-12) return 0;
    for (int k = 0; k < 9; k++) { const double t = A[c][k]; A[c][k] = A[p][k]; A[p][k] = t; }
    for (int r = 0; r < 8; r++) {
      if (r == c) continue;
      const double f = A[r][c] / A[c][c];
      for (int k = c; k < 9; k++) A[r][k] -= f * A[c][k];
    }
  }
  for (int i = 0; i < 8; i++) H[i] = (float)(A[i][8] / A[i][i]);
  H[8] = 1;
  return 1;
}

// The code registered from the anchors (liblizard/src/acquire.c:2128-2197 anchor_register): rounds of the anchor
// search (at most six) through the homography the anchors found so far say (anchor_homo) and the lens model they say
// about it, held to the robust rule (anchor_model_free, :2101-2118: a reading further from the model than half a
// module, mpx / 2 px, or three robust spreads, no longer found), until a round finds nothing new; then each corner
// judged by that map (further than 3 modules off, searched again through the border node search on rim from where
// the joint model of the anchors and the kept corners puts it, kept where it correlates 0.35 or more, else the
// model's place, and H made again from the four); then the anchors' model about H (anchor_model). px: the frame
// (the anchor search's), rim: the border search's image (the frame, or its border blur; NULL: the frame), both w x h. H: in the
// corners' homography, out the registration's; quad: the corners as the finder measured them (in, and out as moved);
// mpx: pixels a module. Out per anchor: ok, peak, dx, dy (about H), u, v; lens: the model about H. Returns 1 where
// the registration holds (OB_ANCH_MIN = 12 anchors or more and a model), else 0 (H, quad unchanged).
int orc_anchor_register(int span, const uint8_t *px, const uint8_t *rim, int w, int h, float *H, float *quad, float mpx, uint8_t *ok,
                        float *peak, float *adx, float *ady, float *au, float *av, double *lens) {
  enum { NA = ANK * ANK, ROUNDS = 6, AMIN = 12, CORNER = 3 };
  const int side = span + 2 * MARGIN;
  float pos[NMAXN];
  const int nn = orc_layout_nodes(side, pos);
  const double ax = w * 0.5f, ay = h * 0.5f;
  double R = 0;
  for (int c = 0; c < 4; c++) { const double d = hypot((c & 1 ? w : 0) - ax, (c & 2 ? h : 0) - ay); if (d > R) R = d; }
  if (!(R > 0)) R = 1;
  float Ha[9], H0[9];
  memcpy(Ha, H, sizeof Ha); memcpy(H0, H, sizeof H0);
  double mf[4 + LENSP];
  int have = 0, nf = 0;
  for (int k = 0; k < NA; k++) { ok[k] = 0; peak[k] = adx[k] = ady[k] = au[k] = av[k] = 0; }
  const int a = span / 64;
  float X[NA], Y[NA];
  for (int k = 0; k < NA; k++) { X[k] = (float)anchor_m0(span, k % ANK) + a * 0.5f; Y[k] = (float)anchor_m0(span, k / ANK) + a * 0.5f; }
  for (int round = 0; round < ROUNDS; round++) {
    uint8_t ok_in[NA], ok2[NA];
    float pk2[NA], dx2[NA], dy2[NA], u2[NA], v2[NA];
    memcpy(ok_in, ok, NA);
    const int now = orc_anchor_find(span, px, w, h, Ha, have ? mf : NULL, ok_in, ok2, pk2, dx2, dy2, u2, v2);
    for (int k = 0; k < NA; k++)
      if (!ok_in[k]) { ok[k] = ok2[k]; peak[k] = pk2[k]; adx[k] = dx2[k]; ady[k] = dy2[k]; au[k] = u2[k]; av[k] = v2[k]; }
    if (now == nf || now < 4) break;
    nf = now;
    float Hn[9];
    if (anchor_homo_o(span, ok, au, av, Hn)) memcpy(Ha, Hn, sizeof Ha);
    // anchor_model_free: the anchors' displacements about Ha, the robust rule at half a module
    double qx[NA], qy[NA], dx[NA], dy[NA];
    unsigned char drop[NA] = {0}, isb[NA];
    int np = 0, at[NA];
    memset(isb, 1, sizeof isb);
    for (int k = 0; k < NA; k++) {
      if (!ok[k]) continue;
      float hu, hv;
      project(Ha, X[k], Y[k], &hu, &hv);
      adx[k] = au[k] - hu; ady[k] = av[k] - hv;
      qx[np] = (hu - ax) / R; qy[np] = (hv - ay) / R; dx[np] = adx[k]; dy[np] = ady[k]; at[np] = k; np++;
    }
    have = np >= 4 && lensm_fit_o(np, qx, qy, dx, dy, isb, drop, 0.5 * mpx, ax, ay, R, mf);
    if (!have) break;
    for (int i = 0; i < np; i++) if (drop[i]) ok[at[i]] = 0;
    nf = 0;
    for (int k = 0; k < NA; k++) nf += ok[k];
  }
  if (!have || nf < AMIN) return 0;
  // the anchors and the corners about the corners' H; each corner judged by the anchors' own map
  double qx[NA + 4], qy[NA + 4], dx[NA + 4], dy[NA + 4], mc[4 + LENSP];
  unsigned char drop[NA + 4] = {0};
  int np = 4;
  for (int c = 0; c < 4; c++) {
    float u, v;
    project(H0, pos[(c == 1 || c == 2) ? nn - 1 : 0], pos[c >= 2 ? nn - 1 : 0], &u, &v);
    qx[c] = (u - ax) / R; qy[c] = (v - ay) / R; dx[c] = dy[c] = 0;
  }
  for (int k = 0; k < NA; k++) {
    if (!ok[k]) continue;
    float hu, hv;
    project(H0, X[k], Y[k], &hu, &hv);
    qx[np] = (hu - ax) / R; qy[np] = (hv - ay) / R; dx[np] = au[k] - hu; dy[np] = av[k] - hv; np++;
  }
  for (int c = 0; c < 4; c++) {
    float pu, pv, mu, mv;
    project(Ha, pos[(c == 1 || c == 2) ? nn - 1 : 0], pos[c >= 2 ? nn - 1 : 0], &pu, &pv);
    lens_at(mf, pu, pv, &mu, &mv);
    drop[c] = hypotf(pu + mu - quad[2 * c], pv + mv - quad[2 * c + 1]) > CORNER * mpx;
  }
  const int fit = lensm_fit_o(np, qx, qy, dx, dy, NULL, drop, 0, ax, ay, R, mc);
  const float src[8] = {pos[0], pos[0], pos[nn - 1], pos[0], pos[nn - 1], pos[nn - 1], pos[0], pos[nn - 1]};
  int moved = 0;
  if (fit) {
    unsigned char *kind = malloc((size_t)side * side);
    onode_t *nodes = calloc((size_t)nn * nn, sizeof(onode_t));
    if (!kind || !nodes) { free(kind); free(nodes); return -1; }
    mesh_kind(span, kind);
    const omesh_t M = {kind, side, nn, pos};
    for (int c = 0; c < 4; c++) nodes[((c >= 2) ? nn - 1 : 0) * nn + ((c == 1 || c == 2) ? nn - 1 : 0)].done = 1;
    for (int c = 0; c < 4; c++) {
      if (!drop[c]) continue;
      const int i = (c == 1 || c == 2) ? nn - 1 : 0, j = c >= 2 ? nn - 1 : 0;
      float hu, hv, mu, mv;
      project(H0, pos[i], pos[j], &hu, &hv);
      lens_at(mc, hu, hv, &mu, &mv);
      onode_t *nd = &nodes[j * nn + i];
      nd->done = 0;
      refine_node(&M, rim ? rim : px, w, h, H0, i, j, nodes, mc);
      if (nd->score >= 0.35f) { quad[2 * c] = hu + nd->dx; quad[2 * c + 1] = hv + nd->dy; }
      else { quad[2 * c] = hu + mu; quad[2 * c + 1] = hv + mv; }
      moved++;
    }
    free(kind); free(nodes);
  }
  float Hc[9];
  if (moved && homography_o(src, quad, Hc)) memcpy(H, Hc, 9 * sizeof(float));
  for (int k = 0; k < NA; k++) if (ok[k]) { float hu, hv; project(H, X[k], Y[k], &hu, &hv); adx[k] = au[k] - hu; ady[k] = av[k] - hv; }
  return orc_lens_fit(span, w, h, H, ok, adx, ady, lens);
}

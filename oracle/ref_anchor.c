// Harness around the reference's anchor search (liblizard/src/acquire.c:1876-2036 anchor_find), compiled from the
// reference's own sources where they lie. TEST INFRASTRUCTURE ONLY: oracle/Makefile builds it into the reference's
// portable build (-DOB_SCALAR: the scalar twins of the SIMD paths), oracle/_ref/libref_scalar.so, where the
// reference tree is present, so that the tests can hold the anchor search's restatement and the GPU kernel to the
// reference's own outputs. anchor_find is private to acquire.c, so the harness compiles acquire.c in.
#include "acquire.c"

// One frame's search: the format's ring span (modules), the frame (w x h greys, rows w apart), H (module -> image,
// 9 floats), the lens model (NULL for none: K, ax, ay, R, then the LENS_P coefficients) and the anchors already
// found (ok_in, 49 flags or NULL, row-major j * 7 + i). Out per anchor: ok, peak, dx, dy, u, v (the fields
// anchor_find leaves; an anchor found before keeps zeros here). Returns the anchors ok, or -1.
int refs_anchor_find(int span, const uint8_t *px, int w, int h, const float *H9, const double *lens, const uint8_t *ok_in,
                     uint8_t *ok, float *peak, float *dx, float *dy, float *u, float *v) {
  ob_layout_t L;
  if (ob_layout_init(&L, span + 2 * OB_MARGIN)) return -1;
  image_t im;
  ob_image_init(&im, px, w, h, 1.0f);
  homo_t H;
  memcpy(H.h, H9, sizeof H.h);
  lensm_t lm;
  memset(&lm, 0, sizeof lm);
  if (lens) {
    lm.K = (int)lens[0]; lm.ax = lens[1]; lm.ay = lens[2]; lm.R = lens[3];
    for (int a = 0; a < LENS_P; a++) lm.t[a] = lens[4 + a];
  }
  anchor_t A[OB_ANCH_K * OB_ANCH_K];
  memset(A, 0, sizeof A);
  for (int k = 0; k < OB_ANCH_K * OB_ANCH_K; k++) A[k].ok = ok_in ? ok_in[k] : 0;
  const int found = anchor_find(&L, &im, &H, lens ? &lm : NULL, A);
  for (int k = 0; k < OB_ANCH_K * OB_ANCH_K; k++) {
    ok[k] = (uint8_t)A[k].ok; peak[k] = A[k].peak; dx[k] = A[k].dx; dy[k] = A[k].dy; u[k] = A[k].u; v[k] = A[k].v;
  }
  ob_layout_free(&L);
  return found;
}

// The lens model's coefficient count (LENS_P) and the anchors' grid (OB_ANCH_K), for the caller's buffers.
int refs_lens_p(void) { return LENS_P; }

// The lens model the reference fits from the anchors about H (liblizard/src/acquire.c:2038-2055 anchor_model), for a
// frame of iw x ih pixels: ok, dx, dy per anchor (row-major j * 7 + i). lens out: K, ax, ay, R, then the LENS_P
// coefficients. Returns 1 where a model fits, else 0.
int refs_anchor_model(int span, int iw, int ih, const float *H9, const uint8_t *ok, const float *dx, const float *dy, double *lens) {
  ob_layout_t L;
  if (ob_layout_init(&L, span + 2 * OB_MARGIN)) return -1;
  homo_t H;
  memcpy(H.h, H9, sizeof H.h);
  const int a = ob_anchor_side(&L);
  anchor_t A[OB_ANCH_K * OB_ANCH_K];
  memset(A, 0, sizeof A);
  for (int j = 0; j < OB_ANCH_K; j++)
    for (int i = 0; i < OB_ANCH_K; i++) {
      anchor_t *an = &A[j * OB_ANCH_K + i];
      an->X = (float)ob_anchor_m0(&L, i) + a * 0.5f; an->Y = (float)ob_anchor_m0(&L, j) + a * 0.5f;
      an->ok = ok[j * OB_ANCH_K + i]; an->dx = dx[j * OB_ANCH_K + i]; an->dy = dy[j * OB_ANCH_K + i];
    }
  lensm_t m;
  memset(&m, 0, sizeof m);
  const int fit = anchor_model(&L, &H, iw, ih, A, &m);
  lens[0] = m.K; lens[1] = m.ax; lens[2] = m.ay; lens[3] = m.R;
  for (int k = 0; k < LENS_P; k++) lens[4 + k] = m.t[k];
  ob_layout_free(&L);
  return fit;
}

// The border nodes' refinement as the registration's mesh step runs it (liblizard/src/acquire.c:5044-5058): the four
// corners taken as measured (done, no displacement), then every marked node in rings outward from the corners, each
// refine_node'd from its measured neighbours, with the lens model when given (NULL: none). The layout's format word
// cells are flagged as the format's frame flags them (lizard_phy.c fmt_paint). nodes_out: nx * ny x (dx, dy, score,
// done). Returns nx (= ny), or -1.
int refs_border_nodes(int span, const uint8_t *px, int w, int h, const float *H9, const double *lens, float *nodes_out) {
  ob_layout_t L;
  if (ob_layout_init(&L, span + 2 * OB_MARGIN)) return -1;
  uint8_t cw[OB_FMT_BYTES_MAX];
  memset(cw, 0, sizeof cw);
  ob_layout_set_fmt(&L, cw);
  image_t im;
  ob_image_init(&im, px, w, h, 1.0f);
  homo_t H;
  memcpy(H.h, H9, sizeof H.h);
  lensm_t lm;
  memset(&lm, 0, sizeof lm);
  if (lens) {
    lm.K = (int)lens[0]; lm.ax = lens[1]; lm.ay = lens[2]; lm.R = lens[3];
    for (int a = 0; a < LENS_P; a++) lm.t[a] = lens[4 + a];
  }
  const int nx = L.nx, ny = L.ny, nn = nx * ny;
  node_t *nodes = calloc((size_t)nn, sizeof(node_t));
  for (int c = 0; c < 4; c++) nodes[((c >= 2) ? ny - 1 : 0) * nx + ((c == 1 || c == 2) ? nx - 1 : 0)].done = 1;
  // the marked nodes ring by ring, rows within a ring (the counting sort of acquire.c:5046-5052)
  int start[OB_MAX_NODES + 2] = {0}, order[4 * OB_MAX_NODES], no = 0;
#define RING(i, j) (((i) < nx - 1 - (i) ? (i) : nx - 1 - (i)) + ((j) < ny - 1 - (j) ? (j) : ny - 1 - (j)))
  for (int j = 0; j < ny; j++) for (int i = 0; i < nx; i++) if (L.node_mark[j * nx + i]) start[RING(i, j) + 1]++;
  for (int k = 1; k < OB_MAX_NODES + 2; k++) start[k] += start[k - 1];
  for (int j = 0; j < ny; j++) for (int i = 0; i < nx; i++) if (L.node_mark[j * nx + i]) { order[start[RING(i, j)]++] = j * nx + i; no++; }
#undef RING
  for (int k = 0; k < no; k++) {
    if (nodes[order[k]].done) continue;
    refine_node(&L, &im, &H, order[k] % nx, order[k] / nx, nodes, lens ? &lm : 0);
  }
  for (int k = 0; k < nn; k++) {
    nodes_out[4 * k] = nodes[k].dx; nodes_out[4 * k + 1] = nodes[k].dy; nodes_out[4 * k + 2] = nodes[k].score; nodes_out[4 * k + 3] = (float)nodes[k].done;
  }
  free(nodes);
  ob_layout_free(&L);
  return nx;
}

// The code registered from the anchors as the reference's acquisition runs it (liblizard/src/acquire.c:2128-2197
// anchor_register) after its corners' step (:5028-5037: the four corners done, no displacement): px the frame, rim
// the border search's image (NULL: the frame), H9 the corners' homography (in; out the registration's), quad the
// corners in the image (in; out as moved), mpx pixels a module. Out per anchor: ok, peak, dx, dy, u, v; lens the
// model about H (K, ax, ay, R, coefficients). Returns anchor_register's result (1 held, 0 not), or -1.
int refs_anchor_register(int span, const uint8_t *px, const uint8_t *rim_px, int w, int h, float *H9, float *quad, float mpx, uint8_t *ok,
                         float *peak, float *dx, float *dy, float *u, float *v, double *lens) {
  ob_layout_t L;
  if (ob_layout_init(&L, span + 2 * OB_MARGIN)) return -1;
  uint8_t cw[OB_FMT_BYTES_MAX];
  memset(cw, 0, sizeof cw);
  ob_layout_set_fmt(&L, cw);
  image_t im, rim;
  ob_image_init(&im, px, w, h, 1.0f);
  ob_image_init(&rim, rim_px ? rim_px : px, w, h, 1.0f);
  homo_t H;
  memcpy(H.h, H9, sizeof H.h);
  const int nx = L.nx, ny = L.ny;
  node_t *nodes = calloc((size_t)nx * ny, sizeof(node_t));
  if (!nodes) { ob_layout_free(&L); return -1; }
  for (int c = 0; c < 4; c++) nodes[((c >= 2) ? ny - 1 : 0) * nx + ((c == 1 || c == 2) ? nx - 1 : 0)].done = 1;
  anchor_t A[OB_ANCH_K * OB_ANCH_K];
  memset(A, 0, sizeof A);
  lensm_t m;
  memset(&m, 0, sizeof m);
  const int held = anchor_register(&L, &im, &rim, &H, w, h, mpx, quad, nodes, A, &m);
  memcpy(H9, H.h, sizeof H.h);
  for (int k = 0; k < OB_ANCH_K * OB_ANCH_K; k++) {
    ok[k] = (uint8_t)A[k].ok; peak[k] = A[k].peak; dx[k] = A[k].dx; dy[k] = A[k].dy; u[k] = A[k].u; v[k] = A[k].v;
  }
  lens[0] = m.K; lens[1] = m.ax; lens[2] = m.ay; lens[3] = m.R;
  for (int k = 0; k < LENS_P; k++) lens[4 + k] = m.t[k];
  free(nodes);
  ob_layout_free(&L);
  return held;
}

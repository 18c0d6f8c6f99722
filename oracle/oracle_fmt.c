// Oracle (test infrastructure only): the format word, restated in plain C from the reference. Its Reed-Solomon code
// over GF(256) (liblizard/src/rs.c), the word's place in the border and its soft decode (liblizard/src/fmt.c,
// liblizard/src/layout.c:57-87), and its read off a captured frame through the registration
// (liblizard/src/acquire.c:4503-4559 ob_thin_read_fmt, with ob_map_point acquire.c:5090-5105, project and sample
// liblizard/src/internal.h:11-23, 107-112). Pinned against the reference's own rs.c, fmt.c and ob_thin_read_fmt
// compiled here (oracle/ref_harness.c refh_fmt_*), bit for bit.
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "oracle.h"

// ---------------------------------------------------------------- GF(256), polynomial 0x11d (rs.c:1-17)

static uint8_t gexp[512], glog[256];
static int gready;

static void gf_init(void) {
  if (gready) return;
  int x = 1;
  for (int i = 0; i < 255; i++) {
    gexp[i] = (uint8_t)x;
    glog[x] = (uint8_t)i;
    x <<= 1;
    if (x & 256) x ^= 0x11d;
  }
  for (int i = 255; i < 512; i++) gexp[i] = gexp[i - 255];
  gready = 1;
}
static uint8_t gmul(uint8_t a, uint8_t b) { return a && b ? gexp[glog[a] + glog[b]] : 0; }
static uint8_t ginv(uint8_t a) { return gexp[255 - glog[a]]; }
// The locator of position j of an n-byte codeword, and the log of its inverse (rs.c:65-70).
static uint8_t loc(int n, int j) { return gexp[(n - 1 - j) % 255]; }
static int loc_inv_log(int n, int j) { return (255 - (n - 1 - j)) % 255; }

// Systematic encode, generator roots alpha^0 .. alpha^(nroots - 1), highest degree first (rs.c:19-35).
void orc_rs_encode(uint8_t *cw, int k, int nroots) {
  gf_init();
  uint8_t g[256] = {1};
  for (int i = 0; i < nroots; i++) {
    g[i + 1] = 0;
    for (int j = i + 1; j > 0; j--) g[j] ^= gmul(g[j - 1], gexp[i]);
  }
  uint8_t *par = cw + k;
  memset(par, 0, (size_t)nroots);
  for (int i = 0; i < k; i++) {
    const uint8_t fb = cw[i] ^ par[0];
    memmove(par, par + 1, (size_t)nroots - 1);
    par[nroots - 1] = 0;
    if (fb)
      for (int j = 0; j < nroots; j++) par[j] ^= gmul(fb, g[j + 1]);
  }
}

static int syndromes(const uint8_t *cw, int n, int nroots, uint8_t *S) {
  int any = 0;
  for (int i = 0; i < nroots; i++) {
    uint8_t s = 0;
    for (int j = 0; j < n; j++) s = gmul(s, gexp[i]) ^ cw[j];
    S[i] = s;
    any |= s;
  }
  return any;
}

// Chien search and Forney's values for locator lam of degree deg; the word corrected in place. Returns the roots
// found, or -1 where they are not deg or a derivative vanishes (rs.c:63-86, 127-141).
static int chien_forney(uint8_t *cw, int n, int nroots, const uint8_t *S, const uint8_t *lam, int deg) {
  int pos[256], found = 0;
  for (int j = 0; j < n; j++) {
    const int e = loc_inv_log(n, j);
    uint8_t v = 0;
    for (int i = deg; i >= 0; i--) v = gmul(v, gexp[e]) ^ lam[i];
    if (!v) pos[found++] = j;
  }
  if (found != deg) return -1;
  uint8_t W[256] = {0};
  for (int i = 0; i < nroots; i++)
    for (int j = 0; j <= i && j <= deg; j++) W[i] ^= gmul(S[i - j], lam[j]);
  for (int q = 0; q < found; q++) {
    const int j = pos[q];
    const uint8_t xi = gexp[loc_inv_log(n, j)];
    uint8_t num = 0, den = 0, p = 1;
    for (int i = 0; i < nroots; i++) { num ^= gmul(W[i], p); p = gmul(p, xi); }
    p = 1;
    for (int i = 1; i <= deg; i += 2) { den ^= gmul(lam[i], p); p = gmul(p, gmul(xi, xi)); }
    if (!den) return -1;
    cw[j] ^= gmul(gmul(num, ginv(den)), loc(n, j));
  }
  return found;
}

// Errors only: Berlekamp-Massey for the locator, at most nroots / 2 errors (rs.c:37-87).
int orc_rs_decode(uint8_t *cw, int n, int nroots) {
  gf_init();
  uint8_t S[256];
  if (!syndromes(cw, n, nroots, S)) return 0;
  uint8_t C[256] = {1}, B[256] = {1}, T[256];
  int L = 0, m = 1;
  uint8_t b = 1;
  for (int r = 0; r < nroots; r++) {
    uint8_t d = S[r];
    for (int i = 1; i <= L; i++) d ^= gmul(C[i], S[r - i]);
    if (!d) { m++; continue; }
    memcpy(T, C, sizeof T);
    const uint8_t f = gmul(d, ginv(b));
    for (int i = 0; i + m < 256; i++) C[i + m] ^= gmul(f, B[i]);
    if (2 * L <= r) { L = r + 1 - L; memcpy(B, T, sizeof B); b = d; m = 1; }
    else m++;
  }
  if (L > nroots / 2) return -1;
  return chien_forney(cw, n, nroots, S, C, L);
}

// Errors and erasures: Berlekamp-Massey started from the erasures' locator; corrected only where the locator's
// degree is the register's length and 2 errors + erasures <= nroots (rs.c:89-146 solve, rs_decode_er).
int orc_rs_decode_er(uint8_t *cw, int n, int nroots, const int *eras, int neras) {
  gf_init();
  uint8_t S[256];
  const int any = syndromes(cw, n, nroots, S);
  if (!any && !neras) return 0;
  if (neras > nroots) return -1;
  uint8_t lam[257] = {1}, b[257], t[257];
  for (int k = 0; k < neras; k++) {
    const uint8_t X = loc(n, eras[k]);
    for (int i = k + 1; i > 0; i--) lam[i] ^= gmul(lam[i - 1], X);
  }
  memcpy(b, lam, sizeof b);
  int el = neras;
  for (int r = neras + 1; r <= nroots; r++) {
    uint8_t d = 0;
    for (int i = 0; i < r && i <= el; i++) d ^= gmul(lam[i], S[r - i - 1]);
    if (!d) { memmove(b + 1, b, 256); b[0] = 0; continue; }
    t[0] = lam[0];
    for (int i = 0; i < 256; i++) t[i + 1] = lam[i + 1] ^ gmul(d, b[i]);
    if (2 * el <= r + neras - 1) {
      el = r + neras - el;
      const uint8_t di = ginv(d);
      for (int i = 0; i < 257; i++) b[i] = gmul(lam[i], di);
    } else {
      memmove(b + 1, b, 256);
      b[0] = 0;
    }
    memcpy(lam, t, sizeof lam);
  }
  int deg = 0;
  for (int i = 0; i <= nroots; i++) if (lam[i]) deg = i;
  if (deg != el || 2 * (el - neras) + neras > nroots) return -1;
  return chien_forney(cw, n, nroots, S, lam, deg);
}

// ---------------------------------------------------------------- the word (fmt.c, layout.c)

enum { BAND_RUN = 4, CELL = 2, RESERVE = 15, MARGIN = 15, FMT_MAGIC = 0x4c, FMT_DATA = 3, FMT_MIN = 16, FMT_MAX = 64,
       FMT_SIDE_CELLS = 32, VERSION_MIN = 4, VERSION_MAX = 64 };

static int thin_cells(int side, int reserve) { return side > 2 * reserve ? (side - 2 * reserve) / CELL : 0; }   // layout.c:66
static int track_cells(int side, int reserve) { return (thin_cells(side, reserve) + 1) / 2; }                     // layout.c:67
// Modules from the reserve to track cell j and to word cell i (layout.h:110-112).
static int band_pair(int k) { return (k / BAND_RUN) * 2 * BAND_RUN + k % BAND_RUN; }
static int track_at(int j) { return band_pair(j) * CELL; }
static int word_at(int i) { return (band_pair(i) + BAND_RUN) * CELL; }

// Word cells a side and the codeword's bytes (fmt.c:6-20).
int orc_fmt_side_cells(int side, int reserve) {
  const int w = thin_cells(side, reserve) / (2 * BAND_RUN) * BAND_RUN;
  return w >= FMT_SIDE_CELLS ? w : 0;
}
int orc_fmt_bytes(int side, int reserve) {
  const int b = 4 * (orc_fmt_side_cells(side, reserve) / 8);
  return b > FMT_MAX ? FMT_MAX : b;
}
// Byte k on frame side k % 4, eight cells at 8 (k / 4) (fmt.c:22-30).
int orc_fmt_bit(const uint8_t *cw, int bytes, int edge, int cell) {
  const int k = 4 * (cell >> 3) + edge;
  if (edge < 0 || edge > 3 || cell < 0 || k >= bytes) return 0;
  return (cw[k] >> (7 - (cell & 7))) & 1;
}
// The magic, the version, the rate, then bytes - 3 roots (fmt.c:32-41).
int orc_fmt_encode(int version, int fps, uint8_t *cw, int bytes) {
  if (bytes < FMT_MIN || bytes > FMT_MAX || version < VERSION_MIN || version > VERSION_MAX || fps < 0 || fps > 255) return -1;
  memset(cw, 0, (size_t)bytes);
  cw[0] = FMT_MAGIC;
  cw[1] = (uint8_t)version;
  cw[2] = (uint8_t)fps;
  orc_rs_encode(cw, FMT_DATA, bytes - FMT_DATA);
  return 0;
}
// The timing track's bit for track cell j of a side (layout.c:57-61).
int orc_thin_track(int side, int j) {
  uint32_t v = (uint32_t)(side * 4099 + (j >> 1)) * 2654435761u + 40503u;
  v ^= v >> 15;
  v *= 2246822519u;
  v ^= v >> 13;
  return (int)((v ^ (uint32_t)j) & 1);
}

static int accept(const uint8_t *cw, int32_t *vf) {   // fmt.c:46-52
  if (cw[0] != FMT_MAGIC || cw[1] < VERSION_MIN || cw[1] > VERSION_MAX) return 0;
  vf[0] = cw[1];
  vf[1] = cw[2];
  return 1;
}

// The word from soft values q[side * cells + i] (> 0 dark): hard bytes through RS, then the least confident bytes
// erased two more a step while three roots stay over the erasures (fmt.c:54-86). vf: version, fps. 0, or -1.
int orc_fmt_decode(const float *q, int cells, int bytes, int32_t *vf) {
  const int nroots = bytes - FMT_DATA;
  if (bytes < FMT_MIN || bytes > FMT_MAX || cells < 8 * ((bytes + 3) / 4)) return -1;
  uint8_t cw[FMT_MAX], got[FMT_MAX];
  float worst[FMT_MAX];
  for (int k = 0; k < bytes; k++) {
    const float *qs = q + (k & 3) * cells + 8 * (k >> 2);
    uint8_t v = 0;
    float lo = 1;
    for (int b = 0; b < 8; b++) {
      const float s = qs[b], a = s < 0 ? -s : s;
      v = (uint8_t)((v << 1) | (s > 0));
      if (a < lo) lo = a;
    }
    cw[k] = v;
    worst[k] = lo;
  }
  memcpy(got, cw, (size_t)bytes);
  if (orc_rs_decode(got, bytes, nroots) >= 0 && accept(got, vf)) return 0;
  int order[FMT_MAX];
  uint8_t used[FMT_MAX] = {0};
  for (int ne = 0; ne < bytes; ne++) {   // the least confident first, the lower index on a tie
    int pick = -1;
    for (int k = 0; k < bytes; k++) if (!used[k] && (pick < 0 || worst[k] < worst[pick])) pick = k;
    used[pick] = 1;
    order[ne] = pick;
  }
  for (int ne = 2; ne <= nroots - 3; ne += 2) {
    memcpy(got, cw, (size_t)bytes);
    if (orc_rs_decode_er(got, bytes, nroots, order, ne) >= 0 && accept(got, vf)) return 0;
  }
  return -1;
}

// ---------------------------------------------------------------- the read (acquire.c)

// Bilinear read at gamma 1: x and y less half a pixel, clamped into the frame, a grey level's value k / 255
// (internal.h:11-23, acquire.c:50-54).
static float sample_px(const uint8_t *px, int w, int h, float x, float y) {
  x -= 0.5f;
  y -= 0.5f;
  if (x < 0) x = 0; else if (x > w - 1.001f) x = w - 1.001f;
  if (y < 0) y = 0; else if (y > h - 1.001f) y = h - 1.001f;
  const int xi = x >= 0 ? (int)x : 0, yi = y >= 0 ? (int)y : 0;
  const float fx = x - xi, fy = y - yi;
  const uint8_t *p = px + yi * w + xi;
  const float a = p[0] / 255.0f, b = p[1] / 255.0f, c = p[w] / 255.0f, d = p[w + 1] / 255.0f;
  return (a + (b - a) * fx) * (1 - fy) + (c + (d - c) * fx) * fy;
}

static int node_cell(const float *node, int nn, float m) {   // acquire.c:5090-5094
  int lo = 0, hi = nn - 2;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (m >= node[mid]) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Module point (mx, my) in the image: the homography and the node mesh's bilinear displacement (acquire.c:5095-5105,
// internal.h:107-112). reg: H (9 floats) then (dx, dy) of nx x ny nodes.
static void map_point(const float *reg, const float *nodes, int nn, float mx, float my, float *pu, float *pv) {
  const int j = node_cell(nodes, nn, my), i = node_cell(nodes, nn, mx);
  const float v = (my - nodes[j]) / (nodes[j + 1] - nodes[j]), u = (mx - nodes[i]) / (nodes[i + 1] - nodes[i]);
  const float *n00 = reg + 9 + 2 * (j * nn + i), *n10 = n00 + 2, *n01 = n00 + 2 * nn, *n11 = n01 + 2;
  const float dx = (n00[0] * (1 - u) + n10[0] * u) * (1 - v) + (n01[0] * (1 - u) + n11[0] * u) * v;
  const float dy = (n00[1] * (1 - u) + n10[1] * u) * (1 - v) + (n01[1] * (1 - u) + n11[1] * u) * v;
  const float *h = reg;
  const float w = h[6] * mx + h[7] * my + 1;
  *pu = (h[0] * mx + h[1] * my + h[2]) / w + dx;
  *pv = (h[3] * mx + h[4] * my + h[5]) / w + dy;
}

// Layout coordinates on side 0..3 (top, right, bottom, left) at t along it and depth d (acquire.c:3806-3810).
static void side_xy(int W, int side, float t, float d, float *x, float *y) {
  *x = side == 0 || side == 2 ? t : side == 3 ? d : W - d;
  *y = side == 0 ? d : side == 2 ? W - d : t;
}

static float read_at(const uint8_t *px, int iw, int ih, const float *reg, const float *nodes, int nn, int W, int side, float t, float d) {
  float x, y, u, v;
  side_xy(W, side, t, d, &x, &y);
  map_point(reg, nodes, nn, x, y, &u, &v);
  return sample_px(px, iw, ih, u, v);
}

// The word's soft values off a frame of a ring of `span` modules (its border a square of span + 30 modules), through
// the registration reg (H, then the mesh of the nn x nn nodes at module coordinates nodes): each word cell against
// the mean level of the track's Manchester pairs within 12 modules, then the two means' midpoint of the word's own
// cells, over the border's contrast, clipped to +-0.5, > 0 dark (acquire.c:4503-4559). q: 4 x cells. Returns cells,
// or 0 where the band is not read (too small, too little contrast).
int orc_fmt_read(int span, const uint8_t *px, int iw, int ih, const float *reg, const float *nodes, int nn, float *q) {
  const int W = span + 2 * MARGIN, cells = orc_fmt_side_cells(W, RESERVE);
  if (cells < 1) return 0;
  float dark = 0, light = 0;
  int nref = 0;
  for (int side = 0; side < 4; side++)
    for (int t = RESERVE; t < W - RESERVE; t += 16, nref++) {
      dark += read_at(px, iw, ih, reg, nodes, nn, W, side, t + 0.5f, 1 + 2 / 2.0f);
      light += read_at(px, iw, ih, reg, nodes, nn, W, side, t + 0.5f, 3 + 2 / 2.0f);
    }
  if (!nref) return 0;
  const float con = (light - dark) / nref;
  if (con < 0.08f) return 0;
  const int REACH = 12 / (2 * CELL), PAIRMOD = 4 * CELL;
  float *mid = malloc(((size_t)W / PAIRMOD + 2) * sizeof(float));
  if (!mid) return 0;
  for (int side = 0; side < 4; side++) {
    const int npair = track_cells(W, RESERVE) / 2;
    if (npair < 1) { free(mid); return 0; }
    for (int pr = 0; pr < npair; pr++) {
      float s = 0;
      for (int k = 0; k < 2; k++) s += read_at(px, iw, ih, reg, nodes, nn, W, side, RESERVE + track_at(2 * pr + k) + CELL / 2.0f, 5 + 2 / 2.0f);
      mid[pr] = 0.5f * s;
    }
    for (int i = 0; i < cells; i++) {
      const int off = word_at(i);
      const float smp = read_at(px, iw, ih, reg, nodes, nn, W, side, RESERVE + off + CELL / 2.0f, 5 + 2 / 2.0f);
      const int at = off / PAIRMOD, lo = at - REACH < 0 ? 0 : at - REACH, hi = at + REACH >= npair ? npair - 1 : at + REACH;
      float m = 0;
      for (int k = lo; k <= hi; k++) m += mid[k];
      q[side * cells + i] = smp - m / (hi - lo + 1);
    }
  }
  free(mid);
  float ref = 0;
  for (int it = 0; it < 4; it++) {
    float lo = 0, hi = 0;
    int nlo = 0;
    for (int i = 0; i < 4 * cells; i++) {
      if (q[i] < ref) { lo += q[i]; nlo++; }
      else hi += q[i];
    }
    if (nlo < cells / 2 || 4 * cells - nlo < cells / 2) break;
    ref = 0.5f * (lo / nlo + hi / (4 * cells - nlo));
  }
  for (int i = 0; i < 4 * cells; i++) {
    const float s = (ref - q[i]) / con;
    q[i] = s > 0.5f ? 0.5f : s < -0.5f ? -0.5f : s;
  }
  return cells;
}

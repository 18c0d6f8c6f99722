// Oracle, receiver part: the format's tables, the spectrum in FP64, the pilot alignment, the soft demap and the
// block stage (decline gate, bit map, LDPC, CRC, pilots). TEST INFRASTRUCTURE ONLY (see oracle.h).
//
// The demap and block stages restate the arithmetic of the reference's x86-64 build exactly (its float moments in
// four chains, its float turns and quantiser), so from identical spectra they give identical soft values. The
// spectrum itself is FP64 here: the transform and detrend of liblizard/src/lizard_phy.c:1577-1716 computed from
// their definitions, the oracle the FP32 transforms are measured against.
#include "oracle.h"
#include "../lizard_gb300/csrc/lizard_codes.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

enum { SUB = 320, STRIP = 64, ANCH_K = 7, ANCH_MARGIN = 2, MARGIN = 15, TURNS = 4096 };
static const double PI = 3.14159265358979323846;

struct orc_fmt {
  int n, subch, span, blocks, used, bw, vblocks, tiers, bytes_per_block;
  float scale;
  int tier_rate[4], tier_blocks[4], tier_slots[4];
  int *block_tier, *block_slot;
  int *pos;              // subch * 320 packed spectrum offsets, pos order (liblizard/src/lizard_phy.c:505-535)
  int16_t *uv;           // (u, v) of each, u in (-n/2, n/2)
  uint8_t *white;        // whitening bit of every frame slot
  int *perm[4];          // per tier: codeword bit of block slot i < nt
  orc_code_t code[4];
  int elo[ANCH_K], ehi[ANCH_K];
  double hole_inv[6][6];
  double *cx, *qx, *x1r, *x1i, *x2r, *x2i, sx2, sq2;
  float *cxf, *qxf;
  float rot[2 * TURNS];
};

// liblizard/src/lizard_phy.c:563-569: a block's slots, its code's sent bits then its pilots.
static int block_slots(int rate) {
  orc_code_t c;
  if (orc_code_init(&c, rate)) return 0;
  return c.nt + (rate == 6 ? 16 : rate == 4 ? 32 : 0);
}

// liblizard/src/lizard_phy.c:578-613 tier_search: least squares in integers over the non-filling tiers' counts,
// pruned, the first of equals kept; the second tier (3/4) fills the rest.
static void tier_search(int k, int n, const int *slots, const int *tgt, long long all, long long used, long long cost, int *cnt, long long *best, int *keep) {
  if (k == n) {
    const long long rest = all - used;
    if (rest < slots[1]) return;
    if (*best < 0 || cost < *best) { *best = cost; for (int t = 0; t < n; t++) keep[t] = cnt[t]; keep[1] = (int)(rest / slots[1]); }
    return;
  }
  if (k == 1) { tier_search(2, n, slots, tgt, all, used, cost, cnt, best, keep); return; }
  for (int a = 0; used + (long long)slots[k] * a <= all - slots[1]; a++) {
    const long long d = 1000LL * slots[k] * a - (long long)tgt[k] * all;
    if (*best >= 0 && cost + d * d >= *best) { if (d > 0) break; continue; }
    cnt[k] = a;
    tier_search(k + 1, n, slots, tgt, all, used + (long long)slots[k] * a, cost + d * d, cnt, best, keep);
  }
}

int orc_tiers_for(int subch, int32_t *rate, int32_t *blocks, int32_t *slots) {
  if (subch < 64 || subch % 16 || subch > 1024) return 0;
  static const int RATE[4] = { 6, 4, 3, 2 }, TGT[4] = { 390, 0, 150, 200 };
  int sl[4], cnt[4] = { 0 }, keep[4] = { 0 };
  for (int q = 0; q < 4; q++) sl[q] = block_slots(RATE[q]);
  long long best = -1;
  tier_search(0, 4, sl, TGT, (long long)subch * SUB * 2, 0, 0, cnt, &best, keep);
  int t = 0;
  for (int q = 0; q < 4; q++) if (keep[q]) { rate[t] = RATE[q]; blocks[t] = keep[q]; slots[t] = sl[q]; t++; }
  return t;
}

static int gcd(int a, int b) { while (b) { const int t = a % b; a = b; b = t; } return a; }

void orc_fmt_free(orc_fmt_t *f) {
  if (!f) return;
  free(f->block_tier); free(f->pos); free(f->uv); free(f->white);
  for (int t = 0; t < 4; t++) free(f->perm[t]);
  free(f->cx); free(f->cxf);
  free(f);
}

orc_fmt_t *orc_fmt_new(int n, int subch, int span) {
  static const int PICS[7] = { 384, 512, 768, 1024, 1152, 1280, 1536 };
  int ok = 0;
  for (int i = 0; i < 7; i++) ok |= n == PICS[i];
  if (!span) span = 256;
  if (!ok || (span != 128 && span != 256 && span != 512)) return 0;
  orc_fmt_t *f = calloc(1, sizeof *f);
  if (!f) return 0;
  f->n = n; f->subch = subch; f->span = span; f->bytes_per_block = LIZG_BLOCK_BYTES;
  int32_t rate[4], nb[4], sl[4];
  f->tiers = orc_tiers_for(subch, rate, nb, sl);
  if (!f->tiers) { orc_fmt_free(f); return 0; }
  for (int t = 0; t < f->tiers; t++) {
    f->tier_rate[t] = rate[t]; f->tier_blocks[t] = nb[t]; f->tier_slots[t] = sl[t]; f->blocks += nb[t];
    orc_code_init(&f->code[t], rate[t]);
  }
  // pos: the used half-plane coefficients by (u^2 + v^2, v, u) rising, excluding v = 0, u <= 0 and the Nyquist row
  // and column (liblizard/src/lizard_phy.c:505-535); packed as (v / bw) n bw + ((u + n) % n) bw + v % bw.
  const int need = subch * SUB, h = n / 2;
  const int rmax = 2 * (h - 1) * (h - 1);
  int *at = calloc((size_t)rmax + 1, sizeof(int));
  int cap = 0;
  for (int v = 0; v < h; v++) for (int u = -h + 1; u < h; u++) { if (v == 0 && u <= 0) continue; at[u * u + v * v]++; cap++; }
  if (need > cap) { free(at); orc_fmt_free(f); return 0; }
  int cut = 0, placed = 0;
  for (;; cut++) { const int k = at[cut]; at[cut] = placed; placed += k; if (placed >= need) break; }
  int *cu = malloc((size_t)placed * sizeof(int)), *cv = malloc((size_t)placed * sizeof(int));
  for (int v = 0; v < h; v++) for (int u = -h + 1; u < h; u++) {
    if (v == 0 && u <= 0) continue;
    const int r2 = u * u + v * v;
    if (r2 <= cut) { cu[at[r2]] = u; cv[at[r2]] = v; at[r2]++; }
  }
  free(at);
  f->bw = h < STRIP ? h : STRIP;
  f->pos = malloc((size_t)need * sizeof(int));
  f->uv = malloc((size_t)need * 2 * sizeof(int16_t));
  int vmax = 0;
  for (int i = 0; i < need; i++) {
    f->pos[i] = (cv[i] / f->bw) * n * f->bw + ((cu[i] + n) % n) * f->bw + cv[i] % f->bw;
    f->uv[2 * i] = (int16_t)cu[i]; f->uv[2 * i + 1] = (int16_t)cv[i];
    if (cv[i] > vmax) vmax = cv[i];
  }
  free(cu); free(cv);
  f->vblocks = vmax / f->bw + 1;
  f->scale = (float)n / span;
  // blocks from the frame's first slot, inner first (liblizard/src/lizard_phy.c:551-555)
  f->block_tier = malloc((size_t)f->blocks * 2 * sizeof(int));
  f->block_slot = f->block_tier + f->blocks;
  for (int t = 0, b = 0, s = 0; t < f->tiers; t++) for (int q = 0; q < f->tier_blocks[t]; q++, b++, s += f->tier_slots[t]) {
    f->block_tier[b] = t; f->block_slot[b] = s; f->used = s + f->tier_slots[t];
  }
  // whitening: PRBS-23, x^23 + x^18 + 1 from all ones (liblizard/src/lizard_phy.c:95-101)
  f->white = malloc((size_t)subch * SUB * 2);
  uint32_t s = 0x7fffff;
  for (int i = 0; i < subch * SUB * 2; i++) { const uint32_t b = ((s >> 22) ^ (s >> 17)) & 1; s = ((s << 1) | b) & 0x7fffff; f->white[i] = (uint8_t)b; }
  // bit map: slot i carries sent bit i P mod nt, P the first number from round(0.3819660113 nt) prime to nt; sent bit
  // j is codeword bit j, past the code's k - np the np never sent skipped (liblizard/src/lizard_phy.c:111-116, 557-562)
  for (int t = 0; t < f->tiers; t++) {
    const orc_code_t *c = &f->code[t];
    f->perm[t] = malloc((size_t)c->nt * sizeof(int));
    int P = (int)(0.3819660113 * c->nt + 0.5);
    while (gcd(P, c->nt) != 1) P++;
    for (int i = 0; i < c->nt; i++) { const int j = (int)((long)i * P % c->nt); f->perm[t][i] = j < c->k - c->np ? j : j + c->np; }
  }
  // detrend basis c = (2 i + 1 - n) / n and q = c^2 less its mean, their norms and transforms, all in double
  // (liblizard/src/lizard_phy.c:389-398)
  f->cx = malloc((size_t)6 * n * sizeof(double));
  f->qx = f->cx + n; f->x1r = f->cx + 2 * n; f->x1i = f->cx + 3 * n; f->x2r = f->cx + 4 * n; f->x2i = f->cx + 5 * n;
  f->cxf = malloc((size_t)2 * n * sizeof(float)); f->qxf = f->cxf + n;
  double m2 = 0;
  for (int i = 0; i < n; i++) { const double c = (2.0 * i + 1 - n) / n; m2 += c * c; }
  f->sx2 = m2; m2 /= n; f->sq2 = 0;
  for (int i = 0; i < n; i++) {
    const double c = (2.0 * i + 1 - n) / n, q = c * c - m2;
    f->cx[i] = c; f->qx[i] = q; f->sq2 += q * q; f->cxf[i] = (float)c; f->qxf[i] = (float)q;
  }
  for (int u = 0; u < n; u++) {
    double ar = 0, ai = 0, br = 0, bi = 0;
    for (int i = 0; i < n; i++) {
      const int k = (int)((long)u * i % n);
      const double cs = cos(-2 * PI * k / n), sn = sin(-2 * PI * k / n);
      ar += f->cx[i] * cs; ai += f->cx[i] * sn; br += f->qx[i] * cs; bi += f->qx[i] * sn;
    }
    f->x1r[u] = ar; f->x1i[u] = ai; f->x2r[u] = br; f->x2i[u] = bi;
  }
  // the anchors' squares as erased: 7 ranges each axis, square i at module m0_i of side span / 64
  // (liblizard/src/acquire.c:41-45), widened by 2 samples (liblizard/src/lizard_phy.c:400-407)
  const int a = span / 64;
  for (int i = 0; i < ANCH_K; i++) {
    const int m0 = (int)floor(MARGIN + (double)span * (i + 0.5) / ANCH_K - a / 2.0 + 0.5);
    const int lo = (int)floorf((m0 - MARGIN) * f->scale) - ANCH_MARGIN, hi = (int)ceilf((m0 + a - MARGIN) * f->scale) - 1 + ANCH_MARGIN;
    f->elo[i] = lo < 0 ? 0 : lo; f->ehi[i] = hi > n - 1 ? n - 1 : hi;
  }
  // the shading fit's normal matrix over every eighth sample outside the squares, inverted by Gauss-Jordan with
  // partial pivots (liblizard/src/lizard_phy.c:408-425)
  double g[6][12] = {{0}};
  for (int y = 0; y < n; y += 8) for (int x = 0; x < n; x += 8) {
    int ix = 0, iy = 0;
    for (int i = 0; i < ANCH_K; i++) { ix |= x >= f->elo[i] && x <= f->ehi[i]; iy |= y >= f->elo[i] && y <= f->ehi[i]; }
    if (ix && iy) continue;
    const double b[6] = { 1, f->cxf[x], f->qxf[x], f->cxf[y], f->qxf[y], (double)f->cxf[x] * f->cxf[y] };
    for (int r = 0; r < 6; r++) for (int c = 0; c < 6; c++) g[r][c] += b[r] * b[c];
  }
  for (int r = 0; r < 6; r++) g[r][6 + r] = 1;
  for (int c = 0; c < 6; c++) {
    int p = c;
    for (int r = c + 1; r < 6; r++) if (fabs(g[r][c]) > fabs(g[p][c])) p = r;
    for (int k = 0; k < 12; k++) { const double t = g[c][k]; g[c][k] = g[p][k]; g[p][k] = t; }
    const double d = g[c][c];
    for (int k = 0; k < 12; k++) g[c][k] /= d;
    for (int r = 0; r < 6; r++) if (r != c) { const double m = g[r][c]; for (int k = 0; k < 12; k++) g[r][k] -= m * g[c][k]; }
  }
  for (int r = 0; r < 6; r++) for (int c = 0; c < 6; c++) f->hole_inv[r][c] = g[r][6 + c];
  for (int i = 0; i < TURNS; i++) { const double th = 2.0 * PI * i / TURNS; f->rot[2 * i] = (float)cos(th); f->rot[2 * i + 1] = (float)sin(th); }
  return f;
}

// info: n, subch, span, blocks, used, bw, vblocks, tiers, then per tier rate, blocks, slots (12 more).
int orc_fmt_info(const orc_fmt_t *f, int32_t *info) {
  info[0] = f->n; info[1] = f->subch; info[2] = f->span; info[3] = f->blocks; info[4] = f->used; info[5] = f->bw;
  info[6] = f->vblocks; info[7] = f->tiers;
  for (int t = 0; t < 4; t++) { info[8 + 3 * t] = t < f->tiers ? f->tier_rate[t] : 0; info[9 + 3 * t] = t < f->tiers ? f->tier_blocks[t] : 0; info[10 + 3 * t] = t < f->tiers ? f->tier_slots[t] : 0; }
  return 0;
}
// The tables out: pos (subch * 320), uv (2 * subch * 320), white (subch * 640), block_tier and block_slot (blocks
// each), perm of tier t (nt), erase ranges (14), hole_inv (36 doubles). Any pointer may be NULL.
int orc_fmt_tables(const orc_fmt_t *f, int32_t *pos, int16_t *uv, uint8_t *white, int32_t *btier, int32_t *bslot, int32_t *erase, double *hole_inv) {
  const int need = f->subch * SUB;
  if (pos) memcpy(pos, f->pos, (size_t)need * sizeof(int));
  if (uv) memcpy(uv, f->uv, (size_t)need * 2 * sizeof(int16_t));
  if (white) memcpy(white, f->white, (size_t)need * 2);
  if (btier) memcpy(btier, f->block_tier, (size_t)f->blocks * sizeof(int));
  if (bslot) memcpy(bslot, f->block_slot, (size_t)f->blocks * sizeof(int));
  if (erase) for (int i = 0; i < ANCH_K; i++) { erase[i] = f->elo[i]; erase[ANCH_K + i] = f->ehi[i]; }
  if (hole_inv) memcpy(hole_inv, f->hole_inv, sizeof f->hole_inv);
  return 0;
}
int orc_fmt_perm(const orc_fmt_t *f, int tier, int32_t *perm) {
  if (tier < 0 || tier >= f->tiers) return -1;
  memcpy(perm, f->perm[tier], (size_t)f->code[tier].nt * sizeof(int));
  return f->code[tier].nt;
}

static int in_sq(const orc_fmt_t *f, int t) {
  for (int i = 0; i < ANCH_K; i++) if (t >= f->elo[i] && t <= f->ehi[i]) return 1;
  return 0;
}

// ------------------------------------------------------------------ the spectrum, FP64

typedef struct { double r, i; } cd_t;

// Mixed-radix decimation in time, recursive, on a twiddle table of the full length N (tw[k] = e^{-2 pi i k / N});
// n divides N. out[k] = sum_j in[j s] e^{-2 pi i j k / n}.
static void dft(const cd_t *in, int s, int n, cd_t *out, const cd_t *tw, int N, cd_t *tmp) {
  if (n == 1) { out[0] = in[0]; return; }
  const int p = n % 4 == 0 && n != 8 ? 4 : n % 2 == 0 ? 2 : n % 3 == 0 ? 3 : n % 5 == 0 ? 5 : n;
  const int m = n / p;
  if (p == n) {   // a prime length left: direct
    for (int k = 0; k < n; k++) {
      double ar = 0, ai = 0;
      for (int j = 0; j < n; j++) { const cd_t w = tw[(long)j * k % n * (N / n)]; ar += in[j * s].r * w.r - in[j * s].i * w.i; ai += in[j * s].r * w.i + in[j * s].i * w.r; }
      out[k].r = ar; out[k].i = ai;
    }
    return;
  }
  for (int q = 0; q < p; q++) dft(in + q * s, s * p, m, tmp + q * m, tw, N, out);
  for (int k = 0; k < n; k++) {
    double ar = 0, ai = 0;
    for (int q = 0; q < p; q++) {
      const cd_t x = tmp[q * m + k % m], w = tw[(long)q * k % n * (N / n)];
      ar += x.r * w.r - x.i * w.i; ai += x.r * w.i + x.i * w.r;
    }
    out[k].r = ar; out[k].i = ai;
  }
  // tmp now free for the caller's next use; out holds the result
}

// One length-n transform of n points at stride s, into out (scratch 2n).
static void dft_n(const cd_t *in, int s, int n, cd_t *out, const cd_t *tw, cd_t *scratch) {
  cd_t *tmp = scratch;
  dft(in, s, n, out, tw, n, tmp);
}

// The hole fit, the erase and the detrend projections of liblizard/src/lizard_phy.c:1598-1627, 1635-1640, 1642-1674,
// in double, on a row-major n x n grid (grid[y n + x], values in grey / 255). grid is erased in place.
static void erase_and_project(const orc_fmt_t *f, float *grid, double proj[5]) {
  const int n = f->n, c = n / 8;
  double rhs[6] = { 0 }, beta[6] = { 0 };
  for (int ky = 0; ky < c; ky++) for (int kx = 0; kx < c; kx++) {
    const int x = 8 * kx, y = 8 * ky;
    if (in_sq(f, y) && in_sq(f, x)) continue;
    const double v = grid[(size_t)y * n + x];
    const double b[6] = { 1, f->cxf[x], f->qxf[x], f->cxf[y], f->qxf[y], (double)f->cxf[x] * f->cxf[y] };
    for (int r = 0; r < 6; r++) rhs[r] += b[r] * v;
  }
  for (int r = 0; r < 6; r++) for (int k = 0; k < 6; k++) beta[r] += f->hole_inv[r][k] * rhs[k];
  for (int j = 0; j < ANCH_K; j++) for (int i = 0; i < ANCH_K; i++)
    for (int y = f->elo[j]; y <= f->ehi[j]; y++) for (int x = f->elo[i]; x <= f->ehi[i]; x++) {
      const double b[6] = { 1, f->cxf[x], f->qxf[x], f->cxf[y], f->qxf[y], (double)f->cxf[x] * f->cxf[y] };
      double v = 0;
      for (int r = 0; r < 6; r++) v += beta[r] * b[r];
      grid[(size_t)y * n + x] = (float)v;
    }
  double px = 0, py = 0, pxy = 0, pxx = 0, pyy = 0;
  for (int y = 0; y < n; y++) {
    double rs = 0, rx = 0, rq = 0;
    for (int x = 0; x < n; x++) { const double z = grid[(size_t)y * n + x]; rs += z; rx += z * f->cxf[x]; rq += z * f->qxf[x]; }
    px += rx; py += rs * f->cxf[y]; pxy += rx * f->cxf[y]; pxx += rq; pyy += rs * f->qxf[y];
  }
  proj[0] = px / (n * f->sx2); proj[1] = py / (n * f->sx2); proj[2] = pxy / (f->sx2 * f->sx2); proj[3] = pxx / (n * f->sq2); proj[4] = pyy / (n * f->sq2);
}

// coef[2 i], coef[2 i + 1]: the detrended spectrum T(u_i, v_i) = sum_{x, y} z(x, y) e^{-2 pi i (u x + v y) / n} less
// the surface's transform (liblizard/src/lizard_phy.c:1697-1716), in pos order. grid (row-major, grey / 255) is erased
// in place; proj (5) gets px, py, pxy, pxx, pyy after normalisation.
int orc_spectrum(const orc_fmt_t *f, float *grid, double *coef, double *proj_out) {
  const int n = f->n, V = f->vblocks * f->bw, need = f->subch * SUB;
  double proj[5];
  erase_and_project(f, grid, proj);
  if (proj_out) memcpy(proj_out, proj, sizeof proj);
  cd_t *tw = malloc((size_t)n * sizeof(cd_t)), *col = malloc((size_t)n * sizeof(cd_t)), *out = malloc((size_t)n * sizeof(cd_t));
  cd_t *scr = malloc((size_t)2 * n * sizeof(cd_t)), *Y = malloc((size_t)n * V * sizeof(cd_t)), *T = malloc((size_t)n * V * sizeof(cd_t));
  for (int k = 0; k < n; k++) { tw[k].r = cos(-2 * PI * k / n); tw[k].i = sin(-2 * PI * k / n); }
  // columns x: Y(x, v) = sum_y z(x, y) e^{-2 pi i v y / n}, v < V
  for (int x = 0; x < n; x++) {
    for (int y = 0; y < n; y++) { col[y].r = grid[(size_t)y * n + x]; col[y].i = 0; }
    dft_n(col, 1, n, out, tw, scr);
    for (int v = 0; v < V; v++) Y[(size_t)v * n + x] = out[v];
  }
  // rows v: T(u, v) = sum_x Y(x, v) e^{-2 pi i u x / n}
  for (int v = 0; v < V; v++) {
    dft_n(Y + (size_t)v * n, 1, n, out, tw, scr);
    memcpy(T + (size_t)v * n, out, (size_t)n * sizeof(cd_t));
  }
  for (int i = 0; i < need; i++) {
    const int u = (f->uv[2 * i] + n) % n, v = f->uv[2 * i + 1];
    double tr = T[(size_t)v * n + u].r, ti = T[(size_t)v * n + u].i;
    const double ar = proj[2] * f->x1r[u], ai = proj[2] * f->x1i[u];
    tr -= ar * f->x1r[v] - ai * f->x1i[v]; ti -= ar * f->x1i[v] + ai * f->x1r[v];
    if (v == 0) { tr -= n * (proj[0] * f->x1r[u] + proj[3] * f->x2r[u]); ti -= n * (proj[0] * f->x1i[u] + proj[3] * f->x2i[u]); }
    if (u == 0) { tr -= n * (proj[1] * f->x1r[v] + proj[4] * f->x2r[v]); ti -= n * (proj[1] * f->x1i[v] + proj[4] * f->x2i[v]); }
    coef[2 * i] = tr; coef[2 * i + 1] = ti;
  }
  free(tw); free(col); free(out); free(scr); free(Y); free(T);
  return need;
}

// ------------------------------------------------------------------ pilots and soft values (x86-64 arithmetic)

// liblizard/src/lizard_phy.c:214-218 turned_uv: the turn index in float, the rotation in float, no fused operations.
static void turned(const orc_fmt_t *f, const float *coef, int i, float dx, float dy, float *yr, float *yi) {
  const float uu = (float)f->uv[2 * i], vv = (float)f->uv[2 * i + 1];
  const float a = uu * dx, b = vv * dy, sc = (float)TURNS / (float)f->n;
  const float t = (a + b) * sc;
  const unsigned k = (unsigned)(int)nearbyintf(t) & (TURNS - 1);
  const float c = f->rot[2 * k], sn = f->rot[2 * k + 1], r = coef[2 * i], im = coef[2 * i + 1];
  const float p1 = r * c, p2 = im * sn, p3 = im * c, p4 = r * sn;
  *yr = p1 + p2; *yi = p3 - p4;
}

// liblizard/src/lizard_phy.c:280-329 pilot_align: two weighted least-squares fits of the grid shift from the 7/8 and
// 3/4 blocks' tails, the second about the first's answer; taken only where chi^2 > 13.8. Returns the pilots used.
int orc_pilot_align(const orc_fmt_t *f, const float *coef, float d[2]) {
  const double k = 2.0 * PI / f->n;
  double dx = 0, dy = 0, a = 0, b = 0, c = 0, p = 0, q = 0, yy = 0;
  int used = 0;
  for (int it = 0; it < 2; it++) {
    a = b = c = p = q = yy = 0; used = 0;
    for (int blk = 0; blk < f->blocks; blk++) {
      const orc_code_t *code = &f->code[f->block_tier[blk]];
      const int nb = f->tier_slots[f->block_tier[blk]], first = f->block_slot[blk] / 2;
      const uint8_t *wh = f->white + 2 * (size_t)first;
      if (code->nt >= nb) continue;
      for (int s = code->nt / 2; s < nb / 2; s++) {
        const int i = first + s;
        float yr, yi;
        turned(f, coef, i, (float)dx, (float)dy, &yr, &yi);
        const double xr = wh[2 * s] ? -1.0 : 1.0, xi = wh[2 * s + 1] ? -1.0 : 1.0;
        const double zr = yr * xr + yi * xi, zi = yi * xr - yr * xi;
        const double cu = k * zr * f->uv[2 * i], cv = k * zr * f->uv[2 * i + 1];
        a += cu * cu; b += cu * cv; c += cv * cv; p += cu * zi; q += cv * zi; yy += zi * zi;
        used++;
      }
    }
    const double det = a * c - b * b;
    if (used < 8 || !(det > 0)) { d[0] = d[1] = 0; return used; }
    dx += (p * c - q * b) / det; dy += (a * q - b * p) / det;
  }
  const double det = a * c - b * b, ex = (p * c - q * b) / det, ey = (a * q - b * p) / det;
  const double s2 = (yy - ex * p - ey * q) / (used - 2);
  const double chi = s2 > 0 ? (dx * dx * a + 2 * dx * dy * b + dy * dy * c) / s2 : 0;
  if (!(chi > 13.8) || !(dx == dx) || !(dy == dy)) { d[0] = d[1] = 0; return used; }
  d[0] = (float)dx; d[1] = (float)dy;
  return used;
}

// liblizard/src/lizard_phy.c:73-75: ten Brink's J at sigma = 2 sqrt(g).
static double axis_info(double g) { return g > 0 ? pow(1 - pow(2, -0.3073 * pow(2 * sqrt(g), 1.7870)), 1.1064) : 0; }

// Soft values of every slot of the frame (liblizard/src/lizard_phy.c:1728-1772 with the x86-64 soft4 of :1411-1451):
// per sub-channel the float moments in four chains (coefficient s in chain s mod 4, |y|^2 a multiply, a multiply
// and an add), summed (c0 + c1) + (c2 + c3); the scale and estimate in double (sub_scale, :1320-1332); each axis value
// times 8 k in float, NaN to 0, clamped to +-80, rounded half to even. turn: the pilots' shift applied as each
// coefficient is read, or NULL.
int orc_demap(const orc_fmt_t *f, const float *coef, const float *turn, int8_t *llrf, double *sub_est, float *sub_rms) {
  for (int j = 0; j < f->subch; j++) {
    float gr[SUB], gi[SUB];
    for (int s = 0; s < SUB; s++) {
      const int i = j * SUB + s;
      if (turn) turned(f, coef, i, turn[0], turn[1], &gr[s], &gi[s]);
      else { gr[s] = coef[2 * i]; gi[s] = coef[2 * i + 1]; }
    }
    float m2c[4] = { 0, 0, 0, 0 }, m4c[4] = { 0, 0, 0, 0 };
    for (int s = 0; s < SUB; s++) {
      const float rr = gr[s] * gr[s], ii = gi[s] * gi[s], e = rr + ii, ee = e * e;
      m2c[s & 3] = m2c[s & 3] + e; m4c[s & 3] = m4c[s & 3] + ee;
    }
    const float fm2 = (m2c[0] + m2c[1]) + (m2c[2] + m2c[3]), fm4 = (m4c[0] + m4c[1]) + (m4c[2] + m4c[3]);
    double m2 = (double)fm2 / SUB, m4 = (double)fm4 / SUB;
    sub_rms[j] = m2 > 0 ? (float)sqrt(m2 / 2) : 0;
    double a2 = 2 * m2 * m2 - m4;
    a2 = a2 > 0 ? sqrt(a2) : 0;
    double nv = m2 - a2;
    if (nv < 0.02 * m2) nv = 0.02 * m2;
    sub_est[j] = axis_info(a2 / nv);
    const float k = (float)(0.7 * 2 * sqrt(2 * a2) / nv), k8 = 8 * k;
    for (int s = 0; s < SUB; s++) {
      float x = k8 * gr[s], y = k8 * gi[s];
      x = x != x ? 0.0f : x; y = y != y ? 0.0f : y;
      x = x < -80.0f ? -80.0f : x > 80.0f ? 80.0f : x; y = y < -80.0f ? -80.0f : y > 80.0f ? 80.0f : y;
      llrf[2 * (j * SUB + s)] = (int8_t)nearbyintf(x); llrf[2 * (j * SUB + s) + 1] = (int8_t)nearbyintf(y);
    }
  }
  return f->subch;
}

// The block stage of liblizard/src/lizard_phy.c:1775-1871: each block's estimate (its sub-channels' information
// weighted by the slots it holds there), its pilot reading, the decline gate (0.2 k / nt, float), the bit map in
// (codeword bit perm[i] = the slot's value, negated where whitened; the 7/8 code's known zeros at 127), the decoder
// (30 iterations, stall 9 / 0.95) and the CRC check. its[b]: -2 declined, else the decoder's return; ok[b] 1 where
// verified; blocks gets the verified 476-byte blocks. Returns the count verified.
int orc_blocks(const orc_fmt_t *f, const int8_t *llrf, const double *sub_est, const float *sub_rms, const float *coef,
               const float *turn, int max_iter, uint8_t *blocks, uint8_t *ok, int8_t *its, float *est, float *pilot) {
  int good = 0;
  int8_t *cl = malloc(7680);
  uint8_t *bits = malloc(7680);
  for (int b = 0; b < f->blocks; b++) {
    const int t = f->block_tier[b], nb = f->tier_slots[t], s0 = f->block_slot[b];
    const orc_code_t *code = &f->code[t];
    ok[b] = 0; its[b] = 0; pilot[b] = NAN;
    double info = 0;
    for (int j = s0 / (2 * SUB); j * 2 * SUB < s0 + nb; j++) {
      const int lo = s0 > 2 * SUB * j ? s0 : 2 * SUB * j, hi = s0 + nb < 2 * SUB * (j + 1) ? s0 + nb : 2 * SUB * (j + 1);
      info += sub_est[j] * (hi - lo);
    }
    est[b] = (float)(info / nb);
    if (code->nt < nb) {
      const uint8_t *wh = f->white + s0;
      double cs = 0;
      int got = 0;
      for (int i = code->nt; i < nb; i++) {
        const int gs = s0 + i, ci = gs / 2;
        const float rms = sub_rms[gs / (2 * SUB)];
        if (!(rms > 0)) continue;
        float yr = coef[2 * ci], yi = coef[2 * ci + 1];
        if (turn) turned(f, coef, ci, turn[0], turn[1], &yr, &yi);
        const float y = (i & 1) ? yi : yr;
        cs += (wh[i] ? -1.0 : 1.0) * y / rms;
        got++;
      }
      if (got) pilot[b] = (float)(cs / (nb - code->nt));
    }
    if (est[b] < 0.2f * (float)code->k / (float)code->nt) { its[b] = -2; continue; }
    const int8_t *llr = llrf + s0;
    const uint8_t *wh = f->white + s0;
    for (int i = code->k - code->np; i < code->k; i++) cl[i] = 0;
    for (int i = 0; i < code->nt; i++) cl[f->perm[t][i]] = wh[i] ? (int8_t)-llr[i] : llr[i];
    for (int i = (f->bytes_per_block + 4) * 8; i < code->k; i++) cl[i] = 127;
    const int r = orc_ldpc_decode(code, cl, bits, max_iter, 9, 0.95f);
    its[b] = (int8_t)r;
    if (r < 0) continue;
    uint8_t *dst = blocks + (size_t)b * f->bytes_per_block;
    for (int j = 0; j < f->bytes_per_block; j++) {
      uint8_t v = 0;
      for (int q = 0; q < 8; q++) v = (uint8_t)(v << 1 | bits[8 * j + q]);
      dst[j] = v;
    }
    uint32_t crc = 0;
    for (int i = 0; i < 32; i++) crc = (crc << 1) | bits[f->bytes_per_block * 8 + i];
    if (crc != orc_crc32c(dst, f->bytes_per_block)) continue;
    ok[b] = 1; good++;
  }
  free(cl); free(bits);
  return good;
}

// ------------------------------------------------------------------ the sampler (row a)

// The node lattice of a square layout of `side` modules (liblizard/src/layout.c:110-117).
int orc_layout_nodes(int side, float *pos) {
  int cnt = 0;
  for (float c = 3.5f; c < side - 3.5f - 8 && cnt < 39; c += 16) pos[cnt++] = c;
  pos[cnt++] = side - 3.5f;
  return cnt;
}

static int cell_of(const float *node, int nn, float m) {
  int k = 0;
  for (int q = 1; q <= nn - 2; q++) if (m >= node[q]) k = q;
  return k;
}

// The picture grid of a luma frame through a registration (H: 9 floats, then the nx x ny mesh's (dx, dy)), by the
// reference's exact walk: liblizard/src/acquire.c:5121-5196 (the scalar branch) and internal.h:11-23 sample(), float
// operations in the same order, one rounding each.
int orc_sample_grid(int n, int span, const uint8_t *luma, int w, int h, int pitch, const float *reg, float *grid) {
  float node[40];
  const int nn = orc_layout_nodes(span + 2 * MARGIN, node);
  const float scale = (float)n / span, g0 = MARGIN + 0.5f / scale, step = 1.0f / scale;
  const float *H = reg, *nodes = reg + 9;
  for (int y = 0; y < n; y++) {
    const float my = g0 + (float)y * step;
    const int j = cell_of(node, nn, my);
    const float v = (my - node[j]) / (node[j + 1] - node[j]);
    const float kw = H[7] * my + 1, ku = H[1] * my + H[2], kv = H[4] * my + H[5];
    for (int x = 0; x < n; x++) {
      const float mx = g0 + (float)x * step;
      const int i = cell_of(node, nn, mx);
      const float *n00 = nodes + 2 * (j * nn + i), *n10 = n00 + 2, *n01 = n00 + 2 * nn, *n11 = n01 + 2;
      const float inv = 1.0f / (node[i + 1] - node[i]);
      const float ex = ((n10[0] - n00[0]) * (1 - v) + (n11[0] - n01[0]) * v) * inv, cx = n00[0] * (1 - v) + n01[0] * v - ex * node[i];
      const float ey = ((n10[1] - n00[1]) * (1 - v) + (n11[1] - n01[1]) * v) * inv, cy = n00[1] * (1 - v) + n01[1] * v - ey * node[i];
      const float rw = 1 / (H[6] * mx + kw);
      const float pu = (H[0] * mx + ku) * rw, pv = (H[3] * mx + kv) * rw;
      const float dx = cx + ex * mx, dy = cy + ey * mx;
      float sx = pu + dx - 0.5f, sy = pv + dy - 0.5f;
      if (sx < 0) sx = 0; else if (sx > w - 1.001f) sx = w - 1.001f;
      if (sy < 0) sy = 0; else if (sy > h - 1.001f) sy = h - 1.001f;
      const int xi = sx >= 0 ? (int)sx : 0, yi = sy >= 0 ? (int)sy : 0;
      const float fx = sx - xi, fy = sy - yi;
      const uint8_t *p = luma + (size_t)yi * pitch + xi;
      const float a = p[0] / 255.0f, b = p[1] / 255.0f, c = p[pitch] / 255.0f, d = p[pitch + 1] / 255.0f;
      grid[(size_t)y * n + x] = (a + (b - a) * fx) * (1 - fy) + (c + (d - c) * fx) * fy;
    }
  }
  return nn;
}

// ------------------------------------------------------------------ the sampler as the decode runs it (row a)

// The decode's picture read at gamma 1 on x86-64 (liblizard/src/acquire.c:5302-5440 sample_grid_lin, reached through
// ob_sample_grid_pic :5465-5480), restated in plain C: one call samples columns x0 .. x0 + nx - 1 of rows
// 0 .. ny - 1 of the regular grid at (mx0 + x step, my0 + y step), in chunks of 256 columns. Per chunk and mesh row
// every column's displacement terms D + v E (liblizard/src/acquire.c:5330-5346, the column's place u in its mesh cell
// first, :5310-5316); per row the homography's numerators and denominator as four-column lanes stepped by four
// columns at a time (:5348-5358: lane l starts at l (h step) + (h m0 + row terms), each step adds 4 (h step)); then
// the point (less the half pixel, x a 512th on) read in integers (:723-779 lin_pts, lin_grey, lin_get): 16.16
// coordinates clamped at 0 and 32767, the integer parts clamped to w - 2 and h - 2, fx the x fraction's top byte, fy
// the y fraction's top 15 bits; each row's pair blended as 256 a + (b - a) fx, the rows' halved difference times fy
// rounded (PMULHRSW), plus the top row's half: 128 times the grey, times 257 / 2^23 as a float. No fused operations.
static int lin_q16(float v) {
  if (!(v > 0)) v = 0;                 // MAXPS with 0: below 0, and NaN, read as 0
  if (v > 32767.0f) v = 32767.0f;
  return (int)(v * 65536.0f);          // CVTTPS2DQ: truncation; the product is exact
}
static float lin_read_point(const uint8_t *luma, int w, int h, int pitch, float X, float Y) {
  const int xq = lin_q16(X), yq = lin_q16(Y);
  int xi = xq >> 16, yi = yq >> 16;
  if (xi > w - 2) xi = w - 2;
  if (yi > h - 2) yi = h - 2;
  const int fx = (xq >> 8) & 0xff, fy = (yq & 0xffff) >> 1;
  const uint8_t *p = luma + (size_t)yi * pitch + xi;
  const int a = p[0], b = p[1], c = p[pitch], d = p[pitch + 1];
  const int top = 256 * a + (b - a) * fx, bot = 256 * c + (d - c) * fx;
  const int hd = (bot - top) >> 1;                        // floor of the halved difference (PAVGW with the complement)
  const int r = ((hd * fy + (1 << 14)) >> 15) + (top >> 1);   // PMULHRSW's rounding, plus the top row's half
  return (float)r * (257.0f / 8388608.0f);
}
static void sample_lin_call(const float *node, int nn, const float *H, const float *nodes, const uint8_t *luma, int w, int h, int pitch,
                            float mx0, float my0, float step, int x0, int nx, int y0, int ny, float *out, int opitch) {
  for (int c0 = 0; c0 < nx; c0 += 256) {
    const int cx0 = x0 + c0, cnx = nx - c0 < 256 ? nx - c0 : 256;
    float tu[256];
    int ti[256];
    for (int k = 0; k < cnx; k++) {
      const float mx = mx0 + (float)(cx0 + k) * step;
      const int i = cell_of(node, nn, mx);
      const float inv = 1.0f / (node[i + 1] - node[i]);
      ti[k] = i;
      tu[k] = (mx - node[i]) * inv;
    }
    const float m0 = mx0 + (float)cx0 * step;
    const float hw = H[6] * step, hu = H[0] * step, hv = H[3] * step;
    const float Cw = 4 * hw, Cu = 4 * hu, Cv = 4 * hv;
    for (int yy = 0; yy < ny; yy++) {
      const float my = my0 + (float)(y0 + yy) * step;
      const int j = cell_of(node, nn, my);
      const float vv = (my - node[j]) / (node[j + 1] - node[j]);
      const float bw = H[6] * m0 + (H[7] * my + 1), bu = H[0] * m0 + (H[1] * my + H[2]), bv = H[3] * m0 + (H[4] * my + H[5]);
      float nw[4], nu[4], nv[4];
      for (int l = 0; l < 4; l++) { nw[l] = (float)l * hw + bw; nu[l] = (float)l * hu + bu; nv[l] = (float)l * hv + bv; }
      for (int k = 0; k < cnx; k++) {
        const int l = k & 3;
        if (k && !l) for (int q = 0; q < 4; q++) { nw[q] = nw[q] + Cw; nu[q] = nu[q] + Cu; nv[q] = nv[q] + Cv; }
        const float *a = nodes + 2 * (j * nn + ti[k]), *b = a + 2 * nn;
        const float U = tu[k];
        const float dx = (a[0] - (0.5f - 1.0f / 512)) + (a[2] - a[0]) * U, ex = (b[0] - a[0]) + ((b[2] - b[0]) - (a[2] - a[0])) * U;
        const float dy = (a[1] - 0.5f) + (a[3] - a[1]) * U, ey = (b[1] - a[1]) + ((b[3] - b[1]) - (a[3] - a[1])) * U;
        const float rw = 1.0f / nw[l];
        const float X = (dx + ex * vv) + nu[l] * rw, Y = (dy + ey * vv) + nv[l] * rw;
        out[(size_t)yy * opitch + k + c0] = lin_read_point(luma, w, h, pitch, X, Y);
      }
    }
  }
}

// The picture grid as the decode samples it (liblizard/src/lizard_phy.c:1634: one call a strip of 64 columns over
// every row) into grid (row-major n x n), and the shading fit's samples (:1611: one call over every eighth row and
// column at eight steps) into shade ((n / 8)^2, row-major; NULL: not taken). reg = H (9) then the mesh's (dx, dy).
int orc_sample_decode(int n, int span, const uint8_t *luma, int w, int h, int pitch, const float *reg, float *grid, float *shade) {
  float node[40];
  const int nn = orc_layout_nodes(span + 2 * MARGIN, node);
  const float scale = (float)n / span, g0 = MARGIN + 0.5f / scale, step = 1.0f / scale;
  for (int x0 = 0; x0 < n; x0 += 64) sample_lin_call(node, nn, reg, reg + 9, luma, w, h, pitch, g0, g0, step, x0, 64, 0, n, grid + x0, n);
  if (shade) sample_lin_call(node, nn, reg, reg + 9, luma, w, h, pitch, g0, g0, 8 * step, 0, n / 8, 0, n / 8, shade, n / 8);
  return nn;
}

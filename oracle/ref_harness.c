// Harness around the reference codec compiled from its own sources (oracle/Makefile builds it into oracle/_ref/
// only where the reference tree is present). TEST INFRASTRUCTURE ONLY: it lets the tests hold the oracle's
// restatement to the reference's own outputs, and lets the CPU baseline time the reference decoder. It defines the
// two globals the codec expects its host to provide (liblizard/core/cpu/codec.c:49) and exports plain entry points.
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "ldpc.h"
// The receiver's workspace is private to lizard_phy.c, so the harness compiles it in (the pattern of the reference's
// own liblizard/test/phy_x86.c:9) to read the spectrum, soft values and per-block results a finish leaves there.
#include "lizard_phy.c"

uint32_t ob_debug_hash;

uint32_t ob_crc32c(const uint8_t *p, int n);

uint32_t ref_crc32c(const uint8_t *p, int n) { return ob_crc32c(p, n); }

// One code's shape: n, k, m, np, nt, edges, mb, kb (liblizard/src/ldpc.h:12-28).
int ref_ldpc_shape(int rate, int32_t *dims) {
  ldpc_t c;
  if (ldpc_init(&c, rate)) return -1;
  dims[0] = c.n; dims[1] = c.k; dims[2] = c.m; dims[3] = c.np; dims[4] = c.nt; dims[5] = c.edges; dims[6] = c.mb; dims[7] = c.kb;
  ldpc_free(&c);
  return 0;
}

int ref_ldpc_encode(int rate, const uint8_t *data, uint8_t *cw) {
  ldpc_t c;
  if (ldpc_init(&c, rate)) return -1;
  ldpc_encode(&c, data, cw);
  ldpc_free(&c);
  return 0;
}

// count codewords of one rate, each n int8 LLRs back to back; out n bits a codeword (one a byte).
int ref_ldpc_decode_many(int rate, const int8_t *llr, int count, uint8_t *out, int32_t *its, int max_iter, int stall_it, float ratio) {
  ldpc_t c;
  if (ldpc_init(&c, rate)) return -1;
  for (int i = 0; i < count; i++)
    its[i] = ldpc_decode_stall(&c, llr + (size_t)i * c.n, out + (size_t)i * c.n, max_iter, stall_it, ratio);
  ldpc_free(&c);
  return 0;
}

// The mixed-rate batch on `threads` host threads, the same contract as the oracle's orc_ldpc_batch: each thread its
// own ldpc_t per rate (the decoder's workspace lives in it), codewords taken 16 at a time.
typedef struct {
  const int8_t *llr; const int64_t *off; const int32_t *rate; int count, max_iter, stall_it; float ratio;
  uint8_t *out; int32_t *its; uint8_t *ok; int next; pthread_mutex_t mu;
} ref_batch_t;

static int code_slot(int rate) { return rate == 6 ? 0 : rate == 4 ? 1 : rate == 3 ? 2 : rate == 2 ? 3 : -1; }

static void *ref_worker(void *arg) {
  ref_batch_t *b = arg;
  static const int RATES[4] = { 6, 4, 3, 2 };
  ldpc_t c[4];
  for (int t = 0; t < 4; t++) ldpc_init(&c[t], RATES[t]);
  uint8_t *bits = malloc(7680);
  for (;;) {
    pthread_mutex_lock(&b->mu);
    const int i0 = b->next; b->next += 16;
    pthread_mutex_unlock(&b->mu);
    if (i0 >= b->count) break;
    for (int i = i0; i < i0 + 16 && i < b->count; i++) {
      const ldpc_t *cc = &c[code_slot(b->rate[i])];
      b->its[i] = ldpc_decode_stall(cc, b->llr + b->off[i], bits, b->max_iter, b->stall_it, b->ratio);
      uint8_t *o = b->out + b->off[i] / 8;
      for (int j = 0; j < cc->n / 8; j++) {
        uint8_t v = 0;
        for (int t = 0; t < 8; t++) v = (uint8_t)(v << 1 | bits[8 * j + t]);
        o[j] = v;
      }
      const uint32_t want = (uint32_t)o[476] << 24 | (uint32_t)o[477] << 16 | (uint32_t)o[478] << 8 | o[479];
      b->ok[i] = ob_crc32c(o, 476) == want;
    }
  }
  free(bits);
  for (int t = 0; t < 4; t++) ldpc_free(&c[t]);
  return 0;
}

int ref_ldpc_batch(const int8_t *llr, const int64_t *off, const int32_t *rate, int count, int max_iter, int stall_it,
                   float ratio, uint8_t *out, int32_t *its, uint8_t *ok, int threads) {
  for (int i = 0; i < count; i++) if (code_slot(rate[i]) < 0) return -1;
  ref_batch_t b = { llr, off, rate, count, max_iter, stall_it, ratio, out, its, ok, 0, PTHREAD_MUTEX_INITIALIZER };
  if (threads < 1) threads = 1;
  if (threads > 256) threads = 256;
  pthread_t th[256];
  for (int t = 1; t < threads; t++) pthread_create(&th[t], 0, ref_worker, &b);
  ref_worker(&b);
  for (int t = 1; t < threads; t++) pthread_join(th[t], 0);
  return 0;
}


// ------------------------------------------------------------------ the receiver

lizard_t *ref_fmt_new(int n, int subch, int span) {
  lizard_t *f = calloc(1, sizeof *f);
  if (!f) return 0;
  if (lizard_init(f, n, subch, span)) { free(f); return 0; }
  return f;
}
void ref_fmt_free(lizard_t *f) { if (f) { lizard_free(f); free(f); } }

// n, subch, blocks, used, bw, vblocks, tiers, pxm, px, then per tier rate, blocks, slots.
void ref_fmt_info(const lizard_t *f, int32_t *o) {
  o[0] = f->n; o[1] = f->subch; o[2] = f->blocks; o[3] = f->used; o[4] = f->bw; o[5] = f->vblocks; o[6] = f->tiers; o[7] = f->pxm; o[8] = f->px;
  for (int t = 0; t < 4; t++) { o[9 + 3 * t] = t < f->tiers ? f->tier[t].rate : 0; o[10 + 3 * t] = t < f->tiers ? f->tier[t].blocks : 0; o[11 + 3 * t] = t < f->tiers ? f->tier[t].slots : 0; }
}
void ref_fmt_tables(const lizard_t *f, int32_t *pos, uint8_t *white, int32_t *btier, int32_t *bslot, int32_t *erase, double *hole_inv) {
  const struct lizard_ws *w = f->ws;
  memcpy(pos, f->pos, (size_t)f->subch * LIZARD_SUB * sizeof(int));
  memcpy(white, w->white, (size_t)f->subch * LIZARD_SUB * 2);
  memcpy(btier, f->block_tier, (size_t)f->blocks * sizeof(int));
  memcpy(bslot, f->block_slot, (size_t)f->blocks * sizeof(int));
  for (int i = 0; i < OB_ANCH_K; i++) { erase[i] = w->elo[i]; erase[OB_ANCH_K + i] = w->ehi[i]; }
  memcpy(hole_inv, w->hole_inv, sizeof w->hole_inv);
}
int ref_fmt_perm(const lizard_t *f, int t, int32_t *perm) {
  if (t < 0 || t >= f->tiers) return -1;
  memcpy(perm, f->ws->perm[t], (size_t)f->code[t].nt * sizeof(int));
  return f->code[t].nt;
}

// The sender: blocks (blocks x 476) encoded with pilot count c, the drive (px^2 floats) and its grey square with the
// quiet margin (W^2 bytes, W = px + 2 LIZARD_QUIET pxm). Returns W.
int ref_encode(lizard_t *f, const uint8_t *blocks, int c, float *drive, uint8_t *grey) {
  lizard_parity(f, c);
  lizard_encode(f, blocks, drive);
  if (grey) lizard_paint_grey(f, drive, grey);
  return f->px + 2 * LIZARD_QUIET * f->pxm;
}

// The finish on a supplied picture grid (row-major n x n, grey / 255), as lizard_finish(f, grid, ...) runs it with a
// registration held: the transform and detrend in FP32, the pilots, the soft values, the blocks. Out (any NULL):
// coef (2 floats a coefficient, pos order), llrf (subch x 640), sub_est (subch doubles), sub_rms, align (2), and per
// block its, est, pilot; blocks and ok as lizard_finish gives them. Returns the blocks verified.
int ref_finish_grid(lizard_t *f, const float *grid, float *coef, int8_t *llrf, double *sub_est, float *sub_rms, float *align,
                    int8_t *its, float *est, float *pilot, uint8_t *blocks, uint8_t *ok) {
  struct lizard_ws *w = f->ws;
  const int n = f->n, sw = LIZARD_STRIP;
  float *strips = malloc((size_t)n * n * sizeof(float));
  for (int y = 0; y < n; y++) for (int x = 0; x < n; x++) strips[(size_t)(x / sw) * n * sw + (size_t)y * sw + x % sw] = grid[(size_t)y * n + x];
  lizard_debug(f, 1, 0, 0);
  memset(&w->hold_reg, 0, sizeof w->hold_reg);
  w->hold_valid = 1;
  ob_result_t res;
  uint8_t *bl = blocks ? blocks : malloc((size_t)f->blocks * LIZARD_BLOCK);
  uint8_t *okk = ok ? ok : malloc((size_t)f->blocks);
  const int good = lizard_finish(f, strips, bl, okk, &res);
  if (coef) memcpy(coef, w->dbg_coef, (size_t)f->subch * LIZARD_SUB * 2 * sizeof(float));
  if (llrf) memcpy(llrf, w->llrf, (size_t)f->subch * LIZARD_SUB * 2);
  if (sub_est) memcpy(sub_est, w->sub_est, (size_t)f->subch * sizeof(double));
  if (sub_rms) memcpy(sub_rms, w->sub_rms, (size_t)f->subch * sizeof(float));
  if (align) { align[0] = w->align[0]; align[1] = w->align[1]; }
  if (its) memcpy(its, w->blk_its, (size_t)f->blocks);
  if (est) memcpy(est, w->blk_est, (size_t)f->blocks * sizeof(float));
  if (pilot) memcpy(pilot, w->blk_pilot, (size_t)f->blocks * sizeof(float));
  if (!blocks) free(bl);
  if (!ok) free(okk);
  free(strips);
  return good;
}

// The whole decode of a luma frame (registration, then the finish), for the end-to-end comparisons. reg_out (any
// NULL): the registration found, H (9 floats) then the node mesh's (dx, dy) for nx x ny nodes; node_xy: the mesh
// nodes' module coordinates (nx then ny floats), nn: {nx, ny}.
int ref_decode_frame(lizard_t *f, const uint8_t *luma, int iw, int ih, uint8_t *blocks, uint8_t *ok, int8_t *its,
                     float *reg_out, float *node_xy, int32_t *nn) {
  ob_result_t res;
  if (!lizard_acquire(f, luma, iw, ih, 1.0f, &res)) { memset(ok, 0, (size_t)f->blocks); return -1; }
  const struct lizard_ws *w = f->ws;
  const ob_layout_t *L = &f->frame;
  if (nn) { nn[0] = L->nx; nn[1] = L->ny; }
  if (node_xy) { memcpy(node_xy, L->node_x, (size_t)L->nx * sizeof(float)); memcpy(node_xy + L->nx, L->node_y, (size_t)L->ny * sizeof(float)); }
  if (reg_out) {
    memcpy(reg_out, w->hold_reg.H.h, 9 * sizeof(float));
    for (int k = 0; k < L->nx * L->ny; k++) { reg_out[9 + 2 * k] = w->hold_reg.nodes[k].dx; reg_out[10 + 2 * k] = w->hold_reg.nodes[k].dy; }
  }
  const int good = lizard_finish(f, 0, blocks, ok, &res);
  if (its) memcpy(its, w->blk_its, (size_t)f->blocks);
  return good;
}

// The picture sampler on a given registration (H, nodes as ref_decode_frame reports them): the exact walk
// (ob_sample_grid) when fast = 0, the decode's own integer read (ob_sample_grid_pic) when 1; the n x n grid
// row-major.
int ref_sample_grid(lizard_t *f, const uint8_t *luma, int iw, int ih, const float *reg, int fast, float *grid) {
  image_t im;
  ob_image_init(&im, luma, iw, ih, 1.0f);
  const ob_layout_t *L = &f->frame;
  ob_reg_t r;
  memcpy(r.H.h, reg, 9 * sizeof(float));
  r.nodes = calloc((size_t)L->nx * L->ny, sizeof(node_t));
  for (int k = 0; k < L->nx * L->ny; k++) { r.nodes[k].dx = reg[9 + 2 * k]; r.nodes[k].dy = reg[10 + 2 * k]; }
  const float g0 = f->margin + 0.5f / f->scale, step = 1.0f / f->scale;
  const int n = f->n;
  if (fast) ob_sample_grid_pic(L, &im, &r, g0, g0, step, 0, n, 0, n, grid, n);
  else ob_sample_grid(L, &im, &r, g0, g0, step, 0, n, 0, n, grid, n);
  free(r.nodes);
  return 0;
}

// ------------------------------------------------------------------ the format word

// The format word's read and decode as acquire_hold runs them (lizard_phy.c:1553-1556), on a frame of a ring of
// `span` modules through the registration reg (H, then (dx, dy) of the layout's nodes): q (4 x cells soft values),
// word: read, ok, version, fps. Returns the cells a side (0: the band holds no word).
int refh_fmt_read(int span, const uint8_t *luma, int iw, int ih, const float *reg, float *q, int32_t *word) {
  ob_layout_t L;
  if (ob_layout_init(&L, span + 2 * OB_MARGIN)) return -1;
  image_t im;
  ob_image_init(&im, luma, iw, ih, 1.0f);
  ob_reg_t r;
  memcpy(r.H.h, reg, 9 * sizeof(float));
  r.nodes = calloc((size_t)L.nx * L.ny, sizeof(node_t));
  for (int k = 0; k < L.nx * L.ny; k++) { r.nodes[k].dx = reg[9 + 2 * k]; r.nodes[k].dy = reg[10 + 2 * k]; }
  const int cells = ob_fmt_side_cells(L.w, L.reserve), bytes = ob_fmt_bytes(L.w, L.reserve);
  ob_fmt_t ft = {0, 0};
  word[0] = cells && ob_thin_read_fmt(&L, &im, &r, q, cells);
  word[1] = word[0] && ob_fmt_decode(q, cells, bytes, &ft) == 0;
  word[2] = word[1] ? ft.version : 0;
  word[3] = word[1] ? ft.fps : 0;
  free(r.nodes);
  ob_layout_free(&L);
  return cells;
}

// ob_fmt_decode on given soft values (fmt.c:54-86), the word's version and fps into vf.
int refh_fmt_decode(const float *q, int cells, int bytes, int32_t *vf) {
  ob_fmt_t ft = {0, 0};
  const int rc = ob_fmt_decode(q, cells, bytes, &ft);
  vf[0] = ft.version;
  vf[1] = ft.fps;
  return rc;
}

// The layout's word geometry for a ring of `span` modules: cells a side, bytes; and the painted word of a format
// with sub-channels subch and display rate fps (fmt.c:32-41 through lizard_phy.c fmt_paint).
int refh_fmt_geometry(int span, int32_t *cells_bytes) {
  const int side = span + 2 * OB_MARGIN;
  cells_bytes[0] = ob_fmt_side_cells(side, OB_THIN_RESERVE);
  cells_bytes[1] = ob_fmt_bytes(side, OB_THIN_RESERVE);
  return 0;
}
int refh_fmt_encode(int version, int fps, uint8_t *cw, int bytes) {
  const ob_fmt_t ft = {version, fps};
  return ob_fmt_encode(&ft, cw, bytes);
}
// The layout's cell kinds (side x side modules, CELL_* values) of a format with the word for fps painted.
int refh_layout_kind(lizard_t *f, int fps, uint8_t *kind) {
  lizard_fmt_fps(f, fps);
  memcpy(kind, f->frame.kind, (size_t)f->frame.w * f->frame.h);
  return f->frame.w;
}

// The picture grid as the decode itself samples it (lizard_phy.c:1634: ob_sample_grid_pic a strip of LIZARD_STRIP
// columns at a time) into grid (row-major n x n), and the shading fit's samples (:1611: one call over every eighth
// row and column) into shade ((n / 8)^2, row-major, or NULL), on a given registration (H, then the nodes).
int ref_sample_decode(lizard_t *f, const uint8_t *luma, int iw, int ih, const float *reg, float *grid, float *shade) {
  image_t im;
  ob_image_init(&im, luma, iw, ih, 1.0f);
  const ob_layout_t *L = &f->frame;
  ob_reg_t r;
  memcpy(r.H.h, reg, 9 * sizeof(float));
  r.nodes = calloc((size_t)L->nx * L->ny, sizeof(node_t));
  for (int k = 0; k < L->nx * L->ny; k++) { r.nodes[k].dx = reg[9 + 2 * k]; r.nodes[k].dy = reg[10 + 2 * k]; }
  const float g0 = f->margin + 0.5f / f->scale, step = 1.0f / f->scale;
  const int n = f->n, sw = LIZARD_STRIP, c = n / 8;
  float *strip = malloc((size_t)n * sw * sizeof(float));
  for (int x0 = 0; x0 < n; x0 += sw) {
    ob_sample_grid_pic(L, &im, &r, g0, g0, step, x0, sw, 0, n, strip, sw);
    for (int y = 0; y < n; y++) memcpy(grid + (size_t)y * n + x0, strip + (size_t)y * sw, sw * sizeof(float));
  }
  if (shade) ob_sample_grid_pic(L, &im, &r, g0, g0, 8 * step, 0, c, 0, c, shade, c);
  free(strip);
  free(r.nodes);
  return im.lin;
}

// Oracle, LDPC and CRC part. TEST INFRASTRUCTURE ONLY (see oracle.h): the product never links this file.
#include "oracle.h"
#include "../lizard_gb300/csrc/lizard_codes.h"
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

// liblizard/src/ldpc.c:50-113: n = (kb + mb) z, k = kb z, m = mb z, np = np_cols z, nt = n - np; edges counted as
// (data circulants + 2) z over the block rows, less one (check 0 has no previous parity bit).
int orc_code_init(orc_code_t *c, int rate) {
  memset(c, 0, sizeof *c);
  const int slot = lizg_code_of_rate(rate);
  if (slot < 0) return -1;
  const lizg_code_def_t *d = &LIZG_CODES[slot];
  c->rate = rate; c->z = LIZG_Z; c->mb = d->mb; c->kb = d->kb;
  c->n = (d->kb + d->mb) * c->z; c->k = d->kb * c->z; c->m = d->mb * c->z;
  c->np = d->np_cols * c->z; c->nt = c->n - c->np;
  for (int r = 0; r <= d->mb; r++) c->rowptr[r] = d->rowptr[r];
  for (int e = 0; e < d->rowptr[d->mb]; e++) { c->col[e] = d->circ[e] >> 8; c->shift[e] = d->circ[e] & 255; }
  c->edges = (d->rowptr[d->mb] + 2 * d->mb) * c->z - 1;
  return 0;
}

static int modz(int a, int z) { a %= z; return a < 0 ? a + z : a; }

// H as the reference's CSR (liblizard/src/ldpc.c:69-78), hashed as liblizard/test/ldpc_table.c:13-18 does.
uint32_t orc_h_hash(const orc_code_t *c) {
  uint32_t h = 2166136261u;
  int e = 0;
  for (int chk = 0; chk <= c->m; chk++) {
    h = (h ^ (uint32_t)e) * 16777619u;
    if (chk == c->m) break;
    const int r = chk % c->mb;
    e += c->rowptr[r + 1] - c->rowptr[r] + (chk > 0) + 1;
  }
  for (int chk = 0; chk < c->m; chk++) {
    const int i = chk / c->mb, r = chk % c->mb;
    for (int s = c->rowptr[r]; s < c->rowptr[r + 1]; s++) h = (h ^ (uint32_t)(c->col[s] * c->z + modz(i - c->shift[s], c->z))) * 16777619u;
    if (chk > 0) h = (h ^ (uint32_t)(c->k + chk - 1)) * 16777619u;
    h = (h ^ (uint32_t)(c->k + chk)) * 16777619u;
  }
  return h;
}

// liblizard/src/ldpc.c:117-126: the parity bit of check chk is the running XOR of every data bit of checks 0..chk.
void orc_ldpc_encode(const orc_code_t *c, const uint8_t *data, uint8_t *cw) {
  memcpy(cw, data, (size_t)c->k);
  uint8_t acc = 0;
  for (int chk = 0; chk < c->m; chk++) {
    const int i = chk / c->mb, r = chk % c->mb;
    for (int s = c->rowptr[r]; s < c->rowptr[r + 1]; s++) acc ^= data[c->col[s] * c->z + modz(i - c->shift[s], c->z)];
    cw[c->k + chk] = acc;
  }
}

// Decoder state: posteriors of the data bits in code order, of the parity bits as [block row][position] (parity bit
// k + i mb + r at Lp[r z + i], liblizard/src/ldpc.c:1109), and one message a slot a position, laid out as the
// reference's wr: block row r's slots (its data circulants, the previous parity, its own parity) from
// rowptr[r] + 2 r (liblizard/src/ldpc.c:1115). z is 128 for every code (liblizard/src/ldpc_base.h:19).
enum { Z = 128 };
typedef struct { int16_t L[7680]; int8_t R[216 * Z]; } orc_state_t;

// Block row r's posteriors in check order, slot by slot (liblizard/src/ldpc.c:646-660 layer_gather): a data
// circulant of shift s puts data bit col z + (i - s) mod z at position i; the previous parity slot of row 0 is the
// last block row moved up a position under a certain zero (8191); plain copies otherwise.
static void gather(const orc_code_t *c, const int16_t *L, int r, int16_t Q[][Z]) {
  const int p0 = c->rowptr[r], nd = c->rowptr[r + 1] - p0;
  const int16_t *Lp = L + c->k;
  for (int e = 0; e < nd; e++) {
    const int16_t *col = L + c->col[p0 + e] * Z;
    const int sh = c->shift[p0 + e];
    for (int i = 0; i < sh; i++) Q[e][i] = col[Z - sh + i];
    for (int i = sh; i < Z; i++) Q[e][i] = col[i - sh];
  }
  if (r > 0) memcpy(Q[nd], Lp + (r - 1) * Z, Z * 2);
  else { Q[nd][0] = 8191; memcpy(Q[nd] + 1, Lp + (c->mb - 1) * Z, (Z - 1) * 2); }
  memcpy(Q[nd + 1], Lp + r * Z, Z * 2);
}

static void scatter(const orc_code_t *c, int16_t *L, int r, int16_t Q[][Z]) {
  const int p0 = c->rowptr[r], nd = c->rowptr[r + 1] - p0;
  int16_t *Lp = L + c->k;
  for (int e = 0; e < nd; e++) {
    int16_t *col = L + c->col[p0 + e] * Z;
    const int sh = c->shift[p0 + e];
    for (int i = 0; i < sh; i++) col[Z - sh + i] = Q[e][i];
    for (int i = sh; i < Z; i++) col[i - sh] = Q[e][i];
  }
  if (r > 0) memcpy(Lp + (r - 1) * Z, Q[nd], Z * 2);
  else memcpy(Lp + (c->mb - 1) * Z, Q[nd] + 1, (Z - 1) * 2);
  memcpy(Lp + r * Z, Q[nd + 1], Z * 2);
}

// One layer (block row r), its z checks independent and side by side. The four-times kernel's arithmetic
// (liblizard/src/ldpc.c:340-423): the extrinsic q = L - R in 16 bits (row 0's certain zero keeps 8191: its message
// is cleared before every use, liblizard/src/ldpc.c:1116); its byte saturated to [-128, 127] and held at -127; the
// check's sign the XOR of the bytes' signs; min1, min2 over the bytes' magnitudes (min2 = min(min2, max(min1, a)));
// scaled (x * 13) >> 4 capped at 127; an edge whose magnitude equals min1 takes min2's; the message carries the
// check's sign times its byte's; the posterior q + R with no clamp (the clamp never acts, liblizard/src/ldpc.c:96-103).
static void layer(const orc_code_t *c, orc_state_t *s, int r) {
  const int ns = c->rowptr[r + 1] - c->rowptr[r] + 2;
  int8_t *R = s->R + (size_t)(c->rowptr[r] + 2 * r) * Z;
  int16_t Q[64][Z], m1[Z], m2[Z], sg[Z], s1[Z], s2[Z];
  gather(c, s->L, r, Q);
  if (r == 0) R[(ns - 2) * Z] = 0;
  for (int i = 0; i < Z; i++) { m1[i] = 255; m2[i] = 255; sg[i] = 0; }
  for (int e = 0; e < ns; e++) {
    int16_t *q = Q[e];
    const int8_t *m = R + e * Z;
    for (int i = 0; i < Z; i++) {
      const int16_t v = (int16_t)(q[i] - m[i]);
      q[i] = v;
      const int16_t b = v > 127 ? 127 : v < -127 ? -127 : v;
      const int16_t a = b < 0 ? (int16_t)-b : b;
      sg[i] ^= b;
      const int16_t mx = m1[i] > a ? m1[i] : a;
      m2[i] = m2[i] < mx ? m2[i] : mx;
      m1[i] = m1[i] < a ? m1[i] : a;
    }
  }
  for (int i = 0; i < Z; i++) {
    const int16_t a = (int16_t)((m1[i] * 13) >> 4), b = (int16_t)((m2[i] * 13) >> 4);
    s1[i] = a > 127 ? 127 : a; s2[i] = b > 127 ? 127 : b;
  }
  for (int e = 0; e < ns; e++) {
    int16_t *q = Q[e];
    int8_t *m = R + e * Z;
    for (int i = 0; i < Z; i++) {
      const int16_t v = q[i], b = v > 127 ? 127 : v < -127 ? -127 : v, a = b < 0 ? (int16_t)-b : b;
      const int16_t mag = a == m1[i] ? s2[i] : s1[i];
      const int16_t rr = ((sg[i] ^ b) < 0) ? (int16_t)-mag : mag;
      m[i] = (int8_t)rr;
      q[i] = (int16_t)(v + rr);
    }
  }
  scatter(c, s->L, r, Q);
}

// Violated checks: the XOR of the signs of every posterior a check holds, row 0's missing bit a zero
// (liblizard/src/ldpc.c:903-930). The order the reference tests the layers in does not change the count.
static int unsat(const orc_code_t *c, const orc_state_t *s) {
  int bad = 0;
  int16_t Q[64][Z];
  for (int r = 0; r < c->mb; r++) {
    const int ns = c->rowptr[r + 1] - c->rowptr[r] + 2;
    gather(c, s->L, r, Q);
    if (r == 0) Q[ns - 2][0] = 0;
    for (int e = 1; e < ns; e++) for (int i = 0; i < Z; i++) Q[0][i] ^= Q[e][i];
    for (int i = 0; i < Z; i++) bad += Q[0][i] < 0;
  }
  return bad;
}

// liblizard/src/ldpc.c:1080-1172, the four-times path's stop: the checks tested after every iteration; at iteration
// stall_it (stall_it > 1) the violated checks are counted and the block given up (-3) while the count is above
// stall_ratio of the count after the first iteration (float arithmetic, as the reference compares them).
int orc_ldpc_decode(const orc_code_t *c, const int8_t *llr, uint8_t *out, int max_iter, int stall_it, float stall_ratio) {
  orc_state_t *s = malloc(sizeof *s);
  if (!s || c->z != Z) { free(s); return -1; }
  const int mb = c->mb;
  for (int v = 0; v < c->k; v++) s->L[v] = llr[v];
  for (int chk = 0; chk < c->m; chk++) s->L[c->k + (chk % mb) * Z + chk / mb] = llr[c->k + chk];
  memset(s->R, 0, sizeof s->R);
  int used = -1, first = 0;
  for (int it = 0; it < max_iter; it++) {
    for (int step = 0; step < mb; step++) layer(c, s, (it & 1) ? mb - 1 - step : step);
    const int bad = unsat(c, s);
    if (!bad) { used = it + 1; break; }
    if (stall_it > 1 && it == stall_it - 1) { if ((float)bad > stall_ratio * (float)first) { used = -3; break; } }
    else if (it == 0 && stall_it > 1) first = bad;
  }
  for (int v = 0; v < c->k; v++) out[v] = s->L[v] < 0;
  for (int chk = 0; chk < c->m; chk++) out[c->k + chk] = s->L[c->k + (chk % mb) * Z + chk / mb] < 0;
  free(s);
  return used;
}

uint32_t orc_crc32c(const uint8_t *p, int n) {
  uint32_t c = 0xffffffffu;
  for (int i = 0; i < n; i++) {
    c ^= p[i];
    for (int k = 0; k < 8; k++) c = (c >> 1) ^ (0x82f63b78u & (0u - (c & 1)));
  }
  return ~c;
}

typedef struct {
  const int8_t *llr; const int64_t *off; const int32_t *rate; int count, max_iter, stall_it; float ratio;
  uint8_t *out; int32_t *its; uint8_t *ok; int next; pthread_mutex_t mu; orc_code_t codes[4];
} batch_t;

// The block check of liblizard/src/lizard_phy.c:1828-1868: 476 bytes packed MSB first from bits 0..3807, their
// CRC-32C against bits 3808..3839 read MSB first.
static void *batch_worker(void *arg) {
  batch_t *b = arg;
  uint8_t *bits = malloc(7680);
  for (;;) {
    pthread_mutex_lock(&b->mu);
    const int i0 = b->next; b->next += 16;
    pthread_mutex_unlock(&b->mu);
    if (i0 >= b->count) break;
    for (int i = i0; i < i0 + 16 && i < b->count; i++) {
      const orc_code_t *c = &b->codes[lizg_code_of_rate(b->rate[i])];
      b->its[i] = orc_ldpc_decode(c, b->llr + b->off[i], bits, b->max_iter, b->stall_it, b->ratio);
      uint8_t *o = b->out + b->off[i] / 8;
      for (int j = 0; j < c->n / 8; j++) {
        uint8_t v = 0;
        for (int t = 0; t < 8; t++) v = (uint8_t)(v << 1 | bits[8 * j + t]);
        o[j] = v;
      }
      const uint32_t want = (uint32_t)o[476] << 24 | (uint32_t)o[477] << 16 | (uint32_t)o[478] << 8 | o[479];
      b->ok[i] = orc_crc32c(o, 476) == want;
    }
  }
  free(bits);
  return 0;
}

int orc_ldpc_batch(const int8_t *llr, const int64_t *off, const int32_t *rate, int count, int max_iter, int stall_it,
                   float stall_ratio, uint8_t *out, int32_t *its, uint8_t *ok, int threads) {
  batch_t b = { llr, off, rate, count, max_iter, stall_it, stall_ratio, out, its, ok, 0, PTHREAD_MUTEX_INITIALIZER, {{0}} };
  for (int t = 0; t < 4; t++) if (orc_code_init(&b.codes[t], LIZG_CODES[t].rate)) return -1;
  for (int i = 0; i < count; i++) if (lizg_code_of_rate(rate[i]) < 0) return -1;
  if (threads < 1) threads = 1;
  pthread_t th[256];
  if (threads > 256) threads = 256;
  for (int t = 1; t < threads; t++) pthread_create(&th[t], 0, batch_worker, &b);
  batch_worker(&b);
  for (int t = 1; t < threads; t++) pthread_join(th[t], 0);
  return 0;
}

// Harness around the reference codec compiled from its own sources (oracle/Makefile builds it into oracle/_ref/
// only where the reference tree is present). TEST INFRASTRUCTURE ONLY: it lets the tests hold the oracle's
// restatement to the reference's own outputs, and lets the CPU baseline time the reference decoder. It defines the
// two globals the codec expects its host to provide (liblizard/core/cpu/codec.c:49) and exports plain entry points.
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "ldpc.h"
#include "lizard_phy.h"
#include "internal.h"

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

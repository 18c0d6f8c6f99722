// Oracle: a plain-C restatement of the reference receiver's integer and floating-point arithmetic on the hot path
// (liblizard/src/ldpc.c, liblizard/src/layout.c, liblizard/src/lizard_phy.c). TEST INFRASTRUCTURE ONLY: the parity
// tests, the smoke check and the CPU-baseline leg of the benchmark call it to check or time against; nothing in the
// product links it. Every function cites the reference lines it restates.
//
// Parity pins: the LDPC tables are held to the reference's recorded H hashes (liblizard/test/ldpc_table.c:20); the
// CRC to the standard check value (liblizard/test/crc_check.c:20); the encoder, whitening and bit map to the SPEC 7.4
// vectors (research/SPEC.md:1181-1251, committed under tests/golden/); and the decoder to outputs of the reference
// itself, compiled from its sources here (oracle/Makefile -> oracle/_ref/), on seeded random channels.
#ifndef LIZARD_ORACLE_H
#define LIZARD_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

// One LDPC code as the reference's ldpc_init lays it out (liblizard/src/ldpc.c:50-113).
typedef struct {
  int rate, z, mb, kb, n, k, m, np, nt, edges;
  int rowptr[31];          // data circulants of block row r: [rowptr[r], rowptr[r + 1])
  int col[160], shift[160];
} orc_code_t;

int orc_code_init(orc_code_t *c, int rate);
// FNV-1a over H's row pointers and column indices, as liblizard/test/ldpc_table.c:13-18 hashes them.
uint32_t orc_h_hash(const orc_code_t *c);
// Systematic staircase encode, one bit a byte (liblizard/src/ldpc.c:117-126).
void orc_ldpc_encode(const orc_code_t *c, const uint8_t *data, uint8_t *cw);
// Layered normalised min-sum with the stall rule, in the arithmetic of the reference's four-times kernel
// (liblizard/src/ldpc.c:340-423 SSE4.1, 1080-1172 decode). Returns iterations used, -1 at the cap, -3 on a stall.
int orc_ldpc_decode(const orc_code_t *c, const int8_t *llr, uint8_t *out, int max_iter, int stall_it, float stall_ratio);
// CRC-32C, reflected 0x82F63B78, init and xorout all ones (liblizard/src/layout.c:44-54).
uint32_t orc_crc32c(const uint8_t *p, int n);

// A batch of codewords of mixed rates decoded on `threads` host threads (each codeword independent). llr holds
// codeword i at llr + off[i], its rate index in rate[i]. out gets the n hard bits of each packed MSB first at
// out + off[i] / 8; its[i] the decoder's return; ok[i] 1 where the first 476 bytes' CRC-32C equals bits 3808..3839.
int orc_ldpc_batch(const int8_t *llr, const int64_t *off, const int32_t *rate, int count, int max_iter, int stall_it,
                   float stall_ratio, uint8_t *out, int32_t *its, uint8_t *ok, int threads);

#ifdef __cplusplus
}
#endif
#endif

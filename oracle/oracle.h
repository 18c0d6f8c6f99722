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
#include <stddef.h>
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

// ------------------------------------------------------------------ the receiver (oracle_phy.c)
typedef struct orc_fmt orc_fmt_t;
// The format at (n, subch, span) (liblizard/src/lizard_phy.c:485-562), NULL for none.
orc_fmt_t *orc_fmt_new(int n, int subch, int span);
void orc_fmt_free(orc_fmt_t *f);
// The rate profile (liblizard/src/lizard_phy.c:578-621): tiers' rate, blocks and slots; returns the tier count.
int orc_tiers_for(int subch, int32_t *rate, int32_t *blocks, int32_t *slots);
int orc_fmt_info(const orc_fmt_t *f, int32_t *info);
int orc_fmt_tables(const orc_fmt_t *f, int32_t *pos, int16_t *uv, uint8_t *white, int32_t *btier, int32_t *bslot, int32_t *erase, double *hole_inv);
int orc_fmt_perm(const orc_fmt_t *f, int tier, int32_t *perm);
// The detrended spectrum of a row-major grid in FP64 at the used coefficients, pos order (erases grid in place).
int orc_spectrum(const orc_fmt_t *f, float *grid, double *coef, double *proj_out);
// The pilots' grid shift (liblizard/src/lizard_phy.c:280-329).
int orc_pilot_align(const orc_fmt_t *f, const float *coef, float d[2]);
// Soft values of every slot (x86-64 arithmetic), each sub-channel's estimate and rms.
int orc_demap(const orc_fmt_t *f, const float *coef, const float *turn, int8_t *llrf, double *sub_est, float *sub_rms);
// The block stage: decline, bit map, LDPC (max_iter, stall 9 / 0.95), CRC, pilots.
int orc_blocks(const orc_fmt_t *f, const int8_t *llrf, const double *sub_est, const float *sub_rms, const float *coef,
               const float *turn, int max_iter, uint8_t *blocks, uint8_t *ok, int8_t *its, float *est, float *pilot);

// The sampler's exact walk (liblizard/src/acquire.c:5121-5196): reg = H (9) then the node mesh's (dx, dy).
int orc_layout_nodes(int side, float *pos);
int orc_sample_grid(int n, int span, const uint8_t *luma, int w, int h, int pitch, const float *reg, float *grid);
// The sampler as the x86-64 decode runs it (liblizard/src/acquire.c:5302-5440 with its integer read :723-779; the calls
// of liblizard/src/lizard_phy.c:1611, 1634): the grid (n x n) in strips of 64 columns, and the shading fit's samples.
int orc_sample_decode(int n, int span, const uint8_t *luma, int w, int h, int pitch, const float *reg, float *grid, float *shade);

// The anchor search (liblizard/src/acquire.c:1876-2036, the portable build): one frame (w x h greys, rows w apart),
// H (module -> image, 9 floats), the lens model (NULL, or K, ax, ay, R, then 11 coefficients), the anchors already
// found (49 flags or NULL). Out per anchor (row-major j * 7 + i): ok, peak, dx, dy, u, v. Returns the anchors ok.
int orc_anchor_find(int span, const uint8_t *px, int w, int h, const float *H, const double *lens, const uint8_t *ok_in,
                    uint8_t *ok, float *peak, float *dx, float *dy, float *u, float *v);
// The lens model from the anchors about H (liblizard/src/acquire.c:2038-2055 anchor_model, lensm_fit's first round):
// lens out K, ax, ay, R, then 11 coefficients; 1 where a model fits.
int orc_lens_fit(int span, int iw, int ih, const float *H, const uint8_t *ok, const float *dx, const float *dy, double *lens);
// The registration's border nodes (acquire.c:1242-1374 refine_node, 5044-5058 the pass): nn * nn x (dx, dy, score,
// done) out. Returns nn.
int orc_border_nodes(int span, const uint8_t *px, int w, int h, const float *H, const double *lens, float *nodes_out);
// The code registered from the anchors (liblizard/src/acquire.c:2128-2197 anchor_register): px the frame, rim the border
// search's image (the frame, or its border blur), H the corners' homography (in) and the registration's (out), quad
// the corners in the image (in, out as moved), mpx pixels a module. Out per anchor: ok, peak, dx, dy, u, v; lens the
// model about H. Returns 1 where it holds, 0 where not, -1 on no memory.
int orc_anchor_register(int span, const uint8_t *px, const uint8_t *rim, int w, int h, float *H, float *quad, float mpx, uint8_t *ok,
                        float *peak, float *dx, float *dy, float *u, float *v, double *lens);

// Camera-format ingest (liblizard/api/codec.cpp:128-140; liblizard/core/ingest/develop.cpp): a frame's pixels in one of
// liz_pixfmt's formats to tight luma rows, and the develop of P010 / RAW16 / RAW10 / RAW12 (ImageFormat values).
int orc_ingest_pixels(const uint8_t *px, int w, int h, int stride, int fmt, uint8_t *out);
void orc_gamma_lut(uint8_t *t);
int orc_develop(int fmt, const uint8_t *plane, uint32_t row_stride, uint32_t pixel_stride, uint32_t x0, uint32_t y0, uint32_t bin,
                const float *levels, uint32_t ox, uint32_t oy, uint32_t w, uint32_t h, uint8_t *out, size_t out_stride);

// ---------------------------------------------------------------- the format word (oracle_fmt.c)
// Reed-Solomon over GF(256), polynomial 0x11d, roots alpha^0 .. alpha^(nroots - 1) (liblizard/src/rs.c).
void orc_rs_encode(uint8_t *cw, int k, int nroots);
int orc_rs_decode(uint8_t *cw, int n, int nroots);
int orc_rs_decode_er(uint8_t *cw, int n, int nroots, const int *eras, int neras);
// The word's geometry, encode, cell bits, the track's bits and the soft decode (liblizard/src/fmt.c, layout.c:57-87).
int orc_fmt_side_cells(int side, int reserve);
int orc_fmt_bytes(int side, int reserve);
int orc_fmt_bit(const uint8_t *cw, int bytes, int edge, int cell);
int orc_fmt_encode(int version, int fps, uint8_t *cw, int bytes);
int orc_thin_track(int side, int j);
int orc_fmt_decode(const float *q, int cells, int bytes, int32_t *vf);
// The word's soft values off a frame through a registration (liblizard/src/acquire.c:4503-4559).
int orc_fmt_read(int span, const uint8_t *px, int iw, int ih, const float *reg, const float *nodes, int nn, float *q);

#ifdef __cplusplus
}
#endif
#endif

// lizard_gb300: the LIZARD receive hot path on one GB300 (sm_103a), behind a plain C ABI.
//
// Conventions, as the reference's C API keeps them (liblizard/include/lizard.h:12-18, 50-60):
//   - every function returns 0 (or a count) on success and a negative LIZG_E_* code on failure; nothing throws
//     across this boundary; lizg_last_error() is a thread-local message for the last failure on the calling thread;
//   - buffers are the caller's; handles are opaque; a handle is used from one host thread at a time, different
//     handles may run concurrently;
//   - "dev" entry points take device pointers and a cudaStream_t passed as void* (NULL: the legacy default stream)
//     and return once the work is queued; the other entry points take host pointers and return when done.
#ifndef LIZARD_GB300_H
#define LIZARD_GB300_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  LIZG_OK = 0,
  LIZG_E_ARG = -1,      // a NULL pointer, a count or size out of range, a rate with no code
  LIZG_E_NOMEM = -2,    // a device or host allocation failed
  LIZG_E_CUDA = -3,     // a CUDA call failed (the message names it)
  LIZG_E_STATE = -4,    // the handle is in no state for the call
};

// The receiver's picture read (lizg_rx_set_read). The reference has two: its SIMD builds' decode reads the picture in
// integers (ob_sample_grid_pic, liblizard/src/acquire.c:5465-5480; the x86-64 form :5302-5440, called a strip of 64
// columns at a time and once for the shading fit, liblizard/src/lizard_phy.c:1611, 1634), its portable build with
// the exact float walk (ob_sample_grid, acquire.c:5121-5196). The two differ by up to about 1/200 of a grey level.
enum {
  LIZG_READ_DECODE = 0,  // the x86-64 decode's integer read, bit for bit (the default)
  LIZG_READ_EXACT = 1,   // the exact walk, bit for bit
};

// Thread-local text of the last failure on this thread ("" if none). Replaces liz_last_error
// (liblizard/include/lizard.h:63).
const char *lizg_last_error(void);
// Library version string.
const char *lizg_version(void);

// ---------------------------------------------------------------- LDPC + CRC-32C (rows d, e of the hot path)
//
// Rate indices are the reference's (liblizard/src/ldpc.h:30-33): 6 = 7/8 (n 4608, of which 4480 sent), 4 = 3/4
// (n 5120), 3 = 2/3 (n 5760), 2 = 1/2 (n 7680). LLRs are int8, codeword order, > 0 meaning bit 0; the 7/8 code's
// 128 never-sent bits (3840..3967) are fed as the caller knows them (+127, liblizard/src/lizard_phy.c:1823).

// Codeword length n of a rate index, 0 for a rate with no code (liblizard/src/ldpc.h:28 n).
int lizg_ldpc_n(int rate);

// Replaces ldpc_encode (liblizard/src/ldpc.h:42): k data bits in, n codeword bits out, one bit a byte. Host code.
int lizg_ldpc_encode(int rate, const uint8_t *data, uint8_t *codeword);
// The same for count codewords of one rate back to back (k bytes in, n bytes out each). Host code; the synthetic
// input generator's encoder.
int lizg_ldpc_encode_many(int rate, const uint8_t *data, int count, uint8_t *codewords);

// Replaces ob_crc32c (liblizard/src/layout.c:44-54): CRC-32C of n bytes. Host code.
uint32_t lizg_crc32c(const uint8_t *p, size_t n);

// Replaces ldpc_decode_stall (liblizard/src/ldpc.h:48) one codeword at a time, the reference's own signature and
// meaning, decoded on the GPU: n LLRs in, n hard bits out (one a byte). Returns the iterations used, -1 if the
// syndrome never cleared within max_iter, -3 if the stall rule gave the block up, or a negative LIZG_E_* - 100.
int lizg_ldpc_decode_stall(int rate, const int8_t *llr, uint8_t *out, int max_iter, int stall_it, float stall_ratio);

// A batch of codewords of mixed rates, the batched form of the reference's per-block loop
// (liblizard/src/lizard_phy.c:1775-1871, ldpc_decode_stall + bit pack + CRC-32C compare). The batch is laid out
// back to back: codeword i's n_i LLR bytes at llr + off_i, off_i = n_0 + ... + n_{i-1}. For each codeword the
// result is its n hard bits packed most significant bit first at bits + off_i / 8 (the first 476 bytes are the
// block, the next 4 its CRC as sent), its decoder return in its[i] (as lizg_ldpc_decode_stall), and ok[i] = 1 where
// the CRC-32C of the first 476 bytes equals the 32 bits after them (0 otherwise, or when its[i] < 0 the CRC is still
// computed on the hard decisions; the reference skips such blocks: a caller treats ok only where its[i] > 0).
typedef struct lizg_ldpc_plan lizg_ldpc_plan;

// Plans a batch: `rate` (count entries, host memory) fixes the layout; the plan keeps its own device copy of the
// work lists. max_iter 1..255; stall_it 0 (off) or 2..max_iter; stall_ratio as the reference's float.
lizg_ldpc_plan *lizg_ldpc_plan_new(const int32_t *rate, int count, int max_iter, int stall_it, float stall_ratio);
void lizg_ldpc_plan_free(lizg_ldpc_plan *p);
// Total LLR bytes of the planned batch (sum of n_i), and the packed output bytes (that over 8).
int64_t lizg_ldpc_plan_llr_bytes(const lizg_ldpc_plan *p);
// Decodes the planned batch from device memory into device memory, queued on `stream`.
int lizg_ldpc_plan_run_dev(lizg_ldpc_plan *p, const int8_t *d_llr, uint8_t *d_bits, int32_t *d_its, uint8_t *d_ok, void *stream);
// The same from host memory to host memory (pinned or not), waiting for the result. When all four buffers are
// page-locked (cudaHostAlloc, cudaHostRegister) and llr and bits 16-byte aligned, the decoder reads the LLRs and
// writes the results in place in host memory; otherwise the batch is staged through device memory in chunks of
// consecutive codewords (two from 64 MB of LLRs up), each chunk's copy in and out overlapping the other's decode.
// The outputs do not depend on the route or the chunking.
int lizg_ldpc_plan_run(lizg_ldpc_plan *p, const int8_t *llr, uint8_t *bits, int32_t *its, uint8_t *ok, void *stream);
// Sets the chunk count of the staged route (1..16, clamped to the codeword count); returns the count set.
int lizg_ldpc_plan_set_chunks(lizg_ldpc_plan *p, int chunks);
// in_place 1 (the default) allows the in-place route for page-locked buffers, 0 always stages.
int lizg_ldpc_plan_set_transfer(lizg_ldpc_plan *p, int in_place);
// The route the last lizg_ldpc_plan_run took: 1 in place, 0 staged.
int lizg_ldpc_plan_transfer(const lizg_ldpc_plan *p);
// Kernel launches the last run made (for the benchmark's launch count).
int lizg_ldpc_plan_launches(const lizg_ldpc_plan *p);

// No counterpart in the reference: the batch decode for callers that cannot allocate device memory (a plug-in inside
// a host application that owns the device allocator, a pipeline whose memory is reserved up front). It allocates
// nothing: its scratch (work lists, offsets, counters) is a fixed array inside the library's device image, sized for
// LIZG_NOALLOC_MAX_CODEWORDS codewords, held on every GPU that loads the library until the process exits. Inputs
// and outputs are the caller's device buffers, laid out as the plan's (codewords back to back, offsets from the
// rates); d_rate holds the count rate indices in device memory; a codeword whose rate has no code gets its = -4.
// Queued on `stream`. The first call on a device looks up the array's address there; make that first call before
// any stream capture. Every call shares the one array, so calls whose work overlaps on the GPU (other streams, other
// host threads) race; serialise them. count above the maximum is refused with LIZG_E_ARG. The address is kept for
// the life of the process: do not use this entry point across a device reset (cudaDeviceReset, or the primary
// context torn down), after which it would be stale. The four codes run one after another on `stream` (the plan API
// overlaps them on side streams), so a mixed-rate batch takes a little longer than through a plan.
enum { LIZG_NOALLOC_MAX_CODEWORDS = 8192 };
int lizg_ldpc_decode_noalloc(const int8_t *d_llr, const int32_t *d_rate, int count, int max_iter, int stall_it,
                             float stall_ratio, uint8_t *d_bits, int32_t *d_its, uint8_t *d_ok, void *stream);

// No counterpart in the reference (its decoder has one form a build): the decoder's kernel variants and their
// choice. Each code has a few variants that decode bit for bit alike and differ in the warps a codeword takes (1, 2
// or 4) and in the layer form (messages held in registers, or recomputed in a loop). Variant 0 is the default on
// every device. lizg_ldpc_autotune times every variant of every code on the current device over a seeded batch of
// `count` codewords, codeword c at ebn0_db[c mod n_ebn0] (BPSK/AWGN, the batch's LLR quantisation), and keeps the
// fastest per code for that device; choice[4] (may be NULL) receives the indices in code order 7/8, 3/4, 2/3, 1/2.
// Every later decode on the device (plans, the single-codeword call, the receiver, the allocation-free call) uses
// the kept variant.
// lizg_ldpc_set_variant fixes one by hand; lizg_ldpc_variant returns the current index and its warps a codeword and
// form (bit 0: the loop form; bit 1: the pair form, two checks a thread in 16-bit halves); lizg_ldpc_variants the
// number of variants of a rate.
int lizg_ldpc_autotune(int count, const float *ebn0_db, int n_ebn0, int32_t *choice);
int lizg_ldpc_variants(int rate);
int lizg_ldpc_variant(int rate, int32_t *wpc, int32_t *loop_form);
int lizg_ldpc_set_variant(int rate, int index);

// ---------------------------------------------------------------- the receiver (rows a-e)
//
// A receiver handle for one format: the picture size n (384, 512, 768, 1024, 1152, 1280, 1536), the sub-channels
// (a multiple of 16 from 64 to 1024: LIZARD-subch) and the ring's span in modules (128, 256, 512; 0 for 256), with the
// format's tables on the device and working buffers for up to max_frames frames a call. It is the batched, GPU
// form of the reference's per-frame codec (lizard_init and lizard_finish / lizard_finish_ext,
// liblizard/src/lizard_phy.h:177, 230-240).
typedef struct lizg_rx lizg_rx;

// The format's tables, host code, no device needed (any pointer NULL to skip). info (22 ints): n, subch, span,
// blocks, used slots, bw, vblocks, tiers, V (spectrum rows kept), pilots, then per tier (up to 4) its rate index,
// blocks and slots a block. uv: (u, v) of every used coefficient in the reference's pos order (2 x subch x 320);
// white: the whitening bit of every slot (subch x 640); each block's tier and first slot; erase: the anchors' erase
// ranges (7 lo then 7 hi); hole_inv: the shading fit's inverse normal matrix (36); detrend: the reference's
// lizard_tables layout, cx, qx, x1r, x1i, x2r, x2i (n each) then sx2, sq2 (liblizard/src/lizard_phy.h:249,
// lizard_phy.c:1928-1934); perm: every tier's bit map back to back (block slot -> codeword bit, nt each). Replaces
// the tables of lizard_init / ws_init (liblizard/src/lizard_phy.c:348-562). Returns 0, or LIZG_E_ARG for no format.
int lizg_format_tables(int n, int subch, int span, int32_t *info, int16_t *uv, uint8_t *white, int32_t *block_tier,
                       int32_t *block_slot, int32_t *erase, double *hole_inv, float *detrend, int16_t *perm);
lizg_rx *lizg_rx_new(int n, int subch, int span, int max_frames);
void lizg_rx_free(lizg_rx *r);
// info (24 ints): n, subch, span, blocks, used slots, bw, vblocks, tiers, V (spectrum rows kept), pilots, then per
// tier (up to 4) its rate index, blocks and slots a block, then the registration mesh's nx, ny.
int lizg_rx_info(const lizg_rx *r, int32_t *info);
// The registration mesh's node centres in module coordinates for a ring of span modules (the layout is span + 30
// modules square, liblizard/src/layout.c:110-117): nn = {nx, ny}; returns nx. Host code.
int lizg_layout_nodes(int span, float *node_x, float *node_y, int32_t *nn);
// Tier t's bit map: block slot i -> codeword bit (nt entries); returns nt.
int lizg_rx_perm(const lizg_rx *r, int tier, int16_t *perm);
// Kernel launches the last finish made.
int lizg_rx_launches(const lizg_rx *r);
// 1 where one of the handle's passes gave up a bounded wait (the row pass's wait for its bulk tensor copies, which
// complete in microseconds; the pass then leaves its tile), else 0. Waits for the device. Host code.
int lizg_rx_fault(lizg_rx *r);
// The picture read of the handle's later finishes from captured frames (LIZG_READ_DECODE or LIZG_READ_EXACT); returns
// the previous one, or LIZG_E_ARG. Host code.
int lizg_rx_set_read(lizg_rx *r, int read);
// The handle's LDPC kernel variant for each of its tiers (tier t's code: lizg_rx_info), chosen by timing on the
// caller's own frames: one lizg_rx_finish_luma_dev of the batch (d_luma, d_reg as that call takes them) for the
// soft values, then every variant of each tier's code timed on them in the receiver's own form (a codeword per block,
// the batch's frames x the tier's blocks); the fastest is kept by the handle for its later finishes (its format and
// batch size: the choice per picture size and code rate). All variants decode bit for bit alike, so the blocks never
// change; the global choice of lizg_ldpc_autotune, tuned on large batches of one code, is what the handle uses
// without it. Then the whole decode stage with those variants, a launch a tier on forked streams, against one
// persistent launch across the tiers (lizg_rx_set_ldpc_mixed); the faster is kept too. choice (may be NULL): 4
// entries, each tier's variant index (lizg_ldpc_variant's numbering), -1 past the format's tiers. Synchronises the
// stream. No counterpart in the reference (one decoder form a build).
int lizg_rx_autotune(lizg_rx *r, const uint8_t *d_luma, int w, int h, int pitch, int64_t frame_stride, const float *d_reg, int frames,
                     int32_t *choice, void *stream);
// The handle's decode stage: 0, a launch a tier on the tiers' own streams (the default); 1, every tier's blocks in one
// persistent launch (a queue of (tier, block) items, the longer codes first, each decoded by its code's form in a slice
// sized for the longest code: fewer launches and no tail a tier, for small batches). The blocks are the same either
// way. Returns the previous setting, or LIZG_E_ARG. Host code.
int lizg_rx_set_ldpc_mixed(lizg_rx *r, int mixed);
// Tier t's LDPC kernel variant as the handle's finishes launch it: its own after lizg_rx_autotune, else the device's
// (lizg_ldpc_variant). Host code.
int lizg_rx_variant(const lizg_rx *r, int tier);

// Per-frame outputs, device pointers, frames x blocks entries each unless noted. Required: blocks (476 bytes a block,
// the decoded bytes whether or not verified), ok (1 where the CRC-32C verified a decoded block), its (LDPC
// iterations; -1 never converged, -2 declined, -3 stalled: liblizard/src/lizard_phy.h:186-188). Optional (NULL: kept
// inside the handle): est (the block's information estimate), pilot (its pilot reading, NaN where none), align
// (frames x 3: the pilots' grid shift dx, dy and 1 where it was turned back), llrf (frames x subch x 640 soft values,
// slot order), sub_est (frames x subch doubles), sub_rms (frames x subch).
typedef struct {
  uint8_t *blocks, *ok;
  int32_t *its;
  float *est, *pilot, *align;
  int8_t *llrf;
  double *sub_est;
  float *sub_rms;
} lizg_rx_out;

// Rows c-e from spectra: d_coef holds frames x subch x 320 complex floats (re, im), each frame's detrended spectrum at
// the used coefficients in pos order (what the reference's lizard_debug reads back, liblizard/src/lizard_phy.c:1719).
// The replacement for lizard_finish_ext's path after the transform (liblizard/src/lizard_phy.c:1720-1871).
int lizg_rx_finish_coef_dev(lizg_rx *r, const float *d_coef, int frames, const lizg_rx_out *out, void *stream);
// Rows b-e from picture grids: d_grid holds frames x n x n floats (row y, column x; grey / 255), each frame's picture
// sampled at its n x n grid. The anchors' squares are erased to the shading surface, the detrend projections taken,
// the 2D FFT made and the surface's spectrum subtracted (liblizard/src/lizard_phy.c:1596-1716), then as
// lizg_rx_finish_coef_dev. d_coef (optional, NULL to skip) receives each frame's spectrum at the used coefficients
// (frames x subch x 320 complex floats, pos order). The replacement for lizard_finish(f, grid, ...)
// (liblizard/src/lizard_phy.h:236). d_grid is not modified.
int lizg_rx_finish_grid_dev(lizg_rx *r, const float *d_grid, int frames, const lizg_rx_out *out, float *d_coef, void *stream);
// The transform alone (row b: the anchors' erase, the detrend, the 2D transform) on picture grids, the used
// coefficients into d_coef (frames x subch x 320 complex, pos order), as lizard_finish computes them before the soft
// stage (liblizard/src/lizard_phy.c:1566-1716). For callers that read spectra (the refinement's tangent pictures).
int lizg_rx_spectrum_grid_dev(lizg_rx *r, const float *d_grid, int frames, float *d_coef, void *stream);
// Rows a-e from captured frames: d_luma holds frames 8-bit luma images (w x h, rows pitch bytes apart, frames
// frame_stride bytes apart); d_reg holds each frame's registration, 9 + 2 nx ny floats: the homography H (module
// coordinates to image pixels, h[8] = 1, liblizard/src/internal.h:105-112) then the node mesh's (dx, dy) pixel
// displacements row by row (liblizard/src/internal.h:123-124, what the reference's acquisition leaves held). Each
// frame's picture is sampled on its n x n grid by the handle's read (lizg_rx_set_read), the shading fit's samples as
// the reference's finish takes them, then as lizg_rx_finish_grid_dev. d_grid (optional) receives the sampled grids
// (frames x n x n). The replacement for lizard_finish(f, NULL, ...) on a held registration
// (liblizard/src/lizard_phy.c:1566-1871).
int lizg_rx_finish_luma_dev(lizg_rx *r, const uint8_t *d_luma, int w, int h, int pitch, int64_t frame_stride, const float *d_reg,
                            int frames, const lizg_rx_out *out, float *d_grid, float *d_coef, void *stream);
// lizg_rx_finish_luma_dev replayed from a CUDA graph: the first call with a given set of buffers and sizes captures
// the whole per-frame pipeline on the handle's own stream; later calls with the same arguments launch the captured
// graph on `stream` in one call (different arguments capture again). For a caller that decodes frame after frame
// into the same buffers, where the launches would otherwise cost more than the work.
int lizg_rx_finish_luma_graph(lizg_rx *r, const uint8_t *d_luma, int w, int h, int pitch, int64_t frame_stride, const float *d_reg,
                              int frames, const lizg_rx_out *out, float *d_grid, float *d_coef, void *stream);
// lizg_rx_finish_luma_dev from host memory, for a caller with no device buffers of its own (the reference's codec
// finishing a frame it registered on the CPU): luma frames (w x h, rows pitch bytes apart, frames frame_stride apart)
// and their registrations (frames x (9 + 2 nx ny) floats) copied to the handle's device buffers (grown to the largest
// call), decoded on the handle's own stream, and blocks (frames x blocks x 476), ok and its (frames x blocks) written
// before the call returns. Returns the blocks verified. The replacement for lizard_finish(f, NULL, blocks, ok, res)
// on a held registration (liblizard/src/lizard_phy.h:236), its per-block iterations as lizard_block_stats gives them.
int lizg_rx_finish_luma_host(lizg_rx *r, const uint8_t *luma, int w, int h, int pitch, int64_t frame_stride, const float *reg, int frames,
                             uint8_t *blocks, uint8_t *ok, int32_t *its);

// ---------------------------------------------------------------- the multi-stream engine
//
// The device side of the reference's batched receiver engine (liz_receiver_new / _push / _batch_cap,
// liblizard/include/lizard.h:252-294) for frames already registered: many camera streams of different formats
// decoded together. An engine holds one receiver handle per picture format (lizg_engine_add_format returns its
// index; lizg_engine_rx the handle, for lizg_rx_info and the like). lizg_engine_run_dev takes one batch per format
// (each format at most once a run): the format's frames, registrations and outputs as lizg_rx_finish_luma_dev
// takes them. By default every batch runs on its format's own stream, replayed from that format's CUDA graph
// (captured on the first run with those buffers), forked from `stream` and joined back to it, so the formats' work
// overlaps on the GPU. Queued; returns once launched. lizg_engine_launches: the kernels the last run launched.
//
// lizg_engine_set_mixed(e, 1) runs the batches stage-wise across formats instead, as work queues: every stage one
// launch over every format's items whatever their picture sizes and codes: the shading sums with the sampler's tables,
// the column pass's (frame, column tile) items, the surface factors, the row pass's (frame, row tile) items, the
// pilots' fit, the soft values, the block stage, and the decode as one persistent grid over every format's (tier,
// block) items of all four codes (the 1/2 code's first); 8 launches for up to 8 formats. The whole run is one CUDA
// graph, captured on the first run with those batches. The outputs are the same bit for bit either way.
// Returns the previous setting. lizg_engine_autotune first tunes each format's decode on its batch
// (lizg_rx_autotune on the format's handle), then runs the batches both ways (each four times, the first not timed),
// keeps the faster and returns it (0 or 1); ms (may be NULL) gets the two best times, per format first.
// Both write the batches' outputs as a run does.
typedef struct lizg_engine lizg_engine;
typedef struct {
  int format;
  const uint8_t *d_luma;
  int w, h, pitch;
  int64_t frame_stride;
  const float *d_reg;
  int frames;
  lizg_rx_out out;
} lizg_engine_batch;
lizg_engine *lizg_engine_new(void);
void lizg_engine_free(lizg_engine *e);
int lizg_engine_add_format(lizg_engine *e, int n, int subch, int span, int max_frames);
lizg_rx *lizg_engine_rx(lizg_engine *e, int format);
int lizg_engine_run_dev(lizg_engine *e, const lizg_engine_batch *b, int nb, void *stream);
int lizg_engine_launches(const lizg_engine *e);
int lizg_engine_set_mixed(lizg_engine *e, int mixed);
int lizg_engine_autotune(lizg_engine *e, const lizg_engine_batch *b, int nb, void *stream, float *ms);

// ---------------------------------------------------------------- the batching front (camera frames in, blocks out)
//
// The reference's receiver engine as the apps drive it (liz_receiver_new / _push / _batch_cap / _stats / _series /
// _wants_luma / _free, liblizard/include/lizard.h:252-294), for frames whose registration is already held (the
// registration front half is the caller's). A push copies the luma plane and its registration into a page-locked
// slot of the front's, or drops the frame when every slot waits (counted), and calls release(user, tag) before it
// returns: the caller's buffer is its own again. It never waits on the device. The front's own thread takes the
// waiting frames in push order, up to the batch cap of one frame size at a time (a launch goes as soon as a frame
// waits), decodes them in one lizg_rx_finish_luma_dev call on its own stream, and calls frame() for each from that
// thread: its tag and timestamp, its verified blocks packed (count x 476 bytes, as liz_decode packs them), and every
// block's CRC verdict and LDPC iterations. One handle is one format: n, subch, span as lizg_rx_new takes them.
typedef struct lizg_receiver lizg_receiver;
typedef struct {
  int n, subch, span;      // the format of the frames pushed
  int max_w, max_h;        // the largest luma plane a push brings
  int batch_cap;           // the most frames a launch takes, 1 to 32 (0: 32)
  int slots;               // frames that may wait, 1 to 128 (0: 64)
  int read;                // LIZG_READ_DECODE or LIZG_READ_EXACT
  void (*frame)(void *user, uint64_t tag, int64_t timestamp_ns, const uint8_t *verified, int count, const uint8_t *ok,
                const int32_t *its, int blocks);   // NULL none; called from the front's thread
  void (*log)(void *user, const char *line);       // NULL none; called from the front's thread
  void *user;
} lizg_receiver_config;
// NULL on failure (lizg_last_error). Replaces liz_receiver_new (liblizard/include/lizard.h:270).
lizg_receiver *lizg_receiver_new(const lizg_receiver_config *config, void (*release)(void *user, uint64_t tag));
// Every frame pushed decoded and delivered, then the handle let go. Replaces liz_receiver_free (:271).
void lizg_receiver_free(lizg_receiver *r);
// One frame's luma plane (w x h, rows stride bytes apart) at timestamp_ns on the camera's clock, with its registration
// (9 + 2 nx ny floats: H, then the node mesh, as lizg_rx_finish_luma_dev takes it). Copied or dropped, and
// release(tag) called, before it returns. LIZG_OK, or LIZG_E_ARG. Replaces liz_receiver_push (:274), the registration
// added.
int lizg_receiver_push(lizg_receiver *r, const uint8_t *luma, int w, int h, int stride, int64_t timestamp_ns, uint64_t tag,
                       const float *reg);
// The most frames a launch takes, 1 to 32 (0: 32). Replaces liz_receiver_batch_cap (:287).
void lizg_receiver_batch_cap(lizg_receiver *r, int frames);
// 1: frames come as luma planes. Replaces liz_receiver_wants_luma (:279).
int lizg_receiver_wants_luma(lizg_receiver *r);
// A snapshot as JSON (frames in, dropped, decoded, waiting, batches and their mean size B, the cap, blocks verified and
// new, GPU ms a frame, frames a second, goodput), valid until the next call on the handle. Replaces
// liz_receiver_stats (:280).
const char *lizg_receiver_stats(lizg_receiver *r);
// The format's version (subch / 16), then 8 doubles a frame decoded after since_ms on the camera's clock, oldest
// first: ms, verified blocks, new blocks, decoded (1, or 0 where the batch failed), the pilots' mean reading and its
// standard error over the even blocks, then over the odd (NaN where none read). At most cap doubles; returns how many.
// Replaces liz_receiver_series (:284).
int lizg_receiver_series(lizg_receiver *r, double since_ms, double *out, int cap);
// Waits until every frame pushed so far is decoded and delivered; returns the frames decoded. No counterpart in the
// reference (its receiver only ever runs on): for a caller that must know its frames are through (a test, a shutdown).
int lizg_receiver_flush(lizg_receiver *r);

// ---------------------------------------------------------------- registration assist: the anchor search
//
// Replaces anchor_find (liblizard/src/acquire.c:1876-2036), the registration's search for the picture's 7 x 7 anchors
// about where H (and the lens model, when given) puts them, for a batch of frames on the GPU. The arithmetic is the
// reference's portable build's (its scalar twins of the SIMD paths): a window of (16 + 2 r)^2 samples a / 16 modules
// apart (a = span / 64 the anchor's side, r = ceil(3 / (a / 16)) steps of reach), the normalised correlation with
// the anchor's two concentric squares at every offset, the first largest, a parabola each way. Anchor k of frame f
// (k = j * 7 + i, row j, column i) is out[f * 49 + k]: ok (the peak reaches 0.6 off the window's edge), the peak,
// dx, dy (its middle in the image less where H puts it, pixels) and u, v (its middle in the image).
// Frame f: its w x h greys at d_luma + f * frame_stride (rows w apart, as the reference's image_t), its H (module ->
// image, 9 floats) at d_H + f * h_stride (a receiver's registrations can be passed as they are: h_stride = 9 + 2 nx ny),
// its lens model at d_lens + f * 15 (K, ax, ay, R, then 11 coefficients, the reference's lensm_t) or d_lens NULL for
// none. d_skip (frames x 49, may be NULL) marks anchors found before: their outputs are left as they are.
typedef struct {
  uint8_t *ok;
  float *peak, *dx, *dy, *u, *v;
} lizg_anchor_out;
int lizg_anchor_find_dev(int span, const uint8_t *d_luma, int w, int h, int64_t frame_stride, const float *d_H, int h_stride,
                         const double *d_lens, const uint8_t *d_skip, int frames, const lizg_anchor_out *out, void *stream);

// ---------------------------------------------------------------- camera-format ingest
//
// Replaces the host's conversion of a captured image to the decoder's luma: liz_decode's pixel formats
// (liblizard/api/codec.cpp:128-140; ob_luma, liblizard/src/acquire.c:67-83) and the camera develop of P010, RAW16,
// RAW10 and RAW12 (liblizard/core/ingest/develop.cpp:9-102, developLuma), on the GPU for a batch of frames, byte for
// byte the reference's. Outputs are tight luma rows: frame f's w x h bytes at d_luma + f w h.
enum { LIZG_PIX_GREY8 = 1, LIZG_PIX_RGBX8 = 2, LIZG_PIX_RGBA8 = 3, LIZG_PIX_BGRA8 = 4 };               // liz_pixfmt's values
enum { LIZG_RAW_RAW16 = 0x20, LIZG_RAW_RAW10 = 0x25, LIZG_RAW_RAW12 = 0x26, LIZG_RAW_P010 = 0x36 };   // ImageFormat's values
// frames x (w x h pixels of fmt, rows stride bytes apart) at d_px + f frame_stride.
int lizg_ingest_pixels_dev(const uint8_t *d_px, int w, int h, int stride, int64_t frame_stride, int fmt, int frames, uint8_t *d_luma, void *stream);
// A camera frame's plane 0 as the reference's RawFrame (develop.h): its format, rowStride bytes a row, pixelStride
// bytes a sample (RAW16, P010), the developed frame's (0, 0) at sample (x0, y0), bin 1 or 2 (P010: 1), levels: the
// black level per 2 x 2 position, the white level, the gain per position.
typedef struct {
  int format;
  uint32_t row_stride, pixel_stride, x0, y0, bin;
  float levels[9];
} lizg_raw_frame;
// The developed crop of w x h pixels at (ox, oy) of frames planes (frame f at d_plane + f plane_stride, each
// plane_bytes long; a crop that would read past a row or the plane is refused with LIZG_E_ARG).
int lizg_develop_dev(const lizg_raw_frame *r, const uint8_t *d_plane, int64_t plane_bytes, int64_t plane_stride, int frames, uint32_t ox,
                     uint32_t oy, uint32_t w, uint32_t h, uint8_t *d_out, void *stream);

// ---------------------------------------------------------------- the sender (GPU encoder)
//
// Replaces the sender's lizard_encode + lizard_paint_grey (liblizard/src/lizard_phy.c:1087-1236, 700-716; with
// lizard_parity and lizard_fmt_fps, :446-450, 478-481) for a batch of frames: blocks to the ring's drive and its grey
// page. The transform's floats are this library's, so a drive value may differ from the reference's in its last
// bits and a grey level by one at a rounding tie; every block reads back the same.
typedef struct lizg_encoder lizg_encoder;
// The format (n, subch, span as lizg_rx_new takes them) and the most frames a call.
lizg_encoder *lizg_encoder_new(int n, int subch, int span, int max_frames);
void lizg_encoder_free(lizg_encoder *e);
// The display rate the format word states (lizard_fmt_fps): 0..255, 0 none (the default).
int lizg_encoder_fps(lizg_encoder *e, int fps);
// blocks, pxm (pixels a module), px (the drive's side), W (the page's side, px + 4 pxm), max_frames.
int lizg_encoder_info(const lizg_encoder *e, int32_t *out);
// d_blocks: frames x blocks x 476 bytes. pilots: the painted count's two bits (lizard_parity, 0..3). Out (either may be
// NULL, not both): d_drive frames x px x px floats in 0..1, d_grey frames x W x W bytes.
int lizg_encode_dev(lizg_encoder *e, const uint8_t *d_blocks, int frames, int pilots, float *d_drive, uint8_t *d_grey, void *stream);
// The border's cell kinds of a ring of span modules with the format word (version, fps) painted: (span + 30)^2 bytes,
// 2 dark, 1 light, 0 the picture's, | 8 on the word's cells (liblizard/src/layout.c:69-141, CELL_*). Host only.
// Returns the side.
int lizg_layout_kind(int span, int version, int fps, uint8_t *kind);

// ---------------------------------------------------------------- format word
//
// Replaces the read of the format word when a registration is held (liblizard/src/lizard_phy.c:1553-1556:
// ob_thin_read_fmt, liblizard/src/acquire.c:4503-4559, then ob_fmt_decode, liblizard/src/fmt.c:54-86) for a batch of
// registered frames, so that a batch can learn each frame's version on the device. Soft values and words are the
// reference's bit for bit.
// The word's cells a side and codeword bytes in a ring of span modules (128, 256, 512: 32 / 16, 64 / 32, 128 / 64).
int lizg_fmt_geometry(int span, int32_t *cells, int32_t *bytes);
// frames x (w x h luma, rows w apart) at d_luma + f frame_stride; d_reg: frames x reg_stride floats, H (9) then
// (dx, dy) of the layout's nodes, as the receiver takes it. Out: d_q (NULL, or frames x 4 cells soft values,
// side * cells + cell, > 0 dark; 0 where the band was not read) and d_word (frames x 4: read, ok, version, fps).
int lizg_fmt_read_dev(int span, const uint8_t *d_luma, int w, int h, int64_t frame_stride, const float *d_reg, int reg_stride, int frames,
                      float *d_q, int32_t *d_word, void *stream);
// ob_fmt_decode alone on soft values read elsewhere (lizard_fmt_check, lizard_phy.c:1881-1889): frames x 4 cells in,
// frames x 4 (1, ok, version, fps) out.
int lizg_fmt_decode_dev(int span, const float *d_q, int frames, int32_t *d_word, void *stream);

// ---------------------------------------------------------------- registration assist: the border nodes
//
// Replaces the registration's border pass (liblizard/src/acquire.c:5044-5058: refine_node, acquire.c:1242-1374, over
// the border lattice's marked nodes in rings outward from the corners) for a batch of frames: the corners taken as
// measured, each other node's displacement from its measured neighbours and the border pattern's correlation,
// bit for bit the reference's portable build. d_H: frames x h_stride floats (H first); d_lens: frames x 15 doubles
// (K, ax, ay, R, 11 coefficients, as lizg_refine_dev fits them) or NULL. Out: d_nodes, frames x nn x nn x (dx, dy,
// score, done), nn the layout's nodes an axis (lizg_layout_nodes).
int lizg_border_nodes_dev(int span, const uint8_t *d_luma, int w, int h, int64_t frame_stride, const float *d_H, int h_stride,
                          const double *d_lens, int frames, float *d_nodes, void *stream);

// ---------------------------------------------------------------- registration refined from the pilots
//
// Gauss-Newton on the 8 homography parameters against the known pilots, measured through the receiver's own front
// (lizg_rx_spectrum_grid_dev), the Jacobian from eight tangent pictures (forward mode); the plain registration kept
// where the pilots' mismatch does not fall. Not in the reference: a refinement of the held registration against the
// pilots, run ahead of the soft stage.
typedef struct lizg_gn lizg_gn;
// The format, and the frames refined at once (chunk, 1..64: each holds 9 pictures and their spectra).
lizg_gn *lizg_gn_new(int n, int subch, int span, int chunk);
void lizg_gn_free(lizg_gn *g);
// d_reg: frames x (9 + 2 nodes) registrations, H refined in place (the mesh kept). steps: Gauss-Newton steps (the
// benchmark takes 3). Out (either NULL): d_loss, each frame's final mismatch; d_improved, 1 where a step was kept.
int lizg_gn_refine_dev(lizg_gn *g, const uint8_t *d_luma, int w, int h, int64_t frame_stride, float *d_reg, int frames, int steps, float *d_loss,
                       int32_t *d_improved, void *stream);
// The 9 pictures a step reads (the sampled picture, then its tangents in h0..h7), frames x 9 x n x n, frames <= chunk.
int lizg_gn_pictures_dev(lizg_gn *g, const uint8_t *d_luma, int w, int h, int64_t frame_stride, const float *d_reg, int frames, float *d_pics,
                         void *stream);

// ---------------------------------------------------------------- registration assist: refinement from the anchors
//
// For frames registered by a homography alone (a finder's four corners), the lens the camera adds, found from the
// anchors and written into the registration's node mesh, on the GPU. Each of `rounds` rounds (1..8) searches the
// anchors not yet found (lizg_anchor_find_dev's search, through H and, after the first round, the lens model so
// far) and fits the lens model the found anchors give about H: the reference's anchor_model
// (liblizard/src/acquire.c:2038-2055: the four corner nodes with no displacement and the anchors found, the model of
// 8 + K terms, K = 0..3 chosen by AICc, lensm_fit's first round 1630-1669), in double. This refinement keeps H and
// writes the model's displacement at every node into the mesh (zeros where no model fits); lizg_anchor_register_dev
// below runs the reference's whole registration from the anchors (H refitted, the corners judged).
// d_reg: frames x (9 + 2 nx ny) floats, H kept, the mesh overwritten. d_found (frames, may be NULL): anchors found;
// d_lens (frames x 15, may be NULL): the model (K, ax, ay, R, 11 coefficients). The handle keeps the anchors'
// device buffers for up to max_frames frames of one ring span (128, 256 or 512).
typedef struct lizg_refiner lizg_refiner;
lizg_refiner *lizg_refiner_new(int span, int max_frames);
void lizg_refiner_free(lizg_refiner *r);
int lizg_refine_dev(lizg_refiner *r, const uint8_t *d_luma, int w, int h, int64_t frame_stride, float *d_reg, int frames, int rounds,
                    int32_t *d_found, double *d_lens, void *stream);
// The reference's own registration from the anchors (liblizard/src/acquire.c:2128-2197 anchor_register, its portable
// build) for a batch of frames whose H a finder's four corners gave: up to six rounds of the anchor search through the
// homography the anchors found so far say (anchor_homo, :2062-2094, refitted each round) and the lens model they say
// about it, held to the robust rule (anchor_model_free, :2101-2118: a reading further from the model than half a
// module or three robust spreads is no longer found), until a round finds nothing new; then each corner judged by
// that map: one further than 3 modules from where the anchors put it searched again (the border node search on the
// corner, d_rim, through the corners' H and the joint model of the anchors and the kept corners), kept where it
// correlates 0.35 or more, else the model's place, and H made again from the four (homography, :611-654); then the
// anchors' model about H (anchor_model). It holds where 12 or more anchors and a model remain. d_reg: frames x
// (9 + 2 nx ny) floats: in, the corners' H; out, the registration's H and the model's displacement at every node
// (zeros where it did not hold). d_rim: the border search's image (the frame's border blur as the reference's
// acquisition makes it, or NULL: d_luma itself), frames as d_luma. d_quad (frames x 8, may be NULL: the corner nodes
// through H): the corners in the image, out as moved; pixels a module are their sides over the lattice's. d_held
// (frames, may be NULL): 1 where it held. d_lens (frames x 15, may be NULL): the model about H. anchors (may be NULL):
// each frame's 49 anchors (ok, peak, dx and dy about H, u, v).
int lizg_anchor_register_dev(lizg_refiner *r, const uint8_t *d_luma, const uint8_t *d_rim, int w, int h, int64_t frame_stride, float *d_reg,
                             float *d_quad, int frames, int32_t *d_held, double *d_lens, const lizg_anchor_out *anchors, void *stream);

// ---------------------------------------------------------------- registration refined by its adjoint (H and the anchor field)
//
// No reference counterpart: a refinement of the held registration before the soft stage, Gauss-Newton over the 8
// homography parameters and a 7 x 7 field of displacements at the anchors' centres (carried into the mesh as the
// reference's interior fill carries its anchors' readings, liblizard/src/acquire.c:2199-2217, 2335-2385: cubic
// Hermite knots at the node lattice's ends, held at zero, and at the anchors' centres), against three terms: the
// known pilots as the receiver's own front measures them, the timing track's cells, and the anchors' centres where
// the anchor search found them. The gradient comes from one adjoint pass (the pilots' residuals inverse-transformed
// to every picture sample, the warp recomputed at each sample); the step's normal equations take the pilots' J^T J
// from the tangents' own Gram scaled by the pilots' share of the picture's energy, the track's and the anchors'
// exactly. Each step is kept where the weighted mismatch falls, halved from the best registration otherwise; the
// registration given is the baseline and the fallback. chunk: frames a pass (1..256; at n = 1536 about 28 MB of
// device memory a frame; a chunk of 152, a frame an SM for the step's solve, suits a GB300).
// d_reg: frames x (9 + 2 nx ny), refined in place (H and the mesh). anchors (may be NULL: no anchor term): the anchor
// search's outputs through the same registration (lizg_anchor_find_dev, frames x 49 each). d_gate (frames bytes, may
// be NULL): 0 leaves a frame's registration as it is and spends nothing on it (for instance the frames whose plain
// decode verified every block). d_loss, d_improved (frames, may be NULL): the weighted mismatch at the registration
// kept, and 1 where a step was kept.
enum { LIZG_FIELD_PARAMS = 8 + 2 * 49 };
typedef struct lizg_field lizg_field;
lizg_field *lizg_field_new(int n, int subch, int span, int chunk);
void lizg_field_free(lizg_field *g);
int lizg_field_refine_dev(lizg_field *g, const uint8_t *d_luma, int w, int h, int64_t frame_stride, float *d_reg, int frames, int steps,
                          const lizg_anchor_out *anchors, const uint8_t *d_gate, float *d_loss, int32_t *d_improved, void *stream);
// The three terms at given parameters, unweighted, for checks: d_theta frames x LIZG_FIELD_PARAMS (H[0..7], then the
// field's (x, y) a knot, row by row, pixels) about the registration d_reg (its mesh the field is added to); d_terms
// frames x 3 x (1 + LIZG_FIELD_PARAMS) doubles: per term (pilots, track, anchors) its loss (a sum of squares) then
// its gradient in the parameters. frames at most the chunk.
int lizg_field_terms_dev(lizg_field *g, const uint8_t *d_luma, int w, int h, int64_t frame_stride, const float *d_reg, const float *d_theta,
                         int frames, const lizg_anchor_out *anchors, double *d_terms, void *stream);

#ifdef __cplusplus
}
#endif
#endif

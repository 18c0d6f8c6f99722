// Internal declarations shared by the host shim (api.cpp) and the kernels (*.cu). Not part of the C ABI.
#ifndef LIZG_INTERNAL_H
#define LIZG_INTERNAL_H
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <atomic>
#include <vector>
#include "lizard_gb300.h"

namespace lizg {

// A kernel's opt-in to more than 48 KB of dynamic shared memory, made once a device (the attribute is the current
// device's, so a process driving several GPUs sets it on each). Setting it twice is harmless, so a race only repeats it.
struct SmemOptIn {
  std::atomic<uint64_t> done{0};
  cudaError_t set(const void *kernel, int bytes) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const uint64_t bit = dev >= 0 && dev < 64 ? 1ull << dev : 0;
    if (bit && (done.load(std::memory_order_acquire) & bit)) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess && bit) done.fetch_or(bit, std::memory_order_release);
    return e;
  }
};


constexpr int kSubDev = 320, kTurnsDev = 4096;

// A format's tables on the device plus the batch's frame count, passed by value to the receive kernels.
struct FmtDev {
  int n, subch, blocks, frames, npilot, V;
  float turn_scale;                  // (float)4096 / (float)n
  int tier_first[4], tier_blocks[4], tier_slots[4], tier_nt[4], tier_k[4];
  const int16_t *uv;                 // (u, v) a coefficient, pos order
  const uint8_t *white;              // whitening bit a frame slot
  const int16_t *perm[4];            // per tier: block slot -> codeword bit
  const int32_t *block_tier, *block_slot;
  const int32_t *pilot_coef;         // the block tails' coefficients in block order
  const uint8_t *pilot_white;        // their whitening (bit 0 real, bit 1 imaginary)
  const float2 *rot;                 // cos, sin of 2 pi k / 4096
};

// A format's transform tables (row b), passed by value to the transform kernels.
struct FftDev {
  int n, vrows;                      // picture size; rows v kept (the used coefficients' v <= vrows - 1)
  const float2 *tws;                 // the passes' twiddles: pass s at Ns, [r - 1][k] = e^{-2 pi i r k / (Ns R)}
  const float *cx, *qx;              // detrend basis
  const float2 *x1, *x2;             // their DFTs
  double sx2, sq2;
  int elo[7], ehi[7];                // anchors' erase ranges
  double hole_inv[36];
};

// The transform's per-batch device buffers.
struct FftBufs {
  double *hole;                      // frames x bands x 6: the shading fit's partial right-hand sides
  double *part;                      // frames x column tiles x 5: the detrend projections' raw sums a tile
  float2 *fac;                       // frames x (2 n + vrows): the surface spectrum's factors
  float2 *Y;                         // frames x vrows x n: the column transforms' kept rows
  const int32_t *tpos;               // vrows x n: the pos index of spectrum point (u mod n, v), -1 where unused
  int need;                          // used coefficients a frame (subch x 320)
  float2 *C;                         // frames x need: the detrended spectrum's used coefficients in pos order
  // frames x n x nx, filled before the column pass when the samples come straight from captured frames. The exact
  // walk: for each picture row y of a frame, the mesh displacement line of each cell i < nx - 1 (ex, cx, ey, cy, as
  // cell_terms gives them) and at i = nx - 1 the homography's row terms (kw, ku, kv, 0). The decode's read: the
  // homography's row terms of row y at y (n entries), then each column x's displacement terms at mesh row j
  // (lin_cell) at n + j n + x (j < ny - 1, ny = nx)
  float4 *ctab;
  // Y as a 2D tensor (rows frames x vrows, each n complex as 2n floats; boxes of 128 complex by one row) for the row
  // pass's bulk tensor loads, and a device word the passes set when a bounded wait gave up
  const CUtensorMap *ymap;
  int *err;
};
// Encodes the tensor map of a Y buffer of `rows` rows of n complex points (the row pass's loads). 0, or a CUresult.
int fft_y_map(CUtensorMap *map, float2 *Y, int n, int64_t rows);

// The transform CTA's dynamic shared memory bound and the complex points its lines hold at most.
constexpr int kFftSmemMax = 96 * 1024;
constexpr int kFftPoints = 6144;

// The sampler's format-side inputs (row a): picture size, grid origin and step in modules, the node lattice.
struct SampleDev {
  int n, nx, ny;
  int read;                          // LIZG_READ_DECODE (the decode's integer read) or LIZG_READ_EXACT (the exact walk)
  float g0, step;                    // margin + 0.5 / scale, 1 / scale (floats, as the reference computes them)
  const float *node_x, *node_y;      // node centres' module coordinates
  // per picture column x: its module coordinate mx, mesh cell i and 1 / (node_x[i + 1] - node_x[i]); per row y: my,
  // mesh cell j and the row's place v in it. Built once a format by sample_tables_kernel with the walk's own float
  // operations, so reading them gives the walk's values.
  const float4 *colt;                // (mx, i as float bits, inv, 0)
  const float4 *rowt;                // (my, j as float bits, v, 0)
};

// Where the transform reads a frame's picture samples from: a grid (grid set; frame f at grid + f gstride, row-major
// n x n) or the captured frames through their registrations (the sampler fused in).
struct SrcDev {
  const float *grid;
  int64_t gstride;
  const uint8_t *luma;
  int w, h, pitch;
  int64_t fstride;
  const float *reg;
  int regstride;
  SampleDev sd;
};

// The receiver's per-batch soft-value and block state, in device memory.
struct RxState {
  const int8_t *llrf;     // frames x subch x 640 soft values, slot order
  const uint8_t *decl;    // frames x blocks: 1 where the decline gate skipped the block
  uint8_t *blocks;        // frames x blocks x 476 decoded bytes
  int64_t llr_stride;     // bytes a frame of llrf
};

// One launch of the LDPC kernel over the codewords of one code.
struct LdpcLaunch {
  const int8_t *llr;      // the batch's LLRs, codeword i at llr + off[i]
  uint8_t *bits;          // packed hard bits, codeword i at bits + off[i] / 8
  int32_t *its;           // per codeword: iterations, -1 or -3
  uint8_t *ok;            // per codeword: CRC-32C of the first 476 bytes matches
  const int32_t *list;    // the codeword indices of this code
  const int64_t *off;     // per codeword LLR offset
  int count;              // entries of list
  const int *count_dev;   // or, when set, the entries of list as a device word written by an earlier kernel
  int *counter;           // work counter, zero at launch
  int max_iter, stall_it;
  float stall_ratio;
  // receiver mode (rx.llrf set): items are (frame, block) of one tier; its/ok indexed frame x blocks + block
  RxState rx;
  FmtDev fd;
  int tier;
};

cudaError_t ldpc_upload_tables();
// The calling thread's current device made ready (tables uploaded once); its SM count. 0, or a LIZG_E_* code with
// the message recorded.
int device_ready(int *sms);
// Records a failure message for lizg_last_error(); returns code.
int record_error(int code, const char *what);
// spec: frames x spec_stride complex coefficients in pos order.
cudaError_t demap_launch(const FmtDev &fd, const float2 *spec, int64_t spec_stride, float *align, int8_t *llrf,
                         double *sub_est, float *sub_rms, float *est, float *pilot, uint8_t *decl, cudaStream_t st);
// One format's share of the soft stage run across formats: its tables and frames, its spectra and outputs as
// demap_launch takes them. demap_mixed_launch: the pilots' fit, the soft values and the block stage, each one launch
// over count <= kDemapMixSegs formats.
constexpr int kDemapMixSegs = 8;
struct DemapSeg {
  FmtDev fd;
  const float2 *spec;
  int64_t stride;
  float *align;
  int8_t *llrf;
  double *sub_est;
  float *sub_rms, *est, *pilot;
  uint8_t *decl;
};
cudaError_t demap_mixed_launch(const DemapSeg *a, int count, cudaStream_t st);
cudaError_t fft_launch(const FftDev &xd, int frames, const SrcDev &src, const FftBufs &b, int sms, cudaStream_t st);
// One format's share of a transform stage run across formats (the engine's stage-wise run): its tables, source,
// buffers and frames. fft_pre_launch: the shading fit's sums and the sampler's table; fft_fac_launch: the surface
// factors; the mixed launches: one column (row) pass grid over count <= kFftMixSegs formats' tiles.
constexpr int kFftMixSegs = 8;
struct FftSegArgs {
  FftDev xd;
  SrcDev src;
  FftBufs b;
  int frames;
};
cudaError_t fft_pre_launch(const FftSegArgs &a, cudaStream_t st);
cudaError_t fft_fac_launch(const FftSegArgs &a, cudaStream_t st);
cudaError_t fft_cols_mixed_launch(const FftSegArgs *a, int count, cudaStream_t st);
// The light stages across formats (captured frames only): the shading sums and the sampler's tables in one launch,
// the surface factors in one launch.
cudaError_t fft_pre_mixed_launch(const FftSegArgs *a, int count, cudaStream_t st);
cudaError_t fft_fac_mixed_launch(const FftSegArgs *a, int count, cudaStream_t st);
cudaError_t fft_rows_mixed_launch(const FftSegArgs *a, int count, cudaStream_t st);
// The transform plan of picture size n (three passes' radices, lines a CTA): 0, or -1 for a size off the ladder.
// The sender's inverse transform: the half-plane spectrum S (frames x vrows x n, rows along u, overwritten) to the
// clipped picture pic (frames x n x n, 0.5 + clamp(P, +-lim) sc). tws: the transform's twiddles.
struct EncFft {
  int n, vrows;
  const float2 *tws;
  float lim, sc;
};
cudaError_t enc_fft_launch(const EncFft &e, int frames, float2 *S, float *pic, cudaStream_t st);
// The border's cell kinds of a ring of span modules, (span + 30)^2: 2 dark, 1 light, 0 the picture's, | 8 on the format
// word's cells (encode.cu).
void layout_kind(int span, int version, int fps, std::vector<uint8_t> &kind);
int fft_plan(int n, int radix[3], int *lines);
// The shading fit's bands a frame.
int fft_hole_bands(int n);
cudaError_t sample_launch(const SampleDev &sd, int frames, const uint8_t *luma, int w, int h, int pitch, int64_t fstride,
                          const float *reg, int regstride, float *grid, cudaStream_t st);
cudaError_t sample_tables_launch(SampleDev sd, float4 *colt, float4 *rowt, cudaStream_t st);
// The node lattice of a layout of side modules (liblizard/src/layout.c:110-117): returns nx (= ny).
int layout_nodes(int side, float *pos);
// The anchor search for a batch of frames (arguments as lizg_anchor_find_dev's, already checked).
// The border node search on the four corners alone (refine_node, the anchors' registration's second look at the
// corners it disagrees with): frame f's corner c searched where d_redo[4 f + c], through H and (where d_lens_on) the
// lens model; d_nodes frames x nn^2 x (dx, dy, score, done) as lizg_border_nodes_dev writes them.
cudaError_t border_corners_launch(int span, const uint8_t *d_rim, int w, int h, int64_t frame_stride, const float *d_H, int h_stride,
                                  const double *d_lens, const int *d_lens_on, const uint8_t *d_redo, int frames, float *d_nodes, cudaStream_t st);
// d_lens_on (frames, may be NULL): 0 where a frame searches through H alone; d_active (frames, may be NULL): 0 where a
// frame is not searched.
cudaError_t anchor_find_launch(int span, const uint8_t *d_luma, int w, int h, int64_t frame_stride, const float *d_H, int h_stride,
                               const double *d_lens, const uint8_t *d_skip, int frames, const lizg_anchor_out &out, cudaStream_t st,
                               const int *d_lens_on = nullptr, const uint8_t *d_active = nullptr);
// code: 0 = 7/8, 1 = 3/4, 2 = 2/3, 3 = 1/2. sms: the device's SM count (the persistent grid's bound).
cudaError_t ldpc_launch(int code, const LdpcLaunch &a, int sms, cudaStream_t st);
// The receivers' decode of every tier in one persistent launch: a queue of segments, segment s items
// [first[s], first[s + 1]) of tier a[s].tier (code code[s]) of the receiver whose fields a[s] holds (its, ok, rx, fd,
// the stop rule, as a tier's launch takes them; count and counter unused): one receiver's tiers, or every format's
// of an engine; counter zero at launch.
constexpr int kMixSegs = 32;
struct LdpcMix {
  LdpcLaunch a[kMixSegs];
  int first[kMixSegs + 1], code[kMixSegs];
  int nseg;
  int *counter;
};
cudaError_t ldpc_mixed_launch(const LdpcMix &m, int sms, cudaStream_t st);
// The decoder's kernel variants of a code (all bit for bit alike), and a launch of variant v of them.
int ldpc_variant_count(int code);
int ldpc_choice(int code);   // the device's choice for the code (lizg_ldpc_autotune, lizg_ldpc_set_variant)
cudaError_t ldpc_launch_variant(int code, int v, const LdpcLaunch &a, int sms, cudaStream_t st);
// Row (b) alone from captured frames: the handle's read through each frame's registration, the anchors' erase, the
// detrend and the 2D transform, the used coefficients into d_coef (frames x subch x 320 complex, pos order); no soft
// stage. For the registration's refinements, which measure their mismatch where the receiver measures it.
int rx_spectrum_luma(lizg_rx *r, const uint8_t *d_luma, int w, int h, int pitch, int64_t frame_stride, const float *d_reg, int frames,
                     float *d_coef, cudaStream_t st);
// One receiver call split into its stages, for the engine's stage-wise run across formats: the transform's share
// (fft), the soft stage's arguments and buffers, and the tiers' decode launches. rx_call checks the call as
// lizg_rx_finish_luma_dev does; rx_call_tier gives the decode of tier t (count set, counter left to the caller),
// returning its code.
struct RxCall {
  lizg_rx *r;
  FftSegArgs fft;
  FmtDev fd;
  int tiers;
  const lizg_rx_out *out;
  int8_t *llrf;
  double *sub_est;
  float *sub_rms, *est, *pilot, *align;
  uint8_t *decl;
};
int rx_call(lizg_rx *r, const uint8_t *d_luma, int w, int h, int pitch, int64_t frame_stride, const float *d_reg, int frames,
            const lizg_rx_out *out, RxCall &c);
int rx_call_tier(const RxCall &c, int t, LdpcLaunch &a);
int rx_read(const lizg_rx *r);   // the handle's read (LIZG_READ_DECODE or LIZG_READ_EXACT)

}  // namespace lizg

#endif

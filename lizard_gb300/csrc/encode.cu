// The sender on sm_103a (the GPU encoder): a batch of frames' blocks to the ring's drive and its grey page, as the
// reference's lizard_encode and lizard_paint_grey make them (liblizard/src/lizard_phy.c:1087-1236, 700-716):
//   - each block's data bits and CRC-32C, the LDPC code's parity as the running XOR of the checks' data bits
//     (liblizard/src/ldpc.c:117-126), its slots through the tier's bit map and the whitening, the pilots' count bit
//     past the codeword (map_out, :121-159), Gray QPSK of unit magnitude at each coefficient (:1134-1141); the
//     padding past the last block the whitening alone (:1146-1152);
//   - the half-plane's Hermitian inverse, clipped at 2 sqrt(640 subch) and mapped to 0..1 (fft.cu enc_*);
//   - the picture onto the ring's pixels by the Lanczos-3 resampler over the picture and its guard interval, the
//     picture periodic (:962-1075), six weights a pass in order; the border's cells 0 or 1 at pxm pixels a module
//     (:1153-1165), the format word among them; the anchors' squares over the picture (:1218-1234);
//   - the page: round(drive 255) inside a white margin of 2 modules (lizard_paint_grey).
// The transform's floats are this library's (a different order from the reference's), so a drive pixel may differ in
// its last bits and a grey level by one at a rounding tie; every other step is the reference's float order
// (-fmad=false). A receiver reads the same blocks.
#include <cuda_runtime.h>
#include <stdint.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>
#include "format.h"
#include "lizard_codes.h"
#include "lizard_gb300.h"
#include "lizg_internal.h"

namespace lizg {

constexpr int kEncThreads = 256, kCp = 3, kQuiet = 2, kMaxCheckRows = 30;
constexpr float kQpsk = 0.70710678f;

struct EncTier {
  const int16_t *perm;
  const uint8_t *rowptr;
  const uint16_t *circ;
  int nt, k, m, slots, mb;
};

struct EncDev {
  int n, subch, blocks, used, vrows;
  const int32_t *tix, *block_tier, *block_slot;
  const uint8_t *white;
  EncTier tier[kMaxTiers];
  int pxm, px, W, q, o, side, aside, a0[kAnchK];   // drive geometry (pixels), the anchors' first pixels
  int copy;   // every tap is the one sample's (the ring's pixels an exact copy of the picture's samples)
  const int32_t *rs_i0;
  const float *rs_w;
  const uint8_t *kind;
  // per ring pixel p < q: the exact copy's picture index (rs_i0 + 2) mod n and the first tap's rs_i0 mod n (both in
  // [0, n)); per drive pixel d < px: its border cell d / pxm
  const int32_t *rs_cp, *rs_c0, *cellx;
};

// ---------------------------------------------------------------- blocks to coefficients

// A block of a frame, one CTA: its bits, its codeword, its slots, its coefficients into the spectrum S.
__global__ void __launch_bounds__(kEncThreads) enc_blocks_kernel(EncDev e, const uint8_t *blocks, int pilots, float2 *S) {
  __shared__ uint8_t bits[8192];   // data bits, then parity bits
  __shared__ uint8_t syn[kMaxCheckRows * LIZG_Z];
  __shared__ uint32_t crc_tab[256];
  __shared__ uint32_t s_crc, s_carry[kEncThreads / 32];
  const int f = blockIdx.x / e.blocks, b = blockIdx.x % e.blocks, tid = threadIdx.x;
  const EncTier &t = e.tier[e.block_tier[b]];
  const uint8_t *src = blocks + ((int64_t)f * e.blocks + b) * LIZG_BLOCK_BYTES;
  // CRC-32C of the block (Castagnoli, reflected 0x82F63B78, liblizard/src/layout.c:44-54), a byte table
  for (int i = tid; i < 256; i += blockDim.x) {
    uint32_t c = (uint32_t)i;
    for (int k = 0; k < 8; k++) c = (c >> 1) ^ (0x82f63b78u & (0u - (c & 1)));
    crc_tab[i] = c;
  }
  __syncthreads();
  if (tid == 0) {
    uint32_t c = 0xffffffffu;
    for (int i = 0; i < LIZG_BLOCK_BYTES; i++) c = (c >> 8) ^ crc_tab[(c ^ src[i]) & 255];
    s_crc = ~c;
  }
  __syncthreads();
  const uint32_t crc = s_crc;
  for (int i = tid; i < t.k; i += blockDim.x) {   // the block MSB first, its CRC MSB first, zeros past them
    uint8_t v = 0;
    if (i < 8 * LIZG_BLOCK_BYTES) v = (src[i >> 3] >> (7 - (i & 7))) & 1;
    else if (i < 8 * LIZG_BLOCK_BYTES + 32) v = (crc >> (31 - (i - 8 * LIZG_BLOCK_BYTES))) & 1;
    bits[i] = v;
  }
  __syncthreads();
  // each check's data bits: check c = i mb + r holds data bit col z + (i - shift) mod z of row r's circulants
  for (int c = tid; c < t.m; c += blockDim.x) {
    const int i = c / t.mb, r = c - i * t.mb;
    uint32_t acc = 0;
    for (int k = t.rowptr[r]; k < t.rowptr[r + 1]; k++) {
      const int col = t.circ[k] >> 8, sh = t.circ[k] & 255;
      acc ^= bits[col * LIZG_Z + ((i - sh) & (LIZG_Z - 1))];
    }
    syn[c] = (uint8_t)acc;
  }
  __syncthreads();
  // the parity: the running XOR over the checks, a run of checks a thread, the runs' carries scanned
  const int run = (t.m + kEncThreads - 1) / kEncThreads, c0 = tid * run, c1 = min(t.m, c0 + run);
  uint32_t mine = 0;
  for (int c = c0; c < c1; c++) mine ^= syn[c];
  uint32_t incl = mine;
  const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t up = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl ^= up;
  }
  if (lane == 31) s_carry[warp] = incl;
  __syncthreads();
  uint32_t carry = incl ^ mine;   // the XOR of every run before this thread's within its warp
  for (int w = 0; w < warp; w++) carry ^= s_carry[w];
  for (int c = c0; c < c1; c++) {
    carry ^= syn[c];
    bits[t.k + c] = (uint8_t)carry;
  }
  __syncthreads();
  // the slots and their coefficients: slot i = codeword bit perm[i] (i < nt) or the pilots' count bit, whitened
  const int first = e.block_slot[b] / 2;
  const uint32_t qbit = (uint32_t)(pilots >> (b & 1)) & 1;
  const uint8_t *wh = e.white + 2 * (int64_t)first;
  float2 *Sf = S + (int64_t)f * e.vrows * e.n;
  for (int s = tid; s < t.slots / 2; s += blockDim.x) {
    const int i0 = 2 * s, i1 = 2 * s + 1;
    const uint32_t b0 = (i0 < t.nt ? bits[t.perm[i0]] : qbit) ^ wh[i0], b1 = (i1 < t.nt ? bits[t.perm[i1]] : qbit) ^ wh[i1];
    Sf[e.tix[first + s]] = make_float2(b0 ? -kQpsk : kQpsk, b1 ? -kQpsk : kQpsk);
  }
}

// The coefficients past the last block: the whitening alone.
__global__ void __launch_bounds__(kEncThreads) enc_pad_kernel(EncDev e, int per, float2 *S) {
  const int f = blockIdx.x / per, s = e.used / 2 + (blockIdx.x % per) * blockDim.x + threadIdx.x;
  if (s >= e.subch * kSub) return;
  S[(int64_t)f * e.vrows * e.n + e.tix[s]] = make_float2(e.white[2 * s] ? -kQpsk : kQpsk, e.white[2 * s + 1] ? -kQpsk : kQpsk);
}

// ---------------------------------------------------------------- resample and paint

// Down the picture: row y of the q x n intermediate from the six picture rows its taps read (the picture periodic).
__global__ void __launch_bounds__(kEncThreads) enc_vert_kernel(EncDev e, const float *pic, float *tmp) {
  const int f = blockIdx.x / e.q, y = blockIdx.x % e.q;
  const float *wt = e.rs_w + 6 * y;
  const float *pf = pic + (int64_t)f * e.n * e.n;
  const float *r[6];
#pragma unroll
  for (int t = 0; t < 6; t++) {
    int i = (e.rs_i0[y] + t) % e.n;
    if (i < 0) i += e.n;
    r[t] = pf + (int64_t)i * e.n;
  }
  float *out = tmp + ((int64_t)f * e.q + y) * e.n;
  for (int k = threadIdx.x; k < e.n; k += blockDim.x)
    out[k] = wt[0] * r[0][k] + wt[1] * r[1][k] + wt[2] * r[2][k] + wt[3] * r[3][k] + wt[4] * r[4][k] + wt[5] * r[5][k];
}

// A row of the page: the white margin, the border's cells, the picture resampled across, the anchors over it, each
// drive value to its grey level as lizard_paint_grey rounds it.
__global__ void __launch_bounds__(kEncThreads) enc_paint_kernel(EncDev e, const float *tmp, float *drive, uint8_t *grey) {
  const int f = blockIdx.x / e.W, Y = blockIdx.x % e.W, m = kQuiet * e.pxm;
  uint8_t *g = grey ? grey + ((int64_t)f * e.W + Y) * e.W : nullptr;
  const bool in_rows = Y >= m && Y < m + e.px;
  const int dy = Y - m;
  int aj = -1;
  if (in_rows)
    for (int j = 0; j < kAnchK; j++) if (dy >= e.a0[j] && dy < e.a0[j] + e.aside) aj = j;
  const float half = 0.5f * (float)e.aside;
  // the row's terms: the picture rows it reads (the exact copy's one, the resampled intermediate's one) and its cells
  const bool pic_row = in_rows && dy >= e.o && dy < e.o + e.q;
  const float *crow = pic_row ? tmp + ((int64_t)f * e.n + e.rs_cp[dy - e.o]) * e.n : nullptr;
  const float *rrow = pic_row ? tmp + ((int64_t)f * e.q + (dy - e.o)) * e.n : nullptr;
  const uint8_t *krow = in_rows ? e.kind + (int64_t)(dy / e.pxm) * e.side : nullptr;
  for (int X = threadIdx.x; X < e.W; X += blockDim.x) {
    if (!in_rows || X < m || X >= m + e.px) {
      if (g) g[X] = 255;
      continue;
    }
    const int dx = X - m;
    int ai = -1;
    if (aj >= 0)
      for (int i = 0; i < kAnchK; i++) if (dx >= e.a0[i] && dx < e.a0[i] + e.aside) ai = i;
    const bool pic = pic_row && dx >= e.o && dx < e.o + e.q;
    float d;
    if (ai >= 0) {   // the anchor's pattern: light middle and rim, a dark ring (Chebyshev distance from its middle)
      const float ddx = fabsf((float)(dx - e.a0[ai]) + 0.5f - half), ddy = fabsf((float)(dy - e.a0[aj]) + 0.5f - half);
      const float r = fmaxf(ddx, ddy) / half;
      d = r < 0.25f || r >= 0.6f ? 1.0f : 0.0f;
    } else if (e.copy && pic) {
      // an exact copy: both passes' six terms are 0 x, 1 x the sample, 0 x ..., whose sums are the sample itself
      const float v = crow[e.rs_cp[dx - e.o]];
      d = v < 0 ? 0.0f : v > 1 ? 1.0f : v;
    } else if (pic) {   // the picture and its guard interval
      const int x = dx - e.o;
      const float *wt = e.rs_w + 6 * x;
      int c = e.rs_c0[x];
      float v = wt[0] * rrow[c];
#pragma unroll
      for (int t = 1; t < 6; t++) {
        c = c + 1 == e.n ? 0 : c + 1;
        v = v + wt[t] * rrow[c];
      }
      d = v < 0 ? 0.0f : v > 1 ? 1.0f : v;
    } else {   // the border's cell
      d = (krow[e.cellx[dx]] & 3) == 2 ? 0.0f : 1.0f;
    }
    if (drive) drive[((int64_t)f * e.px + dy) * e.px + dx] = d;
    if (g) {
      const float tt = d * 255.0f + 0.5f;
      int v = tt >= 2147483647.0f ? 255 : tt <= -2147483648.0f ? 0 : (int)tt;
      g[X] = (uint8_t)(v < 0 ? 0 : v > 255 ? 255 : v);
    }
  }
}

// ---------------------------------------------------------------- host: the layout, the word, the resampler's taps

// Reed-Solomon parity of the format word over GF(256), polynomial 0x11d, roots alpha^0 .. (liblizard/src/rs.c:19-35).
static void word_encode(uint8_t *cw, int k, int nroots) {
  uint8_t ex[512], lg[256];
  int x = 1;
  for (int i = 0; i < 255; i++) { ex[i] = (uint8_t)x; lg[x] = (uint8_t)i; x <<= 1; if (x & 256) x ^= 0x11d; }
  for (int i = 255; i < 512; i++) ex[i] = ex[i - 255];
  auto mul = [&](int a, int b) -> uint8_t { return a && b ? ex[lg[a] + lg[b]] : 0; };
  uint8_t gen[256] = {1};
  for (int i = 0; i < nroots; i++) {
    gen[i + 1] = 0;
    for (int j = i + 1; j > 0; j--) gen[j] ^= mul(gen[j - 1], ex[i]);
  }
  uint8_t *par = cw + k;
  std::memset(par, 0, (size_t)nroots);
  for (int i = 0; i < k; i++) {
    const uint8_t fb = cw[i] ^ par[0];
    std::memmove(par, par + 1, (size_t)nroots - 1);
    par[nroots - 1] = 0;
    if (fb) for (int j = 0; j < nroots; j++) par[j] ^= mul(fb, gen[j + 1]);
  }
}

static int track_bit(int side, int j) {   // liblizard/src/layout.c:57-61
  uint32_t v = (uint32_t)(side * 4099 + (j >> 1)) * 2654435761u + 40503u;
  v ^= v >> 15;
  v *= 2246822519u;
  v ^= v >> 13;
  return (int)((v ^ (uint32_t)j) & 1);
}

// The border's cell kinds, side x side modules: the corner marks, the line, the timing track, the format word's
// cells (liblizard/src/layout.c:69-141 thin_init, thin_corner, ob_layout_set_fmt). 2 dark, 1 light, 0 the picture's;
// | 8 on the word's cells (CELL_WORD: the registration's templates skip them).
void layout_kind(int span, int version, int fps, std::vector<uint8_t> &kind) {
  const int side = span + 2 * kMargin, S = 12, reserve = 15, margin = kMargin;
  kind.assign((size_t)side * side, 1);
  for (int y = 0; y < side; y++)
    for (int x = 0; x < side; x++) {
      const int dx = std::min(x, side - 1 - x), dy = std::min(y, side - 1 - y), d = std::min(dx, dy);
      uint8_t k;
      if (dx < S && dy < S) {   // a corner mark
        const bool in = dx >= 1 && dx <= S - 2 && dy >= 1 && dy <= S - 2;
        const int cd = std::min(dx, dy);
        k = in && !(cd >= 3 && cd < 5) ? 2 : 1;
      } else {
        bool dark = d >= 1 && d <= 2;
        if (d >= 5 && d < 7) {
          const int along = dy <= dx ? x : y, len = side;
          const int sd = dy <= dx ? (y < side / 2 ? 0 : 2) : (x < side / 2 ? 3 : 1);
          const int cell = (along - reserve) / 2, run = cell / 4;
          if (along >= reserve && along < len - reserve && !(run & 1)) dark = track_bit(sd, run / 2 * 4 + cell % 4);
        }
        k = d >= margin - kCp ? 0 : dark ? 2 : 1;
      }
      kind[(size_t)y * side + x] = k;
    }
  // the word: RS(bytes, 3) of magic, version, fps over the word cells; blank (light) where the version is no format's
  const int thin = (side - 2 * reserve) / 2, wc = thin / 8 * 4, cells = wc >= 32 ? wc : 0, bytes = std::min(64, 4 * (cells / 8));
  uint8_t cw[64] = {0};
  if (bytes >= 16 && version >= 4 && version <= 64 && fps >= 0 && fps <= 255) {
    cw[0] = 0x4c; cw[1] = (uint8_t)version; cw[2] = (uint8_t)fps;
    word_encode(cw, 3, bytes - 3);
  }
  for (int sd = 0; sd < 4; sd++)
    for (int i = 0; i < cells; i++) {
      const int kb = 4 * (i >> 3) + sd;
      const int bit = kb < bytes ? (cw[kb] >> (7 - (i & 7))) & 1 : 0;
      const int off = ((i / 4) * 8 + i % 4 + 4) * 2;
      for (int j = 0; j < 2; j++)
        for (int ee = 0; ee < 2; ee++) {
          const int t = reserve + off + j, dd = 5 + ee;
          const int x = sd == 0 || sd == 2 ? t : sd == 3 ? dd : side - 1 - dd;
          const int y = sd == 0 ? dd : sd == 2 ? side - 1 - dd : t;
          kind[(size_t)y * side + x] = (bit ? 2 : 1) | 8;
        }
    }
}

static double lanczos3(double x) {   // liblizard/src/lizard_phy.c:970-975
  x = std::fabs(x);
  if (x >= 3) return 0;
  const double px = 3.14159265358979323846 * x;
  return 3 * std::sin(px) * std::sin(px / 3) / (px * px);
}

}  // namespace lizg

struct lizg_encoder {
  lizg::Format f;
  lizg::EncDev e{};
  lizg::EncFft xf{};
  int max_frames = 0, fps = 0;
  std::vector<void *> owned;
  float2 *S = nullptr, *tws = nullptr;
  float *pic = nullptr, *tmp = nullptr;
  uint8_t *kind = nullptr;
};

namespace {
template <class T>
bool upload(lizg_encoder *x, const T **dst, const T *src, size_t count) {
  void *p = nullptr;
  if (cudaMalloc(&p, std::max<size_t>(1, count) * sizeof(T)) != cudaSuccess) return false;
  x->owned.push_back(p);
  if (count && cudaMemcpy(p, src, count * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) return false;
  *dst = static_cast<const T *>(p);
  return true;
}
bool alloc(lizg_encoder *x, void **dst, size_t bytes) {
  if (cudaMalloc(dst, std::max<size_t>(1, bytes)) != cudaSuccess) return false;
  x->owned.push_back(*dst);
  return true;
}
bool paint_kind(lizg_encoder *x) {
  std::vector<uint8_t> kind;
  lizg::layout_kind(x->f.span, x->f.subch % 16 == 0 ? x->f.subch / 16 : 0, x->fps, kind);
  return cudaMemcpy(x->kind, kind.data(), kind.size(), cudaMemcpyHostToDevice) == cudaSuccess;
}
}  // namespace

extern "C" {

lizg_encoder *lizg_encoder_new(int n, int subch, int span, int max_frames) {
  using namespace lizg;
  if (max_frames < 1 || max_frames > 4096) { record_error(LIZG_E_ARG, "lizg_encoder_new: max_frames must be 1..4096"); return nullptr; }
  int sms = 0;
  if (device_ready(&sms)) return nullptr;
  lizg_encoder *x = new (std::nothrow) lizg_encoder();
  if (!x) { record_error(LIZG_E_NOMEM, "lizg_encoder_new: out of host memory"); return nullptr; }
  Format &f = x->f;
  int rad[3], lines = 0;
  if (format_build(n, subch, span, f) || fft_plan(n, rad, &lines) || 2 * (f.vmax + 1) > n) {
    delete x;
    record_error(LIZG_E_ARG, "lizg_encoder_new: no such format");
    return nullptr;
  }
  x->max_frames = max_frames;
  EncDev &e = x->e;
  e.n = n; e.subch = subch; e.blocks = f.blocks; e.used = f.used; e.vrows = f.vmax + 1;
  e.pxm = (int)std::ceil((float)n / span - 1e-4f);
  e.side = span + 2 * kMargin;
  e.px = e.side * e.pxm;
  e.W = e.px + 2 * kQuiet * e.pxm;
  e.q = (span + 2 * kCp) * e.pxm;
  e.o = (kMargin - kCp) * e.pxm;
  const int a = span / 64;
  e.aside = a * e.pxm;
  for (int i = 0; i < kAnchK; i++) e.a0[i] = (int)std::floor(kMargin + (double)span * (i + 0.5) / kAnchK - a / 2.0 + 0.5) * e.pxm;
  bool ok = upload(x, &e.tix, f.tix.data(), f.tix.size()) && upload(x, &e.white, f.white.data(), f.white.size()) &&
            upload(x, &e.block_tier, f.block_tier.data(), f.block_tier.size()) && upload(x, &e.block_slot, f.block_slot.data(), f.block_slot.size());
  for (int t = 0; ok && t < f.tiers; t++) {
    const lizg_code_def_t &d = LIZG_CODES[f.tier[t].code];
    EncTier &et = e.tier[t];
    et.nt = f.tier[t].nt; et.k = f.tier[t].k; et.mb = d.mb; et.m = d.mb * LIZG_Z; et.slots = f.tier[t].slots;
    ok = upload(x, &et.perm, f.perm[t].data(), f.perm[t].size()) && upload(x, &et.rowptr, d.rowptr, (size_t)d.mb + 1) &&
         upload(x, &et.circ, d.circ, (size_t)d.rowptr[d.mb]) && et.m <= kMaxCheckRows * LIZG_Z && et.k + et.m <= 8192;
  }
  // the resampler's taps (liblizard/src/lizard_phy.c:980-1000)
  std::vector<int32_t> i0(e.q);
  std::vector<float> w(6 * (size_t)e.q);
  const double sc = (double)n / span;
  for (int p = 0; p < e.q; p++) {
    const double u = (p + 0.5) * sc / e.pxm - kCp * sc - 0.5, r = std::floor(u + 0.5);
    if (std::fabs(u - r) < 1e-6) {
      i0[p] = (int)r - 2;
      for (int t = 0; t < 6; t++) w[6 * p + t] = t == 2 ? 1.0f : 0.0f;
      continue;
    }
    const int a0 = (int)std::floor(u) - 2;
    double tw[6], sum = 0;
    for (int t = 0; t < 6; t++) { tw[t] = lanczos3(u - (a0 + t)); sum += tw[t]; }
    i0[p] = a0;
    for (int t = 0; t < 6; t++) w[6 * p + t] = (float)(tw[t] / sum);
  }
  ok = ok && upload(x, &e.rs_i0, i0.data(), i0.size()) && upload(x, &e.rs_w, w.data(), w.size());
  {
    std::vector<int32_t> cp(e.q), c0(e.q), cell(e.px);
    for (int p = 0; p < e.q; p++) {
      int a = (i0[p] + 2) % n, b = i0[p] % n;
      cp[p] = a < 0 ? a + n : a;
      c0[p] = b < 0 ? b + n : b;
    }
    for (int d = 0; d < e.px; d++) cell[d] = d / e.pxm;
    ok = ok && upload(x, &e.rs_cp, cp.data(), cp.size()) && upload(x, &e.rs_c0, c0.data(), c0.size()) && upload(x, &e.cellx, cell.data(), cell.size());
  }
  e.copy = 1;
  for (int p = 0; p < e.q && e.copy; p++)
    for (int t = 0; t < 6; t++) e.copy &= w[6 * p + t] == (t == 2 ? 1.0f : 0.0f);
  // the transform's twiddles
  std::vector<float2> tws(n);
  for (int st = 0, ns = 1; st < 3; ns *= rad[st], st++)
    for (int qq = 1; qq < rad[st]; qq++)
      for (int k = 0; k < ns; k++) {
        const double th = -2.0 * 3.14159265358979323846 * qq * k / ((double)ns * rad[st]);
        tws[ns + (qq - 1) * ns + k] = make_float2((float)std::cos(th), (float)std::sin(th));
      }
  const float2 *dtw = nullptr;
  ok = ok && upload(x, &dtw, tws.data(), tws.size());
  x->xf.n = n; x->xf.vrows = e.vrows; x->xf.tws = dtw;
  x->xf.lim = 2.0f * 2.0f * std::sqrt(0.5f * (float)(subch * kSub));   // LIZARD_CLIP 2, twice the half-plane's rms
  x->xf.sc = 0.5f / x->xf.lim;
  ok = ok && alloc(x, reinterpret_cast<void **>(&x->S), sizeof(float2) * (size_t)max_frames * e.vrows * n) &&
       alloc(x, reinterpret_cast<void **>(&x->pic), sizeof(float) * (size_t)max_frames * n * n) &&
       alloc(x, reinterpret_cast<void **>(&x->tmp), sizeof(float) * (size_t)max_frames * e.q * n) &&
       alloc(x, reinterpret_cast<void **>(&x->kind), (size_t)e.side * e.side);
  e.kind = x->kind;
  ok = ok && paint_kind(x);
  if (!ok) {
    lizg_encoder_free(x);
    record_error(LIZG_E_NOMEM, "lizg_encoder_new: device allocation or copy failed");
    return nullptr;
  }
  return x;
}

void lizg_encoder_free(lizg_encoder *x) {
  if (!x) return;
  for (void *p : x->owned) cudaFree(p);
  delete x;
}

int lizg_encoder_fps(lizg_encoder *x, int fps) {
  if (!x || fps < 0 || fps > 255) return lizg::record_error(LIZG_E_ARG, "lizg_encoder_fps: NULL handle or fps outside 0..255");
  x->fps = fps;
  return paint_kind(x) ? 0 : lizg::record_error(LIZG_E_CUDA, "lizg_encoder_fps: copy failed");
}

int lizg_layout_kind(int span, int version, int fps, uint8_t *kind) {
  if ((span != 128 && span != 256 && span != 512) || !kind) return lizg::record_error(LIZG_E_ARG, "lizg_layout_kind: span must be 128, 256 or 512");
  std::vector<uint8_t> k;
  lizg::layout_kind(span, version, fps, k);
  std::memcpy(kind, k.data(), k.size());
  return span + 2 * lizg::kMargin;
}

int lizg_encoder_info(const lizg_encoder *x, int32_t *out) {
  if (!x || !out) return lizg::record_error(LIZG_E_ARG, "lizg_encoder_info: NULL argument");
  out[0] = x->e.blocks; out[1] = x->e.pxm; out[2] = x->e.px; out[3] = x->e.W; out[4] = x->max_frames;
  return 0;
}

int lizg_encode_dev(lizg_encoder *x, const uint8_t *d_blocks, int frames, int pilots, float *d_drive, uint8_t *d_grey, void *stream) {
  using namespace lizg;
  if (!x || !d_blocks || (!d_drive && !d_grey) || frames < 1 || frames > x->max_frames || pilots < 0 || pilots > 3)
    return record_error(LIZG_E_ARG, "lizg_encode_dev: NULL argument, frames outside 1..max_frames or pilots outside 0..3");
  const EncDev &e = x->e;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t err = cudaMemsetAsync(x->S, 0, sizeof(float2) * (size_t)frames * e.vrows * e.n, st);
  if (err == cudaSuccess) {
    enc_blocks_kernel<<<frames * e.blocks, kEncThreads, 0, st>>>(e, d_blocks, pilots, x->S);
    const int pad = e.subch * kSub - e.used / 2, per = (pad + kEncThreads - 1) / kEncThreads;
    if (per > 0) enc_pad_kernel<<<frames * per, kEncThreads, 0, st>>>(e, per, x->S);
    err = cudaGetLastError();
  }
  if (err == cudaSuccess) err = enc_fft_launch(x->xf, frames, x->S, x->pic, st);
  if (err == cudaSuccess) {
    if (!e.copy) enc_vert_kernel<<<frames * e.q, kEncThreads, 0, st>>>(e, x->pic, x->tmp);
    enc_paint_kernel<<<frames * e.W, kEncThreads, 0, st>>>(e, e.copy ? x->pic : x->tmp, d_drive, d_grey);   // a copy reads the picture
    err = cudaGetLastError();
  }
  return err == cudaSuccess ? 0 : record_error(LIZG_E_CUDA, (std::string("lizg_encode_dev: ") + cudaGetErrorString(err)).c_str());
}

}  // extern "C"

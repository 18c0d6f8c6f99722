// Camera-format ingest on sm_103a: captured frames in the formats cameras and apps hand over turned into the 8-bit
// luma rows the receiver reads, on the device, a batch of frames a launch. Two sources, restated from the reference:
//   - liz_decode's pixel formats (liblizard/api/codec.cpp:128-140): GREY8 rows compacted, RGBA8 / RGBX8 by ob_luma's
//     (77 r + 150 g + 29 b + 128) >> 8 (liblizard/src/acquire.c:67-83), BGRA8 the same from B, G, R;
//   - the camera develop (liblizard/core/ingest/develop.cpp:9-102): P010's top byte; RAW16 / RAW10 / RAW12 less the
//     CFA position's black level, times its gain scale, clipped to [0, 4096] and read through the 4097-step gamma 1/2.2
//     table, each 2 x 2 quad averaged when binned by 2.
// Compiled with -fmad=false (the develop's float order is the reference's). The pixel formats: a CTA takes a band of
// kBand rows, a thread four output pixels (one 16-byte load where aligned). The develop: a CTA takes a tile, its
// source rows staged into shared memory with 16-byte loads, the gamma table beside them. Bytes in and bytes out,
// bound by HBM.
#include <cuda_runtime.h>
#include <stdint.h>
#include <algorithm>
#include <climits>
#include <cmath>
#include <mutex>
#include <string>
#include "lizard_gb300.h"
#include "lizg_internal.h"

namespace lizg {

constexpr int kBand = 16, kIngThreads = 256;   // rows a pixel-format CTA takes; threads a CTA
constexpr int kRaw16 = 0x20, kRaw10 = 0x25, kRaw12 = 0x26, kP010 = 0x36;

static __device__ __align__(16) uint8_t g_gamma[4112];   // the 4097 steps of gamma 1 / 2.2 (develop.cpp:17-22), made on the host

// ob_luma of one RGBA / RGBX / BGRA pixel word (liblizard/src/acquire.c:67-83).
template <int FMT>
__device__ __forceinline__ uint32_t luma_of(uint32_t p) {
  const uint32_t c0 = p & 255, c1 = (p >> 8) & 255, c2 = (p >> 16) & 255;
  return FMT == LIZG_PIX_BGRA8 ? (77 * c2 + 150 * c1 + 29 * c0 + 128) >> 8 : (77 * c0 + 150 * c1 + 29 * c2 + 128) >> 8;
}

// A CTA takes a band of kBand rows, a warp a row, a lane 16 pixels at a time: four 16-byte loads in and one 16-byte
// store out where both ends are aligned, pixel by pixel elsewhere.
template <int FMT>
__global__ void __launch_bounds__(kIngThreads) pixels_kernel(const uint8_t *px, int w, int h, int stride, int64_t fstride, uint8_t *out) {
  const int bands = (h + kBand - 1) / kBand, f = blockIdx.x / bands, y0 = (blockIdx.x % bands) * kBand, y1 = min(h, y0 + kBand);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int bpp = FMT == LIZG_PIX_GREY8 ? 1 : 4;
  for (int y = y0 + warp; y < y1; y += kIngThreads / 32) {
    const uint8_t *row = px + f * fstride + (int64_t)y * stride;
    uint8_t *d = out + ((int64_t)f * h + y) * w;
    for (int x = 16 * lane; x < w; x += 512) {
      const uint8_t *src = row + bpp * x;
      if (x + 16 <= w && ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(d + x)) & 15) == 0) {
        if (FMT == LIZG_PIX_GREY8) {
          *reinterpret_cast<uint4 *>(d + x) = *reinterpret_cast<const uint4 *>(src);
        } else {
          uint32_t o[4];
#pragma unroll
          for (int j = 0; j < 4; j++) {
            const uint4 q = *reinterpret_cast<const uint4 *>(src + 16 * j);
            o[j] = luma_of<FMT>(q.x) | luma_of<FMT>(q.y) << 8 | luma_of<FMT>(q.z) << 16 | luma_of<FMT>(q.w) << 24;
          }
          *reinterpret_cast<uint4 *>(d + x) = make_uint4(o[0], o[1], o[2], o[3]);
        }
      } else {
        for (int k = x; k < min(w, x + 16); k++) {
          if (FMT == LIZG_PIX_GREY8) d[k] = row[k];
          else d[k] = (uint8_t)luma_of<FMT>(row[4 * k] | row[4 * k + 1] << 8 | row[4 * k + 2] << 16);
        }
      }
    }
  }
}

struct Develop {
  uint32_t row_stride, pixel_stride, x0, y0, ox, oy, w, h;
  int64_t pstride;
  float L[5], k[4];
  int tw, rb, row_cap, tiles_x, frames;   // a tile (tw x rb output pixels), the staged bytes a source row may take
};

// The first and last byte a run of samples [sa, sb] of a row occupies.
template <int FMT>
__device__ __forceinline__ void byte_span(uint32_t sa, uint32_t sb, uint32_t ps, int64_t *lo, int64_t *hi) {
  if (FMT == kRaw10) { *lo = (int64_t)(sa >> 2) * 5; *hi = (int64_t)(sb >> 2) * 5 + 4; }
  else if (FMT == kRaw12) { *lo = (int64_t)(sa >> 1) * 3; *hi = (int64_t)(sb >> 1) * 3 + 2; }
  else { *lo = (int64_t)sa * ps; *hi = (int64_t)sb * ps + 1; }
}

// Sample x of a row staged from the byte of sample sa on (develop.cpp:30-36).
template <int FMT>
__device__ __forceinline__ int raw_at(const uint8_t *r, uint32_t x, uint32_t sa, uint32_t ps) {
  if (FMT == kRaw16) { const int o = (int)(x - sa) * (int)ps; return r[o] | (r[o + 1] << 8); }
  if (FMT == kRaw10) { const int o = 5 * (int)((x >> 2) - (sa >> 2)); const int k = x & 3; return (r[o + k] << 2) | ((r[o + 4] >> (2 * k)) & 3); }
  const int o = 3 * (int)((x >> 1) - (sa >> 1));
  return (x & 1) ? ((r[o + 1] << 4) | (r[o + 2] >> 4)) : ((r[o] << 4) | (r[o + 2] & 15));
}

// The linear light of sample v at a CFA position of black Lp and scale kp: ((float)v - Lp) * kp clipped to [0, 4096]
// (develop.cpp rawLinear).
__device__ __forceinline__ float ln2(float v, float Lp, float kp) { return fminf(fmaxf((v - Lp) * kp, 0.0f), 4096.0f); }
__device__ __forceinline__ float ln(int v, float Lp, float kp) { return ln2((float)v, Lp, kp); }

// The bytes of a run of 16 samples (RAW10: four groups, 20 bytes; RAW12: eight groups, 24 bytes) whose first byte is
// p in shared memory, as words: the aligned words around the run funnel-shifted into place, byte j of the run in byte
// j & 3 of W[j >> 2].
template <int FMT>
__device__ __forceinline__ void run_words(const uint8_t *p, uint32_t (&W)[FMT == kRaw10 ? 5 : 6]) {
  constexpr int NW = FMT == kRaw10 ? 5 : 6;
  const int mis = (int)(reinterpret_cast<uintptr_t>(p) & 3);
  const uint32_t *a = reinterpret_cast<const uint32_t *>(p - mis);
  const uint32_t sh = 8u * (uint32_t)mis;
  uint32_t raw[NW + 1];
#pragma unroll
  for (int i = 0; i <= NW; i++) raw[i] = a[i];
#pragma unroll
  for (int i = 0; i < NW; i++) W[i] = __funnelshift_r(raw[i], raw[i + 1], sh);
}

// Byte J of a run, alone in the low byte.
template <int J>
__device__ __forceinline__ uint32_t run_byte(const uint32_t *W) { return __byte_perm(W[J >> 2], 0u, 0x4440u | (J & 3)); }

// Bits [B, B + N) of a run's bytes (B + N within one word), placed at bit S, the rest zero.
template <int B, int N, int S>
__device__ __forceinline__ uint32_t run_bits(const uint32_t *W) {
  constexpr int at = B & 31, m = ((1 << N) - 1) << S;
  const uint32_t w = W[B >> 5];
  return (S >= at ? w << (S - at) : w >> (at - S)) & (uint32_t)m;
}

// Sample I (0..15) of a run: RAW10 group I / 4 holds four high bytes, then a byte of the four 2-bit tails; RAW12
// group I / 2 two high bytes, then a byte of the two 4-bit tails.
template <int FMT, int I>
__device__ __forceinline__ uint32_t run_value(const uint32_t *W) {
  if (FMT == kRaw10) {
    constexpr int g = I / 4, k = I % 4;
    return (run_byte<5 * g + k>(W) << 2) | run_bits<8 * (5 * g + 4) + 2 * k, 2, 0>(W);
  } else {
    constexpr int g = I / 2, e = I % 2;
    return (run_byte<3 * g + e>(W) << 4) | run_bits<8 * (3 * g + 2) + 4 * e, 4, 0>(W);
  }
}

// Sample I of a run as a float, exactly: the bits of 2^23 + v less 2^23.
template <int FMT, int I>
__device__ __forceinline__ float run_float(const uint32_t *W) { return __int_as_float((int)(0x4b000000u | run_value<FMT, I>(W))) - 8388608.0f; }

// (int)x for x in [0, 2^23): x + 2^23 rounded toward zero keeps floor(x) in its mantissa.
__device__ __forceinline__ int floor_small(float x) { return __float_as_int(__fadd_rz(x, 8388608.0f)) & 0x7fffff; }

// NB output bytes (packed four to a word, first in the low byte) to q, in the widest stores its alignment allows.
template <int NB>
__device__ __forceinline__ void put(uint8_t *q, const uint32_t (&o)[NB / 4]) {
  const uintptr_t a = reinterpret_cast<uintptr_t>(q);
  if ((a & (NB - 1)) == 0) {
    if constexpr (NB == 16) *reinterpret_cast<uint4 *>(q) = make_uint4(o[0], o[1], o[2], o[3]);
    else *reinterpret_cast<uint2 *>(q) = make_uint2(o[0], o[1]);
  } else if ((a & 3) == 0) {
#pragma unroll
    for (int i = 0; i < NB / 4; i++) reinterpret_cast<uint32_t *>(q)[i] = o[i];
  } else {
#pragma unroll
    for (int i = 0; i < NB; i++) q[i] = (uint8_t)(o[i >> 2] >> (8 * (i & 3)));
  }
}

// P010: each sample's top byte, straight from the plane. A CTA takes a band of kBand rows, a warp a row, a lane 16
// samples at a time (two 16-byte loads, one 16-byte store where the pixel stride is 2 and both ends aligned).
__global__ void __launch_bounds__(kIngThreads) p010_kernel(const uint8_t *plane, Develop d, uint8_t *out) {
  const int bands = ((int)d.h + kBand - 1) / kBand, f = blockIdx.x / bands, ya = (blockIdx.x % bands) * kBand, yb = min((int)d.h, ya + kBand);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, w = (int)d.w;
  for (int y = ya + warp; y < yb; y += kIngThreads / 32) {
    const uint8_t *row = plane + f * d.pstride + (size_t)(d.y0 + d.oy + y) * d.row_stride + (size_t)(d.x0 + d.ox) * d.pixel_stride;
    uint8_t *q = out + ((int64_t)f * d.h + y) * w;
    for (int x = 16 * lane; x < w; x += 512) {
      const uint8_t *src = row + 2 * x;
      if (d.pixel_stride == 2 && x + 16 <= w && ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(q + x)) & 15) == 0) {
        const uint4 a = *reinterpret_cast<const uint4 *>(src), b = *reinterpret_cast<const uint4 *>(src + 16);
        *reinterpret_cast<uint4 *>(q + x) = make_uint4(__byte_perm(a.x, a.y, 0x7531u), __byte_perm(a.z, a.w, 0x7531u),
                                                        __byte_perm(b.x, b.y, 0x7531u), __byte_perm(b.z, b.w, 0x7531u));
      } else {
        for (int k = x; k < min(w, x + 16); k++) q[k] = row[(size_t)k * d.pixel_stride + 1];
      }
    }
  }
}

// A row's black levels and scales by column parity: {even, odd} columns of its first source row (0, 1), and of the
// second when binned (2, 3). Positions 0 1 on even source rows, 2 3 on odd; selected, not indexed, so that the levels
// stay in registers.
struct RowLevels {
  float L[4], k[4];
};
__device__ __forceinline__ RowLevels row_levels(const Develop &d, bool ro) {
  RowLevels v;
  v.L[0] = ro ? d.L[2] : d.L[0]; v.L[1] = ro ? d.L[3] : d.L[1]; v.L[2] = ro ? d.L[0] : d.L[2]; v.L[3] = ro ? d.L[1] : d.L[3];
  v.k[0] = ro ? d.k[2] : d.k[0]; v.k[1] = ro ? d.k[3] : d.k[1]; v.k[2] = ro ? d.k[0] : d.k[2]; v.k[3] = ro ? d.k[1] : d.k[3];
  return v;
}

// Output pixels [xq, xe) (at most four) of a row, sample by sample (develop.cpp:38-102): any format, any crop.
template <int FMT, int BIN>
__device__ __forceinline__ void develop_quad(const Develop &d, const uint8_t *r0, const uint8_t *r1, uint32_t sa, int xq, int xe,
                                             const RowLevels &lv, const uint8_t *lut, uint8_t *q) {
  uint32_t o = 0;   // four output bytes, first in the low byte
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const uint32_t rx = d.x0 + BIN * (d.ox + min(xq + k, xe - 1));
    const bool odd = rx & 1;   // an odd first column swaps the pair's CFA positions (selected, not indexed)
    const float La = odd ? lv.L[1] : lv.L[0], ka = odd ? lv.k[1] : lv.k[0];
    if (BIN == 2) {
      const float Lb = odd ? lv.L[0] : lv.L[1], kb = odd ? lv.k[0] : lv.k[1];
      const float Lc = odd ? lv.L[3] : lv.L[2], kc = odd ? lv.k[3] : lv.k[2], Ld = odd ? lv.L[2] : lv.L[3], kd = odd ? lv.k[2] : lv.k[3];
      const float v = ln(raw_at<FMT>(r0, rx, sa, d.pixel_stride), La, ka) + ln(raw_at<FMT>(r0, rx + 1, sa, d.pixel_stride), Lb, kb) +
                      ln(raw_at<FMT>(r1, rx, sa, d.pixel_stride), Lc, kc) + ln(raw_at<FMT>(r1, rx + 1, sa, d.pixel_stride), Ld, kd);
      o |= (uint32_t)lut[(int)(v * 0.25f)] << (8 * k);
    } else {
      o |= (uint32_t)lut[(int)ln(raw_at<FMT>(r0, rx, sa, d.pixel_stride), La, ka)] << (8 * k);
    }
  }
  if (xq + 4 <= xe && ((reinterpret_cast<uintptr_t>(q + xq) & 3) == 0)) *reinterpret_cast<uint32_t *>(q + xq) = o;
  else for (int k = 0; k < 4 && xq + k < xe; k++) q[xq + k] = (uint8_t)(o >> (8 * k));
}

// Sixteen output pixels from a run of 16 samples of one source row, unbinned: each sample's byte from its CFA
// position's table T[parity][v] = gamma(lin(v)).
template <int FMT, int I>
__device__ __forceinline__ uint32_t tab_px(const uint32_t *W, const uint8_t *T) {
  constexpr int kBits = FMT == kRaw10 ? 10 : 12;
  return T[((I & 1) << kBits) + run_value<FMT, I>(W)];
}
template <int FMT>
__device__ __forceinline__ void develop_run_tab(const uint32_t *W, const uint8_t *T, uint32_t (&ow)[4]) {
#define LIZG_W(j) __byte_perm(__byte_perm(tab_px<FMT, 4 * j>(W, T), tab_px<FMT, 4 * j + 1>(W, T), 0x0040u), \
                              __byte_perm(tab_px<FMT, 4 * j + 2>(W, T), tab_px<FMT, 4 * j + 3>(W, T), 0x0040u), 0x5410u)
  ow[0] = LIZG_W(0); ow[1] = LIZG_W(1); ow[2] = LIZG_W(2); ow[3] = LIZG_W(3);
#undef LIZG_W
}

// Eight output pixels from runs of 16 samples of two source rows, binned by 2: the quad's four linear values summed in
// the reference's order, averaged, read through the gamma table.
template <int FMT, int I>
__device__ __forceinline__ uint32_t bin_px(const uint32_t *W0, const uint32_t *W1, const RowLevels &lv, const uint8_t *lut) {
  const float v = ln2(run_float<FMT, 2 * I>(W0), lv.L[0], lv.k[0]) + ln2(run_float<FMT, 2 * I + 1>(W0), lv.L[1], lv.k[1]) +
                  ln2(run_float<FMT, 2 * I>(W1), lv.L[2], lv.k[2]) + ln2(run_float<FMT, 2 * I + 1>(W1), lv.L[3], lv.k[3]);
  return lut[floor_small(v * 0.25f)];
}
template <int FMT>
__device__ __forceinline__ void develop_run_bin(const uint32_t *W0, const uint32_t *W1, const RowLevels &lv, const uint8_t *lut, uint32_t (&ow)[2]) {
#define LIZG_W(j) __byte_perm(__byte_perm(bin_px<FMT, 4 * j>(W0, W1, lv, lut), bin_px<FMT, 4 * j + 1>(W0, W1, lv, lut), 0x0040u), \
                              __byte_perm(bin_px<FMT, 4 * j + 2>(W0, W1, lv, lut), bin_px<FMT, 4 * j + 3>(W0, W1, lv, lut), 0x0040u), 0x5410u)
  ow[0] = LIZG_W(0); ow[1] = LIZG_W(1);
#undef LIZG_W
}

// The develop, persistent: a CTA first lays out the gamma table (and, for RAW10 / RAW12 unbinned, each CFA position's
// table of output bytes by sample value), then takes tiles of tw x rb output pixels in turn. A tile's source rows are
// staged into shared memory, each at its global address's 16-byte phase so that the middle moves in aligned 16-byte
// asynchronous copies (the head and tail bytes one at a time, every read inside the plane), a warp a row. Where a
// RAW10 / RAW12 crop starts on a packing group a warp then takes an output row, a lane a run of 16 samples at a time
// (20 or 24 bytes read as words); elsewhere (RAW16, other crops, the ragged end of a row) four pixels at a time.
template <int FMT, int BIN>
__global__ void __launch_bounds__(kIngThreads) develop_kernel(const uint8_t *plane, Develop d, uint8_t *out) {
  constexpr bool kPacked = FMT == kRaw10 || FMT == kRaw12;
  constexpr int kBits = FMT == kRaw10 ? 10 : 12;
  constexpr bool kTab = kPacked && BIN == 1;
  constexpr int kTabBytes = kTab ? 4 << kBits : 0;
  extern __shared__ __align__(16) uint8_t sm[];
  uint8_t *lut = sm, *tab = sm + 4112, *rows = sm + 4112 + kTabBytes;
  __shared__ int s_base[16];   // staged row s: the byte of the tile's first sample at rows[s_base[s]]
  for (int i = threadIdx.x; i < 4112 / 16; i += blockDim.x)
    reinterpret_cast<uint4 *>(lut)[i] = reinterpret_cast<const uint4 *>(g_gamma)[i];
  if (kTab) {   // T[p][v] = gamma(lin(v)) at CFA position p
    __syncthreads();
#pragma unroll
    for (int p = 0; p < 4; p++) {
      const float Lp = d.L[p], kp = d.k[p];
      for (int v = threadIdx.x; v < (1 << kBits); v += blockDim.x) tab[(p << kBits) + v] = lut[(int)ln(v, Lp, kp)];
    }
  }
  const bool grouped = kPacked && ((d.x0 + BIN * d.ox) & (FMT == kRaw10 ? 3u : 1u)) == 0;
  constexpr int kRun = 16 / BIN;   // output pixels of a run of 16 samples
  const int tpr = (d.tw + 3) / 4, rpp = (int)blockDim.x / tpr, uu = (int)threadIdx.x % tpr, rr = (int)threadIdx.x / tpr;
  const int bands = ((int)d.h + d.rb - 1) / d.rb, per = bands * d.tiles_x, total = d.frames * per;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  for (int t = blockIdx.x; t < total; t += gridDim.x) {
    const int f = t / per, band = (t % per) / d.tiles_x, tx = t % d.tiles_x;
    const int ya = band * d.rb, yb = min((int)d.h, ya + d.rb), xa = tx * d.tw, xb = min((int)d.w, xa + d.tw);
    const uint8_t *pl = plane + f * d.pstride;
    const uint32_t sa = d.x0 + BIN * (d.ox + xa), sb = d.x0 + BIN * (d.ox + xb) - 1;
    int64_t blo, bhi;
    byte_span<FMT>(sa, sb, d.pixel_stride, &blo, &bhi);
    const int n = (int)(bhi - blo + 1), srows = (yb - ya) * BIN;
    __syncthreads();   // the previous tile's rows are read
    for (int s = warp; s < srows; s += nwarps) {
      const uint32_t ry = d.y0 + BIN * (d.oy + ya) + s;
      const uint8_t *g = pl + (size_t)ry * d.row_stride + blo;
      const int phase = (int)(reinterpret_cast<uintptr_t>(g) & 15), head = min(n, (16 - phase) & 15);
      if (lane == 0) s_base[s] = s * d.row_cap + phase;
      uint8_t *r = rows + s * d.row_cap + phase;
      const int chunks = (n - head) / 16, tail0 = head + 16 * chunks;
      if (lane < head) r[lane] = g[lane];
      for (int i = lane; i < chunks; i += 32) {
        const uint32_t sa16 = (uint32_t)__cvta_generic_to_shared(r + head + 16 * i);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa16), "l"(g + head + 16 * i) : "memory");
      }
      if (tail0 + lane < n) r[tail0 + lane] = g[tail0 + lane];
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    __syncthreads();
    uint8_t *dst = out + (int64_t)f * d.w * d.h;
    if (grouped) {
      const int runs = (xb - xa) / kRun;   // whole runs; the ragged rest four pixels at a time
      for (int yl = warp; yl < yb - ya; yl += nwarps) {
        const int y = ya + yl;
        const uint8_t *r0 = rows + s_base[BIN * yl], *r1 = rows + s_base[BIN * yl + BIN - 1];
        const bool ro = (d.y0 + BIN * (d.oy + y)) & 1;
        uint8_t *q = dst + (int64_t)y * d.w;
        const RowLevels lv = row_levels(d, ro);
        for (int u = lane; u < runs; u += 32) {
          const int x = xa + kRun * u;
          const uint32_t rx = d.x0 + BIN * (d.ox + x);   // the run's first sample, on a group
          const int o = FMT == kRaw10 ? 5 * (int)((rx >> 2) - (sa >> 2)) : 3 * (int)((rx >> 1) - (sa >> 1));
          if constexpr (BIN == 1) {
            uint32_t W[FMT == kRaw10 ? 5 : 6], ow[4];
            run_words<FMT>(r0 + o, W);
            develop_run_tab<FMT>(W, tab + ((ro ? 2 : 0) << kBits), ow);
            put<16>(q + x, ow);
          } else {
            uint32_t W0[FMT == kRaw10 ? 5 : 6], W1[FMT == kRaw10 ? 5 : 6], ow[2];
            run_words<FMT>(r0 + o, W0);
            run_words<FMT>(r1 + o, W1);
            develop_run_bin<FMT>(W0, W1, lv, lut, ow);
            put<8>(q + x, ow);
          }
        }
        for (int xq = xa + kRun * runs + 4 * lane; xq < xb; xq += 128) develop_quad<FMT, BIN>(d, r0, r1, sa, xq, xb, lv, lut, q);
      }
    } else if (rr < rpp) {
      for (int yl = rr; yl < yb - ya; yl += rpp) {
        const int y = ya + yl, x = xa + 4 * uu;
        if (x >= xb) break;
        const uint8_t *r0 = rows + s_base[BIN * yl], *r1 = rows + s_base[BIN * yl + BIN - 1];
        develop_quad<FMT, BIN>(d, r0, r1, sa, x, xb, row_levels(d, (d.y0 + BIN * (d.oy + y)) & 1), lut, dst + (int64_t)y * d.w);
      }
    }
  }
}

static std::mutex g_gamma_mu;
static bool g_gamma_done[64];

static cudaError_t gamma_ready() {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_gamma_mu);
  if (dev >= 0 && dev < 64 && g_gamma_done[dev]) return cudaSuccess;
  uint8_t t[4112] = {};
  for (int i = 0; i <= 4096; i++) t[i] = (uint8_t)std::lround(255.0 * std::pow(i / 4096.0, 1 / 2.2));
  const cudaError_t e = cudaMemcpyToSymbol(g_gamma, t, sizeof t);
  if (e == cudaSuccess && dev >= 0 && dev < 64) g_gamma_done[dev] = true;
  return e;
}

}  // namespace lizg

extern "C" {

int lizg_ingest_pixels_dev(const uint8_t *d_px, int w, int h, int stride, int64_t frame_stride, int fmt, int frames, uint8_t *d_luma, void *stream) {
  using namespace lizg;
  const int bpp = fmt == LIZG_PIX_GREY8 ? 1 : (fmt == LIZG_PIX_RGBX8 || fmt == LIZG_PIX_RGBA8 || fmt == LIZG_PIX_BGRA8) ? 4 : 0;
  if (!bpp) return record_error(LIZG_E_ARG, "lizg_ingest_pixels_dev: no such pixel format");
  if (!d_px || !d_luma || w < 1 || h < 1 || frames < 1 || stride < w * bpp || frame_stride < (int64_t)stride * (h - 1) + (int64_t)w * bpp)
    return record_error(LIZG_E_ARG, "lizg_ingest_pixels_dev: NULL buffer or bad geometry");
  int sms = 0;
  if (int rc = device_ready(&sms)) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const unsigned grid = (unsigned)frames * ((h + kBand - 1) / kBand);
  switch (fmt) {
    case LIZG_PIX_GREY8: pixels_kernel<LIZG_PIX_GREY8><<<grid, kIngThreads, 0, st>>>(d_px, w, h, stride, frame_stride, d_luma); break;
    case LIZG_PIX_BGRA8: pixels_kernel<LIZG_PIX_BGRA8><<<grid, kIngThreads, 0, st>>>(d_px, w, h, stride, frame_stride, d_luma); break;
    default: pixels_kernel<LIZG_PIX_RGBA8><<<grid, kIngThreads, 0, st>>>(d_px, w, h, stride, frame_stride, d_luma); break;
  }
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : record_error(LIZG_E_CUDA, (std::string("lizg_ingest_pixels_dev: ") + cudaGetErrorString(e)).c_str());
}

int lizg_develop_dev(const lizg_raw_frame *r, const uint8_t *d_plane, int64_t plane_bytes, int64_t plane_stride, int frames, uint32_t ox,
                     uint32_t oy, uint32_t w, uint32_t h, uint8_t *d_out, void *stream) {
  using namespace lizg;
  if (!r || !d_plane || !d_out || frames < 1 || w < 1 || h < 1) return record_error(LIZG_E_ARG, "lizg_develop_dev: NULL buffer or empty frame");
  const int fmt = r->format;
  if (fmt != kRaw16 && fmt != kRaw10 && fmt != kRaw12 && fmt != kP010) return record_error(LIZG_E_ARG, "lizg_develop_dev: no such camera format");
  const uint32_t bin = fmt == kP010 ? 1 : r->bin;
  if (bin != 1 && bin != 2) return record_error(LIZG_E_ARG, "lizg_develop_dev: bin must be 1 or 2");
  if (fmt == kRaw16 && r->pixel_stride < 2) return record_error(LIZG_E_ARG, "lizg_develop_dev: RAW16 needs a pixel stride of 2 or more");
  if (fmt == kP010 && r->pixel_stride < 2) return record_error(LIZG_E_ARG, "lizg_develop_dev: P010 needs a pixel stride of 2 or more");
  if ((fmt == kRaw16 || fmt == kP010) && r->pixel_stride > 16) return record_error(LIZG_E_ARG, "lizg_develop_dev: pixel stride above 16");
  // every byte the develop reads lies in the plane: the last row and the last sample's bytes
  const uint64_t last_row = (uint64_t)r->y0 + (uint64_t)bin * (oy + h) - 1, last_x = (uint64_t)r->x0 + (uint64_t)bin * (ox + w) - 1;
  uint64_t last_byte;
  if (fmt == kRaw10) last_byte = last_x / 4 * 5 + 4;
  else if (fmt == kRaw12) last_byte = last_x / 2 * 3 + 2;
  else last_byte = last_x * r->pixel_stride + 1;
  if (last_byte >= r->row_stride || last_row * r->row_stride + last_byte >= (uint64_t)plane_bytes || (frames > 1 && plane_stride < plane_bytes))
    return record_error(LIZG_E_ARG, "lizg_develop_dev: the crop reads past the plane");
  int sms = 0;
  if (int rc = device_ready(&sms)) return rc;
  cudaError_t e = gamma_ready();
  if (e != cudaSuccess) return record_error(LIZG_E_CUDA, (std::string("lizg_develop_dev: ") + cudaGetErrorString(e)).c_str());
  Develop d{};
  d.row_stride = r->row_stride; d.pixel_stride = r->pixel_stride; d.x0 = r->x0; d.y0 = r->y0; d.ox = ox; d.oy = oy; d.w = w; d.h = h;
  d.pstride = plane_stride;
  for (int p = 0; p < 5; p++) d.L[p] = r->levels[p];
  for (int p = 0; p < 4; p++) d.k[p] = r->levels[5 + p] * 4096.f / std::fmax(1.f, r->levels[4] - r->levels[p]);   // rawScales
  // the tile: 1024 output pixels across (fewer where a source row's bytes would pass 8 KB), 16 source rows
  const double bps = fmt == kRaw10 ? 1.25 : fmt == kRaw12 ? 1.5 : (double)r->pixel_stride;
  int tw = 1024;
  while (tw > 16 && bin * tw * bps > 8000) tw /= 2;
  d.tw = (int)std::min<uint32_t>(w, (uint32_t)tw);
  d.rb = 16 / (int)bin;
  d.row_cap = ((int)((bin * d.tw + 8) * bps) + 48 + 15) & ~15;   // a multiple of 16: every staged row starts aligned
  d.tiles_x = (int)((w + d.tw - 1) / d.tw);
  d.frames = frames;
  const int64_t tiles = (int64_t)frames * (int64_t)((h + d.rb - 1) / d.rb) * d.tiles_x;
  if (tiles > INT32_MAX) return record_error(LIZG_E_ARG, "lizg_develop_dev: too many tiles in one call");
  // shared memory: the gamma table, the per-position byte tables (RAW10 / RAW12 unbinned), 16 staged rows
  const int tab = (fmt == kRaw10 || fmt == kRaw12) && bin == 1 ? 4 << (fmt == kRaw10 ? 10 : 12) : 0;
  const int smem = 4112 + tab + 16 * d.row_cap;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  auto go = [&](auto kern) -> cudaError_t {
    cudaError_t ee = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (ee != cudaSuccess) return ee;
    int occ = 0;   // persistent: as many CTAs as fit at once, each taking tiles in turn
    ee = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kIngThreads, smem);
    if (ee != cudaSuccess) return ee;
    const unsigned grid = (unsigned)std::min<int64_t>(tiles, (int64_t)sms * std::max(occ, 1));
    kern<<<grid, kIngThreads, smem, st>>>(d_plane, d, d_out);
    return cudaGetLastError();
  };
  if (fmt == kP010) {
    p010_kernel<<<(unsigned)frames * ((h + kBand - 1) / kBand), kIngThreads, 0, st>>>(d_plane, d, d_out);
    e = cudaGetLastError();
  }
  else if (fmt == kRaw16) e = bin == 2 ? go(develop_kernel<kRaw16, 2>) : go(develop_kernel<kRaw16, 1>);
  else if (fmt == kRaw10) e = bin == 2 ? go(develop_kernel<kRaw10, 2>) : go(develop_kernel<kRaw10, 1>);
  else e = bin == 2 ? go(develop_kernel<kRaw12, 2>) : go(develop_kernel<kRaw12, 1>);
  return e == cudaSuccess ? 0 : record_error(LIZG_E_CUDA, (std::string("lizg_develop_dev: ") + cudaGetErrorString(e)).c_str());
}

}  // extern "C"

// Camera-format ingest on sm_103a: captured frames in the formats cameras and apps hand over turned into the 8-bit
// luma rows the receiver reads, on the device, a batch of frames a launch. Two sources, restated from the reference:
//   - liz_decode's pixel formats (liblizard/api/codec.cpp:128-140): GREY8 rows compacted, RGBA8 / RGBX8 by ob_luma's
//     (77 r + 150 g + 29 b + 128) >> 8 (liblizard/src/acquire.c:67-83), BGRA8 the same from B, G, R;
//   - the camera develop (liblizard/core/ingest/develop.cpp:9-102): P010's top byte; RAW16 / RAW10 / RAW12 less the
//     CFA position's black level, times its gain scale, clipped to [0, 4096] and read through the 4097-step gamma 1/2.2
//     table, each 2 x 2 quad averaged when binned by 2.
// Compiled with -fmad=false (the develop's float order is the reference's). A CTA takes a band of kBand rows of a
// frame, a thread four output pixels at a time; the gamma table sits in the CTA's shared memory. The work is bytes in
// and bytes out, bound by HBM.
#include <cuda_runtime.h>
#include <stdint.h>
#include <cmath>
#include <mutex>
#include <string>
#include "lizard_gb300.h"
#include "lizg_internal.h"

namespace lizg {

constexpr int kBand = 16, kIngThreads = 256;
constexpr int kRaw16 = 0x20, kRaw10 = 0x25, kRaw12 = 0x26, kP010 = 0x36;

static __device__ uint8_t g_gamma[4100];   // the 4097 steps of gamma 1 / 2.2 (develop.cpp:17-22), made on the host

template <int FMT>
__global__ void __launch_bounds__(kIngThreads) pixels_kernel(const uint8_t *px, int w, int h, int stride, int64_t fstride, uint8_t *out) {
  const int bands = (h + kBand - 1) / kBand, f = blockIdx.x / bands, y0 = (blockIdx.x % bands) * kBand, y1 = min(h, y0 + kBand);
  const uint8_t *src = px + f * fstride;
  uint8_t *dst = out + (int64_t)f * w * h;
  const int quads = (w + 3) / 4;
  for (int t = threadIdx.x; t < (y1 - y0) * quads; t += blockDim.x) {
    const int y = y0 + t / quads, x = 4 * (t % quads);
    const uint8_t *row = src + (int64_t)y * stride;
    uint8_t o[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int xx = min(x + k, w - 1);
      if (FMT == LIZG_PIX_GREY8) o[k] = row[xx];
      else if (FMT == LIZG_PIX_BGRA8) o[k] = (uint8_t)((77 * row[4 * xx + 2] + 150 * row[4 * xx + 1] + 29 * row[4 * xx] + 128) >> 8);
      else o[k] = (uint8_t)((77 * row[4 * xx] + 150 * row[4 * xx + 1] + 29 * row[4 * xx + 2] + 128) >> 8);
    }
    uint8_t *d = dst + (int64_t)y * w + x;
    if (x + 4 <= w && ((reinterpret_cast<uintptr_t>(d) & 3) == 0)) *reinterpret_cast<uchar4 *>(d) = make_uchar4(o[0], o[1], o[2], o[3]);
    else for (int k = 0; k < 4 && x + k < w; k++) d[k] = o[k];
  }
}

struct Develop {
  uint32_t row_stride, pixel_stride, x0, y0, ox, oy, w, h;
  int64_t pstride;
  float L[5], k[4];
};

template <int FMT>
__device__ __forceinline__ int raw_at(const uint8_t *row, uint32_t x, uint32_t ps) {
  if (FMT == kRaw16) { const uint8_t *p = row + (size_t)x * ps; return p[0] | (p[1] << 8); }
  if (FMT == kRaw10) { const uint8_t *g = row + (size_t)(x >> 2) * 5; const int k = x & 3; return (g[k] << 2) | ((g[4] >> (2 * k)) & 3); }
  const uint8_t *g = row + (size_t)(x >> 1) * 3;
  return (x & 1) ? ((g[1] << 4) | (g[2] >> 4)) : ((g[0] << 4) | (g[2] & 15));
}

__device__ __forceinline__ float lin(int v, const Develop &d, int p) {
  const float f = ((float)v - d.L[p]) * d.k[p];
  return f <= 0 ? 0.f : f >= 4096.f ? 4096.f : f;
}

template <int FMT, int BIN>
__global__ void __launch_bounds__(kIngThreads) develop_kernel(const uint8_t *plane, Develop d, uint8_t *out) {
  __shared__ uint8_t lut[4100];
  for (int i = threadIdx.x; i < 4097; i += blockDim.x) lut[i] = g_gamma[i];
  __syncthreads();
  const int bands = ((int)d.h + kBand - 1) / kBand, f = blockIdx.x / bands, y0 = (blockIdx.x % bands) * kBand, y1 = min((int)d.h, y0 + kBand);
  const uint8_t *pl = plane + f * d.pstride;
  uint8_t *dst = out + (int64_t)f * d.w * d.h;
  const int quads = ((int)d.w + 3) / 4;
  for (int t = threadIdx.x; t < (y1 - y0) * quads; t += blockDim.x) {
    const uint32_t y = y0 + t / quads, x = 4 * (t % quads);
    uint8_t o[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const uint32_t xx = min(x + k, d.w - 1);
      if (FMT == kP010) {
        o[k] = pl[(size_t)(d.y0 + d.oy + y) * d.row_stride + (size_t)(d.x0 + d.ox + xx) * d.pixel_stride + 1];
      } else if (BIN == 2) {
        const uint32_t ry = d.y0 + 2 * (d.oy + y), rx = d.x0 + 2 * (d.ox + xx);
        const uint8_t *r0 = pl + (size_t)ry * d.row_stride, *r1 = r0 + d.row_stride;
        const int p0 = (ry & 1) << 1, p1 = ((ry + 1) & 1) << 1, q0 = rx & 1, q1 = (rx + 1) & 1;
        const float v = lin(raw_at<FMT>(r0, rx, d.pixel_stride), d, p0 | q0) + lin(raw_at<FMT>(r0, rx + 1, d.pixel_stride), d, p0 | q1) +
                        lin(raw_at<FMT>(r1, rx, d.pixel_stride), d, p1 | q0) + lin(raw_at<FMT>(r1, rx + 1, d.pixel_stride), d, p1 | q1);
        o[k] = lut[(int)(v * 0.25f)];
      } else {
        const uint32_t ry = d.y0 + d.oy + y, rx = d.x0 + d.ox + xx;
        o[k] = lut[(int)lin(raw_at<FMT>(pl + (size_t)ry * d.row_stride, rx, d.pixel_stride), d, ((ry & 1) << 1) | (rx & 1))];
      }
    }
    uint8_t *q = dst + (int64_t)y * d.w + x;
    if (x + 4 <= d.w && ((reinterpret_cast<uintptr_t>(q) & 3) == 0)) *reinterpret_cast<uchar4 *>(q) = make_uchar4(o[0], o[1], o[2], o[3]);
    else for (int k = 0; k < 4 && x + k < d.w; k++) q[k] = o[k];
  }
}

static std::mutex g_gamma_mu;
static bool g_gamma_done[64];

static cudaError_t gamma_ready() {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_gamma_mu);
  if (dev >= 0 && dev < 64 && g_gamma_done[dev]) return cudaSuccess;
  uint8_t t[4100] = {};
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
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const unsigned grid = (unsigned)frames * ((h + kBand - 1) / kBand);
  if (fmt == kP010) develop_kernel<kP010, 1><<<grid, kIngThreads, 0, st>>>(d_plane, d, d_out);
  else if (fmt == kRaw16) { if (bin == 2) develop_kernel<kRaw16, 2><<<grid, kIngThreads, 0, st>>>(d_plane, d, d_out); else develop_kernel<kRaw16, 1><<<grid, kIngThreads, 0, st>>>(d_plane, d, d_out); }
  else if (fmt == kRaw10) { if (bin == 2) develop_kernel<kRaw10, 2><<<grid, kIngThreads, 0, st>>>(d_plane, d, d_out); else develop_kernel<kRaw10, 1><<<grid, kIngThreads, 0, st>>>(d_plane, d, d_out); }
  else { if (bin == 2) develop_kernel<kRaw12, 2><<<grid, kIngThreads, 0, st>>>(d_plane, d, d_out); else develop_kernel<kRaw12, 1><<<grid, kIngThreads, 0, st>>>(d_plane, d, d_out); }
  e = cudaGetLastError();
  return e == cudaSuccess ? 0 : record_error(LIZG_E_CUDA, (std::string("lizg_develop_dev: ") + cudaGetErrorString(e)).c_str());
}

}  // extern "C"

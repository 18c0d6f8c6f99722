// Oracle (test infrastructure only): camera-format ingest to the decoder's 8-bit luma, restated in plain C from the
// reference: the pixel formats of liz_decode (liblizard/api/codec.cpp:128-140, ob_luma liblizard/src/acquire.c:67-83)
// and the camera develop of P010, RAW16, RAW10 and RAW12 (liblizard/core/ingest/develop.cpp:9-102). Pinned against
// the reference's own develop.cpp compiled here (oracle/ref_develop.cpp) and its own ob_luma (oracle/_ref/libref.so).
#include <math.h>
#include <stdint.h>
#include <string.h>
#include "oracle.h"

enum { PIX_GREY8 = 1, PIX_RGBX8 = 2, PIX_RGBA8 = 3, PIX_BGRA8 = 4, RAW16 = 0x20, RAW10 = 0x25, RAW12 = 0x26, P010 = 0x36 };

// A frame of w x h pixels (rows stride bytes apart) to tight luma rows (liblizard/api/codec.cpp:128-140).
int orc_ingest_pixels(const uint8_t *px, int w, int h, int stride, int fmt, uint8_t *out) {
  for (int y = 0; y < h; y++) {
    const uint8_t *row = px + (size_t)y * stride;
    uint8_t *o = out + (size_t)y * w;
    if (fmt == PIX_GREY8) memcpy(o, row, (size_t)w);
    else if (fmt == PIX_BGRA8) for (int x = 0; x < w; x++) o[x] = (uint8_t)((77 * row[4 * x + 2] + 150 * row[4 * x + 1] + 29 * row[4 * x] + 128) >> 8);
    else if (fmt == PIX_RGBA8 || fmt == PIX_RGBX8) for (int x = 0; x < w; x++) o[x] = (uint8_t)((77 * row[4 * x] + 150 * row[4 * x + 1] + 29 * row[4 * x + 2] + 128) >> 8);
    else return -1;
  }
  return 0;
}

// The 4097 steps of gamma 1 / 2.2 (develop.cpp:17-22).
void orc_gamma_lut(uint8_t *t) {
  for (int i = 0; i <= 4096; i++) t[i] = (uint8_t)lround(255.0 * pow(i / 4096.0, 1 / 2.2));
}

// Sample x of a plane's row (develop.cpp:30-36).
static int raw_at(int fmt, const uint8_t *row, uint32_t x, uint32_t ps) {
  if (fmt == RAW16) { const uint8_t *p = row + (size_t)x * ps; return p[0] | (p[1] << 8); }
  if (fmt == RAW10) { const uint8_t *g = row + (size_t)(x >> 2) * 5; const int k = x & 3; return (g[k] << 2) | ((g[4] >> (2 * k)) & 3); }
  const uint8_t *g = row + (size_t)(x >> 1) * 3;
  return (x & 1) ? ((g[1] << 4) | (g[2] >> 4)) : ((g[0] << 4) | (g[2] & 15));
}

static float lin(int v, const float *L, const float *k, int p) {
  const float f = ((float)v - L[p]) * k[p];
  return f <= 0 ? 0.f : f >= 4096.f ? 4096.f : f;
}

// The developed frame's w x h from (ox, oy) into out, rows out_stride apart (develop.cpp:38-102 developLuma). levels:
// black per 2 x 2 position, white, gain per position.
int orc_develop(int fmt, const uint8_t *plane, uint32_t row_stride, uint32_t pixel_stride, uint32_t x0, uint32_t y0, uint32_t bin,
                const float *levels, uint32_t ox, uint32_t oy, uint32_t w, uint32_t h, uint8_t *out, size_t out_stride) {
  if (fmt == P010) {
    for (uint32_t y = 0; y < h; y++) {
      const uint8_t *row = plane + (size_t)(y0 + oy + y) * row_stride + (size_t)(x0 + ox) * pixel_stride + 1;
      uint8_t *o = out + y * out_stride;
      for (uint32_t x = 0; x < w; x++) o[x] = row[(size_t)x * pixel_stride];
    }
    return 0;
  }
  if (fmt != RAW16 && fmt != RAW10 && fmt != RAW12) return -1;
  uint8_t lut[4097];
  orc_gamma_lut(lut);
  const float *L = levels;
  float k[4];
  for (int p = 0; p < 4; p++) k[p] = L[5 + p] * 4096.f / fmaxf(1.f, L[4] - L[p]);
  for (uint32_t y = 0; y < h; y++) {
    uint8_t *o = out + y * out_stride;
    if (bin == 2) {
      const uint32_t ry = y0 + 2 * (oy + y);
      const uint8_t *r0 = plane + (size_t)ry * row_stride, *r1 = r0 + row_stride;
      const int p0 = (ry & 1) << 1, p1 = ((ry + 1) & 1) << 1;
      for (uint32_t x = 0; x < w; x++) {
        const uint32_t rx = x0 + 2 * (ox + x);
        const int q0 = rx & 1, q1 = (rx + 1) & 1;
        const float v = lin(raw_at(fmt, r0, rx, pixel_stride), L, k, p0 | q0) + lin(raw_at(fmt, r0, rx + 1, pixel_stride), L, k, p0 | q1) +
                        lin(raw_at(fmt, r1, rx, pixel_stride), L, k, p1 | q0) + lin(raw_at(fmt, r1, rx + 1, pixel_stride), L, k, p1 | q1);
        o[x] = lut[(int)(v * 0.25f)];
      }
    } else {
      const uint32_t ry = y0 + oy + y;
      const uint8_t *row = plane + (size_t)ry * row_stride;
      const int pr = (ry & 1) << 1;
      for (uint32_t x = 0; x < w; x++) {
        const uint32_t rx = x0 + ox + x;
        o[x] = lut[(int)lin(raw_at(fmt, row, rx, pixel_stride), L, k, pr | (rx & 1))];
      }
    }
  }
  return 0;
}

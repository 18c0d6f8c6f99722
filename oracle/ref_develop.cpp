// Harness around the reference's camera develop (liblizard/core/ingest/develop.cpp), compiled from the reference's
// own source where it lies. TEST INFRASTRUCTURE ONLY: oracle/Makefile builds it into oracle/_ref/libref_develop.so
// where the reference tree is present, so that the tests can hold the develop's restatement and the GPU kernel to the
// reference's own bytes. Plain C entry points over the reference's C++ API.
#include <cstdint>
#include <cstring>
#include "develop.h"

extern "C" int refd_develop(int format, const uint8_t *plane, uint32_t row_stride, uint32_t pixel_stride, uint32_t x0, uint32_t y0,
                            uint32_t bin, const float *levels, uint32_t ox, uint32_t oy, uint32_t w, uint32_t h, uint8_t *out, size_t out_stride) {
  if (!lizard::rawFormatKnown(format)) return -1;
  lizard::RawFrame r;
  r.plane = plane; r.rowStride = row_stride; r.pixelStride = pixel_stride; r.format = format;
  r.x0 = x0; r.y0 = y0; r.bin = bin;
  std::memcpy(r.levels, levels, sizeof r.levels);
  lizard::developLuma(r, ox, oy, w, h, out, out_stride);
  return 0;
}

extern "C" void refd_gamma_lut(uint8_t *t) { std::memcpy(t, lizard::gammaLut(), 4097); }

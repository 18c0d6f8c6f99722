// lizard_finish on the GPU, for the reference's own per-frame codec. The reference splits a decode where the
// registration ends (lizard_acquire / lizard_finish, liblizard/src/lizard_phy.h:193-240) and hands out what the
// acquisition holds (lizard_held_image / lizard_held_reg, liblizard/src/internal.h:199-202); this file takes that
// registration and frame to lizard_gb300's receiver (rows a-e: the decode's own integer read, the detrended transform,
// pilots, soft values, LDPC, CRC) in place of the C's lizard_finish, and lets the hold go as lizard_finish would.
// The blocks verified, their bytes and their LDPC iterations are lizard_finish's (the identical CRC-passing set).
//
// It is compiled inside the reference's tree, its liblizard/src on the include path, and linked against
// liblizard_gb300.so; the reference's codec.c (liblizard/core/cpu/codec.c) would call lizard_finish_gpu where it now
// calls lizard_finish.
#include <stdlib.h>
#include <string.h>

#include "internal.h"
#include "lizard_phy.h"
#include "lizard_gb300.h"

#include "lizard_finish_gpu.h"

struct lizard_gpu {
  lizg_rx *rx;
  int n, subch, span, blocks, nodes;
  float *reg;      // H (9), then the mesh's (dx, dy)
  int32_t *its;    // per block
};

lizard_gpu *lizard_gpu_new(const lizard_t *f) {
  lizard_gpu *g = calloc(1, sizeof *g);
  if (!g) return NULL;
  g->n = f->n; g->subch = f->subch; g->span = f->frame.w - 2 * f->margin; g->blocks = f->blocks;
  g->nodes = f->frame.nx * f->frame.ny;
  g->reg = malloc(sizeof(float) * (9 + 2 * (size_t)g->nodes));
  g->its = malloc(sizeof(int32_t) * (size_t)g->blocks);
  g->rx = g->reg && g->its ? lizg_rx_new(g->n, g->subch, g->span, 1) : NULL;
  if (!g->rx) { lizard_gpu_free(g); return NULL; }
  return g;
}

void lizard_gpu_free(lizard_gpu *g) {
  if (!g) return;
  lizg_rx_free(g->rx);
  free(g->reg);
  free(g->its);
  free(g);
}

int lizard_finish_gpu(lizard_gpu *g, const lizard_t *f, uint8_t *blocks, uint8_t *ok, int8_t *its) {
  memset(ok, 0, (size_t)f->blocks);
  if (!g || f->n != g->n || f->subch != g->subch || f->blocks != g->blocks) { lizard_release(f); return LIZG_E_ARG; }
  const image_t *im = lizard_held_image(f);
  const ob_reg_t *reg = lizard_held_reg(f);
  if (!im->lin) { lizard_release(f); return LIZG_E_STATE; }   // the GPU reads the frame at gamma 1, as the decode does
  memcpy(g->reg, reg->H.h, 9 * sizeof(float));
  for (int k = 0; k < g->nodes; k++) { g->reg[9 + 2 * k] = reg->nodes[k].dx; g->reg[10 + 2 * k] = reg->nodes[k].dy; }
  const int rc = lizg_rx_finish_luma_host(g->rx, im->px, im->w, im->h, im->w, (int64_t)im->w * im->h, g->reg, 1, blocks, ok, g->its);
  lizard_release(f);
  if (rc < 0) return rc;
  if (its) for (int b = 0; b < f->blocks; b++) its[b] = (int8_t)g->its[b];
  return rc;
}

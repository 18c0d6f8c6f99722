// Drives the reference's own codec with its finish on the GPU (lizard_gb300/integration/lizard_finish_gpu.c): one
// luma frame (a file: int32 w, int32 h, then w x h bytes) registered by the reference's lizard_acquire, finished by
// lizard_finish_gpu, then registered again and finished by the reference's own lizard_finish, and the two compared.
// Exit 0: the same verified blocks, bytes and iterations; 1: they differ; 2: bad input or no registration; 3: no GPU
// handle could be made (the message printed). TEST INFRASTRUCTURE: built by oracle/Makefile's `integration` target.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "internal.h"
#include "lizard_phy.h"
#include "lizard_gb300.h"
#include "lizard_finish_gpu.h"

int main(int argc, char **argv) {
  if (argc != 5) { fprintf(stderr, "usage: %s frame.raw n subch span\n", argv[0]); return 2; }
  FILE *fp = fopen(argv[1], "rb");
  int32_t wh[2];
  if (!fp || fread(wh, sizeof wh, 1, fp) != 1) return 2;
  uint8_t *luma = malloc((size_t)wh[0] * wh[1]);
  if (!luma || fread(luma, 1, (size_t)wh[0] * wh[1], fp) != (size_t)wh[0] * wh[1]) return 2;
  fclose(fp);
  lizard_t f;
  if (lizard_init(&f, atoi(argv[2]), atoi(argv[3]), atoi(argv[4]))) return 2;
  lizard_gpu *g = lizard_gpu_new(&f);
  if (!g) { printf("nogpu: %s\n", lizg_last_error()); return 3; }
  uint8_t *b0 = calloc((size_t)f.blocks, 476), *b1 = calloc((size_t)f.blocks, 476), *ok0 = calloc(f.blocks, 1), *ok1 = calloc(f.blocks, 1);
  int8_t *its0 = calloc(f.blocks, 1);
  ob_result_t res;
  if (!lizard_acquire(&f, luma, wh[0], wh[1], 1.0f, &res)) return 2;
  const int v0 = lizard_finish_gpu(g, &f, b0, ok0, its0);
  if (!lizard_acquire(&f, luma, wh[0], wh[1], 1.0f, &res)) return 2;
  const int v1 = lizard_finish(&f, NULL, b1, ok1, &res);
  const int8_t *its1;
  const float *est;
  lizard_block_stats(&f, &its1, &est);
  int same = v0 == v1 && !memcmp(ok0, ok1, f.blocks) && !memcmp(its0, its1, f.blocks);
  for (int b = 0; b < f.blocks; b++) if (ok0[b] && memcmp(b0 + 476 * b, b1 + 476 * b, 476)) same = 0;
  printf("gpu %d cpu %d same %d\n", v0, v1, same);
  lizard_gpu_free(g);
  lizard_free(&f);
  return same ? 0 : 1;
}

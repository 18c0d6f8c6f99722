// lizard_finish on the GPU for the reference's per-frame codec (see lizard_finish_gpu.c). Include after the
// reference's lizard_phy.h.
#ifndef LIZARD_FINISH_GPU_H
#define LIZARD_FINISH_GPU_H
#include <stdint.h>

typedef struct lizard_gpu lizard_gpu;
// One GPU receiver for the format f was made for (its picture size, sub-channels and ring); NULL where none can be made
// (lizg_last_error says why: no CUDA device, no memory).
lizard_gpu *lizard_gpu_new(const lizard_t *f);
void lizard_gpu_free(lizard_gpu *g);
// After lizard_acquire(f, ...) returned a registration: the held frame finished on the GPU, as lizard_finish(f, NULL,
// blocks, ok, res) finishes it. blocks: f->blocks x 476 bytes; ok[b] 1 where block b verified; its (may be NULL): the
// LDPC iterations a block took (-1 never converged, -2 declined, -3 stalled), as lizard_block_stats gives them. The
// hold is let go. Returns the blocks verified, or a negative LIZG_E_* code.
int lizard_finish_gpu(lizard_gpu *g, const lizard_t *f, uint8_t *blocks, uint8_t *ok, int8_t *its);
#endif

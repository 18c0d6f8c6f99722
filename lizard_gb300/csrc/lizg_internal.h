// Internal declarations shared by the host shim (api.cpp) and the kernels (*.cu). Not part of the C ABI.
#ifndef LIZG_INTERNAL_H
#define LIZG_INTERNAL_H
#include <cuda_runtime.h>
#include <stdint.h>

namespace lizg {

// One launch of the LDPC kernel over the codewords of one code.
struct LdpcLaunch {
  const int8_t *llr;      // the batch's LLRs, codeword i at llr + off[i]
  uint8_t *bits;          // packed hard bits, codeword i at bits + off[i] / 8
  int32_t *its;           // per codeword: iterations, -1 or -3
  uint8_t *ok;            // per codeword: CRC-32C of the first 476 bytes matches
  const int32_t *list;    // the codeword indices of this code
  const int64_t *off;     // per codeword LLR offset
  int count;              // entries of list
  int *counter;           // work counter, zero at launch
  int max_iter, stall_it;
  float stall_ratio;
};

cudaError_t ldpc_upload_tables();
// code: 0 = 7/8, 1 = 3/4, 2 = 2/3, 3 = 1/2. sms: the device's SM count (the persistent grid's bound).
cudaError_t ldpc_launch(int code, const LdpcLaunch &a, int sms, cudaStream_t st);

}  // namespace lizg

#endif

// The C ABI (include/lizard_gb300.h): error handling, device setup and the LDPC batch plans. Host C++; the kernels
// are in *.cu. Errors never cross the ABI as exceptions: every entry point catches, records a thread-local message
// and returns a negative code, as the reference's guard does (liblizard/api/api.hpp:21-42).
#include "lizard_gb300.h"
#include "lizard_codes.h"
#include "lizg_internal.h"
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

namespace {

thread_local std::string g_err;

int fail(int code, const char *what) { g_err = what; return code; }
int fail_cuda(cudaError_t e, const char *what) {
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  return LIZG_E_CUDA;
}

// Per-device one-time setup: the code tables into constant memory, the SM count.
struct DeviceState { bool ready = false; int sms = 0; };
std::mutex g_dev_mu;
DeviceState g_dev[64];

int device_setup(int *sms) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail_cuda(e, "cudaGetDevice");
  if (dev < 0 || dev >= 64) return fail(LIZG_E_STATE, "device index out of range");
  std::lock_guard<std::mutex> lk(g_dev_mu);
  DeviceState &d = g_dev[dev];
  if (!d.ready) {
    if ((e = cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return fail_cuda(e, "cudaDeviceGetAttribute");
    if ((e = lizg::ldpc_upload_tables()) != cudaSuccess) return fail_cuda(e, "uploading the LDPC tables");
    d.ready = true;
  }
  *sms = d.sms;
  return 0;
}

int code_n(int code) { const lizg_code_def_t &d = LIZG_CODES[code]; return (d.kb + d.mb) * LIZG_Z; }
int code_k(int code) { return LIZG_CODES[code].kb * LIZG_Z; }

}  // namespace

namespace lizg {
int device_ready(int *sms) { return device_setup(sms); }
int record_error(int code, const char *what) { return fail(code, what); }
}  // namespace lizg

// The host-memory entry point splits the batch into up to kLdpcChunks runs of consecutive codewords, so chunk j + 1
// copies in while chunk j decodes and chunk j's results copy out while chunk j + 1 decodes.
constexpr int kLdpcChunks = 16;

struct lizg_ldpc_plan {
  int count = 0, max_iter = 0, stall_it = 0, launches = 0;
  float ratio = 0;
  int64_t llr_bytes = 0;
  int counts[4] = {0, 0, 0, 0};
  int32_t *d_list = nullptr;       // codeword indices grouped by code, each code's in ascending order
  int64_t *d_off = nullptr;        // per codeword LLR offset
  int *d_counter = nullptr;        // four work counters a chunk
  int list_at[4] = {0, 0, 0, 0};   // each code's first entry in d_list
  std::vector<int> list;           // host copy of d_list
  std::vector<int64_t> off;        // host copy of d_off
  // the host-memory entry: 1 lets the decoder read and write pinned host buffers in place, 0 always stages; the
  // last run's route (1 in place, 0 staged)
  int in_place = 1, last_in_place = 0;
  // the pipelined chunks: chunk j is codewords first[j] .. first[j + 1] - 1, its code c entries d_list[at[j][c]] on
  int chunks = 1;
  int first[kLdpcChunks + 1] = {};
  int at[kLdpcChunks][4] = {}, cnt[kLdpcChunks][4] = {};
  // staging for the host-memory entry point, made on its first use
  int8_t *s_llr = nullptr; uint8_t *s_bits = nullptr; int32_t *s_its = nullptr; uint8_t *s_ok = nullptr;
  int device = -1;
  // The four codes' launches run on their own streams, forked from and joined back to the caller's stream, so one
  // code's persistent CTAs take over the SMs another code's tail frees. The chunks' copies out run on `out`.
  cudaStream_t side[4] = {nullptr, nullptr, nullptr, nullptr}, out = nullptr;
  cudaEvent_t fork = nullptr, done = nullptr, in[kLdpcChunks] = {}, join[kLdpcChunks][4] = {};
};

namespace {

// Splits the batch into `k` chunks of about equal LLR bytes at codeword boundaries, and finds each chunk's entries in
// each code's ascending list.
void plan_chunks(lizg_ldpc_plan *p, int k) {
  k = std::max(1, std::min({k, kLdpcChunks, p->count}));
  p->chunks = k;
  p->first[0] = 0;
  int i = 0;
  for (int j = 1; j < k; j++) {
    const int64_t target = p->llr_bytes * j / k;
    while (i < p->count && p->off[(size_t)i] < target) i++;
    // strictly after the previous boundary, and leaving a codeword for each chunk still to come (a large last
    // codeword can put every offset below the target)
    p->first[j] = std::min(std::max(i, p->first[j - 1] + 1), p->count - (k - j));
  }
  p->first[k] = p->count;
  for (int c = 0; c < 4; c++) {
    const int *b = p->list.data() + p->list_at[c], *e = b + p->counts[c];
    for (int j = 0; j < k; j++) {
      const int *lo = std::lower_bound(b, e, p->first[j]), *hi = std::lower_bound(b, e, p->first[j + 1]);
      p->at[j][c] = (int)(lo - p->list.data());
      p->cnt[j][c] = (int)(hi - lo);
    }
  }
}

// Queues the code launches of one chunk (or of the whole batch): each code's side stream waits for `after`, runs its
// entries, and records its join event.
int launch_codes(lizg_ldpc_plan *p, const int8_t *d_llr, uint8_t *d_bits, int32_t *d_its, uint8_t *d_ok, const int *at,
                 const int *cnt, int *counter, cudaEvent_t after, cudaEvent_t *join, int sms) {
  cudaError_t e;
  for (int c = 0; c < 4; c++) {   // longest code first: 7/8 has the most codewords
    if (!cnt[c]) continue;
    if ((e = cudaStreamWaitEvent(p->side[c], after, 0)) != cudaSuccess) return fail_cuda(e, "cudaStreamWaitEvent");
    lizg::LdpcLaunch a{};
    a.llr = d_llr; a.bits = d_bits; a.its = d_its; a.ok = d_ok; a.list = p->d_list + at[c]; a.off = p->d_off;
    a.count = cnt[c]; a.counter = counter + c; a.max_iter = p->max_iter; a.stall_it = p->stall_it; a.stall_ratio = p->ratio;
    if ((e = lizg::ldpc_launch(c, a, sms, p->side[c])) != cudaSuccess) return fail_cuda(e, "LDPC kernel launch");
    if ((e = cudaEventRecord(join[c], p->side[c])) != cudaSuccess) return fail_cuda(e, "cudaEventRecord");
    p->launches++;
  }
  return 0;
}

}  // namespace

extern "C" {

const char *lizg_last_error(void) { return g_err.c_str(); }
const char *lizg_version(void) { return "lizard_gb300 0.1 (sm_103a)"; }

int lizg_ldpc_n(int rate) {
  const int c = lizg_code_of_rate(rate);
  return c < 0 ? 0 : code_n(c);
}

// liblizard/src/ldpc.c:117-126: systematic; check chk's parity bit is the running XOR of the data bits of checks
// 0..chk, check chk = i mb + r holding data bit col z + (i - shift) mod z of each circulant of block row r.
int lizg_ldpc_encode(int rate, const uint8_t *data, uint8_t *cw) {
  const int c = lizg_code_of_rate(rate);
  if (c < 0 || !data || !cw) return fail(LIZG_E_ARG, "lizg_ldpc_encode: bad rate or NULL buffer");
  const lizg_code_def_t &d = LIZG_CODES[c];
  const int z = LIZG_Z, k = code_k(c), m = d.mb * z;
  std::memcpy(cw, data, (size_t)k);
  uint8_t acc = 0;
  for (int chk = 0; chk < m; chk++) {
    const int i = chk / d.mb, r = chk % d.mb;
    for (int e = d.rowptr[r]; e < d.rowptr[r + 1]; e++) {
      const int col = d.circ[e] >> 8, sh = d.circ[e] & 255;
      acc ^= data[col * z + ((i - sh) % z + z) % z] & 1;
    }
    cw[k + chk] = acc;
  }
  return 0;
}

int lizg_ldpc_encode_many(int rate, const uint8_t *data, int count, uint8_t *cw) {
  const int c = lizg_code_of_rate(rate);
  if (c < 0 || !data || !cw || count < 0) return fail(LIZG_E_ARG, "lizg_ldpc_encode_many: bad rate, count or NULL buffer");
  for (int i = 0; i < count; i++) lizg_ldpc_encode(rate, data + (size_t)i * code_k(c), cw + (size_t)i * code_n(c));
  return 0;
}

uint32_t lizg_crc32c(const uint8_t *p, size_t n) {
  static uint32_t tab[256];
  static std::once_flag once;
  std::call_once(once, [] {
    for (uint32_t t = 0; t < 256; t++) {
      uint32_t c = t;
      for (int k = 0; k < 8; k++) c = (c >> 1) ^ (0x82F63B78u & (0u - (c & 1u)));
      tab[t] = c;
    }
  });
  uint32_t c = 0xffffffffu;
  for (size_t i = 0; i < n; i++) c = tab[(c ^ p[i]) & 255u] ^ (c >> 8);
  return ~c;
}

lizg_ldpc_plan *lizg_ldpc_plan_new(const int32_t *rate, int count, int max_iter, int stall_it, float stall_ratio) {
  if (!rate || count <= 0 || max_iter < 1 || max_iter > 255 || stall_it < 0 || stall_it == 1 || stall_it > max_iter) {
    fail(LIZG_E_ARG, "lizg_ldpc_plan_new: bad count, max_iter or stall_it");
    return nullptr;
  }
  int sms = 0;
  if (device_setup(&sms)) return nullptr;
  lizg_ldpc_plan *p = new (std::nothrow) lizg_ldpc_plan;
  if (!p) { fail(LIZG_E_NOMEM, "lizg_ldpc_plan_new: out of host memory"); return nullptr; }
  p->count = count; p->max_iter = max_iter; p->stall_it = stall_it; p->ratio = stall_ratio;
  cudaGetDevice(&p->device);
  p->off.assign((size_t)count, 0);
  p->list.assign((size_t)count, 0);
  int64_t at = 0;
  for (int i = 0; i < count; i++) {
    const int c = lizg_code_of_rate(rate[i]);
    if (c < 0) { fail(LIZG_E_ARG, "lizg_ldpc_plan_new: a rate with no code"); delete p; return nullptr; }
    p->off[(size_t)i] = at; at += code_n(c); p->counts[c]++;
  }
  p->llr_bytes = at;
  int fill[4];
  for (int c = 0, s = 0; c < 4; s += p->counts[c], c++) { p->list_at[c] = s; fill[c] = s; }
  for (int i = 0; i < count; i++) p->list[(size_t)fill[lizg_code_of_rate(rate[i])]++] = i;
  // two chunks from 64 MB of LLRs up: half the copy in overlaps decode; more chunks add more launch tails than the
  // overlap saves (65,536 codewords on a GB300: 19.6 ms at 1 chunk, 19.2 at 2, 20.6 at 8, 22.1 at 16)
  plan_chunks(p, p->llr_bytes >= (64 << 20) ? 2 : 1);
  cudaError_t e;
  if ((e = cudaMalloc(&p->d_list, sizeof(int32_t) * (size_t)count)) != cudaSuccess ||
      (e = cudaMalloc(&p->d_off, sizeof(int64_t) * (size_t)count)) != cudaSuccess ||
      (e = cudaMalloc(&p->d_counter, sizeof(int) * 4 * kLdpcChunks)) != cudaSuccess ||
      (e = cudaMemcpy(p->d_list, p->list.data(), sizeof(int32_t) * (size_t)count, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(p->d_off, p->off.data(), sizeof(int64_t) * (size_t)count, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&p->done, cudaEventDisableTiming)) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&p->out, cudaStreamNonBlocking)) != cudaSuccess) {
    fail_cuda(e, "lizg_ldpc_plan_new");
    lizg_ldpc_plan_free(p);
    return nullptr;
  }
  for (int c = 0; c < 4; c++) {
    if ((e = cudaStreamCreateWithFlags(&p->side[c], cudaStreamNonBlocking)) != cudaSuccess) {
      fail_cuda(e, "lizg_ldpc_plan_new: streams");
      lizg_ldpc_plan_free(p);
      return nullptr;
    }
  }
  for (int j = 0; j < kLdpcChunks; j++) {
    bool bad = (e = cudaEventCreateWithFlags(&p->in[j], cudaEventDisableTiming)) != cudaSuccess;
    for (int c = 0; c < 4 && !bad; c++) bad = (e = cudaEventCreateWithFlags(&p->join[j][c], cudaEventDisableTiming)) != cudaSuccess;
    if (bad) {
      fail_cuda(e, "lizg_ldpc_plan_new: events");
      lizg_ldpc_plan_free(p);
      return nullptr;
    }
  }
  return p;
}

void lizg_ldpc_plan_free(lizg_ldpc_plan *p) {
  if (!p) return;
  cudaFree(p->d_list); cudaFree(p->d_off); cudaFree(p->d_counter);
  cudaFree(p->s_llr); cudaFree(p->s_bits); cudaFree(p->s_its); cudaFree(p->s_ok);
  for (int c = 0; c < 4; c++) if (p->side[c]) cudaStreamDestroy(p->side[c]);
  if (p->out) cudaStreamDestroy(p->out);
  for (int j = 0; j < kLdpcChunks; j++) {
    if (p->in[j]) cudaEventDestroy(p->in[j]);
    for (int c = 0; c < 4; c++) if (p->join[j][c]) cudaEventDestroy(p->join[j][c]);
  }
  if (p->fork) cudaEventDestroy(p->fork);
  if (p->done) cudaEventDestroy(p->done);
  delete p;
}

int lizg_ldpc_plan_set_transfer(lizg_ldpc_plan *p, int in_place) {
  if (!p || (in_place != 0 && in_place != 1)) return fail(LIZG_E_ARG, "lizg_ldpc_plan_set_transfer: in_place must be 0 or 1");
  p->in_place = in_place;
  return 0;
}

int lizg_ldpc_plan_transfer(const lizg_ldpc_plan *p) { return p ? p->last_in_place : LIZG_E_ARG; }

int lizg_ldpc_plan_set_chunks(lizg_ldpc_plan *p, int chunks) {
  if (!p || chunks < 1 || chunks > kLdpcChunks) return fail(LIZG_E_ARG, "lizg_ldpc_plan_set_chunks: chunks must be 1..16");
  plan_chunks(p, chunks);
  return p->chunks;
}

int64_t lizg_ldpc_plan_llr_bytes(const lizg_ldpc_plan *p) { return p ? p->llr_bytes : LIZG_E_ARG; }
int lizg_ldpc_plan_launches(const lizg_ldpc_plan *p) { return p ? p->launches : LIZG_E_ARG; }

int lizg_ldpc_plan_run_dev(lizg_ldpc_plan *p, const int8_t *d_llr, uint8_t *d_bits, int32_t *d_its, uint8_t *d_ok, void *stream) {
  try {
    if (!p || !d_llr || !d_bits || !d_its || !d_ok) return fail(LIZG_E_ARG, "lizg_ldpc_plan_run_dev: NULL argument");
    if ((reinterpret_cast<uintptr_t>(d_llr) | reinterpret_cast<uintptr_t>(d_bits)) & 15)
      return fail(LIZG_E_ARG, "lizg_ldpc_plan_run_dev: llr and bits must be 16-byte aligned");
    int sms = 0;
    if (int rc = device_setup(&sms)) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemsetAsync(p->d_counter, 0, sizeof(int) * 4, st);
    if (e != cudaSuccess) return fail_cuda(e, "cudaMemsetAsync");
    if ((e = cudaEventRecord(p->fork, st)) != cudaSuccess) return fail_cuda(e, "cudaEventRecord");
    p->launches = 0;
    if (int rc = launch_codes(p, d_llr, d_bits, d_its, d_ok, p->list_at, p->counts, p->d_counter, p->fork, p->join[0], sms)) return rc;
    for (int c = 0; c < 4; c++)
      if (p->counts[c] && (e = cudaStreamWaitEvent(st, p->join[0][c], 0)) != cudaSuccess) return fail_cuda(e, "cudaStreamWaitEvent");
    return 0;
  } catch (...) {
    return fail(LIZG_E_STATE, "lizg_ldpc_plan_run_dev: unexpected exception");
  }
}

namespace {

// The device address of `bytes` bytes of page-locked host memory at h, or null: both ends must lie in memory the
// runtime reports as host memory mapped for this device, at one device offset apart.
void *mapped_host(const void *h, int64_t bytes) {
  cudaPointerAttributes a0{}, a1{};
  const char *c = static_cast<const char *>(h);
  if (cudaPointerGetAttributes(&a0, c) != cudaSuccess || cudaPointerGetAttributes(&a1, c + bytes - 1) != cudaSuccess) {
    cudaGetLastError();   // a pointer the runtime does not know is not an error here
    return nullptr;
  }
  if (a0.type != cudaMemoryTypeHost || a1.type != cudaMemoryTypeHost || !a0.devicePointer || !a1.devicePointer) return nullptr;
  if (static_cast<char *>(a1.devicePointer) - static_cast<char *>(a0.devicePointer) != bytes - 1) return nullptr;
  return a0.devicePointer;
}

}  // namespace

// Host memory in and out. When all four buffers are page-locked (cudaHostAlloc, cudaHostRegister) and llr and bits
// are 16-byte aligned, the decoder reads each codeword's LLRs once from host memory and writes its bits, its and ok
// there (NVLink-C2C on a Grace host): the transfer overlaps the decode with no staging copy. Otherwise the batch is
// staged through device memory, pipelined over the plan's chunks: the caller's stream copies chunk j in and forks chunk j's
// code launches; the copy-out stream waits for them and copies chunk j's bits, its and ok back. Chunk j's copy out
// is queued after chunk j + 1's launches, so a copy to pageable memory (which returns only when done) still lets
// the next chunk's copy in and decode run meanwhile.
int lizg_ldpc_plan_run(lizg_ldpc_plan *p, const int8_t *llr, uint8_t *bits, int32_t *its, uint8_t *ok, void *stream) {
  try {
    if (!p || !llr || !bits || !its || !ok) return fail(LIZG_E_ARG, "lizg_ldpc_plan_run: NULL argument");
    int sms = 0;
    if (int rc = device_setup(&sms)) return rc;
    cudaError_t e;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    p->last_in_place = 0;
    if (p->in_place) {
      void *dl = mapped_host(llr, p->llr_bytes), *db = mapped_host(bits, p->llr_bytes / 8);
      void *di = mapped_host(its, sizeof(int32_t) * (int64_t)p->count), *dk = mapped_host(ok, p->count);
      if (dl && db && di && dk && !((reinterpret_cast<uintptr_t>(dl) | reinterpret_cast<uintptr_t>(db)) & 15)) {
        if (int rc = lizg_ldpc_plan_run_dev(p, static_cast<const int8_t *>(dl), static_cast<uint8_t *>(db), static_cast<int32_t *>(di),
                                            static_cast<uint8_t *>(dk), stream)) return rc;
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail_cuda(e, "lizg_ldpc_plan_run: decode");
        p->last_in_place = 1;
        return 0;
      }
    }
    if (!p->s_llr) {
      if ((e = cudaMalloc(&p->s_llr, (size_t)p->llr_bytes)) != cudaSuccess || (e = cudaMalloc(&p->s_bits, (size_t)p->llr_bytes / 8)) != cudaSuccess ||
          (e = cudaMalloc(&p->s_its, sizeof(int32_t) * (size_t)p->count)) != cudaSuccess || (e = cudaMalloc(&p->s_ok, (size_t)p->count)) != cudaSuccess)
        return fail_cuda(e, "lizg_ldpc_plan_run: staging buffers");
    }
    if ((e = cudaMemsetAsync(p->d_counter, 0, sizeof(int) * 4 * (size_t)p->chunks, st)) != cudaSuccess) return fail_cuda(e, "cudaMemsetAsync");
    // the copy-out stream starts after whatever the caller queued before this call
    if ((e = cudaEventRecord(p->fork, st)) != cudaSuccess || (e = cudaStreamWaitEvent(p->out, p->fork, 0)) != cudaSuccess)
      return fail_cuda(e, "lizg_ldpc_plan_run: fork");
    p->launches = 0;
    auto copy_out = [&](int j) -> int {
      for (int c = 0; c < 4; c++)
        if (p->cnt[j][c] && (e = cudaStreamWaitEvent(p->out, p->join[j][c], 0)) != cudaSuccess) return fail_cuda(e, "cudaStreamWaitEvent");
      const int i0 = p->first[j], i1 = p->first[j + 1];
      const int64_t b0 = p->off[(size_t)i0] / 8, b1 = (i1 < p->count ? p->off[(size_t)i1] : p->llr_bytes) / 8;
      if ((e = cudaMemcpyAsync(bits + b0, p->s_bits + b0, (size_t)(b1 - b0), cudaMemcpyDeviceToHost, p->out)) != cudaSuccess ||
          (e = cudaMemcpyAsync(its + i0, p->s_its + i0, sizeof(int32_t) * (size_t)(i1 - i0), cudaMemcpyDeviceToHost, p->out)) != cudaSuccess ||
          (e = cudaMemcpyAsync(ok + i0, p->s_ok + i0, (size_t)(i1 - i0), cudaMemcpyDeviceToHost, p->out)) != cudaSuccess)
        return fail_cuda(e, "copy out");
      return 0;
    };
    for (int j = 0; j < p->chunks; j++) {
      const int i0 = p->first[j], i1 = p->first[j + 1];
      const int64_t b0 = p->off[(size_t)i0], b1 = i1 < p->count ? p->off[(size_t)i1] : p->llr_bytes;
      if ((e = cudaMemcpyAsync(p->s_llr + b0, llr + b0, (size_t)(b1 - b0), cudaMemcpyHostToDevice, st)) != cudaSuccess) return fail_cuda(e, "copy in");
      if ((e = cudaEventRecord(p->in[j], st)) != cudaSuccess) return fail_cuda(e, "cudaEventRecord");
      if (int rc = launch_codes(p, p->s_llr, p->s_bits, p->s_its, p->s_ok, p->at[j], p->cnt[j], p->d_counter + 4 * j, p->in[j], p->join[j], sms)) return rc;
      if (j)
        if (int rc = copy_out(j - 1)) return rc;
    }
    if (int rc = copy_out(p->chunks - 1)) return rc;
    if ((e = cudaEventRecord(p->done, p->out)) != cudaSuccess || (e = cudaStreamWaitEvent(st, p->done, 0)) != cudaSuccess)
      return fail_cuda(e, "lizg_ldpc_plan_run: join");
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail_cuda(e, "lizg_ldpc_plan_run: decode");
    return 0;
  } catch (...) {
    return fail(LIZG_E_STATE, "lizg_ldpc_plan_run: unexpected exception");
  }
}

// One codeword through a batch plan of one, the reference's per-block call and output form (one bit a byte).
int lizg_ldpc_decode_stall(int rate, const int8_t *llr, uint8_t *out, int max_iter, int stall_it, float stall_ratio) {
  const int c = lizg_code_of_rate(rate);
  if (c < 0 || !llr || !out) return fail(LIZG_E_ARG, "lizg_ldpc_decode_stall: bad rate or NULL buffer") - 100;
  const int32_t r = rate;
  lizg_ldpc_plan *p = lizg_ldpc_plan_new(&r, 1, max_iter, stall_it, stall_ratio);
  if (!p) return LIZG_E_ARG - 100;
  const int n = code_n(c);
  std::vector<uint8_t> packed((size_t)n / 8);
  int32_t its = 0;
  uint8_t ok = 0;
  const int rc = lizg_ldpc_plan_run(p, llr, packed.data(), &its, &ok, nullptr);
  lizg_ldpc_plan_free(p);
  if (rc) return rc - 100;
  for (int v = 0; v < n; v++) out[v] = (packed[(size_t)v / 8] >> (7 - v % 8)) & 1;
  return its;
}

}  // extern "C"

// The C ABI (include/lizard_gb300.h): error handling, device setup and the LDPC batch plans. Host C++; the kernels
// are in *.cu. Errors never cross the ABI as exceptions: every entry point catches, records a thread-local message
// and returns a negative code, as the reference's guard does (liblizard/api/api.hpp:21-42).
#include "lizard_gb300.h"
#include "lizard_codes.h"
#include "lizg_internal.h"
#include <cuda_runtime.h>
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

struct lizg_ldpc_plan {
  int count = 0, max_iter = 0, stall_it = 0, launches = 0;
  float ratio = 0;
  int64_t llr_bytes = 0;
  int counts[4] = {0, 0, 0, 0};
  int32_t *d_list = nullptr;       // codeword indices grouped by code
  int64_t *d_off = nullptr;        // per codeword LLR offset
  int *d_counter = nullptr;        // four work counters
  int list_at[4] = {0, 0, 0, 0};   // each code's first entry in d_list
  // staging for the host-memory entry point, made on its first use
  int8_t *s_llr = nullptr; uint8_t *s_bits = nullptr; int32_t *s_its = nullptr; uint8_t *s_ok = nullptr;
  int device = -1;
  // The four codes' launches run on their own streams, forked from and joined back to the caller's stream, so one
  // code's persistent CTAs take over the SMs another code's tail frees.
  cudaStream_t side[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t fork = nullptr, join[4] = {nullptr, nullptr, nullptr, nullptr};
};

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
  std::vector<int64_t> off((size_t)count);
  std::vector<int32_t> list((size_t)count);
  int64_t at = 0;
  for (int i = 0; i < count; i++) {
    const int c = lizg_code_of_rate(rate[i]);
    if (c < 0) { fail(LIZG_E_ARG, "lizg_ldpc_plan_new: a rate with no code"); delete p; return nullptr; }
    off[(size_t)i] = at; at += code_n(c); p->counts[c]++;
  }
  p->llr_bytes = at;
  int fill[4];
  for (int c = 0, s = 0; c < 4; s += p->counts[c], c++) { p->list_at[c] = s; fill[c] = s; }
  for (int i = 0; i < count; i++) list[(size_t)fill[lizg_code_of_rate(rate[i])]++] = i;
  cudaError_t e;
  if ((e = cudaMalloc(&p->d_list, sizeof(int32_t) * (size_t)count)) != cudaSuccess ||
      (e = cudaMalloc(&p->d_off, sizeof(int64_t) * (size_t)count)) != cudaSuccess ||
      (e = cudaMalloc(&p->d_counter, sizeof(int) * 4)) != cudaSuccess ||
      (e = cudaMemcpy(p->d_list, list.data(), sizeof(int32_t) * (size_t)count, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(p->d_off, off.data(), sizeof(int64_t) * (size_t)count, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming)) != cudaSuccess) {
    fail_cuda(e, "lizg_ldpc_plan_new");
    lizg_ldpc_plan_free(p);
    return nullptr;
  }
  for (int c = 0; c < 4; c++) {
    if ((e = cudaStreamCreateWithFlags(&p->side[c], cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&p->join[c], cudaEventDisableTiming)) != cudaSuccess) {
      fail_cuda(e, "lizg_ldpc_plan_new: streams");
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
  for (int c = 0; c < 4; c++) { if (p->side[c]) cudaStreamDestroy(p->side[c]); if (p->join[c]) cudaEventDestroy(p->join[c]); }
  if (p->fork) cudaEventDestroy(p->fork);
  delete p;
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
    for (int c = 0; c < 4; c++) {   // longest code first: 7/8 has the most codewords
      if (!p->counts[c]) continue;
      if ((e = cudaStreamWaitEvent(p->side[c], p->fork, 0)) != cudaSuccess) return fail_cuda(e, "cudaStreamWaitEvent");
      lizg::LdpcLaunch a{};
      a.llr = d_llr; a.bits = d_bits; a.its = d_its; a.ok = d_ok; a.list = p->d_list + p->list_at[c]; a.off = p->d_off;
      a.count = p->counts[c]; a.counter = p->d_counter + c; a.max_iter = p->max_iter; a.stall_it = p->stall_it; a.stall_ratio = p->ratio;
      if ((e = lizg::ldpc_launch(c, a, sms, p->side[c])) != cudaSuccess) return fail_cuda(e, "LDPC kernel launch");
      if ((e = cudaEventRecord(p->join[c], p->side[c])) != cudaSuccess) return fail_cuda(e, "cudaEventRecord");
      if ((e = cudaStreamWaitEvent(st, p->join[c], 0)) != cudaSuccess) return fail_cuda(e, "cudaStreamWaitEvent");
      p->launches++;
    }
    return 0;
  } catch (...) {
    return fail(LIZG_E_STATE, "lizg_ldpc_plan_run_dev: unexpected exception");
  }
}

int lizg_ldpc_plan_run(lizg_ldpc_plan *p, const int8_t *llr, uint8_t *bits, int32_t *its, uint8_t *ok, void *stream) {
  try {
    if (!p || !llr || !bits || !its || !ok) return fail(LIZG_E_ARG, "lizg_ldpc_plan_run: NULL argument");
    cudaError_t e;
    if (!p->s_llr) {
      if ((e = cudaMalloc(&p->s_llr, (size_t)p->llr_bytes)) != cudaSuccess || (e = cudaMalloc(&p->s_bits, (size_t)p->llr_bytes / 8)) != cudaSuccess ||
          (e = cudaMalloc(&p->s_its, sizeof(int32_t) * (size_t)p->count)) != cudaSuccess || (e = cudaMalloc(&p->s_ok, (size_t)p->count)) != cudaSuccess)
        return fail_cuda(e, "lizg_ldpc_plan_run: staging buffers");
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if ((e = cudaMemcpyAsync(p->s_llr, llr, (size_t)p->llr_bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess) return fail_cuda(e, "copy in");
    if (int rc = lizg_ldpc_plan_run_dev(p, p->s_llr, p->s_bits, p->s_its, p->s_ok, stream)) return rc;
    if ((e = cudaMemcpyAsync(bits, p->s_bits, (size_t)p->llr_bytes / 8, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(its, p->s_its, sizeof(int32_t) * (size_t)p->count, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(ok, p->s_ok, (size_t)p->count, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
      return fail_cuda(e, "copy out");
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

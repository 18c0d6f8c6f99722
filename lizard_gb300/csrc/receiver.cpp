// The batching front (include/lizard_gb300.h lizg_receiver_*): the shape of the reference's receiver engine
// (liz_receiver_new / _push / _batch_cap / _stats / _series / _wants_luma / _free, liblizard/include/lizard.h:252-294;
// its contract liblizard/core/rx/receiver.h:55-126) for frames whose registration is already held. A push copies the
// frame into a page-locked slot (or drops it when every slot is taken), hands the caller's buffer back through
// release(tag) before it returns, and never waits on the device. One thread of the front's own takes the waiting
// frames in push order, up to the batch cap of one frame size at a time, copies them to the device, decodes them in
// one lizg_rx_finish_luma_dev call on its own stream, and hands each frame's verified blocks to the caller's frame
// callback. Host C++.
#include "lizard_gb300.h"
#include "lizard_codes.h"
#include "lizg_internal.h"
#include <cuda_runtime.h>
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_set>
#include <vector>

namespace {

constexpr int kMaxBatch = 32;
constexpr int kSeriesKeep = 4096;   // frames the series keeps (8 doubles each)

struct Slot {
  uint8_t *luma = nullptr;   // max_w x max_h, rows w apart
  float *reg = nullptr;      // 9 + 2 nx ny
  int w = 0, h = 0;
  int64_t ts = 0;
  uint64_t tag = 0;
};

double now_s() { return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count(); }

}  // namespace

struct lizg_receiver {
  lizg_receiver_config cfg{};
  void (*release)(void *, uint64_t) = nullptr;
  lizg_rx *rx = nullptr;
  int device = 0, blocks = 0, regn = 0, cap = kMaxBatch;
  // page-locked slots and the device batch
  uint8_t *h_luma = nullptr, *h_blocks = nullptr, *h_ok = nullptr;
  float *h_reg = nullptr, *h_pilot = nullptr;
  int32_t *h_its = nullptr;
  uint8_t *d_luma = nullptr, *d_blocks = nullptr, *d_ok = nullptr;
  float *d_reg = nullptr, *d_pilot = nullptr;
  int32_t *d_its = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  std::vector<Slot> slots;
  std::vector<int> free_slots;
  std::deque<int> pending;
  std::mutex mu;
  std::condition_variable work_cv, idle_cv;
  std::thread worker;
  bool stop = false;
  int inflight = 0;
  // the figures stats and series report
  uint64_t frames_in = 0, dropped = 0, decoded = 0, batches = 0, verified = 0, fresh = 0;
  double gpu_ms = 0, t_first = 0, t_last = 0;
  std::unordered_set<uint32_t> ids;
  std::deque<double> series;
  std::string stats_text;
  std::vector<uint8_t> packed;   // a frame's verified blocks for the frame callback
};

namespace {

void logf(lizg_receiver *r, const std::string &line) {
  if (r->cfg.log) r->cfg.log(r->cfg.user, line.c_str());
}

// The pilots' readings of a frame's blocks: mean and standard error over the even blocks and the odd, NaN where a
// parity read none (liblizard/src/lizard_phy.c:451-472 lizard_pilot).
void pilot_summary(const float *pilot, int blocks, double r[2], double sd[2]) {
  for (int g = 0; g < 2; g++) {
    double s = 0, s2 = 0;
    int k = 0;
    for (int b = g; b < blocks; b += 2)
      if (pilot[b] == pilot[b]) { s += pilot[b]; s2 += (double)pilot[b] * pilot[b]; k++; }
    if (!k) { r[g] = sd[g] = NAN; continue; }
    const double mean = s / k, var = k > 1 ? (s2 - s * mean) / (k - 1) : 0;
    r[g] = (float)mean;
    sd[g] = (float)std::sqrt((var > 0 ? var : 0) / k);
  }
}

void decode_batch(lizg_receiver *r, const std::vector<int> &batch) {
  const int K = (int)batch.size(), w = r->slots[batch[0]].w, h = r->slots[batch[0]].h;
  const size_t fb = (size_t)w * h;
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < K && e == cudaSuccess; k++) {
    const Slot &s = r->slots[batch[k]];
    e = cudaMemcpyAsync(r->d_luma + k * fb, s.luma, fb, cudaMemcpyHostToDevice, r->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(r->d_reg + (size_t)k * r->regn, s.reg, sizeof(float) * r->regn, cudaMemcpyHostToDevice, r->st);
  }
  const lizg_rx_out out{r->d_blocks, r->d_ok, r->d_its, nullptr, r->d_pilot, nullptr, nullptr, nullptr, nullptr};
  int rc = 0;
  if (e == cudaSuccess) {
    cudaEventRecord(r->e0, r->st);
    rc = lizg_rx_finish_luma_dev(r->rx, r->d_luma, w, h, w, (int64_t)fb, r->d_reg, K, &out, nullptr, nullptr, r->st);
    cudaEventRecord(r->e1, r->st);
  }
  const size_t nb = (size_t)K * r->blocks;
  if (e == cudaSuccess && !rc) {
    cudaMemcpyAsync(r->h_blocks, r->d_blocks, nb * LIZG_BLOCK_BYTES, cudaMemcpyDeviceToHost, r->st);
    cudaMemcpyAsync(r->h_ok, r->d_ok, nb, cudaMemcpyDeviceToHost, r->st);
    cudaMemcpyAsync(r->h_its, r->d_its, nb * sizeof(int32_t), cudaMemcpyDeviceToHost, r->st);
    cudaMemcpyAsync(r->h_pilot, r->d_pilot, nb * sizeof(float), cudaMemcpyDeviceToHost, r->st);
    e = cudaStreamSynchronize(r->st);
  }
  const bool good = e == cudaSuccess && !rc;
  if (!good) {
    logf(r, std::string("lizg_receiver: a batch failed: ") + (rc ? lizg_last_error() : cudaGetErrorString(e)));
    std::memset(r->h_ok, 0, nb);
    for (size_t i = 0; i < nb; i++) { r->h_its[i] = 0; r->h_pilot[i] = NAN; }
  }
  float ms = 0;
  if (good) cudaEventElapsedTime(&ms, r->e0, r->e1);
  for (int k = 0; k < K; k++) {
    const Slot &s = r->slots[batch[k]];
    const uint8_t *ok = r->h_ok + (size_t)k * r->blocks, *bl = r->h_blocks + (size_t)k * r->blocks * LIZG_BLOCK_BYTES;
    int count = 0, fresh = 0;
    for (int b = 0; b < r->blocks; b++) {
      if (!ok[b]) continue;
      std::memcpy(r->packed.data() + (size_t)count * LIZG_BLOCK_BYTES, bl + (size_t)b * LIZG_BLOCK_BYTES, LIZG_BLOCK_BYTES);
      count++;
      const uint8_t *id = bl + (size_t)b * LIZG_BLOCK_BYTES;
      fresh += r->ids.insert((uint32_t)id[0] | (uint32_t)id[1] << 8 | (uint32_t)id[2] << 16 | (uint32_t)id[3] << 24).second;
    }
    double pr[2], psd[2];
    pilot_summary(r->h_pilot + (size_t)k * r->blocks, r->blocks, pr, psd);
    {
      std::lock_guard<std::mutex> lk(r->mu);
      r->verified += count;
      r->fresh += fresh;
      const double row[8] = {(double)s.ts / 1e6, (double)count, (double)fresh, good ? 1.0 : 0.0, pr[0], psd[0], pr[1], psd[1]};
      r->series.insert(r->series.end(), row, row + 8);
      while (r->series.size() > 8 * (size_t)kSeriesKeep) r->series.erase(r->series.begin(), r->series.begin() + 8);
    }
    if (r->cfg.frame)
      r->cfg.frame(r->cfg.user, s.tag, s.ts, r->packed.data(), count, ok, r->h_its + (size_t)k * r->blocks, r->blocks);
  }
  std::lock_guard<std::mutex> lk(r->mu);
  r->gpu_ms += ms;
  r->batches++;
  r->decoded += K;
  r->t_last = now_s();
}

void run(lizg_receiver *r) {
  cudaSetDevice(r->device);
  std::vector<int> batch;
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(r->mu);
      r->work_cv.wait(lk, [&] { return r->stop || !r->pending.empty(); });
      if (r->pending.empty()) return;   // stopping, every frame pushed decoded
      batch.clear();
      const Slot &first = r->slots[r->pending.front()];
      while (!r->pending.empty() && (int)batch.size() < r->cap) {
        const Slot &s = r->slots[r->pending.front()];
        if (s.w != first.w || s.h != first.h) break;   // a launch takes frames of one size
        batch.push_back(r->pending.front());
        r->pending.pop_front();
      }
      r->inflight = (int)batch.size();
    }
    decode_batch(r, batch);
    {
      std::lock_guard<std::mutex> lk(r->mu);
      for (int i : batch) r->free_slots.push_back(i);
      r->inflight = 0;
    }
    r->idle_cv.notify_all();
  }
}

void destroy(lizg_receiver *r) {
  if (r->worker.joinable()) {
    { std::lock_guard<std::mutex> lk(r->mu); r->stop = true; }
    r->work_cv.notify_all();
    r->worker.join();
  }
  cudaFreeHost(r->h_luma); cudaFreeHost(r->h_reg); cudaFreeHost(r->h_blocks); cudaFreeHost(r->h_ok); cudaFreeHost(r->h_its); cudaFreeHost(r->h_pilot);
  cudaFree(r->d_luma); cudaFree(r->d_reg); cudaFree(r->d_blocks); cudaFree(r->d_ok); cudaFree(r->d_its); cudaFree(r->d_pilot);
  if (r->e0) cudaEventDestroy(r->e0);
  if (r->e1) cudaEventDestroy(r->e1);
  if (r->st) cudaStreamDestroy(r->st);
  lizg_rx_free(r->rx);
  delete r;
}

}  // namespace

extern "C" {

lizg_receiver *lizg_receiver_new(const lizg_receiver_config *c, void (*release)(void *user, uint64_t tag)) {
  if (!c) { lizg::record_error(LIZG_E_ARG, "lizg_receiver_new: NULL config"); return nullptr; }
  if (c->max_w < 2 || c->max_h < 2 || (int64_t)c->max_w * c->max_h > (1ll << 28)) {
    lizg::record_error(LIZG_E_ARG, "lizg_receiver_new: max_w x max_h out of range");
    return nullptr;
  }
  if (c->batch_cap < 0 || c->batch_cap > kMaxBatch || c->slots < 0 || c->slots > 4 * kMaxBatch) {
    lizg::record_error(LIZG_E_ARG, "lizg_receiver_new: batch_cap 0..32, slots 0..128");
    return nullptr;
  }
  if (c->read != LIZG_READ_DECODE && c->read != LIZG_READ_EXACT) { lizg::record_error(LIZG_E_ARG, "lizg_receiver_new: read is a LIZG_READ_* value"); return nullptr; }
  int sms = 0;
  if (lizg::device_ready(&sms)) return nullptr;
  lizg_receiver *r = new (std::nothrow) lizg_receiver;
  if (!r) { lizg::record_error(LIZG_E_NOMEM, "lizg_receiver_new: out of host memory"); return nullptr; }
  r->cfg = *c;
  r->release = release;
  r->cap = c->batch_cap ? c->batch_cap : kMaxBatch;
  cudaGetDevice(&r->device);
  r->rx = lizg_rx_new(c->n, c->subch, c->span, kMaxBatch);
  if (!r->rx) { destroy(r); return nullptr; }   // the message is lizg_rx_new's
  lizg_rx_set_read(r->rx, c->read);
  int32_t info[24];
  lizg_rx_info(r->rx, info);
  r->blocks = info[3];
  r->regn = 9 + 2 * info[22] * info[23];
  const int S = c->slots ? c->slots : 2 * kMaxBatch;
  const size_t fb = (size_t)c->max_w * c->max_h, nb = (size_t)kMaxBatch * r->blocks;
  cudaError_t e = cudaSuccess;
  auto ok = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
  ok(cudaHostAlloc(reinterpret_cast<void **>(&r->h_luma), fb * S, cudaHostAllocDefault));
  ok(cudaHostAlloc(reinterpret_cast<void **>(&r->h_reg), sizeof(float) * r->regn * S, cudaHostAllocDefault));
  ok(cudaHostAlloc(reinterpret_cast<void **>(&r->h_blocks), nb * LIZG_BLOCK_BYTES, cudaHostAllocDefault));
  ok(cudaHostAlloc(reinterpret_cast<void **>(&r->h_ok), nb, cudaHostAllocDefault));
  ok(cudaHostAlloc(reinterpret_cast<void **>(&r->h_its), nb * sizeof(int32_t), cudaHostAllocDefault));
  ok(cudaHostAlloc(reinterpret_cast<void **>(&r->h_pilot), nb * sizeof(float), cudaHostAllocDefault));
  ok(cudaMalloc(&r->d_luma, fb * kMaxBatch));
  ok(cudaMalloc(&r->d_reg, sizeof(float) * r->regn * kMaxBatch));
  ok(cudaMalloc(&r->d_blocks, nb * LIZG_BLOCK_BYTES));
  ok(cudaMalloc(&r->d_ok, nb));
  ok(cudaMalloc(&r->d_its, nb * sizeof(int32_t)));
  ok(cudaMalloc(&r->d_pilot, nb * sizeof(float)));
  ok(cudaStreamCreateWithFlags(&r->st, cudaStreamNonBlocking));
  ok(cudaEventCreate(&r->e0));
  ok(cudaEventCreate(&r->e1));
  if (e != cudaSuccess) {
    lizg::record_error(LIZG_E_NOMEM, (std::string("lizg_receiver_new: ") + cudaGetErrorString(e)).c_str());
    destroy(r);
    return nullptr;
  }
  r->slots.resize(S);
  for (int i = 0; i < S; i++) {
    r->slots[i].luma = r->h_luma + fb * i;
    r->slots[i].reg = r->h_reg + (size_t)r->regn * i;
    r->free_slots.push_back(S - 1 - i);
  }
  r->packed.resize((size_t)r->blocks * LIZG_BLOCK_BYTES);
  try {
    r->worker = std::thread(run, r);
  } catch (...) {
    lizg::record_error(LIZG_E_STATE, "lizg_receiver_new: no thread");
    destroy(r);
    return nullptr;
  }
  return r;
}

void lizg_receiver_free(lizg_receiver *r) {
  if (r) destroy(r);
}

int lizg_receiver_push(lizg_receiver *r, const uint8_t *luma, int w, int h, int stride, int64_t timestamp_ns, uint64_t tag, const float *reg) {
  if (!r || !luma || !reg || w < 2 || h < 2 || stride < w) return lizg::record_error(LIZG_E_ARG, "lizg_receiver_push: a receiver, a luma plane and its registration");
  if (w > r->cfg.max_w || h > r->cfg.max_h || (int64_t)w * h > (int64_t)r->cfg.max_w * r->cfg.max_h)
    return lizg::record_error(LIZG_E_ARG, "lizg_receiver_push: the frame is larger than the config's max_w x max_h");
  int slot = -1;
  {
    std::lock_guard<std::mutex> lk(r->mu);
    r->frames_in++;
    if (!r->t_first) r->t_first = now_s();
    if (r->free_slots.empty()) r->dropped++;
    else { slot = r->free_slots.back(); r->free_slots.pop_back(); }
  }
  if (slot >= 0) {
    Slot &s = r->slots[slot];
    for (int y = 0; y < h; y++) std::memcpy(s.luma + (size_t)y * w, luma + (size_t)y * stride, (size_t)w);
    std::memcpy(s.reg, reg, sizeof(float) * r->regn);
    s.w = w; s.h = h; s.ts = timestamp_ns; s.tag = tag;
  }
  if (r->release) r->release(r->cfg.user, tag);   // copied or dropped: the caller's buffer is its own again
  if (slot >= 0) {
    { std::lock_guard<std::mutex> lk(r->mu); r->pending.push_back(slot); }
    r->work_cv.notify_one();
  }
  return LIZG_OK;
}

void lizg_receiver_batch_cap(lizg_receiver *r, int frames) {
  if (!r) return;
  std::lock_guard<std::mutex> lk(r->mu);
  r->cap = frames <= 0 ? kMaxBatch : std::min(frames, kMaxBatch);
}

int lizg_receiver_wants_luma(lizg_receiver *r) { return r ? 1 : lizg::record_error(LIZG_E_ARG, "lizg_receiver_wants_luma: NULL receiver"); }

int lizg_receiver_flush(lizg_receiver *r) {
  if (!r) return lizg::record_error(LIZG_E_ARG, "lizg_receiver_flush: NULL receiver");
  std::unique_lock<std::mutex> lk(r->mu);
  r->idle_cv.wait(lk, [&] { return r->pending.empty() && r->inflight == 0; });
  return (int)r->decoded;
}

const char *lizg_receiver_stats(lizg_receiver *r) {
  if (!r) { lizg::record_error(LIZG_E_ARG, "lizg_receiver_stats: NULL receiver"); return ""; }
  std::lock_guard<std::mutex> lk(r->mu);
  const double secs = r->t_last > r->t_first ? r->t_last - r->t_first : 0;
  char buf[768];
  std::snprintf(buf, sizeof buf,
                "{\"state\":\"running\",\"decoder\":\"gpu\",\"format\":{\"n\":%d,\"subch\":%d,\"span\":%d},\"read\":\"%s\",\"framesIn\":%llu,"
                "\"dropped\":%llu,\"decoded\":%llu,\"waiting\":%d,\"batches\":%llu,\"B\":%.2f,\"cap\":%d,\"verified\":%llu,\"fresh\":%llu,"
                "\"gpuMsPerFrame\":%.4f,\"fps\":%.1f,\"goodputMBps\":%.3f}",
                r->cfg.n, r->cfg.subch, r->cfg.span, r->cfg.read == LIZG_READ_DECODE ? "decode" : "exact", (unsigned long long)r->frames_in,
                (unsigned long long)r->dropped, (unsigned long long)r->decoded, (int)r->pending.size() + r->inflight,
                (unsigned long long)r->batches, r->batches ? (double)r->decoded / r->batches : 0.0, r->cap, (unsigned long long)r->verified,
                (unsigned long long)r->fresh, r->decoded ? r->gpu_ms / r->decoded : 0.0, secs > 0 ? r->decoded / secs : 0.0,
                secs > 0 ? r->fresh * (double)(LIZG_BLOCK_BYTES - 4) / secs / 1e6 : 0.0);
  r->stats_text = buf;
  return r->stats_text.c_str();
}

int lizg_receiver_series(lizg_receiver *r, double since_ms, double *out, int cap) {
  if (!r || (!out && cap > 0)) return lizg::record_error(LIZG_E_ARG, "lizg_receiver_series: a receiver and a place for the series");
  std::lock_guard<std::mutex> lk(r->mu);
  std::vector<double> v;
  v.push_back(r->cfg.subch / 16);   // the format's version (LIZARD-subch carries subch / 16 as its size)
  for (size_t i = 0; i + 8 <= r->series.size(); i += 8)
    if (r->series[i] > since_ms) v.insert(v.end(), r->series.begin() + i, r->series.begin() + i + 8);
  const int n = std::min<int>((int)v.size(), cap);
  if (n > 0) std::memcpy(out, v.data(), sizeof(double) * n);
  return n;
}

}  // extern "C"

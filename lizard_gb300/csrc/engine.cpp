// The multi-stream engine (include/lizard_gb300.h lizg_engine_*): one receiver handle per picture format, each
// format's batch of frames replayed from its own CUDA graph on its own stream, all forked from the caller's stream
// and joined back to it, so frames of every format in flight run at once. Host C++.
#include "lizard_gb300.h"
#include "lizg_internal.h"
#include <cuda_runtime.h>
#include <new>
#include <string>
#include <vector>

struct lizg_engine {
  struct Fmt {
    lizg_rx *rx = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t join = nullptr;
  };
  std::vector<Fmt> fmts;
  cudaEvent_t fork = nullptr;
  int launches = 0;
};

extern "C" {

lizg_engine *lizg_engine_new(void) {
  int sms = 0;
  if (lizg::device_ready(&sms)) return nullptr;
  lizg_engine *e = new (std::nothrow) lizg_engine;
  if (!e) { lizg::record_error(LIZG_E_NOMEM, "lizg_engine_new: out of host memory"); return nullptr; }
  const cudaError_t c = cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming);
  if (c != cudaSuccess) {
    lizg::record_error(LIZG_E_CUDA, (std::string("lizg_engine_new: ") + cudaGetErrorString(c)).c_str());
    delete e;
    return nullptr;
  }
  return e;
}

void lizg_engine_free(lizg_engine *e) {
  if (!e) return;
  for (auto &f : e->fmts) {
    lizg_rx_free(f.rx);
    if (f.st) cudaStreamDestroy(f.st);
    if (f.join) cudaEventDestroy(f.join);
  }
  if (e->fork) cudaEventDestroy(e->fork);
  delete e;
}

int lizg_engine_add_format(lizg_engine *e, int n, int subch, int span, int max_frames) {
  if (!e) return lizg::record_error(LIZG_E_ARG, "lizg_engine_add_format: NULL engine");
  lizg_engine::Fmt f;
  f.rx = lizg_rx_new(n, subch, span, max_frames);
  if (!f.rx) return LIZG_E_ARG;   // lizg_rx_new recorded why
  cudaError_t c = cudaStreamCreateWithFlags(&f.st, cudaStreamNonBlocking);
  if (c == cudaSuccess) c = cudaEventCreateWithFlags(&f.join, cudaEventDisableTiming);
  if (c != cudaSuccess) {
    lizg_rx_free(f.rx);
    if (f.st) cudaStreamDestroy(f.st);
    return lizg::record_error(LIZG_E_CUDA, (std::string("lizg_engine_add_format: ") + cudaGetErrorString(c)).c_str());
  }
  e->fmts.push_back(f);
  return (int)e->fmts.size() - 1;
}

lizg_rx *lizg_engine_rx(lizg_engine *e, int format) {
  if (!e || format < 0 || format >= (int)e->fmts.size()) { lizg::record_error(LIZG_E_ARG, "lizg_engine_rx: no such format"); return nullptr; }
  return e->fmts[format].rx;
}

int lizg_engine_run_dev(lizg_engine *e, const lizg_engine_batch *b, int nb, void *stream) {
  if (!e || !b || nb < 1) return lizg::record_error(LIZG_E_ARG, "lizg_engine_run_dev: NULL engine or no batches");
  std::vector<char> seen(e->fmts.size(), 0);
  for (int i = 0; i < nb; i++) {
    if (b[i].format < 0 || b[i].format >= (int)e->fmts.size()) return lizg::record_error(LIZG_E_ARG, "lizg_engine_run_dev: no such format");
    if (seen[b[i].format]++) return lizg::record_error(LIZG_E_ARG, "lizg_engine_run_dev: a format twice in one run");
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t c = cudaEventRecord(e->fork, st);
  if (c != cudaSuccess) return lizg::record_error(LIZG_E_CUDA, (std::string("lizg_engine_run_dev: ") + cudaGetErrorString(c)).c_str());
  e->launches = 0;
  for (int i = 0; i < nb; i++) {
    lizg_engine::Fmt &f = e->fmts[b[i].format];
    if ((c = cudaStreamWaitEvent(f.st, e->fork, 0)) != cudaSuccess)
      return lizg::record_error(LIZG_E_CUDA, (std::string("lizg_engine_run_dev: ") + cudaGetErrorString(c)).c_str());
    const int rc = lizg_rx_finish_luma_graph(f.rx, b[i].d_luma, b[i].w, b[i].h, b[i].pitch, b[i].frame_stride, b[i].d_reg, b[i].frames,
                                             &b[i].out, nullptr, nullptr, f.st);
    if (rc) return rc;
    e->launches += lizg_rx_launches(f.rx);
    if ((c = cudaEventRecord(f.join, f.st)) != cudaSuccess || (c = cudaStreamWaitEvent(st, f.join, 0)) != cudaSuccess)
      return lizg::record_error(LIZG_E_CUDA, (std::string("lizg_engine_run_dev: ") + cudaGetErrorString(c)).c_str());
  }
  return 0;
}

int lizg_engine_launches(const lizg_engine *e) { return e ? e->launches : LIZG_E_ARG; }

}  // extern "C"

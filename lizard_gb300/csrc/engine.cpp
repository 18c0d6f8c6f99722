// The multi-stream engine (include/lizard_gb300.h lizg_engine_*): one receiver handle per picture format, run in one
// of two ways. A graph a format: each format's batch of frames replayed from its own CUDA graph on its own stream, all
// forked from the caller's stream and joined back to it, so frames of every format in flight run at once. Stage-wise
// across formats: every stage one launch over every format's work items (the column pass's and the row pass's
// (frame, tile) items of every picture size, the decode's (tier, block) items of every format's codes, the light
// per-frame stages' frames, bands and blocks), the whole run captured as one CUDA graph.
// lizg_engine_autotune tunes each format's decode on its batch (lizg_rx_autotune), then times both ways on the
// caller's batches and keeps the faster. Host C++.
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
  int mixed = 0;                 // 1: stage-wise across formats (lizg_engine_set_mixed)
  int *counters = nullptr;       // the mixed decode's work counters, one a launch
  int ncounters = 0;
  // the stage-wise run's captured graph and the call it was captured for
  cudaStream_t cap = nullptr;
  cudaGraphExec_t graph = nullptr;
  std::vector<uintptr_t> graph_key;
  int graph_launches = 0;
};

namespace {

int cuda_fail(const char *who, cudaError_t c) {
  return lizg::record_error(LIZG_E_CUDA, (std::string(who) + ": " + cudaGetErrorString(c)).c_str());
}

// Every format's stream forked from st, fn(i, stream) queued on batch i's format's stream, each joined back to st.
template <class Fn>
int fork_each(lizg_engine *e, const lizg_engine_batch *b, int nb, cudaStream_t st, Fn fn) {
  cudaError_t c = cudaEventRecord(e->fork, st);
  if (c != cudaSuccess) return cuda_fail("lizg_engine_run_dev", c);
  for (int i = 0; i < nb; i++) {
    lizg_engine::Fmt &f = e->fmts[b[i].format];
    if ((c = cudaStreamWaitEvent(f.st, e->fork, 0)) != cudaSuccess) return cuda_fail("lizg_engine_run_dev", c);
    if (int rc = fn(i, f.st)) return rc;
    if ((c = cudaEventRecord(f.join, f.st)) != cudaSuccess || (c = cudaStreamWaitEvent(st, f.join, 0)) != cudaSuccess)
      return cuda_fail("lizg_engine_run_dev", c);
  }
  return 0;
}

// The stage-wise run, queued on st, every stage one launch over every format's work items (kFftMixSegs formats a
// launch; more formats take more launches): the shading sums with the sampler's tables, the column pass, the surface
// factors, the row pass, the pilots' fit, the soft values, the block stage, then the decode over every format's tiers,
// the 1/2 code's first, then 2/3, 3/4, 7/8.
int run_mixed(lizg_engine *e, const lizg_engine_batch *b, int nb, cudaStream_t st) {
  int sms = 0;
  if (int rc = lizg::device_ready(&sms)) return rc;
  std::vector<lizg::RxCall> calls(nb);
  for (int i = 0; i < nb; i++)
    if (int rc = lizg::rx_call(e->fmts[b[i].format].rx, b[i].d_luma, b[i].w, b[i].h, b[i].pitch, b[i].frame_stride, b[i].d_reg, b[i].frames,
                               &b[i].out, calls[i]))
      return rc;
  int launches = 0;
  cudaError_t c;
  auto grids = [&](cudaError_t (*fn)(const lizg::FftSegArgs *, int, cudaStream_t)) {
    std::vector<lizg::FftSegArgs> segs;
    for (int i0 = 0; i0 < nb; i0 += lizg::kFftMixSegs) {
      segs.clear();
      for (int i = i0; i < nb && i < i0 + lizg::kFftMixSegs; i++) segs.push_back(calls[i].fft);
      const cudaError_t x = fn(segs.data(), (int)segs.size(), st);
      if (x != cudaSuccess) return cuda_fail("lizg_engine_run_dev", x);
      launches++;
    }
    return 0;
  };
  if (int rc = grids(lizg::fft_pre_mixed_launch)) return rc;
  if (int rc = grids(lizg::fft_cols_mixed_launch)) return rc;
  if (int rc = grids(lizg::fft_fac_mixed_launch)) return rc;
  if (int rc = grids(lizg::fft_rows_mixed_launch)) return rc;
  {
    std::vector<lizg::DemapSeg> segs;
    for (int i0 = 0; i0 < nb; i0 += lizg::kDemapMixSegs) {
      segs.clear();
      for (int i = i0; i < nb && i < i0 + lizg::kDemapMixSegs; i++) {
        const lizg::RxCall &x = calls[i];
        segs.push_back(lizg::DemapSeg{x.fd, x.fft.b.C, x.fft.b.need, x.align, x.llrf, x.sub_est, x.sub_rms, x.est, x.pilot, x.decl});
      }
      if ((c = lizg::demap_mixed_launch(segs.data(), (int)segs.size(), st)) != cudaSuccess) return cuda_fail("lizg_engine_run_dev", c);
      launches += 3;
    }
  }
  // the decode's segments, the longer codes first, kMixSegs a launch
  std::vector<lizg::LdpcLaunch> seg;
  std::vector<int> code;
  for (int cd = 3; cd >= 0; cd--)
    for (int i = 0; i < nb; i++)
      for (int t = 0; t < calls[i].tiers; t++) {
        lizg::LdpcLaunch a{};
        if (lizg::rx_call_tier(calls[i], t, a) != cd || a.count <= 0) continue;
        seg.push_back(a);
        code.push_back(cd);
      }
  const int nl = ((int)seg.size() + lizg::kMixSegs - 1) / lizg::kMixSegs;
  if (nl > e->ncounters) return lizg::record_error(LIZG_E_ARG, "lizg_engine_run_dev: more decode segments than counters");
  if (nl && (c = cudaMemsetAsync(e->counters, 0, sizeof(int) * nl, st)) != cudaSuccess) return cuda_fail("lizg_engine_run_dev", c);
  for (int l = 0; l < nl; l++) {
    lizg::LdpcMix m{};
    for (int k = l * lizg::kMixSegs; k < (int)seg.size() && m.nseg < lizg::kMixSegs; k++) {
      m.a[m.nseg] = seg[k];
      m.code[m.nseg] = code[k];
      m.first[m.nseg + 1] = m.first[m.nseg] + seg[k].count;
      m.nseg++;
    }
    m.counter = e->counters + l;
    if ((c = lizg::ldpc_mixed_launch(m, sms, st)) != cudaSuccess) return cuda_fail("lizg_engine_run_dev", c);
    launches++;
  }
  e->launches = launches;
  return 0;
}

// The stage-wise run replayed from a CUDA graph, captured on the first run with these batches (and the receivers'
// reads); other batches capture again. The graph reads the buffers the batches name, so their contents may change.
int run_mixed_graph(lizg_engine *e, const lizg_engine_batch *b, int nb, cudaStream_t st) {
  std::vector<uintptr_t> key;
  for (int i = 0; i < nb; i++) {
    const lizg_engine_batch &x = b[i];
    const uintptr_t k[] = {(uintptr_t)x.format, (uintptr_t)x.d_luma, (uintptr_t)x.w, (uintptr_t)x.h, (uintptr_t)x.pitch, (uintptr_t)x.frame_stride,
                           (uintptr_t)x.d_reg, (uintptr_t)x.frames, (uintptr_t)x.out.blocks, (uintptr_t)x.out.ok, (uintptr_t)x.out.its,
                           (uintptr_t)x.out.est, (uintptr_t)x.out.pilot, (uintptr_t)x.out.align, (uintptr_t)x.out.llrf, (uintptr_t)x.out.sub_est,
                           (uintptr_t)x.out.sub_rms};
    key.insert(key.end(), k, k + sizeof k / sizeof k[0]);
    key.push_back((uintptr_t)lizg::rx_read(e->fmts[x.format].rx));
  }
  key.push_back((uintptr_t)e->counters);
  cudaError_t c;
  if (!e->graph || key != e->graph_key) {
    if (e->graph) { cudaGraphExecDestroy(e->graph); e->graph = nullptr; }
    if (!e->cap && (c = cudaStreamCreateWithFlags(&e->cap, cudaStreamNonBlocking)) != cudaSuccess) return cuda_fail("graph stream", c);
    if ((c = cudaStreamBeginCapture(e->cap, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return cuda_fail("begin capture", c);
    const int rc = run_mixed(e, b, nb, e->cap);
    cudaGraph_t g = nullptr;
    c = cudaStreamEndCapture(e->cap, &g);
    if (rc) { if (g) cudaGraphDestroy(g); return rc; }
    if (c != cudaSuccess) return cuda_fail("end capture", c);
    c = cudaGraphInstantiate(&e->graph, g, 0);
    cudaGraphDestroy(g);
    if (c != cudaSuccess) { e->graph = nullptr; return cuda_fail("instantiate", c); }
    e->graph_key = key;
    e->graph_launches = e->launches;
  }
  if ((c = cudaGraphLaunch(e->graph, st)) != cudaSuccess) return cuda_fail("graph launch", c);
  e->launches = e->graph_launches;
  return 0;
}

// A graph a format, each on its format's stream.
int run_per_format(lizg_engine *e, const lizg_engine_batch *b, int nb, cudaStream_t st) {
  int launches = 0;
  const int rc = fork_each(e, b, nb, st, [&](int i, cudaStream_t s) {
    lizg_rx *r = e->fmts[b[i].format].rx;
    const int x = lizg_rx_finish_luma_graph(r, b[i].d_luma, b[i].w, b[i].h, b[i].pitch, b[i].frame_stride, b[i].d_reg, b[i].frames, &b[i].out,
                                            nullptr, nullptr, s);
    if (!x) launches += lizg_rx_launches(r);
    return x;
  });
  if (!rc) e->launches = launches;
  return rc;
}

int check_batches(lizg_engine *e, const lizg_engine_batch *b, int nb, const char *who) {
  if (!e || !b || nb < 1) return lizg::record_error(LIZG_E_ARG, (std::string(who) + ": NULL engine or no batches").c_str());
  std::vector<char> seen(e->fmts.size(), 0);
  for (int i = 0; i < nb; i++) {
    if (b[i].format < 0 || b[i].format >= (int)e->fmts.size()) return lizg::record_error(LIZG_E_ARG, (std::string(who) + ": no such format").c_str());
    if (seen[b[i].format]++) return lizg::record_error(LIZG_E_ARG, (std::string(who) + ": a format twice in one run").c_str());
  }
  return 0;
}

}  // namespace

extern "C" {

lizg_engine *lizg_engine_new(void) {
  int sms = 0;
  if (lizg::device_ready(&sms)) return nullptr;
  lizg_engine *e = new (std::nothrow) lizg_engine;
  if (!e) { lizg::record_error(LIZG_E_NOMEM, "lizg_engine_new: out of host memory"); return nullptr; }
  const cudaError_t c = cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming);
  if (c != cudaSuccess) {
    cuda_fail("lizg_engine_new", c);
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
  if (e->graph) cudaGraphExecDestroy(e->graph);
  if (e->cap) cudaStreamDestroy(e->cap);
  cudaFree(e->counters);
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
    return cuda_fail("lizg_engine_add_format", c);
  }
  // the stage-wise decode's counters: one a launch of kMixSegs tiers, four tiers a format at most
  const int need = (4 * ((int)e->fmts.size() + 1) + lizg::kMixSegs - 1) / lizg::kMixSegs;
  if (need > e->ncounters) {
    int *p = nullptr;
    if ((c = cudaMalloc(&p, sizeof(int) * need)) != cudaSuccess) {
      lizg_rx_free(f.rx);
      cudaStreamDestroy(f.st);
      cudaEventDestroy(f.join);
      return lizg::record_error(LIZG_E_NOMEM, "lizg_engine_add_format: device memory");
    }
    cudaFree(e->counters);
    e->counters = p;
    e->ncounters = need;
  }
  e->fmts.push_back(f);
  return (int)e->fmts.size() - 1;
}

lizg_rx *lizg_engine_rx(lizg_engine *e, int format) {
  if (!e || format < 0 || format >= (int)e->fmts.size()) { lizg::record_error(LIZG_E_ARG, "lizg_engine_rx: no such format"); return nullptr; }
  return e->fmts[format].rx;
}

int lizg_engine_run_dev(lizg_engine *e, const lizg_engine_batch *b, int nb, void *stream) {
  if (int rc = check_batches(e, b, nb, "lizg_engine_run_dev")) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  return e->mixed ? run_mixed_graph(e, b, nb, st) : run_per_format(e, b, nb, st);
}

int lizg_engine_set_mixed(lizg_engine *e, int mixed) {
  if (!e || (mixed != 0 && mixed != 1)) return lizg::record_error(LIZG_E_ARG, "lizg_engine_set_mixed: no engine, or not 0 or 1");
  const int was = e->mixed;
  e->mixed = mixed;
  return was;
}

int lizg_engine_autotune(lizg_engine *e, const lizg_engine_batch *b, int nb, void *stream, float *ms_out) {
  if (int rc = check_batches(e, b, nb, "lizg_engine_autotune")) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // each format's decode tuned on its own batch first (each tier's kernel variant, one launch across the tiers or a
  // launch a tier): timed on the batch, a tier's launch lasts as long as its slowest codeword, so the choice follows
  // the batch's failing codewords as well as its throughput
  for (int i = 0; i < nb; i++)
    if (int rc = lizg_rx_autotune(e->fmts[b[i].format].rx, b[i].d_luma, b[i].w, b[i].h, b[i].pitch, b[i].frame_stride, b[i].d_reg,
                                  b[i].frames, nullptr, stream))
      return rc;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t c = cudaEventCreate(&e0);
  if (c == cudaSuccess) c = cudaEventCreate(&e1);
  float best[2] = {0, 0};
  int rc = 0;
  for (int mode = 0; mode < 2 && !rc && c == cudaSuccess; mode++) {
    e->mixed = mode;
    for (int rep = 0; rep < 4 && !rc && c == cudaSuccess; rep++) {   // the first run captures and warms up
      if ((c = cudaEventRecord(e0, st)) != cudaSuccess) break;
      if ((rc = lizg_engine_run_dev(e, b, nb, stream))) break;
      if ((c = cudaEventRecord(e1, st)) != cudaSuccess || (c = cudaEventSynchronize(e1)) != cudaSuccess) break;
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep == 1 || (rep > 1 && ms < best[mode])) best[mode] = ms;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  e->mixed = !rc && c == cudaSuccess && best[1] < best[0] ? 1 : 0;
  if (rc) return rc;
  if (c != cudaSuccess) return cuda_fail("lizg_engine_autotune", c);
  if (ms_out) { ms_out[0] = best[0]; ms_out[1] = best[1]; }
  return e->mixed;
}

int lizg_engine_launches(const lizg_engine *e) { return e ? e->launches : LIZG_E_ARG; }

}  // extern "C"

// The receiver plan (include/lizard_gb300.h lizg_rx_*): one format's device tables and a batch's working buffers,
// and the order the receive kernels run in. Host C++.
#include "lizard_gb300.h"
#include "format.h"
#include "lizard_codes.h"
#include "lizg_internal.h"
#include <cuda_runtime.h>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

struct lizg_rx {
  lizg::Format f;
  int max_frames = 0, device = -1;
  // device tables
  int16_t *uv = nullptr, *perm[4] = {nullptr, nullptr, nullptr, nullptr};
  int32_t *block_tier = nullptr, *block_slot = nullptr, *pilot_coef = nullptr;
  uint8_t *white = nullptr, *pilot_white = nullptr;
  float2 *rot = nullptr;
  // transform tables
  lizg::FftDev xd{};
  float2 *tw = nullptr, *x1 = nullptr, *x2 = nullptr;
  float *cx = nullptr, *qx = nullptr;
  // working buffers for max_frames frames
  int8_t *llrf = nullptr;
  double *sub_est = nullptr;
  float *sub_rms = nullptr, *est = nullptr, *pilot = nullptr, *align = nullptr;
  uint8_t *decl = nullptr;
  int *counters = nullptr;
  double *hole = nullptr, *part = nullptr;
  float2 *fac = nullptr;
  lizg::SampleDev sd{};
  float *node_xy = nullptr;
  float4 *sample_t = nullptr;
  float2 *Y = nullptr, *C = nullptr;   // column transforms' kept rows; the spectrum's used coefficients in pos order
  float4 *ctab = nullptr;              // the sampler's row and mesh-cell terms, frames x n x nx
  int32_t *tpos = nullptr;             // vrows x n: the pos index of each kept spectrum point, -1 where unused
  CUtensorMap ymap;                    // Y as the row pass's bulk tensor loads see it
  int *dev_err = nullptr;              // set by a pass whose bounded wait gave up
  // per-tier streams, forked from and joined to the caller's
  cudaStream_t side[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t fork = nullptr, join[4] = {nullptr, nullptr, nullptr, nullptr};
  int launches = 0;
  int variant[4] = {-1, -1, -1, -1};   // each tier's LDPC kernel variant (lizg_rx_autotune), -1: the global choice
  int mixed = 0;                        // 1: every tier's decode in one persistent launch (lizg_rx_set_ldpc_mixed)
  std::vector<void *> owned;
  // the captured pipeline of lizg_rx_finish_luma_graph and the call it was captured for
  cudaStream_t cap = nullptr;
  cudaGraphExec_t graph = nullptr;
  std::vector<uintptr_t> graph_key;
  int graph_launches = 0;
  // lizg_rx_finish_luma_host's device copies of its inputs and outputs, grown to the largest call, and its stream
  struct Staged {
    uint8_t *luma = nullptr, *blocks = nullptr, *ok = nullptr;
    float *reg = nullptr;
    int32_t *its = nullptr;
    size_t luma_bytes = 0;
    int frames = 0;
    cudaStream_t st = nullptr;
  } hs;
};

namespace {

template <class T>
cudaError_t dev_copy(lizg_rx *r, T **dst, const T *src, size_t count) {
  cudaError_t e = cudaMalloc(reinterpret_cast<void **>(dst), sizeof(T) * (count ? count : 1));
  if (e != cudaSuccess) return e;
  r->owned.push_back(*dst);
  if (count) e = cudaMemcpy(*dst, src, sizeof(T) * count, cudaMemcpyHostToDevice);
  return e;
}

template <class T>
cudaError_t dev_alloc(lizg_rx *r, T **dst, size_t count) {
  cudaError_t e = cudaMalloc(reinterpret_cast<void **>(dst), sizeof(T) * (count ? count : 1));
  if (e == cudaSuccess) r->owned.push_back(*dst);
  return e;
}

lizg::FmtDev fmt_dev(const lizg_rx *r, int frames) {
  lizg::FmtDev d{};
  const lizg::Format &f = r->f;
  d.n = f.n; d.subch = f.subch; d.blocks = f.blocks; d.frames = frames; d.npilot = (int)f.pilot_coef.size();
  d.V = f.vblocks * f.bw;
  d.turn_scale = (float)lizg::kTurns / (float)f.n;
  for (int t = 0; t < f.tiers; t++) {
    d.tier_first[t] = f.tier_first[t]; d.tier_blocks[t] = f.tier[t].blocks; d.tier_slots[t] = f.tier[t].slots;
    d.tier_nt[t] = f.tier[t].nt; d.tier_k[t] = f.tier[t].k; d.perm[t] = r->perm[t];
  }
  d.uv = r->uv; d.white = r->white; d.block_tier = r->block_tier; d.block_slot = r->block_slot;
  d.pilot_coef = r->pilot_coef; d.pilot_white = r->pilot_white; d.rot = r->rot;
  return d;
}

}  // namespace

extern "C" {

lizg_rx *lizg_rx_new(int n, int subch, int span, int max_frames) {
  if (max_frames < 1 || max_frames > 4096) { lizg::record_error(LIZG_E_ARG, "lizg_rx_new: max_frames must be 1..4096"); return nullptr; }
  int sms = 0;
  if (lizg::device_ready(&sms)) return nullptr;
  lizg_rx *r = new (std::nothrow) lizg_rx;
  if (!r) { lizg::record_error(LIZG_E_NOMEM, "lizg_rx_new: out of host memory"); return nullptr; }
  if (lizg::format_build(n, subch, span, r->f)) {
    lizg::record_error(LIZG_E_ARG, "lizg_rx_new: no format at this (n, subch, span)");
    delete r;
    return nullptr;
  }
  r->max_frames = max_frames;
  cudaGetDevice(&r->device);
  const lizg::Format &f = r->f;
  const size_t need = (size_t)f.subch * lizg::kSub;
  std::vector<float2> rot(lizg::kTurns);
  for (int i = 0; i < lizg::kTurns; i++) {
    const double th = 2.0 * 3.14159265358979323846 * i / lizg::kTurns;
    rot[i] = make_float2((float)std::cos(th), (float)std::sin(th));
  }
  cudaError_t e = cudaSuccess;
  auto ok = [&](cudaError_t x) { if (e == cudaSuccess) e = x; return e == cudaSuccess; };
  ok(dev_copy(r, &r->uv, f.uv.data(), f.uv.size()));
  ok(dev_copy(r, &r->white, f.white.data(), f.white.size()));
  for (int t = 0; t < f.tiers; t++) ok(dev_copy(r, &r->perm[t], f.perm[t].data(), f.perm[t].size()));
  ok(dev_copy(r, &r->block_tier, f.block_tier.data(), f.block_tier.size()));
  ok(dev_copy(r, &r->block_slot, f.block_slot.data(), f.block_slot.size()));
  ok(dev_copy(r, &r->pilot_coef, f.pilot_coef.data(), f.pilot_coef.size()));
  ok(dev_copy(r, &r->pilot_white, f.pilot_white.data(), f.pilot_white.size()));
  ok(dev_copy(r, &r->rot, rot.data(), rot.size()));
  // the transform's plan (three passes a ladder size) and tables: the passes' twiddles and the detrend's DFTs in double
  {
    lizg::FftDev &xd = r->xd;
    xd.n = n; xd.vrows = f.vmax + 1;
    int rad[3], lines = 0;
    if (lizg::fft_plan(n, rad, &lines)) {
      lizg::record_error(LIZG_E_ARG, "lizg_rx_new: no transform plan for this n");
      lizg_rx_free(r);
      return nullptr;
    }
    std::vector<float2> tws(n), x1(n), x2(n);
    for (int st = 0, ns = 1; st < 3; ns *= rad[st], st++)
      for (int q = 1; q < rad[st]; q++)
        for (int k = 0; k < ns; k++) {
          const double th = -2.0 * 3.14159265358979323846 * q * k / ((double)ns * rad[st]);
          tws[ns + (q - 1) * ns + k] = make_float2((float)std::cos(th), (float)std::sin(th));
        }
    for (int t = 0; t < n; t++) { x1[t] = make_float2(f.x1r[t], f.x1i[t]); x2[t] = make_float2(f.x2r[t], f.x2i[t]); }
    ok(dev_copy(r, &r->tw, tws.data(), tws.size()));
    ok(dev_copy(r, &r->x1, x1.data(), x1.size()));
    ok(dev_copy(r, &r->x2, x2.data(), x2.size()));
    ok(dev_copy(r, &r->cx, f.cx.data(), f.cx.size()));
    ok(dev_copy(r, &r->qx, f.qx.data(), f.qx.size()));
    xd.tws = r->tw; xd.x1 = r->x1; xd.x2 = r->x2; xd.cx = r->cx; xd.qx = r->qx; xd.sx2 = f.sx2; xd.sq2 = f.sq2;
    for (int i = 0; i < lizg::kAnchK; i++) { xd.elo[i] = f.elo[i]; xd.ehi[i] = f.ehi[i]; }
    for (int i = 0; i < 36; i++) xd.hole_inv[i] = f.hole_inv[i / 6][i % 6];
  }
  {
    float nodes[40];
    const int nn = lizg::layout_nodes(f.span + 2 * lizg::kMargin, nodes);
    std::vector<float> nxy(nodes, nodes + nn);
    nxy.insert(nxy.end(), nodes, nodes + nn);
    ok(dev_copy(r, &r->node_xy, nxy.data(), nxy.size()));
    r->sd.n = n; r->sd.nx = nn; r->sd.ny = nn;
    r->sd.g0 = lizg::kMargin + 0.5f / f.scale; r->sd.step = 1.0f / f.scale;
    r->sd.node_x = r->node_xy; r->sd.node_y = r->node_xy + nn;
    ok(dev_alloc(r, &r->sample_t, 2 * (size_t)n));
    if (e == cudaSuccess) {
      r->sd.colt = r->sample_t; r->sd.rowt = r->sample_t + n;
      ok(lizg::sample_tables_launch(r->sd, r->sample_t, r->sample_t + n, nullptr));
      ok(cudaDeviceSynchronize());
    }
  }
  const size_t F = (size_t)max_frames;
  ok(dev_alloc(r, &r->hole, F * lizg::fft_hole_bands(n) * 6));
  ok(dev_alloc(r, &r->fac, F * (2 * (size_t)n + r->xd.vrows)));
  ok(dev_alloc(r, &r->part, F * (size_t)(n / 2) * 5));   // column tiles (at most n / 2) x 5
  ok(dev_alloc(r, &r->Y, F * (size_t)r->xd.vrows * n));
  ok(dev_alloc(r, &r->dev_err, 1));
  if (e == cudaSuccess) e = cudaMemset(r->dev_err, 0, sizeof(int));
  if (e == cudaSuccess && lizg::fft_y_map(&r->ymap, r->Y, n, F * (int64_t)r->xd.vrows)) e = cudaErrorInvalidValue;
  ok(dev_alloc(r, &r->ctab, F * n * (size_t)r->sd.nx));
  ok(dev_alloc(r, &r->C, F * need));
  {
    std::vector<int32_t> tp((size_t)r->xd.vrows * n, -1);
    for (size_t i = 0; i < need; i++) tp[f.tix[i]] = (int32_t)i;
    ok(dev_copy(r, &r->tpos, tp.data(), tp.size()));
  }
  ok(dev_alloc(r, &r->llrf, F * 2 * need));
  ok(dev_alloc(r, &r->sub_est, F * f.subch));
  ok(dev_alloc(r, &r->sub_rms, F * f.subch));
  ok(dev_alloc(r, &r->est, F * f.blocks));
  ok(dev_alloc(r, &r->pilot, F * f.blocks));
  ok(dev_alloc(r, &r->align, F * 3));
  ok(dev_alloc(r, &r->decl, F * f.blocks));
  ok(dev_alloc(r, &r->counters, 4));
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r->fork, cudaEventDisableTiming);
  for (int t = 0; t < 4 && e == cudaSuccess; t++) {
    if ((e = cudaStreamCreateWithFlags(&r->side[t], cudaStreamNonBlocking)) == cudaSuccess)
      e = cudaEventCreateWithFlags(&r->join[t], cudaEventDisableTiming);
  }
  if (e != cudaSuccess) {
    lizg::record_error(LIZG_E_CUDA, (std::string("lizg_rx_new: ") + cudaGetErrorString(e)).c_str());
    lizg_rx_free(r);
    return nullptr;
  }
  return r;
}

void lizg_rx_free(lizg_rx *r) {
  if (!r) return;
  for (void *p : r->owned) cudaFree(p);
  for (int t = 0; t < 4; t++) { if (r->side[t]) cudaStreamDestroy(r->side[t]); if (r->join[t]) cudaEventDestroy(r->join[t]); }
  if (r->fork) cudaEventDestroy(r->fork);
  if (r->graph) cudaGraphExecDestroy(r->graph);
  if (r->cap) cudaStreamDestroy(r->cap);
  cudaFree(r->hs.luma); cudaFree(r->hs.reg); cudaFree(r->hs.blocks); cudaFree(r->hs.ok); cudaFree(r->hs.its);
  if (r->hs.st) cudaStreamDestroy(r->hs.st);
  delete r;
}

int lizg_rx_info(const lizg_rx *r, int32_t *info) {
  if (!r || !info) return lizg::record_error(LIZG_E_ARG, "lizg_rx_info: NULL argument");
  const lizg::Format &f = r->f;
  const int32_t head[10] = {f.n, f.subch, f.span, f.blocks, f.used, f.bw, f.vblocks, f.tiers, f.vblocks * f.bw, (int32_t)f.pilot_coef.size()};
  std::memcpy(info, head, sizeof head);
  for (int t = 0; t < 4; t++) {
    info[10 + 3 * t] = t < f.tiers ? f.tier[t].rate : 0;
    info[11 + 3 * t] = t < f.tiers ? f.tier[t].blocks : 0;
    info[12 + 3 * t] = t < f.tiers ? f.tier[t].slots : 0;
  }
  info[22] = r->sd.nx; info[23] = r->sd.ny;
  return 0;
}

int lizg_layout_nodes(int span, float *node_x, float *node_y, int32_t *nn) {
  if (span != 128 && span != 256 && span != 512) return lizg::record_error(LIZG_E_ARG, "lizg_layout_nodes: span must be 128, 256 or 512");
  float p[40];
  const int k = lizg::layout_nodes(span + 2 * lizg::kMargin, p);
  if (node_x) std::memcpy(node_x, p, (size_t)k * sizeof(float));
  if (node_y) std::memcpy(node_y, p, (size_t)k * sizeof(float));
  if (nn) { nn[0] = k; nn[1] = k; }
  return k;
}

int lizg_format_tables(int n, int subch, int span, int32_t *info, int16_t *uv, uint8_t *white, int32_t *block_tier,
                       int32_t *block_slot, int32_t *erase, double *hole_inv, float *detrend, int16_t *perm) {
  lizg::Format f;
  if (lizg::format_build(n, subch, span, f)) return lizg::record_error(LIZG_E_ARG, "lizg_format_tables: no format at this (n, subch, span)");
  if (info) {
    const int32_t head[10] = {f.n, f.subch, f.span, f.blocks, f.used, f.bw, f.vblocks, f.tiers, f.vblocks * f.bw, (int32_t)f.pilot_coef.size()};
    std::memcpy(info, head, sizeof head);
    for (int t = 0; t < 4; t++) {
      info[10 + 3 * t] = t < f.tiers ? f.tier[t].rate : 0;
      info[11 + 3 * t] = t < f.tiers ? f.tier[t].blocks : 0;
      info[12 + 3 * t] = t < f.tiers ? f.tier[t].slots : 0;
    }
  }
  if (uv) std::memcpy(uv, f.uv.data(), f.uv.size() * sizeof(int16_t));
  if (white) std::memcpy(white, f.white.data(), f.white.size());
  if (block_tier) std::memcpy(block_tier, f.block_tier.data(), f.block_tier.size() * sizeof(int32_t));
  if (block_slot) std::memcpy(block_slot, f.block_slot.data(), f.block_slot.size() * sizeof(int32_t));
  if (erase) for (int i = 0; i < lizg::kAnchK; i++) { erase[i] = f.elo[i]; erase[lizg::kAnchK + i] = f.ehi[i]; }
  if (hole_inv) std::memcpy(hole_inv, f.hole_inv, sizeof f.hole_inv);
  if (detrend) {
    const std::vector<float> *parts[6] = {&f.cx, &f.qx, &f.x1r, &f.x1i, &f.x2r, &f.x2i};
    for (int k = 0; k < 6; k++) std::memcpy(detrend + (size_t)k * f.n, parts[k]->data(), (size_t)f.n * sizeof(float));
    detrend[6 * f.n] = (float)f.sx2; detrend[6 * f.n + 1] = (float)f.sq2;
  }
  if (perm) for (int t = 0, at = 0; t < f.tiers; at += (int)f.perm[t].size(), t++) std::memcpy(perm + at, f.perm[t].data(), f.perm[t].size() * sizeof(int16_t));
  return 0;
}

int lizg_rx_perm(const lizg_rx *r, int tier, int16_t *perm) {
  if (!r || !perm || tier < 0 || tier >= r->f.tiers) return lizg::record_error(LIZG_E_ARG, "lizg_rx_perm: bad tier");
  std::memcpy(perm, r->f.perm[tier].data(), r->f.perm[tier].size() * sizeof(int16_t));
  return (int)r->f.perm[tier].size();
}

int lizg_rx_launches(const lizg_rx *r) { return r ? r->launches : LIZG_E_ARG; }

int lizg_rx_fault(lizg_rx *r) {
  if (!r) return lizg::record_error(LIZG_E_ARG, "lizg_rx_fault: NULL handle");
  int v = 0;
  const cudaError_t e = cudaMemcpy(&v, r->dev_err, sizeof(int), cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? v : lizg::record_error(LIZG_E_CUDA, (std::string("lizg_rx_fault: ") + cudaGetErrorString(e)).c_str());
}

int lizg_rx_set_read(lizg_rx *r, int read) {
  if (!r || (read != LIZG_READ_DECODE && read != LIZG_READ_EXACT)) return lizg::record_error(LIZG_E_ARG, "lizg_rx_set_read: no handle or no such read");
  const int was = r->sd.read;
  r->sd.read = read;
  return was;
}

// Tier t's decode launch of a batch's soft values (count and counter left to the caller).
static lizg::LdpcLaunch tier_launch(const lizg_rx *r, const lizg::FmtDev &fd, int frames, const int8_t *llrf, const lizg_rx_out *out, int t) {
  lizg::LdpcLaunch a{};
  a.its = out->its; a.ok = out->ok;
  a.count = frames * r->f.tier[t].blocks;
  a.max_iter = 30; a.stall_it = 9; a.stall_ratio = 0.95f;   // the receiver's (liblizard/src/lizard_phy.c:80-82, 1824)
  a.rx.llrf = llrf; a.rx.decl = r->decl; a.rx.blocks = out->blocks; a.rx.llr_stride = 2 * (int64_t)r->f.subch * lizg::kSub;
  a.fd = fd; a.tier = t;
  return a;
}

// Row (d) and (e) on a batch's soft values: the LDPC decode and CRC of every block not declined, a launch a tier on
// the tiers' own streams (forked from st, joined back), or every tier in one persistent launch (r->mixed).
static int rx_ldpc(lizg_rx *r, const lizg::FmtDev &fd, int frames, int8_t *llrf, const lizg_rx_out *out, cudaStream_t st, int sms) {
  const lizg::Format &f = r->f;
  cudaError_t e;
  if ((e = cudaMemsetAsync(r->counters, 0, 4 * sizeof(int), st)) != cudaSuccess || (e = cudaEventRecord(r->fork, st)) != cudaSuccess)
    return lizg::record_error(LIZG_E_CUDA, (std::string("rx fork: ") + cudaGetErrorString(e)).c_str());
  if (r->mixed) {
    // every tier in one launch on the caller's stream, the longer codes' tiers first
    lizg::LdpcMix m{};
    for (int c = 3; c >= 0; c--)
      for (int t = 0; t < f.tiers; t++)
        if (f.tier[t].code == c) {
          m.a[m.nseg] = tier_launch(r, fd, frames, llrf, out, t);
          m.code[m.nseg] = c;
          m.first[m.nseg + 1] = m.first[m.nseg] + m.a[m.nseg].count;
          m.nseg++;
        }
    m.counter = r->counters;
    if ((e = lizg::ldpc_mixed_launch(m, sms, st)) != cudaSuccess)
      return lizg::record_error(LIZG_E_CUDA, (std::string("rx LDPC: ") + cudaGetErrorString(e)).c_str());
    r->launches++;
    return 0;
  }
  for (int t = 0; t < f.tiers; t++) {
    lizg::LdpcLaunch a = tier_launch(r, fd, frames, llrf, out, t);
    a.counter = r->counters + t;
    if ((e = cudaStreamWaitEvent(r->side[t], r->fork, 0)) != cudaSuccess ||
        (e = (r->variant[t] >= 0 ? lizg::ldpc_launch_variant(f.tier[t].code, r->variant[t], a, sms, r->side[t])
                                 : lizg::ldpc_launch(f.tier[t].code, a, sms, r->side[t]))) != cudaSuccess ||
        (e = cudaEventRecord(r->join[t], r->side[t])) != cudaSuccess || (e = cudaStreamWaitEvent(st, r->join[t], 0)) != cudaSuccess)
      return lizg::record_error(LIZG_E_CUDA, (std::string("rx LDPC: ") + cudaGetErrorString(e)).c_str());
    r->launches++;
  }
  return 0;
}

// Rows (c), (d), (e) on a batch of spectra (spec: frame f's coefficient i, pos order, at spec[f stride + i]):
// the pilots' fit, the soft values, the block stage, then the LDPC and CRC of every block not declined, the four
// codes on their own streams.
static int finish_spec(lizg_rx *r, const float2 *spec, int64_t stride, int frames, const lizg_rx_out *out, cudaStream_t st, int sms) {
  const lizg::Format &f = r->f;
  lizg::FmtDev fd = fmt_dev(r, frames);
  const int64_t need = (int64_t)f.subch * lizg::kSub;
  int8_t *llrf = out->llrf ? out->llrf : r->llrf;
  double *sub_est = out->sub_est ? out->sub_est : r->sub_est;
  float *sub_rms = out->sub_rms ? out->sub_rms : r->sub_rms;
  float *est = out->est ? out->est : r->est;
  float *pilot = out->pilot ? out->pilot : r->pilot;
  float *align = out->align ? out->align : r->align;
  cudaError_t e = lizg::demap_launch(fd, spec, stride, align, llrf, sub_est, sub_rms, est, pilot, r->decl, st);
  if (e != cudaSuccess) return lizg::record_error(LIZG_E_CUDA, (std::string("demap: ") + cudaGetErrorString(e)).c_str());
  r->launches += 3;
  return rx_ldpc(r, fd, frames, llrf, out, st, sms);
}

static int check_call(lizg_rx *r, const void *in, int frames, const lizg_rx_out *out, const char *who, int *sms) {
  if (!r || !in || !out || !out->blocks || !out->ok || !out->its) return lizg::record_error(LIZG_E_ARG, (std::string(who) + ": NULL argument").c_str());
  if (frames < 1 || frames > r->max_frames) return lizg::record_error(LIZG_E_ARG, (std::string(who) + ": frames out of 1..max_frames").c_str());
  return lizg::device_ready(sms);
}

int lizg_rx_finish_coef_dev(lizg_rx *r, const float *d_coef, int frames, const lizg_rx_out *out, void *stream) {
  int sms = 0;
  if (int rc = check_call(r, d_coef, frames, out, "lizg_rx_finish_coef_dev", &sms)) return rc;
  r->launches = 0;
  return finish_spec(r, reinterpret_cast<const float2 *>(d_coef), (int64_t)r->f.subch * lizg::kSub, frames, out, static_cast<cudaStream_t>(stream), sms);
}

// Rows (b) to (e) from a picture source: the anchors' erase and the detrended 2D transform, then as above.
static int finish_src(lizg_rx *r, const lizg::SrcDev &src, int frames, const lizg_rx_out *out, float *d_coef, cudaStream_t st, int sms) {
  const int need = r->f.subch * lizg::kSub;
  float2 *C = d_coef ? reinterpret_cast<float2 *>(d_coef) : r->C;   // the caller's spectrum buffer when given
  const lizg::FftBufs b{r->hole, r->part, r->fac, r->Y, r->tpos, need, C, r->ctab, &r->ymap, r->dev_err};
  cudaError_t e = lizg::fft_launch(r->xd, frames, src, b, sms, st);
  if (e != cudaSuccess) return lizg::record_error(LIZG_E_CUDA, (std::string("transform: ") + cudaGetErrorString(e)).c_str());
  r->launches += src.grid ? 4 : 5;   // sampling in the column pass adds the sampler's row and cell table
  return finish_spec(r, C, need, frames, out, st, sms);
}

int lizg_rx_finish_grid_dev(lizg_rx *r, const float *d_grid, int frames, const lizg_rx_out *out, float *d_coef, void *stream) {
  int sms = 0;
  if (int rc = check_call(r, d_grid, frames, out, "lizg_rx_finish_grid_dev", &sms)) return rc;
  lizg::SrcDev src{};
  src.grid = d_grid; src.gstride = (int64_t)r->f.n * r->f.n; src.sd = r->sd;
  r->launches = 0;
  return finish_src(r, src, frames, out, d_coef, static_cast<cudaStream_t>(stream), sms);
}

// Row (b) alone on picture grids: the anchors' erase, the detrend and the 2D transform, the used coefficients into
// d_coef (frames x subch x 320 complex, pos order). No soft values, no decode.
int lizg_rx_spectrum_grid_dev(lizg_rx *r, const float *d_grid, int frames, float *d_coef, void *stream) {
  if (!r || !d_grid || !d_coef) return lizg::record_error(LIZG_E_ARG, "lizg_rx_spectrum_grid_dev: NULL argument");
  if (frames < 1 || frames > r->max_frames) return lizg::record_error(LIZG_E_ARG, "lizg_rx_spectrum_grid_dev: frames out of 1..max_frames");
  int sms = 0;
  if (int rc = lizg::device_ready(&sms)) return rc;
  lizg::SrcDev src{};
  src.grid = d_grid; src.gstride = (int64_t)r->f.n * r->f.n; src.sd = r->sd;
  const int need = r->f.subch * lizg::kSub;
  const lizg::FftBufs b{r->hole, r->part, r->fac, r->Y, r->tpos, need, reinterpret_cast<float2 *>(d_coef), r->ctab, &r->ymap, r->dev_err};
  cudaError_t e = lizg::fft_launch(r->xd, frames, src, b, sms, static_cast<cudaStream_t>(stream));
  r->launches = 4;
  return e == cudaSuccess ? 0 : lizg::record_error(LIZG_E_CUDA, (std::string("lizg_rx_spectrum_grid_dev: ") + cudaGetErrorString(e)).c_str());
}

// Rows (a) to (e) on a batch of captured luma frames, each with its registration (H, then the node mesh). The
// sampler runs inside the transform's passes (no grid in HBM) unless the caller asks for the grid.
int lizg_rx_finish_luma_dev(lizg_rx *r, const uint8_t *d_luma, int w, int h, int pitch, int64_t frame_stride, const float *d_reg,
                            int frames, const lizg_rx_out *out, float *d_grid, float *d_coef, void *stream) {
  int sms = 0;
  if (int rc = check_call(r, d_luma, frames, out, "lizg_rx_finish_luma_dev", &sms)) return rc;
  if (!d_reg || w < 2 || h < 2 || pitch < w || frame_stride < (int64_t)pitch * h)
    return lizg::record_error(LIZG_E_ARG, "lizg_rx_finish_luma_dev: bad frame geometry or NULL registration");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int regstride = 9 + 2 * r->sd.nx * r->sd.ny;
  r->launches = 0;
  lizg::SrcDev src{};
  src.sd = r->sd;
  src.luma = d_luma; src.w = w; src.h = h; src.pitch = pitch; src.fstride = frame_stride; src.reg = d_reg; src.regstride = regstride;
  if (d_grid) {
    // the grid sampled first; the transform reads it, the shading fit's samples still come from the frame as the
    // reference's finish takes them
    cudaError_t e = lizg::sample_launch(r->sd, frames, d_luma, w, h, pitch, frame_stride, d_reg, regstride, d_grid, st);
    if (e != cudaSuccess) return lizg::record_error(LIZG_E_CUDA, (std::string("sampler: ") + cudaGetErrorString(e)).c_str());
    r->launches = 1;
    src.grid = d_grid; src.gstride = (int64_t)r->f.n * r->f.n;
  }
  return finish_src(r, src, frames, out, d_coef, st, sms);
}

}  // extern "C"

int lizg::rx_spectrum_luma(lizg_rx *r, const uint8_t *d_luma, int w, int h, int pitch, int64_t frame_stride, const float *d_reg, int frames,
                           float *d_coef, cudaStream_t st) {
  if (!r || !d_luma || !d_reg || !d_coef || frames < 1 || frames > r->max_frames || w < 2 || h < 2 || pitch < w)
    return lizg::record_error(LIZG_E_ARG, "spectrum from frames: bad arguments");
  int sms = 0;
  if (int rc = lizg::device_ready(&sms)) return rc;
  lizg::SrcDev src{};
  src.sd = r->sd;
  src.luma = d_luma; src.w = w; src.h = h; src.pitch = pitch; src.fstride = frame_stride; src.reg = d_reg;
  src.regstride = 9 + 2 * r->sd.nx * r->sd.ny;
  const lizg::FftBufs b{r->hole, r->part, r->fac, r->Y, r->tpos, r->f.subch * lizg::kSub, reinterpret_cast<float2 *>(d_coef), r->ctab, &r->ymap, r->dev_err};
  const cudaError_t e = lizg::fft_launch(r->xd, frames, src, b, sms, st);
  return e == cudaSuccess ? 0 : lizg::record_error(LIZG_E_CUDA, (std::string("spectrum from frames: ") + cudaGetErrorString(e)).c_str());
}

int lizg::rx_call(lizg_rx *r, const uint8_t *d_luma, int w, int h, int pitch, int64_t frame_stride, const float *d_reg, int frames,
                  const lizg_rx_out *out, RxCall &c) {
  int sms = 0;
  if (int rc = check_call(r, d_luma, frames, out, "lizg_engine_run_dev", &sms)) return rc;
  if (!d_reg || w < 2 || h < 2 || pitch < w || frame_stride < (int64_t)pitch * h)
    return lizg::record_error(LIZG_E_ARG, "lizg_engine_run_dev: bad frame geometry or NULL registration");
  c = RxCall{};
  c.r = r;
  c.fft.xd = r->xd;
  c.fft.frames = frames;
  SrcDev &src = c.fft.src;
  src.sd = r->sd;
  src.luma = d_luma; src.w = w; src.h = h; src.pitch = pitch; src.fstride = frame_stride; src.reg = d_reg;
  src.regstride = 9 + 2 * r->sd.nx * r->sd.ny;
  c.fft.b = FftBufs{r->hole, r->part, r->fac, r->Y, r->tpos, r->f.subch * lizg::kSub, r->C, r->ctab, &r->ymap, r->dev_err};
  c.fd = fmt_dev(r, frames);
  c.tiers = r->f.tiers;
  c.out = out;
  c.llrf = out->llrf ? out->llrf : r->llrf;
  c.sub_est = out->sub_est ? out->sub_est : r->sub_est;
  c.sub_rms = out->sub_rms ? out->sub_rms : r->sub_rms;
  c.est = out->est ? out->est : r->est;
  c.pilot = out->pilot ? out->pilot : r->pilot;
  c.align = out->align ? out->align : r->align;
  c.decl = r->decl;
  return 0;
}

int lizg::rx_read(const lizg_rx *r) { return r->sd.read; }

int lizg::rx_call_tier(const RxCall &c, int t, LdpcLaunch &a) {
  a = tier_launch(c.r, c.fd, c.fft.frames, c.llrf, c.out, t);
  return c.r->f.tier[t].code;
}

extern "C" {

// The same call as lizg_rx_finish_luma_dev, replayed from a CUDA graph: the first call with a given set of buffers
// and sizes captures the whole per-frame pipeline (its 10 to 12 kernels, the per-code fork and join) on the handle's
// own stream; later calls with the same arguments launch the captured graph on `stream` in one call. Different
// arguments capture again. The graph reads the buffers the call names, so their contents may change between calls.
int lizg_rx_finish_luma_graph(lizg_rx *r, const uint8_t *d_luma, int w, int h, int pitch, int64_t frame_stride, const float *d_reg,
                              int frames, const lizg_rx_out *out, float *d_grid, float *d_coef, void *stream) {
  int sms = 0;
  if (int rc = check_call(r, d_luma, frames, out, "lizg_rx_finish_luma_graph", &sms)) return rc;
  const std::vector<uintptr_t> key = {(uintptr_t)d_luma, (uintptr_t)w, (uintptr_t)h, (uintptr_t)pitch, (uintptr_t)frame_stride,
                                      (uintptr_t)d_reg, (uintptr_t)frames, (uintptr_t)out->blocks, (uintptr_t)out->ok, (uintptr_t)out->its,
                                      (uintptr_t)out->est, (uintptr_t)out->pilot, (uintptr_t)out->align, (uintptr_t)out->llrf,
                                      (uintptr_t)out->sub_est, (uintptr_t)out->sub_rms, (uintptr_t)d_grid, (uintptr_t)d_coef, (uintptr_t)r->sd.read,
                                      (uintptr_t)(r->variant[0] + 1), (uintptr_t)(r->variant[1] + 1), (uintptr_t)(r->variant[2] + 1),
                                      (uintptr_t)(r->variant[3] + 1), (uintptr_t)r->mixed};
  cudaError_t e;
  if (!r->graph || key != r->graph_key) {
    if (r->graph) { cudaGraphExecDestroy(r->graph); r->graph = nullptr; }
    if (!r->cap && (e = cudaStreamCreateWithFlags(&r->cap, cudaStreamNonBlocking)) != cudaSuccess)
      return lizg::record_error(LIZG_E_CUDA, (std::string("graph stream: ") + cudaGetErrorString(e)).c_str());
    if ((e = cudaStreamBeginCapture(r->cap, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
      return lizg::record_error(LIZG_E_CUDA, (std::string("begin capture: ") + cudaGetErrorString(e)).c_str());
    const int rc = lizg_rx_finish_luma_dev(r, d_luma, w, h, pitch, frame_stride, d_reg, frames, out, d_grid, d_coef, r->cap);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(r->cap, &g);
    if (rc) { if (g) cudaGraphDestroy(g); return rc; }
    if (e != cudaSuccess) return lizg::record_error(LIZG_E_CUDA, (std::string("end capture: ") + cudaGetErrorString(e)).c_str());
    e = cudaGraphInstantiate(&r->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { r->graph = nullptr; return lizg::record_error(LIZG_E_CUDA, (std::string("instantiate: ") + cudaGetErrorString(e)).c_str()); }
    r->graph_key = key;
    r->graph_launches = r->launches;
  }
  if ((e = cudaGraphLaunch(r->graph, static_cast<cudaStream_t>(stream))) != cudaSuccess)
    return lizg::record_error(LIZG_E_CUDA, (std::string("graph launch: ") + cudaGetErrorString(e)).c_str());
  r->launches = r->graph_launches;
  return 0;
}

// Rows (a) to (e) from frames and registrations in host memory: copied to the handle's device buffers (grown to the
// largest call), decoded as lizg_rx_finish_luma_dev on the handle's own stream, the blocks, verdicts and iterations
// copied back before the call returns.
int lizg_rx_finish_luma_host(lizg_rx *r, const uint8_t *luma, int w, int h, int pitch, int64_t frame_stride, const float *reg, int frames,
                             uint8_t *blocks, uint8_t *ok, int32_t *its) {
  if (!r || !luma || !reg || !blocks || !ok || !its) return lizg::record_error(LIZG_E_ARG, "lizg_rx_finish_luma_host: NULL argument");
  if (frames < 1 || frames > r->max_frames) return lizg::record_error(LIZG_E_ARG, "lizg_rx_finish_luma_host: frames out of 1..max_frames");
  if (w < 2 || h < 2 || pitch < w || frame_stride < (int64_t)pitch * h) return lizg::record_error(LIZG_E_ARG, "lizg_rx_finish_luma_host: bad frame geometry");
  int sms = 0;
  if (int rc = lizg::device_ready(&sms)) return rc;
  auto &hs = r->hs;
  const size_t lb = (size_t)w * h * frames, nb = (size_t)r->f.blocks * frames, rs = 9 + 2 * (size_t)r->sd.nx * r->sd.ny;
  cudaError_t e = cudaSuccess;
  auto fail = [&](const char *what) { return lizg::record_error(LIZG_E_CUDA, (std::string("lizg_rx_finish_luma_host: ") + what + ": " + cudaGetErrorString(e)).c_str()); };
  if (!hs.st && (e = cudaStreamCreateWithFlags(&hs.st, cudaStreamNonBlocking)) != cudaSuccess) return fail("stream");
  if (lb > hs.luma_bytes) {
    cudaFree(hs.luma); hs.luma = nullptr; hs.luma_bytes = 0;
    if ((e = cudaMalloc(&hs.luma, lb)) != cudaSuccess) return lizg::record_error(LIZG_E_NOMEM, "lizg_rx_finish_luma_host: device memory");
    hs.luma_bytes = lb;
  }
  if (frames > hs.frames) {
    cudaFree(hs.reg); cudaFree(hs.blocks); cudaFree(hs.ok); cudaFree(hs.its);
    hs.reg = nullptr; hs.blocks = hs.ok = nullptr; hs.its = nullptr; hs.frames = 0;
    if (cudaMalloc(&hs.reg, rs * sizeof(float) * frames) != cudaSuccess || cudaMalloc(&hs.blocks, nb * LIZG_BLOCK_BYTES) != cudaSuccess ||
        cudaMalloc(&hs.ok, nb) != cudaSuccess || cudaMalloc(&hs.its, nb * sizeof(int32_t)) != cudaSuccess)
      return lizg::record_error(LIZG_E_NOMEM, "lizg_rx_finish_luma_host: device memory");
    hs.frames = frames;
  }
  if (pitch == w && frame_stride == (int64_t)w * h) e = cudaMemcpyAsync(hs.luma, luma, lb, cudaMemcpyHostToDevice, hs.st);
  else
    for (int k = 0; k < frames && e == cudaSuccess; k++)
      e = cudaMemcpy2DAsync(hs.luma + (size_t)k * w * h, w, luma + k * frame_stride, pitch, w, h, cudaMemcpyHostToDevice, hs.st);
  if (e != cudaSuccess || (e = cudaMemcpyAsync(hs.reg, reg, rs * sizeof(float) * frames, cudaMemcpyHostToDevice, hs.st)) != cudaSuccess) return fail("copy in");
  const lizg_rx_out out{hs.blocks, hs.ok, hs.its, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  if (int rc = lizg_rx_finish_luma_dev(r, hs.luma, w, h, w, (int64_t)w * h, hs.reg, frames, &out, nullptr, nullptr, hs.st)) return rc;
  if ((e = cudaMemcpyAsync(blocks, hs.blocks, nb * LIZG_BLOCK_BYTES, cudaMemcpyDeviceToHost, hs.st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(ok, hs.ok, nb, cudaMemcpyDeviceToHost, hs.st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(its, hs.its, nb * sizeof(int32_t), cudaMemcpyDeviceToHost, hs.st)) != cudaSuccess)
    return fail("copy out");
  if ((e = cudaStreamSynchronize(hs.st)) != cudaSuccess) return fail("decode");
  int verified = 0;
  for (size_t i = 0; i < nb; i++) verified += ok[i] != 0;
  return verified;
}

int lizg_rx_set_ldpc_mixed(lizg_rx *r, int mixed) {
  if (!r || (mixed != 0 && mixed != 1)) return lizg::record_error(LIZG_E_ARG, "lizg_rx_set_ldpc_mixed: no handle, or not 0 or 1");
  const int was = r->mixed;
  r->mixed = mixed;
  return was;
}

int lizg_rx_variant(const lizg_rx *r, int tier) {
  if (!r || tier < 0 || tier >= r->f.tiers) return lizg::record_error(LIZG_E_ARG, "lizg_rx_variant: no handle or no such tier");
  return r->variant[tier] >= 0 ? r->variant[tier] : lizg::ldpc_choice(r->f.tier[tier].code);
}

int lizg_rx_autotune(lizg_rx *r, const uint8_t *d_luma, int w, int h, int pitch, int64_t frame_stride, const float *d_reg, int frames,
                     int32_t *choice, void *stream) {
  if (!r || !d_luma || !d_reg) return lizg::record_error(LIZG_E_ARG, "lizg_rx_autotune: NULL argument");
  if (frames < 1 || frames > r->max_frames) return lizg::record_error(LIZG_E_ARG, "lizg_rx_autotune: frames out of 1..max_frames");
  int sms = 0;
  if (int rc = lizg::device_ready(&sms)) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const lizg::Format &f = r->f;
  const size_t nb = (size_t)f.blocks * frames;
  uint8_t *blocks = nullptr, *ok = nullptr;
  int32_t *its = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaMalloc(&blocks, nb * LIZG_BLOCK_BYTES);
  if (e == cudaSuccess) e = cudaMalloc(&ok, nb);
  if (e == cudaSuccess) e = cudaMalloc(&its, nb * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  int rc = 0;
  int best[4] = {-1, -1, -1, -1};
  if (e == cudaSuccess) {
    // the soft values of the batch, in the handle's own buffers
    for (int t = 0; t < 4; t++) r->variant[t] = -1;
    r->mixed = 0;
    const lizg_rx_out out{blocks, ok, its, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    rc = lizg_rx_finish_luma_dev(r, d_luma, w, h, pitch, frame_stride, d_reg, frames, &out, nullptr, nullptr, stream);
    const lizg::FmtDev fd = fmt_dev(r, frames);
    for (int t = 0; t < f.tiers && !rc && e == cudaSuccess; t++) {
      lizg::LdpcLaunch a = tier_launch(r, fd, frames, r->llrf, &out, t);   // as finish_spec launches it
      a.counter = r->counters + t;
      float best_ms = 0;
      for (int v = 0; v < lizg::ldpc_variant_count(f.tier[t].code) && e == cudaSuccess; v++) {
        float ms_min = 0;
        for (int rep = 0; rep < 4 && e == cudaSuccess; rep++) {   // the first run warms up
          if ((e = cudaMemsetAsync(r->counters + t, 0, sizeof(int), st)) != cudaSuccess || (e = cudaEventRecord(e0, st)) != cudaSuccess ||
              (e = lizg::ldpc_launch_variant(f.tier[t].code, v, a, sms, st)) != cudaSuccess || (e = cudaEventRecord(e1, st)) != cudaSuccess ||
              (e = cudaEventSynchronize(e1)) != cudaSuccess)
            break;
          float ms = 0;
          cudaEventElapsedTime(&ms, e0, e1);
          if (rep == 1 || (rep > 1 && ms < ms_min)) ms_min = ms;
        }
        if (e == cudaSuccess && (best[t] < 0 || ms_min < best_ms)) { best[t] = v; best_ms = ms_min; }
      }
    }
    // then the whole decode stage with those variants, a launch a tier on forked streams against one persistent launch
    // across the tiers; the faster kept
    float stage_ms[2] = {0, 0};
    for (int mixed = 0; mixed < 2 && !rc && e == cudaSuccess; mixed++) {
      for (int t = 0; t < 4; t++) r->variant[t] = t < f.tiers ? best[t] : -1;
      r->mixed = mixed;
      const lizg_rx_out out{blocks, ok, its, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
      for (int rep = 0; rep < 4 && !rc && e == cudaSuccess; rep++) {
        if ((e = cudaEventRecord(e0, st)) != cudaSuccess) break;
        if ((rc = rx_ldpc(r, fd, frames, r->llrf, &out, st, sms))) break;
        if ((e = cudaEventRecord(e1, st)) != cudaSuccess || (e = cudaEventSynchronize(e1)) != cudaSuccess) break;
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep == 1 || (rep > 1 && ms < stage_ms[mixed])) stage_ms[mixed] = ms;
      }
    }
    r->mixed = stage_ms[1] < stage_ms[0] ? 1 : 0;
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  if (rc || e != cudaSuccess) r->mixed = 0;
  cudaFree(blocks); cudaFree(ok); cudaFree(its);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (rc) return rc;
  if (e != cudaSuccess) return lizg::record_error(LIZG_E_CUDA, (std::string("lizg_rx_autotune: ") + cudaGetErrorString(e)).c_str());
  for (int t = 0; t < 4; t++) {
    r->variant[t] = t < f.tiers ? best[t] : -1;
    if (choice) choice[t] = r->variant[t];
  }
  return 0;
}

}  // extern "C"

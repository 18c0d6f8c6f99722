// The format word on sm_103a: its read off the border of a registered frame and its Reed-Solomon soft decode, a
// batch of frames a launch, one CTA a frame. Restated from the reference:
//   - the read (liblizard/src/acquire.c:4503-4559 ob_thin_read_fmt): bilinear samples through the homography and
//     the node mesh (ob_map_point acquire.c:5090-5105, sample internal.h:11-23) of the line, the gap, the timing
//     track's Manchester pairs and the word's cells; each word cell against the mean of the pairs within 12 modules;
//     the word's own two means' midpoint, over the border's contrast, clipped to +-0.5;
//   - the decode (liblizard/src/fmt.c:54-86, rs.c): hard bytes through errors-only RS, then the least confident bytes
//     erased two more a step, accepted only with the magic and a version in 4..64.
// Compiled with -fmad=false: every float operation rounds once, in the reference's order, so the soft values are
// the reference's bit for bit. The ordered float sums (the contrast, the two means) are one thread's each; the RS
// work is one warp's, its lanes over syndromes, coefficients and positions.
#include <cuda_runtime.h>
#include <stdint.h>
#include <algorithm>
#include <mutex>
#include <string>
#include "format.h"
#include "lizard_gb300.h"
#include "lizg_internal.h"

namespace lizg {

constexpr int kFmtThreads = 128, kFmtMaxCells = 128, kFmtMaxBytes = 64, kFmtMaxPairs = 64, kFmtMaxRefs = 32, kPoly = 128;
constexpr int kReserve = 15, kMagic = 0x4c, kVersionMin = 4, kVersionMax = 64;

static __device__ __align__(16) uint8_t g_gf[768];   // exp[512] then log[256] of GF(256), polynomial 0x11d (rs.c:7-14)

struct FmtGeom {
  int W, cells, bytes, npair, nrs, nn;   // border side (modules), word cells a side, codeword bytes, track pairs a
                                         // side, reference points a side, mesh nodes an axis
  int iw, ih, reg_stride;
  int64_t frame_stride;
  float nodes[40];
};

// ---------------------------------------------------------------- the read

__device__ __forceinline__ float grey_k(int k) { return (float)k / 255.0f; }   // the image's table, i / 255.0f

__device__ float sample_px(const uint8_t *px, int w, int h, float x, float y) {   // internal.h:11-23
  x -= 0.5f;
  y -= 0.5f;
  if (x < 0) x = 0; else if (x > w - 1.001f) x = w - 1.001f;
  if (y < 0) y = 0; else if (y > h - 1.001f) y = h - 1.001f;
  const int xi = x >= 0 ? (int)x : 0, yi = y >= 0 ? (int)y : 0;
  const float fx = x - xi, fy = y - yi;
  const uint8_t *p = px + (int64_t)yi * w + xi;
  const float a = grey_k(p[0]), b = grey_k(p[1]), c = grey_k(p[w]), d = grey_k(p[w + 1]);
  return (a + (b - a) * fx) * (1 - fy) + (c + (d - c) * fx) * fy;
}

__device__ int node_cell(const float *node, int nn, float m) {   // acquire.c:5090-5094
  int lo = 0, hi = nn - 2;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (m >= node[mid]) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// The image point of module point (mx, my): H, then the mesh's bilinear displacement (acquire.c:5095-5105).
__device__ void map_point(const float *reg, const FmtGeom &g, float mx, float my, float *pu, float *pv) {
  const int j = node_cell(g.nodes, g.nn, my), i = node_cell(g.nodes, g.nn, mx);
  const float v = (my - g.nodes[j]) / (g.nodes[j + 1] - g.nodes[j]), u = (mx - g.nodes[i]) / (g.nodes[i + 1] - g.nodes[i]);
  const float *n00 = reg + 9 + 2 * (j * g.nn + i), *n10 = n00 + 2, *n01 = n00 + 2 * g.nn, *n11 = n01 + 2;
  const float dx = (n00[0] * (1 - u) + n10[0] * u) * (1 - v) + (n01[0] * (1 - u) + n11[0] * u) * v;
  const float dy = (n00[1] * (1 - u) + n10[1] * u) * (1 - v) + (n01[1] * (1 - u) + n11[1] * u) * v;
  const float w = reg[6] * mx + reg[7] * my + 1;
  *pu = (reg[0] * mx + reg[1] * my + reg[2]) / w + dx;
  *pv = (reg[3] * mx + reg[4] * my + reg[5]) / w + dy;
}

// The sample at t along side 0..3 (top, right, bottom, left) and depth d (acquire.c:3806-3810).
__device__ float read_at(const uint8_t *px, const float *reg, const FmtGeom &g, int side, float t, float d) {
  const float x = side == 0 || side == 2 ? t : side == 3 ? d : g.W - d;
  const float y = side == 0 ? d : side == 2 ? g.W - d : t;
  float u, v;
  map_point(reg, g, x, y, &u, &v);
  return sample_px(px, g.iw, g.ih, u, v);
}

__device__ __forceinline__ int band_pair(int k) { return (k / 4) * 8 + k % 4; }   // layout.h:110-112

// ---------------------------------------------------------------- GF(256) and Reed-Solomon, a warp

struct Gf {
  const uint8_t *ex, *lg;
  __device__ __forceinline__ uint8_t mul(uint32_t a, uint32_t b) const { return a && b ? ex[lg[a] + lg[b]] : 0; }
  __device__ __forceinline__ uint8_t inv(uint32_t a) const { return ex[255 - lg[a]]; }
};

__device__ __forceinline__ uint32_t warp_xor(uint32_t v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v ^= __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Syndromes S[i] = cw(alpha^i), i < nroots (rs.c:39-45). Returns whether any is nonzero.
__device__ bool syndromes(const Gf &gf, const uint8_t *cw, int n, int nroots, uint8_t *S, int lane) {
  bool any = false;
  for (int i = lane; i < nroots; i += 32) {
    uint8_t s = 0;
    for (int j = 0; j < n; j++) s = gf.mul(s, gf.ex[i]) ^ cw[j];
    S[i] = s;
    any |= s != 0;
  }
  __syncwarp();
  return __any_sync(0xffffffffu, any);
}

// Chien search for the locator lam of degree deg, then Forney's values (rs.c:63-86, 127-141): positions j = lane,
// lane + 32. Corrects cw in place; returns the roots found, or -1 (not deg roots, or a vanishing derivative).
__device__ int chien_forney(const Gf &gf, uint8_t *cw, int n, int nroots, const uint8_t *S, const uint8_t *lam, int deg, uint8_t *Wv, int lane) {
  bool root[2] = {false, false};
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int j = lane + 32 * h;
    if (j < n) {
      const int e = (255 - (n - 1 - j)) % 255;
      uint8_t v = 0;
      for (int i = deg; i >= 0; i--) v = gf.mul(v, gf.ex[e]) ^ lam[i];
      root[h] = v == 0;
    }
  }
  const int found = __popc(__ballot_sync(0xffffffffu, root[0])) + __popc(__ballot_sync(0xffffffffu, root[1]));
  if (found != deg) return -1;
  for (int i = lane; i < nroots; i += 32) {
    uint8_t w = 0;
    for (int j = 0; j <= i && j <= deg; j++) w ^= gf.mul(S[i - j], lam[j]);
    Wv[i] = w;
  }
  __syncwarp();
  bool bad = false;
  uint8_t fix[2] = {0, 0};
#pragma unroll
  for (int h = 0; h < 2; h++) {
    if (!root[h]) continue;
    const int j = lane + 32 * h;
    const uint8_t xi = gf.ex[(255 - (n - 1 - j)) % 255];
    uint8_t num = 0, den = 0, p = 1;
    for (int i = 0; i < nroots; i++) { num ^= gf.mul(Wv[i], p); p = gf.mul(p, xi); }
    p = 1;
    for (int i = 1; i <= deg; i += 2) { den ^= gf.mul(lam[i], p); p = gf.mul(p, gf.mul(xi, xi)); }
    if (!den) bad = true;
    else fix[h] = gf.mul(gf.mul(num, gf.inv(den)), gf.ex[(n - 1 - j) % 255]);
  }
  if (__any_sync(0xffffffffu, bad)) return -1;
#pragma unroll
  for (int h = 0; h < 2; h++) if (root[h]) cw[lane + 32 * h] ^= fix[h];
  __syncwarp();
  return found;
}

// Errors only (rs.c:37-87): Berlekamp-Massey with the discrepancy's sum and the register update across lanes.
// Coefficients past kPoly never reach one below it, so the reference's 256 and these 128 agree on every one read.
__device__ int rs_decode_w(const Gf &gf, uint8_t *cw, int n, int nroots, const uint8_t *S, bool any, uint8_t *C, uint8_t *B, uint8_t *T,
                           uint8_t *Wv, int lane) {
  if (!any) return 0;
  for (int i = lane; i < kPoly; i += 32) { C[i] = i == 0; B[i] = i == 0; }
  __syncwarp();
  int L = 0, m = 1;
  uint8_t b = 1;
  for (int r = 0; r < nroots; r++) {
    uint32_t part = 0;
    for (int i = 1 + lane; i <= L; i += 32) part ^= gf.mul(C[i], S[r - i]);
    const uint8_t d = (uint8_t)(S[r] ^ warp_xor(part));
    if (!d) { m++; continue; }
    for (int i = lane; i < kPoly; i += 32) T[i] = C[i];
    __syncwarp();
    const uint8_t f = gf.mul(d, gf.inv(b));
    for (int i = lane; i + m < kPoly; i += 32) C[i + m] ^= gf.mul(f, B[i]);
    __syncwarp();
    if (2 * L <= r) {
      L = r + 1 - L;
      for (int i = lane; i < kPoly; i += 32) B[i] = T[i];
      b = d;
      m = 1;
    } else {
      m++;
    }
    __syncwarp();
  }
  if (L > nroots / 2) return -1;
  return chien_forney(gf, cw, n, nroots, S, C, L, Wv, lane);
}

// Errors and erasures (rs.c:89-146): the erasures' locator, Berlekamp-Massey from it, accepted only where the
// locator's degree is the register's length and 2 errors + erasures <= nroots.
__device__ int rs_decode_er_w(const Gf &gf, uint8_t *cw, int n, int nroots, const uint8_t *S, bool any, const int *eras, int neras, uint8_t *lam,
                              uint8_t *b, uint8_t *t, uint8_t *Wv, int lane) {
  if (!any && !neras) return 0;
  if (neras > nroots) return -1;
  for (int i = lane; i < kPoly; i += 32) lam[i] = i == 0;
  __syncwarp();
  for (int k = 0; k < neras; k++) {   // lam *= (1 - X_k x), each coefficient from the old ones
    const uint8_t X = gf.ex[(n - 1 - eras[k]) % 255];
    uint8_t nv[kPoly / 32];
#pragma unroll
    for (int h = 0; h < kPoly / 32; h++) {
      const int i = lane + 32 * h;
      nv[h] = i >= 1 && i <= k + 1 ? lam[i] ^ gf.mul(lam[i - 1], X) : lam[i];
    }
    __syncwarp();
#pragma unroll
    for (int h = 0; h < kPoly / 32; h++) lam[lane + 32 * h] = nv[h];
    __syncwarp();
  }
  for (int i = lane; i < kPoly; i += 32) b[i] = lam[i];
  __syncwarp();
  int el = neras;
  auto shift_b = [&]() {   // b *= x
    uint8_t nv[kPoly / 32];
#pragma unroll
    for (int h = 0; h < kPoly / 32; h++) { const int i = lane + 32 * h; nv[h] = i ? b[i - 1] : 0; }
    __syncwarp();
#pragma unroll
    for (int h = 0; h < kPoly / 32; h++) b[lane + 32 * h] = nv[h];
    __syncwarp();
  };
  for (int r = neras + 1; r <= nroots; r++) {
    uint32_t part = 0;
    for (int i = lane; i < r && i <= el; i += 32) part ^= gf.mul(lam[i], S[r - i - 1]);
    const uint8_t d = (uint8_t)warp_xor(part);
    if (!d) { shift_b(); continue; }
    for (int i = lane; i < kPoly; i += 32) t[i] = i == 0 ? lam[0] : lam[i] ^ gf.mul(d, b[i - 1]);
    __syncwarp();
    if (2 * el <= r + neras - 1) {
      el = r + neras - el;
      const uint8_t di = gf.inv(d);
      for (int i = lane; i < kPoly; i += 32) b[i] = gf.mul(lam[i], di);
      __syncwarp();
    } else {
      shift_b();
    }
    for (int i = lane; i < kPoly; i += 32) lam[i] = t[i];
    __syncwarp();
  }
  int deg = 0;
  for (int i = lane; i <= nroots; i += 32) if (lam[i]) deg = i;
#pragma unroll
  for (int o = 16; o; o >>= 1) deg = max(deg, __shfl_xor_sync(0xffffffffu, deg, o));
  if (deg != el || 2 * (el - neras) + neras > nroots) return -1;
  return chien_forney(gf, cw, n, nroots, S, lam, deg, Wv, lane);
}

struct RsWork {
  uint8_t cw[kFmtMaxBytes], got[kFmtMaxBytes], S[kFmtMaxBytes], Wv[kFmtMaxBytes];
  uint8_t p0[kPoly], p1[kPoly], p2[kPoly];
  float worst[kFmtMaxBytes];
  int order[kFmtMaxBytes];
};

// The word from soft values q (4 x cells, > 0 dark), one warp (fmt.c:54-86). word: ok, version, fps.
__device__ void fmt_decode_w(const Gf &gf, const float *q, int cells, int bytes, RsWork &w, int32_t *ok_ver_fps, int lane) {
  const int nroots = bytes - 3;
  for (int k = lane; k < bytes; k += 32) {
    const float *qs = q + (k & 3) * cells + 8 * (k >> 2);
    uint32_t v = 0;
    float lo = 1;
    for (int bb = 0; bb < 8; bb++) {
      const float s = qs[bb], a = s < 0 ? -s : s;
      v = ((v << 1) | (s > 0)) & 255u;
      if (a < lo) lo = a;
    }
    w.cw[k] = (uint8_t)v;
    w.worst[k] = lo;
  }
  __syncwarp();
  const bool any = syndromes(gf, w.cw, bytes, nroots, w.S, lane);
  auto accept = [&](const uint8_t *c) { return c[0] == kMagic && c[1] >= kVersionMin && c[1] <= kVersionMax; };
  auto copy = [&]() {
    for (int k = lane; k < bytes; k += 32) w.got[k] = w.cw[k];
    __syncwarp();
  };
  copy();
  int rc = rs_decode_w(gf, w.got, bytes, nroots, w.S, any, w.p0, w.p1, w.p2, w.Wv, lane);
  bool done = rc >= 0 && accept(w.got);
  if (!done) {
    // the least confident first, the lower index on a tie
    for (int k = lane; k < bytes; k += 32) {
      int rank = 0;
      for (int j = 0; j < bytes; j++) rank += w.worst[j] < w.worst[k] || (w.worst[j] == w.worst[k] && j < k);
      w.order[rank] = k;
    }
    __syncwarp();
    for (int ne = 2; ne <= nroots - 3 && !done; ne += 2) {
      copy();
      rc = rs_decode_er_w(gf, w.got, bytes, nroots, w.S, any, w.order, ne, w.p0, w.p1, w.p2, w.Wv, lane);
      done = rc >= 0 && accept(w.got);
    }
  }
  if (lane == 0) {
    ok_ver_fps[0] = done;
    ok_ver_fps[1] = done ? w.got[1] : 0;
    ok_ver_fps[2] = done ? w.got[2] : 0;
  }
}

__device__ void load_gf(uint8_t *s_gf) {
  for (int i = threadIdx.x; i < 768 / 16; i += blockDim.x) reinterpret_cast<uint4 *>(s_gf)[i] = reinterpret_cast<const uint4 *>(g_gf)[i];
}

// ---------------------------------------------------------------- the kernels

// One CTA a frame: every sample the read takes, then the soft values in the reference's order, then the decode.
__global__ void __launch_bounds__(kFmtThreads) fmt_read_kernel(const uint8_t *luma, const float *regs, FmtGeom g, float *q_out, int32_t *word) {
  __shared__ __align__(16) uint8_t s_gf[768];
  __shared__ float s_ref[2][4 * kFmtMaxRefs], s_trk[4][kFmtMaxPairs][2], s_mid[4][kFmtMaxPairs], s_q[4 * kFmtMaxCells];
  __shared__ float s_con;
  __shared__ int s_read;
  __shared__ RsWork s_rs;
  const int f = blockIdx.x, tid = threadIdx.x;
  const uint8_t *px = luma + f * g.frame_stride;
  const float *reg = regs + (int64_t)f * g.reg_stride;
  load_gf(s_gf);
  // the samples: the line and the gap every 16 modules, the track's pairs, the word's cells
  const int nref = 4 * g.nrs, ntrk = 4 * g.npair * 2, nwrd = 4 * g.cells;
  for (int it = tid; it < 2 * nref + ntrk + nwrd; it += blockDim.x) {
    if (it < 2 * nref) {
      const int which = it / nref, k = it % nref, side = k / g.nrs, t = kReserve + 16 * (k % g.nrs);
      s_ref[which][k] = read_at(px, reg, g, side, t + 0.5f, which ? 3 + 2 / 2.0f : 1 + 2 / 2.0f);
    } else if (it < 2 * nref + ntrk) {
      const int k = it - 2 * nref, side = k / (2 * g.npair), pr = (k / 2) % g.npair, e = k & 1;
      s_trk[side][pr][e] = read_at(px, reg, g, side, kReserve + band_pair(2 * pr + e) * 2 + 2 / 2.0f, 5 + 2 / 2.0f);
    } else {
      const int k = it - 2 * nref - ntrk, side = k / g.cells, i = k % g.cells;
      s_q[k] = read_at(px, reg, g, side, kReserve + (band_pair(i) + 4) * 2 + 2 / 2.0f, 5 + 2 / 2.0f);
    }
  }
  __syncthreads();
  if (tid == 0) {   // the border's contrast, the sums in the reference's order
    float dark = 0, light = 0;
    for (int k = 0; k < nref; k++) { dark += s_ref[0][k]; light += s_ref[1][k]; }
    const float con = nref ? (light - dark) / nref : 0.0f;
    s_con = con;
    s_read = g.cells > 0 && nref > 0 && con >= 0.08f && g.npair >= 1;
  }
  for (int k = tid; k < 4 * g.npair; k += blockDim.x) {
    const int side = k / g.npair, pr = k % g.npair;
    float s = 0;
    s += s_trk[side][pr][0];
    s += s_trk[side][pr][1];
    s_mid[side][pr] = 0.5f * s;
  }
  __syncthreads();
  int32_t *out = word + 4 * f;
  if (!s_read) {
    if (tid < 4) out[tid] = 0;
    if (q_out) for (int k = tid; k < nwrd; k += blockDim.x) q_out[(int64_t)f * nwrd + k] = 0.0f;
    return;
  }
  for (int k = tid; k < nwrd; k += blockDim.x) {   // each cell against the track's pairs within 12 modules
    const int side = k / g.cells, i = k % g.cells, off = (band_pair(i) + 4) * 2;
    const int at = off / 8, lo = at - 3 < 0 ? 0 : at - 3, hi = at + 3 >= g.npair ? g.npair - 1 : at + 3;
    float m = 0;
    for (int j = lo; j <= hi; j++) m += s_mid[side][j];
    s_q[k] = s_q[k] - m / (hi - lo + 1);
  }
  __syncthreads();
  __shared__ float s_ref2;
  if (tid < 32) {   // the word's two means: lane 0 the dark side's sum, lane 1 the light side's, in index order
    float ref = 0;
    for (int it = 0; it < 4; it++) {
      float acc = 0;
      int cnt = 0;
      for (int i = 0; i < nwrd; i++) {
        const float v = s_q[i];
        const bool below = v < ref;
        if (tid < 2 && below == (tid == 0)) acc += v;
        cnt += below;
      }
      const float lo = __shfl_sync(0xffffffffu, acc, 0), hi = __shfl_sync(0xffffffffu, acc, 1);
      if (cnt < g.cells / 2 || nwrd - cnt < g.cells / 2) break;
      ref = 0.5f * (lo / cnt + hi / (nwrd - cnt));
    }
    if (tid == 0) s_ref2 = ref;
  }
  __syncthreads();
  const float ref = s_ref2, con = s_con;
  for (int k = tid; k < nwrd; k += blockDim.x) {
    const float s = (ref - s_q[k]) / con;
    s_q[k] = s > 0.5f ? 0.5f : s < -0.5f ? -0.5f : s;
    if (q_out) q_out[(int64_t)f * nwrd + k] = s_q[k];
  }
  __syncthreads();
  if (tid < 32) {
    const Gf gf{s_gf, s_gf + 512};
    int32_t ovf[3];
    fmt_decode_w(gf, s_q, g.cells, g.bytes, s_rs, ovf, tid);
    if (tid == 0) { out[0] = 1; out[1] = ovf[0]; out[2] = ovf[1]; out[3] = ovf[2]; }
  }
}

// The decode alone on given soft values: a warp a frame.
__global__ void __launch_bounds__(32) fmt_decode_kernel(const float *q, int cells, int bytes, int32_t *word) {
  __shared__ __align__(16) uint8_t s_gf[768];
  __shared__ float s_q[4 * kFmtMaxCells];
  __shared__ RsWork s_rs;
  const int f = blockIdx.x, lane = threadIdx.x;
  load_gf(s_gf);
  for (int k = lane; k < 4 * cells; k += 32) s_q[k] = q[(int64_t)f * 4 * cells + k];
  __syncwarp();
  const Gf gf{s_gf, s_gf + 512};
  int32_t ovf[3];
  fmt_decode_w(gf, s_q, cells, bytes, s_rs, ovf, lane);
  if (lane == 0) { word[4 * f] = 1; word[4 * f + 1] = ovf[0]; word[4 * f + 2] = ovf[1]; word[4 * f + 3] = ovf[2]; }
}

static std::mutex g_gf_mu;
static bool g_gf_done[64];

static cudaError_t gf_ready() {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_gf_mu);
  if (dev >= 0 && dev < 64 && g_gf_done[dev]) return cudaSuccess;
  uint8_t t[768] = {};
  int x = 1;
  for (int i = 0; i < 255; i++) {
    t[i] = (uint8_t)x;
    t[512 + x] = (uint8_t)i;
    x <<= 1;
    if (x & 256) x ^= 0x11d;
  }
  for (int i = 255; i < 512; i++) t[i] = t[i - 255];
  const cudaError_t e = cudaMemcpyToSymbol(g_gf, t, sizeof t);
  if (e == cudaSuccess && dev >= 0 && dev < 64) g_gf_done[dev] = true;
  return e;
}

// The word's geometry for a ring of span modules (fmt.c:6-20, layout.c:66-67).
static bool geometry(int span, FmtGeom *g) {
  if (span != 128 && span != 256 && span != 512) return false;
  g->W = span + 2 * kMargin;
  const int thin = (g->W - 2 * kReserve) / 2, wc = thin / 8 * 4;
  g->cells = wc >= 32 ? wc : 0;
  g->bytes = std::min(64, 4 * (g->cells / 8));
  g->npair = (thin + 1) / 2 / 2;
  g->nrs = (g->W - 2 * kReserve + 15) / 16;
  g->nn = layout_nodes(g->W, g->nodes);
  return g->cells > 0 && g->cells <= kFmtMaxCells && g->npair <= kFmtMaxPairs && g->nrs <= kFmtMaxRefs;
}

}  // namespace lizg

extern "C" {

int lizg_fmt_geometry(int span, int32_t *cells, int32_t *bytes) {
  lizg::FmtGeom g{};
  if (!lizg::geometry(span, &g)) return lizg::record_error(LIZG_E_ARG, "lizg_fmt_geometry: span must be 128, 256 or 512");
  if (cells) *cells = g.cells;
  if (bytes) *bytes = g.bytes;
  return 0;
}

int lizg_fmt_read_dev(int span, const uint8_t *d_luma, int w, int h, int64_t frame_stride, const float *d_reg, int reg_stride, int frames,
                      float *d_q, int32_t *d_word, void *stream) {
  using namespace lizg;
  FmtGeom g{};
  if (!geometry(span, &g)) return record_error(LIZG_E_ARG, "lizg_fmt_read_dev: span must be 128, 256 or 512");
  if (!d_luma || !d_reg || !d_word || frames < 1 || w < 2 || h < 2 || (frames > 1 && frame_stride < (int64_t)w * h))
    return record_error(LIZG_E_ARG, "lizg_fmt_read_dev: NULL buffer, empty batch or frame under 2 x 2");
  if (reg_stride < 9 + 2 * g.nn * g.nn) return record_error(LIZG_E_ARG, "lizg_fmt_read_dev: reg_stride under 9 + 2 nodes");
  g.iw = w; g.ih = h; g.reg_stride = reg_stride; g.frame_stride = frame_stride;
  int sms = 0;
  if (int rc = device_ready(&sms)) return rc;
  cudaError_t e = gf_ready();
  if (e == cudaSuccess) {
    fmt_read_kernel<<<frames, kFmtThreads, 0, static_cast<cudaStream_t>(stream)>>>(d_luma, d_reg, g, d_q, d_word);
    e = cudaGetLastError();
  }
  return e == cudaSuccess ? 0 : record_error(LIZG_E_CUDA, (std::string("lizg_fmt_read_dev: ") + cudaGetErrorString(e)).c_str());
}

int lizg_fmt_decode_dev(int span, const float *d_q, int frames, int32_t *d_word, void *stream) {
  using namespace lizg;
  FmtGeom g{};
  if (!geometry(span, &g)) return record_error(LIZG_E_ARG, "lizg_fmt_decode_dev: span must be 128, 256 or 512");
  if (!d_q || !d_word || frames < 1) return record_error(LIZG_E_ARG, "lizg_fmt_decode_dev: NULL buffer or empty batch");
  int sms = 0;
  if (int rc = device_ready(&sms)) return rc;
  cudaError_t e = gf_ready();
  if (e == cudaSuccess) {
    fmt_decode_kernel<<<frames, 32, 0, static_cast<cudaStream_t>(stream)>>>(d_q, g.cells, g.bytes, d_word);
    e = cudaGetLastError();
  }
  return e == cudaSuccess ? 0 : record_error(LIZG_E_CUDA, (std::string("lizg_fmt_decode_dev: ") + cudaGetErrorString(e)).c_str());
}

}  // extern "C"

// The registration's border nodes on sm_103a, a batch of frames a launch, one CTA a frame: every marked node of the
// border's lattice refined in the reference's order (liblizard/src/acquire.c:5044-5058: rings outward from the
// corners, rows within a ring), each by refine_node (acquire.c:1242-1374, its portable build): the prior from its
// measured neighbours (less the lens model's part, then the model's at the node), the border pattern's correlation
// over a 7 x 7 grid of half-module offsets read off one grid of samples, two passes of 3 x 3 searches at a quarter
// and an eighth of a module, a parabola each way; a node that correlates under 0.35 keeps its prior.
//
// Compiled with -fmad=false: every float operation rounds once, in the reference's order, so each node's
// displacement and score are the reference's bit for bit. The nodes depend on one another through their priors, so
// a frame's nodes run in order; within a node the samples, the 49 coarse correlations and each search step's
// candidates run across the CTA's threads, each correlation's sums in template order by one thread.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <algorithm>
#include <mutex>
#include <string>
#include <vector>
#include "format.h"
#include "lizard_gb300.h"
#include "lizg_internal.h"
#include "reg_dev.cuh"

namespace lizg {

constexpr int kMeshThreads = 256, kFB = 18, kGMax = 2 * kFB + 5, kMaxNodes = 40, kCorner = 12;
constexpr float kNodeNone = -2.0f, kNodeMin = 0.35f;

struct MeshArgs {
  int span, side, nn, no, w, h, hstride;
  int64_t fstride;
  float pos[kMaxNodes];
  const uint8_t *luma, *kind;
  const float *H;
  const double *lens;   // frames x kLensStride, or NULL
  const int *lens_on;   // frames: 0 where frame f has no model (NULL: every frame has lens's)
  const uint8_t *redo;  // frames x 4: the corners searched again (the anchors' registration); NULL: the border pass
  const int16_t *order;
  float *nodes;         // frames x nn^2 x (dx, dy, score, done)
};

__device__ __forceinline__ bool in_capture(int w, int h, float u, float v) { return u >= 0.5f && u <= w - 0.5f && v >= 0.5f && v <= h - 0.5f; }

__device__ bool node_inside(int w, int h, const float *H, int cx0, int cy0, const int *r, float pdx, float pdy, float ax, float bx, float ay, float by) {
  const float x0 = cx0 + r[0] + 0.5f + ax, x1 = cx0 + r[1] - 0.5f + bx, y0 = cy0 + r[2] + 0.5f + ay, y1 = cy0 + r[3] - 0.5f + by;
  for (int c = 0; c < 4; c++) {   // acquire.c:848-859
    const float x = c & 1 ? x1 : x0, y = c & 2 ? y1 : y0;
    float u, v;
    if (!(H[6] * x + H[7] * y + 1 > 0)) return false;
    project(H, x, y, &u, &v);
    if (!(u + pdx >= 1.5f && u + pdx <= w - 1.5f && v + pdy >= 1.5f && v + pdy <= h - 1.5f)) return false;
  }
  return true;
}

struct MeshShared {
  float G[kGMax * kGMax + 8], GM[kGMax * kGMax + 8];
  float tv[kFB * kFB];
  uint8_t kind[kFB * kFB];                 // the rect's cell kinds, staged for the template
  int at[kFB * kFB], pk[kFB * kFB];        // a template cell's place in the coarse grid, and in the rect (dy side + dx)
  float S[8][kFB * kFB];                   // the search step's candidates' samples at the template's cells
  uint8_t SI[8][kFB * kFB];                // and whether each is inside the capture
  float sc[49];
  float g[3][3], cand_ox[8], cand_oy[8];
  int have[3][3], cand_cell[8], ncand;
  int rect[4], cells, nmin, edge, ce, side, tall, GW, GH, ma, mb, stop;
  float pdx, pdy, jxx, jxy, jyx, jyy, st, stt, vt, best, box, boy, step;
  float h[9];
  double lens[kLensStride];
};

__global__ void __launch_bounds__(kMeshThreads) border_nodes_kernel(MeshArgs a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  MeshShared &m = *reinterpret_cast<MeshShared *>(smraw);
  float *nodes = reinterpret_cast<float *>(smraw + ((sizeof(MeshShared) + 15) & ~(size_t)15));   // nn^2 x 4
  const int f = blockIdx.x, tid = threadIdx.x, nn = a.nn;
  const uint8_t *px = a.luma + f * a.fstride;
  const bool have_lens = a.lens != nullptr && (!a.lens_on || a.lens_on[f]);
  if (tid < 9) m.h[tid] = a.H[(int64_t)f * a.hstride + tid];
  if (have_lens && tid < kLensStride) m.lens[tid] = a.lens[(int64_t)f * kLensStride + tid];
  for (int k = tid; k < nn * nn; k += blockDim.x) {
    const int i = k % nn, j = k / nn, corner = (i == 0 || i == nn - 1) && (j == 0 || j == nn - 1);
    const int c = j == 0 ? (i == 0 ? 0 : 1) : (i == 0 ? 3 : 2);   // corners in the layout's order
    const bool again = corner && a.redo && a.redo[(int64_t)f * 4 + c];
    nodes[4 * k] = 0; nodes[4 * k + 1] = 0; nodes[4 * k + 2] = 0; nodes[4 * k + 3] = corner && !again ? 1.0f : 0.0f;
  }
  __syncthreads();
  const float *H = m.h;
  for (int ko = 0; ko < a.no; ko++) {
    const int idx = a.redo ? ((ko >= 2 ? nn - 1 : 0) * nn + ((ko == 1 || ko == 2) ? nn - 1 : 0)) : a.order[ko];
    if (nodes[4 * idx + 3] != 0.0f) continue;   // uniform: read after the last barrier
    const int i = idx % nn, j = idx / nn, cx0 = (int)a.pos[i], cy0 = (int)a.pos[j];
    if (tid == 0) {
      int ex = (j == 0 || j == nn - 1) ? 6 : 2, ey = (i == 0 || i == nn - 1) ? 6 : 2;
      if (ex == 6 && ey == 6) { ex = kCorner - 1 < kFB - 3 ? kCorner - 1 : kFB - 3; ey = ex; }
      m.rect[0] = -ex < -cx0 ? -cx0 : -ex; m.rect[1] = ex + 1 > a.side - cx0 ? a.side - cx0 : ex + 1;
      m.rect[2] = -ey < -cy0 ? -cy0 : -ey; m.rect[3] = ey + 1 > a.side - cy0 ? a.side - cy0 : ey + 1;
      float pdx = 0, pdy = 0;
      int pn = 0;
      for (int dj = -1; dj <= 1; dj++)
        for (int di = -1; di <= 1; di++) {
          const int ii = i + di, jj = j + dj;
          if (ii < 0 || jj < 0 || ii >= nn || jj >= nn || nodes[4 * (jj * nn + ii) + 3] == 0.0f) continue;
          float rx = nodes[4 * (jj * nn + ii)], ry = nodes[4 * (jj * nn + ii) + 1];
          if (have_lens) { float u, v, mx, my; project(H, a.pos[ii], a.pos[jj], &u, &v); lens_at(m.lens, u, v, &mx, &my); rx -= mx; ry -= my; }
          pdx += rx; pdy += ry; pn++;
        }
      if (pn) { pdx /= pn; pdy /= pn; }
      if (have_lens) { float u, v, mx, my; project(H, a.pos[i], a.pos[j], &u, &v); lens_at(m.lens, u, v, &mx, &my); pdx += mx; pdy += my; }
      m.pdx = pdx; m.pdy = pdy;
      m.edge = !node_inside(a.w, a.h, H, cx0, cy0, m.rect, pdx, pdy, -1.5f, 1.5f, -1.5f, 1.5f);
      const float mcx = cx0 + 0.5f, mcy = cy0 + 0.5f;
      float ppx, ppy, ax, ay, bx, by;
      project(H, mcx, mcy, &ppx, &ppy); project(H, mcx + 1, mcy, &ax, &ay); project(H, mcx, mcy + 1, &bx, &by);
      m.jxx = ax - ppx; m.jxy = ay - ppy; m.jyx = bx - ppx; m.jyy = by - ppy;
      m.side = m.rect[1] - m.rect[0]; m.tall = m.rect[3] - m.rect[2];
      m.GW = 2 * m.side + 5; m.GH = 2 * m.tall + 5;
    }
    __syncthreads();
    for (int t = tid; t < m.side * m.tall; t += blockDim.x)   // the rect's kinds, read once across the CTA
      m.kind[t] = a.kind[(cy0 + m.rect[2] + t / m.side) * a.side + cx0 + m.rect[0] + t % m.side];
    __syncthreads();
    if (tid == 0) {
      // the template: the border's own cells about the node (not the picture's, not the word's), in row order
      float st = 0, stt = 0;
      int cells = 0;
      for (int dy = 0; dy < m.tall; dy++)
        for (int dx = 0; dx < m.side; dx++) {
          const int kind = m.kind[dy * m.side + dx];
          if (kind == 0 || (kind & 8)) continue;
          m.tv[cells] = (kind & 3) == 2 ? -1.0f : 1.0f;
          m.at[cells] = (2 * dy + 3) * m.GW + 2 * dx + 3;
          m.pk[cells] = dy * m.side + dx;
          st += m.tv[cells]; stt += m.tv[cells] * m.tv[cells]; cells++;
        }
      m.cells = cells; m.st = st; m.stt = stt;
      m.vt = stt - st * st / cells;
      m.nmin = (cells + 1) / 2;
    }
    __syncthreads();
    // the coarse grid: every half-module point the 49 offsets read, through H and the prior
    const int lo = m.rect[0], ylo = m.rect[2], GW = m.GW, GH = m.GH, cells = m.cells;
    const float pdx = m.pdx, pdy = m.pdy;
    for (int t = tid; t < GW * GH; t += blockDim.x) {
      const int gy = t / GW, gx = t - gy * GW;
      const float my = (float)(2 * (cy0 + ylo) + gy - 2) * 0.5f, mx = (float)(2 * (cx0 + lo) + gx - 2) * 0.5f;
      float u, v;
      project(H, mx, my, &u, &v);
      m.G[t] = sample(px, a.w, a.h, u + pdx, v + pdy);
      m.GM[t] = !m.edge || in_capture(a.w, a.h, u + pdx, v + pdy) ? 1.0f : 0.0f;
    }
    if (tid < 4) { m.G[GW * GH + tid] = 0; m.GM[GW * GH + tid] = 0; }
    __syncthreads();
    if (tid < 49) {   // offset (a, b) = (tid % 7 - 3, tid / 7 - 3), its sums in template order
      const int b = tid / 7 - 3, aa = tid % 7 - 3;
      const float *g0 = m.G + b * GW + aa, *m0 = m.GM + b * GW + aa;
      float ss = 0, sss = 0, sts = 0, sn = 0;
      for (int k = 0; k < cells; k++) { const float v = g0[m.at[k]]; ss += v; sss += v * v; sts += m.tv[k] * v; }
      if (m.edge) for (int k = 0; k < cells; k++) sn += m0[m.at[k]];
      const float vs = sss - ss * ss / cells;
      m.sc[tid] = m.edge && sn < m.nmin ? kNodeNone : m.vt <= 0 || vs <= 1e-9f ? 0 : (sts - m.st * ss / cells) / sqrtf(m.vt * vs);
    }
    __syncthreads();
    if (tid == 0) {
      float best = kNodeNone, box = 0, boy = 0;
      for (int k = 0; k < 49; k++) if (m.sc[k] > best) { best = m.sc[k]; box = (k % 7 - 3) * 0.5f; boy = (k / 7 - 3) * 0.5f; }
      m.best = best; m.box = box; m.boy = boy;
      for (int b2 = 0; b2 < 3; b2++) for (int a2 = 0; a2 < 3; a2++) m.have[b2][a2] = 0;
      m.g[1][1] = best; m.have[1][1] = 1; m.ma = m.mb = 1; m.step = 0.25f;
    }
    __syncthreads();
    for (int pass = 0; pass < 2; pass++) {
      for (int move = 0; move < 8; move++) {
        if (tid == 0) {   // centre the 3 x 3 on the last move, then list the points not yet read
          if (m.ma != 1 || m.mb != 1) {
            float ng[3][3];
            int nh[3][3];
            for (int b2 = 0; b2 < 3; b2++)
              for (int a2 = 0; a2 < 3; a2++) {
                const int sb = b2 + m.mb - 1, sa = a2 + m.ma - 1;
                const bool in = sb >= 0 && sb < 3 && sa >= 0 && sa < 3;
                nh[b2][a2] = in && m.have[sb][sa];
                ng[b2][a2] = in ? m.g[sb][sa] : 0;
              }
            for (int b2 = 0; b2 < 3; b2++) for (int a2 = 0; a2 < 3; a2++) { m.g[b2][a2] = ng[b2][a2]; m.have[b2][a2] = nh[b2][a2]; }
            m.ma = m.mb = 1;
          }
          m.ce = !node_inside(a.w, a.h, H, cx0, cy0, m.rect, pdx, pdy, m.box - m.step, m.box + m.step, m.boy - m.step, m.boy + m.step);
          int c = 0;
          for (int b2 = -1; b2 <= 1; b2++)
            for (int a2 = -1; a2 <= 1; a2++)
              if (!m.have[b2 + 1][a2 + 1]) { m.cand_ox[c] = m.box + a2 * m.step; m.cand_oy[c] = m.boy + b2 * m.step; m.cand_cell[c] = (b2 + 1) * 3 + a2 + 1; c++; }
          m.ncand = c;
        }
        __syncthreads();
        const int ncand = m.ncand;
        for (int t = tid; t < ncand * cells; t += blockDim.x) {   // the candidates' samples at the template's cells
          const int c = t / cells, k = t - c * cells, dy = m.pk[k] / m.side, dx = m.pk[k] - dy * m.side;
          const float my = cy0 + (m.rect[2] + dy) + 0.5f + m.cand_oy[c], mx = cx0 + (m.rect[0] + dx) + 0.5f + m.cand_ox[c];
          float u, v;
          project(H, mx, my, &u, &v);
          m.S[c][k] = sample(px, a.w, a.h, u + pdx, v + pdy);
          m.SI[c][k] = in_capture(a.w, a.h, u + pdx, v + pdy);
        }
        __syncthreads();
        if (tid < ncand) {   // each candidate's correlation, its sums in template order (node_ncc)
          float st = 0, ss = 0, stt = 0, sss = 0, sts = 0;
          int nin = 0;
          for (int k = 0; k < cells; k++) {
            if (m.ce) nin += m.SI[tid][k];
            const float tt = m.tv[k], s = m.S[tid][k];
            st += tt; ss += s; stt += tt * tt; sss += s * s; sts += tt * s;
          }
          float r;
          if (m.ce && nin < m.nmin) r = kNodeNone;
          else {
            const float vt = stt - st * st / cells, vs = sss - ss * ss / cells;
            r = vt <= 0 || vs <= 1e-9f ? 0 : (sts - st * ss / cells) / sqrtf(vt * vs);
          }
          const int cc = m.cand_cell[tid];
          m.g[cc / 3][cc % 3] = r;
          m.have[cc / 3][cc % 3] = 1;
        }
        __syncthreads();
        if (tid == 0) {
          int ba = 1, bb = 1;
          for (int b2 = 0; b2 < 3; b2++) for (int a2 = 0; a2 < 3; a2++) if (m.g[b2][a2] > m.g[bb][ba]) { ba = a2; bb = b2; }
          m.stop = ba == 1 && bb == 1;
          if (!m.stop) { m.box += (ba - 1) * m.step; m.boy += (bb - 1) * m.step; m.ma = ba; m.mb = bb; }
        }
        __syncthreads();
        if (m.stop) break;
      }
      if (tid == 0) {
        if (pass == 0) {
          const float c = m.g[m.mb][m.ma];
          for (int b2 = 0; b2 < 3; b2++) for (int a2 = 0; a2 < 3; a2++) m.have[b2][a2] = 0;
          m.g[1][1] = c; m.have[1][1] = 1; m.ma = m.mb = 1;
        }
        m.step *= 0.5f;
      }
      __syncthreads();
    }
    if (tid == 0) {   // a parabola each way, then the node (its prior where the pattern did not hold)
      const float best = m.g[1][1];
      float box = m.box, boy = m.boy;
      const float dxx = m.g[1][0] - 2 * m.g[1][1] + m.g[1][2], dyy = m.g[0][1] - 2 * m.g[1][1] + m.g[2][1];
      if (dxx < -1e-6f && m.g[1][0] > kNodeNone && m.g[1][2] > kNodeNone) box += 0.125f * 0.5f * (m.g[1][0] - m.g[1][2]) / dxx;
      if (dyy < -1e-6f && m.g[0][1] > kNodeNone && m.g[2][1] > kNodeNone) boy += 0.125f * 0.5f * (m.g[0][1] - m.g[2][1]) / dyy;
      float *nd = nodes + 4 * idx;
      nd[3] = 1.0f; nd[2] = best;
      if (best < kNodeMin) { nd[0] = pdx; nd[1] = pdy; }
      else { nd[0] = pdx + box * m.jxx + boy * m.jyx; nd[1] = pdy + box * m.jxy + boy * m.jyy; }
    }
    __syncthreads();
  }
  float *out = a.nodes + (int64_t)f * nn * nn * 4;
  for (int k = tid; k < 4 * nn * nn; k += blockDim.x) out[k] = nodes[k];
}

struct MeshSpan {
  uint8_t *kind = nullptr;
  int16_t *order = nullptr;
  int no = 0, nn = 0;
  float pos[kMaxNodes];
};

static std::mutex g_mesh_mu;
static MeshSpan g_mesh[64][3];   // a device's spans 128, 256, 512

// The span's layout on the device: its cell kinds (the word's cells flagged) and the marked nodes' order, made once.
static cudaError_t mesh_ready(int span, MeshSpan **out) {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  const int si = span == 128 ? 0 : span == 256 ? 1 : 2;
  std::lock_guard<std::mutex> lk(g_mesh_mu);
  MeshSpan &ms = g_mesh[dev][si];
  if (!ms.kind) {
    const int side = span + 2 * kMargin;
    std::vector<uint8_t> kind;
    layout_kind(span, 0, 0, kind);
    const int nn = layout_nodes(side, ms.pos);
    std::vector<int16_t> order;
    for (int ring = 0; ring <= nn; ring++)
      for (int j = 0; j < nn; j++)
        for (int i = 0; i < nn; i++) {
          const bool ex = i == 0 || i == nn - 1, ey = j == 0 || j == nn - 1;
          if (!((ex || ey) && !(ex && ey))) continue;
          if (std::min(i, nn - 1 - i) + std::min(j, nn - 1 - j) == ring) order.push_back((int16_t)(j * nn + i));
        }
    uint8_t *dk = nullptr;
    int16_t *dord = nullptr;
    cudaError_t e = cudaMalloc(&dk, kind.size());
    if (e == cudaSuccess) e = cudaMalloc(&dord, order.size() * sizeof(int16_t));
    if (e == cudaSuccess) e = cudaMemcpy(dk, kind.data(), kind.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dord, order.data(), order.size() * sizeof(int16_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { cudaFree(dk); cudaFree(dord); return e; }
    ms.kind = dk; ms.order = dord; ms.no = (int)order.size(); ms.nn = nn;
  }
  *out = &ms;
  return cudaSuccess;
}

cudaError_t border_corners_launch(int span, const uint8_t *d_rim, int w, int h, int64_t frame_stride, const float *d_H, int h_stride,
                                  const double *d_lens, const int *d_lens_on, const uint8_t *d_redo, int frames, float *d_nodes, cudaStream_t st) {
  MeshSpan *ms = nullptr;
  cudaError_t e = mesh_ready(span, &ms);
  if (e != cudaSuccess) return e;
  MeshArgs a{};
  a.span = span; a.side = span + 2 * kMargin; a.nn = ms->nn; a.no = 4; a.w = w; a.h = h; a.hstride = h_stride;
  a.fstride = frame_stride;
  for (int k = 0; k < kMaxNodes; k++) a.pos[k] = k < ms->nn ? ms->pos[k] : 0.0f;
  a.luma = d_rim; a.kind = ms->kind; a.H = d_H; a.lens = d_lens; a.lens_on = d_lens_on; a.redo = d_redo; a.order = ms->order; a.nodes = d_nodes;
  const size_t smem = ((sizeof(MeshShared) + 15) & ~(size_t)15) + (size_t)ms->nn * ms->nn * 4 * sizeof(float);
  if ((e = cudaFuncSetAttribute(border_nodes_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess) return e;
  border_nodes_kernel<<<frames, kMeshThreads, smem, st>>>(a);
  return cudaGetLastError();
}

}  // namespace lizg

extern "C" int lizg_border_nodes_dev(int span, const uint8_t *d_luma, int w, int h, int64_t frame_stride, const float *d_H, int h_stride,
                                     const double *d_lens, int frames, float *d_nodes, void *stream) {
  using namespace lizg;
  if (span != 128 && span != 256 && span != 512) return record_error(LIZG_E_ARG, "lizg_border_nodes_dev: span must be 128, 256 or 512");
  if (!d_luma || !d_H || !d_nodes || frames < 1 || w < 2 || h < 2 || h_stride < 9 || (frames > 1 && frame_stride < (int64_t)w * h))
    return record_error(LIZG_E_ARG, "lizg_border_nodes_dev: NULL buffer, empty batch, frame under 2 x 2 or H stride under 9");
  int sms = 0;
  if (int rc = device_ready(&sms)) return rc;
  MeshSpan *ms = nullptr;
  cudaError_t e = mesh_ready(span, &ms);
  if (e == cudaSuccess) {
    MeshArgs a{};
    a.span = span; a.side = span + 2 * kMargin; a.nn = ms->nn; a.no = ms->no; a.w = w; a.h = h; a.hstride = h_stride;
    a.fstride = frame_stride;
    for (int k = 0; k < kMaxNodes; k++) a.pos[k] = k < ms->nn ? ms->pos[k] : 0.0f;
    a.luma = d_luma; a.kind = ms->kind; a.H = d_H; a.lens = d_lens; a.order = ms->order; a.nodes = d_nodes;
    const size_t smem = ((sizeof(MeshShared) + 15) & ~(size_t)15) + (size_t)ms->nn * ms->nn * 4 * sizeof(float);
    e = cudaFuncSetAttribute(border_nodes_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) {
      border_nodes_kernel<<<frames, kMeshThreads, smem, static_cast<cudaStream_t>(stream)>>>(a);
      e = cudaGetLastError();
    }
  }
  return e == cudaSuccess ? 0 : record_error(LIZG_E_CUDA, (std::string("lizg_border_nodes_dev: ") + cudaGetErrorString(e)).c_str());
}

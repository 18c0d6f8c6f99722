// Row (c) of the hot path on sm_103a: the pilots' grid-shift fit, the soft QPSK demap to int8 LLRs, and the
// per-block estimate / pilot reading / decline gate. Compiled with -fmad=false: every float and double operation here
// rounds once, in the reference's order, so from the same spectrum these kernels give the reference's soft values
// bit for bit (liblizard/src/lizard_phy.c:280-329 pilot_align, :1320-1332 sub_scale, :1411-1451 the x86-64 soft4,
// :1775-1818 the block estimate, pilots and decline).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <cooperative_groups.h>
#include "lizg_internal.h"

namespace cg = cooperative_groups;

namespace lizg {

// Coefficient i (spectra are in pos order) turned back by the grid shift (dx, dy): the turn's index in float,
// nearest-even, mod 4096, and the rotation by the table's cos / sin, as liblizard/src/lizard_phy.c:214-218 computes them.
__device__ __forceinline__ float2 turned(const FmtDev &fd, const float2 *spec, int i, float dx, float dy) {
  const float2 z = spec[i];
  const float uu = (float)fd.uv[2 * i], vv = (float)fd.uv[2 * i + 1];
  const float t = (uu * dx + vv * dy) * fd.turn_scale;
  const unsigned k = (unsigned)__float2int_rn(t) & (kTurnsDev - 1);
  const float2 cs = fd.rot[k];
  return make_float2(z.x * cs.x + z.y * cs.y, z.y * cs.x - z.x * cs.y);
}

// A cluster of kPilotCtas CTAs a frame: CTA r works out the six products of pilots [r chunk, (r + 1) chunk) into its
// shared memory; then six threads of CTA 0 add one sum each in pilot order, reading the cluster's shared memory, so
// the double sums are the reference's (liblizard/src/lizard_phy.c:283-317), and CTA 0's thread 0 solves for the
// shift and hands it to every CTA for the second fit. Writes align[3 f ..] = dx, dy, and 1 where the shift is turned
// back. (The products are spread over the cluster's SMs because double arithmetic is slow on one SM.)
constexpr int kPilotCtas = 8;

// Frame f's fit by the calling cluster. tm: this CTA's dynamic shared memory (chunk x 6 doubles at least).
__device__ __forceinline__ void pilot_align_frame(const FmtDev &fd, const float2 *spec, int64_t spec_stride, float *align, int f, double *tm) {
  __shared__ double sums[6], dxy[2];
  __shared__ int give_up;
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank(), used = fd.npilot;
  const int chunk = (used + kPilotCtas - 1) / kPilotCtas, p0 = rank * chunk, p1 = min(used, p0 + chunk);
  const float2 *sp = spec + f * spec_stride;
  const double k = 2.0 * 3.14159265358979323846 / fd.n;
  if (threadIdx.x == 0) { dxy[0] = dxy[1] = 0; give_up = 0; }
  cl.sync();
  for (int it = 0; it < 2; it++) {
    const double dx = dxy[0], dy = dxy[1];
    for (int pi = p0 + (int)threadIdx.x; pi < p1; pi += blockDim.x) {
      const int i = fd.pilot_coef[pi], w = fd.pilot_white[pi];
      const float2 y = turned(fd, sp, i, (float)dx, (float)dy);
      const double xr = (w & 1) ? -1.0 : 1.0, xi = (w & 2) ? -1.0 : 1.0;
      const double zr = (double)y.x * xr + (double)y.y * xi, zi = (double)y.y * xr - (double)y.x * xi;
      const double cu = k * zr * fd.uv[2 * i], cv = k * zr * fd.uv[2 * i + 1];
      double *t = tm + 6 * (pi - p0);
      t[0] = cu * cu; t[1] = cu * cv; t[2] = cv * cv; t[3] = cu * zi; t[4] = cv * zi; t[5] = zi * zi;
    }
    cl.sync();
    if (rank == 0) {
      if (threadIdx.x < 6) {
        // in pilot order, CTA by CTA; the loads of eight terms issued ahead of their adds
        double acc = 0;
        for (int r = 0; r < kPilotCtas; r++) {
          const double *rt = cl.map_shared_rank(tm, r) + threadIdx.x;
          const int cnt = max(0, min(used, (r + 1) * chunk) - r * chunk);
          int q = 0;
          for (; q + 8 <= cnt; q += 8) {
            double v[8];
#pragma unroll
            for (int e = 0; e < 8; e++) v[e] = rt[6 * (q + e)];
#pragma unroll
            for (int e = 0; e < 8; e++) acc += v[e];
          }
          for (; q < cnt; q++) acc += rt[6 * q];
        }
        sums[threadIdx.x] = acc;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        const double a = sums[0], b = sums[1], c = sums[2], p = sums[3], q = sums[4];
        const double det = a * c - b * b;
        int gu = 0;
        double nx = dx, ny = dy;
        if (used < 8 || !(det > 0)) gu = 1;
        else { nx = dx + (p * c - q * b) / det; ny = dy + (a * q - b * p) / det; }
        for (int r = 0; r < kPilotCtas; r++) {
          double *rd = cl.map_shared_rank(dxy, r);
          rd[0] = nx; rd[1] = ny;
          *cl.map_shared_rank(&give_up, r) = gu;
        }
      }
    }
    cl.sync();
    if (give_up) break;
  }
  if (rank != 0 || threadIdx.x != 0) return;
  float d0 = 0, d1 = 0;
  if (!give_up) {
    const double a = sums[0], b = sums[1], c = sums[2], p = sums[3], q = sums[4], yy = sums[5], dx = dxy[0], dy = dxy[1];
    const double det = a * c - b * b, ex = (p * c - q * b) / det, ey = (a * q - b * p) / det;
    const double s2 = (yy - ex * p - ey * q) / (used - 2);
    const double chi = s2 > 0 ? (dx * dx * a + 2 * dx * dy * b + dy * dy * c) / s2 : 0;
    if (chi > 13.8 && dx == dx && dy == dy) { d0 = (float)dx; d1 = (float)dy; }
  }
  align[3 * f] = d0; align[3 * f + 1] = d1;
  align[3 * f + 2] = (used > 0 && (d0 != 0 || d1 != 0)) ? 1.0f : 0.0f;
}

__global__ void __cluster_dims__(kPilotCtas, 1, 1) __launch_bounds__(128) pilot_align_kernel(FmtDev fd, const float2 *spec, int64_t spec_stride,
                                                                                           float *align) {
  extern __shared__ double tm[];              // chunk x 6: this CTA's pilots' products
  pilot_align_frame(fd, spec, spec_stride, align, blockIdx.x / kPilotCtas, tm);
}

// ten Brink's J (liblizard/src/lizard_phy.c:73-75)
__device__ __forceinline__ double axis_info(double g) { return g > 0 ? pow(1 - pow(2.0, -0.3073 * pow(2 * sqrt(g), 1.7870)), 1.1064) : 0; }

// Four lanes a sub-channel, 64 sub-channels a CTA. Lane q of a group sums the moments of coefficients q, q + 4, ...
// in order (the reference's four float chains) and the chains are added (c0 + c1) + (c2 + c3); one thread a
// sub-channel then works out the scale in double (so a warp's double work serves 32 sub-channels); the soft values
// are each axis times 8 k, NaN to 0, clamped to +-80, rounded half to even.
constexpr int kDemapBatch = 8;   // 320 / 4 = 80 coefficients a lane, 10 batches
static_assert(kSubDev % (4 * kDemapBatch) == 0, "whole batches");

__device__ __forceinline__ void demap_block(const FmtDev &fd, const float2 *spec, int64_t spec_stride, const float *align, int8_t *llrf,
                                            double *sub_est, float *sub_rms, int blk) {
  __shared__ float s_m[64][2], s_k8[64];
  const int grp = threadIdx.x >> 2, qd = threadIdx.x & 3, gid = blk * 64 + grp;
  const int f = gid / fd.subch, j = gid - f * fd.subch;
  const bool live = f < fd.frames;
  const float2 *sp = spec + (live ? f : 0) * spec_stride;
  const bool turn = live && align[3 * f + 2] != 0.0f;
  const float dx = live ? align[3 * f] : 0, dy = live ? align[3 * f + 1] : 0;
  float m2 = 0, m4 = 0;
  if (live) {
    // eight of the lane's coefficients loaded at a time (independent loads in flight), then summed in order
    for (int s0 = qd; s0 < kSubDev; s0 += 4 * kDemapBatch) {
      float2 y[kDemapBatch];
#pragma unroll
      for (int b = 0; b < kDemapBatch; b++) {
        const int i = j * kSubDev + s0 + 4 * b;
        y[b] = turn ? turned(fd, sp, i, dx, dy) : sp[i];
      }
#pragma unroll
      for (int b = 0; b < kDemapBatch; b++) {
        const float e = y[b].x * y[b].x + y[b].y * y[b].y;
        m2 = m2 + e; m4 = m4 + e * e;
      }
    }
  }
  // (c0 + c1) + (c2 + c3)
  const float o2 = __shfl_down_sync(0xffffffffu, m2, 1), o4 = __shfl_down_sync(0xffffffffu, m4, 1);
  const float p2 = m2 + o2, p4 = m4 + o4;
  const float r2 = __shfl_down_sync(0xffffffffu, p2, 2), r4 = __shfl_down_sync(0xffffffffu, p4, 2);
  if (qd == 0) { s_m[grp][0] = p2 + r2; s_m[grp][1] = p4 + r4; }
  __syncthreads();
  if (threadIdx.x < 64) {
    const int g2 = blk * 64 + threadIdx.x, f2 = g2 / fd.subch, j2 = g2 - f2 * fd.subch;
    float k8 = 0;
    if (f2 < fd.frames) {
      const double M2 = (double)s_m[threadIdx.x][0] / kSubDev, M4 = (double)s_m[threadIdx.x][1] / kSubDev;
      sub_rms[f2 * fd.subch + j2] = M2 > 0 ? (float)sqrt(M2 / 2) : 0;
      double a2 = 2 * M2 * M2 - M4;
      a2 = a2 > 0 ? sqrt(a2) : 0;
      double nv = M2 - a2;
      if (nv < 0.02 * M2) nv = 0.02 * M2;
      sub_est[f2 * fd.subch + j2] = axis_info(a2 / nv);
      const float kk = (float)(0.7 * 2 * sqrt(2 * a2) / nv);
      k8 = 8 * kk;
    }
    s_k8[threadIdx.x] = k8;
  }
  __syncthreads();
  if (!live) return;
  const float k8 = s_k8[grp];
  int8_t *out = llrf + (int64_t)f * fd.subch * 2 * kSubDev + 2 * j * kSubDev;
  for (int s0 = qd; s0 < kSubDev; s0 += 4 * kDemapBatch) {
    float2 y[kDemapBatch];
#pragma unroll
    for (int b = 0; b < kDemapBatch; b++) {
      const int i = j * kSubDev + s0 + 4 * b;
      y[b] = turn ? turned(fd, sp, i, dx, dy) : sp[i];
    }
#pragma unroll
    for (int b = 0; b < kDemapBatch; b++) {
      float x = k8 * y[b].x, z = k8 * y[b].y;
      x = x != x ? 0.0f : fminf(fmaxf(x, -80.0f), 80.0f);
      z = z != z ? 0.0f : fminf(fmaxf(z, -80.0f), 80.0f);
      char2 v;
      v.x = (signed char)__float2int_rn(x);
      v.y = (signed char)__float2int_rn(z);
      *reinterpret_cast<char2 *>(out + 2 * (s0 + 4 * b)) = v;
    }
  }
}

__global__ void __launch_bounds__(256) demap_kernel(FmtDev fd, const float2 *spec, int64_t spec_stride, const float *align,
                                                    int8_t *llrf, double *sub_est, float *sub_rms) {
  demap_block(fd, spec, spec_stride, align, llrf, sub_est, sub_rms, blockIdx.x);
}

// One thread a block: its estimate (its sub-channels' information weighted by the slots it holds there, in double, in
// order), its pilot reading (the tail's axis values against the whitening in units of their sub-channel's rms, in
// double, in order; NaN where none was read) and the decline gate (est < 0.2 k / nt in float): decl[f blocks + b] = 1.
constexpr int kBlocksThreads = 128;
__device__ __forceinline__ void blocks_block(const FmtDev &fd, const float2 *spec, int64_t spec_stride, const float *align,
                                             const double *sub_est, const float *sub_rms, float *est, float *pilot, uint8_t *decl, int blk) {
  const int g = blk * kBlocksThreads + threadIdx.x;
  if (g >= fd.frames * fd.blocks) return;
  const int f = g / fd.blocks, b = g - f * fd.blocks;
  const int t = fd.block_tier[b], nb = fd.tier_slots[t], s0 = fd.block_slot[b], nt = fd.tier_nt[t];
  const double *se = sub_est + f * fd.subch;
  const float *sr = sub_rms + f * fd.subch;
  double info = 0;
  for (int j = s0 / (2 * kSubDev); j * 2 * kSubDev < s0 + nb; j++) {
    const int lo = max(s0, 2 * kSubDev * j), hi = min(s0 + nb, 2 * kSubDev * (j + 1));
    info += se[j] * (hi - lo);
  }
  const float e = (float)(info / nb);
  est[g] = e;
  float pv = __int_as_float(0x7fc00000);   // NaN: no pilot read
  if (nt < nb) {
    const float2 *sp = spec + f * spec_stride;
    const bool turn = align[3 * f + 2] != 0.0f;
    const float dx = align[3 * f], dy = align[3 * f + 1];
    double cs = 0;
    int got = 0;
    for (int i = nt; i < nb; i++) {
      const int gs = s0 + i, ci = gs / 2;
      const float rms = sr[gs / (2 * kSubDev)];
      if (!(rms > 0)) continue;
      const float2 y = turn ? turned(fd, sp, ci, dx, dy) : sp[ci];
      const float yv = (i & 1) ? y.y : y.x;
      cs += (fd.white[gs] ? -1.0 : 1.0) * yv / rms;
      got++;
    }
    if (got) pv = (float)(cs / (nb - nt));
  }
  pilot[g] = pv;
  decl[g] = e < 0.2f * (float)fd.tier_k[t] / (float)nt;
}

__global__ void __launch_bounds__(kBlocksThreads) blocks_kernel(FmtDev fd, const float2 *spec, int64_t spec_stride, const float *align,
                                                                const double *sub_est, const float *sub_rms, float *est, float *pilot,
                                                                uint8_t *decl) {
  blocks_block(fd, spec, spec_stride, align, sub_est, sub_rms, est, pilot, decl, blockIdx.x);
}

// The three stages over several formats' batches, one launch each: format k's frames (clusters), demap CTAs and block
// CTAs at [pf[k], pf[k + 1]), [df[k], df[k + 1]) and [bf[k], bf[k + 1]).
struct DemapMix {
  DemapSeg seg[kDemapMixSegs];
  int pf[kDemapMixSegs + 1], df[kDemapMixSegs + 1], bf[kDemapMixSegs + 1];
  int nseg;
};
static_assert(sizeof(DemapMix) <= 32000, "the mixed launches' arguments fit a launch");
__device__ __forceinline__ int seg_at(const int *first, int nseg, int b) {
  int k = 0;
  while (k < nseg - 1 && b >= first[k + 1]) k++;
  return k;
}

__global__ void __cluster_dims__(kPilotCtas, 1, 1) __launch_bounds__(128) pilot_align_mixed_kernel(const __grid_constant__ DemapMix m) {
  extern __shared__ double tm[];
  const int c = blockIdx.x / kPilotCtas, k = seg_at(m.pf, m.nseg, c);
  const DemapSeg &g = m.seg[k];
  pilot_align_frame(g.fd, g.spec, g.stride, g.align, c - m.pf[k], tm);
}

__global__ void __launch_bounds__(256) demap_mixed_kernel(const __grid_constant__ DemapMix m) {
  const int k = seg_at(m.df, m.nseg, blockIdx.x);
  const DemapSeg &g = m.seg[k];
  demap_block(g.fd, g.spec, g.stride, g.align, g.llrf, g.sub_est, g.sub_rms, blockIdx.x - m.df[k]);
}

__global__ void __launch_bounds__(kBlocksThreads) blocks_mixed_kernel(const __grid_constant__ DemapMix m) {
  const int k = seg_at(m.bf, m.nseg, blockIdx.x);
  const DemapSeg &g = m.seg[k];
  blocks_block(g.fd, g.spec, g.stride, g.align, g.sub_est, g.sub_rms, g.est, g.pilot, g.decl, blockIdx.x - m.bf[k]);
}

cudaError_t demap_mixed_launch(const DemapSeg *a, int count, cudaStream_t st) {
  if (count < 1 || count > kDemapMixSegs) return cudaErrorInvalidValue;
  DemapMix m{};
  m.nseg = count;
  int psm = 8;
  for (int k = 0; k < count; k++) {
    const FmtDev &fd = a[k].fd;
    m.seg[k] = a[k];
    const int chunk = (fd.npilot + kPilotCtas - 1) / kPilotCtas, bytes = 6 * (chunk > 0 ? chunk : 1) * (int)sizeof(double);
    psm = bytes > psm ? bytes : psm;
    m.pf[k + 1] = m.pf[k] + fd.frames;
    m.df[k + 1] = m.df[k] + (fd.frames * fd.subch + 63) / 64;
    m.bf[k + 1] = m.bf[k] + (fd.frames * fd.blocks + kBlocksThreads - 1) / kBlocksThreads;
  }
  if (psm > 48 * 1024) return cudaErrorInvalidValue;
  pilot_align_mixed_kernel<<<m.pf[count] * kPilotCtas, 128, psm, st>>>(m);
  demap_mixed_kernel<<<m.df[count], 256, 0, st>>>(m);
  blocks_mixed_kernel<<<m.bf[count], kBlocksThreads, 0, st>>>(m);
  return cudaGetLastError();
}

cudaError_t demap_launch(const FmtDev &fd, const float2 *spec, int64_t spec_stride, float *align, int8_t *llrf,
                         double *sub_est, float *sub_rms, float *est, float *pilot, uint8_t *decl, cudaStream_t st) {
  const int chunk = (fd.npilot + kPilotCtas - 1) / kPilotCtas;
  const int psm = 6 * (chunk > 0 ? chunk : 1) * (int)sizeof(double);
  if (psm > 48 * 1024) return cudaErrorInvalidValue;
  pilot_align_kernel<<<fd.frames * kPilotCtas, 128, psm, st>>>(fd, spec, spec_stride, align);
  const int groups = fd.frames * fd.subch;
  demap_kernel<<<(groups + 63) / 64, 256, 0, st>>>(fd, spec, spec_stride, align, llrf, sub_est, sub_rms);
  const int nbk = fd.frames * fd.blocks;
  blocks_kernel<<<(nbk + kBlocksThreads - 1) / kBlocksThreads, kBlocksThreads, 0, st>>>(fd, spec, spec_stride, align, sub_est, sub_rms, est,
                                                                                       pilot, decl);
  return cudaGetLastError();
}

}  // namespace lizg

// Row (b) of the hot path on sm_103a: the anchors' erase, the detrend projections and the 2D mixed-radix FFT of the
// n x n picture grid, restated from the reference's decode (liblizard/src/lizard_phy.c:1596-1716) for the GPU.
//
// Four kernels a batch (five when the samples come straight from captured frames):
//   hole_rhs_kernel   a CTA takes a band of the frame's every-eighth-sample rows: the shading fit's right-hand side
//                     over the samples outside the anchors' squares, one partial sum a band (6 doubles);
//   cell_table_kernel (captured frames only) each picture row's homography terms and the mesh displacement line of
//                     each mesh cell along it, so the column pass reads them instead of walking the mesh per sample;
//   fft_cols_kernel   a CTA takes 2L picture columns of a frame (L complex lines: column x0 + l real, x0 + L + l
//                     imaginary), forms the shading surface beta from the bands' partials, erases the anchors' squares
//                     as it loads them, sums each column's detrend moments, transforms the L lines along y in shared
//                     memory and separates the two real columns of each, writing Y[v][x] for the kept rows v;
//   fac_kernel        one CTA a frame: the five projections from the columns' moments, then the surface spectrum's
//                     per-column and per-row factors (the double products the reference rounds to float);
//   fft_rows_kernel   a CTA takes L kept rows v of a frame, transforms along x and subtracts the surface's spectrum
//                     (the xy term everywhere, the x terms on v = 0, the y terms on u = 0), writing the used
//                     coefficients in pos order.
// L is the most lines of n points that fit 6144 complex points (so every CTA holds about the same 48 KB of samples).
//
// The transforms are Stockham autosort passes of radix 16, 9, 8, 6, 5, 4, 3 or 2 (every ladder size takes three),
// each pass in place: every thread reads its butterflies' points into registers, the CTA waits, every thread writes
// its outputs. Shared memory holds a line with one spare slot after every 16 points (so the passes' 16-point runs,
// read or written, fall on distinct banks within a half-warp) and lines 16 / L (mod 16) slots apart; the passes'
// twiddles sit beside the lines, per pass [r - 1][k], so a warp reads consecutive entries. FP32 throughout, as the
// reference's; the twiddles and the surface factors are worked out in double.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include "lizg_internal.h"
#include "sample_dev.cuh"

namespace lizg {

constexpr int kThreads = 384;   // threads of a transform CTA
constexpr int kHoleBand = 16;   // every-eighth-sample rows a hole_rhs CTA takes

__device__ __forceinline__ float2 cmul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }

// A point's slot in its line: one spare slot after every 16.
__device__ __forceinline__ int pad(int p) { return p + (p >> 4); }

// Forward DFTs (e^{-i}) of R points in place.
template <int R> __device__ __forceinline__ void dft(float2 *v);

template <> __device__ __forceinline__ void dft<2>(float2 *v) { const float2 a = v[0], b = v[1]; v[0] = cadd(a, b); v[1] = csub(a, b); }
template <> __device__ __forceinline__ void dft<4>(float2 *v) {
  const float2 s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]), s13 = cadd(v[1], v[3]), d13 = csub(v[1], v[3]);
  v[0] = cadd(s02, s13); v[2] = csub(s02, s13);
  v[1] = make_float2(d02.x + d13.y, d02.y - d13.x);   // d02 - i d13
  v[3] = make_float2(d02.x - d13.y, d02.y + d13.x);   // d02 + i d13
}
template <> __device__ __forceinline__ void dft<3>(float2 *v) {
  const float s3 = 0.86602540378443864676f;
  const float2 a = v[0], t = cadd(v[1], v[2]), d = csub(v[1], v[2]);
  const float2 m = make_float2(a.x - 0.5f * t.x, a.y - 0.5f * t.y);
  v[0] = cadd(a, t);
  v[1] = make_float2(m.x + s3 * d.y, m.y - s3 * d.x);   // m - i s3 d
  v[2] = make_float2(m.x - s3 * d.y, m.y + s3 * d.x);   // m + i s3 d
}
template <> __device__ __forceinline__ void dft<5>(float2 *v) {
  const float c1 = 0.30901699437494742410f, c2 = -0.80901699437494742410f;   // cos 2pi/5, cos 4pi/5
  const float s1 = 0.95105651629515357212f, s2 = 0.58778525229247312917f;    // sin 2pi/5, sin 4pi/5
  const float2 a = v[0], p1 = cadd(v[1], v[4]), m1 = csub(v[1], v[4]), p2 = cadd(v[2], v[3]), m2 = csub(v[2], v[3]);
  const float2 r1 = make_float2(a.x + c1 * p1.x + c2 * p2.x, a.y + c1 * p1.y + c2 * p2.y);
  const float2 r2 = make_float2(a.x + c2 * p1.x + c1 * p2.x, a.y + c2 * p1.y + c1 * p2.y);
  const float2 q1 = make_float2(s1 * m1.x + s2 * m2.x, s1 * m1.y + s2 * m2.y);   // times -i below
  const float2 q2 = make_float2(s2 * m1.x - s1 * m2.x, s2 * m1.y - s1 * m2.y);
  v[0] = make_float2(a.x + p1.x + p2.x, a.y + p1.y + p2.y);
  v[1] = make_float2(r1.x + q1.y, r1.y - q1.x);
  v[4] = make_float2(r1.x - q1.y, r1.y + q1.x);
  v[2] = make_float2(r2.x + q2.y, r2.y - q2.x);
  v[3] = make_float2(r2.x - q2.y, r2.y + q2.x);
}

// e^{-2 pi i m / R} for the m a composite DFT turns by that are not eighth turns.
template <int R> __device__ __forceinline__ float2 wconst(int m);
template <> __device__ __forceinline__ float2 wconst<16>(int m) {
  return m == 1 ? make_float2(0.92387953251128673848f, -0.38268343236508978178f)
       : m == 3 ? make_float2(0.38268343236508983729f, -0.92387953251128673848f)
                : make_float2(-0.92387953251128684951f, 0.38268343236508967076f);   // m = 9
}
template <> __device__ __forceinline__ float2 wconst<8>(int) { return make_float2(1.0f, 0.0f); }   // every turn of 8 is an eighth
template <> __device__ __forceinline__ float2 wconst<6>(int m) {
  return m == 1 ? make_float2(0.5f, -0.86602540378443864676f) : make_float2(-0.5f, -0.86602540378443864676f);   // m = 2
}
template <> __device__ __forceinline__ float2 wconst<9>(int m) {
  return m == 1 ? make_float2(0.76604444311897801345f, -0.64278760968653925190f)
       : m == 2 ? make_float2(0.17364817766693041445f, -0.98480775301220802032f)
                : make_float2(-0.93969262078590831688f, -0.34202014332566887944f);   // m = 4
}
// a e^{-2 pi i m / R} for a constant m (after unrolling): quarter and eighth turns by adds, the rest by cos/sin.
template <int R> __device__ __forceinline__ float2 twc(float2 a, int m) {
  m %= R;
  const float c = 0.70710678118654757274f;
  if (m == 0) return a;
  if (4 * m == R) return make_float2(a.y, -a.x);
  if (2 * m == R) return make_float2(-a.x, -a.y);
  if (4 * m == 3 * R) return make_float2(-a.y, a.x);
  if (8 * m == R) return make_float2(c * (a.x + a.y), c * (a.y - a.x));
  if (8 * m == 3 * R) return make_float2(c * (a.y - a.x), -c * (a.x + a.y));
  return cmul(a, wconst<R>(m));
}

// R = P Q points by P-point DFTs over the Q interleaved subsequences, twiddles, then Q-point DFTs:
// X[k1 + P k2] = sum_n2 W_Q^{n2 k2} W_R^{n2 k1} sum_n1 x[Q n1 + n2] W_P^{n1 k1}.
template <int P, int Q> __device__ __forceinline__ void dft_pq(float2 *x) {
  constexpr int R = P * Q;
  float2 a[Q][P];
#pragma unroll
  for (int n2 = 0; n2 < Q; n2++) {
#pragma unroll
    for (int n1 = 0; n1 < P; n1++) a[n2][n1] = x[Q * n1 + n2];
    dft<P>(a[n2]);
#pragma unroll
    for (int k1 = 1; k1 < P; k1++) a[n2][k1] = twc<R>(a[n2][k1], n2 * k1);
  }
#pragma unroll
  for (int k1 = 0; k1 < P; k1++) {
    float2 b[Q];
#pragma unroll
    for (int n2 = 0; n2 < Q; n2++) b[n2] = a[n2][k1];
    dft<Q>(b);
#pragma unroll
    for (int k2 = 0; k2 < Q; k2++) x[k1 + P * k2] = b[k2];
  }
}
template <> __device__ __forceinline__ void dft<8>(float2 *v) { dft_pq<4, 2>(v); }
template <> __device__ __forceinline__ void dft<16>(float2 *v) { dft_pq<4, 4>(v); }
template <> __device__ __forceinline__ void dft<6>(float2 *v) { dft_pq<3, 2>(v); }
template <> __device__ __forceinline__ void dft<9>(float2 *v) { dft_pq<3, 3>(v); }

// The transform plan of each ladder size: three passes' radices and the lines a CTA holds (the most lines of n
// points within kFftPoints, n a multiple of twice that). Host and device read the same table.
struct Plan {
  int r0, r1, r2, lines;
};
__host__ __device__ constexpr Plan plan_of(int n) {
  return n == 384    ? Plan{16, 8, 3, 16}
         : n == 512  ? Plan{16, 16, 2, 8}
         : n == 768  ? Plan{16, 16, 3, 8}
         : n == 1024 ? Plan{16, 16, 4, 4}
         : n == 1152 ? Plan{16, 8, 9, 4}
         : n == 1280 ? Plan{16, 16, 5, 4}
         : n == 1536 ? Plan{16, 16, 6, 4}
                     : Plan{0, 0, 0, 0};
}
// Slots from one line to the next: the padded line rounded up to 16 slots, plus 16 / L, so that the L lines x
// 16 / L rows a half-warp stores while loading (and reads while separating) fall on 16 distinct slots.
__host__ __device__ constexpr int lstride_of(int n) { return (n + n / 16 + 15) / 16 * 16 + 16 / plan_of(n).lines; }

// One Stockham pass of radix R over the CTA's lines (Lr <= L of them) in place, n = N points a line. Butterfly j of
// a line (j < NR = N / R, k = j mod NS) reads points j + r NR, turns point r by e^{-2 pi i r k / (NS R)}
// (tw[NS + (r - 1) NS + k]) and writes its DFT's output r to (j / NS) NS R + k + r NS. A thread takes butterflies tid,
// tid + kThreads, ... (at most B = ceil(L NR / kThreads) of them).
// The thread's index, read afresh: the passes' offsets hang on it, so a loop round the passes recomputes them pass by
// pass instead of holding every pass's offsets live across the loop.
__device__ __forceinline__ int tid_fresh() {
  int t;
  asm volatile("mov.u32 %0, %%tid.x;" : "=r"(t));
  return t;
}

template <int N, int R, int NS, int L>
__device__ __forceinline__ void pass(float2 *buf, const float2 *tw, int Lr) {
  constexpr int NR = N / R, LSTR = lstride_of(N), B = (L * NR + kThreads - 1) / kThreads;
  const int total = Lr * NR, tid = tid_fresh();
  float2 v[B][R];
#pragma unroll
  for (int b = 0; b < B; b++) {
    const int t = tid + b * kThreads;
    if (t < total) {
      const int l = t / NR, j = t - l * NR, k = j % NS;
      const float2 *in = buf + l * LSTR;
#pragma unroll
      for (int r = 0; r < R; r++) v[b][r] = in[pad(j + r * NR)];
      if (NS > 1) {
#pragma unroll
        for (int r = 1; r < R; r++) v[b][r] = cmul(v[b][r], tw[NS + (r - 1) * NS + k]);
      }
      dft<R>(v[b]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int b = 0; b < B; b++) {
    const int t = tid + b * kThreads;
    if (t < total) {
      const int l = t / NR, j = t - l * NR, jq = j / NS, k = j - jq * NS;
      float2 *out = buf + l * LSTR;
      const int base = jq * NS * R + k;
#pragma unroll
      for (int r = 0; r < R; r++) out[pad(base + r * NS)] = v[b][r];
    }
  }
  __syncthreads();
}

// The Lr lines at buf (line l at buf + l lstride_of(N), point p at slot pad(p)) transformed along their N points in
// place by the size's three passes. tw: the passes' twiddles, pass s's at NS (a multiple of 16 past the first pass,
// so a half-warp's 16 twiddles are one aligned 128-byte row). Every thread of the CTA takes part.
template <int N>
__device__ __forceinline__ void fft_lines(float2 *buf, const float2 *tw, int Lr) {
  constexpr Plan P = plan_of(N);
  pass<N, P.r0, 1, P.lines>(buf, tw, Lr);
  pass<N, P.r1, P.r0, P.lines>(buf, tw, Lr);
  pass<N, P.r2, P.r0 * P.r1, P.lines>(buf, tw, Lr);
}

// A frame's shading-fit sample (x, y) = (8 kx, 8 ky): from the captured frame through its registration when the
// frame is given (the decode's read as the reference's finish takes these samples, one call over every eighth row and
// column, liblizard/src/lizard_phy.c:1611; or the exact walk), else from a supplied grid.
__device__ __forceinline__ float shade_at(const SrcDev &s, int f, int kx, int ky) {
  const int x = 8 * kx, y = 8 * ky;
  if (!s.luma) return s.grid[f * s.gstride + (int64_t)y * s.sd.n + x];
  const float *H = s.reg + (int64_t)f * s.regstride;
  const uint8_t *px = s.luma + f * s.fstride;
  const float4 ct = s.sd.colt[x], rt = s.sd.rowt[y];
  if (s.sd.read != LIZG_READ_DECODE) return sample_xy_exact(s.sd, px, s.w, s.h, s.pitch, H, H + 9, ct, rt);
  const RowTerms r = row_terms(H, rt);
  const LinCol c = lin_col_shade(s.sd, H, kx);
  LinNum n = lin_start(c, r.kw, r.ku, r.kv);
  lin_steps(c, n, c.g);
  return lin_point(px, s.w, s.h, s.pitch, n, lin_cell(s.sd, H + 9, ct, r.j), r.v);
}

__device__ __forceinline__ bool in_square(const FftDev &xd, int t) {
  bool in = false;
#pragma unroll
  for (int i = 0; i < 7; i++) in |= t >= xd.elo[i] && t <= xd.ehi[i];
  return in;
}

// The shading basis 1, c(x), q(x), c(y), q(y), c(x) c(y) at sample (x, y) (liblizard/src/lizard_phy.c:336-340).
__device__ __forceinline__ void hole_basis(const FftDev &xd, int x, int y, double b[6]) {
  const double cx = xd.cx[x], cy = xd.cx[y];
  b[0] = 1; b[1] = cx; b[2] = xd.qx[x]; b[3] = cy; b[4] = xd.qx[y]; b[5] = cx * cy;
}

// The shading fit's right-hand side (liblizard/src/lizard_phy.c:1609-1623) over kHoleBand of the frame's
// every-eighth rows: hole[f][band][0..5]. A warp takes a row: its samples outside the squares summed in float as
// z, z c(x), z q(x) (the basis is separable: 1, c(x), q(x), c(y), q(y), c(x) c(y)), then the row's six terms added
// in double; the warps' sums added in warp order.
__device__ __forceinline__ void hole_rhs_band(const FftDev &xd, const SrcDev &src, int bands, double *hole, int f, int band) {
  const int n = xd.n, c = n / 8;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, ky1 = min(c, (band + 1) * kHoleBand);
  double rhs[6] = {0, 0, 0, 0, 0, 0};
  for (int ky = band * kHoleBand + warp; ky < ky1; ky += 8) {
    const int y = 8 * ky;
    const bool ysq = in_square(xd, y);
    float s0 = 0, s1 = 0, s2 = 0;
    for (int kx = lane; kx < c; kx += 32) {
      const int x = 8 * kx;
      if (ysq && in_square(xd, x)) continue;
      const float v = shade_at(src, f, kx, ky);
      s0 += v; s1 += __ldg(xd.cx + x) * v; s2 += __ldg(xd.qx + x) * v;
    }
    for (int o = 16; o > 0; o >>= 1) {
      s0 += __shfl_xor_sync(0xffffffffu, s0, o);
      s1 += __shfl_xor_sync(0xffffffffu, s1, o);
      s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    const double cy = xd.cx[y], qy = xd.qx[y];
    rhs[0] += s0; rhs[1] += s1; rhs[2] += s2; rhs[3] += cy * s0; rhs[4] += qy * s0; rhs[5] += cy * s1;
  }
  __shared__ double red[8][6];
  if (lane == 0)
    for (int r = 0; r < 6; r++) red[warp][r] = rhs[r];
  __syncthreads();
  if (threadIdx.x < 6) {
    double acc = 0;
    for (int w = 0; w < 8; w++) acc += red[w][threadIdx.x];
    hole[((int64_t)f * bands + band) * 6 + threadIdx.x] = acc;
  }
}
__global__ void __launch_bounds__(256) hole_rhs_kernel(FftDev xd, SrcDev src, int bands, double *hole) {
  hole_rhs_band(xd, src, bands, hole, blockIdx.x / bands, blockIdx.x % bands);
}

// The transform CTA's shared memory: the lines, the twiddles, the moments' reduction.
struct SmemMap {
  float2 *buf, *tw;
  double *red;
};
__host__ __device__ constexpr int smem_bytes_of(int n) {
  return (plan_of(n).lines * lstride_of(n) + n) * (int)sizeof(float2) + (kThreads / 32) * 6 * plan_of(n).lines * (int)sizeof(double);
}
template <int N>
__device__ __forceinline__ SmemMap smem_map(unsigned char *raw) {
  SmemMap m;
  m.buf = reinterpret_cast<float2 *>(raw);
  m.tw = m.buf + plan_of(N).lines * lstride_of(N);
  m.red = reinterpret_cast<double *>(m.tw + N);
  return m;
}

__host__ __device__ constexpr int cmax_i(int x, int y) { return x > y ? x : y; }

// The mixed-size grids' kernel arguments: each format's tables and buffers, and its first CTA (first[nseg] CTAs in all).
struct FftColsSeg {
  FftDev xd;
  SrcDev src;
  const float4 *ctab;
  const double *hole;
  double *part;
  float2 *Y;
  int bands;
};
struct FftColsMix {
  FftColsSeg seg[kFftMixSegs];
  int first[kFftMixSegs + 1];
  int nseg;
};
struct FftRowsSeg {
  CUtensorMap ymap;
  FftDev xd;
  const float2 *fac;
  const int32_t *tpos;
  float2 *C;
  int *err;
  int need;
};
struct FftRowsMix {
  FftRowsSeg seg[kFftMixSegs];
  int first[kFftMixSegs + 1];
  int nseg;
};
static_assert(sizeof(FftColsMix) <= 32000 && sizeof(FftRowsMix) <= 32000, "the mixed grids' arguments fit a launch");

// The surface's value at (x, y) inside an anchor's square (liblizard/src/lizard_phy.c:341-346).
__device__ __forceinline__ float hole_value(const FftDev &xd, const double *beta, int x, int y) {
  double bb[6], h = 0;
  hole_basis(xd, x, y, bb);
  for (int r = 0; r < 6; r++) h += beta[r] * bb[r];
  return (float)h;
}

// The sampler's per-row quantities of a batch, worked out once a frame before the column pass reads them, with the
// same functions and inputs as the per-sample walk (the cell's 1 / width as the column table computes it), so the
// column pass reads the walk's own values. A thread an entry, entries in table order. The exact walk: for picture row
// y and mesh cell i < nx - 1 the displacement line cell_terms gives, and at i = nx - 1 the homography's row terms
// (kw, ku, kv). The decode's read: the row terms of row y at y < n, then each column x's displacement terms at mesh
// row j (lin_cell) at n + j n + x.
__device__ __forceinline__ void cell_table_entry(const SrcDev &src, int per_frame, float4 *ctab, int f, int t) {
  if (t >= per_frame) return;
  const SampleDev &sd = src.sd;
  const float *H = src.reg + (int64_t)f * src.regstride;
  float4 o;
  if (sd.read == LIZG_READ_DECODE) {
    if (t < sd.n) {
      const RowTerms r = row_terms(H, sd.rowt[t]);
      o = make_float4(r.kw, r.ku, r.kv, 0.0f);
    } else {
      const int j = (t - sd.n) / sd.n, x = t - sd.n - j * sd.n;
      o = lin_cell(sd, H + 9, sd.colt[x], j);
    }
  } else {
    const int nn = sd.nx, y = t / nn, i = t - y * nn;
    const RowTerms r = row_terms(H, sd.rowt[y]);
    if (i == nn - 1) {
      o = make_float4(r.kw, r.ku, r.kv, 0.0f);
    } else {
      const float inv = __fdiv_rn(1.0f, __fsub_rn(sd.node_x[i + 1], sd.node_x[i]));
      const CellTerms c = cell_terms(sd, H + 9, i, inv, r);
      o = make_float4(c.ex, c.cx, c.ey, c.cy);
    }
  }
  ctab[(int64_t)f * per_frame + t] = o;
}
__global__ void __launch_bounds__(256) cell_table_kernel(SrcDev src, int per_frame, float4 *ctab) {
  cell_table_entry(src, per_frame, ctab, blockIdx.y, blockIdx.x * blockDim.x + threadIdx.x);
}

// One column tile's samples: thread t takes line l = t mod L (columns xa = x0 + l as the real part, xb = x0 + L + l as
// the imaginary part) at rows y = t / L, t / L + kThreads / L, ...; the anchors' squares erased to the shading
// surface as they are read. Each row's two samples are summed into the five detrend projections' raw sums, z c(x),
// z c(y), z c(x) c(y), z q(x), z q(y) (liblizard/src/lizard_phy.c:1584-1591, 1657-1667), in p. SRC: kSrcGrid reads a
// supplied grid; kSrcExact and kSrcDecode sample the captured frame by the exact walk or the decode's read.
constexpr int kSrcGrid = 0, kSrcExact = 1, kSrcDecode = 2;
template <int N, int SRC>
__device__ __forceinline__ void load_tile(const FftDev &xd, const SrcDev &src, const float4 *ctab, int f, int x0, const double *beta,
                                          float2 *line, float p[5]) {
  constexpr int L = plan_of(N).lines, ystep = kThreads / L;
  const int l = threadIdx.x % L, xa = x0 + l, xb = x0 + L + l;
  const bool ina = in_square(xd, xa), inb = in_square(xd, xb);
  const float cxa = __ldg(xd.cx + xa), qxa = __ldg(xd.qx + xa), cxb = __ldg(xd.cx + xb), qxb = __ldg(xd.qx + xb);
  float mxa = 0, mxb = 0, h6a = 0, h0a = 0, h3a = 0, h6b = 0, h0b = 0, h3b = 0;
  int ia = 0, ib = 0, nn = 1;
  const uint8_t *px = nullptr;
  const float4 *T = nullptr;   // the frame's row and cell table
  LinCol lc{};                 // the decode's read: column xa's lanes (xb shares its lane, L / 4 steps on)
  if (SRC != kSrcGrid) {
    const float *H = src.reg + (int64_t)f * src.regstride;
    nn = src.sd.nx;
    T = ctab + (int64_t)f * N * nn;
    px = src.luma + f * src.fstride;
    const float4 ca = src.sd.colt[xa], cb = src.sd.colt[xb];
    mxa = ca.x; ia = __float_as_int(ca.y);
    mxb = cb.x; ib = __float_as_int(cb.y);
    if (SRC == kSrcExact) {
      h6a = __fmul_rn(H[6], mxa); h0a = __fmul_rn(H[0], mxa); h3a = __fmul_rn(H[3], mxa);
      h6b = __fmul_rn(H[6], mxb); h0b = __fmul_rn(H[0], mxb); h3b = __fmul_rn(H[3], mxb);
    } else {
      lc = lin_col_grid(src.sd, H, xa);   // a tile's 2L columns lie in one strip of 64 (2L divides 64)
    }
  }
#pragma unroll 2   // 2 of 2, 4 and 8 is the fastest on a GB300 (61.1k, 59.3k, 57.7k batch frames/s)
  for (int y = threadIdx.x / L; y < N; y += ystep) {
    const bool ysq = (ina || inb) && in_square(xd, y);
    float va, vb;
    if (SRC == kSrcGrid) {
      const float *g = src.grid + f * src.gstride + (int64_t)y * N;
      va = g[xa]; vb = g[xb];
    } else if (SRC == kSrcExact) {
      const float4 *Ty = T + y * nn;
      const float4 rt = Ty[nn - 1], ta = Ty[ia], tb = ib == ia ? ta : Ty[ib];
      RowTerms r;
      r.kw = rt.x; r.ku = rt.y; r.kv = rt.z;
      const CellTerms ca{ta.x, ta.y, ta.z, ta.w}, cb{tb.x, tb.y, tb.z, tb.w};
      va = sample_at(px, src.w, src.h, src.pitch, mxa, h6a, h0a, h3a, r, ca);
      vb = sample_at(px, src.w, src.h, src.pitch, mxb, h6b, h0b, h3b, r, cb);
    } else {
      const float4 rt = T[y], rw = __ldg(&src.sd.rowt[y]);
      const int j = __float_as_int(rw.y);
      const float4 ta = T[N + j * N + xa], tb = T[N + j * N + xb];
      LinNum s = lin_start(lc, rt.x, rt.y, rt.z);
      lin_steps(lc, s, lc.g);
      va = lin_point(px, src.w, src.h, src.pitch, s, ta, rw.z);
      lin_steps(lc, s, L / 4);
      vb = lin_point(px, src.w, src.h, src.pitch, s, tb, rw.z);
    }
    if (ina && ysq) va = hole_value(xd, beta, xa, y);
    if (inb && ysq) vb = hole_value(xd, beta, xb, y);
    const float cy = __ldg(xd.cx + y), qy = __ldg(xd.qx + y);
    const float t0 = va + vb, t1 = cxa * va + cxb * vb, t2 = qxa * va + qxb * vb;
    p[0] += t1; p[1] += cy * t0; p[2] += cy * t1; p[3] += t2; p[4] += qy * t0;
    line[pad(y)] = make_float2(va, vb);
  }
}

// The column pass's per-CTA scalars in shared memory.
struct ColsShared {
  double rhs[6], beta[6];
  float part[kThreads / 32][5];
};

// The column pass on one tile (frame f, columns x0 = 2 L tile .. x0 + 2L - 1): the shading surface beta from the
// frame's bands, the tile's samples (erased, projections summed: part[f][tile][0..4]), the L lines' transforms along
// y, and the two real columns of each line separated: A(v) = (Z(v) + conj Z(n - v)) / 2, B(v) = -i (Z(v) - conj
// Z(n - v)) / 2, written to Y[f][v][x] for the kept rows v. Every thread of the CTA takes part.
template <int N>
__device__ __forceinline__ void cols_tile(const FftDev &xd, const SrcDev &src, const float4 *ctab, int bands, const double *hole,
                                          double *part, float2 *Y, int f, int tile, unsigned char *smraw, ColsShared &s) {
  constexpr int n = N, L = plan_of(N).lines, LSTR = lstride_of(N), tiles = n / (2 * L), ystep = kThreads / L;
  const SmemMap sm = smem_map<N>(smraw);
  const int tid = threadIdx.x, l = tid % L, warp = tid >> 5, lane = tid & 31, x0 = tile * 2 * L;
  for (int i = tid; i < n; i += kThreads) sm.tw[i] = xd.tws[i];
  float2 *line = sm.buf + l * LSTR;
  if (tid < 6) {
    double acc = 0;
    for (int b = 0; b < bands; b++) acc += hole[((int64_t)f * bands + b) * 6 + tid];
    s.rhs[tid] = acc;
  }
  __syncthreads();
  if (tid == 0) {
#pragma unroll
    for (int r = 0; r < 6; r++) {
      double acc = 0;
#pragma unroll
      for (int k = 0; k < 6; k++) acc += xd.hole_inv[r * 6 + k] * s.rhs[k];
      s.beta[r] = acc;
    }
  }
  __syncthreads();
  float p[5] = {0, 0, 0, 0, 0};
  if (src.grid) load_tile<N, kSrcGrid>(xd, src, ctab, f, x0, s.beta, line, p);
  else if (src.sd.read == LIZG_READ_DECODE) load_tile<N, kSrcDecode>(xd, src, ctab, f, x0, s.beta, line, p);
  else load_tile<N, kSrcExact>(xd, src, ctab, f, x0, s.beta, line, p);
#pragma unroll
  for (int q = 0; q < 5; q++)
    for (int o = 16; o > 0; o >>= 1) p[q] += __shfl_xor_sync(0xffffffffu, p[q], o);
  if (lane == 0)
    for (int q = 0; q < 5; q++) s.part[warp][q] = p[q];
  __syncthreads();
  if (tid < 5) {
    double acc = 0;
    for (int w = 0; w < kThreads / 32; w++) acc += s.part[w][tid];
    part[((int64_t)f * tiles + tile) * 5 + tid] = acc;
  }
  fft_lines<N>(sm.buf, sm.tw, L);
  float2 *Yf = Y + (int64_t)f * xd.vrows * n;
  const int xa = x0 + l, xb = x0 + L + l;
  for (int v = tid / L; v < xd.vrows; v += ystep) {
    const float2 zv = line[pad(v)], zm = line[pad(v ? n - v : 0)];
    Yf[(int64_t)v * n + xa] = make_float2(0.5f * (zv.x + zm.x), 0.5f * (zv.y - zm.y));
    Yf[(int64_t)v * n + xb] = make_float2(0.5f * (zv.y + zm.y), -0.5f * (zv.x - zm.x));
  }
}

// The column pass of one picture size: CTA b takes tile b mod tiles of frame b / tiles.
template <int N>
__global__ void __launch_bounds__(kThreads, 3) fft_cols_kernel(FftDev xd, SrcDev src, const float4 *ctab, int bands, const double *hole, double *part,
                                                                float2 *Y) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ ColsShared s;
  constexpr int tiles = N / (2 * plan_of(N).lines);
  cols_tile<N>(xd, src, ctab, bands, hole, part, Y, blockIdx.x / tiles, blockIdx.x % tiles, smraw, s);
}

// The column pass over several picture sizes in one grid: a queue of (format, frame, tile) items, format k's at CTAs
// [first[k], first[k + 1]), each taken by its size's body (every size's tile holds about the same 48 KB of samples,
// so one CTA shape serves them all; the dynamic shared memory is the largest size's).
__global__ void __launch_bounds__(kThreads, 3) fft_cols_mixed_kernel(const __grid_constant__ FftColsMix m) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ ColsShared s;
  int k = 0;
  while (k < m.nseg - 1 && (int)blockIdx.x >= m.first[k + 1]) k++;
  const FftColsSeg &g = m.seg[k];
  const int b = (int)blockIdx.x - m.first[k], tiles = g.xd.n / (2 * plan_of(g.xd.n).lines), f = b / tiles, tile = b - f * tiles;
  switch (g.xd.n) {
    case 384: cols_tile<384>(g.xd, g.src, g.ctab, g.bands, g.hole, g.part, g.Y, f, tile, smraw, s); break;
    case 512: cols_tile<512>(g.xd, g.src, g.ctab, g.bands, g.hole, g.part, g.Y, f, tile, smraw, s); break;
    case 768: cols_tile<768>(g.xd, g.src, g.ctab, g.bands, g.hole, g.part, g.Y, f, tile, smraw, s); break;
    case 1024: cols_tile<1024>(g.xd, g.src, g.ctab, g.bands, g.hole, g.part, g.Y, f, tile, smraw, s); break;
    case 1152: cols_tile<1152>(g.xd, g.src, g.ctab, g.bands, g.hole, g.part, g.Y, f, tile, smraw, s); break;
    case 1280: cols_tile<1280>(g.xd, g.src, g.ctab, g.bands, g.hole, g.part, g.Y, f, tile, smraw, s); break;
    default: cols_tile<1536>(g.xd, g.src, g.ctab, g.bands, g.hole, g.part, g.Y, f, tile, smraw, s); break;
  }
}

// The five projections of each frame from its column tiles' sums, in tile order, normalised
// (liblizard/src/lizard_phy.c:1697), then the surface spectrum's factors (liblizard/src/lizard_phy.c:1702-1716),
// rounded to float as there: fac[f] = xy[u] (pxy X1[u]) for u < n, x0[u] (n (px X1[u] + pxx X2[u])) for u < n,
// y0[v] (n (py X1[v] + pyy X2[v])) for v < vrows.
__device__ __forceinline__ void fac_frame(const FftDev &xd, int tiles, const double *part, float2 *fac, int f) {
  const int n = xd.n;
  __shared__ double s_p[5];
  if (threadIdx.x < 5) {
    double acc = 0;
    for (int t = 0; t < tiles; t++) acc += part[((int64_t)f * tiles + t) * 5 + threadIdx.x];
    s_p[threadIdx.x] = acc;
  }
  __syncthreads();
  const double px = s_p[0] / (n * xd.sx2), py = s_p[1] / (n * xd.sx2), pxy = s_p[2] / (xd.sx2 * xd.sx2);
  const double pxx = s_p[3] / (n * xd.sq2), pyy = s_p[4] / (n * xd.sq2);
  float2 *o = fac + (int64_t)f * (2 * n + xd.vrows);
  for (int u = threadIdx.x; u < n; u += blockDim.x) {
    const float2 x1 = xd.x1[u], x2 = xd.x2[u];
    o[u] = make_float2((float)(pxy * x1.x), (float)(pxy * x1.y));
    o[n + u] = make_float2((float)(n * (px * x1.x + pxx * x2.x)), (float)(n * (px * x1.y + pxx * x2.y)));
  }
  for (int v = threadIdx.x; v < xd.vrows; v += blockDim.x) {
    const float2 x1 = xd.x1[v], x2 = xd.x2[v];
    o[2 * n + v] = make_float2((float)(n * (py * x1.x + pyy * x2.x)), (float)(n * (py * x1.y + pyy * x2.y)));
  }
}
__global__ void __launch_bounds__(256) fac_kernel(FftDev xd, int tiles, const double *part, float2 *fac) {
  fac_frame(xd, tiles, part, fac, blockIdx.x);
}

// The shading sums, the sampler's tables and the surface factors over several formats' batches, one launch a stage:
// format k's shading-band CTAs at [hf[k], hf[k + 1]), then its table CTAs at [tf[k], tf[k + 1]) (one launch takes
// both), its frames' factor CTAs at [ff[k], ff[k + 1]).
struct FftLightSeg {
  FftDev xd;
  SrcDev src;
  double *hole, *part;
  float4 *ctab;
  float2 *fac;
  int bands, per_frame, tblocks, tiles;
};
struct FftLightMix {
  FftLightSeg seg[kFftMixSegs];
  int hf[kFftMixSegs + 1], tf[kFftMixSegs + 1], ff[kFftMixSegs + 1];
  int nseg;
};
static_assert(sizeof(FftLightMix) <= 32000, "the light stages' arguments fit a launch");
__device__ __forceinline__ int seg_at(const int *first, int nseg, int b) {
  int k = 0;
  while (k < nseg - 1 && b >= first[k + 1]) k++;
  return k;
}
__global__ void __launch_bounds__(256) fft_pre_mixed_kernel(const __grid_constant__ FftLightMix m) {
  const int b = blockIdx.x;
  if (b < m.hf[m.nseg]) {
    const int k = seg_at(m.hf, m.nseg, b);
    const FftLightSeg &g = m.seg[k];
    const int lb = b - m.hf[k];
    hole_rhs_band(g.xd, g.src, g.bands, g.hole, lb / g.bands, lb % g.bands);
  } else {
    const int k = seg_at(m.tf, m.nseg, b);
    const FftLightSeg &g = m.seg[k];
    const int lb = b - m.tf[k], f = lb / g.tblocks;
    cell_table_entry(g.src, g.per_frame, g.ctab, f, (lb - f * g.tblocks) * 256 + threadIdx.x);
  }
}
__global__ void __launch_bounds__(256) fac_mixed_kernel(const __grid_constant__ FftLightMix m) {
  const int k = seg_at(m.ff, m.nseg, blockIdx.x);
  const FftLightSeg &g = m.seg[k];
  fac_frame(g.xd, g.tiles, g.part, g.fac, blockIdx.x - m.ff[k]);
}

// A bounded wait on an mbarrier's phase (try_wait blocks a while in hardware before it answers): false when the
// limit ran out.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int limit) {
  for (int i = 0; i < limit; i++) {
    uint32_t done;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(done) : "r"(bar), "r"(parity) : "memory");
    if (done) return true;
  }
  return false;
}

// The row pass on one tile (frame f, rows v0 = L rtile .. v0 + L - 1): transforms them along x and takes the surface's
// spectrum off: the xy term pxy X1[u] X1[v] everywhere, the x terms on v = 0, the y terms on u = 0. The used
// coefficients go straight to their place in pos order: C[f][tpos[v][u]] (tpos -1 where (u, v) is not used).
// The tile's rows come in by the tensor memory accelerator: bulk tensor copies of 128 complex points of a row each,
// issued by one thread, landing densely at the start of each line's slots (at a 128-byte boundary) and counted on an
// mbarrier; then every thread moves its points from the dense rows to the padded lines (all read, then all written).
template <int N>
__device__ __forceinline__ void rows_tile(const FftDev &xd, const float2 *fac, const CUtensorMap *ymap, const int32_t *tpos, int need, float2 *C,
                                          int *err, int f, int rtile, unsigned char *smraw, uint64_t *s_bar) {
  constexpr int n = N, L = plan_of(N).lines, LSTR = lstride_of(N), SEGS = N / 128, PER = (L * N + kThreads - 1) / kThreads;
  static_assert(LSTR >= N + 16, "a line's slots hold its dense row at a 128-byte boundary");
  const SmemMap sm = smem_map<N>(smraw);
  const int tid = threadIdx.x;
  const int v0 = rtile * L, Lr = min(L, xd.vrows - v0);
  const uint32_t bar = (uint32_t)__cvta_generic_to_shared(s_bar);
  // line l's dense row: at the first 128-byte boundary of its slots (room: a line's slots exceed n by 16 or more)
  auto dense = [&](int l) { return (uint32_t)(((uint32_t)__cvta_generic_to_shared(sm.buf + l * LSTR) + 127u) & ~127u); };
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  if (tid == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"((uint32_t)(Lr * N * 8)) : "memory");
    const int y0 = f * xd.vrows + v0;
    for (int l = 0; l < Lr; l++)
      for (int s = 0; s < SEGS; s++)
        asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n"
                     ::"r"(dense(l) + 1024u * s), "l"(ymap), "r"(256 * s), "r"(y0 + l), "r"(bar) : "memory");
  }
  for (int i = tid; i < n; i += kThreads) sm.tw[i] = xd.tws[i];
  if (!mbar_wait(bar, 0, 1 << 22)) {   // never expected: record it, wait for the copies once more, leave the tile
    atomicOr(err, 1);
    mbar_wait(bar, 0, 1 << 22);
    return;
  }
  // dense rows to padded lines: thread t takes points t, t + kThreads, ... of the tile (line-major), all read first
  float2 v[PER];
#pragma unroll
  for (int k = 0; k < PER; k++) {
    const int p = tid + k * kThreads, l = p / N, u = p - l * N;
    if (p < L * N && l < Lr) {
      float2 t;
      asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];\n" : "=f"(t.x), "=f"(t.y) : "r"(dense(l) + 8u * u));
      v[k] = t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < PER; k++) {
    const int p = tid + k * kThreads, l = p / N, u = p - l * N;
    if (p < L * N && l < Lr) sm.buf[l * LSTR + pad(u)] = v[k];
  }
  __syncthreads();
  fft_lines<N>(sm.buf, sm.tw, Lr);
  float2 *Cf = C + (int64_t)f * need;
  const int32_t *tp = tpos + (int64_t)v0 * n;
  const float2 *fx = fac + (int64_t)f * (2 * n + xd.vrows), *fx0 = fx + n, *fy0 = fx + 2 * n;
  for (int u = tid; u < n; u += kThreads) {
    int iv[L];   // the rows' pos indices at this u, loaded ahead of their use
#pragma unroll
    for (int l = 0; l < L; l++) iv[l] = l < Lr ? __ldg(tp + l * n + u) : -1;
    const float2 a = fx[u];
#pragma unroll
    for (int l = 0; l < L; l++) {
      const int i = iv[l];
      if (i < 0) continue;
      const int v = v0 + l;
      float2 o = sm.buf[l * LSTR + pad(u)];
      const float2 x1v = xd.x1[v];
      o.x -= a.x * x1v.x - a.y * x1v.y;
      o.y -= a.x * x1v.y + a.y * x1v.x;
      if (v == 0) { const float2 c = fx0[u]; o.x -= c.x; o.y -= c.y; }
      if (u == 0) { const float2 c = fy0[v]; o.x -= c.x; o.y -= c.y; }
      Cf[i] = o;
    }
  }
}

// The row pass of one picture size: CTA b takes row tile b mod tiles of frame b / tiles.
template <int N>
__global__ void __launch_bounds__(kThreads, 3) fft_rows_kernel(FftDev xd, const float2 *fac, const __grid_constant__ CUtensorMap ymap,
                                                               const int32_t *tpos, int need, float2 *C, int *err) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ __align__(8) uint64_t s_bar;
  const int tiles = (xd.vrows + plan_of(N).lines - 1) / plan_of(N).lines;
  rows_tile<N>(xd, fac, &ymap, tpos, need, C, err, blockIdx.x / tiles, blockIdx.x % tiles, smraw, &s_bar);
}

// The row pass over several picture sizes in one grid: format k's (frame, row tile) items at CTAs
// [first[k], first[k + 1]), each with its own tensor map over its Y.
__global__ void __launch_bounds__(kThreads, 3) fft_rows_mixed_kernel(const __grid_constant__ FftRowsMix m) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ __align__(8) uint64_t s_bar;
  int k = 0;
  while (k < m.nseg - 1 && (int)blockIdx.x >= m.first[k + 1]) k++;
  const FftRowsSeg &g = m.seg[k];
  const int L = plan_of(g.xd.n).lines, tiles = (g.xd.vrows + L - 1) / L, b = (int)blockIdx.x - m.first[k], f = b / tiles, rt = b - f * tiles;
  switch (g.xd.n) {
    case 384: rows_tile<384>(g.xd, g.fac, &g.ymap, g.tpos, g.need, g.C, g.err, f, rt, smraw, &s_bar); break;
    case 512: rows_tile<512>(g.xd, g.fac, &g.ymap, g.tpos, g.need, g.C, g.err, f, rt, smraw, &s_bar); break;
    case 768: rows_tile<768>(g.xd, g.fac, &g.ymap, g.tpos, g.need, g.C, g.err, f, rt, smraw, &s_bar); break;
    case 1024: rows_tile<1024>(g.xd, g.fac, &g.ymap, g.tpos, g.need, g.C, g.err, f, rt, smraw, &s_bar); break;
    case 1152: rows_tile<1152>(g.xd, g.fac, &g.ymap, g.tpos, g.need, g.C, g.err, f, rt, smraw, &s_bar); break;
    case 1280: rows_tile<1280>(g.xd, g.fac, &g.ymap, g.tpos, g.need, g.C, g.err, f, rt, smraw, &s_bar); break;
    default: rows_tile<1536>(g.xd, g.fac, &g.ymap, g.tpos, g.need, g.C, g.err, f, rt, smraw, &s_bar); break;
  }
}

int fft_plan(int n, int radix[3], int *lines) {
  const Plan p = plan_of(n);
  if (!p.lines) return -1;
  radix[0] = p.r0; radix[1] = p.r1; radix[2] = p.r2;
  *lines = p.lines;
  return 0;
}

int fft_hole_bands(int n) { return (n / 8 + kHoleBand - 1) / kHoleBand; }

int fft_y_map(CUtensorMap *map, float2 *Y, int n, int64_t rows) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    cudaDriverEntryPointQueryResult q;
    void *fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess || !fn) return -1;
    encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  const cuuint64_t dims[2] = {(cuuint64_t)2 * n, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)2 * n * sizeof(float)};
  const cuuint32_t box[2] = {256, 1}, estr[2] = {1, 1};
  return (int)encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, Y, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
}

// The shading fit's partial sums, then (captured frames only) the sampler's row and cell table.
cudaError_t fft_pre_launch(const FftSegArgs &a, cudaStream_t st) {
  const int bands = fft_hole_bands(a.xd.n);
  hole_rhs_kernel<<<a.frames * bands, 256, 0, st>>>(a.xd, a.src, bands, a.b.hole);
  if (!a.src.grid) {
    if (!a.b.ctab || a.src.sd.nx != a.src.sd.ny) return cudaErrorInvalidValue;
    const int per_frame = a.xd.n * a.src.sd.nx;
    cell_table_kernel<<<dim3((per_frame + 255) / 256, a.frames), 256, 0, st>>>(a.src, per_frame, a.b.ctab);
  }
  return cudaGetLastError();
}

cudaError_t fft_fac_launch(const FftSegArgs &a, cudaStream_t st) {
  fac_kernel<<<a.frames, 256, 0, st>>>(a.xd, a.xd.n / (2 * plan_of(a.xd.n).lines), a.b.part, a.b.fac);
  return cudaGetLastError();
}

template <int N>
static cudaError_t fft_launch_n(const FftDev &xd, int frames, const SrcDev &src, const FftBufs &b, int sms, cudaStream_t st) {
  constexpr int L = plan_of(N).lines, smem = smem_bytes_of(N), tiles = N / (2 * L);
  static_assert(smem <= kFftSmemMax, "transform CTA's shared memory");
  static_assert(N % (2 * L) == 0 && L * N <= kFftPoints && kThreads % L == 0 && L <= 32, "transform plan");
  static SmemOptIn opt_cols, opt_rows;
  cudaError_t e;
  if ((e = opt_cols.set(reinterpret_cast<const void *>(fft_cols_kernel<N>), smem)) != cudaSuccess ||
      (e = opt_rows.set(reinterpret_cast<const void *>(fft_rows_kernel<N>), smem)) != cudaSuccess)
    return e;
  (void)sms;
  const FftSegArgs a{xd, src, b, frames};
  if ((e = fft_pre_launch(a, st)) != cudaSuccess) return e;
  fft_cols_kernel<N><<<frames * tiles, kThreads, smem, st>>>(xd, src, b.ctab, fft_hole_bands(N), b.hole, b.part, b.Y);
  if ((e = fft_fac_launch(a, st)) != cudaSuccess) return e;
  if (!b.ymap || !b.err) return cudaErrorInvalidValue;
  fft_rows_kernel<N><<<frames * ((xd.vrows + L - 1) / L), kThreads, smem, st>>>(xd, b.fac, *b.ymap, b.tpos, b.need, b.C, b.err);
  return cudaGetLastError();
}

// The largest transform CTA's shared memory over the ladder: the mixed grids' dynamic size.
constexpr int kFftSmemLadder = cmax_i(cmax_i(cmax_i(smem_bytes_of(384), smem_bytes_of(512)), cmax_i(smem_bytes_of(768), smem_bytes_of(1024))),
                                      cmax_i(cmax_i(smem_bytes_of(1152), smem_bytes_of(1280)), smem_bytes_of(1536)));
static_assert(kFftSmemLadder <= kFftSmemMax, "transform CTA's shared memory");

static int ladder_size(int n) { return plan_of(n).lines != 0; }

static cudaError_t light_mix(const FftSegArgs *a, int count, FftLightMix &m) {
  if (count < 1 || count > kFftMixSegs) return cudaErrorInvalidValue;
  m = FftLightMix{};
  m.nseg = count;
  for (int k = 0; k < count; k++) {
    const FftSegArgs &s = a[k];
    if (!ladder_size(s.xd.n) || s.frames < 1 || s.src.grid || !s.b.ctab || s.src.sd.nx != s.src.sd.ny) return cudaErrorInvalidValue;
    FftLightSeg &g = m.seg[k];
    g.xd = s.xd; g.src = s.src; g.hole = s.b.hole; g.part = s.b.part; g.ctab = s.b.ctab; g.fac = s.b.fac;
    g.bands = fft_hole_bands(s.xd.n); g.per_frame = s.xd.n * s.src.sd.nx; g.tblocks = (g.per_frame + 255) / 256;
    g.tiles = s.xd.n / (2 * plan_of(s.xd.n).lines);
    m.hf[k + 1] = m.hf[k] + s.frames * g.bands;
    m.ff[k + 1] = m.ff[k] + s.frames;
  }
  m.tf[0] = m.hf[count];
  for (int k = 0; k < count; k++) m.tf[k + 1] = m.tf[k] + a[k].frames * m.seg[k].tblocks;
  return cudaSuccess;
}

cudaError_t fft_pre_mixed_launch(const FftSegArgs *a, int count, cudaStream_t st) {
  FftLightMix m;
  if (cudaError_t e = light_mix(a, count, m)) return e;
  fft_pre_mixed_kernel<<<m.tf[count], 256, 0, st>>>(m);
  return cudaGetLastError();
}

cudaError_t fft_fac_mixed_launch(const FftSegArgs *a, int count, cudaStream_t st) {
  FftLightMix m;
  if (cudaError_t e = light_mix(a, count, m)) return e;
  fac_mixed_kernel<<<m.ff[count], 256, 0, st>>>(m);
  return cudaGetLastError();
}

cudaError_t fft_cols_mixed_launch(const FftSegArgs *a, int count, cudaStream_t st) {
  if (count < 1 || count > kFftMixSegs) return cudaErrorInvalidValue;
  static SmemOptIn opt;
  cudaError_t e;
  if ((e = opt.set(reinterpret_cast<const void *>(fft_cols_mixed_kernel), kFftSmemLadder)) != cudaSuccess) return e;
  FftColsMix m{};
  m.nseg = count;
  int smem = 0;
  for (int k = 0; k < count; k++) {
    const FftSegArgs &s = a[k];
    if (!ladder_size(s.xd.n) || s.frames < 1) return cudaErrorInvalidValue;
    FftColsSeg &g = m.seg[k];
    g.xd = s.xd; g.src = s.src; g.ctab = s.b.ctab; g.hole = s.b.hole; g.part = s.b.part; g.Y = s.b.Y; g.bands = fft_hole_bands(s.xd.n);
    m.first[k + 1] = m.first[k] + s.frames * (s.xd.n / (2 * plan_of(s.xd.n).lines));
    smem = cmax_i(smem, smem_bytes_of(s.xd.n));
  }
  fft_cols_mixed_kernel<<<m.first[count], kThreads, smem, st>>>(m);
  return cudaGetLastError();
}

cudaError_t fft_rows_mixed_launch(const FftSegArgs *a, int count, cudaStream_t st) {
  if (count < 1 || count > kFftMixSegs) return cudaErrorInvalidValue;
  static SmemOptIn opt;
  cudaError_t e;
  if ((e = opt.set(reinterpret_cast<const void *>(fft_rows_mixed_kernel), kFftSmemLadder)) != cudaSuccess) return e;
  FftRowsMix m{};
  m.nseg = count;
  int smem = 0;
  for (int k = 0; k < count; k++) {
    const FftSegArgs &s = a[k];
    if (!ladder_size(s.xd.n) || s.frames < 1 || !s.b.ymap || !s.b.err) return cudaErrorInvalidValue;
    FftRowsSeg &g = m.seg[k];
    const int L = plan_of(s.xd.n).lines;
    g.xd = s.xd; g.ymap = *s.b.ymap; g.fac = s.b.fac; g.tpos = s.b.tpos; g.C = s.b.C; g.err = s.b.err; g.need = s.b.need;
    m.first[k + 1] = m.first[k] + s.frames * ((s.xd.vrows + L - 1) / L);
    smem = cmax_i(smem, smem_bytes_of(s.xd.n));
  }
  fft_rows_mixed_kernel<<<m.first[count], kThreads, smem, st>>>(m);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- the sender's inverse (liblizard/src/lizard_phy.c:1134-1199)

// The half-plane spectrum's rows (v < vrows, each along u) inverse-transformed in place: S[v][x] = sum_u S[v][u]
// e^{+2 pi i u x / n}, as the conjugate of the forward transform of the conjugate. L rows a CTA.
template <int N>
__global__ void __launch_bounds__(kThreads, 3) enc_cols_kernel(EncFft e, float2 *S) {
  extern __shared__ __align__(16) unsigned char smraw[];
  constexpr int L = plan_of(N).lines, LSTR = lstride_of(N);
  float2 *buf = reinterpret_cast<float2 *>(smraw), *tw = buf + L * LSTR;
  const int tiles = (e.vrows + L - 1) / L, f = blockIdx.x / tiles, v0 = (blockIdx.x % tiles) * L, Lr = min(L, e.vrows - v0);
  for (int i = threadIdx.x; i < N; i += kThreads) tw[i] = e.tws[i];
  float2 *rows = S + ((int64_t)f * e.vrows + v0) * N;
  for (int t = threadIdx.x; t < Lr * N; t += kThreads) {
    const int l = t / N, p = t - l * N;
    const float2 z = rows[(int64_t)l * N + p];
    buf[l * LSTR + pad(p)] = make_float2(z.x, -z.y);
  }
  __syncthreads();
  fft_lines<N>(buf, tw, Lr);
  for (int t = threadIdx.x; t < Lr * N; t += kThreads) {
    const int l = t / N, p = t - l * N;
    const float2 z = buf[l * LSTR + pad(p)];
    rows[(int64_t)l * N + p] = make_float2(z.x, -z.y);
  }
}

// The picture's columns: 2L of them a CTA, columns xa = x0 + l and xb = x0 + L + l sharing line l as H_a + i H_b, each
// H the column's Hermitian completion over v (H(0) = 2 Re T(0), H(v) = T(v), H(n - v) = conj T(v) for 0 < v < vrows,
// zero between), inverse-transformed along v: the real part column xa, the imaginary part column xb
// (liblizard/src/lizard_phy.c:733-773 turn_pack). Then clipped at +-lim and mapped to 0.5 + v sc (clip_row, :775-782),
// into pic[y][x].
template <int N>
__global__ void __launch_bounds__(kThreads, 3) enc_rows_kernel(EncFft e, const float2 *T, float *pic) {
  extern __shared__ __align__(16) unsigned char smraw[];
  constexpr int L = plan_of(N).lines, LSTR = lstride_of(N), tiles = N / (2 * L);
  float2 *buf = reinterpret_cast<float2 *>(smraw), *tw = buf + L * LSTR;
  const int f = blockIdx.x / tiles, x0 = (blockIdx.x % tiles) * 2 * L;
  for (int i = threadIdx.x; i < N; i += kThreads) tw[i] = e.tws[i];
  const float2 *Tf = T + (int64_t)f * e.vrows * N;
  for (int t = threadIdx.x; t < L * N; t += kThreads) {   // l fastest: a row's 2L columns read together
    const int v = t / L, l = t - v * L;
    float2 z = make_float2(0.0f, 0.0f);
    if (v == 0) {
      const float2 a = Tf[x0 + l], b = Tf[x0 + L + l];
      z = make_float2(2.0f * a.x, 2.0f * b.x);
    } else if (v < e.vrows) {
      const float2 a = Tf[(int64_t)v * N + x0 + l], b = Tf[(int64_t)v * N + x0 + L + l];
      z = make_float2(a.x - b.y, a.y + b.x);
    } else if (v > N - e.vrows) {
      const int m = N - v;
      const float2 a = Tf[(int64_t)m * N + x0 + l], b = Tf[(int64_t)m * N + x0 + L + l];
      z = make_float2(a.x + b.y, b.x - a.y);
    }
    buf[l * LSTR + pad(v)] = make_float2(z.x, -z.y);
  }
  __syncthreads();
  fft_lines<N>(buf, tw, L);
  float *pf = pic + (int64_t)f * N * N;
  for (int t = threadIdx.x; t < L * N; t += kThreads) {
    const int y = t / L, l = t - y * L;
    const float2 z = buf[l * LSTR + pad(y)];
    float a = z.x, b = -z.y;
    a = a > e.lim ? e.lim : a;
    a = a < -e.lim ? -e.lim : a;
    b = b > e.lim ? e.lim : b;
    b = b < -e.lim ? -e.lim : b;
    pf[(int64_t)y * N + x0 + l] = __fadd_rn(0.5f, __fmul_rn(a, e.sc));   // rounded as clip_row rounds, unfused
    pf[(int64_t)y * N + x0 + L + l] = __fadd_rn(0.5f, __fmul_rn(b, e.sc));
  }
}

template <int N>
static cudaError_t enc_fft_launch_n(const EncFft &e, int frames, float2 *S, float *pic, cudaStream_t st) {
  constexpr int L = plan_of(N).lines, smem = (L * lstride_of(N) + N) * (int)sizeof(float2);
  static SmemOptIn opt_cols, opt_rows;
  cudaError_t err;
  if ((err = opt_cols.set(reinterpret_cast<const void *>(enc_cols_kernel<N>), smem)) != cudaSuccess ||
      (err = opt_rows.set(reinterpret_cast<const void *>(enc_rows_kernel<N>), smem)) != cudaSuccess)
    return err;
  enc_cols_kernel<N><<<frames * ((e.vrows + L - 1) / L), kThreads, smem, st>>>(e, S);
  enc_rows_kernel<N><<<frames * (N / (2 * L)), kThreads, smem, st>>>(e, S, pic);
  return cudaGetLastError();
}

cudaError_t enc_fft_launch(const EncFft &e, int frames, float2 *S, float *pic, cudaStream_t st) {
  switch (e.n) {
    case 384: return enc_fft_launch_n<384>(e, frames, S, pic, st);
    case 512: return enc_fft_launch_n<512>(e, frames, S, pic, st);
    case 768: return enc_fft_launch_n<768>(e, frames, S, pic, st);
    case 1024: return enc_fft_launch_n<1024>(e, frames, S, pic, st);
    case 1152: return enc_fft_launch_n<1152>(e, frames, S, pic, st);
    case 1280: return enc_fft_launch_n<1280>(e, frames, S, pic, st);
    case 1536: return enc_fft_launch_n<1536>(e, frames, S, pic, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t fft_launch(const FftDev &xd, int frames, const SrcDev &src, const FftBufs &b, int sms, cudaStream_t st) {
  switch (xd.n) {
    case 384: return fft_launch_n<384>(xd, frames, src, b, sms, st);
    case 512: return fft_launch_n<512>(xd, frames, src, b, sms, st);
    case 768: return fft_launch_n<768>(xd, frames, src, b, sms, st);
    case 1024: return fft_launch_n<1024>(xd, frames, src, b, sms, st);
    case 1152: return fft_launch_n<1152>(xd, frames, src, b, sms, st);
    case 1280: return fft_launch_n<1280>(xd, frames, src, b, sms, st);
    case 1536: return fft_launch_n<1536>(xd, frames, src, b, sms, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace lizg

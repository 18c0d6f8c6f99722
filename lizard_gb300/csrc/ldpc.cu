// Layered normalised min-sum LDPC decoding of the four LIZARD codes plus the block's CRC-32C check, on sm_103a.
//
// A codeword is decoded by a group of 1, 2 or 4 warps. A block row (a layer) has z = 128 checks that share no bit;
// in the scalar form lane l of the group's warp w takes checks l + 32 t of every layer (t over the warp's share of
// 0..3) and keeps their min1 / min2 / sign in registers between the layer's two passes; in the pair form a thread
// takes checks i and i + 64 as the two 16-bit halves of one register (the layout is described at layer_pair). The
// codeword's posteriors (int16) and check-to-bit messages (int8) live in the group's slice of shared memory for the
// whole decode; global memory is touched once to read the LLRs and once to write the packed hard bits, so the
// kernel is bound by the ALU pipe (every min/max form issues there) and shared-memory latency, not by HBM.
//
// Persistent grid: one CTA per SM (its shared memory holds as many codewords as fit), groups pull codeword indices
// from a work counter, so codewords that stop early free their group for the next one. Each code has several
// variants (warps a codeword, registers or a loop over the row's slots, scalar or pair form), all bit-identical;
// one per code runs, chosen by timing on the device or by hand.
//
// Arithmetic: the reference's four-times kernel, liblizard/src/ldpc.c:340-423 (and its NEON original, 300-328):
// the extrinsic L - R saturated to a byte held at [-127, 127]; min1/min2 over byte magnitudes; (x * 13) >> 4 capped
// at 127; an edge whose magnitude is min1 takes min2; no posterior clamp. Row 0's missing previous parity bit is a
// certain zero of 8191 (liblizard/src/ldpc.c:655-676). Stop rule: liblizard/src/ldpc.c:1128-1145.
#include <cuda_runtime.h>
#include <stdint.h>
#include "lizard_codes.h"
#include "lizg_internal.h"
#include "lizard_gb300.h"
#include <cmath>
#include <mutex>
#include <random>
#include <string>
#include <vector>

namespace lizg {

// Per-code compile-time shape: block rows, codeword bits, data bits, data circulants, slots (data circulants plus
// two staircase slots a row), and the warps a CTA runs (as many codeword states as fit in 227 KB of shared memory).
template <int C> struct Code;
// NDMAX: the most data circulants any block row has. WARPS: codewords a CTA holds. A kernel variant also fixes WPC,
// the warps a codeword (lane l of warp w of a codeword takes checks l + 32 t, t = w (4 / WPC) .. (w + 1) (4 / WPC) - 1,
// of every layer), and the layer form (registers, or the loop form that recomputes the extrinsics).
template <> struct Code<0> { static constexpr int MB = 5, N = 4608, K = 3968, NDATA = 103, NDMAX = 21, WARPS = 9; };
template <> struct Code<1> { static constexpr int MB = 10, N = 5120, K = 3840, NDATA = 132, NDMAX = 14, WARPS = 7; };
template <> struct Code<2> { static constexpr int MB = 15, N = 5760, K = 3840, NDATA = 146, NDMAX = 10, WARPS = 6; };
template <> struct Code<3> { static constexpr int MB = 30, N = 7680, K = 3840, NDATA = 150, NDMAX = 5, WARPS = 5; };

template <int C> __host__ __device__ constexpr int slots() { return Code<C>::NDATA + 2 * Code<C>::MB; }
// A warp's state: posteriors (N int16) then messages (slots x 128 int8), rounded to 16 bytes.
template <int C> __host__ __device__ constexpr int warp_bytes() { return (Code<C>::N * 2 + slots<C>() * 128 + 15) & ~15; }
constexpr int kCrcBytes = (256 + 32 + 1) * 4 + 12;   // table, per-lane shifts, init term; padded to 16
template <int C> constexpr int cta_smem() { return kCrcBytes + Code<C>::WARPS * warp_bytes<C>(); }
template <int C, int WPC> __host__ __device__ constexpr int cta_threads() { return Code<C>::WARPS * WPC * 32; }

static_assert(cta_smem<0>() <= 227 * 1024, "7/8 state does not fit");
static_assert(cta_smem<1>() <= 227 * 1024, "3/4 state does not fit");
static_assert(cta_smem<2>() <= 227 * 1024, "2/3 state does not fit");
static_assert(cta_smem<3>() <= 227 * 1024, "1/2 state does not fit");

// Block-row tables of the four codes: rowptr and (col << 8 | shift) circulants, read warp-uniformly (broadcast).
struct DevCode { int rowptr[31]; uint16_t circ[152]; };
__constant__ DevCode c_codes[4];
// CRC-32C shift constants: x^(8 (476 - end_l)) mod P for lane l's 15-byte chunk, then the all-ones init's term.
__constant__ uint32_t c_crc_shift[33];

constexpr uint32_t kCrcPoly = 0x82F63B78u;   // CRC-32C, reflected
constexpr int kBlockBytes = LIZG_BLOCK_BYTES;

// a * b mod P in the reflected representation (bit 31 is x^0).
__device__ __forceinline__ uint32_t gf_mul(uint32_t a, uint32_t b) {
  uint32_t p = 0;
#pragma unroll
  for (int i = 0; i < 32; i++) {
    p ^= b & (0u - ((a >> (31 - i)) & 1u));
    b = (b >> 1) ^ (kCrcPoly & (0u - (b & 1u)));
  }
  return p;
}

__device__ __forceinline__ int sat127(int v) { return max(-127, min(127, v)); }

// One layer (block row r). Lane l takes checks i = l + 32 t, t = 0..3 (TW of them from T0 at a time). Pass 1 loads every slot's
// extrinsic q = L - R into registers (the row's circulants unrolled to the code's widest row, so the register arrays
// are statically indexed) and folds them into two interleaved min1/min2 chains a check, merged at the end; pass 2
// makes the messages and posteriors from the registers without reading shared memory again.
template <int C, int TW>
__device__ __forceinline__ void layer_part(int16_t *L, int8_t *R, int r, int lane, int T0, int p0, int nd, const int *colb, const int *sh) {
  using T = Code<C>;
  constexpr int NDM = T::NDMAX;
  int8_t *Rr = R + (p0 + 2 * r) * 128 + lane;
  int16_t *Lp = L + T::K;
  int q[NDM + 2][TW];
#pragma unroll
  for (int e = 0; e < NDM; e++) {
    if (e < nd) {
#pragma unroll
      for (int t = 0; t < TW; t++) q[e][t] = L[colb[e] + ((lane + 32 * (T0 + t) - sh[e]) & 127)] - Rr[e * 128 + 32 * (T0 + t)];
    }
  }
  const int prev = r > 0 ? (r - 1) * 128 + lane : (T::MB - 1) * 128 + lane - 1;
#pragma unroll
  for (int t = 0; t < TW; t++) {
    const int tt = T0 + t;
    q[NDM][t] = (r == 0 && lane + 32 * tt == 0) ? 8191 : Lp[prev + 32 * tt] - Rr[nd * 128 + 32 * tt];
    q[NDM + 1][t] = Lp[r * 128 + lane + 32 * tt] - Rr[(nd + 1) * 128 + 32 * tt];
  }
  int m1[TW], m2[TW], sg[TW];
#pragma unroll
  for (int t = 0; t < TW; t++) {
    int a1 = min(abs(q[NDM][t]), 127), a2 = 255, b1 = min(abs(q[NDM + 1][t]), 127), b2 = 255, s = q[NDM][t] ^ q[NDM + 1][t];
#pragma unroll
    for (int e = 0; e < NDM; e++) {
      if (e < nd) {
        const int a = min(abs(q[e][t]), 127);
        s ^= q[e][t];
        if (e & 1) { b2 = min(b2, max(b1, a)); b1 = min(b1, a); }
        else { a2 = min(a2, max(a1, a)); a1 = min(a1, a); }
      }
    }
    m1[t] = min(a1, b1);
    m2[t] = min(max(a1, b1), min(a2, b2));
    sg[t] = s;
  }
  int s1[TW], s2[TW];
#pragma unroll
  for (int t = 0; t < TW; t++) {
    const int x1 = min(127, (m1[t] * 13) >> 4), x2 = min(127, (m2[t] * 13) >> 4);
    s1[t] = sg[t] < 0 ? -x1 : x1;     // the check's sign folded in
    s2[t] = sg[t] < 0 ? -x2 : x2;
  }
  auto msg = [&](int v, int t) {
    const int a = min(abs(v), 127);
    const int m = (a == m1[t]) ? s2[t] : s1[t];
    return v < 0 ? -m : m;
  };
#pragma unroll
  for (int e = 0; e < NDM; e++) {
    if (e < nd) {
#pragma unroll
      for (int t = 0; t < TW; t++) {
        const int m = msg(q[e][t], t);
        Rr[e * 128 + 32 * (T0 + t)] = (int8_t)m;
        L[colb[e] + ((lane + 32 * (T0 + t) - sh[e]) & 127)] = (int16_t)(q[e][t] + m);
      }
    }
  }
#pragma unroll
  for (int t = 0; t < TW; t++) {
    const int tt = T0 + t;
    if (!(r == 0 && lane + 32 * tt == 0)) {
      const int m = msg(q[NDM][t], t);
      Rr[nd * 128 + 32 * tt] = (int8_t)m;
      Lp[prev + 32 * tt] = (int16_t)(q[NDM][t] + m);
    }
    const int m = msg(q[NDM + 1][t], t);
    Rr[(nd + 1) * 128 + 32 * tt] = (int8_t)m;
    Lp[r * 128 + lane + 32 * tt] = (int16_t)(q[NDM + 1][t] + m);
  }
}

template <int C, int TW>
__device__ __forceinline__ void layer(int16_t *L, int8_t *R, int r, int lane, int T0) {
  constexpr int NDM = Code<C>::NDMAX;
  const DevCode &cd = c_codes[C];
  const int p0 = cd.rowptr[r], nd = cd.rowptr[r + 1] - p0;
  int colb[NDM], sh[NDM];
#pragma unroll
  for (int e = 0; e < NDM; e++) {
    if (e < nd) { const int cs = cd.circ[p0 + e]; colb[e] = (cs >> 8) * 128; sh[e] = cs & 255; }
  }
  layer_part<C, TW>(L, R, r, lane, T0, p0, nd, colb, sh);
}

// The same layer with the row's slots in a loop, the extrinsics recomputed in pass 2: fewer registers, which the
// 7/8 code's 21-circulant rows need.
template <int C, int TW>
__device__ __forceinline__ void layer_loop(int16_t *L, int8_t *R, int r, int lane, int T0) {
  using T = Code<C>;
  const DevCode &cd = c_codes[C];
  const int p0 = cd.rowptr[r], nd = cd.rowptr[r + 1] - p0;
  int8_t *Rr = R + (p0 + 2 * r) * 128;
  int16_t *Lp = L + T::K;
  int m1[TW], m2[TW], sg[TW];
#pragma unroll
  for (int q = 0; q < TW; q++) { m1[q] = 255; m2[q] = 255; sg[q] = 0; }
  // Pass 1: the extrinsics' bytes, their signs and two least magnitudes.
  auto acc = [&](int q, int v) {
    const int b = sat127(v), a = abs(b);
    sg[q] ^= b;
    m2[q] = min(m2[q], max(m1[q], a));
    m1[q] = min(m1[q], a);
  };
  for (int e = 0; e < nd; e++) {
    const int cs = cd.circ[p0 + e], sh = cs & 255;
    const int16_t *col = L + (cs >> 8) * 128;
    const int8_t *Re = Rr + e * 128;
#pragma unroll
    for (int q = 0; q < TW; q++) { const int i = lane + 32 * (T0 + q); acc(q, col[(i - sh) & 127] - Re[i]); }
  }
  {
    const int8_t *Re = Rr + nd * 128;
#pragma unroll
    for (int q = 0; q < TW; q++) {
      const int i = lane + 32 * (T0 + q);
      int v;
      if (r > 0) v = Lp[(r - 1) * 128 + i] - Re[i];
      else v = (i == 0) ? 8191 : Lp[(T::MB - 1) * 128 + i - 1] - Re[i];
      acc(q, v);
    }
    Re += 128;
#pragma unroll
    for (int q = 0; q < TW; q++) { const int i = lane + 32 * (T0 + q); acc(q, Lp[r * 128 + i] - Re[i]); }
  }
  int s1[TW], s2[TW];
#pragma unroll
  for (int q = 0; q < TW; q++) { s1[q] = min(127, (m1[q] * 13) >> 4); s2[q] = min(127, (m2[q] * 13) >> 4); }
  // Pass 2: new messages and posteriors.
  auto upd = [&](int q, int v, int8_t *rp, int16_t *lp) {
    const int b = sat127(v), a = abs(b);
    const int mag = (a == m1[q]) ? s2[q] : s1[q];
    const int m = ((sg[q] ^ b) < 0) ? -mag : mag;
    *rp = (int8_t)m;
    *lp = (int16_t)(v + m);
  };
  for (int e = 0; e < nd; e++) {
    const int cs = cd.circ[p0 + e], sh = cs & 255;
    int16_t *col = L + (cs >> 8) * 128;
    int8_t *Re = Rr + e * 128;
#pragma unroll
    for (int q = 0; q < TW; q++) {
      const int i = lane + 32 * (T0 + q);
      int16_t *lp = col + ((i - sh) & 127);
      upd(q, *lp - Re[i], Re + i, lp);
    }
  }
  {
    int8_t *Re = Rr + nd * 128;
#pragma unroll
    for (int q = 0; q < TW; q++) {
      const int i = lane + 32 * (T0 + q);
      if (r > 0) { int16_t *lp = Lp + (r - 1) * 128 + i; upd(q, *lp - Re[i], Re + i, lp); }
      else if (i != 0) { int16_t *lp = Lp + (T::MB - 1) * 128 + i - 1; upd(q, *lp - Re[i], Re + i, lp); }
    }
    Re += 128;
#pragma unroll
    for (int q = 0; q < TW; q++) { const int i = lane + 32 * (T0 + q); int16_t *lp = Lp + r * 128 + i; upd(q, *lp - Re[i], Re + i, lp); }
  }
}

// Violated checks over the whole code, summed over the warp (count = 1); or, with count = 0, 1 as soon as a block
// row holds a violated check and 0 if none does (the reference's layers_clear, liblizard/src/ldpc.c:930-949), the
// rows tested in the order the iteration updated them (rev: last row first), which finds a violated one soonest.
template <int C, int TW>
__device__ __forceinline__ int unsat(const int16_t *L, int lane, int T0, int count, int rev) {
  using T = Code<C>;
  constexpr int NDM = T::NDMAX;
  const DevCode &cd = c_codes[C];
  const int16_t *Lp = L + T::K;
  int bad = 0;
  for (int k = 0; k < T::MB; k++) {
    const int r = rev ? T::MB - 1 - k : k;
    const int p0 = cd.rowptr[r], nd = cd.rowptr[r + 1] - p0;
    const int prev = r > 0 ? (r - 1) * 128 + lane : (T::MB - 1) * 128 + lane - 1;
    int x[TW];
#pragma unroll
    for (int t = 0; t < TW; t++) { const int tt = T0 + t; x[t] = Lp[r * 128 + lane + 32 * tt] ^ ((r == 0 && lane + 32 * tt == 0) ? 0 : Lp[prev + 32 * tt]); }
#pragma unroll
    for (int e = 0; e < NDM; e++) {
      if (e < nd) {
        const int cs = cd.circ[p0 + e], cb = (cs >> 8) * 128, sh = cs & 255;
#pragma unroll
        for (int t = 0; t < TW; t++) x[t] ^= L[cb + ((lane + 32 * (T0 + t) - sh) & 127)];
      }
    }
#pragma unroll
    for (int t = 0; t < TW; t++) bad += x[t] < 0;
    if (!count && __any_sync(0xffffffffu, bad)) return 1;
  }
  return count ? __reduce_add_sync(0xffffffffu, bad) : 0;
}

// ---------------------------------------------------------------- the 16-bit pair form
//
// Checks i and i + 64 of a layer (i < 64) share a thread, their extrinsics, minima, signs and messages riding in the
// two 16-bit halves of one 32-bit register (low half check i), so one 16x2 instruction serves two checks. Every
// 128-column block of posteriors is stored as 64 words, word w = (column w, column w + 64): the columns a circulant
// of shift sh gives checks i and i + 64, (i - sh) mod 128 and that plus 64, always share a word, in check order when
// (i - sh) mod 128 < 64 and swapped otherwise; one byte permute puts them in check order and the same one puts them
// back. A slot's messages are 64 byte pairs (low byte check i). 16x2 add/subtract and min/max are native on sm_103a;
// the absolute value and equality tests are built from them (the 16x2 abs and compare forms are slow sequences).
// The arithmetic per check is that of layer_part, half for half.

__device__ __forceinline__ uint32_t add2(uint32_t a, uint32_t b) { uint32_t d; asm("add.s16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b)); return d; }
__device__ __forceinline__ uint32_t sub2(uint32_t a, uint32_t b) { return __vsub2(a, b); }
__device__ __forceinline__ uint32_t minu2(uint32_t a, uint32_t b) { uint32_t d; asm("min.u16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b)); return d; }
__device__ __forceinline__ uint32_t maxu2(uint32_t a, uint32_t b) { uint32_t d; asm("max.u16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b)); return d; }
__device__ __forceinline__ uint32_t maxs2(uint32_t a, uint32_t b) { uint32_t d; asm("max.s16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b)); return d; }
// byte permute; a selector nibble with bit 3 set replicates the sign of the byte its low bits name
__device__ __forceinline__ uint32_t prmt(uint32_t a, uint32_t s) { uint32_t d; asm("prmt.b32 %0, %1, 0, %2;" : "=r"(d) : "r"(a), "r"(s)); return d; }

constexpr uint32_t kKeep = 0x3210u, kSwap = 0x1032u;   // halves as they are; halves exchanged
constexpr uint32_t kSext = 0x9180u;                    // two int8 (bytes 0, 1) -> two int16
constexpr uint32_t kSign = 0xBB99u;                    // each half's sign spread over the half
constexpr uint32_t kPack = 0x0020u;                    // each half's low byte -> bytes 0, 1
constexpr uint32_t k127 = 0x007F007Fu, k255 = 0x00FF00FFu;

// Index of code-order bit v (data bits, then parity bit k + c, c = i mb + r) in the pair layout of the posteriors.
template <int C>
__device__ __forceinline__ int lpos_pair(int v) {
  using T = Code<C>;
  if (v < T::K) return (v & ~127) + ((v & 63) << 1) + ((v >> 6) & 1);
  const int c = v - T::K, r = c % T::MB, i = c / T::MB;
  return T::K + r * 128 + ((i & 63) << 1) + (i >> 6);
}

// min(|q|, 127) of both halves (q's halves within +-32767)
__device__ __forceinline__ uint32_t mag127(uint32_t q) { return minu2(maxs2(q, sub2(0u, q)), k127); }

// The check pair's state after pass 1: least and second magnitudes, their scaled messages, the sign parity.
struct PairCheck {
  uint32_t s2, dl, nm1_7, sg;
  __device__ __forceinline__ void finish(uint32_t a1, uint32_t a2, uint32_t b1, uint32_t b2, uint32_t s) {
    const uint32_t m1 = minu2(a1, b1), m2 = minu2(maxu2(a1, b1), minu2(a2, b2));
    // (m * 13) >> 4 a half: m <= 127, so m * 13 stays inside its half and the result under 104 (the cap at 127
    // never binds); the shift's spill from the high half into the low half's top bits is masked off
    const uint32_t s1 = ((m1 * 13u) >> 4) & 0x0FFF0FFFu;
    s2 = ((m2 * 13u) >> 4) & 0x0FFF0FFFu;
    dl = s2 - s1;             // both halves >= 0: no borrow between them
    nm1_7 = 0u - (m1 << 7);
    sg = s;
  }
  // The message to an edge of extrinsic q (halves): s2 where min(|q|, 127) is the least magnitude, else s1
  // ((a - m1) << 7 is 0 there and at least 128 > dl elsewhere), negated where the other edges' signs multiply to -1.
  __device__ __forceinline__ uint32_t msg(uint32_t q) const {
    const uint32_t t = minu2(dl, (mag127(q) << 7) + nm1_7);
    const uint32_t mag = s2 - t;
    const uint32_t neg = prmt(q ^ sg, kSign);
    return sub2(mag ^ neg, neg);
  }
};

__device__ __forceinline__ void fold(uint32_t &m1, uint32_t &m2, uint32_t a) {
  m2 = minu2(m2, maxu2(m1, a));
  m1 = minu2(m1, a);
}

// One layer in the pair form, the row's slots unrolled to the code's widest row (registers hold each edge's
// extrinsics, word index and permute; the magnitudes are recomputed in pass 2). Pair ip = lane + 32 (P0 + p).
template <int C, int NP>
__device__ __forceinline__ void layer_pair(int16_t *L, int8_t *R, int r, int lane, int P0) {
  using T = Code<C>;
  constexpr int NDM = T::NDMAX;
  const DevCode &cd = c_codes[C];
  const int p0 = cd.rowptr[r], nd = cd.rowptr[r + 1] - p0;
  uint32_t *Lw = reinterpret_cast<uint32_t *>(L);
  uint32_t *Pw = Lw + T::K / 2;   // parity words: row r's pair i at r * 64 + i
  uint16_t *Rh = reinterpret_cast<uint16_t *>(R) + (p0 + 2 * r) * 64;
  uint32_t q[NDM][NP], sel[NDM][NP];
  int w[NDM][NP];
  uint32_t a1[NP], a2[NP], b1[NP], b2[NP], sg[NP], qp[NP], qo[NP], lp[NP];
  int wp[NP];
  uint32_t sp[NP];
#pragma unroll
  for (int p = 0; p < NP; p++) {
    const int ip = lane + 32 * (P0 + p);
    // the staircase: previous row's parity (row 0: the last row's, one check back; check 0 has none and takes a
    // certain zero of 8191), then this row's
    wp[p] = r > 0 ? (r - 1) * 64 + ip : (T::MB - 1) * 64 + ((ip - 1) & 63);
    sp[p] = (r == 0 && ip == 0) ? kSwap : kKeep;
    lp[p] = prmt(Pw[wp[p]], sp[p]);
    qp[p] = sub2(lp[p], prmt(Rh[nd * 64 + ip], kSext));
    if (r == 0 && ip == 0) qp[p] = (qp[p] & 0xFFFF0000u) | 8191u;
    qo[p] = sub2(Pw[r * 64 + ip], prmt(Rh[(nd + 1) * 64 + ip], kSext));
    a1[p] = mag127(qp[p]); a2[p] = k255;
    b1[p] = mag127(qo[p]); b2[p] = k255;
    sg[p] = qp[p] ^ qo[p];
  }
#pragma unroll
  for (int e = 0; e < NDM; e++) {
    if (e < nd) {
      const int cs = cd.circ[p0 + e], colw = (cs >> 8) * 64, sh = cs & 255;
#pragma unroll
      for (int p = 0; p < NP; p++) {
        const int d = (lane + 32 * (P0 + p) - sh) & 127;
        w[e][p] = colw | (d & 63);
        sel[e][p] = (d & 64) ? kSwap : kKeep;
        q[e][p] = sub2(prmt(Lw[w[e][p]], sel[e][p]), prmt(Rh[e * 64 + lane + 32 * (P0 + p)], kSext));
        sg[p] ^= q[e][p];
        if (e & 1) fold(b1[p], b2[p], mag127(q[e][p]));
        else fold(a1[p], a2[p], mag127(q[e][p]));
      }
    }
  }
  PairCheck ck[NP];
#pragma unroll
  for (int p = 0; p < NP; p++) ck[p].finish(a1[p], a2[p], b1[p], b2[p], sg[p]);
#pragma unroll
  for (int e = 0; e < NDM; e++) {
    if (e < nd) {
#pragma unroll
      for (int p = 0; p < NP; p++) {
        const uint32_t m = ck[p].msg(q[e][p]);
        Rh[e * 64 + lane + 32 * (P0 + p)] = (uint16_t)prmt(m, kPack);
        Lw[w[e][p]] = prmt(add2(q[e][p], m), sel[e][p]);
      }
    }
  }
#pragma unroll
  for (int p = 0; p < NP; p++) {
    const int ip = lane + 32 * (P0 + p);
    uint32_t m = ck[p].msg(qp[p]);
    Rh[nd * 64 + ip] = (uint16_t)prmt(m, kPack);   // check 0's half of row 0 is never read back
    uint32_t v = add2(qp[p], m);
    if (r == 0 && ip == 0) v = (v & 0xFFFF0000u) | (lp[p] & 0xFFFFu);   // that column belongs to no check here
    Pw[wp[p]] = prmt(v, sp[p]);
    m = ck[p].msg(qo[p]);
    Rh[(nd + 1) * 64 + ip] = (uint16_t)prmt(m, kPack);
    Pw[r * 64 + ip] = add2(qo[p], m);
  }
}

// The same with the row's data slots in a loop, the extrinsics reloaded and recomputed in pass 2 (the 7/8 code's
// 21-circulant rows).
template <int C, int NP>
__device__ __forceinline__ void layer_pair_loop(int16_t *L, int8_t *R, int r, int lane, int P0) {
  using T = Code<C>;
  const DevCode &cd = c_codes[C];
  const int p0 = cd.rowptr[r], nd = cd.rowptr[r + 1] - p0;
  uint32_t *Lw = reinterpret_cast<uint32_t *>(L);
  uint32_t *Pw = Lw + T::K / 2;
  uint16_t *Rh = reinterpret_cast<uint16_t *>(R) + (p0 + 2 * r) * 64;
  uint32_t a1[NP], a2[NP], b1[NP], b2[NP], sg[NP], qp[NP], qo[NP], lp[NP];
  int wp[NP];
  uint32_t sp[NP];
#pragma unroll
  for (int p = 0; p < NP; p++) {
    const int ip = lane + 32 * (P0 + p);
    wp[p] = r > 0 ? (r - 1) * 64 + ip : (T::MB - 1) * 64 + ((ip - 1) & 63);
    sp[p] = (r == 0 && ip == 0) ? kSwap : kKeep;
    lp[p] = prmt(Pw[wp[p]], sp[p]);
    qp[p] = sub2(lp[p], prmt(Rh[nd * 64 + ip], kSext));
    if (r == 0 && ip == 0) qp[p] = (qp[p] & 0xFFFF0000u) | 8191u;
    qo[p] = sub2(Pw[r * 64 + ip], prmt(Rh[(nd + 1) * 64 + ip], kSext));
    a1[p] = mag127(qp[p]); a2[p] = k255;
    b1[p] = mag127(qo[p]); b2[p] = k255;
    sg[p] = qp[p] ^ qo[p];
  }
  for (int e = 0; e < nd; e++) {
    const int cs = cd.circ[p0 + e], colw = (cs >> 8) * 64, sh = cs & 255;
#pragma unroll
    for (int p = 0; p < NP; p++) {
      const int d = (lane + 32 * (P0 + p) - sh) & 127;
      const uint32_t q = sub2(prmt(Lw[colw | (d & 63)], (d & 64) ? kSwap : kKeep), prmt(Rh[e * 64 + lane + 32 * (P0 + p)], kSext));
      sg[p] ^= q;
      fold(a1[p], a2[p], mag127(q));
    }
  }
  PairCheck ck[NP];
#pragma unroll
  for (int p = 0; p < NP; p++) ck[p].finish(a1[p], a2[p], b1[p], b2[p], sg[p]);
  for (int e = 0; e < nd; e++) {
    const int cs = cd.circ[p0 + e], colw = (cs >> 8) * 64, sh = cs & 255;
#pragma unroll
    for (int p = 0; p < NP; p++) {
      const int d = (lane + 32 * (P0 + p) - sh) & 127, wi = colw | (d & 63);
      const uint32_t sl = (d & 64) ? kSwap : kKeep;
      uint16_t *rp = Rh + e * 64 + lane + 32 * (P0 + p);
      const uint32_t q = sub2(prmt(Lw[wi], sl), prmt(*rp, kSext));
      const uint32_t m = ck[p].msg(q);
      *rp = (uint16_t)prmt(m, kPack);
      Lw[wi] = prmt(add2(q, m), sl);
    }
  }
#pragma unroll
  for (int p = 0; p < NP; p++) {
    const int ip = lane + 32 * (P0 + p);
    uint32_t m = ck[p].msg(qp[p]);
    Rh[nd * 64 + ip] = (uint16_t)prmt(m, kPack);
    uint32_t v = add2(qp[p], m);
    if (r == 0 && ip == 0) v = (v & 0xFFFF0000u) | (lp[p] & 0xFFFFu);
    Pw[wp[p]] = prmt(v, sp[p]);
    m = ck[p].msg(qo[p]);
    Rh[(nd + 1) * 64 + ip] = (uint16_t)prmt(m, kPack);
    Pw[r * 64 + ip] = add2(qo[p], m);
  }
}

// unsat in the pair form: the sign bits (15 and 31) of the XOR of a check pair's posteriors.
template <int C, int NP>
__device__ __forceinline__ int unsat_pair(const int16_t *L, int lane, int P0, int count, int rev) {
  using T = Code<C>;
  constexpr int NDM = T::NDMAX;
  const DevCode &cd = c_codes[C];
  const uint32_t *Lw = reinterpret_cast<const uint32_t *>(L);
  const uint32_t *Pw = Lw + T::K / 2;
  int bad = 0;
  for (int k = 0; k < T::MB; k++) {
    const int r = rev ? T::MB - 1 - k : k;
    const int p0 = cd.rowptr[r], nd = cd.rowptr[r + 1] - p0;
    uint32_t x[NP];
#pragma unroll
    for (int p = 0; p < NP; p++) {
      const int ip = lane + 32 * (P0 + p);
      uint32_t prev;
      if (r > 0) prev = Pw[(r - 1) * 64 + ip];
      else prev = ip == 0 ? prmt(Pw[(T::MB - 1) * 64 + 63], kSwap) & 0xFFFF0000u : Pw[(T::MB - 1) * 64 + ip - 1];
      x[p] = Pw[r * 64 + ip] ^ prev;
    }
#pragma unroll
    for (int e = 0; e < NDM; e++) {
      if (e < nd) {
        const int cs = cd.circ[p0 + e], colw = (cs >> 8) * 64, sh = cs & 255;
#pragma unroll
        for (int p = 0; p < NP; p++) {
          const int d = (lane + 32 * (P0 + p) - sh) & 127;
          x[p] ^= prmt(Lw[colw | (d & 63)], (d & 64) ? kSwap : kKeep);
        }
      }
    }
#pragma unroll
    for (int p = 0; p < NP; p++) bad += __popc(x[p] & 0x80008000u);
    if (!count && __any_sync(0xffffffffu, bad)) return 1;
  }
  return count ? __reduce_add_sync(0xffffffffu, bad) : 0;
}

// The WPC warps of one codeword meet here between layers (a named barrier a codeword; 0 is __syncthreads').
template <int WPC>
__device__ __forceinline__ void group_sync(int g) {
  if (WPC == 1) __syncwarp();
  else asm volatile("bar.sync %0, %1;" ::"r"(g + 1), "r"(WPC * 32) : "memory");
}

// Index of code-order bit v in the posteriors: the pair layout, or data bits in order then parity bit k + c
// (c = i mb + r) at [r][i].
template <int C, bool PAIR>
__device__ __forceinline__ int lpos(int v) {
  using T = Code<C>;
  if (PAIR) return lpos_pair<C>(v);
  if (v < T::K) return v;
  const int c = v - T::K;
  return T::K + (c % T::MB) * 128 + c / T::MB;
}

// One codeword (item `item` of the launch: a codeword of the batch's list, or in receiver mode block `item` of tier
// `tier` across the frames) decoded by the calling thread's group of WPC warps in its slice of shared memory (the
// posteriors, then the messages); red: the group's WPC slots for the unsatisfied-check count. Ends with the group
// synchronised (a declined block returns at once, having touched nothing of the group's).
template <int C, int WPC, bool LOOP, bool PAIR>
__device__ __forceinline__ void decode_item(const LdpcLaunch &a, int tier, int item, uint8_t *slice, const uint32_t *crc_tab,
                                            const uint32_t *crc_k, int *red, int g) {
  using T = Code<C>;
  constexpr int CPL = 4 / WPC, GT = WPC * 32, NP = PAIR ? 2 / WPC : 1;
  static_assert(!PAIR || WPC <= 2, "the pair form runs 64 check pairs a layer on one or two warps");
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, sub = warp % WPC, tg = sub * 32 + lane, t0 = sub * CPL;
  int16_t *L = reinterpret_cast<int16_t *>(slice);
  int8_t *R = reinterpret_cast<int8_t *>(L + T::N);
  int cw, gi = 0;
  int64_t off = 0;
  if (a.rx.llrf) {
    // Receiver mode: item -> (frame, block) of this tier. A declined block is not tried (its -2). Otherwise its
    // slots' soft values go through the bit map into codeword order, whitening taken off by sign, the never-sent
    // bits at 0 and the 7/8 code's known zeros past the block's 3840 bits at 127
    // (liblizard/src/lizard_phy.c:156-192, 1818-1823).
    const int f = item / a.fd.tier_blocks[tier], b = a.fd.tier_first[tier] + item % a.fd.tier_blocks[tier];
    gi = f * a.fd.blocks + b;
    cw = gi;
    if (a.rx.decl[gi]) {
      if (tg == 0) { a.its[gi] = -2; a.ok[gi] = 0; }
      return;
    }
    const int s0 = a.fd.block_slot[b], nt = a.fd.tier_nt[tier];
    const int8_t *sl = a.rx.llrf + f * a.rx.llr_stride + s0;
    const uint8_t *wh = a.fd.white + s0;
    const int16_t *perm = a.fd.perm[tier];
    for (int i = tg; i < nt; i += GT) {
      const int v = perm[i];
      const int8_t x = sl[i];
      const int8_t y = wh[i] ? (int8_t)(-x) : x;
      L[lpos<C, PAIR>(v)] = y;
    }
    for (int v = LIZG_INFO_BITS + tg; v < T::K; v += GT) L[lpos<C, PAIR>(v)] = 127;
  } else {
    cw = a.list[item];
    off = a.off[cw];
    // LLRs in: data bits in code order, parity bit k + c (c = i mb + r) at [r][i].
    const int4 *src = reinterpret_cast<const int4 *>(a.llr + off);
    for (int t = tg; t < T::N / 16; t += GT) {
      const int4 w = __ldg(src + t);
      const int8_t *bb = reinterpret_cast<const int8_t *>(&w);
#pragma unroll
      for (int j = 0; j < 16; j++) {
        L[lpos<C, PAIR>(t * 16 + j)] = bb[j];
      }
    }
  }
  // messages cleared
  int4 *rz = reinterpret_cast<int4 *>(R);
  for (int t = tg; t < slots<C>() * 128 / 16; t += GT) rz[t] = make_int4(0, 0, 0, 0);
  group_sync<WPC>(g);

  int used = -1, first = 0;
  for (int it = 0; it < a.max_iter; it++) {
    for (int step = 0; step < T::MB; step++) {
      const int r = (it & 1) ? T::MB - 1 - step : step;
      if (PAIR && LOOP) layer_pair_loop<C, NP>(L, R, r, lane, sub * NP);
      else if (PAIR) layer_pair<C, NP>(L, R, r, lane, sub * NP);
      else if (LOOP) layer_loop<C, CPL>(L, R, r, lane, t0);
      else layer<C, CPL>(L, R, r, lane, t0);
      group_sync<WPC>(g);
    }
    // the count only where the stall rule reads it (after the first iteration and at stall_it), else a clear test
    const bool counted = a.stall_it > 1 && (it == 0 || it == a.stall_it - 1);
    int bad = PAIR ? unsat_pair<C, NP>(L, lane, sub * NP, counted, it & 1) : unsat<C, CPL>(L, lane, t0, counted, it & 1);
    if (WPC > 1) {
      if (lane == 0) red[sub] = bad;
      group_sync<WPC>(g);
      bad = 0;
#pragma unroll
      for (int w = 0; w < WPC; w++) bad += red[w];
      group_sync<WPC>(g);
    }
    if (bad == 0) { used = it + 1; break; }
    if (a.stall_it > 1 && it == a.stall_it - 1) {
      if ((float)bad > __fmul_rn(a.stall_ratio, (float)first)) { used = -3; break; }
    } else if (it == 0 && a.stall_it > 1) first = bad;
  }

  // Hard bits packed MSB first into the message area (no longer needed), then the CRC over the block's bytes.
  uint8_t *pk = reinterpret_cast<uint8_t *>(R);
  for (int j = tg; j < T::N / 8; j += GT) {
    int byte = 0;
#pragma unroll
    for (int t = 0; t < 8; t++) {
      const int v = 8 * j + t;
      const int16_t x = L[lpos<C, PAIR>(v)];
      byte = (byte << 1) | (x < 0);
    }
    pk[j] = (uint8_t)byte;
  }
  group_sync<WPC>(g);
  if (sub == 0) {
    const int s0 = 15 * lane, s1 = min(s0 + 15, kBlockBytes);
    uint32_t c = 0;
    for (int j = s0; j < s1; j++) c = crc_tab[(c ^ pk[j]) & 255u] ^ (c >> 8);
    c = gf_mul(c, crc_k[lane]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c ^= __shfl_xor_sync(0xffffffffu, c, o);
    const uint32_t crc = ~(c ^ crc_k[32]);
    const uint32_t want = (uint32_t)pk[476] << 24 | (uint32_t)pk[477] << 16 | (uint32_t)pk[478] << 8 | pk[479];
    // the batch reports the CRC of whatever was decided; the receiver verifies only decoded blocks (its > 0)
    if (lane == 0) { a.its[cw] = used; a.ok[cw] = (a.rx.llrf ? used > 0 : true) && crc == want; }
  }
  if (a.rx.llrf) {
    // the block's 476 bytes, verified or not (ok says which)
    uint8_t *dst = a.rx.blocks + (int64_t)gi * kBlockBytes;
    for (int t = tg; t < kBlockBytes; t += GT) dst[t] = pk[t];
  } else {
    int4 *dst = reinterpret_cast<int4 *>(a.bits + off / 8);
    const int4 *pv = reinterpret_cast<const int4 *>(pk);
    for (int t = tg; t < T::N / 128; t += GT) dst[t] = pv[t];
  }
  group_sync<WPC>(g);
}

// The per-code persistent kernel: every group pulls codewords of the launch's code from its work counter.
template <int C, int WPC, bool LOOP, bool PAIR>
__global__ void __launch_bounds__(cta_threads<C, WPC>(), 1) ldpc_decode_kernel(LdpcLaunch a) {
  using T = Code<C>;
  static_assert(cta_threads<C, WPC>() <= 1024, "a CTA of at most 1024 threads");
  static_assert(T::WARPS <= 15, "one named barrier a codeword");
  extern __shared__ __align__(16) uint8_t smem[];
  __shared__ int s_item[T::WARPS], s_red[T::WARPS][WPC];
  uint32_t *crc_tab = reinterpret_cast<uint32_t *>(smem);
  uint32_t *crc_k = crc_tab + 256;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = warp / WPC, sub = warp % WPC, tg = sub * 32 + lane;
  uint8_t *slice = smem + kCrcBytes + g * warp_bytes<C>();
  for (int t = threadIdx.x; t < 256; t += blockDim.x) {
    uint32_t c = (uint32_t)t;
    for (int k = 0; k < 8; k++) c = (c >> 1) ^ (kCrcPoly & (0u - (c & 1u)));
    crc_tab[t] = c;
  }
  for (int t = threadIdx.x; t < 33; t += blockDim.x) crc_k[t] = c_crc_shift[t];
  __syncthreads();
  (void)lane;
  const int count = a.count_dev ? *a.count_dev : a.count;
  for (;;) {
    if (tg == 0) s_item[g] = atomicAdd(a.counter, 1);
    group_sync<WPC>(g);
    const int item = s_item[g];
    group_sync<WPC>(g);   // every warp of the codeword has read it before its next write
    if (item >= count) break;
    decode_item<C, WPC, LOOP, PAIR>(a, a.tier, item, slice, crc_tab, crc_k, s_red[g], g);
  }
}

// The receivers' decode in one persistent launch across their tiers (every code): a queue of (receiver, tier, block)
// items, the tiers of the longer codes first, pulled by groups of two warps, each item decoded by its code's form (the
// pair form with the loop for 7/8, messages in registers for the others) in a slice sized for the longest code. One
// launch in place of a launch a tier on forked streams: for the small batches where the launches and their tails are
// the cost, and for an engine's formats together.
constexpr int cmax(int x, int y) { return x > y ? x : y; }
constexpr int kMixSlice = cmax(cmax(warp_bytes<0>(), warp_bytes<1>()), cmax(warp_bytes<2>(), warp_bytes<3>()));
constexpr int kMixWpc = 2, kMixGroups = (227 * 1024 - kCrcBytes) / kMixSlice, kMixThreads = kMixGroups * kMixWpc * 32;
static_assert(kMixGroups >= 1 && kMixGroups <= 15, "groups of the mixed launch");
static_assert(sizeof(LdpcMix) <= 32000, "the mixed launch's arguments fit a launch");
__global__ void __launch_bounds__(kMixThreads, 1) ldpc_mixed_kernel(const __grid_constant__ LdpcMix m) {
  extern __shared__ __align__(16) uint8_t smem[];
  __shared__ int s_item[kMixGroups], s_red[kMixGroups][kMixWpc];
  uint32_t *crc_tab = reinterpret_cast<uint32_t *>(smem);
  uint32_t *crc_k = crc_tab + 256;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = warp / kMixWpc, sub = warp % kMixWpc, tg = sub * 32 + lane;
  uint8_t *slice = smem + kCrcBytes + g * kMixSlice;
  for (int t = threadIdx.x; t < 256; t += blockDim.x) {
    uint32_t c = (uint32_t)t;
    for (int k = 0; k < 8; k++) c = (c >> 1) ^ (kCrcPoly & (0u - (c & 1u)));
    crc_tab[t] = c;
  }
  for (int t = threadIdx.x; t < 33; t += blockDim.x) crc_k[t] = c_crc_shift[t];
  __syncthreads();
  (void)lane;
  const int total = m.first[m.nseg];
  for (;;) {
    if (tg == 0) s_item[g] = atomicAdd(m.counter, 1);
    group_sync<kMixWpc>(g);
    const int item = s_item[g];
    group_sync<kMixWpc>(g);
    if (item >= total) break;
    int seg = 0;
    while (seg < m.nseg - 1 && item >= m.first[seg + 1]) seg++;
    const LdpcLaunch &a = m.a[seg];
    const int local = item - m.first[seg];
    switch (m.code[seg]) {
      case 0: decode_item<0, kMixWpc, true, true>(a, a.tier, local, slice, crc_tab, crc_k, s_red[g], g); break;
      case 1: decode_item<1, kMixWpc, false, false>(a, a.tier, local, slice, crc_tab, crc_k, s_red[g], g); break;
      case 2: decode_item<2, kMixWpc, false, false>(a, a.tier, local, slice, crc_tab, crc_k, s_red[g], g); break;
      default: decode_item<3, kMixWpc, false, false>(a, a.tier, local, slice, crc_tab, crc_k, s_red[g], g); break;
    }
  }
}

// x^(8 k) mod P, reflected.
static uint32_t xpow8(int k) {
  uint32_t r = 0x80000000u;
  for (int i = 0; i < 8 * k; i++) r = (r >> 1) ^ (kCrcPoly & (0u - (r & 1u)));
  return r;
}
static uint32_t host_gf_mul(uint32_t a, uint32_t b) {
  uint32_t p = 0;
  for (int i = 0; i < 32; i++) { if (a & (0x80000000u >> i)) p ^= b; b = (b >> 1) ^ (kCrcPoly & (0u - (b & 1u))); }
  return p;
}

cudaError_t ldpc_upload_tables() {
  DevCode h[4] = {};
  for (int c = 0; c < 4; c++) {
    const lizg_code_def_t &d = LIZG_CODES[c];
    for (int r = 0; r <= d.mb; r++) h[c].rowptr[r] = d.rowptr[r];
    for (int e = 0; e < d.rowptr[d.mb]; e++) h[c].circ[e] = d.circ[e];
  }
  cudaError_t err = cudaMemcpyToSymbol(c_codes, h, sizeof h);
  if (err != cudaSuccess) return err;
  uint32_t k[33];
  for (int l = 0; l < 32; l++) { const int end = 15 * l + 15 < kBlockBytes ? 15 * l + 15 : kBlockBytes; k[l] = xpow8(kBlockBytes - end); }
  k[32] = host_gf_mul(0xffffffffu, xpow8(kBlockBytes));
  return cudaMemcpyToSymbol(c_crc_shift, k, sizeof k);
}

// ---------------------------------------------------------------- kernel variants and their choice
//
// Every variant decodes bit for bit alike (the layers' arithmetic and order are the same); they differ in how a
// codeword's checks are spread over warps and in register use, so which is fastest depends on the device, the code
// and the channel. Variant 0 of each code is the default; lizg_ldpc_autotune times them all on the current device
// and keeps the fastest per code.
struct Variant {
  int wpc;
  bool loop, pair;
};
constexpr int kMaxVariants = 8;
static const Variant kVariants[4][kMaxVariants] = {
    // 7/8: 21-circulant rows, the loop form; the pair form first (the fastest on a GB300)
    {{2, true, true}, {1, true, false}, {2, false, false}, {2, true, false}, {2, false, true}, {1, true, true}},
    {{2, false, false}, {1, true, false}, {4, false, false}, {2, true, false}, {2, false, true}, {1, false, true}},   // 3/4
    {{2, false, false}, {1, true, false}, {4, false, false}, {2, false, true}, {1, false, true}},                     // 2/3
    {{4, false, false}, {2, false, false}, {1, false, false}, {2, false, true}, {1, false, true}},                    // 1/2
};
static int variant_count(int code) {
  int k = 0;
  while (k < kMaxVariants && kVariants[code][k].wpc) k++;
  return k;
}

constexpr int kMaxDevices = 64;
static int g_choice[kMaxDevices][4];   // per device and code: the variant index (0 until tuned or set)
static std::mutex g_choice_mu;

static int choice_of(int code) {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_choice_mu);
  return dev >= 0 && dev < kMaxDevices ? g_choice[dev][code] : 0;
}

template <int C, int WPC, bool LOOP, bool PAIR>
static cudaError_t launch_v(const LdpcLaunch &a, int sms, cudaStream_t st) {
  static SmemOptIn opt;
  if (cudaError_t e = opt.set(reinterpret_cast<const void *>(ldpc_decode_kernel<C, WPC, LOOP, PAIR>), cta_smem<C>())) return e;
  const int need = (a.count + Code<C>::WARPS - 1) / Code<C>::WARPS;
  const int grid = need < sms ? need : sms;
  ldpc_decode_kernel<C, WPC, LOOP, PAIR><<<grid, cta_threads<C, WPC>(), cta_smem<C>(), st>>>(a);
  return cudaGetLastError();
}

static cudaError_t launch_variant(int code, int v, const LdpcLaunch &a, int sms, cudaStream_t st) {
  switch (code * kMaxVariants + v) {
    case 0: return launch_v<0, 2, true, true>(a, sms, st);
    case 1: return launch_v<0, 1, true, false>(a, sms, st);
    case 2: return launch_v<0, 2, false, false>(a, sms, st);
    case 3: return launch_v<0, 2, true, false>(a, sms, st);
    case 4: return launch_v<0, 2, false, true>(a, sms, st);
    case 5: return launch_v<0, 1, true, true>(a, sms, st);
    case 8: return launch_v<1, 2, false, false>(a, sms, st);
    case 9: return launch_v<1, 1, true, false>(a, sms, st);
    case 10: return launch_v<1, 4, false, false>(a, sms, st);
    case 11: return launch_v<1, 2, true, false>(a, sms, st);
    case 12: return launch_v<1, 2, false, true>(a, sms, st);
    case 13: return launch_v<1, 1, false, true>(a, sms, st);
    case 16: return launch_v<2, 2, false, false>(a, sms, st);
    case 17: return launch_v<2, 1, true, false>(a, sms, st);
    case 18: return launch_v<2, 4, false, false>(a, sms, st);
    case 19: return launch_v<2, 2, false, true>(a, sms, st);
    case 20: return launch_v<2, 1, false, true>(a, sms, st);
    case 24: return launch_v<3, 4, false, false>(a, sms, st);
    case 25: return launch_v<3, 2, false, false>(a, sms, st);
    case 26: return launch_v<3, 1, false, false>(a, sms, st);
    case 27: return launch_v<3, 2, false, true>(a, sms, st);
    case 28: return launch_v<3, 1, false, true>(a, sms, st);
  }
  return cudaErrorInvalidValue;
}

cudaError_t ldpc_launch(int code, const LdpcLaunch &a, int sms, cudaStream_t st) {
  if (a.count <= 0) return cudaSuccess;
  if (code < 0 || code > 3) return cudaErrorInvalidValue;
  return launch_variant(code, choice_of(code), a, sms, st);
}

int ldpc_variant_count(int code) { return code >= 0 && code <= 3 ? variant_count(code) : 0; }

cudaError_t ldpc_mixed_launch(const LdpcMix &m, int sms, cudaStream_t st) {
  if (m.nseg < 1 || m.nseg > kMixSegs) return m.nseg == 0 ? cudaSuccess : cudaErrorInvalidValue;
  if (m.first[m.nseg] <= 0) return cudaSuccess;
  static SmemOptIn opt;
  constexpr int smem = kCrcBytes + kMixGroups * kMixSlice;
  static_assert(smem <= 227 * 1024, "the mixed launch's slices fit");
  if (cudaError_t e = opt.set(reinterpret_cast<const void *>(ldpc_mixed_kernel), smem)) return e;
  const int need = (m.first[m.nseg] + kMixGroups - 1) / kMixGroups;
  ldpc_mixed_kernel<<<need < sms ? need : sms, kMixThreads, smem, st>>>(m);
  return cudaGetLastError();
}
int ldpc_choice(int code) { return code >= 0 && code <= 3 ? choice_of(code) : 0; }

cudaError_t ldpc_launch_variant(int code, int v, const LdpcLaunch &a, int sms, cudaStream_t st) {
  if (a.count <= 0) return cudaSuccess;
  if (code < 0 || code > 3 || v < 0 || v >= variant_count(code)) return cudaErrorInvalidValue;
  return launch_variant(code, v, a, sms, st);
}

}  // namespace lizg

extern "C" {

int lizg_ldpc_variants(int rate) {
  const int c = lizg_code_of_rate(rate);
  if (c < 0) return lizg::record_error(LIZG_E_ARG, "lizg_ldpc_variants: rate must be 6, 4, 3 or 2");
  return lizg::variant_count(c);
}

int lizg_ldpc_variant(int rate, int32_t *wpc, int32_t *loop_form) {
  const int c = lizg_code_of_rate(rate);
  if (c < 0) return lizg::record_error(LIZG_E_ARG, "lizg_ldpc_variant: rate must be 6, 4, 3 or 2");
  int sms = 0;
  if (int rc = lizg::device_ready(&sms)) return rc;
  const int v = lizg::choice_of(c);
  if (wpc) *wpc = lizg::kVariants[c][v].wpc;
  if (loop_form) *loop_form = (lizg::kVariants[c][v].loop ? 1 : 0) | (lizg::kVariants[c][v].pair ? 2 : 0);
  return v;
}

// The calibration batch of a code: count copies of the all-zero codeword (a min-sum decoder treats every codeword
// alike, the channel being symmetric) sent as BPSK over AWGN, codeword c at ebn0_db[c mod n_ebn0], quantised as the
// batch benchmark's LLRs (nearest of 8 clamp(2 y / sigma^2, +-10)), the 7/8 code's unsent known zeros at +127.
static void calibration_llrs(int code, int count, const float *ebn0_db, int n_ebn0, std::vector<int8_t> &llr) {
  const lizg_code_def_t &d = LIZG_CODES[code];
  const int n = (d.mb + d.kb) * 128, k = d.kb * 128, sent = n - (k - LIZG_INFO_BITS);
  const double rate = (double)LIZG_INFO_BITS / sent;
  std::mt19937 gen(20240u + (unsigned)code);
  std::normal_distribution<double> g(0.0, 1.0);
  llr.resize((size_t)count * n);
  for (int c = 0; c < count; c++) {
    const double ebn0 = std::pow(10.0, ebn0_db[c % n_ebn0] / 10.0), sigma = std::sqrt(1.0 / (2.0 * rate * ebn0));
    for (int i = 0; i < n; i++) {
      int8_t q = 127;
      if (i < LIZG_INFO_BITS || i >= k) {
        double l = 2.0 * (1.0 + sigma * g(gen)) / (sigma * sigma);
        l = l > 10 ? 10 : l < -10 ? -10 : l;
        q = (int8_t)std::nearbyint(8 * l);
      }
      llr[(size_t)c * n + i] = q;
    }
  }
}

int lizg_ldpc_autotune(int count, const float *ebn0_db, int n_ebn0, int32_t *choice) {
  if (count < 1 || count > (1 << 16)) return lizg::record_error(LIZG_E_ARG, "lizg_ldpc_autotune: count must be 1..65536");
  if (!ebn0_db || n_ebn0 < 1) return lizg::record_error(LIZG_E_ARG, "lizg_ldpc_autotune: no Eb/N0 given");
  int sms = 0, dev = 0;
  if (int rc = lizg::device_ready(&sms)) return rc;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= lizg::kMaxDevices) return lizg::record_error(LIZG_E_STATE, "lizg_ldpc_autotune: device index out of range");
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  std::vector<void *> bufs;
  cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  for (int c = 0; c < 4 && e == cudaSuccess; c++) {
    const lizg_code_def_t &d = LIZG_CODES[c];
    const int n = (d.mb + d.kb) * 128;
    std::vector<int8_t> llr;
    calibration_llrs(c, count, ebn0_db, n_ebn0, llr);
    std::vector<int32_t> list(count);
    std::vector<int64_t> off(count);
    for (int i = 0; i < count; i++) { list[i] = i; off[i] = (int64_t)i * n; }
    void *d_llr = nullptr, *d_bits = nullptr, *d_its = nullptr, *d_ok = nullptr, *d_list = nullptr, *d_off = nullptr, *d_ctr = nullptr;
    auto al = [&](void **p, size_t b) { if (e == cudaSuccess && (e = cudaMalloc(p, b)) == cudaSuccess) bufs.push_back(*p); };
    al(&d_llr, llr.size()); al(&d_bits, (size_t)count * n / 8); al(&d_its, 4 * (size_t)count); al(&d_ok, (size_t)count);
    al(&d_list, 4 * (size_t)count); al(&d_off, 8 * (size_t)count); al(&d_ctr, 4);
    if (e == cudaSuccess) e = cudaMemcpy(d_llr, llr.data(), llr.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_list, list.data(), 4 * (size_t)count, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_off, off.data(), 8 * (size_t)count, cudaMemcpyHostToDevice);
    lizg::LdpcLaunch a{};
    a.llr = static_cast<const int8_t *>(d_llr); a.bits = static_cast<uint8_t *>(d_bits); a.its = static_cast<int32_t *>(d_its);
    a.ok = static_cast<uint8_t *>(d_ok); a.list = static_cast<const int32_t *>(d_list); a.off = static_cast<const int64_t *>(d_off);
    a.count = count; a.counter = static_cast<int *>(d_ctr); a.max_iter = 20; a.stall_it = 9; a.stall_ratio = 0.95f;
    int best = 0;
    float best_ms = 0;
    for (int v = 0; v < lizg::variant_count(c) && e == cudaSuccess; v++) {
      float ms_min = 0;
      for (int rep = 0; rep < 4 && e == cudaSuccess; rep++) {   // the first run warms up
        if ((e = cudaMemsetAsync(d_ctr, 0, 4, st)) != cudaSuccess || (e = cudaEventRecord(e0, st)) != cudaSuccess ||
            (e = lizg::launch_variant(c, v, a, sms, st)) != cudaSuccess || (e = cudaEventRecord(e1, st)) != cudaSuccess ||
            (e = cudaEventSynchronize(e1)) != cudaSuccess)
          break;
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep == 1 || (rep > 1 && ms < ms_min)) ms_min = ms;
      }
      if (e == cudaSuccess && (v == 0 || ms_min < best_ms)) { best = v; best_ms = ms_min; }
    }
    if (e == cudaSuccess) {
      std::lock_guard<std::mutex> lk(lizg::g_choice_mu);
      lizg::g_choice[dev][c] = best;
    }
    if (choice) choice[c] = best;
    for (void *p : bufs) cudaFree(p);
    bufs.clear();
  }
  for (void *p : bufs) cudaFree(p);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  if (e != cudaSuccess) return lizg::record_error(LIZG_E_CUDA, (std::string("lizg_ldpc_autotune: ") + cudaGetErrorString(e)).c_str());
  return 0;
}

int lizg_ldpc_set_variant(int rate, int index) {
  const int c = lizg_code_of_rate(rate);
  if (c < 0 || index < 0 || index >= lizg::variant_count(c)) return lizg::record_error(LIZG_E_ARG, "lizg_ldpc_set_variant: no such rate or variant");
  int sms = 0, dev = 0;
  if (int rc = lizg::device_ready(&sms)) return rc;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= lizg::kMaxDevices) return lizg::record_error(LIZG_E_STATE, "lizg_ldpc_set_variant: device index out of range");
  std::lock_guard<std::mutex> lk(lizg::g_choice_mu);
  lizg::g_choice[dev][c] = index;
  return 0;
}

}  // extern "C"

namespace lizg {

// ---------------------------------------------------------------- the decode without allocation
//
// For callers that cannot allocate device memory themselves: a driver or plug-in running inside a host that owns
// the allocator (a capture pipeline that hands out frame buffers from its own pool, a runtime whose device memory is
// fully reserved up front) may not call cudaMalloc, yet the plan API needs a few device words of scratch (per-code
// work lists, offsets and counters). Here that scratch is a fixed array in the library's own device image, sized for
// LIZG_NOALLOC_MAX_CODEWORDS codewords; every GPU that loads the library holds it until the process exits.

constexpr int kNoAllocMax = LIZG_NOALLOC_MAX_CODEWORDS;
// Layout: counts[4], counters[4], then (from byte 256) the four codes' work lists (kNoAllocMax entries each), then
// the codewords' LLR offsets.
constexpr size_t kNaLists = 256, kNaOffs = kNaLists + 4 * sizeof(int32_t) * kNoAllocMax, kNaBytes = kNaOffs + sizeof(int64_t) * kNoAllocMax;
static __device__ __align__(256) uint8_t g_noalloc_scratch[kNaBytes];

__device__ __forceinline__ int code_n_dev(int c) { return c == 0 ? 4608 : c == 1 ? 5120 : c == 2 ? 5760 : c == 3 ? 7680 : 0; }

// One CTA of 1024 threads builds the batch's layout in the scratch: codeword i's LLR offset (the n of every valid
// codeword before it), the per-code work lists in codeword order, their counts, the work counters at zero. A
// codeword whose rate index has no code gets its = -4, ok = 0 and no offset share.
__global__ void __launch_bounds__(1024) ldpc_noalloc_prepare(const int32_t *rate, int count, uint8_t *scr, int32_t *its, uint8_t *ok) {
  int *counts = reinterpret_cast<int *>(scr);
  int32_t *lists = reinterpret_cast<int32_t *>(scr + kNaLists);
  int64_t *offs = reinterpret_cast<int64_t *>(scr + kNaOffs);
  constexpr int PER = kNoAllocMax / 1024;
  __shared__ int64_t s_bits[1024];
  __shared__ int s_cnt[4][1024];
  const int tid = threadIdx.x, i0 = tid * PER;
  int code[PER];
  int64_t bits = 0;
  int cnt[4] = {0, 0, 0, 0};
#pragma unroll
  for (int k = 0; k < PER; k++) {
    const int i = i0 + k;
    int c = -1;
    if (i < count) {
      const int r = rate[i];
      c = r == 6 ? 0 : r == 4 ? 1 : r == 3 ? 2 : r == 2 ? 3 : -1;
      if (c < 0) { its[i] = -4; ok[i] = 0; }
      else { bits += code_n_dev(c); cnt[c]++; }
    }
    code[k] = c;
  }
  s_bits[tid] = bits;
  for (int c = 0; c < 4; c++) s_cnt[c][tid] = cnt[c];
  __syncthreads();
  // inclusive scans over the threads (Hillis-Steele)
  for (int d = 1; d < 1024; d <<= 1) {
    const int64_t vb = tid >= d ? s_bits[tid - d] : 0;
    int vc[4];
    for (int c = 0; c < 4; c++) vc[c] = tid >= d ? s_cnt[c][tid - d] : 0;
    __syncthreads();
    s_bits[tid] += vb;
    for (int c = 0; c < 4; c++) s_cnt[c][tid] += vc[c];
    __syncthreads();
  }
  int64_t at = s_bits[tid] - bits;
  int pos[4];
  for (int c = 0; c < 4; c++) pos[c] = s_cnt[c][tid] - cnt[c];
#pragma unroll
  for (int k = 0; k < PER; k++) {
    const int i = i0 + k, c = code[k];
    if (c < 0) continue;
    offs[i] = at;
    at += code_n_dev(c);
    lists[c * kNoAllocMax + pos[c]++] = i;
  }
  if (tid == 0) for (int c = 0; c < 4; c++) { counts[c] = s_cnt[c][1023]; counts[4 + c] = 0; }
}

namespace {
std::mutex g_na_mu;
uint8_t *g_na_ptr[64];   // the scratch's device address, per device
}  // namespace

}  // namespace lizg

extern "C" int lizg_ldpc_decode_noalloc(const int8_t *d_llr, const int32_t *d_rate, int count, int max_iter, int stall_it,
                                        float stall_ratio, uint8_t *d_bits, int32_t *d_its, uint8_t *d_ok, void *stream) {
  using namespace lizg;
  if (!d_llr || !d_rate || !d_bits || !d_its || !d_ok) return record_error(LIZG_E_ARG, "lizg_ldpc_decode_noalloc: NULL argument");
  if (count < 1 || count > kNoAllocMax)
    return record_error(LIZG_E_ARG, "lizg_ldpc_decode_noalloc: count must be 1..LIZG_NOALLOC_MAX_CODEWORDS (8192)");
  if (max_iter < 1 || max_iter > 255 || stall_it < 0 || stall_it == 1 || stall_it > max_iter)
    return record_error(LIZG_E_ARG, "lizg_ldpc_decode_noalloc: bad max_iter or stall_it");
  if ((reinterpret_cast<uintptr_t>(d_llr) | reinterpret_cast<uintptr_t>(d_bits)) & 15)
    return record_error(LIZG_E_ARG, "lizg_ldpc_decode_noalloc: llr and bits must be 16-byte aligned");
  int sms = 0;
  if (int rc = device_ready(&sms)) return rc;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 64) return record_error(LIZG_E_CUDA, "lizg_ldpc_decode_noalloc: cudaGetDevice");
  uint8_t *scr = nullptr;
  {
    // Set-up, once a device with that device current: the scratch array's device address. In host code the
    // array's name is only a stand-in for it.
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_ptr[dev]) {
      void *ptr = nullptr;
      if ((e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch)) != cudaSuccess)
        return record_error(LIZG_E_CUDA, "lizg_ldpc_decode_noalloc: cudaGetSymbolAddress failed");
      g_na_ptr[dev] = static_cast<uint8_t *>(ptr);
    }
    scr = g_na_ptr[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  ldpc_noalloc_prepare<<<1, 1024, 0, st>>>(d_rate, count, scr, d_its, d_ok);
  if ((e = cudaGetLastError()) != cudaSuccess) return record_error(LIZG_E_CUDA, "lizg_ldpc_decode_noalloc: prepare launch");
  int *counts = reinterpret_cast<int *>(scr);
  for (int c = 0; c < 4; c++) {
    LdpcLaunch a{};
    a.llr = d_llr; a.bits = d_bits; a.its = d_its; a.ok = d_ok;
    a.list = reinterpret_cast<const int32_t *>(scr + kNaLists) + c * kNoAllocMax;
    a.off = reinterpret_cast<const int64_t *>(scr + kNaOffs);
    a.count = count;                 // bounds the grid; the kernel reads the code's own count from the scratch
    a.count_dev = counts + c;
    a.counter = counts + 4 + c;
    a.max_iter = max_iter; a.stall_it = stall_it; a.stall_ratio = stall_ratio;
    if ((e = ldpc_launch(c, a, sms, st)) != cudaSuccess) return record_error(LIZG_E_CUDA, "lizg_ldpc_decode_noalloc: decode launch");
  }
  return 0;
}

// Format tables (host). Every table here is fixed by the LIZARD format; the receive kernels read them and the tests
// hold them to the reference's (liblizard/src/lizard_phy.c:348-427 ws_init, :485-562 init, :578-621 the profile).
#include "format.h"
#include "lizard_codes.h"
#include <algorithm>
#include <cmath>

namespace lizg {

namespace {

int gcd(int a, int b) { while (b) { const int t = a % b; a = b; b = t; } return a; }

int code_nt(int c) { const lizg_code_def_t &d = LIZG_CODES[c]; return (d.kb - d.np_cols + d.mb) * LIZG_Z; }

// The profile's search (liblizard/src/lizard_phy.c:578-613): counts of the 7/8, 2/3 and 1/2 tiers chosen by least
// squares from their target shares of the frame's slots (390, 150 and 200 thousandths), the 3/4 tier filling the
// rest; the first of equal costs kept, a branch given up once its cost reaches the best so far.
struct Search {
  int slots[4];
  long long target[4], all, best = -1;
  int cnt[4] = {0, 0, 0, 0}, keep[4] = {0, 0, 0, 0};
  void run(int t, long long used, long long cost) {
    if (t == 4) {
      const long long rest = all - used;
      if (rest < slots[1]) return;
      if (best < 0 || cost < best) {
        best = cost;
        for (int q = 0; q < 4; q++) keep[q] = cnt[q];
        keep[1] = (int)(rest / slots[1]);
      }
      return;
    }
    if (t == 1) { run(2, used, cost); return; }
    for (int a = 0; used + (long long)slots[t] * a <= all - slots[1]; a++) {
      const long long d = 1000LL * slots[t] * a - target[t] * all;
      if (best >= 0 && cost + d * d >= best) { if (d > 0) break; continue; }
      cnt[t] = a;
      run(t + 1, used + (long long)slots[t] * a, cost + d * d);
    }
  }
};

}  // namespace

int block_slots(int rate) {
  const int c = lizg_code_of_rate(rate);
  if (c < 0) return 0;
  return code_nt(c) + LIZG_CODES[c].pilots;
}

int tiers_for(int subch, Tier *out) {
  if (subch < 64 || subch % 16 || subch > 1024) return 0;
  static const int RATE[4] = {6, 4, 3, 2};
  static const int TARGET[4] = {390, 0, 150, 200};
  Search s;
  for (int q = 0; q < 4; q++) { s.slots[q] = block_slots(RATE[q]); s.target[q] = TARGET[q]; }
  s.all = (long long)subch * kSub * 2;
  s.run(0, 0, 0);
  int t = 0;
  for (int q = 0; q < 4; q++) {
    if (!s.keep[q]) continue;
    const int c = lizg_code_of_rate(RATE[q]);
    const lizg_code_def_t &d = LIZG_CODES[c];
    out[t++] = Tier{RATE[q], s.keep[q], s.slots[q], c, code_nt(c), d.kb * LIZG_Z, d.np_cols * LIZG_Z};
  }
  return t;
}

int format_build(int n, int subch, int span, Format &f) {
  static const int PICS[7] = {384, 512, 768, 1024, 1152, 1280, 1536};
  if (std::find(PICS, PICS + 7, n) == PICS + 7) return -1;
  if (!span) span = 256;
  if (span != 128 && span != 256 && span != 512) return -1;
  f = Format();
  f.n = n; f.subch = subch; f.span = span;
  f.tiers = tiers_for(subch, f.tier);
  if (!f.tiers) return -1;
  for (int t = 0; t < f.tiers; t++) {
    f.tier_first[t] = f.blocks;
    for (int q = 0; q < f.tier[t].blocks; q++) {
      f.block_tier.push_back(t);
      f.block_slot.push_back(f.used);
      f.used += f.tier[t].slots;
    }
    f.blocks += f.tier[t].blocks;
  }
  // The used coefficients: the upper half-plane less v = 0, u <= 0 and the Nyquist row and column, in order of
  // (u^2 + v^2, v, u) (liblizard/src/lizard_phy.c:505-535), the first subch x 320.
  const int h = n / 2, need = subch * kSub;
  struct C { int r2, v, u; };
  std::vector<C> all;
  all.reserve((size_t)h * (2 * h - 1));
  for (int v = 0; v < h; v++)
    for (int u = -h + 1; u < h; u++)
      if (v > 0 || u > 0) all.push_back(C{u * u + v * v, v, u});
  if ((int)all.size() < need) return -1;
  std::partial_sort(all.begin(), all.begin() + need, all.end(), [](const C &a, const C &b) {
    return a.r2 != b.r2 ? a.r2 < b.r2 : a.v != b.v ? a.v < b.v : a.u < b.u;
  });
  f.bw = h < kStrip ? h : kStrip;
  int vmax = 0;
  for (int i = 0; i < need; i++) vmax = std::max(vmax, all[i].v);
  f.vblocks = vmax / f.bw + 1;
  f.vmax = vmax;
  f.uv.resize(2 * (size_t)need);
  f.tix.resize(need);
  for (int i = 0; i < need; i++) {
    f.uv[2 * i] = (int16_t)all[i].u; f.uv[2 * i + 1] = (int16_t)all[i].v;
    f.tix[i] = all[i].v * n + (all[i].u + n) % n;
  }
  f.scale = (float)n / span;
  // Whitening: PRBS-23 (x^23 + x^18 + 1) from the all-ones state, a bit a slot (liblizard/src/lizard_phy.c:95-101).
  f.white.resize(2 * (size_t)need);
  uint32_t reg = 0x7fffff;
  for (int i = 0; i < 2 * need; i++) {
    const uint32_t b = ((reg >> 22) ^ (reg >> 17)) & 1u;
    reg = ((reg << 1) | b) & 0x7fffffu;
    f.white[i] = (uint8_t)b;
  }
  // Bit map: slot i of a block carries sent bit i P mod nt, P the first integer from round(nt / phi^2) prime to nt;
  // sent bit j is codeword bit j, or j + np past the code's first k - np (liblizard/src/lizard_phy.c:104-116).
  for (int t = 0; t < f.tiers; t++) {
    const Tier &tr = f.tier[t];
    int P = (int)(0.3819660113 * tr.nt + 0.5);
    while (gcd(P, tr.nt) != 1) P++;
    f.perm[t].resize(tr.nt);
    for (int i = 0; i < tr.nt; i++) {
      const int j = (int)((long long)i * P % tr.nt);
      f.perm[t][i] = (int16_t)(j < tr.k - tr.np ? j : j + tr.np);
    }
  }
  // Pilots: every block tail's coefficients in block order, with their whitening (liblizard/src/lizard_phy.c:295-317).
  for (int b = 0; b < f.blocks; b++) {
    const Tier &tr = f.tier[f.block_tier[b]];
    const int first = f.block_slot[b] / 2;
    for (int s = tr.nt / 2; s < tr.slots / 2; s++) {
      f.pilot_coef.push_back(first + s);
      f.pilot_white.push_back((uint8_t)(f.white[2 * (first + s)] | f.white[2 * (first + s) + 1] << 1));
    }
  }
  // Detrend basis c(i) = (2 i + 1 - n) / n and q(i) = c(i)^2 less its mean, their squared norms and DFTs, in double,
  // kept in float (liblizard/src/lizard_phy.c:389-398).
  f.cx.resize(n); f.qx.resize(n); f.x1r.resize(n); f.x1i.resize(n); f.x2r.resize(n); f.x2i.resize(n);
  std::vector<double> cd(n), qd(n);
  double m2 = 0;
  for (int i = 0; i < n; i++) { cd[i] = (2.0 * i + 1 - n) / n; m2 += cd[i] * cd[i]; }
  f.sx2 = m2;
  m2 /= n;
  f.sq2 = 0;
  for (int i = 0; i < n; i++) { qd[i] = cd[i] * cd[i] - m2; f.sq2 += qd[i] * qd[i]; f.cx[i] = (float)cd[i]; f.qx[i] = (float)qd[i]; }
  const double PI = 3.14159265358979323846;
  std::vector<double> er(n), ei(n);
  for (int k = 0; k < n; k++) { er[k] = std::cos(-2 * PI * k / n); ei[k] = std::sin(-2 * PI * k / n); }
  for (int u = 0; u < n; u++) {
    double ar = 0, ai = 0, br = 0, bi = 0;
    for (int i = 0; i < n; i++) {
      const int k = (int)((long long)u * i % n);
      ar += cd[i] * er[k]; ai += cd[i] * ei[k]; br += qd[i] * er[k]; bi += qd[i] * ei[k];
    }
    f.x1r[u] = (float)ar; f.x1i[u] = (float)ai; f.x2r[u] = (float)br; f.x2i[u] = (float)bi;
  }
  // The anchors' squares as a receiver erases them: the 7 ranges on either axis, square i's first module
  // m0 = floor(15 + span (i + 1/2) / 7 - a / 2 + 1/2) of side a = span / 64 (liblizard/src/acquire.c:41-45), in
  // samples widened by 2 (liblizard/src/lizard_phy.c:400-407).
  const int a = span / 64;
  for (int i = 0; i < kAnchK; i++) {
    const int m0 = (int)std::floor(kMargin + (double)span * (i + 0.5) / kAnchK - a / 2.0 + 0.5);
    const int lo = (int)std::floor((float)(m0 - kMargin) * f.scale) - kAnchMargin;
    const int hi = (int)std::ceil((float)(m0 + a - kMargin) * f.scale) - 1 + kAnchMargin;
    f.elo[i] = std::max(lo, 0); f.ehi[i] = std::min(hi, n - 1);
  }
  // The shading surface's normal matrix over every eighth sample outside the squares, inverted by Gauss-Jordan with
  // partial pivoting (liblizard/src/lizard_phy.c:408-425).
  auto in_sq = [&](int t) { for (int i = 0; i < kAnchK; i++) if (t >= f.elo[i] && t <= f.ehi[i]) return true; return false; };
  double g[6][12] = {};
  for (int y = 0; y < n; y += 8)
    for (int x = 0; x < n; x += 8) {
      if (in_sq(x) && in_sq(y)) continue;
      const double b[6] = {1, f.cx[x], f.qx[x], f.cx[y], f.qx[y], (double)f.cx[x] * f.cx[y]};
      for (int r = 0; r < 6; r++) for (int c = 0; c < 6; c++) g[r][c] += b[r] * b[c];
    }
  for (int r = 0; r < 6; r++) g[r][6 + r] = 1;
  for (int c = 0; c < 6; c++) {
    int p = c;
    for (int r = c + 1; r < 6; r++) if (std::fabs(g[r][c]) > std::fabs(g[p][c])) p = r;
    if (std::fabs(g[p][c]) < 1e-12) return -1;
    for (int k = 0; k < 12; k++) std::swap(g[c][k], g[p][k]);
    const double d = g[c][c];
    for (int k = 0; k < 12; k++) g[c][k] /= d;
    for (int r = 0; r < 6; r++) {
      if (r == c) continue;
      const double m = g[r][c];
      for (int k = 0; k < 12; k++) g[r][k] -= m * g[c][k];
    }
  }
  for (int r = 0; r < 6; r++) for (int c = 0; c < 6; c++) f.hole_inv[r][c] = g[r][6 + c];
  return 0;
}

// The registration mesh's node centres along one axis of a square layout of `side` modules (liblizard/src/layout.c:
// 110-117): every 16 modules from the border's centre line at 3.5, the last one 3.5 from the far edge, at most 40.
int layout_nodes(int side, float *pos) {
  const float line = 3.5f;
  int cnt = 0;
  for (float c = line; c < side - line - 16 / 2 && cnt < 40 - 1; c += 16) pos[cnt++] = c;
  pos[cnt++] = side - line;
  return cnt;
}

}  // namespace lizg

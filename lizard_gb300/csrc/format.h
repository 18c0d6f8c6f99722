// The LIZARD format's host-side tables for one (picture size n, sub-channels, ring span): everything the receive
// kernels need besides the frame itself, built once a format and uploaded to the device.
#ifndef LIZG_FORMAT_H
#define LIZG_FORMAT_H
#include <stdint.h>
#include <vector>

namespace lizg {

enum { kSub = 320, kStrip = 64, kAnchK = 7, kAnchMargin = 2, kMargin = 15, kTurns = 4096, kMaxTiers = 4 };

struct Tier { int rate, blocks, slots, code, nt, k, np; };

struct Format {
  int n = 0, subch = 0, span = 0, blocks = 0, used = 0, bw = 0, vblocks = 0, tiers = 0, vmax = 0;
  float scale = 0;                // picture samples a module, n / span
  Tier tier[kMaxTiers] = {};
  int tier_first[kMaxTiers] = {};  // first block of each tier (blocks of a tier are contiguous)
  std::vector<int32_t> block_tier, block_slot;
  std::vector<int16_t> uv;        // (u, v) of each used coefficient, pos order, u in (-n/2, n/2)
  std::vector<int32_t> tix;       // its index in the spectrum array [v][u mod n]
  std::vector<uint8_t> white;     // whitening bit of each frame slot
  std::vector<int16_t> perm[kMaxTiers];   // block slot i < nt -> codeword bit
  std::vector<int32_t> pilot_coef;        // coefficients of every block tail in block order (pilot fit input)
  std::vector<uint8_t> pilot_white;       // their two whitening bits (bit 0 real, bit 1 imaginary)
  int elo[kAnchK] = {}, ehi[kAnchK] = {};
  double hole_inv[6][6] = {};
  std::vector<float> cx, qx;      // detrend basis (float, as the reference keeps it)
  std::vector<float> x1r, x1i, x2r, x2i;
  double sx2 = 0, sq2 = 0;
};

// The rate profile for subch sub-channels: tiers (rate, blocks, slots), 7/8 then 3/4 then 2/3 then 1/2; 0 for none.
int tiers_for(int subch, Tier *out);
// Builds the format; returns 0, or -1 for a configuration that is no format.
int format_build(int n, int subch, int span, Format &f);
// The slots a block of a rate index takes (its code's sent bits, then 16 pilots at 7/8, 32 at 3/4).
int block_slots(int rate);
// The registration mesh's node centres along an axis of a layout of `side` modules; returns their count.
int layout_nodes(int side, float *pos);

}  // namespace lizg
#endif

// CPU restatement of the reference single-channel (DXT5 alpha / DXT5A / DXN channel) endpoint
// optimizer, every crn_dxt_quality level. TEST INFRASTRUCTURE ONLY (oracle + CPU baseline).
// Restates dxt5_endpoint_optimizer::compute / evaluate_solution (crnlib/crn_dxt5a.cpp:40-262)
// and the dxt5_block packing done by dxt_image::set_block_pixels (crn_dxt_image.cpp:1491-1522).
#include "crn_oracle.h"

#include <cstring>
#include <vector>
#include <algorithm>

namespace crn_oracle_detail {

namespace {

// dxt5_block::get_block_values8 / values6 (crnlib/crn_dxt.cpp:433-453)
inline void palette(unsigned l, unsigned h, int type, unsigned v[8]) {
  v[0] = l;
  v[1] = h;
  if (type == 0) {
    v[2] = (l * 6 + h) / 7; v[3] = (l * 5 + h * 2) / 7; v[4] = (l * 4 + h * 3) / 7;
    v[5] = (l * 3 + h * 4) / 7; v[6] = (l * 2 + h * 5) / 7; v[7] = (l + h * 6) / 7;
  } else {
    v[2] = (l * 4 + h) / 5; v[3] = (l * 3 + h * 2) / 5; v[4] = (l * 2 + h * 3) / 5;
    v[5] = (l + h * 4) / 5; v[6] = 0; v[7] = 255;
  }
}

struct Alpha {
  unsigned vals[16];
  unsigned wts[16];
  int n = 0;
  bool both = true;
  uint64_t err = UINT64_MAX;
  unsigned first = 0, second = 0;
  int type = 0;
  uint8_t best_sel[16], trial_sel[16];

  // evaluate_solution :198-262
  void evaluate(unsigned lo, unsigned hi) {
    for (int type_i = 0; type_i < (both ? 2 : 1); type_i++) {
      unsigned pv[8];
      palette(lo, hi, type_i, pv);
      uint64_t terr = 0;
      for (int i = 0; i < n; i++) {
        unsigned be = 0xFFFFFFFFu;
        int bs = 0;
        for (int j = 0; j < 8; j++) {
          int e = (int)vals[i] - (int)pv[j];
          e = e * e * (int)wts[i];
          if ((unsigned)e < be) {
            be = (unsigned)e;
            bs = j;
            if (!be) break;
          }
        }
        trial_sel[i] = (uint8_t)bs;
        terr += be;
        if (terr > err) break;
      }
      if (terr < err) {
        err = terr;
        first = lo;
        second = hi;
        type = type_i;
        std::memcpy(best_sel, trial_sel, sizeof(best_sel));
        if (!terr) break;
      }
    }
  }
};

}  // namespace

// compute :40-196, then the selector packing of dxt5_block (crn_dxt.h:318-361)
void dxt5a_block(const uint8_t* px16, int comp, bool both, uint8_t* out8, int quality) {
  Alpha a;
  a.both = both;
  int map[256];
  for (int i = 0; i < 256; i++) map[i] = -1;
  for (int i = 0; i < 16; i++) {
    const unsigned v = px16[i * 4 + comp];
    if (map[v] < 0) {
      map[v] = a.n;
      a.vals[a.n] = v;
      a.wts[a.n] = 0;
      a.n++;
    }
    a.wts[map[v]]++;
  }
  uint8_t sel[16];
  unsigned first, second;
  if (a.n == 1) {
    first = second = a.vals[0];
    std::memset(sel, 0, 16);
  } else {
    for (int i = 0; i + 1 < a.n; i++)
      for (int j = i + 1; j < a.n; j++) a.evaluate(a.vals[i], a.vals[j]);
    if (quality >= 3 && a.err) {
      // +-16 (Uber) or +-8 (Better) probe around the running best (the centre moves when the
      // best improves); none below Better (:105-141)
      const int amount = quality == 4 ? 16 : 8;
      static thread_local std::vector<uint8_t> flags;
      flags.assign(256 * 256, 0);
      for (int ld = -amount; ld <= amount; ld++) {
        const int l = (int)a.first + ld;
        if (l < 0) continue;
        if (l > 255) break;
        for (int hd = -amount; hd <= amount; hd++) {
          const int h = (int)a.second + hd;
          if (h < 0) continue;
          if (h > 255) break;
          if (flags[l * 256 + h] || flags[h * 256 + l]) continue;
          flags[l * 256 + h] = 1;
          a.evaluate((unsigned)l, (unsigned)h);
        }
      }
    }
    static const uint8_t inv6[8] = {1, 0, 5, 4, 3, 2, 6, 7};
    static const uint8_t inv8[8] = {1, 0, 7, 6, 5, 4, 3, 2};
    first = a.first;
    second = a.second;
    uint8_t bsel[16];
    std::memcpy(bsel, a.best_sel, 16);
    if (first == second) {
      std::memset(bsel, 0, 16);
    } else if (a.type) {
      if (first > second) {
        std::swap(first, second);
        for (int i = 0; i < a.n; i++) bsel[i] = inv6[bsel[i]];
      }
    } else if (first <= second) {
      std::swap(first, second);
      for (int i = 0; i < a.n; i++) bsel[i] = inv8[bsel[i]];
    }
    for (int i = 0; i < 16; i++) sel[i] = bsel[map[px16[i * 4 + comp]]];
  }
  out8[0] = (uint8_t)first;
  out8[1] = (uint8_t)second;
  uint64_t bits = 0;
  for (int i = 0; i < 16; i++) bits |= (uint64_t)(sel[i] & 7) << (3 * i);
  for (int k = 0; k < 6; k++) out8[2 + k] = (uint8_t)(bits >> (8 * k));
}

}  // namespace crn_oracle_detail

extern "C" int oracle_dxt5a_blocks(const uint8_t* blocks, uint32_t n, int comp, int use_both_block_types,
                                   uint8_t* out, int threads) {
  (void)threads;
  for (uint32_t i = 0; i < n; i++)
    crn_oracle_detail::dxt5a_block(blocks + (size_t)i * 64, comp, use_both_block_types != 0, out + (size_t)i * 8, 4);
  return 0;
}

extern "C" int oracle_dxt5a_blocks_q(const uint8_t* blocks, uint32_t n, int comp, int use_both_block_types,
                                     int quality, uint8_t* out) {
  if (quality < 0 || quality > 4) return -1;
  for (uint32_t i = 0; i < n; i++)
    crn_oracle_detail::dxt5a_block(blocks + (size_t)i * 64, comp, use_both_block_types != 0, out + (size_t)i * 8,
                                   quality);
  return 0;
}

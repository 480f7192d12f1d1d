// CPU restatement of the reference DXT1 endpoint optimizer (every crn_dxt_quality level,
// perceptual / uniform / grayscale metrics, DXT1A transparency and the transparent-black trial;
// endpoint caching off). TEST INFRASTRUCTURE ONLY: the oracle that the CUDA path is checked
// against, and the CPU baseline. Every stage cites the reference function it restates (crnlib/crn_dxt1.cpp
// unless noted). Float/double expression order and types follow the reference exactly;
// build with -ffp-contract=off.
#include "crn_oracle.h"

#include <cmath>
#include <cstring>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>
#include <algorithm>
#include <atomic>

namespace {

// ---------------------------------------------------------------------------------------
// Single-colour optimal endpoint tables (ryg): for every 8-bit value the (max, min) 5/6-bit
// endpoint pair whose 4-colour (2/3 point) or 3-colour (midpoint) interpolation best hits it,
// with a small penalty on endpoint spread. crnlib/crn_ryg_dxt.cpp:58-99, 517-535.
struct SingleColourTables {
  uint8_t m5[256][2], m6[256][2], m5_3[256][2], m6_3[256][2];
  static void build(uint8_t (*t)[2], int bits, bool three) {
    const int size = 1 << bits;
    for (int v = 0; v < 256; v++) {
      int best = 256;
      for (int lo = 0; lo < size; lo++) {
        for (int hi = 0; hi < size; hi++) {
          int le = bits == 5 ? (lo << 3) | (lo >> 2) : (lo << 2) | (lo >> 4);
          int he = bits == 5 ? (hi << 3) | (hi >> 2) : (hi << 2) | (hi >> 4);
          int interp = three ? ((le + he) >> 1) : ((he * 2 + le) / 3);
          int e = std::abs(interp - v) + ((std::abs(he - le) * 8) >> 8);
          if (e < best) {
            t[v][0] = (uint8_t)hi;
            t[v][1] = (uint8_t)lo;
            best = e;
          }
        }
      }
    }
  }
  SingleColourTables() {
    build(m5, 5, false);
    build(m6, 6, false);
    build(m5_3, 5, true);
    build(m6_3, 6, true);
  }
};
const SingleColourTables& sct() {
  static SingleColourTables t;
  return t;
}

struct RGB { int r, g, b; };

inline int expand5(int v) { return (v << 3) | (v >> 2); }
inline int expand6(int v) { return (v << 2) | (v >> 4); }

// dxt1_block::unpack_color (crnlib/crn_dxt.cpp:167-181)
inline RGB unpack565(uint16_t c, bool scaled) {
  int b = c & 31, g = (c >> 5) & 63, r = (c >> 11) & 31;
  if (scaled) { b = expand5(b); g = expand6(g); r = expand5(r); }
  return {r, g, b};
}
// dxt1_block::pack_color with scaled=false (crnlib/crn_dxt.cpp:142-160), after the
// color_quad_u8 constructor clamp to 0..255 (crn_color.h:305-312).
inline int clamp255(int v) { return v < 0 ? 0 : (v > 255 ? 255 : v); }
inline uint16_t pack565(int r, int g, int b) {
  r = clamp255(r); g = clamp255(g); b = clamp255(b);
  r = std::min(r, 31); g = std::min(g, 63); b = std::min(b, 31);
  return (uint16_t)(b | (g << 5) | (r << 11));
}
// pack_color scaled=true, bias 127
inline uint16_t pack565_scaled(int r, int g, int b) {
  unsigned ur = ((unsigned)r * 31U + 127U) / 255U, ug = ((unsigned)g * 63U + 127U) / 255U,
           ub = ((unsigned)b * 31U + 127U) / 255U;
  ur = std::min(ur, 31U); ug = std::min(ug, 63U); ub = std::min(ub, 31U);
  return (uint16_t)(ub | (ug << 5) | (ur << 11));
}

// color::color_distance without alpha (crn_color.h:728-745)
inline unsigned cdist(bool perceptual, const RGB& a, const RGB& b) {
  int dr = a.r - b.r, dg = a.g - b.g, db = a.b - b.b;
  if (perceptual) return (unsigned)(8 * dr * dr + 25 * dg * dg + db * db);
  return (unsigned)(dr * dr + dg * dg + db * db);
}

// color::RGB_to_Y (crn_color.h:792-796): fixed-point luma
inline int luma(const RGB& c) { return (c.r * 19595 + c.g * 38470 + c.b * 7471 + 32768) >> 16; }

// dxt1_endpoint_optimizer::color_distance (crnlib/crn_dxt1.cpp:1342-1368): the grayscale-sampling
// metric when the perceptual one is off
inline unsigned mdist(bool perceptual, bool gray, const RGB& a, const RGB& b) {
  if (!perceptual && gray) {
    const int yd = luma(a) - luma(b);
    return (unsigned)(yd * yd);
  }
  return cdist(perceptual, a, b);
}

struct V3 { float x[3]; float& operator[](int i) { return x[i]; } float operator[](int i) const { return x[i]; } };

struct Coords {
  uint16_t lo, hi;
  Coords canon() const { Coords c = *this; if (c.lo < c.hi) std::swap(c.lo, c.hi); return c; }
};

struct Solution {
  Coords c{0, 0};
  std::vector<uint8_t> sel;
  uint64_t error = UINT64_MAX;
  bool alpha_block = false, alt = false, enforce = false;
  uint8_t enforced = 0;
};

// probe tables per quality (crn_dxt1.cpp:43-53)
const int16_t kFastProbe[4] = {0, 1, 2, 3};
const int16_t kNormalProbe[5] = {0, 1, 3, 5, 7};
const int16_t kBetterProbe[10] = {0, 1, 2, 3, 5, 9, 15, 19, 27, 43};
const int16_t kUberProbe[15] = {0, 1, 2, 3, 5, 7, 9, 10, 13, 15, 19, 27, 43, 59, 91};
enum { kSuperFast = 0, kFast = 1, kNormal = 2, kBetter = 3, kUber = 4 };
const int8_t kAdj[26][3] = {
    {-1, -1, -1}, {0, -1, -1}, {1, -1, -1}, {-1, 0, -1}, {0, 0, -1}, {1, 0, -1}, {-1, 1, -1}, {0, 1, -1},
    {1, 1, -1},   {-1, -1, 0}, {0, -1, 0},  {1, -1, 0},  {-1, 0, 0}, {1, 0, 0},  {-1, 1, 0},  {0, 1, 0},
    {1, 1, 0},    {-1, -1, 1}, {0, -1, 1},  {1, -1, 1},  {-1, 0, 1}, {0, 0, 1},  {1, 0, 1},  {-1, 1, 1},
    {0, 1, 1},    {1, 1, 1}};

// fast_random (crnlib/crn_rand.cpp:310-405): SHR3 xor CONG, default seed per object.
struct FastRandom {
  uint32_t jsr = 0xABCD917A, jcong = 0x17F3DEAD;
  uint32_t next() {
    jsr ^= (jsr << 17); jsr ^= (jsr >> 13); jsr ^= (jsr << 5);
    jcong = 69069 * jcong + 1234567;
    return jsr ^ jcong;
  }
  float frand(float l, float h) {
    float r = (float)(l + (h - l) * (next() * (1.0 / 4294967296.0)));
    return r < l ? l : (r > h ? h : r);
  }
};

// dxt1_endpoint_optimizer::params (crn_dxt1.h:168-201) as dxt_image::set_block_pixels fills them
struct Dxt1Params {
  bool perceptual = true, use_alpha_blocks = true, grayscale = false, pixels_have_alpha = false;
  bool transparent_black = false;
  int quality = kUber;
  int alpha_threshold = 128;
};

class Dxt1Search {
 public:
  // One block (or cluster) of pixels in, one dxt1 solution out (compute :2234-2245).
  void run(const uint8_t* px, uint32_t n_px, const Dxt1Params& p, uint16_t& out_lo, uint16_t& out_hi,
           uint8_t* out_sel, uint64_t& out_err);
  void run(const uint8_t* px, uint32_t n_px, bool perceptual, bool use_alpha_blocks, uint16_t& out_lo,
           uint16_t& out_hi, uint8_t* out_sel, uint64_t& out_err) {
    Dxt1Params p;
    p.perceptual = perceptual;
    p.use_alpha_blocks = use_alpha_blocks;
    run(px, n_px, p, out_lo, out_hi, out_sel, out_err);
  }

 private:
  void compute_internal(const uint8_t* px, uint32_t n_px, const Dxt1Params& p, uint16_t& out_lo, uint16_t& out_hi,
                        uint8_t* out_sel, uint64_t& out_err);
  bool perceptual_ = true, use_alpha_ = true, hc_ = false, gray_ = false, have_alpha_ = false;
  int quality_ = kUber;
  std::vector<RGB> uc_;
  std::vector<uint32_t> w_;
  std::unordered_map<uint32_t, uint32_t> index_;
  uint32_t total_w_ = 0;
  uint64_t rdist_[32][2], gdist_[64][2], bdist_[32][2];  // [c][0]=low, [c][1]=high
  Solution best_, trial_;
  std::vector<uint8_t> trial_sel_;
  std::unordered_set<uint32_t> tried_;
  std::vector<V3> norm_, normw_;
  V3 mean_{}, meanw_{}, axis_{};

  bool evaluate(Coords c, bool alt = false);
  bool evaluate_uber(Coords c, bool alt);
  bool evaluate_fast(Coords c, bool alt);
  bool evaluate_hc(Coords c, bool alt);
  void compute_selectors();
  void compute_vectors(const V3& pw);
  void compute_pca(V3& axis, const std::vector<V3>& v, const V3& def);
  void handle_multicolor();
  void optimize_endpoints(V3 low, V3 high);
  bool try_median4(const V3& low, const V3& high);
  bool refine(int level);
  bool try_average_block_as_solid();
  void component_errors(int comp, uint64_t (&err)[4][256], uint64_t (&rem)[4]);
  void optimize_endpoint_comps();
  void try_combinatorial();
  bool all_selectors_equal() const {
    if (best_.sel.empty()) return false;
    for (size_t i = 1; i < best_.sel.size(); i++) if (best_.sel[i] != best_.sel[0]) return false;
    return true;
  }
};

// evaluate_solution :1312-1340 -- plane-table lower bound, tried-set, then the error kernel.
bool Dxt1Search::evaluate(Coords c, bool alt) {
  RGB c0 = unpack565(c.lo, false), c1 = unpack565(c.hi, false);
  uint64_t re = c0.r < c1.r ? rdist_[c0.r][0] + rdist_[c1.r][1] : rdist_[c0.r][1] + rdist_[c1.r][0];
  uint64_t ge = c0.g < c1.g ? gdist_[c0.g][0] + gdist_[c1.g][1] : gdist_[c0.g][1] + gdist_[c1.g][0];
  uint64_t be = c0.b < c1.b ? bdist_[c0.b][0] + bdist_[c1.b][1] : bdist_[c0.b][1] + bdist_[c1.b][0];
  if (re + ge + be >= best_.error) return false;
  if (!alt) {
    if (!tried_.insert((uint32_t)c.lo | ((uint32_t)c.hi << 16)).second) return false;
  }
  if (hc_) return evaluate_hc(c, alt);
  return quality_ >= kBetter ? evaluate_uber(c, alt) : evaluate_fast(c, alt);
}

// Candidate x unique-colour evaluations of the reference's loops (the encoder's unit of
// algorithmic work): colours visited per evaluated candidate, the larger of the two block types'
// loops where both run. Counted per thread, summed by oracle_dxt1_count_evaluations.
thread_local uint64_t t_evals = 0;

// evaluate_solution_uber :1370-1592
bool Dxt1Search::evaluate_uber(Coords c, bool alt) {
  const int n = (int)uc_.size();
  trial_.c = c;
  trial_.sel.resize(n);
  trial_.error = best_.error;
  trial_.alpha_block = false;
  trial_sel_.resize(n);
  RGB col[4];
  col[0] = unpack565(c.lo, true);
  col[1] = unpack565(c.hi, true);
  const int a = alt ? 1 : 0;
  const int first_type = have_alpha_ ? 1 : 0;
  const int last_type = (have_alpha_ || use_alpha_) ? 1 : 0;
  int visited_max = 0;
  for (int type = first_type; type <= last_type; type++) {
    uint64_t terr = 0;
    int ncol, visited = 0;
    if (type == 0) {
      col[2] = {(col[0].r * 2 + col[1].r + a) / 3, (col[0].g * 2 + col[1].g + a) / 3, (col[0].b * 2 + col[1].b + a) / 3};
      col[3] = {(col[1].r * 2 + col[0].r + a) / 3, (col[1].g * 2 + col[0].g + a) / 3, (col[1].b * 2 + col[0].b + a) / 3};
      ncol = 4;
    } else {
      col[2] = {(col[0].r + col[1].r + a) >> 1, (col[0].g + col[1].g + a) >> 1, (col[0].b + col[1].b + a) >> 1};
      ncol = 3;
    }
    for (int i = n - 1; i >= 0; i--) {
      visited++;
      unsigned be = mdist(perceptual_, gray_, uc_[i], col[0]);
      int bi = 0;
      for (int k = 1; k < ncol; k++) {
        unsigned e = mdist(perceptual_, gray_, uc_[i], col[k]);
        if (e < be) { be = e; bi = k; }
      }
      terr += (uint64_t)be * w_[i];
      if (terr >= trial_.error) break;
      trial_sel_[i] = (uint8_t)bi;
    }
    visited_max = std::max(visited_max, visited);
    if (terr < trial_.error) {
      trial_.error = terr;
      trial_.alpha_block = type != 0;
      trial_.sel = trial_sel_;
      trial_.alt = alt;
    }
  }
  t_evals += (uint64_t)visited_max;
  trial_.enforce = !trial_.alpha_block && trial_.c.lo == trial_.c.hi;
  if (trial_.enforce) {
    uint8_t s;
    if ((trial_.c.lo & 31) != 31) { trial_.c.lo++; s = 1; }
    else { trial_.c.hi--; s = 0; }
    for (int i = 0; i < n; i++) trial_.sel[i] = s;
    trial_.enforced = s;
  }
  if (trial_.error < best_.error) {
    best_ = trial_;
    return true;
  }
  return false;
}

// evaluate_solution_fast :1594-1757: selectors by projection onto the endpoint axis, then the
// distance to the chosen colour. It leaves m_alternate_rounding and m_enforce_selector alone, so
// the bumped equal-endpoint case keeps the flags of the trial before it (never set below Better).
bool Dxt1Search::evaluate_fast(Coords c, bool alt) {
  const int n = (int)uc_.size();
  trial_.c = c;
  trial_.sel.resize(n);
  trial_.error = best_.error;
  trial_.alpha_block = false;
  trial_sel_.resize(n);
  RGB col[4];
  col[0] = unpack565(c.lo, true);
  col[1] = unpack565(c.hi, true);
  int vr = col[1].r - col[0].r, vg = col[1].g - col[0].g, vb = col[1].b - col[0].b;
  if (perceptual_) {
    vr *= 8;
    vg *= 24;
  }
  auto dot = [&](const RGB& q) { return q.r * vr + q.g * vg + q.b * vb; };
  int stops[4];
  stops[0] = dot(col[0]);
  stops[1] = dot(col[1]);
  const int dr = vr * 2, dg = vg * 2, db = vb * 2;
  const int a = alt ? 1 : 0;
  const int first_type = have_alpha_ ? 1 : 0;
  const int last_type = (have_alpha_ || use_alpha_) ? 1 : 0;
  for (int type = first_type; type <= last_type; type++) {
    uint64_t terr = 0;
    if (type == 0) {
      col[2] = {(col[0].r * 2 + col[1].r + a) / 3, (col[0].g * 2 + col[1].g + a) / 3, (col[0].b * 2 + col[1].b + a) / 3};
      col[3] = {(col[1].r * 2 + col[0].r + a) / 3, (col[1].g * 2 + col[0].g + a) / 3, (col[1].b * 2 + col[0].b + a) / 3};
      stops[2] = dot(col[2]);
      stops[3] = dot(col[3]);
      const int c0p = stops[1] + stops[3], halfp = stops[3] + stops[2], c3p = stops[2] + stops[0];
      for (int i = n - 1; i >= 0; i--) {
        const int d = uc_[i].r * dr + uc_[i].g * dg + uc_[i].b * db;
        const int bi = d >= halfp ? (d < c0p ? 3 : 1) : (d < c3p ? 0 : 2);
        terr += (uint64_t)mdist(perceptual_, gray_, uc_[i], col[bi]) * w_[i];
        if (terr >= trial_.error) break;
        trial_sel_[i] = (uint8_t)bi;
      }
    } else {
      col[2] = {(col[0].r + col[1].r + a) >> 1, (col[0].g + col[1].g + a) >> 1, (col[0].b + col[1].b + a) >> 1};
      stops[2] = dot(col[2]);
      const int c02 = stops[0] + stops[2], c21 = stops[2] + stops[1];
      for (int i = n - 1; i >= 0; i--) {
        const int d = uc_[i].r * dr + uc_[i].g * dg + uc_[i].b * db;
        const int bi = d < c02 ? 0 : (d < c21 ? 2 : 1);
        terr += (uint64_t)mdist(perceptual_, gray_, uc_[i], col[bi]) * w_[i];
        if (terr >= trial_.error) break;
        trial_sel_[i] = (uint8_t)bi;
      }
    }
    if (terr < trial_.error) {
      trial_.error = terr;
      trial_.alpha_block = type != 0;
      trial_.sel = trial_sel_;
    }
  }
  if (!trial_.alpha_block && trial_.c.lo == trial_.c.hi) {
    uint8_t s;
    if ((trial_.c.lo & 31) != 31) { trial_.c.lo++; s = 1; }
    else { trial_.c.hi--; s = 0; }
    for (int i = 0; i < n; i++) trial_.sel[i] = s;
  }
  if (trial_.error < best_.error) {
    best_ = trial_;
    return true;
  }
  return false;
}

// evaluate_solution_hc_perceptual / _uniform :1759-1835 (4-colour only; selectors are
// recomputed lazily by compute_selectors_hc)
bool Dxt1Search::evaluate_hc(Coords c, bool alt) {
  RGB c0 = unpack565(c.lo, true), c1 = unpack565(c.hi, true);
  const int a = alt ? 1 : 0;
  RGB c2 = {(c0.r * 2 + c1.r + a) / 3, (c0.g * 2 + c1.g + a) / 3, (c0.b * 2 + c1.b + a) / 3};
  RGB c3 = {(c1.r * 2 + c0.r + a) / 3, (c1.g * 2 + c0.g + a) / 3, (c1.b * 2 + c0.b + a) / 3};
  uint64_t err = 0;
  for (size_t i = 0; i < uc_.size() && err < best_.error; i++) {
    t_evals++;
    unsigned e01 = std::min(cdist(perceptual_, uc_[i], c0), cdist(perceptual_, uc_[i], c1));
    unsigned e23 = std::min(cdist(perceptual_, uc_[i], c2), cdist(perceptual_, uc_[i], c3));
    err += (uint64_t)std::min(e01, e23) * w_[i];
  }
  if (err >= best_.error) return false;
  best_.c = c;
  best_.error = err;
  best_.alpha_block = false;
  best_.alt = alt;
  best_.enforce = c.lo == c.hi;
  if (best_.enforce) {
    if ((best_.c.lo & 31) != 31) { best_.c.lo++; best_.enforced = 1; }
    else { best_.c.hi--; best_.enforced = 0; }
  }
  return true;
}

// compute_selectors / compute_selectors_hc :1837-1869 (no-op outside the hc path)
void Dxt1Search::compute_selectors() {
  if (!hc_) return;
  const int n = (int)uc_.size();
  best_.sel.resize(n);
  if (best_.enforce) {
    std::fill(best_.sel.begin(), best_.sel.end(), best_.enforced);
    return;
  }
  RGB c0 = unpack565(best_.c.lo, true), c1 = unpack565(best_.c.hi, true);
  const int a = best_.alt ? 1 : 0;
  RGB c2 = {(c0.r * 2 + c1.r + a) / 3, (c0.g * 2 + c1.g + a) / 3, (c0.b * 2 + c1.b + a) / 3};
  RGB c3 = {(c1.r * 2 + c0.r + a) / 3, (c1.g * 2 + c0.g + a) / 3, (c1.b * 2 + c0.b + a) / 3};
  for (int i = 0; i < n; i++) {
    unsigned e0 = cdist(perceptual_, uc_[i], c0), e1 = cdist(perceptual_, uc_[i], c1);
    unsigned e2 = cdist(perceptual_, uc_[i], c2), e3 = cdist(perceptual_, uc_[i], c3);
    unsigned e01 = std::min(e0, e1), e23 = std::min(e2, e3);
    best_.sel[i] = e01 <= e23 ? (e01 == e0 ? 0 : 1) : (e23 == e2 ? 2 : 3);
  }
}

// compute_vectors :155-189
void Dxt1Search::compute_vectors(const V3& pw) {
  const size_t n = uc_.size();
  norm_.resize(n);
  normw_.resize(n);
  for (int k = 0; k < 3; k++) { mean_[k] = 0.0f; meanw_[k] = 0.0f; }
  for (size_t i = 0; i < n; i++) {
    V3 v{{(float)uc_[i].r * 1.0f / 255.0f, (float)uc_[i].g * 1.0f / 255.0f, (float)uc_[i].b * 1.0f / 255.0f}};
    V3 vw{{pw[0] * v[0], pw[1] * v[1], pw[2] * v[2]}};
    norm_[i] = v;
    normw_[i] = vw;
    const float wf = (float)w_[i];
    for (int k = 0; k < 3; k++) {
      mean_[k] += v[k] * wf;
      meanw_[k] += vw[k] * wf;
    }
  }
  if (total_w_) {
    const float inv = 1.0f / (float)total_w_;
    for (int k = 0; k < 3; k++) { mean_[k] *= inv; meanw_[k] *= inv; }
  }
  for (size_t i = 0; i < n; i++)
    for (int k = 0; k < 3; k++) { norm_[i][k] -= mean_[k]; normw_[i][k] -= meanw_[k]; }
}

// compute_pca :192-256 (double covariance, 8 power iterations)
void Dxt1Search::compute_pca(V3& axis, const std::vector<V3>& v, const V3& def) {
  double cov[6] = {0, 0, 0, 0, 0, 0};
  for (size_t i = 0; i < v.size(); i++) {
    const float r = v[i][0], g = v[i][1], b = v[i][2];
    if (w_[i] > 1) {
      const double wt = (double)w_[i];
      cov[0] += (double)(r * r) * wt; cov[1] += (double)(r * g) * wt; cov[2] += (double)(r * b) * wt;
      cov[3] += (double)(g * g) * wt; cov[4] += (double)(g * b) * wt; cov[5] += (double)(b * b) * wt;
    } else {
      cov[0] += (double)(r * r); cov[1] += (double)(r * g); cov[2] += (double)(r * b);
      cov[3] += (double)(g * g); cov[4] += (double)(g * b); cov[5] += (double)(b * b);
    }
  }
  double vfr = (double).9f, vfg = (double)1.0f, vfb = (double).7f;
  for (int it = 0; it < 8; it++) {
    double r = vfr * cov[0] + vfg * cov[1] + vfb * cov[2];
    double g = vfr * cov[1] + vfg * cov[3] + vfb * cov[4];
    double b = vfr * cov[2] + vfg * cov[4] + vfb * cov[5];
    double m = std::fabs(r);
    if (std::fabs(g) > m) m = std::fabs(g);
    if (std::fabs(b) > m) m = std::fabs(b);
    if (m > 1e-10) {
      m = 1.0 / m;
      r *= m; g *= m; b *= m;
    }
    double delta = (vfr - r) * (vfr - r) + (vfg - g) * (vfg - g) + (vfb - b) * (vfb - b);
    vfr = r; vfg = g; vfb = b;
    if (it > 2 && delta < 1e-8) break;
  }
  double len = vfr * vfr + vfg * vfg + vfb * vfb;
  if (len < 1e-10) {
    axis = def;
  } else {
    len = 1.0 / std::sqrt(len);
    axis[0] = (float)(vfr * len); axis[1] = (float)(vfg * len); axis[2] = (float)(vfb * len);
  }
}

// vec::normalize (crn_vec.h:674-690): float products accumulated in double.
void normalize3(V3& v) {
  double n = (double)(v[0] * v[0]);
  n += (double)(v[1] * v[1]);
  n += (double)(v[2] * v[2]);
  if (n != 0) {
    const float s = (float)(1.0 / std::sqrt(n));
    v[0] *= s; v[1] *= s; v[2] *= s;
  }
}

// intersection::ray_aabb against [0,1]^3 (crn_intersect.h:44-132). Returns true on cSuccess.
bool ray_unit_box(V3& coord, const V3& o, const V3& d) {
  int quad[3];
  float cand[3] = {0, 0, 0};
  bool inside = true;
  for (int i = 0; i < 3; i++) {
    if (o[i] < 0.0f) { quad[i] = 1; cand[i] = 0.0f; inside = false; }
    else if (o[i] > 1.0f) { quad[i] = 0; cand[i] = 1.0f; inside = false; }
    else quad[i] = 2;
  }
  if (inside) { coord = o; return false; }  // cInside: caller keeps the point
  float mt[3];
  for (int i = 0; i < 3; i++)
    mt[i] = (quad[i] != 2 && d[i] != 0.0f) ? (cand[i] - o[i]) / d[i] : -1.0f;
  int wp = 0;
  for (int i = 1; i < 3; i++) if (mt[wp] < mt[i]) wp = i;
  if (mt[wp] < 0.0f) return false;
  V3 c;
  for (int i = 0; i < 3; i++) {
    if (i != wp) {
      c[i] = o[i] + mt[wp] * d[i];
      if (c[i] < 0.0f || c[i] > 1.0f) return false;
    } else {
      c[i] = cand[i];
    }
  }
  coord = c;
  return true;
}

inline bool within01(const V3& v) {
  for (int i = 0; i < 3; i++) if (v[i] < 0.0f || v[i] > 1.0f) return false;
  return true;
}

// handle_multicolor_block :1069-1178
void Dxt1Search::handle_multicolor() {
  int passes = 1;
  V3 pw{{1.0f, 1.0f, 1.0f}};
  if (perceptual_) {
    float red = 0, blue = 0, avel = 0;
    for (size_t i = 0; i < uc_.size(); i++) {
      const int l = (uc_[i].r + uc_[i].g + uc_[i].b + 1) / 3;
      const float lf = (float)l;
      const float scale = (float)w_[i] / (1.0f > lf ? 1.0f : lf);
      red += scale * (float)uc_[i].r;
      blue += scale * (float)uc_[i].b;
      avel += lf;
    }
    red /= (float)total_w_;
    blue /= (float)total_w_;
    avel /= (float)total_w_;
    avel = std::min(1.0f, avel * 16.0f / 255.0f);
    float mx = red > blue ? red : blue;
    float s = mx * 1.0f / 3.0f;
    s = s < 0.0f ? 0.0f : (s > 1.0f ? 1.0f : s);
    const float p = avel * powf(s, 2.75f);
    if (p >= 1.0f) {
      passes = 1;
    } else {
      passes = 2;
      const float a0[3] = {.212f, .72f, .072f};
      for (int k = 0; k < 3; k++) pw[k] = a0[k] + (pw[k] - a0[k]) * p;
    }
  }
  const V3 def{{.2837149f, 0.9540631f, 0.096277453f}};
  for (int pass = 0; pass < passes; pass++) {
    compute_vectors(pw);
    compute_pca(axis_, normw_, def);
    axis_[0] /= pw[0]; axis_[1] /= pw[1]; axis_[2] /= pw[2];
    normalize3(axis_);
    if (passes > 1) {
      if (std::fabs(axis_[0]) >= .795f) { pw[0] = .424f; pw[1] = .6f; pw[2] = .072f; }
      else if (std::fabs(axis_[2]) >= .795f) { pw[0] = .212f; pw[1] = .6f; pw[2] = .212f; }
      else break;
    }
  }
  float l = 1e+9f, h = -1e+9f;
  for (size_t i = 0; i < norm_.size(); i++) {
    float d = norm_[i][0] * axis_[0];
    d += norm_[i][1] * axis_[1];
    d += norm_[i][2] * axis_[2];
    l = d < l ? d : l;
    h = d > h ? d : h;
  }
  V3 low, high;
  for (int k = 0; k < 3; k++) {
    low[k] = mean_[k] + l * axis_[k];
    high[k] = mean_[k] + h * axis_[k];
  }
  if (!within01(low)) {
    V3 c;
    if (ray_unit_box(c, low, axis_)) low = c;
  }
  if (!within01(high)) {
    V3 c;
    V3 nd{{-axis_[0], -axis_[1], -axis_[2]}};
    if (ray_unit_box(c, high, nd)) high = c;
  }
  optimize_endpoints(low, high);
}

// try_median4 :1181-1308
bool Dxt1Search::try_median4(const V3& low, const V3& high) {
  V3 means[4];
  const size_t n = uc_.size();
  if (n <= 4) {
    for (size_t i = 0; i < 4; i++) means[i] = norm_[std::min(n - 1, i)];
  } else {
    for (int k = 0; k < 3; k++) {
      means[0][k] = low[k] - mean_[k];
      means[3][k] = high[k] - mean_[k];
    }
    for (int k = 0; k < 3; k++) {
      means[1][k] = means[0][k] + (means[3][k] - means[0][k]) * (1.0f / 3.0f);
      means[2][k] = means[0][k] + (means[3][k] - means[0][k]) * (2.0f / 3.0f);
    }
    FastRandom rm;
    unsigned rover = 0;
    float prev_total = 1.0e+37f;
    for (unsigned it = 0; it < 8; it++) {
      V3 nm[4] = {};
      float nw[4] = {0, 0, 0, 0};
      float total = 0;
      for (size_t i = 0; i < n; i++) {
        const V3& v = norm_[i];
        auto sqd = [&](const V3& m) {
          float d2 = 0;
          for (int k = 0; k < 3; k++) { float d = m[k] - v[k]; d2 += d * d; }
          return d2;
        };
        float bd = sqd(means[0]);
        int bi = 0;
        for (int j = 1; j < 4; j++) {
          float d = sqd(means[j]);
          if (d < bd) { bd = d; bi = j; }
        }
        total += bd;
        const float wf = (float)w_[i];
        for (int k = 0; k < 3; k++) nm[bi][k] += v[k] * wf;
        nw[bi] += wf;
      }
      unsigned hi_idx = 0;
      float hi_w = 0;
      bool empty = false;
      for (int j = 0; j < 4; j++) {
        if (nw[j] > 0.0f) {
          for (int k = 0; k < 3; k++) means[j][k] = nm[j][k] / nw[j];
          if (nw[j] > hi_w) { hi_w = nw[j]; hi_idx = j; }
        } else {
          empty = true;
        }
      }
      if (!empty) {
        if (std::fabs(total - prev_total) < .00001f) break;
        prev_total = total;
      } else {
        prev_total = 1.0e+37f;
      }
      if (empty && it != 7) {
        const unsigned ri = (hi_idx + rover) & 3;
        rover++;
        for (int j = 0; j < 4; j++) {
          if (nw[j] == 0.0f) {
            means[j] = means[ri];
            for (int k = 0; k < 3; k++) means[j][k] += rm.frand(-.00196f, .00196f);
          }
        }
      }
    }
  }
  bool improved = false;
  for (int i = 0; i < 3; i++) {
    for (int j = i + 1; j < 4; j++) {
      V3 v0, v1;
      for (int k = 0; k < 3; k++) { v0[k] = means[i][k] + mean_[k]; v1[k] = means[j][k] + mean_[k]; }
      Coords sc{pack565((int)std::floor(.5f + v0[0] * 31.0f), (int)std::floor(.5f + v0[1] * 63.0f),
                        (int)std::floor(.5f + v0[2] * 31.0f)),
                pack565((int)std::floor(.5f + v1[0] * 31.0f), (int)std::floor(.5f + v1[1] * 63.0f),
                        (int)std::floor(.5f + v1[2] * 31.0f))};
      improved |= evaluate(sc.canon());
    }
  }
  improved |= refine(quality_ == kUber ? 1 : 0);
  return improved;
}

// refine_solution :525-698 (least-squares endpoints from the current selectors, then the
// 2 x 27 lattice neighbours for level 1)
bool Dxt1Search::refine(int level) {
  compute_selectors();
  static const int w1tab[4] = {3, 0, 2, 1};
  static const int prods0[4] = {0x00, 0x00, 0x02, 0x02};
  static const int prods1[4] = {0x00, 0x09, 0x01, 0x04};
  static const int prods2[4] = {0x09, 0x00, 0x04, 0x01};
  double ak0 = 0, ak1 = 0, ak2 = 0;
  double at1r = 0, at1g = 0, at1b = 0, at2r = 0, at2g = 0, at2b = 0;
  for (size_t i = 0; i < uc_.size(); i++) {
    const double wt = (double)w_[i];
    const double r = uc_[i].r * wt, g = uc_[i].g * wt, b = uc_[i].b * wt;
    const int step = best_.sel[i] ^ 1;
    const int w1 = w1tab[step];
    ak0 += prods0[step] * wt;
    ak1 += prods1[step] * wt;
    ak2 += prods2[step] * wt;
    at1r += w1 * r; at1g += w1 * g; at1b += w1 * b;
    at2r += r; at2g += g; at2b += b;
  }
  at2r = 3 * at2r - at1r;
  at2g = 3 * at2g - at1g;
  at2b = 3 * at2b - at1b;
  const double xx = ak2, yy = ak1, xy = ak0;
  const double t = xx * yy - xy * xy;
  if (!yy || !xx || std::fabs(t) < (double).0000125f) return false;
  const double frb = (double)(3.0f * 31.0f / 255.0f) / t;
  const double fg = frb * (double)(63.0f / 31.0f);
  auto q = [](double v, int hi) {
    int iv = (int)(v + (double)0.5f);
    return iv < 0 ? 0 : (iv > hi ? hi : iv);
  };
  const int hr = q((at1r * yy - at2r * xy) * frb, 31), hg = q((at1g * yy - at2g * xy) * fg, 63),
            hb = q((at1b * yy - at2b * xy) * frb, 31);
  const int lr = q((at2r * xx - at1r * xy) * frb, 31), lg = q((at2g * xx - at1g * xy) * fg, 63),
            lb = q((at2b * xx - at1b * xy) * frb, 31);
  bool improved = false;
  if (level == 0) {
    Coords nc{(uint16_t)((lr << 11) | (lg << 5) | lb), (uint16_t)((hr << 11) | (hg << 5) | hb)};
    improved |= evaluate(nc.canon());
  } else {
    int e[2][3] = {{hr, hg, hb}, {lr, lg, lb}};
    for (int i = 0; i < 2; i++) {
      for (int rr = -1; rr <= 1; rr++) {
        for (int gr = -1; gr <= 1; gr++) {
          for (int br = -1; br <= 1; br++) {
            int c[2][3] = {{e[0][0], e[0][1], e[0][2]}, {e[1][0], e[1][1], e[1][2]}};
            c[i][0] = std::min(std::max(c[i][0] + rr, 0), 31);
            c[i][1] = std::min(std::max(c[i][1] + gr, 0), 63);
            c[i][2] = std::min(std::max(c[i][2] + br, 0), 31);
            Coords nc{pack565(c[0][0], c[0][1], c[0][2]), pack565(c[1][0], c[1][1], c[1][2])};
            improved |= evaluate(nc.canon());
          }
        }
      }
    }
  }
  return improved;
}

// try_average_block_as_solid :93-153
bool Dxt1Search::try_average_block_as_solid() {
  const SingleColourTables& T = sct();
  uint64_t tr = 0, tg = 0, tb = 0;
  uint32_t tw = 0;
  for (size_t i = 0; i < uc_.size(); i++) {
    tw += w_[i];
    tr += (uint64_t)uc_[i].r * w_[i];
    tg += (uint64_t)uc_[i].g * w_[i];
    tb += (uint64_t)uc_[i].b * w_[i];
  }
  const uint32_t half = tw >> 1;
  const unsigned ar = (unsigned)((tr + half) / tw), ag = (unsigned)((tg + half) / tw), ab = (unsigned)((tb + half) / tw);
  auto solid4 = [&](unsigned r, unsigned g, unsigned b) {
    return Coords{(uint16_t)((T.m5[r][0] << 11) | (T.m6[g][0] << 5) | T.m5[b][0]),
                  (uint16_t)((T.m5[r][1] << 11) | (T.m6[g][1] << 5) | T.m5[b][1])};
  };
  auto solid3 = [&](unsigned r, unsigned g, unsigned b) {
    return Coords{(uint16_t)((T.m5_3[r][0] << 11) | (T.m6_3[g][0] << 5) | T.m5_3[b][0]),
                  (uint16_t)((T.m5_3[r][1] << 11) | (T.m6_3[g][1] << 5) | T.m5_3[b][1])};
  };
  bool improved = evaluate(solid4(ar, ag, ab));
  if (use_alpha_ && best_.error) improved |= evaluate(solid3(ar, ag, ab));
  if (quality_ != kUber) return improved;
  for (size_t i = 0; i < uc_.size(); i++) {
    const unsigned r = uc_[i].r, g = uc_[i].g, b = uc_[i].b;
    if (r == ar && g == ag && b == ab) continue;
    improved |= evaluate(solid4(r, g, b));
    if (use_alpha_ && best_.error) improved |= evaluate(solid3(r, g, b));
  }
  return improved;
}

// compute_endpoint_component_errors :369-413
void Dxt1Search::component_errors(int comp, uint64_t (&err)[4][256], uint64_t (&rem)[4]) {
  uint64_t W[4] = {0, 0, 0, 0}, WP2[4] = {0, 0, 0, 0}, WPP[4] = {0, 0, 0, 0};
  for (size_t i = 0; i < uc_.size(); i++) {
    const uint64_t p = (uint64_t)(comp == 0 ? uc_[i].r : comp == 1 ? uc_[i].g : uc_[i].b);
    const uint64_t w = w_[i];
    const int s = best_.sel[i];
    W[s] += w;
    WP2[s] += w * p * 2;
    WPP[s] += w * p * p;
  }
  const int limit = comp == 1 ? 64 : 32;
  for (int s = 0; s < 2; s++) {
    uint64_t b = err[s][0] = WPP[s];
    for (int c = 1; c < limit; c++) {
      const uint64_t p = (uint64_t)(comp == 1 ? expand6(c) : expand5(c));
      err[s][c] = W[s] * p * p - WP2[s] * p + WPP[s];
      if (err[s][c] < b) b = err[s][c];
    }
    rem[s] = b;
  }
  for (int s = 2; s < 4; s++) {
    uint64_t b = err[s][0] = WPP[s];
    uint64_t d = W[s] - WP2[s];
    const uint64_t dd = W[s] << 1;
    uint64_t e = WPP[s] + d;
    for (int p = 1; p < 256; p++) {
      err[s][p] = e;
      if (e < b) b = e;
      d += dd;
      e += d;
    }
    rem[s] = b;
  }
  for (int s = 3; s > 0; s--) rem[s - 1] += rem[s];
}

// optimize_endpoint_comps :415-486
void Dxt1Search::optimize_endpoint_comps() {
  compute_selectors();
  if (best_.alpha_block || !best_.error) return;
  const RGB src_lo = unpack565(best_.c.lo, true), src_hi = unpack565(best_.c.hi, true);
  uint64_t err[4][256], rem[4];
  for (int comp = 0; comp < 3; comp++) {
    int p0 = comp == 0 ? src_lo.r : comp == 1 ? src_lo.g : src_lo.b;
    int p1 = comp == 0 ? src_hi.r : comp == 1 ? src_hi.g : src_hi.b;
    RGB lo = unpack565(best_.c.lo, false), hi = unpack565(best_.c.hi, false);
    int* plo = comp == 0 ? &lo.r : comp == 1 ? &lo.g : &lo.b;
    int* phi = comp == 0 ? &hi.r : comp == 1 ? &hi.g : &hi.b;
    component_errors(comp, err, rem);
    uint64_t best_err = err[0][*plo] + err[1][*phi] + err[2][(p0 * 2 + p1) / 3] + err[3][(p0 + p1 * 2) / 3];
    if (rem[0] >= best_err) continue;
    const int limit = comp == 1 ? 64 : 32;
    for (int c0 = 0; c0 < limit; c0++) {
      uint64_t e0 = err[0][c0];
      if (e0 + rem[1] >= best_err) continue;
      *plo = c0;
      const uint16_t packed_lo = pack565(lo.r, lo.g, lo.b);
      p0 = comp == 1 ? expand6(c0) : expand5(c0);
      for (int c1 = 0; c1 < limit; c1++) {
        uint64_t e = e0 + err[1][c1];
        if (e + rem[2] >= best_err) continue;
        p1 = comp == 1 ? expand6(c1) : expand5(c1);
        e += err[2][(p0 * 2 + p1) / 3];
        if (e + rem[3] >= best_err) continue;
        e += err[3][(p0 + p1 * 2) / 3];
        if (e >= best_err) continue;
        *phi = c1;
        if (!evaluate(Coords{packed_lo, pack565(hi.r, hi.g, hi.b)})) continue;
        if (!best_.error) return;
        compute_selectors();
        component_errors(comp, err, rem);
        best_err = err[0][c0] + err[1][c1] + err[2][(p0 * 2 + p1) / 3] + err[3][(p0 + p1 * 2) / 3];
        e0 = err[0][c0];
        if (e0 + rem[1] >= best_err) break;
      }
    }
  }
}

// lerp_color :1871-1883
inline RGB lerp_colour(const RGB& a, const RGB& b, float f, int rounding = 1) {
  const float r = rounding ? 1.0f : 0.0f;
  auto one = [&](int x, int y) {
    const float fx = (float)x, fy = (float)y;
    return clamp255((int)(r + (fx + (fy - fx) * f)));
  };
  return {one(a.r, b.r), one(a.g, b.g), one(a.b, b.b)};
}

// try_combinatorial_encoding :1886-1997
void Dxt1Search::try_combinatorial() {
  const size_t n = uc_.size();
  if (n < 2 || n > 4) return;
  std::vector<RGB> tmp(uc_.begin(), uc_.end());
  if (n == 2) {
    for (int k = 0; k < 2; k++) {
      for (int q = 0; q < 2; q++) {
        const int r = q ^ 1;
        static const float fs[10] = {2.0f, 3.0f, .5f, 1.5f, -1.0f, 2.0f, -.5f, .5f, -2.0f, -1.0f};
        for (float f : fs) tmp.push_back(lerp_colour(tmp[q], tmp[r], f, k));
      }
    }
  } else if (n == 3) {
    for (int i = 0; i <= 2; i++) {
      for (int j = 0; j <= 2; j++) {
        if (i == j) continue;
        tmp.push_back(lerp_colour(tmp[i], tmp[j], 1.5f));
        tmp.push_back(lerp_colour(tmp[i], tmp[j], 2.0f / 3.0f));
        tmp.push_back(lerp_colour(tmp[i], tmp[j], 1.0f / 3.0f));
        tmp.push_back(lerp_colour(tmp[i], tmp[j], -.5f));
      }
    }
  }
  std::vector<uint16_t> packed;
  for (const RGB& c : tmp) {
    const uint16_t p = pack565_scaled(c.r, c.g, c.b);
    if (std::find(packed.begin(), packed.end(), p) == packed.end()) packed.push_back(p);
  }
  for (size_t i = 0; best_.error && i + 1 < packed.size(); i++)
    for (size_t j = i + 1; best_.error && j < packed.size(); j++) evaluate(Coords{packed[i], packed[j]});
  const uint64_t saved = best_.error;
  if (saved) best_.error = 1;
  for (size_t i = 0; best_.error && i + 1 < packed.size(); i++)
    for (size_t j = i + 1; best_.error && j < packed.size(); j++) evaluate(Coords{packed[i], packed[j]}, true);
  if (best_.error) best_.error = saved;
}

// optimize_endpoints :703-1067: the probe table, probe spacing and pass count of the quality
// level, then the lattice moves (Normal and up; +-2 moves and per-pass refines at Uber only)
void Dxt1Search::optimize_endpoints(V3 low, V3 high) {
  const V3 orig_low = low, orig_high = high;
  const int16_t* table = kUberProbe;
  int probe_range = 15, passes = 4;
  float dist_per_trial = .015625f;
  switch (quality_) {
    case kSuperFast: table = kFastProbe; probe_range = 4; dist_per_trial = .027063293f; passes = 1; break;
    case kFast: table = kFastProbe; probe_range = 4; dist_per_trial = .027063293f; passes = 2; break;
    case kNormal: table = kNormalProbe; probe_range = 5; dist_per_trial = .027063293f; passes = 2; break;
    case kBetter: table = kBetterProbe; probe_range = 10; passes = 2; break;
    default: break;
  }
  if (quality_ >= kBetter) try_median4(orig_low, orig_high);
  V3 sa[2];
  for (int k = 0; k < 3; k++) sa[1][k] = axis_[k] * dist_per_trial;
  sa[1][0] *= 31.0f; sa[1][1] *= 63.0f; sa[1][2] *= 31.0f;
  for (int k = 0; k < 3; k++) sa[0][k] = -sa[1][k];
  auto clampf = [](float v, float hi) { return v < 0.0f ? 0.0f : (v > hi ? hi : v); };
  low[0] = clampf(low[0] * 31.0f, 31.0f); low[1] = clampf(low[1] * 63.0f, 63.0f); low[2] = clampf(low[2] * 31.0f, 31.0f);
  high[0] = clampf(high[0] * 31.0f, 31.0f); high[1] = clampf(high[1] * 63.0f, 63.0f); high[2] = clampf(high[2] * 31.0f, 31.0f);

  for (int pass = 0; pass < passes; pass++) {
    if (pass) {
      RGB lo = unpack565(best_.c.lo, false), hi = unpack565(best_.c.hi, false);
      low[0] = (float)lo.r; low[1] = (float)lo.g; low[2] = (float)lo.b;
      high[0] = (float)hi.r; high[1] = (float)hi.g; high[2] = (float)hi.b;
    }
    const uint64_t prev_best = best_.error;
    if (!prev_best) break;
    auto sweep = [&](const V3& base, uint16_t* out) {
      int prev[2] = {-1, -1};
      int cnt = 0;
      V3 init;
      for (int k = 0; k < 3; k++) init[k] = base[k] + .5f;
      for (int i = 0; i < probe_range; i++) {
        const int x = table[i];
        for (int s = i ? 0 : 1; s < 2; s++) {
          float pr = init[0] + sa[s][0] * (float)x, pg = init[1] + sa[s][1] * (float)x, pb = init[2] + sa[s][2] * (float)x;
          int r = std::min(std::max((int)std::floor(pr), 0), 31);
          int g = std::min(std::max((int)std::floor(pg), 0), 63);
          int b = std::min(std::max((int)std::floor(pb), 0), 31);
          int packed = b | (g << 5) | (r << 11);
          if (packed != prev[s]) { out[cnt++] = (uint16_t)packed; prev[s] = packed; }
        }
      }
      return cnt;
    };
    uint16_t pl[31], ph[31];
    const int nl = sweep(low, pl), nh = sweep(high, ph);
    for (int i = 0; i < nl; i++)
      for (int j = 0; j < nh; j++) evaluate(Coords{pl[i], ph[j]}.canon());

    if (quality_ >= kNormal) {
      // low endpoint: 26 lattice neighbours, then (Uber) +-2 along each axis; then the high one
      for (int side = 0; side < 2; side++) {
        RGB base = unpack565(side ? best_.c.hi : best_.c.lo, false);
        for (int i = 0; i < 26; i++) {
          int r = base.r + kAdj[i][0], g = base.g + kAdj[i][1], b = base.b + kAdj[i][2];
          if (r < 0 || r > 31 || g < 0 || g > 63 || b < 0 || b > 31) continue;
          const uint16_t m = pack565(r, g, b);
          evaluate((side ? Coords{best_.c.lo, m} : Coords{m, best_.c.hi}).canon());
        }
        if (quality_ == kUber) {
          base = unpack565(side ? best_.c.hi : best_.c.lo, false);
          for (int a = 0; a < 3; a++) {
            const int limit = a == 1 ? 63 : 31;
            for (int s = -2; s <= 2; s += 4) {
              int c[3] = {base.r, base.g, base.b};
              const int qv = c[a] + s;
              if (qv < 0 || qv > limit) continue;
              c[a] = qv;
              const uint16_t m = pack565(c[0], c[1], c[2]);
              evaluate((side ? Coords{best_.c.lo, m} : Coords{m, best_.c.hi}).canon());
            }
          }
        }
      }
    }
    if (!best_.error || (pass && best_.error == prev_best)) break;
    if (quality_ >= kUber) refine(1);
  }
  if (quality_ >= kNormal) {
    if (best_.error && !have_alpha_) {
      bool solid = false;
      if (all_selectors_equal()) solid = try_average_block_as_solid();
      if (!solid && quality_ == kUber) optimize_endpoint_comps();
    }
    if (quality_ == kUber && best_.error) try_combinatorial();
  }
}

// compute :2234-2245: compute_internal, then (DXT1 with 3-colour blocks allowed, no real
// transparency) try_alpha_as_black_optimization :2001-2079, which re-encodes the block with its
// near-black texels (every channel <= 4) made transparent and keeps that 3-colour encoding when
// its error over all texels (black for selector 3) is lower
void Dxt1Search::run(const uint8_t* px, uint32_t n_px, const Dxt1Params& p, uint16_t& out_lo, uint16_t& out_hi,
                     uint8_t* out_sel, uint64_t& out_err) {
  compute_internal(px, n_px, p, out_lo, out_hi, out_sel, out_err);
  if (!(p.use_alpha_blocks && p.transparent_black && !p.pixels_have_alpha)) return;
  size_t dark = 0;
  for (const RGB& c : uc_) dark += (c.r <= 4 && c.g <= 4 && c.b <= 4) ? 1 : 0;
  if (!dark || dark == uc_.size()) return;
  std::vector<uint8_t> trial(px, px + (size_t)n_px * 4);
  for (uint32_t i = 0; i < n_px; i++)
    if (trial[i * 4] <= 4 && trial[i * 4 + 1] <= 4 && trial[i * 4 + 2] <= 4) trial[i * 4 + 3] = 0;
  Dxt1Params tp = p;
  tp.pixels_have_alpha = true;
  uint16_t tlo, thi;
  std::vector<uint8_t> tsel(n_px);
  uint64_t terr_opt;
  compute_internal(trial.data(), n_px, tp, tlo, thi, tsel.data(), terr_opt);
  // dxt1_block::get_block_colors3 (crn_dxt.cpp:234-245)
  RGB c[4];
  c[0] = unpack565(tlo, true);
  c[1] = unpack565(thi, true);
  c[2] = {(c[0].r + c[1].r) >> 1, (c[0].g + c[1].g) >> 1, (c[0].b + c[1].b) >> 1};
  c[3] = {0, 0, 0};
  uint64_t terr = 0;
  for (uint32_t i = 0; i < n_px; i++)
    terr += mdist(perceptual_, gray_, RGB{trial[i * 4], trial[i * 4 + 1], trial[i * 4 + 2]}, c[tsel[i]]);
  if (terr < out_err) {
    out_err = terr;
    out_lo = tlo;
    out_hi = thi;
    std::memcpy(out_sel, tsel.data(), n_px);
  }
}

// compute_internal :2081-2232 + return_solution :263-365
void Dxt1Search::compute_internal(const uint8_t* px, uint32_t n_px, const Dxt1Params& p, uint16_t& out_lo,
                                  uint16_t& out_hi, uint8_t* out_sel, uint64_t& out_err) {
  gray_ = p.grayscale;
  perceptual_ = p.perceptual && !p.grayscale;
  use_alpha_ = p.use_alpha_blocks;
  have_alpha_ = p.pixels_have_alpha;
  quality_ = p.quality;
  hc_ = quality_ == kUber && !have_alpha_ && !use_alpha_ && !gray_;
  uc_.clear();
  w_.clear();
  index_.clear();
  tried_.clear();
  best_ = Solution();
  total_w_ = 0;
  const uint32_t kTransparent = 0xFFFFFFFFu;
  std::vector<uint32_t> px_index(n_px);
  for (uint32_t i = 0; i < n_px; i++) {
    if (have_alpha_ && px[i * 4 + 3] < p.alpha_threshold) {
      px_index[i] = kTransparent;
      continue;
    }
    const uint32_t key = (uint32_t)px[i * 4] | ((uint32_t)px[i * 4 + 1] << 8) | ((uint32_t)px[i * 4 + 2] << 16);
    auto it = index_.find(key);
    if (it == index_.end()) {
      index_.emplace(key, (uint32_t)uc_.size());
      px_index[i] = (uint32_t)uc_.size();
      uc_.push_back({px[i * 4], px[i * 4 + 1], px[i * 4 + 2]});
      w_.push_back(1);
    } else {
      px_index[i] = it->second;
      w_[it->second]++;
    }
    total_w_++;
  }
  const bool has_transparent = total_w_ != n_px;
  // plane tables -> per-channel lower bounds on the endpoint error
  uint64_t plane[3][64][3];
  std::memset(plane, 0, sizeof(plane));
  for (size_t i = 0; i < uc_.size(); i++) {
    const uint64_t w = w_[i];
    const int R = uc_[i].r, G = uc_[i].g, B = uc_[i].b;
    const int r = (R >> 3) + ((R & 7) > (R >> 5) ? 1 : 0);
    const int g = (G >> 2) + ((G & 3) > (G >> 6) ? 1 : 0);
    const int b = (B >> 3) + ((B & 7) > (B >> 5) ? 1 : 0);
    plane[0][r][0] += w; plane[0][r][1] += w * R; plane[0][r][2] += w * R * R;
    plane[1][g][0] += w; plane[1][g][1] += w * G; plane[1][g][2] += w * G * G;
    plane[2][b][0] += w; plane[2][b][1] += w * B; plane[2][b][2] += w * B * B;
  }
  if (perceptual_) {
    for (int c = 0; c < 32; c++) for (int k = 0; k < 3; k++) plane[0][c][k] *= 8;
    for (int c = 0; c < 64; c++) for (int k = 0; k < 3; k++) plane[1][c][k] *= 25;
  }
  for (int ch = 0; ch < 3; ch++) {
    const int lim = ch == 1 ? 64 : 32;
    for (int c = 1; c < lim; c++) for (int k = 0; k < 3; k++) plane[ch][c][k] += plane[ch][c - 1][k];
  }
  for (int c = 0; c < 32; c++) {
    const uint64_t C = (uint64_t)expand5(c);
    rdist_[c][0] = plane[0][c][2] + C * C * plane[0][c][0] - 2 * C * plane[0][c][1];
    rdist_[c][1] = plane[0][31][2] + C * C * plane[0][31][0] - 2 * C * plane[0][31][1] - rdist_[c][0];
    bdist_[c][0] = plane[2][c][2] + C * C * plane[2][c][0] - 2 * C * plane[2][c][1];
    bdist_[c][1] = plane[2][31][2] + C * C * plane[2][31][0] - 2 * C * plane[2][31][1] - bdist_[c][0];
  }
  for (int c = 0; c < 64; c++) {
    const uint64_t C = (uint64_t)expand6(c);
    gdist_[c][0] = plane[1][c][2] + C * C * plane[1][c][0] - 2 * C * plane[1][c][1];
    gdist_[c][1] = plane[1][63][2] + C * C * plane[1][63][0] - 2 * C * plane[1][63][1] - gdist_[c][0];
  }
  if (uc_.empty()) {
    // every texel transparent: a 3-colour block of black endpoints, all selectors 3
    out_lo = out_hi = 0;
    std::memset(out_sel, 3, n_px);
    out_err = 0;
    return;
  }
  if (uc_.size() == 1 && !has_transparent) {
    const SingleColourTables& T = sct();
    const int r = uc_[0].r, g = uc_[0].g, b = uc_[0].b;
    evaluate(Coords{(uint16_t)((T.m5[r][0] << 11) | (T.m6[g][0] << 5) | T.m5[b][0]),
                    (uint16_t)((T.m5[r][1] << 11) | (T.m6[g][1] << 5) | T.m5[b][1])});
    if (use_alpha_ && best_.error)
      evaluate(Coords{(uint16_t)((T.m5_3[r][0] << 11) | (T.m6_3[g][0] << 5) | T.m5_3[b][0]),
                      (uint16_t)((T.m5_3[r][1] << 11) | (T.m6_3[g][1] << 5) | T.m5_3[b][1])});
  } else {
    handle_multicolor();
  }
  // return_solution: transparent texels take selector 3
  compute_selectors();
  bool invert = best_.alpha_block ? best_.c.lo > best_.c.hi : best_.c.lo < best_.c.hi;
  static const uint8_t inv_null[4] = {0, 1, 2, 3}, inv_alpha[4] = {1, 0, 2, 3}, inv_colour[4] = {1, 0, 3, 2};
  const uint8_t* inv = invert ? (best_.alpha_block ? inv_alpha : inv_colour) : inv_null;
  out_lo = invert ? best_.c.hi : best_.c.lo;
  out_hi = invert ? best_.c.lo : best_.c.hi;
  for (uint32_t i = 0; i < n_px; i++) out_sel[i] = px_index[i] == kTransparent ? 3 : inv[best_.sel[px_index[i]]];
  out_err = best_.error;
}

template <typename F>
void parallel_for(uint32_t n, int threads, F f) {
  if (threads <= 1 || n < 64) {
    f(0u, n);
    return;
  }
  std::atomic<uint32_t> next(0);
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; t++) {
    pool.emplace_back([&]() {
      for (;;) {
        uint32_t i0 = next.fetch_add(32);
        if (i0 >= n) break;
        f(i0, std::min(n, i0 + 32));
      }
    });
  }
  for (auto& th : pool) th.join();
}

}  // namespace

// Restated DXT5A optimizer lives in crn_oracle_dxt5a.cpp.
namespace crn_oracle_detail {
void dxt5a_block(const uint8_t* px16, int comp, bool both, uint8_t* out8, int quality);
}

extern "C" int oracle_dxt1_blocks(const uint8_t* blocks, uint32_t n, int perceptual, int use_alpha_blocks,
                                  uint8_t* out, uint64_t* err, int threads) {
  sct();
  parallel_for(n, threads, [&](uint32_t i0, uint32_t i1) {
    Dxt1Search s;
    for (uint32_t i = i0; i < i1; i++) {
      uint16_t lo, hi;
      uint8_t sel[16];
      uint64_t e;
      s.run(blocks + (size_t)i * 64, 16, perceptual != 0, use_alpha_blocks != 0, lo, hi, sel, e);
      uint8_t* o = out + (size_t)i * 8;
      o[0] = lo & 0xFF; o[1] = lo >> 8; o[2] = hi & 0xFF; o[3] = hi >> 8;
      for (int y = 0; y < 4; y++)
        o[4 + y] = (uint8_t)(sel[y * 4] | (sel[y * 4 + 1] << 2) | (sel[y * 4 + 2] << 4) | (sel[y * 4 + 3] << 6));
      if (err) err[i] = e;
    }
  });
  return 0;
}

// The DXT1 block encode of dxt_image::set_block_pixels (crn_dxt_image.cpp:1436-1490) with every
// parameter of the block compressor: for DXT1A, pixels_have_alpha is set per block when a texel's
// alpha is below the threshold.
extern "C" int oracle_dxt1_blocks_ex(const uint8_t* blocks, uint32_t n, const oracle_dxt1_opts* o, uint8_t* out,
                                     uint64_t* err, int threads) {
  if (!o || o->quality < 0 || o->quality > 4) return -1;
  sct();
  parallel_for(n, threads, [&](uint32_t i0, uint32_t i1) {
    Dxt1Search s;
    for (uint32_t i = i0; i < i1; i++) {
      const uint8_t* px = blocks + (size_t)i * 64;
      Dxt1Params p;
      p.perceptual = o->perceptual != 0;
      p.use_alpha_blocks = o->use_alpha_blocks != 0;
      p.quality = o->quality;
      p.grayscale = o->grayscale != 0;
      p.transparent_black = o->transparent_black != 0;
      p.alpha_threshold = o->alpha_threshold;
      p.pixels_have_alpha = false;
      if (o->dxt1a)
        for (int k = 0; k < 16; k++) p.pixels_have_alpha |= px[k * 4 + 3] < o->alpha_threshold;
      uint16_t lo, hi;
      uint8_t sel[16];
      uint64_t e;
      s.run(px, 16, p, lo, hi, sel, e);
      uint8_t* ob = out + (size_t)i * 8;
      ob[0] = lo & 0xFF; ob[1] = lo >> 8; ob[2] = hi & 0xFF; ob[3] = hi >> 8;
      for (int y = 0; y < 4; y++)
        ob[4 + y] = (uint8_t)(sel[y * 4] | (sel[y * 4 + 1] << 2) | (sel[y * 4 + 2] << 4) | (sel[y * 4 + 3] << 6));
      if (err) err[i] = e;
    }
  });
  return 0;
}

// Candidate x unique-colour evaluations the reference's Uber DXT1 search makes on n blocks
// (perceptual / 3-colour flags as oracle_dxt1_blocks): the encoder's algorithmic work count.
extern "C" uint64_t oracle_dxt1_count_evaluations(const uint8_t* blocks, uint32_t n, int perceptual,
                                                  int use_alpha_blocks, int threads) {
  sct();
  std::atomic<uint64_t> total(0);
  parallel_for(n, threads, [&](uint32_t i0, uint32_t i1) {
    Dxt1Search s;
    t_evals = 0;
    for (uint32_t i = i0; i < i1; i++) {
      uint16_t lo, hi;
      uint8_t sel[16];
      uint64_t e;
      s.run(blocks + (size_t)i * 64, 16, perceptual != 0, use_alpha_blocks != 0, lo, hi, sel, e);
    }
    total += t_evals;
  });
  return total.load();
}

extern "C" int oracle_encode_blocks(const uint8_t* blocks, uint32_t n, int fmt, int perceptual,
                                    int use_both_block_types, uint8_t* out, int threads) {
  sct();
  int bpb;
  switch (fmt) {
    case 0: bpb = 8; break;
    case 2: case 7: case 8: bpb = 16; break;
    case 9: bpb = 8; break;
    default: return -1;
  }
  parallel_for(n, threads, [&](uint32_t i0, uint32_t i1) {
    Dxt1Search s;
    for (uint32_t i = i0; i < i1; i++) {
      const uint8_t* px = blocks + (size_t)i * 64;
      uint8_t* o = out + (size_t)i * bpb;
      auto colour = [&](uint8_t* dst, bool alpha_blocks) {
        uint16_t lo, hi;
        uint8_t sel[16];
        uint64_t e;
        s.run(px, 16, perceptual != 0, alpha_blocks, lo, hi, sel, e);
        dst[0] = lo & 0xFF; dst[1] = lo >> 8; dst[2] = hi & 0xFF; dst[3] = hi >> 8;
        for (int y = 0; y < 4; y++)
          dst[4 + y] = (uint8_t)(sel[y * 4] | (sel[y * 4 + 1] << 2) | (sel[y * 4 + 2] << 4) | (sel[y * 4 + 3] << 6));
      };
      switch (fmt) {
        case 0: colour(o, use_both_block_types != 0); break;
        case 2:
          crn_oracle_detail::dxt5a_block(px, 3, use_both_block_types != 0, o, 4);
          colour(o + 8, false);
          break;
        case 7:
          crn_oracle_detail::dxt5a_block(px, 0, use_both_block_types != 0, o, 4);
          crn_oracle_detail::dxt5a_block(px, 1, use_both_block_types != 0, o + 8, 4);
          break;
        case 8:
          crn_oracle_detail::dxt5a_block(px, 1, use_both_block_types != 0, o, 4);
          crn_oracle_detail::dxt5a_block(px, 0, use_both_block_types != 0, o + 8, 4);
          break;
        case 9: crn_oracle_detail::dxt5a_block(px, 3, use_both_block_types != 0, o, 4); break;
      }
    }
  });
  return bpb;
}

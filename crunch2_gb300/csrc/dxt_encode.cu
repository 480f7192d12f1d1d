// DXT1 / DXT5A block encoders for sm_103a, bit-exact with crnlib's optimizers at every quality.
//
// DXT1 (dxt1_endpoint_optimizer, crnlib/crn_dxt1.cpp) runs in two phases inside one kernel:
//   phase 1, lane per block: unique colours, perceptual weighting (powf), the double-precision
//     PCA and projection bounds (handle_multicolor_block :1069-1178) and the LBG seeds of
//     try_median4 (:1181-1308). These are scalar, FP64-heavy and tiny, so lanes work on
//     different blocks and GB300's narrow FP64 pipe is amortised over the warp.
//   phase 2, warp per block, lane per candidate: every candidate list of optimize_endpoints
//     (:703-1067) in reference order. The reference accepts a candidate only if its error is
//     strictly lower than the running best, after a plane-table prune evaluated against that
//     running best. Here 32 candidates are evaluated at once and a ballot resolves the exact
//     sequential outcome: the first lane that beats the current best is accepted, then the next
//     lane after it that beats the new best, and so on. Lists whose candidates are built from
//     the running best (lattice neighbours) are regenerated right after each acceptance.
//     The tried-solution hash set of the reference is not needed: a repeated candidate can
//     never be accepted (its error was already compared against an equal or larger best), so
//     repeats are simply evaluated again. Colours are evaluated farthest-from-the-mean first,
//     which makes the batch early-out fire sooner (an error sum is exact in any order).
// Distances are exact integers computed in FP32 with the expanded square
//   w.(x-p)^2 = w.x^2 + (w.p^2 - 2 w.p.x), all terms integers below 2^24.
// This file must be compiled with --fmad=false: the FP32/FP64 parts restate the reference's
// expression order without fused multiply-adds (the only FMAs are the explicit fmaf of exact
// integer terms).
//
// DXT5A (dxt5_endpoint_optimizer, crnlib/crn_dxt5a.cpp:40-262) is warp per block, lane per
// candidate, with the same first-improvement resolution; its probe grid follows the moving
// centre of the reference.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>
#include <cstring>

#include "crngpu_internal.h"

namespace crngpu {

#define FULL_MASK 0xFFFFFFFFu

constexpr int kBlocksPerWarp = 8;
constexpr int kWarpsPerCta = 4;
// CTAs per SM the encoders are compiled for (registers: 65536 / (128 x 8) = 64 per thread; the
// phase-1 PCA spills a little, the candidate loops do not). 8 beat 4, 5 and 6 on GB300.
constexpr int kCtasPerSm = 8;
constexpr uint32_t kInf = 0xFFFFFFFFu;

// ryg single-colour tables (crnlib/crn_ryg_dxt.cpp:58-99): [value][0]=max, [1]=min endpoint
struct SingleColour { uint8_t m5[256][2], m6[256][2], m5_3[256][2], m6_3[256][2]; };
__constant__ SingleColour c_sct;

// probe tables of optimize_endpoints per quality (crnlib/crn_dxt1.cpp:43-53): superfast and fast,
// normal, better, uber; with their sizes and the probe spacing (:716-745)
__constant__ int16_t c_probe[4][15] = {{0, 1, 2, 3},
                                       {0, 1, 3, 5, 7},
                                       {0, 1, 2, 3, 5, 9, 15, 19, 27, 43},
                                       {0, 1, 2, 3, 5, 7, 9, 10, 13, 15, 19, 27, 43, 59, 91}};
__constant__ int c_probe_size[4] = {4, 5, 10, 15};
constexpr uint32_t kQSuperFast = 0, kQFast = 1, kQNormal = 2, kQBetter = 3, kQUber = 4;
__device__ __forceinline__ int probe_table(uint32_t q) { return q <= kQFast ? 0 : (int)q - 1; }

// ------------------------------------------------------------------------------------------
// small helpers

__device__ __forceinline__ int exp5(int v) { return (v << 3) | (v >> 2); }
__device__ __forceinline__ int exp6(int v) { return (v << 2) | (v >> 4); }
__device__ __forceinline__ uint32_t pack565(int r, int g, int b) { return (uint32_t)(b | (g << 5) | (r << 11)); }
__device__ __forceinline__ uint32_t canon_lo(uint32_t lo, uint32_t hi) { return lo < hi ? hi : lo; }
__device__ __forceinline__ uint32_t canon_hi(uint32_t lo, uint32_t hi) { return lo < hi ? lo : hi; }
__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31; }
// exact float (integer value in [0, 2^23)) -> uint via the 2^23 magic constant
__device__ __forceinline__ uint32_t f2u_exact(float v) { return __float_as_uint(__fadd_rn(v, 8388608.0f)) - 0x4B000000u; }


// A DXT1 solution (dxt1_endpoint_optimizer::potential_solution, crn_dxt1.h:272-311) minus its
// selectors, which are recomputed from it when needed.
struct Sol {
  uint32_t lo, hi, err;
  int alpha, alt, enforce, enforced;
};

// Warp-uniform search state.
struct State {
  Sol best, snap;  // snap: the best at the last compute_selectors() (hc path)
  int n, hc, three;
  int only3;    // the block has transparent texels: 3-colour blocks only (first_block_type 1)
  int fast;     // evaluate_solution_fast (below Better quality, no hc)
  int gray;     // grayscale sampling: distances between luma values
  int quality;  // crn_dxt_quality
  int perceptual;
  float wr, wg;
};

// Candidate list kinds consumed by run_list (the reference's candidate loops).
enum : int { LK_TABLE = 0, LK_PAIRS, LK_NEIGH, LK_MOVE2, LK_REFINE, LK_COMB, LK_COMPS };

struct ListDesc {
  int kind, count, dependent, alt, stop_on_accept;
  int side, nh, row;
  int base[3];  // NEIGH/MOVE2: centre; COMPS: unpacked high endpoint
  int e[6];     // REFINE: fitted endpoints (At1 triple, At2 triple)
  // COMPS: per-component error tables and running bounds
  int comp, p0;
  uint32_t packed_lo, e0, best_err;
  uint32_t W[4], WP2[4], WPP[4], rem[4];
};

// Phase 1's hand-off for one block, written by k_dxt1_seeds to global memory and read by the
// search kernel (64 bytes).
struct __align__(16) Seed {
  float f[9];     // axis[3], low[3], high[3]
  uint32_t m[6];  // try_median4 candidates (lo | hi << 16)
  int n;          // unique colour count (-1: the block is not tried)
};
static_assert(sizeof(Seed) == kDxt1SeedBytes, "seed record size");

// Per-warp shared memory of the phase-1 kernel: a lane per block, 32 blocks per warp.
constexpr int kSeedLanes = 32;
struct SeedShared {
  // scratch, transposed [i][lane] so lanes never share a bank
  uint32_t t_col[16][kSeedLanes];
  uint8_t t_w[16][kSeedLanes];
  float t_norm[3][16][kSeedLanes];
  // the warp's 4x4 blocks (RGBA8, 64 bytes each), staged by bulk copies (TMA) that complete on
  // `bar`; the next group's copies are issued once the lanes have read this one
  __align__(16) uint8_t stage[kSeedLanes * 64];
  uint64_t bar;
};

// Per-warp shared state of the search kernel: the block's seed and the phase-2 working set.
struct WarpShared {
  float4 ucf[16];     // r, g, b as floats, X2 = weighted |x|^2
  int ucw[16];        // weights
  // the same colours in evaluation order (farthest from the block's mean first, by weighted
  // distance): an error sum is exact in any order, and this order makes the early-out fire sooner
  float4 ecf[16];
  uint32_t ecw[16], eci[16];
  uint32_t uci[16];   // r | g << 8 | b << 16
  uint2 lbr[32], lbg[64], lbb[32];  // plane lower bounds: .x = low, .y = high
  uint16_t list[64];  // low-endpoint probes / combinatorial endpoints
  uint16_t list2[32]; // high-endpoint probes
  uint32_t cand[64];  // table candidates (lo | hi << 16) / combinatorial scratch colours
  uint2 pq[64];       // run_list's queue of unpruned candidates of a fixed list: (lo | hi << 16, bound)
  State st;
  ListDesc d;
  Seed sd;  // the current block's phase-1 hand-off
};

// kCtasPerSm CTAs of four warps per SM: each CTA's warps + 1 KB reserved within 228 KB
static_assert((sizeof(WarpShared) * kWarpsPerCta + 1024) * kCtasPerSm <= 228 * 1024,
              "DXT1 encoder shared memory per CTA");
constexpr int kSeedCtasPerSm = 4;
static_assert((sizeof(SeedShared) * kWarpsPerCta + 1024) * kSeedCtasPerSm <= 228 * 1024,
              "DXT1 phase-1 shared memory per CTA");

// ------------------------------------------------------------------------------------------
// Phase 1 (one lane = one block).

struct V3f { float x, y, z; };

// intersection::ray_aabb against [0,1]^3 (crn_intersect.h:44-132); true on cSuccess
__device__ bool ray_unit_box(float o[3], const float d[3], float out[3]) {
  int quad[3];
  float cand[3] = {0.f, 0.f, 0.f};
  bool inside = true;
  for (int i = 0; i < 3; i++) {
    if (o[i] < 0.0f) { quad[i] = 1; cand[i] = 0.0f; inside = false; }
    else if (o[i] > 1.0f) { quad[i] = 0; cand[i] = 1.0f; inside = false; }
    else quad[i] = 2;
  }
  if (inside) return false;
  float mt[3];
  for (int i = 0; i < 3; i++) mt[i] = (quad[i] != 2 && d[i] != 0.0f) ? __fdiv_rn(__fsub_rn(cand[i], o[i]), d[i]) : -1.0f;
  int wp = 0;
  for (int i = 1; i < 3; i++) if (mt[wp] < mt[i]) wp = i;
  if (mt[wp] < 0.0f) return false;
  float c[3];
  for (int i = 0; i < 3; i++) {
    if (i != wp) {
      c[i] = __fadd_rn(o[i], __fmul_rn(mt[wp], d[i]));
      if (c[i] < 0.0f || c[i] > 1.0f) return false;
    } else {
      c[i] = cand[i];
    }
  }
  out[0] = c[0]; out[1] = c[1]; out[2] = c[2];
  return true;
}

// fast_random (crnlib/crn_rand.cpp:310-405) with its default seed
struct FastRandom {
  uint32_t jsr = 0xABCD917Au, jcong = 0x17F3DEADu;
  __device__ float frand(float l, float h) {
    jsr ^= (jsr << 17); jsr ^= (jsr >> 13); jsr ^= (jsr << 5);
    jcong = 69069u * jcong + 1234567u;
    const uint32_t r32 = jsr ^ jcong;
    const double t = __dmul_rn((double)r32, 1.0 / 4294967296.0);
    float r = (float)__dadd_rn((double)l, __dmul_rn((double)__fsub_rn(h, l), t));
    return r < l ? l : (r > h ? h : r);
  }
};

// A near-black texel of try_alpha_as_black_optimization (crnlib/crn_dxt1.cpp:2009-2030): every
// colour channel at most 4.
__device__ __forceinline__ bool is_dark(uint32_t c) {
  return (c & 0xFFu) <= 4u && ((c >> 8) & 0xFFu) <= 4u && ((c >> 16) & 0xFFu) <= 4u;
}

// Whether texel c is left out of the search as transparent: DXT1A texels whose alpha is below the
// threshold, and in the transparent-black trial also the near-black texels (whose alpha the trial
// sets to 0).
__device__ __forceinline__ bool is_transparent(uint32_t c, uint32_t opts) {
  if (!(opts & (kD1Dxt1a | kD1BlackTrial))) return false;
  const uint32_t a = ((opts & kD1BlackTrial) && is_dark(c)) ? 0u : (c >> 24);
  return a < ((opts >> kD1ThresholdShift) & 255u);
}

// Runs handle_multicolor_block up to optimize_endpoints' entry, plus try_median4's seeds, for the
// block whose 16 texels are pix (lane `slot` of the warp); the hand-off goes to *out.
template <bool G>
__device__ void phase1_block(SeedShared& S, int slot, const uint32_t (&pix)[16], uint32_t opts,
                             Seed* __restrict__ out) {
  const int L = slot;
  const bool perceptual = (opts & kD1Perceptual) != 0;
  const uint32_t quality = G ? (opts >> kD1QualityShift) & 7u : kQUber;
  int n = 0;
  if (G && (opts & kD1BlackTrial)) {
    // the trial runs for blocks without real transparency whose unique colours (alpha ignored)
    // are neither free of near-black ones nor all near-black (:2005-2019)
    int dark = 0;
    bool has_t = false;
    #pragma unroll 1
    for (int p = 0; p < 16; p++) {
      const uint32_t c = pix[p] & 0xFFFFFFu;
      has_t |= (opts & kD1Dxt1a) && (pix[p] >> 24) < ((opts >> kD1ThresholdShift) & 255u);
      int i = 0;
      for (; i < n; i++) if (S.t_col[i][L] == c) break;
      if (i == n) { S.t_col[n][L] = c; n++; dark += is_dark(c) ? 1 : 0; }
    }
    if (has_t || !dark || dark == n) { out->n = -1; return; }
    n = 0;
  }
  // unique colours of the opaque texels in first-occurrence order (compute_internal :2113-2131)
  int opaque = 0;
  #pragma unroll 1
  for (int p = 0; p < 16; p++) {
    if (G && is_transparent(pix[p], opts)) continue;
    const uint32_t c = pix[p] & 0xFFFFFFu;
    opaque++;
    int i = 0;
    for (; i < n; i++) if (S.t_col[i][L] == c) break;
    if (i == n) { S.t_col[n][L] = c; S.t_w[n][L] = 1; n++; }
    else S.t_w[i][L]++;
  }
  out->n = n;
  // no opaque texel, or one colour and no transparency (compute_internal :2205-2227): no search
  if (n == 0 || (n == 1 && opaque == 16)) return;
  const float total = (float)opaque;  // m_total_unique_color_weight
  // perceptual weights (:1074-1108); powf restated as the correctly rounded float of pow()
  int passes = 1;
  float pw[3] = {1.0f, 1.0f, 1.0f};
  if (perceptual) {
    float red = 0.f, blue = 0.f, avel = 0.f;
    #pragma unroll 1
    for (int i = 0; i < n; i++) {
      const uint32_t c = S.t_col[i][L];
      const int r = c & 255, g = (c >> 8) & 255, b = c >> 16;
      const int l = (r + g + b + 1) / 3;
      const float lf = (float)l;
      const float scale = __fdiv_rn((float)S.t_w[i][L], 1.0f > lf ? 1.0f : lf);
      red = __fadd_rn(red, __fmul_rn(scale, (float)r));
      blue = __fadd_rn(blue, __fmul_rn(scale, (float)b));
      avel = __fadd_rn(avel, lf);
    }
    red = __fdiv_rn(red, total);
    blue = __fdiv_rn(blue, total);
    avel = __fdiv_rn(avel, total);
    const float a16 = __fdiv_rn(__fmul_rn(avel, 16.0f), 255.0f);
    avel = a16 < 1.0f ? a16 : 1.0f;
    const float mx = red > blue ? red : blue;
    float s = __fdiv_rn(__fmul_rn(mx, 1.0f), 3.0f);
    s = s < 0.0f ? 0.0f : (s > 1.0f ? 1.0f : s);
    const float pwr = (float)pow((double)s, 2.75);
    const float p = __fmul_rn(avel, pwr);
    if (!(p >= 1.0f)) {
      passes = 2;
      const float a0[3] = {.212f, .72f, .072f};
      for (int k = 0; k < 3; k++) pw[k] = __fadd_rn(a0[k], __fmul_rn(__fsub_rn(pw[k], a0[k]), p));
    }
  }
  float mean[3], axis[3];
  #pragma unroll 1
  for (int pass = 0; pass < passes; pass++) {
    // compute_vectors :155-189
    float meanw[3] = {0.f, 0.f, 0.f};
    mean[0] = mean[1] = mean[2] = 0.f;
    #pragma unroll 1
    for (int i = 0; i < n; i++) {
      const uint32_t c = S.t_col[i][L];
      const float wf = (float)S.t_w[i][L];
      const float v[3] = {__fdiv_rn((float)(c & 255), 255.0f), __fdiv_rn((float)((c >> 8) & 255), 255.0f),
                          __fdiv_rn((float)(c >> 16), 255.0f)};
      for (int k = 0; k < 3; k++) {
        mean[k] = __fadd_rn(mean[k], __fmul_rn(v[k], wf));
        meanw[k] = __fadd_rn(meanw[k], __fmul_rn(__fmul_rn(pw[k], v[k]), wf));
      }
    }
    const float inv = __fdiv_rn(1.0f, total);
    for (int k = 0; k < 3; k++) { mean[k] = __fmul_rn(mean[k], inv); meanw[k] = __fmul_rn(meanw[k], inv); }
    // compute_pca :192-256 (double accumulation in colour order)
    double cov[6] = {0, 0, 0, 0, 0, 0};
    #pragma unroll 1
    for (int i = 0; i < n; i++) {
      const uint32_t c = S.t_col[i][L];
      const int w = S.t_w[i][L];
      const float v[3] = {__fdiv_rn((float)(c & 255), 255.0f), __fdiv_rn((float)((c >> 8) & 255), 255.0f),
                          __fdiv_rn((float)(c >> 16), 255.0f)};
      float nv[3];
      for (int k = 0; k < 3; k++) {
        nv[k] = __fsub_rn(v[k], mean[k]);
        S.t_norm[k][i][L] = nv[k];
      }
      const float r = __fsub_rn(__fmul_rn(pw[0], v[0]), meanw[0]);
      const float g = __fsub_rn(__fmul_rn(pw[1], v[1]), meanw[1]);
      const float b = __fsub_rn(__fmul_rn(pw[2], v[2]), meanw[2]);
      const float pr[6] = {__fmul_rn(r, r), __fmul_rn(r, g), __fmul_rn(r, b), __fmul_rn(g, g), __fmul_rn(g, b), __fmul_rn(b, b)};
      if (w > 1) {
        for (int k = 0; k < 6; k++) cov[k] = __dadd_rn(cov[k], __dmul_rn((double)pr[k], (double)w));
      } else {
        for (int k = 0; k < 6; k++) cov[k] = __dadd_rn(cov[k], (double)pr[k]);
      }
    }
    double vf[3] = {(double).9f, (double)1.0f, (double).7f};
    #pragma unroll 1
    for (int it = 0; it < 8; it++) {
      double r = __dadd_rn(__dadd_rn(__dmul_rn(vf[0], cov[0]), __dmul_rn(vf[1], cov[1])), __dmul_rn(vf[2], cov[2]));
      double g = __dadd_rn(__dadd_rn(__dmul_rn(vf[0], cov[1]), __dmul_rn(vf[1], cov[3])), __dmul_rn(vf[2], cov[4]));
      double b = __dadd_rn(__dadd_rn(__dmul_rn(vf[0], cov[2]), __dmul_rn(vf[1], cov[4])), __dmul_rn(vf[2], cov[5]));
      double m = fabs(r);
      if (fabs(g) > m) m = fabs(g);
      if (fabs(b) > m) m = fabs(b);
      if (m > 1e-10) {
        m = __drcp_rn(m);  // 1.0 / m, correctly rounded
        r = __dmul_rn(r, m); g = __dmul_rn(g, m); b = __dmul_rn(b, m);
      }
      const double d0 = __dsub_rn(vf[0], r), d1 = __dsub_rn(vf[1], g), d2 = __dsub_rn(vf[2], b);
      const double delta = __dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)), __dmul_rn(d2, d2));
      vf[0] = r; vf[1] = g; vf[2] = b;
      if (it > 2 && delta < 1e-8) break;
    }
    const double len = __dadd_rn(__dadd_rn(__dmul_rn(vf[0], vf[0]), __dmul_rn(vf[1], vf[1])), __dmul_rn(vf[2], vf[2]));
    if (len < 1e-10) {
      axis[0] = .2837149f; axis[1] = 0.9540631f; axis[2] = 0.096277453f;
    } else {
      const double il = __ddiv_rn(1.0, __dsqrt_rn(len));
      axis[0] = (float)__dmul_rn(vf[0], il); axis[1] = (float)__dmul_rn(vf[1], il); axis[2] = (float)__dmul_rn(vf[2], il);
    }
    for (int k = 0; k < 3; k++) axis[k] = __fdiv_rn(axis[k], pw[k]);
    // vec::normalize (crn_vec.h:674-690): float squares accumulated in double
    double nn = (double)__fmul_rn(axis[0], axis[0]);
    nn = __dadd_rn(nn, (double)__fmul_rn(axis[1], axis[1]));
    nn = __dadd_rn(nn, (double)__fmul_rn(axis[2], axis[2]));
    if (nn != 0.0) {
      const float sc = (float)__ddiv_rn(1.0, __dsqrt_rn(nn));
      for (int k = 0; k < 3; k++) axis[k] = __fmul_rn(axis[k], sc);
    }
    if (passes > 1) {
      if (fabsf(axis[0]) >= .795f) { pw[0] = .424f; pw[1] = .6f; pw[2] = .072f; }
      else if (fabsf(axis[2]) >= .795f) { pw[0] = .212f; pw[1] = .6f; pw[2] = .212f; }
      else break;
    }
  }
  // projection bounds on the axis, then pull outside endpoints back into the unit cube
  float lo_d = 1e+9f, hi_d = -1e+9f;
  #pragma unroll 1
  for (int i = 0; i < n; i++) {
    float d = __fmul_rn(S.t_norm[0][i][L], axis[0]);
    d = __fadd_rn(d, __fmul_rn(S.t_norm[1][i][L], axis[1]));
    d = __fadd_rn(d, __fmul_rn(S.t_norm[2][i][L], axis[2]));
    lo_d = d < lo_d ? d : lo_d;
    hi_d = d > hi_d ? d : hi_d;
  }
  float low[3], high[3];
  for (int k = 0; k < 3; k++) {
    low[k] = __fadd_rn(mean[k], __fmul_rn(lo_d, axis[k]));
    high[k] = __fadd_rn(mean[k], __fmul_rn(hi_d, axis[k]));
  }
  auto within = [](const float* v) {
    for (int i = 0; i < 3; i++) if (v[i] < 0.0f || v[i] > 1.0f) return false;
    return true;
  };
  if (!within(low)) {
    float c[3];
    if (ray_unit_box(low, axis, c)) { low[0] = c[0]; low[1] = c[1]; low[2] = c[2]; }
  }
  if (!within(high)) {
    float c[3];
    const float nd[3] = {-axis[0], -axis[1], -axis[2]};
    if (ray_unit_box(high, nd, c)) { high[0] = c[0]; high[1] = c[1]; high[2] = c[2]; }
  }
  for (int k = 0; k < 3; k++) {
    out->f[k] = axis[k];
    out->f[3 + k] = low[k];
    out->f[6 + k] = high[k];
  }
  // try_median4 seeds (:1181-1308), tried at Better and Uber only (:765-771)
  if (quality < kQBetter) return;
  float means[4][3];
  if (n <= 4) {
    for (int i = 0; i < 4; i++) {
      const int src = i < n - 1 ? i : n - 1;
      for (int k = 0; k < 3; k++) means[i][k] = S.t_norm[k][src][L];
    }
  } else {
    for (int k = 0; k < 3; k++) {
      means[0][k] = __fsub_rn(low[k], mean[k]);
      means[3][k] = __fsub_rn(high[k], mean[k]);
    }
    for (int k = 0; k < 3; k++) {
      means[1][k] = __fadd_rn(means[0][k], __fmul_rn(__fsub_rn(means[3][k], means[0][k]), 1.0f / 3.0f));
      means[2][k] = __fadd_rn(means[0][k], __fmul_rn(__fsub_rn(means[3][k], means[0][k]), 2.0f / 3.0f));
    }
    FastRandom rm;
    unsigned rover = 0;
    float prev_total = 1.0e+37f;
    #pragma unroll 1
    for (int it = 0; it < 8; it++) {
      float nm[4][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
      float nw[4] = {0.f, 0.f, 0.f, 0.f};
      float tot = 0.f;
      #pragma unroll 1
      for (int i = 0; i < n; i++) {
        const float v[3] = {S.t_norm[0][i][L], S.t_norm[1][i][L], S.t_norm[2][i][L]};
        float bd = 0.f;
        int bi = 0;
        for (int j = 0; j < 4; j++) {
          float d2 = 0.f;
          for (int k = 0; k < 3; k++) {
            const float d = __fsub_rn(means[j][k], v[k]);
            d2 = __fadd_rn(d2, __fmul_rn(d, d));
          }
          if (j == 0 || d2 < bd) { bd = d2; bi = j; }
        }
        tot = __fadd_rn(tot, bd);
        const float wf = (float)S.t_w[i][L];
        for (int k = 0; k < 3; k++) nm[bi][k] = __fadd_rn(nm[bi][k], __fmul_rn(v[k], wf));
        nw[bi] = __fadd_rn(nw[bi], wf);
      }
      unsigned hi_idx = 0;
      float hi_w = 0.f;
      bool empty = false;
      for (int j = 0; j < 4; j++) {
        if (nw[j] > 0.0f) {
          for (int k = 0; k < 3; k++) means[j][k] = __fdiv_rn(nm[j][k], nw[j]);
          if (nw[j] > hi_w) { hi_w = nw[j]; hi_idx = j; }
        } else {
          empty = true;
        }
      }
      if (!empty) {
        if (fabsf(__fsub_rn(tot, prev_total)) < .00001f) break;
        prev_total = tot;
      } else {
        prev_total = 1.0e+37f;
      }
      if (empty && it != 7) {
        const unsigned ri = (hi_idx + rover) & 3;
        rover++;
        for (int j = 0; j < 4; j++) {
          if (nw[j] == 0.0f) {
            for (int k = 0; k < 3; k++) means[j][k] = means[ri][k];
            for (int k = 0; k < 3; k++) means[j][k] = __fadd_rn(means[j][k], rm.frand(-.00196f, .00196f));
          }
        }
      }
    }
  }
  int slot_i = 0;
  #pragma unroll 1
  for (int i = 0; i < 3; i++) {
    for (int j = i + 1; j < 4; j++) {
      int q[2][3];
      for (int k = 0; k < 3; k++) {
        const float sc = k == 1 ? 63.0f : 31.0f;
        q[0][k] = (int)floorf(__fadd_rn(.5f, __fmul_rn(__fadd_rn(means[i][k], mean[k]), sc)));
        q[1][k] = (int)floorf(__fadd_rn(.5f, __fmul_rn(__fadd_rn(means[j][k], mean[k]), sc)));
      }
      uint32_t pk[2];
      for (int e = 0; e < 2; e++) {
        // color_quad_u8 clamps to 0..255, pack_color(scaled=false) then clamps to 31/63/31
        const int r = min(clampi(q[e][0], 0, 255), 31), g = min(clampi(q[e][1], 0, 255), 63),
                  b = min(clampi(q[e][2], 0, 255), 31);
        pk[e] = pack565(r, g, b);
      }
      out->m[slot_i++] = canon_lo(pk[0], pk[1]) | (canon_hi(pk[0], pk[1]) << 16);
    }
  }
}

// ------------------------------------------------------------------------------------------
// Phase 2 (one warp = one block). All search state that is uniform across the warp (running
// best, list descriptor, candidate tables) lives in the warp's shared memory, and a single
// non-inlined list runner holds the one copy of the candidate evaluation loop; the list setups
// (refine, solid, per-component, combinatorial) are non-inlined too. The kernel is bound by
// instruction fetch (the largest stall reason), so the code a block's search runs through is kept
// small: one instance of each routine.

__device__ __forceinline__ uint32_t lower_bound(const WarpShared& S, uint32_t lo, uint32_t hi) {
  // evaluate_solution's plane-table prune (crn_dxt1.cpp:1312-1322)
  const int r0 = lo >> 11, g0 = (lo >> 5) & 63, b0 = lo & 31;
  const int r1 = hi >> 11, g1 = (hi >> 5) & 63, b1 = hi & 31;
  const uint32_t re = r0 < r1 ? S.lbr[r0].x + S.lbr[r1].y : S.lbr[r0].y + S.lbr[r1].x;
  const uint32_t ge = g0 < g1 ? S.lbg[g0].x + S.lbg[g1].y : S.lbg[g0].y + S.lbg[g1].x;
  const uint32_t be = b0 < b1 ? S.lbb[b0].x + S.lbb[b1].y : S.lbb[b0].y + S.lbb[b1].x;
  return re + ge + be;
}

// Palette entry -> (q = 2 w p, P2 = w.p^2) for the expanded-square distance.
__device__ __forceinline__ float4 entry(float wr, float wg, int r, int g, int b) {
  const float fr = (float)r, fg = (float)g, fb = (float)b;
  return make_float4(2.f * wr * fr, 2.f * wg * fg, 2.f * fb, wr * fr * fr + wg * fg * fg + fb * fb);
}

// color::RGB_to_Y (crnlib/crn_color.h:792-796): fixed-point luma
__device__ __forceinline__ int luma(int r, int g, int b) { return (r * 19595 + g * 38470 + b * 7471 + 32768) >> 16; }

// The same for the grayscale-sampling metric (crnlib/crn_dxt1.cpp:1342-1368): the squared luma
// difference, with the colour held as (Y, 0, 0, Y^2).
__device__ __forceinline__ float4 entry_m(bool gray, float wr, float wg, int r, int g, int b) {
  if (!gray) return entry(wr, wg, r, g, b);
  const float y = (float)luma(r, g, b);
  return make_float4(2.f * y, 0.f, 0.f, y * y);
}
__device__ __forceinline__ float dist_part(const float4& x, const float4& q) {
  float t = fmaf(-x.x, q.x, q.w);
  t = fmaf(-x.y, q.y, t);
  return fmaf(-x.z, q.z, t);
}

// Selector of unique colour i for solution s; ties go to the lowest index, which is how both
// the uber trial loop and compute_selectors_hc (crn_dxt1.cpp:1845-1869) resolve them.
// The selector evaluate_solution_fast (crnlib/crn_dxt1.cpp:1594-1757) gives colour c: its
// projection onto the endpoint axis against the midpoints of the palette's projections.
struct FastSel {
  int dr, dg, db;     // 2 x the (weighted) axis
  int t0, t1, t2;     // 4-colour: halfPoint, c0Point, c3Point; 3-colour: c02Point, c21Point
  bool three;
  __device__ void init(bool perceptual, bool alpha, int a, int r0, int g0, int b0, int r1, int g1, int b1) {
    int vr = r1 - r0, vg = g1 - g0, vb = b1 - b0;
    if (perceptual) { vr *= 8; vg *= 24; }
    const int s0 = r0 * vr + g0 * vg + b0 * vb, s1 = r1 * vr + g1 * vg + b1 * vb;
    dr = vr * 2; dg = vg * 2; db = vb * 2;
    three = alpha;
    if (!alpha) {
      const int s2 = ((r0 * 2 + r1 + a) / 3) * vr + ((g0 * 2 + g1 + a) / 3) * vg + ((b0 * 2 + b1 + a) / 3) * vb;
      const int s3 = ((r1 * 2 + r0 + a) / 3) * vr + ((g1 * 2 + g0 + a) / 3) * vg + ((b1 * 2 + b0 + a) / 3) * vb;
      t0 = s3 + s2; t1 = s1 + s3; t2 = s2 + s0;
    } else {
      const int s2 = ((r0 + r1 + a) >> 1) * vr + ((g0 + g1 + a) >> 1) * vg + ((b0 + b1 + a) >> 1) * vb;
      t0 = s0 + s2; t1 = s2 + s1;
    }
  }
  __device__ __forceinline__ int pick(uint32_t c) const {
    const int d = (int)(c & 255) * dr + (int)((c >> 8) & 255) * dg + (int)(c >> 16) * db;
    if (!three) return d >= t0 ? (d < t1 ? 3 : 1) : (d < t2 ? 0 : 2);
    return d < t0 ? 0 : (d < t1 ? 2 : 1);
  }
};

template <bool G>
__device__ __noinline__ int selector_of(const WarpShared& S, int i, const Sol& s) {
  if (s.enforce) return s.enforced;
  const float wr = S.st.wr, wg = S.st.wg;
  const bool gray = G && S.st.gray != 0;
  const int r0 = exp5(s.lo >> 11), g0 = exp6((s.lo >> 5) & 63), b0 = exp5(s.lo & 31);
  const int r1 = exp5(s.hi >> 11), g1 = exp6((s.hi >> 5) & 63), b1 = exp5(s.hi & 31);
  const int a = s.alt;
  if (G && S.st.fast) {
    FastSel f;
    f.init(S.st.perceptual != 0, s.alpha != 0, a, r0, g0, b0, r1, g1, b1);
    return f.pick(S.uci[i]);
  }
  float4 q[4];
  q[0] = entry_m(gray, wr, wg, r0, g0, b0);
  q[1] = entry_m(gray, wr, wg, r1, g1, b1);
  if (s.alpha) {
    q[2] = entry_m(gray, wr, wg, (r0 + r1 + a) >> 1, (g0 + g1 + a) >> 1, (b0 + b1 + a) >> 1);
  } else {
    q[2] = entry_m(gray, wr, wg, (r0 * 2 + r1 + a) / 3, (g0 * 2 + g1 + a) / 3, (b0 * 2 + b1 + a) / 3);
    q[3] = entry_m(gray, wr, wg, (r1 * 2 + r0 + a) / 3, (g1 * 2 + g0 + a) / 3, (b1 * 2 + b0 + a) / 3);
  }
  const float4 x = S.ucf[i];
  float bd = dist_part(x, q[0]);
  int bi = 0;
  const int nk = s.alpha ? 3 : 4;
  for (int k = 1; k < nk; k++) {
    const float d = dist_part(x, q[k]);
    if (d < bd) { bd = d; bi = k; }
  }
  return bi;
}

// The selectors m_best_solution.m_selectors holds right now: the best itself on the uber path,
// the best at the last compute_selectors() call on the hc path (selectors are lazy there).
__device__ __forceinline__ const Sol& sel_source(const WarpShared& S) { return S.st.hc ? S.st.snap : S.st.best; }
__device__ __forceinline__ void compute_selectors(WarpShared& S) {
  if (S.st.hc && lane_id() == 0) S.st.snap = S.st.best;
  __syncwarp();
}

__device__ __forceinline__ void accept(WarpShared& S, uint32_t lo, uint32_t hi, uint32_t err, int type, int alt) {
  if (lane_id() == 0) {
    Sol& b = S.st.best;
    b.lo = lo; b.hi = hi; b.err = err; b.alpha = type; b.alt = alt;
    b.enforce = (!type && lo == hi) ? 1 : 0;
    if (b.enforce) {
      if ((b.lo & 31) != 31) { b.lo++; b.enforced = 1; }
      else { b.hi--; b.enforced = 0; }
    }
  }
  __syncwarp();
}

// Candidate i of the current list (descriptor in S.d); false when the reference skips it.
__device__ __forceinline__ bool gen_candidate(const WarpShared& S, const ListDesc& d, int i, uint32_t& lo, uint32_t& hi) {
  switch (d.kind) {
    case LK_TABLE: {
      const uint32_t v = S.cand[i];
      lo = v & 0xFFFFu; hi = v >> 16;
      return true;
    }
    case LK_PAIRS: {
      // i / nh through a float reciprocal: exact for i < 2^10, nh <= 31 (the fraction of
      // (i + 0.5) / nh is at least 1 / 62 away from an integer)
      const int a = __float2int_rz(__fmul_rn(__fadd_rn((float)i, 0.5f), __frcp_rn((float)d.nh))), b = i - a * d.nh;
      const uint32_t p0 = S.list[a], p1 = S.list2[b];
      lo = canon_lo(p0, p1); hi = canon_hi(p0, p1);
      return true;
    }
    case LK_NEIGH:
    case LK_MOVE2: {
      int c[3] = {d.base[0], d.base[1], d.base[2]};
      if (d.kind == LK_NEIGH) {
        // g_adjacency order (crn_dxt1.cpp:489-522): x fastest, then y, then z, centre skipped
        const int idx = i < 13 ? i : i + 1;
        c[0] += idx % 3 - 1; c[1] += (idx / 3) % 3 - 1; c[2] += idx / 9 - 1;
        if (c[0] < 0 || c[0] > 31 || c[1] < 0 || c[1] > 63 || c[2] < 0 || c[2] > 31) return false;
      } else {
        const int a = i >> 1;
        c[a] += (i & 1) ? 2 : -2;
        if (c[a] < 0 || c[a] > (a == 1 ? 63 : 31)) return false;
      }
      const uint32_t moved = pack565(c[0], c[1], c[2]);
      const uint32_t p0 = d.side ? S.st.best.lo : moved, p1 = d.side ? moved : S.st.best.hi;
      lo = canon_lo(p0, p1); hi = canon_hi(p0, p1);
      return true;
    }
    case LK_REFINE: {
      const int which = i / 27, rr = (i / 9) % 3 - 1, gr = (i / 3) % 3 - 1, br = i % 3 - 1;
      int c[6] = {d.e[0], d.e[1], d.e[2], d.e[3], d.e[4], d.e[5]};
      const int o = which * 3;
      c[o] = clampi(c[o] + rr, 0, 31);
      c[o + 1] = clampi(c[o + 1] + gr, 0, 63);
      c[o + 2] = clampi(c[o + 2] + br, 0, 31);
      const uint32_t p0 = pack565(c[0], c[1], c[2]), p1 = pack565(c[3], c[4], c[5]);
      lo = canon_lo(p0, p1); hi = canon_hi(p0, p1);
      return true;
    }
    case LK_COMB:
      lo = S.list[d.row];
      hi = S.list[d.row + 1 + i];
      return true;
    default: {  // LK_COMPS: optimize_endpoint_comps inner loop with its table prune (:440-470)
      const int c1 = i;
      const uint32_t p1 = (uint32_t)(d.comp == 1 ? exp6(c1) : exp5(c1));
      const uint32_t p0 = (uint32_t)d.p0;
      auto E = [&](int s, uint32_t p) { return d.W[s] * p * p - d.WP2[s] * p + d.WPP[s]; };
      uint32_t e = d.e0 + E(1, p1);
      if (e + d.rem[2] >= d.best_err) return false;
      e += E(2, (p0 * 2 + p1) / 3);
      if (e + d.rem[3] >= d.best_err) return false;
      e += E(3, (p0 + p1 * 2) / 3);
      if (e >= d.best_err) return false;
      int h[3] = {d.base[0], d.base[1], d.base[2]};
      h[d.comp] = c1;
      lo = d.packed_lo;
      hi = pack565(h[0], h[1], h[2]);
      return true;
    }
  }
}

// Runs the list described by S.d from position `start` with the reference's sequential
// semantics; see the file comment. Returns, for stop_on_accept lists, the position of the
// first accepted candidate (or -1); otherwise 1 if anything was accepted, else 0.
template <bool G>
__device__ __noinline__ int run_list(WarpShared& S, int start, uint32_t& work) {
  const ListDesc& d = S.d;
  const uint32_t lane = lane_id();
  const int n = S.st.n;
  const bool three = S.st.three != 0, only3 = G && S.st.only3 != 0, fast = G && S.st.fast != 0;
  const bool gray = G && S.st.gray != 0;
  const float wr = S.st.wr, wg = S.st.wg;
  bool any = false;
  int i0 = start;
  // Lists whose candidates do not depend on the running best are compacted: the candidates that
  // survive the plane-table prune (against the best when they are generated) queue up in list order
  // in S.pq, and each batch evaluates 32 of them, so the colour loop runs on full warps. The prune
  // is repeated against the best at the start of the batch; acceptances follow list order, as in
  // the sparse form. Lists regenerated after each acceptance run sparse, 32 positions at a time.
  const bool compact = !d.dependent;
  int qn = 0;  // queued candidates (compact lists)
  // No tried-solution set (m_solutions_tried, crn_dxt1.cpp:1323-1330): a candidate evaluated
  // before had an error at or above the best of that time, and the best only falls, so evaluating
  // it again cannot accept it. The current best itself (once there is one; same palette rounding,
  // endpoints not bumped apart by the equal-endpoint rule) is skipped, as its error would only
  // reach the best at its last colour.
  auto not_best = [&](uint32_t lo, uint32_t hi) {
    const Sol& b = S.st.best;
    return d.alt || b.err == kInf || b.alt || b.enforce || (lo | (hi << 16)) != (b.lo | (b.hi << 16));
  };
  for (;;) {
    uint32_t lo = 0, hi = 0, lb = kInf;
    bool live;
    int take = 32;
    const uint32_t B0 = S.st.best.err;
    if (compact) {
      while (qn < 32 && i0 < d.count) {
        const int i = i0 + (int)lane;
        uint32_t clo = 0, chi = 0;
        const bool valid = i < d.count && gen_candidate(S, d, i, clo, chi);
        const uint32_t clb = valid ? lower_bound(S, clo, chi) : kInf;
        const bool keep = valid && clb < S.st.best.err && not_best(clo, chi);
        const unsigned m = __ballot_sync(FULL_MASK, keep);
        if (keep) S.pq[qn + __popc(m & ((1u << lane) - 1u))] = make_uint2(clo | (chi << 16), clb);
        qn += __popc(m);
        i0 += 32;
      }
      __syncwarp();
      if (!qn) break;
      take = min(qn, 32);
      if ((int)lane < take) {
        const uint2 v = S.pq[lane];
        lo = v.x & 0xFFFFu; hi = v.x >> 16; lb = v.y;
      }
      live = (int)lane < take && lb < B0;
    } else {
      if (i0 >= d.count) break;
      const int i = i0 + (int)lane;
      const bool valid = i < d.count && gen_candidate(S, d, i, lo, hi);
      lb = valid ? lower_bound(S, lo, hi) : kInf;
      live = valid && lb < B0 && not_best(lo, hi);
    }
    if (!__any_sync(FULL_MASK, live)) {  // the whole batch is pruned: nothing to evaluate
      if (compact) {
        const int rest = qn - take;
        const uint2 v = (int)lane < rest ? S.pq[take + lane] : make_uint2(0u, 0u);
        __syncwarp();
        if ((int)lane < rest) S.pq[lane] = v;
        __syncwarp();
        qn = rest;
      } else {
        i0 += 32;
      }
      continue;
    }
    // evaluate every lane's candidate (uber: 4- and 3-colour; hc: 4-colour; fast: the selector
    // by projection, then its distance), stopping early once no live lane can still beat the
    // running best. Blocks with transparent texels evaluate 3-colour blocks only.
    uint32_t e0 = 0, e1 = 0;
    {
      const int a = d.alt;
      const int r0 = exp5(lo >> 11), g0 = exp6((lo >> 5) & 63), b0 = exp5(lo & 31);
      const int r1 = exp5(hi >> 11), g1 = exp6((hi >> 5) & 63), b1 = exp5(hi & 31);
      const float4 q0 = entry_m(gray, wr, wg, r0, g0, b0), q1 = entry_m(gray, wr, wg, r1, g1, b1);
      const float4 q2 = entry_m(gray, wr, wg, (r0 * 2 + r1 + a) / 3, (g0 * 2 + g1 + a) / 3, (b0 * 2 + b1 + a) / 3);
      const float4 q3 = entry_m(gray, wr, wg, (r1 * 2 + r0 + a) / 3, (g1 * 2 + g0 + a) / 3, (b1 * 2 + b0 + a) / 3);
      const float4 q4 = entry_m(gray, wr, wg, (r0 + r1 + a) >> 1, (g0 + g1 + a) >> 1, (b0 + b1 + a) >> 1);
      if (__any_sync(FULL_MASK, live)) {
        int k = 0;
        if (!fast) {
          for (; k < n; k++) {
            const float4 x = S.ecf[k];
            const uint32_t w = S.ecw[k];
            const float m01 = fminf(dist_part(x, q0), dist_part(x, q1));
            e0 += w * f2u_exact(__fadd_rn(x.w, fminf(m01, fminf(dist_part(x, q2), dist_part(x, q3)))));
            if (three) e1 += w * f2u_exact(__fadd_rn(x.w, fminf(m01, dist_part(x, q4))));
            if ((k & 1) == 1 &&
                __all_sync(FULL_MASK, !live || (only3 ? e1 : (three ? min(e0, e1) : e0)) >= B0)) { k++; break; }
          }
        } else {
          FastSel f4, f3;
          const bool perc = S.st.perceptual != 0;
          f4.init(perc, false, a, r0, g0, b0, r1, g1, b1);
          f3.init(perc, true, a, r0, g0, b0, r1, g1, b1);
          for (; k < n; k++) {
            const float4 x = S.ecf[k];
            const uint32_t c = S.eci[k];
            const uint32_t w = S.ecw[k];
            if (!only3) {
              const int s4 = f4.pick(c);
              const float4 q = s4 == 0 ? q0 : s4 == 1 ? q1 : s4 == 2 ? q2 : q3;
              e0 += w * f2u_exact(__fadd_rn(x.w, dist_part(x, q)));
            }
            if (three) {
              const int s3 = f3.pick(c);
              const float4 q = s3 == 0 ? q0 : s3 == 1 ? q1 : q4;
              e1 += w * f2u_exact(__fadd_rn(x.w, dist_part(x, q)));
            }
            if ((k & 3) == 3 &&
                __all_sync(FULL_MASK, !live || (only3 ? e1 : (three ? min(e0, e1) : e0)) >= B0)) { k++; break; }
          }
        }
        if (live) work += (uint32_t)k;
      }
    }
    const bool pick3 = only3 || (three && e1 < e0);
    const uint32_t err = pick3 ? e1 : e0;
    const int type = pick3 ? 1 : 0;
    // resolve the sequential outcome of the batch
    unsigned ok = __ballot_sync(FULL_MASK, live && err < B0);
    int last = -1;
    while (ok) {
      const int j = __ffs(ok) - 1;
      accept(S, __shfl_sync(FULL_MASK, lo, j), __shfl_sync(FULL_MASK, hi, j), __shfl_sync(FULL_MASK, err, j),
             __shfl_sync(FULL_MASK, type, j), d.alt);
      any = true;
      last = j;
      if (d.dependent) break;
      const uint32_t B = S.st.best.err;
      const unsigned after = j == 31 ? 0u : (FULL_MASK << (j + 1));
      ok = __ballot_sync(FULL_MASK, live && lb < B && err < B) & after;
    }
    __syncwarp();
    if (compact) {
      const int rest = qn - take;
      const uint2 v = (int)lane < rest ? S.pq[take + lane] : make_uint2(0u, 0u);
      __syncwarp();
      if ((int)lane < rest) S.pq[lane] = v;
      __syncwarp();
      qn = rest;
    } else if (last >= 0) {
      if (d.stop_on_accept) return i0 + last;
      i0 += last + 1;
    } else {
      i0 += 32;
    }
  }
  return d.stop_on_accept ? -1 : (any ? 1 : 0);
}

__device__ __forceinline__ void set_list(WarpShared& S, int kind, int count, int dependent, int alt) {
  if (lane_id() == 0) {
    S.d.kind = kind; S.d.count = count; S.d.dependent = dependent; S.d.alt = alt; S.d.stop_on_accept = 0;
  }
}

// refine_solution :525-698: least-squares endpoints from the current selectors; level 1 then tries
// the 2 x 27 lattice neighbours of the two fitted endpoints, level 0 the fitted pair alone.
template <bool G>
__device__ __noinline__ bool refine(WarpShared& S, uint32_t& work, int level = 1) {
  compute_selectors(S);
  const uint32_t lane = lane_id();
  const int n = S.st.n;
  int a[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // ak0 ak1 ak2 at1r at1g at1b at2r at2g at2b
  if ((int)lane < n) {
    const int step = selector_of<G>(S, lane, sel_source(S)) ^ 1;
    const int w = S.ucw[lane];
    const uint32_t c = S.uci[lane];
    const int r = (c & 255) * w, g = ((c >> 8) & 255) * w, b = (c >> 16) * w;
    const int w1 = step == 0 ? 3 : step == 1 ? 0 : step == 2 ? 2 : 1;
    const int p0 = step >= 2 ? 2 : 0;
    const int p1 = step == 0 ? 0 : step == 1 ? 9 : step == 2 ? 1 : 4;
    const int p2 = step == 0 ? 9 : step == 1 ? 0 : step == 2 ? 4 : 1;
    a[0] = p0 * w; a[1] = p1 * w; a[2] = p2 * w;
    a[3] = w1 * r; a[4] = w1 * g; a[5] = w1 * b;
    a[6] = r; a[7] = g; a[8] = b;
  }
  for (int k = 0; k < 9; k++) a[k] = __reduce_add_sync(FULL_MASK, a[k]);
  const long long xx = a[2], yy = a[1], xy = a[0];
  const long long t = xx * yy - xy * xy;
  if (!yy || !xx || t == 0) return false;
  int comp = 0;
  if (lane < 6) {  // the six fitted components, one per lane, in double exactly as the reference
    const int k = lane % 3;
    const long long at1 = a[3 + k], at2 = 3LL * a[6 + k] - a[3 + k];
    const double frb = __ddiv_rn((double)__fdiv_rn(93.0f, 255.0f), (double)t);
    const double f = k == 1 ? __dmul_rn(frb, (double)__fdiv_rn(63.0f, 31.0f)) : frb;
    const long long num = lane < 3 ? at1 * yy - at2 * xy : at2 * xx - at1 * xy;
    const double v = __dadd_rn(__dmul_rn((double)num, f), (double)0.5f);
    comp = clampi(__double2int_rz(v), 0, k == 1 ? 63 : 31);
  }
  const int mine = comp;
  for (int k = 0; k < 6; k++) {
    const int v = __shfl_sync(FULL_MASK, mine, k);
    if (lane == 0) S.d.e[k] = v;
  }
  __syncwarp();
  if (level == 0) {
    if (lane == 0) {
      const uint32_t p0 = pack565(S.d.e[0], S.d.e[1], S.d.e[2]), p1 = pack565(S.d.e[3], S.d.e[4], S.d.e[5]);
      S.cand[0] = canon_lo(p0, p1) | (canon_hi(p0, p1) << 16);
    }
    set_list(S, LK_TABLE, 1, 0, 0);
  } else {
    set_list(S, LK_REFINE, 54, 0, 0);
  }
  __syncwarp();
  return run_list<G>(S, 0, work) != 0;
}

template <bool G>
__device__ __noinline__ bool all_selectors_equal(const WarpShared& S) {
  const uint32_t lane = lane_id();
  const int n = S.st.n;
  const int mine = (int)lane < n ? selector_of<G>(S, lane, sel_source(S)) : -1;
  const int first = __shfl_sync(FULL_MASK, mine, 0);
  return __all_sync(FULL_MASK, (int)lane >= n || mine == first);
}

__device__ __forceinline__ uint32_t solid_coords(int r, int g, int b, bool three) {
  const uint32_t lo = three ? pack565(c_sct.m5_3[r][0], c_sct.m6_3[g][0], c_sct.m5_3[b][0])
                            : pack565(c_sct.m5[r][0], c_sct.m6[g][0], c_sct.m5[b][0]);
  const uint32_t hi = three ? pack565(c_sct.m5_3[r][1], c_sct.m6_3[g][1], c_sct.m5_3[b][1])
                            : pack565(c_sct.m5[r][1], c_sct.m6[g][1], c_sct.m5[b][1]);
  return lo | (hi << 16);
}

// try_average_block_as_solid :93-153
template <bool G>
__device__ __noinline__ bool try_solid(WarpShared& S, uint32_t& work) {
  const uint32_t lane = lane_id();
  const int n = S.st.n;
  int tr = 0, tg = 0, tb = 0;
  if ((int)lane < n) {
    const uint32_t c = S.uci[lane];
    const int w = S.ucw[lane];
    tr = (c & 255) * w; tg = ((c >> 8) & 255) * w; tb = (c >> 16) * w;
  }
  tr = __reduce_add_sync(FULL_MASK, tr);
  tg = __reduce_add_sync(FULL_MASK, tg);
  tb = __reduce_add_sync(FULL_MASK, tb);
  const int ar = (tr + 8) / 16, ag = (tg + 8) / 16, ab = (tb + 8) / 16;
  const bool three = S.st.three != 0;
  if (lane == 0) {
    int cnt = 0;
    S.cand[cnt++] = solid_coords(ar, ag, ab, false);
    if (three) S.cand[cnt++] = solid_coords(ar, ag, ab, true);
    // the other colours of the block as solid colours, at Uber only (:126-150)
    #pragma unroll 1
    for (int i = 0; i < ((!G || S.st.quality == (int)kQUber) ? n : 0); i++) {
      const uint32_t c = S.uci[i];
      const int r = c & 255, g = (c >> 8) & 255, b = c >> 16;
      if (r == ar && g == ag && b == ab) continue;
      S.cand[cnt++] = solid_coords(r, g, b, false);
      if (three) S.cand[cnt++] = solid_coords(r, g, b, true);
    }
    S.d.count = cnt;
  }
  __syncwarp();
  set_list(S, LK_TABLE, S.d.count, 0, 0);
  __syncwarp();
  return run_list<G>(S, 0, work) != 0;
}

// compute_endpoint_component_errors :369-413 as closed-form quadratics; fills S.d.W/WP2/WPP/rem
template <bool G>
__device__ __noinline__ void comp_errors(WarpShared& S, int comp) {
  const uint32_t lane = lane_id();
  const int n = S.st.n;
  int sel = -1;
  uint32_t p = 0, w = 0;
  if ((int)lane < n) {
    sel = selector_of<G>(S, lane, sel_source(S));
    p = (S.uci[lane] >> (8 * comp)) & 255;
    w = (uint32_t)S.ucw[lane];
  }
  uint32_t W[4], WP2[4], WPP[4], rem[4];
  for (int k = 0; k < 4; k++) {
    W[k] = __reduce_add_sync(FULL_MASK, sel == k ? w : 0u);
    WP2[k] = __reduce_add_sync(FULL_MASK, sel == k ? w * p * 2 : 0u);
    WPP[k] = __reduce_add_sync(FULL_MASK, sel == k ? w * p * p : 0u);
  }
  const int limit = comp == 1 ? 64 : 32;
  #pragma unroll 1
  for (int k = 0; k < 4; k++) {
    uint32_t m = kInf;
    if (k < 2) {
      for (int c = lane; c < limit; c += 32) {
        const uint32_t pv = (uint32_t)(comp == 1 ? exp6(c) : exp5(c));
        m = min(m, W[k] * pv * pv - WP2[k] * pv + WPP[k]);
      }
    } else {
      for (uint32_t v = lane; v < 256; v += 32) m = min(m, W[k] * v * v - WP2[k] * v + WPP[k]);
    }
    rem[k] = __reduce_min_sync(FULL_MASK, m);
  }
  for (int k = 3; k > 0; k--) rem[k - 1] += rem[k];
  if (lane == 0) {
    for (int k = 0; k < 4; k++) { S.d.W[k] = W[k]; S.d.WP2[k] = WP2[k]; S.d.WPP[k] = WPP[k]; S.d.rem[k] = rem[k]; }
  }
  __syncwarp();
}


// optimize_endpoint_comps :415-486
template <bool G>
__device__ __noinline__ void optimize_comps(WarpShared& S, uint32_t& work) {
  compute_selectors(S);
  if (S.st.best.alpha || !S.st.best.err) return;
  const uint32_t blo = S.st.best.lo, bhi = S.st.best.hi;
  const int src_lo[3] = {exp5(blo >> 11), exp6((blo >> 5) & 63), exp5(blo & 31)};
  const int src_hi[3] = {exp5(bhi >> 11), exp6((bhi >> 5) & 63), exp5(bhi & 31)};
  const uint32_t lane = lane_id();
  #pragma unroll 1
  for (int comp = 0; comp < 3; comp++) {
    const int p0s = src_lo[comp], p1s = src_hi[comp];
    const uint32_t clo = S.st.best.lo, chi = S.st.best.hi;
    int lo_u[3] = {(int)(clo >> 11), (int)((clo >> 5) & 63), (int)(clo & 31)};
    const int hi_u[3] = {(int)(chi >> 11), (int)((chi >> 5) & 63), (int)(chi & 31)};
    comp_errors<G>(S, comp);
    const int limit = comp == 1 ? 64 : 32;
    auto ex = [&](int c) { return (uint32_t)(comp == 1 ? exp6(c) : exp5(c)); };
    // the component's error tables in registers (uniform across the warp)
    uint32_t W[4], WP2[4], WPP[4], rem[4];
    auto load_tables = [&]() {
      for (int k = 0; k < 4; k++) { W[k] = S.d.W[k]; WP2[k] = S.d.WP2[k]; WPP[k] = S.d.WPP[k]; rem[k] = S.d.rem[k]; }
    };
    auto E = [&](int k, uint32_t p) { return W[k] * p * p - WP2[k] * p + WPP[k]; };
    load_tables();
    uint32_t best_err = E(0, ex(lo_u[comp])) + E(1, ex(hi_u[comp])) + E(2, (uint32_t)((p0s * 2 + p1s) / 3)) +
                        E(3, (uint32_t)((p0s + p1s * 2) / 3));
    if (rem[0] >= best_err) continue;
    #pragma unroll 1
    for (int c0 = 0; c0 < limit; c0++) {
      const uint32_t p0 = ex(c0);
      uint32_t e0 = E(0, p0);
      if (e0 + rem[1] >= best_err) continue;
      {
        // does any c1 pass the component-table prune for this c0 (:456-466)? lane c1 and c1 + 32;
        // a pair passes exactly when its component error is below the best's
        bool pass = false;
        for (int c1 = (int)lane; c1 < limit; c1 += 32) {
          const uint32_t p1 = ex(c1);
          uint32_t e = e0 + E(1, p1);
          if (e + rem[2] >= best_err) continue;
          e += E(2, (p0 * 2 + p1) / 3);
          if (e + rem[3] >= best_err) continue;
          e += E(3, (p0 + p1 * 2) / 3);
          pass |= e < best_err;
        }
        if (!__any_sync(FULL_MASK, pass)) continue;
      }
      lo_u[comp] = c0;
      if (lane == 0) {
        S.d.kind = LK_COMPS; S.d.count = limit; S.d.dependent = 1; S.d.alt = 0; S.d.stop_on_accept = 1;
        S.d.comp = comp; S.d.p0 = (int)p0; S.d.e0 = e0; S.d.best_err = best_err;
        S.d.packed_lo = pack565(lo_u[0], lo_u[1], lo_u[2]);
        S.d.base[0] = hi_u[0]; S.d.base[1] = hi_u[1]; S.d.base[2] = hi_u[2];
      }
      __syncwarp();
      int start = 0;
      while (start < limit) {
        const int c1 = run_list<G>(S, start, work);
        if (c1 < 0) break;
        if (!S.st.best.err) return;
        compute_selectors(S);
        comp_errors<G>(S, comp);
        load_tables();
        const uint32_t p1 = ex(c1);
        best_err = E(0, p0) + E(1, p1) + E(2, (p0 * 2 + p1) / 3) + E(3, (p0 + p1 * 2) / 3);
        e0 = E(0, p0);
        if (lane == 0) { S.d.e0 = e0; S.d.best_err = best_err; }
        __syncwarp();
        if (e0 + rem[1] >= best_err) break;
        start = c1 + 1;
      }
    }
  }
}

// try_combinatorial_encoding :1886-1997: blocks of 2..4 colours that were DXT-compressed
// before may have their original endpoints recovered by extrapolation.
template <bool G>
__device__ __noinline__ void try_combinatorial(WarpShared& S, uint32_t& work) {
  const int n = S.st.n;
  if (n < 2 || n > 4) return;
  const uint32_t lane = lane_id();
  if (lane == 0) {
    // temporary colours (r | g << 8 | b << 16) in S.cand, unique packed endpoints in S.list
    int cnt = 0;
    for (int i = 0; i < n; i++) S.cand[cnt++] = S.uci[i];
    auto push = [&](int a, int b, float f, int rounding) {
      const float r = rounding ? 1.0f : 0.0f;
      uint32_t out = 0;
      for (int ch = 0; ch < 3; ch++) {
        const float fx = (float)((S.cand[a] >> (8 * ch)) & 255), fy = (float)((S.cand[b] >> (8 * ch)) & 255);
        const float l = __fadd_rn(fx, __fmul_rn(__fsub_rn(fy, fx), f));
        out |= (uint32_t)clampi(__float2int_rz(__fadd_rn(r, l)), 0, 255) << (8 * ch);
      }
      S.cand[cnt++] = out;
    };
    if (n == 2) {
      const float fs[10] = {2.0f, 3.0f, .5f, 1.5f, -1.0f, 2.0f, -.5f, .5f, -2.0f, -1.0f};
      #pragma unroll 1
      for (int k = 0; k < 2; k++)
        for (int q = 0; q < 2; q++)
          for (int f = 0; f < 10; f++) push(q, q ^ 1, fs[f], k);
    } else if (n == 3) {
      #pragma unroll 1
      for (int i = 0; i <= 2; i++)
        for (int j = 0; j <= 2; j++) {
          if (i == j) continue;
          push(i, j, 1.5f, 1);
          push(i, j, 2.0f / 3.0f, 1);
          push(i, j, 1.0f / 3.0f, 1);
          push(i, j, -.5f, 1);
        }
    }
    int m = 0;
    #pragma unroll 1
    for (int i = 0; i < cnt; i++) {
      const uint32_t c = S.cand[i];
      const uint32_t ur = min(((c & 255) * 31u + 127u) / 255u, 31u);
      const uint32_t ug = min((((c >> 8) & 255) * 63u + 127u) / 255u, 63u);
      const uint32_t ub = min(((c >> 16) * 31u + 127u) / 255u, 31u);
      const uint16_t pk = (uint16_t)(ub | (ug << 5) | (ur << 11));
      bool dup = false;
      for (int k = 0; k < m; k++) if (S.list[k] == pk) { dup = true; break; }
      if (!dup) S.list[m++] = pk;
    }
    S.d.nh = m;
  }
  __syncwarp();
  const int m = S.d.nh;
  #pragma unroll 1
  for (int alt = 0; alt < 2; alt++) {
    uint32_t saved = 0;
    if (alt) {
      saved = S.st.best.err;
      if (lane == 0 && saved) S.st.best.err = 1;
      __syncwarp();
    }
    #pragma unroll 1
    for (int i = 0; S.st.best.err && i + 1 < m; i++) {
      if (lane == 0) {
        S.d.kind = LK_COMB; S.d.count = m - 1 - i; S.d.dependent = 0; S.d.alt = alt; S.d.stop_on_accept = 0;
        S.d.row = i;
      }
      __syncwarp();
      run_list<G>(S, 0, work);
    }
    if (alt) {
      if (lane == 0 && S.st.best.err) S.st.best.err = saved;
      __syncwarp();
    }
  }
}

// optimize_endpoints :703-1067 from the phase-1 projection bounds. The quality level sets the probe
// table, the probe spacing and the pass count (:716-745), whether try_median4 runs (Better and
// up) and its refine level, the lattice moves (Normal and up; the +-2 moves and the per-pass
// refine at Uber only) and the final tries (:1030-1058).
template <bool G>
__device__ void optimize(WarpShared& S, uint32_t& work) {
  const uint32_t lane = lane_id();
  const uint32_t quality = G ? (uint32_t)S.st.quality : kQUber;
  if (quality >= kQBetter) {
    // try_median4: the six LBG pairs, then refine (level 1 at Uber, 0 at Better)
    if (lane < 6) S.cand[lane] = S.sd.m[lane];
    set_list(S, LK_TABLE, 6, 0, 0);
    __syncwarp();
    run_list<G>(S, 0, work);
    refine<G>(S, work, quality == kQUber ? 1 : 0);
  }
  const int table = probe_table(quality);
  const int probe_n = c_probe_size[table];
  const int passes = quality == kQUber ? 4 : quality == kQSuperFast ? 1 : 2;
  const float dist_per_trial = quality >= kQBetter ? .015625f : .027063293f;
  float sa1[3], low[3], high[3];
  const float lim[3] = {31.0f, 63.0f, 31.0f};
  for (int k = 0; k < 3; k++) {
    sa1[k] = __fmul_rn(S.sd.f[k], dist_per_trial);
    const float l = __fmul_rn(S.sd.f[3 + k], lim[k]), h = __fmul_rn(S.sd.f[6 + k], lim[k]);
    low[k] = l < 0.0f ? 0.0f : (l > lim[k] ? lim[k] : l);
    high[k] = h < 0.0f ? 0.0f : (h > lim[k] ? lim[k] : h);
  }
  sa1[0] = __fmul_rn(sa1[0], 31.0f); sa1[1] = __fmul_rn(sa1[1], 63.0f); sa1[2] = __fmul_rn(sa1[2], 31.0f);
  #pragma unroll 1
  for (int pass = 0; pass < passes; pass++) {
    if (pass) {
      const uint32_t blo = S.st.best.lo, bhi = S.st.best.hi;
      low[0] = (float)(blo >> 11); low[1] = (float)((blo >> 5) & 63); low[2] = (float)(blo & 31);
      high[0] = (float)(bhi >> 11); high[1] = (float)((bhi >> 5) & 63); high[2] = (float)(bhi & 31);
    }
    const uint32_t prev = S.st.best.err;
    if (!prev) break;
    // sweep both endpoints along the axis with the quality's probe table, both directions;
    // lane k holds probe (i, s) = ((k+1)/2, (k+1)&1) in the reference's loop order
    {
      const int k = (int)lane;
      const int i = (k + 1) >> 1, s = (k + 1) & 1;
      const float x = (float)c_probe[table][i < probe_n ? i : probe_n - 1];
      uint32_t pl, ph;
      {
        int v[3], w[3];
        for (int c = 0; c < 3; c++) {
          const float step = s ? sa1[c] : -sa1[c];
          v[c] = clampi((int)floorf(__fadd_rn(__fadd_rn(low[c], .5f), __fmul_rn(step, x))), 0, c == 1 ? 63 : 31);
          w[c] = clampi((int)floorf(__fadd_rn(__fadd_rn(high[c], .5f), __fmul_rn(step, x))), 0, c == 1 ? 63 : 31);
        }
        pl = pack565(v[0], v[1], v[2]);
        ph = pack565(w[0], w[1], w[2]);
      }
      const uint32_t pl2 = __shfl_up_sync(FULL_MASK, pl, 2), ph2 = __shfl_up_sync(FULL_MASK, ph, 2);
      const bool in = k < 2 * probe_n - 1;
      const bool rl = in && (k < 2 || pl != pl2), rh = in && (k < 2 || ph != ph2);
      const unsigned ml = __ballot_sync(FULL_MASK, rl), mh = __ballot_sync(FULL_MASK, rh);
      const unsigned below = (1u << lane) - 1u;
      if (rl) S.list[__popc(ml & below)] = (uint16_t)pl;
      if (rh) S.list2[__popc(mh & below)] = (uint16_t)ph;
      if (lane == 0) {
        S.d.kind = LK_PAIRS; S.d.count = __popc(ml) * __popc(mh); S.d.dependent = 0; S.d.alt = 0;
        S.d.stop_on_accept = 0; S.d.nh = __popc(mh);
      }
      __syncwarp();
    }
    run_list<G>(S, 0, work);
    // lattice neighbours: low endpoint (26 adjacent cells, then +-2 per axis), then high
    #pragma unroll 1
    for (int side = 0; side < (quality >= kQNormal ? 2 : 0); side++) {
      for (int kind = LK_NEIGH; kind <= (quality == kQUber ? LK_MOVE2 : LK_NEIGH); kind++) {
        if (lane == 0) {
          const uint32_t base = side ? S.st.best.hi : S.st.best.lo;
          S.d.base[0] = (int)(base >> 11); S.d.base[1] = (int)((base >> 5) & 63); S.d.base[2] = (int)(base & 31);
          S.d.kind = kind; S.d.count = kind == LK_NEIGH ? 26 : 6; S.d.dependent = 1; S.d.alt = 0;
          S.d.stop_on_accept = 0; S.d.side = side;
        }
        __syncwarp();
        run_list<G>(S, 0, work);
      }
    }
    if (!S.st.best.err || (pass && S.st.best.err == prev)) break;
    if (quality == kQUber) refine<G>(S, work);
  }
  if (quality < kQNormal) return;
  if (S.st.best.err && !(G && S.st.only3)) {
    bool solid = false;
    if (all_selectors_equal<G>(S)) solid = try_solid<G>(S, work);
    if (!solid && quality == kQUber) optimize_comps<G>(S, work);
  }
  if (quality == kQUber && S.st.best.err) try_combinatorial<G>(S, work);
}

// Plane tables -> per-channel lower bounds (compute_internal :2133-2203); lane c handles
// planes c (and c + 32 for green).
__device__ void build_lower_bounds(WarpShared& S, int n, bool perceptual) {
  const int c = (int)lane_id();
  uint32_t rw = 0, r1 = 0, r2 = 0, gw = 0, g1 = 0, g2 = 0, gw2 = 0, g12 = 0, g22 = 0, bw = 0, b1 = 0, b2 = 0;
  uint32_t tw = 0, tr1 = 0, tr2 = 0, tg1 = 0, tg2 = 0, tb1 = 0, tb2 = 0;
  #pragma unroll 1
  for (int i = 0; i < n; i++) {
    const uint32_t col = S.uci[i];
    const uint32_t w = (uint32_t)S.ucw[i];
    const int R = col & 255, G = (col >> 8) & 255, B = col >> 16;
    const int pr = (R >> 3) + ((R & 7) > (R >> 5) ? 1 : 0);
    const int pg = (G >> 2) + ((G & 3) > (G >> 6) ? 1 : 0);
    const int pb = (B >> 3) + ((B & 7) > (B >> 5) ? 1 : 0);
    tw += w;
    tr1 += w * R; tr2 += w * R * R; tg1 += w * G; tg2 += w * G * G; tb1 += w * B; tb2 += w * B * B;
    if (pr <= c) { rw += w; r1 += w * R; r2 += w * R * R; }
    if (pg <= c) { gw += w; g1 += w * G; g2 += w * G * G; }
    if (pg <= c + 32) { gw2 += w; g12 += w * G; g22 += w * G * G; }
    if (pb <= c) { bw += w; b1 += w * B; b2 += w * B * B; }
  }
  const uint32_t kr = perceptual ? 8u : 1u, kg = perceptual ? 25u : 1u;
  auto dist = [](uint32_t s2, uint32_t w, uint32_t s1, uint32_t C) { return s2 + C * C * w - 2u * C * s1; };
  {
    const uint32_t C = (uint32_t)exp5(c);
    const uint32_t lo = kr * dist(r2, rw, r1, C);
    S.lbr[c] = make_uint2(lo, kr * dist(tr2, tw, tr1, C) - lo);
    const uint32_t lob = dist(b2, bw, b1, C);
    S.lbb[c] = make_uint2(lob, dist(tb2, tw, tb1, C) - lob);
  }
  {
    const uint32_t C = (uint32_t)exp6(c), C2 = (uint32_t)exp6(c + 32);
    const uint32_t lo = kg * dist(g2, gw, g1, C), lo2 = kg * dist(g22, gw2, g12, C2);
    S.lbg[c] = make_uint2(lo, kg * dist(tg2, tw, tg1, C) - lo);
    S.lbg[c + 32] = make_uint2(lo2, kg * dist(tg2, tw, tg1, C2) - lo2);
  }
}

// Writes one finished block (endpoints as stored, the 32 selector bits). In the transparent-black
// trial the block is written, with its error, only when the trial's error over all texels with
// get_block_colors3's palette (crn_dxt.cpp:234-245; selector 3 is black) is below the error in
// err_io (crn_dxt1.cpp:2043-2075); otherwise err_out (optional) receives `err`. Every lane calls it;
// `pixel` is the lane's texel (lanes < 16).
template <bool G>
__device__ __forceinline__ void block_out(const WarpShared& S, uint32_t lo, uint32_t hi, uint32_t bits, uint32_t err,
                                          uint32_t pixel, bool perceptual, bool gray, uint32_t opts,
                                          uint8_t* __restrict__ out, uint64_t* __restrict__ err_out,
                                          uint64_t* __restrict__ err_io) {
  const uint32_t lane = lane_id();
  if (G && (opts & kD1BlackTrial)) {
    uint32_t e = 0;
    if (lane < 16) {
      const uint32_t sel = (bits >> (2 * lane)) & 3u;
      const int r0 = exp5(lo >> 11), g0 = exp6((lo >> 5) & 63), b0 = exp5(lo & 31);
      const int r1 = exp5(hi >> 11), g1 = exp6((hi >> 5) & 63), b1 = exp5(hi & 31);
      int pr = 0, pg = 0, pb = 0;
      if (sel == 0) { pr = r0; pg = g0; pb = b0; }
      else if (sel == 1) { pr = r1; pg = g1; pb = b1; }
      else if (sel == 2) { pr = (r0 + r1) >> 1; pg = (g0 + g1) >> 1; pb = (b0 + b1) >> 1; }
      const int r = (int)(pixel & 255), g = (int)((pixel >> 8) & 255), b = (int)((pixel >> 16) & 255);
      if (gray) {
        const int d = luma(r, g, b) - luma(pr, pg, pb);
        e = (uint32_t)(d * d);
      } else {
        const int dr = r - pr, dg = g - pg, db = b - pb;
        e = perceptual ? (uint32_t)(8 * dr * dr + 25 * dg * dg + db * db) : (uint32_t)(dr * dr + dg * dg + db * db);
      }
    }
    const uint32_t terr = __reduce_add_sync(FULL_MASK, e);
    if (lane == 0 && (uint64_t)terr < *err_io) {
      *reinterpret_cast<uint2*>(out) = make_uint2(lo | (hi << 16), bits);
      *err_io = terr;
    }
  } else if (lane == 0) {
    *reinterpret_cast<uint2*>(out) = make_uint2(lo | (hi << 16), bits);
    if (err_out) *err_out = err;
  }
  __syncwarp();
}

// One block on one warp: compute_internal (:2081-2232) from phase 1's hand-off, then
// return_solution. opts: a dxt1_options() word. err_out (optional) receives the error.
// In the transparent-black trial (kD1BlackTrial; err_io holds the block's error from the normal
// encode) the block is re-encoded with its near-black texels transparent and rewritten, with its
// error, only when the trial's error over all texels, selector 3 decoding to black, is lower
// (:2001-2079).
template <bool G>
__device__ uint32_t phase2_block(WarpShared& S, const uint8_t* __restrict__ px, uint32_t opts,
                                 uint8_t* __restrict__ out, uint64_t* __restrict__ err_out,
                                 uint64_t* __restrict__ err_io) {
  const uint32_t lane = lane_id();
  if (G && S.sd.n < 0) return 0;  // the trial does not apply to this block
  const bool perceptual = (opts & kD1Perceptual) != 0, use_alpha = (opts & kD1Three) != 0;
  const bool gray = G && (opts & kD1Gray) != 0;
  const uint32_t quality = G ? (opts >> kD1QualityShift) & 7u : kQUber;
  // unique colours of the opaque texels in first-occurrence order via match_any (transparent
  // texels and lanes >= 16 carry sentinels)
  const uint32_t pixel = lane < 16 ? __ldg(reinterpret_cast<const uint32_t*>(px) + lane) : 0;
  const bool transparent = G && lane < 16 && is_transparent(pixel, opts);
  const bool has_t = __any_sync(FULL_MASK, transparent);
  const uint32_t key = (lane < 16 && !transparent) ? (pixel & 0xFFFFFFu) : (0x80000000u | lane);
  const unsigned match = __match_any_sync(FULL_MASK, key);
  const int leader = __ffs(match) - 1;
  const bool is_leader = lane < 16 && !transparent && leader == (int)lane;
  const unsigned lmask = __ballot_sync(FULL_MASK, is_leader);
  const int n = __popc(lmask);
  const int uidx = __popc(lmask & ((1u << leader) - 1u));
  if (G && n == 0) {
    // every texel transparent: black endpoints, all selectors 3 (:2205-2211); the search is skipped
    block_out<G>(S, 0u, 0u, 0xFFFFFFFFu, 0u, pixel, perceptual, gray, opts, out, err_out, err_io);
    return 0;
  }
  const float wr = perceptual ? 8.f : 1.f, wg = perceptual ? 25.f : 1.f;
  if (is_leader) {
    const float r = (float)(key & 255), g = (float)((key >> 8) & 255), b = (float)(key >> 16);
    if (gray) {
      const float y = (float)luma((int)(key & 255), (int)((key >> 8) & 255), (int)(key >> 16));
      S.ucf[uidx] = make_float4(y, 0.f, 0.f, y * y);
    } else {
      S.ucf[uidx] = make_float4(r, g, b, wr * r * r + wg * g * g + b * b);
    }
    S.ucw[uidx] = __popc(match);
    S.uci[uidx] = key;
  }
  __syncwarp();
  {
    // evaluation order: weight x weighted squared distance from the mean, largest first (ties by
    // first occurrence); lane i < n places colour i at its rank
    float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
    uint32_t w = 0, c = 0;
    if ((int)lane < n) { x = S.ucf[lane]; w = (uint32_t)S.ucw[lane]; c = S.uci[lane]; }
    const float fw = (float)w;
    const float sw = (float)__reduce_add_sync(FULL_MASK, w);
    float m[3];
    {
      float a[3] = {__fmul_rn(fw, x.x), __fmul_rn(fw, x.y), __fmul_rn(fw, x.z)};
      for (int k = 0; k < 3; k++) {
        for (int o = 16; o > 0; o >>= 1) a[k] = __fadd_rn(a[k], __shfl_xor_sync(FULL_MASK, a[k], o));
        m[k] = __fdiv_rn(a[k], sw);
      }
    }
    const float dr = __fsub_rn(x.x, m[0]), dg = __fsub_rn(x.y, m[1]), db = __fsub_rn(x.z, m[2]);
    const float key = (int)lane < n ? __fmul_rn(fw, __fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(wr, dr), dr),
                                                                      __fmul_rn(__fmul_rn(wg, dg), dg)),
                                                             __fmul_rn(db, db)))
                                    : -1.f;
    int rank = 0;
    for (int j = 0; j < n; j++) {
      const float kj = __shfl_sync(FULL_MASK, key, j);
      rank += (kj > key || (kj == key && j < (int)lane)) ? 1 : 0;
    }
    if ((int)lane < n) { S.ecf[rank] = x; S.ecw[rank] = w; S.eci[rank] = c; }
  }
  // m_evaluate_hc (:2085): Uber, no 3-colour blocks, no transparency, no grayscale sampling
  const bool hc = quality == kQUber && !use_alpha && !has_t && !gray;
  if (lane == 0) {
    Sol z;
    z.lo = z.hi = 0; z.err = kInf; z.alpha = 0; z.alt = 0; z.enforce = 0; z.enforced = 0;
    S.st.best = z; S.st.snap = z;
    S.st.n = n; S.st.hc = hc ? 1 : 0; S.st.three = (use_alpha || has_t) ? 1 : 0; S.st.wr = wr; S.st.wg = wg;
    S.st.only3 = has_t ? 1 : 0;
    S.st.fast = (!hc && quality < kQBetter) ? 1 : 0;
    S.st.gray = gray ? 1 : 0;
    S.st.quality = (int)quality;
    S.st.perceptual = perceptual ? 1 : 0;
  }
  __syncwarp();
  build_lower_bounds(S, n, perceptual);
  __syncwarp();
  uint32_t work = 0;
  if (n == 1 && !has_t) {
    const uint32_t c = S.uci[0];
    const int r = c & 255, g = (c >> 8) & 255, b = c >> 16;
    if (lane == 0) { S.cand[0] = solid_coords(r, g, b, false); S.cand[1] = solid_coords(r, g, b, true); }
    set_list(S, LK_TABLE, use_alpha ? 2 : 1, 0, 0);
    __syncwarp();
    run_list<G>(S, 0, work);
  } else {
    optimize<G>(S, work);
  }
  // return_solution :263-365 (transparent texels take selector 3)
  compute_selectors(S);
  const Sol best = S.st.best;
  const int my_sel = (int)lane < n ? selector_of<G>(S, lane, sel_source(S)) : 0;
  const int s = __shfl_sync(FULL_MASK, my_sel, (lane < 16 && !transparent) ? uidx : 0);
  const bool invert = best.alpha ? best.lo > best.hi : best.lo < best.hi;
  int sel = s;
  if (invert) sel = best.alpha ? (s < 2 ? (s ^ 1) : s) : (s ^ 1);
  if (transparent) sel = 3;
  const uint32_t bits = __reduce_or_sync(FULL_MASK, lane < 16 ? ((uint32_t)sel << (2 * lane)) : 0u);
  const uint32_t lo = invert ? best.hi : best.lo, hi = invert ? best.lo : best.hi;
  block_out<G>(S, lo, hi, bits, best.err, pixel, perceptual, gray, opts, out, err_out, err_io);
  return work;
}

// ---- TMA staging of a warp's chunk: cp.async.bulk global -> shared completing on an mbarrier.
// The copy is 64 * cnt bytes from a 64-byte aligned block, so source, destination and size meet
// the bulk copy's 16-byte rules. Waits are bounded: after g_stage_wait_polls polls the warp stops
// using the stage and reads its blocks from global memory (the results do not change), and the
// event is counted in g_stage_timeouts. Before the warp exits, a copy still in flight is drained
// with a separate, much longer bound (kStageDrainPolls) that the test hook does not change; a
// drain that runs out is counted in g_stage_drain_failures.
constexpr uint32_t kStageWaitLimit = 1u << 22;
constexpr uint32_t kStageDrainPolls = 1u << 26;
__device__ uint32_t g_stage_wait_polls = kStageWaitLimit;
__device__ unsigned int g_stage_timeouts;
__device__ unsigned int g_stage_drain_failures;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void stage_init(SeedShared& S) {
  if (lane_id() == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&S.bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
}

// lane 0: announce the byte count and start the copies of nrun runs of consecutive blocks into
// S.stage: run j (cnt[j] blocks from src[j]) lands at stage byte offset dst[j]. Every source is a
// block (64-byte aligned), so addresses and sizes meet the bulk copy's 16-byte rules.
__device__ __forceinline__ void stage_issue(SeedShared& S, int nrun, const uint8_t* const* src, const uint32_t* cnt,
                                            const uint32_t* dst) {
  if (lane_id() == 0) {
    uint32_t bytes = 0;
    for (int j = 0; j < nrun; j++) bytes += cnt[j] * 64u;
    const uint32_t bar = smem_u32(&S.bar), base = smem_u32(S.stage);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // earlier generic reads of the stage
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
    for (int j = 0; j < nrun; j++)
      if (cnt[j])
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         base + dst[j]),
                     "l"(src[j]), "r"(cnt[j] * 64u), "r"(bar)
                     : "memory");
  }
}

// every lane: wait for the copy of the given phase parity; false after `polls` polls
__device__ __forceinline__ bool stage_poll(SeedShared& S, uint32_t parity, uint32_t polls) {
  const uint32_t bar = smem_u32(&S.bar);
  for (uint32_t i = 0; i < polls; i++) {
    uint32_t done;
    asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
                 : "=r"(done)
                 : "r"(bar), "r"(parity)
                 : "memory");
    if (__all_sync(FULL_MASK, done != 0)) return true;
  }
  return false;
}

__device__ __forceinline__ bool stage_wait(SeedShared& S, uint32_t parity) {
  if (stage_poll(S, parity, g_stage_wait_polls)) return true;
  if (lane_id() == 0) atomicAdd(&g_stage_timeouts, 1u);
  return false;
}

// A warp's sequence of block groups, each staged in shared memory: the copies for group i + 1 are
// issued as soon as the lanes have read group i from the stage, so they overlap its phase 1.
struct ChunkStager {
  uint32_t parity = 0;
  bool live = true;   // false after a timed-out wait: blocks are then read from global memory
  bool pending = false;
  __device__ void start(SeedShared& S, int nrun, const uint8_t* const* src, const uint32_t* cnt, const uint32_t* dst) {
    stage_init(S);
    stage_issue(S, nrun, src, cnt, dst);
    pending = true;
  }
  // the staged blocks of the current group, or nullptr once staging was abandoned (the caller then
  // reads the blocks from global memory)
  __device__ const uint8_t* acquire(SeedShared& S) {
    if (live && pending) {
      live = stage_wait(S, parity);
      if (live) { parity ^= 1u; pending = false; }
    }
    return live ? S.stage : nullptr;
  }
  __device__ void next(SeedShared& S, int nrun, const uint8_t* const* src, const uint32_t* cnt, const uint32_t* dst) {
    if (!live) return;
    __syncwarp();  // every lane has read the stage
    stage_issue(S, nrun, src, cnt, dst);
    pending = true;
  }
  // before the warp exits: a copy still in flight must land first (bounded by the drain limit)
  __device__ void finish(SeedShared& S) {
    if (pending && !stage_poll(S, parity, kStageDrainPolls) && lane_id() == 0) atomicAdd(&g_stage_drain_failures, 1u);
  }
};

__device__ __forceinline__ void load_pix(const uint8_t* px, uint32_t (&pix)[16]) {
  const uint4* p4 = reinterpret_cast<const uint4*>(px);
  for (int q = 0; q < 4; q++) {
    const uint4 v = p4[q];
    pix[4 * q] = v.x; pix[4 * q + 1] = v.y; pix[4 * q + 2] = v.z; pix[4 * q + 3] = v.w;
  }
}

// Phase 1 over n blocks: warp w takes the groups of 32 consecutive blocks g = w, w + W, ..., a lane
// per block, each group staged by one bulk copy. Warps are ranked CTA-first (warp 0 of every CTA,
// then warp 1, ...), and the grid has a CTA per group up to the resident limit, so a short batch
// (the learned encoder's fallback blocks, a small mip level) puts one working warp on each SM:
// the seeds are bound by the SM's FP64 pipe, which the warps of one CTA would share.
template <bool G>
__global__ void __launch_bounds__(kWarpsPerCta * 32, kSeedCtasPerSm)
    k_dxt1_seeds(const uint8_t* __restrict__ blocks, uint32_t n, uint32_t opts, Seed* __restrict__ seeds,
                 const uint32_t* __restrict__ n_dev) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  if (n_dev) n = min(n, *n_dev);  // a count the host does not read back: n is then only the grid's bound
  SeedShared& S = reinterpret_cast<SeedShared*>(smem_raw)[threadIdx.x >> 5];
  const uint32_t lane = lane_id();
  const uint32_t warp_global = (threadIdx.x >> 5) * gridDim.x + blockIdx.x;
  const uint32_t nwarps = gridDim.x * kWarpsPerCta;
  const uint32_t groups = (n + kSeedLanes - 1) / kSeedLanes;
  const uint32_t zero = 0;
  auto run = [&](uint32_t g, const uint8_t*& src, uint32_t& cnt) {
    src = blocks + (size_t)g * kSeedLanes * 64;
    cnt = min((uint32_t)kSeedLanes, n - g * kSeedLanes);
  };
  ChunkStager st;
  if (warp_global < groups) {
    const uint8_t* src; uint32_t cnt;
    run(warp_global, src, cnt);
    st.start(S, 1, &src, &cnt, &zero);
  }
  for (uint32_t g = warp_global; g < groups; g += nwarps) {
    const uint32_t b = g * kSeedLanes + lane;
    const uint8_t* staged = st.acquire(S);
    uint32_t pix[16];
    if (b < n) load_pix(staged ? staged + (size_t)lane * 64 : blocks + (size_t)b * 64, pix);
    const uint32_t gn = g + nwarps;
    if (gn < groups) {
      const uint8_t* src; uint32_t cnt;
      run(gn, src, cnt);
      st.next(S, 1, &src, &cnt, &zero);
    }
    if (b < n) phase1_block<G>(S, (int)lane, pix, opts, seeds + b);
  }
  st.finish(S);
}

// one lane per 16 bytes: the block's seed into the warp's shared memory
__device__ __forceinline__ void load_seed(WarpShared& S, const Seed* __restrict__ seed) {
  const uint32_t lane = lane_id();
  if (lane < 4) reinterpret_cast<uint4*>(&S.sd)[lane] = __ldg(reinterpret_cast<const uint4*>(seed) + lane);
  __syncwarp();
}

// Phase 2 over n blocks whose seeds k_dxt1_seeds wrote: warp w takes blocks w, w + W, w + 2W, ...
// (every warp's count within one of the others', block costs interleaved across warps).
// G = false: Uber quality, perceptual or uniform, no grayscale sampling, transparency or black trial
// (the default encode, compiled without the general paths); G = true: every option.
template <bool G>
__global__ void __launch_bounds__(kWarpsPerCta * 32, kCtasPerSm)
    k_dxt1_encode(const uint8_t* __restrict__ blocks, uint32_t n, uint32_t opts, const Seed* __restrict__ seeds,
                  uint8_t* __restrict__ out, uint32_t out_stride, uint64_t* __restrict__ err_out,
                  uint64_t* __restrict__ err_io, unsigned long long* __restrict__ work_out,
                  const uint32_t* __restrict__ n_dev) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  if (n_dev) n = min(n, *n_dev);
  WarpShared& S = reinterpret_cast<WarpShared*>(smem_raw)[threadIdx.x >> 5];
  const uint32_t lane = lane_id();
  const uint32_t warp_global = blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5);
  const uint32_t nwarps = gridDim.x * kWarpsPerCta;
  unsigned long long work = 0;
  #pragma unroll 1
  for (uint32_t b = warp_global; b < n; b += nwarps) {
    load_seed(S, seeds + b);
    work += phase2_block<G>(S, blocks + (size_t)b * 64, opts, out + (size_t)b * out_stride,
                            err_out ? err_out + b : nullptr, err_io ? err_io + b : nullptr);
  }
  if (work_out) {
    for (int o = 16; o > 0; o >>= 1) work += __shfl_xor_sync(FULL_MASK, work, o);
    if (lane == 0 && work) atomicAdd(work_out, work);
  }
}

// ------------------------------------------------------------------------------------------
// DXT5A: warp per block, lane per (low, high) candidate.

struct Alpha5 {
  int n;
  uint32_t val[16], wt[16];
  bool both;
  // error of both block types for one (l, h); 8-value preferred on ties
  __device__ __forceinline__ void eval(int l, int h, uint32_t& err, int& type) const {
    int p8[8], p6[8];
    p8[0] = l; p8[1] = h;
    p8[2] = (l * 6 + h) / 7; p8[3] = (l * 5 + h * 2) / 7; p8[4] = (l * 4 + h * 3) / 7;
    p8[5] = (l * 3 + h * 4) / 7; p8[6] = (l * 2 + h * 5) / 7; p8[7] = (l + h * 6) / 7;
    p6[0] = l; p6[1] = h;
    p6[2] = (l * 4 + h) / 5; p6[3] = (l * 3 + h * 2) / 5; p6[4] = (l * 2 + h * 3) / 5; p6[5] = (l + h * 4) / 5;
    p6[6] = 0; p6[7] = 255;
    uint32_t e8 = 0, e6 = 0;
    for (int i = 0; i < n; i++) {
      const int v = (int)val[i];
      int m8 = 1 << 30, m6 = 1 << 30;
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const int d8 = v - p8[j], d6 = v - p6[j];
        m8 = min(m8, d8 * d8);
        m6 = min(m6, d6 * d6);
      }
      e8 += (uint32_t)m8 * wt[i];
      e6 += (uint32_t)m6 * wt[i];
    }
    if (both && e6 < e8) { err = e6; type = 1; }
    else { err = e8; type = 0; }
  }
};

// One DXT5A element (dxt5_endpoint_optimizer::compute, crnlib/crn_dxt5a.cpp:40-196) of the 4x4
// RGBA8 block px on channel comp, written as 8 bytes to o; a whole warp, lane per candidate.
// quality: crn_dxt_quality; the probe grid is +-16 at Uber, +-8 at Better and absent below (:105-110).
__device__ __forceinline__ void alpha_block(const uint8_t* __restrict__ px, int comp, int both, uint32_t quality,
                                            uint8_t* __restrict__ o) {
  const uint32_t lane = lane_id();
  const uint32_t v = lane < 16 ? __ldg(px + lane * 4 + comp) : 0x100u + lane;
  const unsigned match = __match_any_sync(FULL_MASK, v);
  const int leader = __ffs(match) - 1;
  const bool is_leader = lane < 16 && leader == (int)lane;
  const unsigned lmask = __ballot_sync(FULL_MASK, is_leader);
  Alpha5 A;
  A.n = __popc(lmask);
  A.both = both != 0;
  const int uidx = __popc(lmask & ((1u << leader) - 1u));
  // every lane gets the unique values (first-occurrence order) and weights
  {
    unsigned m = lmask;
    for (int i = 0; i < A.n; i++) {
      const int src = __ffs(m) - 1;
      m &= m - 1;
      A.val[i] = __shfl_sync(FULL_MASK, v, src);
      A.wt[i] = (uint32_t)__popc(__shfl_sync(FULL_MASK, match, src));
    }
  }
  uint32_t first = 0, second = 0, berr = kInf;
  int btype = 0;
  if (A.n == 1) {
    if (lane == 0) {
      uint2 w = make_uint2(A.val[0] | (A.val[0] << 8), 0u);
      *reinterpret_cast<uint2*>(o) = w;
    }
    return;
  }
  auto accept_chain = [&](bool valid, int l, int h, uint32_t err, int type, bool dependent) -> int {
    unsigned ok = __ballot_sync(FULL_MASK, valid && err < berr);
    int last = -1;
    while (ok) {
      const int j = __ffs(ok) - 1;
      berr = __shfl_sync(FULL_MASK, err, j);
      first = (uint32_t)__shfl_sync(FULL_MASK, l, j);
      second = (uint32_t)__shfl_sync(FULL_MASK, h, j);
      btype = __shfl_sync(FULL_MASK, type, j);
      last = j;
      if (dependent) break;
      const unsigned after = j == 31 ? 0u : (FULL_MASK << (j + 1));
      ok = __ballot_sync(FULL_MASK, valid && err < berr) & after;
    }
    return last;
  };
  // all unique value pairs i < j (compute :83-96)
  const int npairs = A.n * (A.n - 1) / 2;
  for (int p0 = 0; p0 < npairs; p0 += 32) {
    const int p = p0 + (int)lane;
    int l = 0, h = 0;
    const bool valid = p < npairs;
    if (valid) {
      int i = 0, rem = p;
      while (rem >= A.n - 1 - i) { rem -= A.n - 1 - i; i++; }
      l = (int)A.val[i];
      h = (int)A.val[i + 1 + rem];
    }
    uint32_t err = kInf;
    int type = 0;
    if (valid) A.eval(l, h, err, type);
    accept_chain(valid, l, h, err, type, false);
  }
  // +-R probe around the running best (:98-141); the centre moves with each improvement
  const int R = quality == kQUber ? 16 : 8, D = 2 * R + 1;
  if (berr && quality >= kQBetter) {
    int pos = 0, row_l = (int)first - R;
    const int total = D * D;
    while (pos < total) {
      const int p = pos + (int)lane;
      const int row0 = pos / D;
      int l = 0, h = 0;
      bool valid = p < total;
      if (valid) {
        const int r = p / D, c = p % D;
        l = r == row0 ? row_l : (int)first + (r - R);
        h = (int)second + (c - R);
        valid = l >= 0 && l <= 255 && h >= 0 && h <= 255;
      }
      uint32_t err = kInf;
      int type = 0;
      if (valid) A.eval(l, h, err, type);
      const int last = accept_chain(valid, l, h, err, type, true);
      const int next = last >= 0 ? pos + last + 1 : pos + 32;
      const int nrow = next / D;
      // the reference fixes l when a row starts: a row begun inside this batch used the
      // centre from before the batch, unless it is the accepted candidate's own row
      const int last_row = last >= 0 ? (pos + last) / D : -1;
      if (last >= 0 && nrow == last_row) row_l = __shfl_sync(FULL_MASK, l, last);
      else if (nrow != row0) row_l = (int)first + (nrow - R);
      pos = next;
    }
  }
  // selectors of the winner, reorder rules (:143-185), pack (dxt5_block, crn_dxt.h:318-361)
  int sel = 0;
  if (lane < 16) {
    const int l = (int)first, h = (int)second;
    int pv[8];
    pv[0] = l; pv[1] = h;
    if (btype == 0) {
      pv[2] = (l * 6 + h) / 7; pv[3] = (l * 5 + h * 2) / 7; pv[4] = (l * 4 + h * 3) / 7;
      pv[5] = (l * 3 + h * 4) / 7; pv[6] = (l * 2 + h * 5) / 7; pv[7] = (l + h * 6) / 7;
    } else {
      pv[2] = (l * 4 + h) / 5; pv[3] = (l * 3 + h * 2) / 5; pv[4] = (l * 2 + h * 3) / 5; pv[5] = (l + h * 4) / 5;
      pv[6] = 0; pv[7] = 255;
    }
    const int x = (int)A.val[uidx];
    int bd = 1 << 30;
    for (int j = 0; j < 8; j++) {
      const int d = (x - pv[j]) * (x - pv[j]);
      if (d < bd) { bd = d; sel = j; }
    }
  }
  uint32_t f = first, s = second;
  if (f == s) {
    sel = 0;
  } else if (btype) {
    if (f > s) {
      const uint32_t t = f; f = s; s = t;
      const int inv6[8] = {1, 0, 5, 4, 3, 2, 6, 7};
      sel = inv6[sel];
    }
  } else if (f <= s) {
    const uint32_t t = f; f = s; s = t;
    const int inv8[8] = {1, 0, 7, 6, 5, 4, 3, 2};
    sel = inv8[sel];
  }
  const uint32_t lo_bits = __reduce_or_sync(FULL_MASK, lane < 10 ? ((uint32_t)sel << (3 * lane)) : 0u);
  const uint32_t hi_bits = __reduce_or_sync(FULL_MASK, (lane >= 10 && lane < 16) ? ((uint32_t)sel << (3 * (lane - 10))) : 0u);
  if (lane == 0) {
    const uint64_t bits = (uint64_t)lo_bits | ((uint64_t)hi_bits << 30);
    const uint64_t word = (uint64_t)f | ((uint64_t)s << 8) | (bits << 16);
    *reinterpret_cast<uint2*>(o) = make_uint2((uint32_t)word, (uint32_t)(word >> 32));
  }
}

__global__ void __launch_bounds__(128)
    k_dxt5a_encode(const uint8_t* __restrict__ blocks, uint32_t n, int comp, int both, uint32_t quality,
                   uint8_t* __restrict__ out, uint32_t out_stride) {
  const uint32_t warp_global = blockIdx.x * 4 + (threadIdx.x >> 5);
  const uint32_t nwarps = gridDim.x * 4;
  for (uint32_t bi = warp_global; bi < n; bi += nwarps)
    alpha_block(blocks + (size_t)bi * 64, comp, both, quality, out + (size_t)bi * out_stride);
}

// ------------------------------------------------------------------------------------------
// Batched (many textures, mixed formats): persistent warps over a chunk table. A chunk is a run of
// consecutive blocks of one segment (one element of one texture: its DXT1 colour, DXT5 colour or
// alpha, a DXN channel); the segment gives the output base, stride and encoder options.

static_assert(kSeedLanes % kColourChunkBlocks == 0 && kSeedLanes / kColourChunkBlocks == 4,
              "the phase-1 kernel stages four colour chunks per warp");

// Phase 1 of the batched encode: warp w takes the groups of 4 consecutive chunks g = w, w + W, ...
// (lane 8j + k: block k of chunk 4g + j), each chunk's run of blocks staged by one bulk copy; the
// seed of block b goes to seeds[b].
__global__ void __launch_bounds__(kWarpsPerCta * 32, kSeedCtasPerSm)
    k_dxt1_seeds_chunks(const uint8_t* __restrict__ blocks, const EncodeChunk* __restrict__ chunks, uint32_t nchunks,
                        const EncodeSegment* __restrict__ segs, Seed* __restrict__ seeds) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SeedShared& S = reinterpret_cast<SeedShared*>(smem_raw)[threadIdx.x >> 5];
  const uint32_t lane = lane_id();
  const uint32_t warp_global = blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5);
  const uint32_t nwarps = gridDim.x * kWarpsPerCta;
  constexpr uint32_t kPer = kSeedLanes / kColourChunkBlocks;  // chunks per group
  const uint32_t groups = (nchunks + kPer - 1) / kPer;
  const uint32_t dst[kPer] = {0, 64 * kColourChunkBlocks, 128 * kColourChunkBlocks, 192 * kColourChunkBlocks};
  auto runs = [&](uint32_t g, const uint8_t* (&src)[kPer], uint32_t (&cnt)[kPer]) {
    for (uint32_t j = 0; j < kPer; j++) {
      const uint32_t c = g * kPer + j;
      const EncodeChunk ch = c < nchunks ? chunks[c] : EncodeChunk{0, 0, 0};
      src[j] = blocks + (size_t)ch.first * 64;
      cnt[j] = ch.count;
    }
  };
  ChunkStager st;
  if (warp_global < groups) {
    const uint8_t* src[kPer]; uint32_t cnt[kPer];
    runs(warp_global, src, cnt);
    st.start(S, kPer, src, cnt, dst);
  }
  for (uint32_t g = warp_global; g < groups; g += nwarps) {
    const uint32_t c = g * kPer + lane / kColourChunkBlocks, k = lane % kColourChunkBlocks;
    const EncodeChunk ch = c < nchunks ? chunks[c] : EncodeChunk{0, 0, 0};
    const bool mine = k < ch.count;
    const uint8_t* staged = st.acquire(S);
    uint32_t pix[16];
    if (mine) load_pix(staged ? staged + (size_t)lane * 64 : blocks + ((size_t)ch.first + k) * 64, pix);
    const uint32_t gn = g + nwarps;
    if (gn < groups) {
      const uint8_t* src[kPer]; uint32_t cnt[kPer];
      runs(gn, src, cnt);
      st.next(S, kPer, src, cnt, dst);
    }
    if (mine) phase1_block<false>(S, (int)lane, pix, segs[ch.segment].options, seeds + ch.first + k);
  }
  st.finish(S);
}

// Phase 2 of the batched encode: persistent warps walk the chunk table, a block at a time.
__global__ void __launch_bounds__(kWarpsPerCta * 32, kCtasPerSm)
    k_dxt1_encode_chunks(const uint8_t* __restrict__ blocks, const EncodeChunk* __restrict__ chunks, uint32_t nchunks,
                         const EncodeSegment* __restrict__ segs, const Seed* __restrict__ seeds) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  WarpShared& S = reinterpret_cast<WarpShared*>(smem_raw)[threadIdx.x >> 5];
  const uint32_t warp_global = blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5);
  const uint32_t nwarps = gridDim.x * kWarpsPerCta;
  for (uint32_t c = warp_global; c < nchunks; c += nwarps) {
    const EncodeChunk ch = chunks[c];
    const EncodeSegment sg = segs[ch.segment];
    #pragma unroll 1
    for (uint32_t k = 0; k < ch.count; k++) {
      const uint32_t b = ch.first + k;
      load_seed(S, seeds + b);
      phase2_block<false>(S, blocks + (size_t)b * 64, sg.options, sg.out + (size_t)(b - sg.first_block) * sg.stride,
                          nullptr, nullptr);
    }
  }
}

__global__ void __launch_bounds__(128)
    k_dxt5a_encode_chunks(const uint8_t* __restrict__ blocks, const EncodeChunk* __restrict__ chunks, uint32_t nchunks,
                          const EncodeSegment* __restrict__ segs) {
  const uint32_t warp_global = blockIdx.x * 4 + (threadIdx.x >> 5);
  const uint32_t nwarps = gridDim.x * 4;
  for (uint32_t c = warp_global; c < nchunks; c += nwarps) {
    const EncodeChunk ch = chunks[c];
    const EncodeSegment sg = segs[ch.segment];
    const int comp = (int)((sg.options >> kSegCompShift) & 3u);
    const int both = (sg.options & kSegBothTypes) ? 1 : 0;
    const uint32_t quality = (sg.options >> kSegAlphaQualityShift) & 7u;
    for (uint32_t k = 0; k < ch.count; k++) {
      const uint32_t b = ch.first + k;
      alpha_block(blocks + (size_t)b * 64, comp, both, quality, sg.out + (size_t)(b - sg.first_block) * sg.stride);
    }
  }
}

// ------------------------------------------------------------------------------------------
// Host side

namespace {

// ryg table construction (crnlib/crn_ryg_dxt.cpp:58-99,517-535), same integer algorithm
void build_single_colour(SingleColour& t) {
  auto build = [](uint8_t (*tab)[2], int bits, bool three) {
    const int size = 1 << bits;
    for (int v = 0; v < 256; v++) {
      int best = 256;
      for (int lo = 0; lo < size; lo++) {
        for (int hi = 0; hi < size; hi++) {
          const int le = bits == 5 ? (lo << 3) | (lo >> 2) : (lo << 2) | (lo >> 4);
          const int he = bits == 5 ? (hi << 3) | (hi >> 2) : (hi << 2) | (hi >> 4);
          const int interp = three ? ((le + he) >> 1) : ((he * 2 + le) / 3);
          const int d = interp - v, spread = he - le;
          const int e = (d < 0 ? -d : d) + (((spread < 0 ? -spread : spread) * 8) >> 8);
          if (e < best) { tab[v][0] = (uint8_t)hi; tab[v][1] = (uint8_t)lo; best = e; }
        }
      }
    }
  };
  build(t.m5, 5, false);
  build(t.m6, 6, false);
  build(t.m5_3, 5, true);
  build(t.m6_3, 6, true);
}

struct DeviceInit {
  bool done[64] = {};
};

SingleColour* single_colour_host_tables() {
  static SingleColour* host = [] {  // initialised once, thread-safely
    SingleColour* t = new SingleColour;
    build_single_colour(*t);
    return t;
  }();
  return host;
}

int ensure_tables() {
  static DeviceInit init;
  static std::mutex mu;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_check(e, "cudaGetDevice");
  std::lock_guard<std::mutex> lock(mu);
  if (dev < 64 && init.done[dev]) return CRNGPU_OK;
  if ((e = cudaMemcpyToSymbol(c_sct, single_colour_host_tables(), sizeof(SingleColour))) != cudaSuccess)
    return cuda_check(e, "upload tables");
  if (dev < 64) init.done[dev] = true;
  return CRNGPU_OK;
}

}  // namespace

// ryg single-colour tables on the host: m5[256][2], m6[256][2] (then the 3-colour variants)
const void* single_colour_tables_host() { return single_colour_host_tables(); }

namespace {

int grid_for(const void* kernel, int threads, uint32_t work_units) {
  int dev = 0, sms = 148, per_sm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0);
  if (per_sm < 1) per_sm = 1;
  const uint32_t full = (uint32_t)sms * (uint32_t)per_sm;
  return (int)(work_units < full ? (work_units ? work_units : 1) : full);
}

}  // namespace

// Device-pointer launches (no synchronization).
// Opt-in work counter (profiling hook): candidate x unique-colour evaluations of the DXT1 search.
namespace {
bool g_count = false;
DevBuf g_count_buf;
}

int set_work_counter(bool on, cudaStream_t s) {
  g_count = on;
  if (!on) return CRNGPU_OK;
  cudaError_t e = g_count_buf.ensure(16);
  if (e != cudaSuccess) return cuda_check(e, "alloc counter");
  return cuda_check(cudaMemsetAsync(g_count_buf.ptr, 0, 16, s), "clear counter");
}

int read_work_counter(uint64_t* value, cudaStream_t s) {
  if (!g_count_buf.ptr) { *value = 0; return CRNGPU_OK; }
  cudaError_t e = cudaMemcpyAsync(value, g_count_buf.ptr, 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return cuda_check(e, "read counter");
}

namespace {

// Per-device stream-ordered pool for the seed records between the two DXT1 kernels (memory is
// kept in the pool between calls, so steady-state calls do not go to the driver).
int seed_pool(int dev, cudaMemPool_t* out) {
  static cudaMemPool_t pools[64] = {};
  if (dev < 0 || dev >= 64) { set_error("device index out of range"); return CRNGPU_E_PARAM; }
  std::lock_guard<std::mutex> lock(device_setup_mutex());
  if (!pools[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t p;
    cudaError_t e = cudaMemPoolCreate(&p, &props);
    if (e != cudaSuccess) return cuda_check(e, "create seed pool");
    uint64_t keep = ~0ull;
    if ((e = cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep)) != cudaSuccess)
      return cuda_check(e, "seed pool attribute");
    pools[dev] = p;
  }
  *out = pools[dev];
  return CRNGPU_OK;
}

// Shared-memory attributes and resident CTAs per SM of the DXT1 kernels, set up once per device.
struct Dxt1Launch {
  int sms = 148, seeds_per_sm = 1, search_per_sm[2] = {1, 1};
};
int dxt1_launch_setup(int dev, Dxt1Launch* L) {
  static Dxt1Launch cache[64];
  static bool done[64] = {};
  if (dev < 0 || dev >= 64) { set_error("device index out of range"); return CRNGPU_E_PARAM; }
  std::lock_guard<std::mutex> lock(device_setup_mutex());
  if (!done[dev]) {
    Dxt1Launch c;
    const int smem = (int)(sizeof(WarpShared) * kWarpsPerCta), seed_smem = (int)(sizeof(SeedShared) * kWarpsPerCta);
    cudaError_t e = cudaFuncSetAttribute(k_dxt1_encode<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_dxt1_encode<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_dxt1_encode_chunks, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_dxt1_seeds<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, seed_smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_dxt1_seeds<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, seed_smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_dxt1_seeds_chunks, cudaFuncAttributeMaxDynamicSharedMemorySize, seed_smem);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c.sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c.seeds_per_sm, k_dxt1_seeds<true>, kWarpsPerCta * 32, seed_smem);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c.search_per_sm[0], k_dxt1_encode<false>, kWarpsPerCta * 32, smem);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c.search_per_sm[1], k_dxt1_encode<true>, kWarpsPerCta * 32, smem);
    if (e != cudaSuccess) return cuda_check(e, "set up the DXT1 kernels");
    c.seeds_per_sm = c.seeds_per_sm < 1 ? 1 : c.seeds_per_sm;
    for (int k = 0; k < 2; k++) c.search_per_sm[k] = c.search_per_sm[k] < 1 ? 1 : c.search_per_sm[k];
    cache[dev] = c;
    done[dev] = true;
  }
  *L = cache[dev];
  return CRNGPU_OK;
}

// Phase 1 (k_dxt1_seeds) then phase 2 (k_dxt1_encode) over n blocks, their seed records in
// stream-ordered memory from the seed pool.
// n_dev (optional): the block count in device memory, at most n; the grids are sized for n.
int launch_dxt1_kernel(const uint8_t* d_blocks, uint32_t n, uint32_t opts, uint8_t* d_out, uint32_t out_stride,
                       uint64_t* d_err, uint64_t* d_err_io, cudaStream_t s, const uint32_t* n_dev = nullptr) {
  int rc = ensure_tables();
  if (rc != CRNGPU_OK) return rc;
  if (!n) return CRNGPU_OK;
  if (((opts >> kD1QualityShift) & 7u) > kQUber) { set_error("bad DXT quality"); return CRNGPU_E_PARAM; }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_check(e, "cudaGetDevice");
  Dxt1Launch L;
  if ((rc = dxt1_launch_setup(dev, &L)) != CRNGPU_OK) return rc;
  cudaMemPool_t pool;
  if ((rc = seed_pool(dev, &pool)) != CRNGPU_OK) return rc;
  Seed* seeds = nullptr;
  if ((e = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&seeds), (size_t)n * sizeof(Seed), pool, s)) != cudaSuccess)
    return cuda_check(e, "allocate seed records");
  unsigned long long* work = g_count ? static_cast<unsigned long long*>(g_count_buf.ptr) : nullptr;
  // the general kernels for anything beyond the default Uber encode
  const bool general = (opts & ~(kD1Perceptual | kD1Three | (7u << kD1QualityShift) | (255u << kD1ThresholdShift))) ||
                       ((opts >> kD1QualityShift) & 7u) != kQUber;
  const uint32_t seed_warps = (n + kSeedLanes - 1) / kSeedLanes;
  const uint32_t seed_full = (uint32_t)(L.sms * L.seeds_per_sm);
  const uint32_t seed_grid = std::min<uint32_t>(seed_warps, seed_full);
  const size_t seed_smem = sizeof(SeedShared) * kWarpsPerCta, smem = sizeof(WarpShared) * kWarpsPerCta;
  const uint32_t full = (uint32_t)(L.sms * L.search_per_sm[general ? 1 : 0]);
  const uint32_t grid = std::min<uint32_t>((n + kWarpsPerCta - 1) / kWarpsPerCta, full);
  if (general) {
    k_dxt1_seeds<true><<<seed_grid, kWarpsPerCta * 32, seed_smem, s>>>(d_blocks, n, opts, seeds, n_dev);
    k_dxt1_encode<true><<<grid, kWarpsPerCta * 32, smem, s>>>(d_blocks, n, opts, seeds, d_out, out_stride, d_err,
                                                             d_err_io, work, n_dev);
  } else {
    k_dxt1_seeds<false><<<seed_grid, kWarpsPerCta * 32, seed_smem, s>>>(d_blocks, n, opts, seeds, n_dev);
    k_dxt1_encode<false><<<grid, kWarpsPerCta * 32, smem, s>>>(d_blocks, n, opts, seeds, d_out, out_stride, d_err,
                                                              d_err_io, work, n_dev);
  }
  e = cudaGetLastError();
  const cudaError_t fe = cudaFreeAsync(seeds, s);
  if (e != cudaSuccess) return cuda_check(e, "launch k_dxt1_seeds / k_dxt1_encode");
  return cuda_check(fe, "release seed records");
}

}  // namespace

int launch_dxt1(const uint8_t* d_blocks, uint32_t n, uint32_t opts, uint8_t* d_out, uint32_t out_stride,
                uint64_t* d_err, cudaStream_t s) {
  return launch_dxt1_kernel(d_blocks, n, opts & ~kD1BlackTrial, d_out, out_stride, d_err, nullptr, s);
}

int launch_dxt1_count(const uint8_t* d_blocks, uint32_t n_max, const uint32_t* n_dev, uint32_t opts, uint8_t* d_out,
                      uint32_t out_stride, cudaStream_t s) {
  return launch_dxt1_kernel(d_blocks, n_max, opts & ~kD1BlackTrial, d_out, out_stride, nullptr, nullptr, s, n_dev);
}

int launch_dxt1_black_trial(const uint8_t* d_blocks, uint32_t n, uint32_t opts, uint8_t* d_out, uint32_t out_stride,
                            uint64_t* d_err_io, cudaStream_t s) {
  if (!d_err_io) { set_error("the transparent-black trial needs the blocks' errors"); return CRNGPU_E_PARAM; }
  return launch_dxt1_kernel(d_blocks, n, opts | kD1BlackTrial, d_out, out_stride, nullptr, d_err_io, s);
}

int dxt1_chunks_max_grid() {
  const size_t smem = sizeof(WarpShared) * kWarpsPerCta;
  int dev = 0, per_sm = 1;
  cudaGetDevice(&dev);
  Dxt1Launch L;
  if (dxt1_launch_setup(dev, &L) != CRNGPU_OK) return -1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_dxt1_encode_chunks, kWarpsPerCta * 32, smem);
  return L.sms * (per_sm < 1 ? 1 : per_sm);
}

int dxt5a_chunks_max_grid() {
  int dev = 0, per_sm = 1, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_dxt5a_encode_chunks, 128, 0);
  return sms * (per_sm < 1 ? 1 : per_sm);
}

int launch_dxt1_chunks(const uint8_t* d_blocks, const EncodeChunk* d_chunks, uint32_t nchunks,
                       const EncodeSegment* d_segs, void* d_seeds, int grid, cudaStream_t s) {
  int rc = ensure_tables();
  if (rc != CRNGPU_OK) return rc;
  if (!nchunks) return CRNGPU_OK;
  int dev = 0;
  cudaGetDevice(&dev);
  Dxt1Launch L;
  if ((rc = dxt1_launch_setup(dev, &L)) != CRNGPU_OK) return rc;
  const uint32_t groups = (nchunks + 3) / 4;
  const uint32_t seed_grid =
      std::min<uint32_t>((groups + kWarpsPerCta - 1) / kWarpsPerCta, (uint32_t)(L.sms * L.seeds_per_sm));
  Seed* seeds = static_cast<Seed*>(d_seeds);
  k_dxt1_seeds_chunks<<<seed_grid, kWarpsPerCta * 32, sizeof(SeedShared) * kWarpsPerCta, s>>>(d_blocks, d_chunks,
                                                                                           nchunks, d_segs, seeds);
  k_dxt1_encode_chunks<<<grid, kWarpsPerCta * 32, sizeof(WarpShared) * kWarpsPerCta, s>>>(d_blocks, d_chunks, nchunks,
                                                                                         d_segs, seeds);
  return cuda_check(cudaGetLastError(), "launch k_dxt1_seeds_chunks / k_dxt1_encode_chunks");
}

int launch_dxt5a_chunks(const uint8_t* d_blocks, const EncodeChunk* d_chunks, uint32_t nchunks,
                        const EncodeSegment* d_segs, int grid, cudaStream_t s) {
  if (!nchunks) return CRNGPU_OK;
  k_dxt5a_encode_chunks<<<grid, 128, 0, s>>>(d_blocks, d_chunks, nchunks, d_segs);
  return cuda_check(cudaGetLastError(), "launch k_dxt5a_encode_chunks");
}

// Test hook for the staging waits: polls per wait (drains are not affected).
int set_stage_wait_polls(uint32_t polls) {
  return cuda_check(cudaMemcpyToSymbol(g_stage_wait_polls, &polls, sizeof(polls)), "set stage wait polls");
}

// out[0]: staging waits that ran out, out[1]: drains that ran out; reset clears both.
int stage_wait_counters(uint32_t out[2], bool reset) {
  cudaError_t e = cudaMemcpyFromSymbol(&out[0], g_stage_timeouts, sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemcpyFromSymbol(&out[1], g_stage_drain_failures, sizeof(uint32_t));
  if (e == cudaSuccess && reset) {
    const uint32_t z = 0;
    e = cudaMemcpyToSymbol(g_stage_timeouts, &z, sizeof(z));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_stage_drain_failures, &z, sizeof(z));
  }
  return cuda_check(e, "read stage wait counters");
}

int launch_dxt5a(const uint8_t* d_blocks, uint32_t n, int comp, bool both, uint32_t quality, uint8_t* d_out,
                 uint32_t out_stride, cudaStream_t s) {
  if (!n) return CRNGPU_OK;
  if (quality > kQUber) { set_error("bad DXT quality"); return CRNGPU_E_PARAM; }
  const int grid = grid_for((const void*)k_dxt5a_encode, 128, (n + 3) / 4);
  k_dxt5a_encode<<<grid, 128, 0, s>>>(d_blocks, n, comp, both ? 1 : 0, quality, d_out, out_stride);
  return cuda_check(cudaGetLastError(), "launch k_dxt5a_encode");
}

}  // namespace crngpu

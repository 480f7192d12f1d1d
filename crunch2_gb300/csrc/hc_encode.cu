// Clustered ("hierarchical") DXT1 compression on the GPU: crnlib's dxt_hc
// (crnlib/crn_dxt_hc.cpp:97-316) restated as batched kernels.
//
//   k_hc_tiles        per 2x2-block chunk: the nine candidate tiles (four blocks, two 8x4, two 4x8,
//                     the 8x8 chunk) are compressed with the dxt_fast colour compressor and scored;
//                     of the eight tile layouts the best PSNR minus a per-layout derating wins
//                     (determine_tiles_task, :386-561); each chosen tile gets its two-colour
//                     "palette" vector (palettize_color, :318-351, a weighted 2-means split).
//   k_vq_split<D>     tree_clusterizer (crnlib/crn_tree_clusterizer.h:89-570): a node is split by
//                     furthest/opposite seeds, a 10-step power iteration for its principal axis and
//                     a 2-means loop. Instead of the reference's one-node-at-a-time priority queue,
//                     a round splits the top quarter of the leaves by variance at once, one CTA per
//                     node, until the codebook size is reached.
//   k_nearest_vec6    tile -> nearest endpoint codebook entry (determine_color_endpoint_clusters_task,
//                     :836-886).
//   k_cluster_fit     per endpoint cluster, over all pixels of its tiles: principal-axis start, least-
//                     squares refits from nearest-colour selectors, then the lattice walk of
//                     dxt_endpoint_refiner::optimize_dxt1 (crnlib/crn_dxt_endpoint_refiner.cpp:203-302)
//                     on histogram statistics (determine_color_endpoint_codebook_task, :663-754).
//   k_block_selectors per block: 2-bit linear selectors against its cluster's colours and the block
//                     weight of the selector codebook (:699-733).
//   k_vq_split<16>    the selector codebook (create_color_selector_codebook, :1379-1504).
//   k_selector_assign per block: the best codebook entry through the E2/E4/E8 error tables
//                     (create_color_selector_codebook_task, :1306-1360), accumulating per-entry
//                     error tables; k_selector_finalise re-optimises each entry from them.
//   k_hc_emit         the finished DXT1 blocks and per-block endpoint / selector indices.
// The ETC paths of dxt_hc are out of scope. The reference is not bit-reproducible here (its
// clusterizer result depends on the thread count), so this path is compared on quality.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>
#include <atomic>
#include <thread>

#include <cooperative_groups.h>
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_select.cuh>

#include "crngpu_internal.h"

namespace cg = cooperative_groups;

namespace crngpu {
namespace hc {

struct Level {
  uint32_t first_block, num_blocks, block_width;
  float weight;
};

// ------------------------------------------------------------------------------------------
// small helpers

__host__ __device__ __forceinline__ int exp5(int v) { return (v << 3) | (v >> 2); }
__host__ __device__ __forceinline__ int exp6(int v) { return (v << 2) | (v >> 4); }
__host__ __device__ __forceinline__ void unpack565(uint32_t c, int* o) {
  o[0] = exp5((c >> 11) & 31); o[1] = exp6((c >> 5) & 63); o[2] = exp5(c & 31);
}
__host__ __device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
__host__ __device__ __forceinline__ uint32_t px_r(uint32_t p) { return p & 255u; }
__host__ __device__ __forceinline__ uint32_t px_g(uint32_t p) { return (p >> 8) & 255u; }
__host__ __device__ __forceinline__ uint32_t px_b(uint32_t p) { return (p >> 16) & 255u; }

// color::color_distance (crnlib/crn_color.h:728-745) for RGB: weights 8/25/1 (perceptual) or 1/1/1.
__host__ __device__ __forceinline__ uint32_t cdist(bool perc, int r0, int g0, int b0, int r1, int g1, int b1) {
  const int dr = r0 - r1, dg = g0 - g1, db = b0 - b1;
  return perc ? (uint32_t)(dr * dr * 8 + dg * dg * 25 + db * db) : (uint32_t)(dr * dr + dg * dg + db * db);
}

// 4-colour palette of (first, second) in DXT order (dxt1_block::get_block_colors4,
// crnlib/crn_dxt.cpp:247-260): c0, c1, (2 c0 + c1) / 3, (c0 + 2 c1) / 3.
__host__ __device__ __forceinline__ void colors4(uint32_t c0, uint32_t c1, int (*c)[3]) {
  unpack565(c0, c[0]);
  unpack565(c1, c[1]);
  for (int k = 0; k < 3; k++) {
    c[2][k] = (c[0][k] * 2 + c[1][k]) / 3;
    c[3][k] = (c[1][k] * 2 + c[0][k]) / 3;
  }
}

// DXT order <-> linear order (g_dxt1_from_linear / g_dxt1_to_linear, crnlib/crn_dxt.cpp:38-39)
__constant__ uint8_t c_from_linear[4] = {0, 2, 3, 1};
__constant__ uint8_t c_to_linear[4] = {0, 3, 1, 2};

// ------------------------------------------------------------------------------------------
// dxt_fast colour compressor (crnlib/crn_dxt_fast.cpp:30-764), restated for n pixels (n = 16, 32
// or 64) held in registers/local memory as packed RGBA8 words.

struct SolidTables { uint8_t m5[256][2], m6[256][2]; };

__host__ __device__ __forceinline__ int mul_8bit(int a, int b) {
  const int t = a * b + 128;
  return (t + (t >> 8)) >> 8;
}
__host__ __device__ __forceinline__ uint32_t fast_pack(int r, int g, int b) {
  return (uint32_t)((mul_8bit(r, 31) << 11) + (mul_8bit(g, 63) << 5) + mul_8bit(b, 31));
}

// eval_colors (:76-96): color[0] = c0, color[1] = c1, color[2] = (2 c0 + c1) / 3, color[3] = (2 c1 + c0) / 3
__host__ __device__ __forceinline__ void fast_eval(uint32_t c0, uint32_t c1, int (*col)[3]) { colors4(c0, c1, col); }

// match_block_colors (:99-148); false if all selectors are equal
__host__ __device__ bool fast_match(int n, const uint32_t* px, int (*col)[3], uint8_t* sel) {
  const int dirr = col[0][0] - col[1][0], dirg = col[0][1] - col[1][1], dirb = col[0][2] - col[1][2];
  int stops[4];
  for (int i = 0; i < 4; i++) stops[i] = col[i][0] * dirr + col[i][1] * dirg + col[i][2] * dirb;
  const int c0Point = (stops[1] + stops[3]) >> 1, halfPoint = (stops[3] + stops[2]) >> 1,
            c3Point = (stops[2] + stops[0]) >> 1;
  bool status = false;
  for (int i = 0; i < n; i++) {
    const int dot = (int)px_r(px[i]) * dirr + (int)px_g(px[i]) * dirg + (int)px_b(px[i]) * dirb;
    uint8_t s;
    if (dot < halfPoint) s = (dot < c0Point) ? 1 : 3;
    else s = (dot < c3Point) ? 2 : 0;
    sel[i] = s;
    if (s != sel[0]) status = true;
  }
  return status;
}

// optimize_block_colors (:151-286): principal axis by power iteration, extreme pixels along it
__host__ __device__ bool fast_optimize(int n, const uint32_t* px, uint32_t& max16, uint32_t& min16, int* ave) {
  int mn[3], mx[3];
  for (int ch = 0; ch < 3; ch++) {
    long long mu = 0;
    int lo = 255, hi = 0;
    for (int i = 0; i < n; i++) {
      const int v = (px[i] >> (8 * ch)) & 255;
      mu += v;
      lo = lo < v ? lo : v;
      hi = hi > v ? hi : v;
    }
    ave[ch] = (int)((mu + (n / 2)) / n);
    mn[ch] = lo;
    mx[ch] = hi;
  }
  if (mn[0] == mx[0] && mn[1] == mx[1] && mn[2] == mx[2]) return false;
  double cov[6] = {0, 0, 0, 0, 0, 0};
  for (int i = 0; i < n; i++) {
    const double r = (int)px_r(px[i]) - ave[0], g = (int)px_g(px[i]) - ave[1], b = (int)px_b(px[i]) - ave[2];
    cov[0] += r * r; cov[1] += r * g; cov[2] += r * b; cov[3] += g * g; cov[4] += g * b; cov[5] += b * b;
  }
  double covf[6];
  for (int i = 0; i < 6; i++) covf[i] = cov[i] * (double)(1.0f / 255.0f);
  double vfr = mx[0] - mn[0], vfg = mx[1] - mn[1], vfb = mx[2] - mn[2];
  for (int it = 0; it < 4; it++) {
    const double r = vfr * covf[0] + vfg * covf[1] + vfb * covf[2];
    const double g = vfr * covf[1] + vfg * covf[3] + vfb * covf[4];
    const double b = vfr * covf[2] + vfg * covf[4] + vfb * covf[5];
    vfr = r; vfg = g; vfb = b;
  }
  double magn = fmax(fmax(fabs(vfr), fabs(vfg)), fabs(vfb));
  int v_r, v_g, v_b;
  if (magn < 4.0) {
    v_r = 148; v_g = 300; v_b = 58;
  } else {
    magn = 512.0 / magn;
    v_r = (int)(vfr * magn); v_g = (int)(vfg * magn); v_b = (int)(vfb * magn);
  }
  int mind = (int)px_r(px[0]) * v_r + (int)px_g(px[0]) * v_g + (int)px_b(px[0]) * v_b, maxd = mind;
  uint32_t minp = px[0], maxp = px[0];
  for (int i = 1; i < n; i++) {
    const int dot = (int)px_r(px[i]) * v_r + (int)px_g(px[i]) * v_g + (int)px_b(px[i]) * v_b;
    if (dot < mind) { mind = dot; minp = px[i]; }
    if (dot > maxd) { maxd = dot; maxp = px[i]; }
  }
  max16 = fast_pack(px_r(maxp), px_g(maxp), px_b(maxp));
  min16 = fast_pack(px_r(minp), px_g(minp), px_b(minp));
  return true;
}

// refine_block (:288-335): least-squares endpoints from the selectors (Cramer's rule)
__host__ __device__ bool fast_refine(int n, const uint32_t* px, uint32_t& max16, uint32_t& min16, const uint8_t* sel) {
  const int w1Tab[4] = {3, 0, 2, 1};
  const int prods_0[4] = {0x00, 0x00, 0x02, 0x02};
  const int prods_1[4] = {0x00, 0x09, 0x01, 0x04};
  const int prods_2[4] = {0x09, 0x00, 0x04, 0x01};
  double akku_0 = 0, akku_1 = 0, akku_2 = 0;
  double At1_r = 0, At1_g = 0, At1_b = 0, At2_r = 0, At2_g = 0, At2_b = 0;
  for (int i = 0; i < n; i++) {
    const double r = px_r(px[i]), g = px_g(px[i]), b = px_b(px[i]);
    const int step = sel[i], w1 = w1Tab[step];
    akku_0 += prods_0[step]; akku_1 += prods_1[step]; akku_2 += prods_2[step];
    At1_r += w1 * r; At1_g += w1 * g; At1_b += w1 * b;
    At2_r += r; At2_g += g; At2_b += b;
  }
  At2_r = 3 * At2_r - At1_r; At2_g = 3 * At2_g - At1_g; At2_b = 3 * At2_b - At1_b;
  const double xx = akku_2, yy = akku_1, xy = akku_0;
  const double t = xx * yy - xy * xy;
  if (!yy || !xx || (fabs(t) < (double)0.0000125f)) return false;
  const double frb = (double)(3.0f * 31.0f / 255.0f) / t;
  const double fg = frb * (double)(63.0f / 31.0f);
  const uint32_t oldMin = min16, oldMax = max16;
  max16 = (uint32_t)clampi((int)((At1_r * yy - At2_r * xy) * frb + (double)0.5f), 0, 31) << 11;
  max16 |= (uint32_t)clampi((int)((At1_g * yy - At2_g * xy) * fg + (double)0.5f), 0, 63) << 5;
  max16 |= (uint32_t)clampi((int)((At1_b * yy - At2_b * xy) * frb + (double)0.5f), 0, 31);
  min16 = (uint32_t)clampi((int)((At2_r * xx - At1_r * xy) * frb + (double)0.5f), 0, 31) << 11;
  min16 |= (uint32_t)clampi((int)((At2_g * xx - At1_g * xy) * fg + (double)0.5f), 0, 63) << 5;
  min16 |= (uint32_t)clampi((int)((At2_b * xx - At1_b * xy) * frb + (double)0.5f), 0, 31);
  return (oldMin != min16) || (oldMax != max16);
}

// compress_color_block (:725-764, refine = false) and the squared RGB error of the result against
// get_block_colors4 (crn_dxt_hc.cpp:459-472)
__host__ __device__ void fast_compress(int n, const uint32_t* px, const SolidTables* __restrict__ st, uint32_t& lo16,
                                       uint32_t& hi16, uint8_t* sel) {
  int ave[3];
  bool solid = false;
  if (!fast_optimize(n, px, lo16, hi16, ave)) {
    solid = true;
  } else {
    int col[4][3];
    if (lo16 == hi16) {
      for (int i = 0; i < n; i++) sel[i] = 0;
      solid = true;
    } else {
      fast_eval(lo16, hi16, col);
      if (!fast_match(n, px, col, sel)) {
        solid = true;
      } else if (fast_refine(n, px, lo16, hi16, sel)) {
        if (lo16 != hi16) {
          fast_eval(lo16, hi16, col);
          fast_match(n, px, col, sel);
        } else {
          for (int i = 0; i < n; i++) sel[i] = 0;
        }
      }
    }
  }
  if (solid) {
    // compress_solid_block (:712-723): ryg optimal single-colour endpoints, selectors 2
    lo16 = ((uint32_t)st->m5[ave[0]][0] << 11) | ((uint32_t)st->m6[ave[1]][0] << 5) | st->m5[ave[2]][0];
    hi16 = ((uint32_t)st->m5[ave[0]][1] << 11) | ((uint32_t)st->m6[ave[1]][1] << 5) | st->m5[ave[2]][1];
    for (int i = 0; i < n; i++) sel[i] = 2;
  }
  if (lo16 < hi16) {
    const uint32_t t = lo16; lo16 = hi16; hi16 = t;
    for (int i = 0; i < n; i++) sel[i] ^= 1;
  }
}

__host__ __device__ uint32_t fast_tile_error(int n, const uint32_t* px, const SolidTables* __restrict__ st) {
  uint8_t sel[64];
  uint32_t lo16, hi16;
  fast_compress(n, px, st, lo16, hi16, sel);
  int col[4][3];
  colors4(lo16, hi16, col);
  uint32_t err = 0;
  for (int i = 0; i < n; i++) {
    const int* c = col[sel[i]];
    const int dr = (int)px_r(px[i]) - c[0], dg = (int)px_g(px[i]) - c[1], db = (int)px_b(px[i]) - c[2];
    err += (uint32_t)(dr * dr + dg * dg + db * db);
  }
  return err;
}

// dxt_fast::find_representative_colors (crnlib/crn_dxt_fast.cpp:855-994): the rounded mean, the
// pixel furthest from it and the one furthest from that, both pulled halfway to the mean, then up to
// four 2-means refinements along their axis; the darker colour first.
__host__ __device__ void find_rep_colors(int n, const uint32_t* px, int* lo, int* hi) {
  uint64_t s64[3] = {0, 0, 0};
  for (int i = 0; i < n; i++) { s64[0] += px_r(px[i]); s64[1] += px_g(px[i]); s64[2] += px_b(px[i]); }
  int ave[3];
  for (int c = 0; c < 3; c++) ave[c] = (int)((s64[c] + (uint64_t)(n / 2)) / (uint64_t)n);
  auto comp = [&](int i, int c) { return c == 0 ? (int)px_r(px[i]) : c == 1 ? (int)px_g(px[i]) : (int)px_b(px[i]); };
  int fd = -1, fi = 0;
  for (int i = 0; i < n; i++) {
    const int r = comp(i, 0) - ave[0], g = comp(i, 1) - ave[1], b = comp(i, 2) - ave[2];
    const int d = r * r + g * g + b * b;
    if (d > fd) { fd = d; fi = i; }
  }
  int l[3] = {comp(fi, 0), comp(fi, 1), comp(fi, 2)};
  int od = -1, oi = 0;
  for (int i = 0; i < n; i++) {
    const int r = comp(i, 0) - l[0], g = comp(i, 1) - l[1], b = comp(i, 2) - l[2];
    const int d = r * r + g * g + b * b;
    if (d > od) { od = d; oi = i; }
  }
  int h[3] = {comp(oi, 0), comp(oi, 1), comp(oi, 2)};
  for (int c = 0; c < 3; c++) { l[c] = (l[c] + ave[c]) >> 1; h[c] = (h[c] + ave[c]) >> 1; }
  for (int iter = 0; iter < 4; iter++) {
    if (l[0] == h[0] && l[1] == h[1] && l[2] == h[2]) break;
    uint64_t nc[2][3] = {{0, 0, 0}, {0, 0, 0}};
    uint32_t w[2] = {0, 0};
    int vr = h[0] - l[0], vg = h[1] - l[1], vb = h[2] - l[2];
    const int lo_dot = vr * l[0] + vg * l[1] + vb * l[2], hi_dot = vr * h[0] + vg * h[1] + vb * h[2];
    const int mid = lo_dot + hi_dot;
    vr *= 2; vg *= 2; vb *= 2;
    for (int i = 0; i < n; i++) {
      const int dot = comp(i, 0) * vr + comp(i, 1) * vg + comp(i, 2) * vb;
      const int m = dot > mid ? 1 : 0;
      for (int c = 0; c < 3; c++) nc[m][c] += (uint64_t)comp(i, c);
      w[m]++;
    }
    if (!w[0] || !w[1]) break;
    int n8[2][3];
    for (int j = 0; j < 2; j++)
      for (int c = 0; c < 3; c++) n8[j][c] = (int)(uint8_t)((nc[j][c] + (w[j] / 2)) / w[j]);
    if (n8[0][0] == l[0] && n8[0][1] == l[1] && n8[0][2] == l[2] && n8[1][0] == h[0] && n8[1][1] == h[1] &&
        n8[1][2] == h[2])
      break;
    for (int c = 0; c < 3; c++) { l[c] = n8[0][c]; h[c] = n8[1][c]; }
  }
  const int e0 = l[0] * l[0] + l[1] * l[1] + l[2] * l[2], e1 = h[0] * h[0] + h[1] * h[1] + h[2] * h[2];
  for (int c = 0; c < 3; c++) {
    lo[c] = e0 > e1 ? h[c] : l[c];
    hi[c] = e0 > e1 ? l[c] : h[c];
  }
}

// ------------------------------------------------------------------------------------------
// split_vectors (crnlib/crn_tree_clusterizer.h:573-753) for up to 64 weighted vec3: the two
// centroids of a 2-means split seeded by furthest/opposite points and the principal axis.
__host__ __device__ void split_vec3(const float (*v)[3], const uint32_t* w, int size, float* res) {
  float cen[3] = {0, 0, 0};
  double ttsum = 0;
  uint64_t tw = 0;
  for (int i = 0; i < size; i++) {
    for (int k = 0; k < 3; k++) cen[k] += v[i][k] * (float)w[i];
    tw += w[i];
    ttsum += (double)(v[i][0] * v[i][0] + v[i][1] * v[i][1] + v[i][2] * v[i][2]) * w[i];
  }
  const float variance = (float)(ttsum - (double)(cen[0] * cen[0] + cen[1] * cen[1] + cen[2] * cen[2]) / (double)tw);
  for (int k = 0; k < 3; k++) cen[k] *= 1.0f / (float)tw;
  for (int k = 0; k < 3; k++) res[k] = res[3 + k] = cen[k];
  if (variance <= 0.0f || size == 1) return;
  auto d2 = [](const float* a, const float* b) {
    const float x = a[0] - b[0], y = a[1] - b[1], z = a[2] - b[2];
    return x * x + y * y + z * z;
  };
  int fi = 0, oi = 0;
  float fd = -1.0f, od = -1.0f;
  for (int i = 0; i < size; i++) { const float d = d2(v[i], cen); if (d > fd) { fd = d; fi = i; } }
  for (int i = 0; i < size; i++) { const float d = d2(v[i], v[fi]); if (d > od) { od = d; oi = i; } }
  float L[3], R[3];
  for (int k = 0; k < 3; k++) { L[k] = (v[fi][k] + cen[k]) * 0.5f; R[k] = (v[oi][k] + cen[k]) * 0.5f; }
  if (size > 2) {
    float cov[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int i = 0; i < size; i++) {
      const float d[3] = {v[i][0] - cen[0], v[i][1] - cen[1], v[i][2] - cen[2]};
      for (int x = 0; x < 3; x++)
        for (int y = x; y < 3; y++) cov[x][y] += d[x] * d[y] * (float)w[i];
    }
    for (int x = 0; x < 3; x++)
      for (int y = x; y < 3; y++) { cov[x][y] /= (float)tw; cov[y][x] = cov[x][y]; }
    float axis[3] = {1, 1, 1};
    for (int it = 0; it < 10; it++) {
      float x[3];
      double max_sum = 0;
      for (int i = 0; i < 3; i++) {
        double sum = 0;
        for (int j = 0; j < 3; j++) sum += axis[j] * cov[i][j];
        x[i] = (float)sum;
        max_sum = i ? fmax(max_sum, sum) : sum;
      }
      if (max_sum != 0.0) for (int i = 0; i < 3; i++) x[i] *= (float)(1.0 / max_sum);
      for (int i = 0; i < 3; i++) axis[i] = x[i];
    }
    const float len = sqrtf(axis[0] * axis[0] + axis[1] * axis[1] + axis[2] * axis[2]);
    if (len > 0) for (int i = 0; i < 3; i++) axis[i] /= len;
    float nl[3] = {0, 0, 0}, nr[3] = {0, 0, 0};
    double lw = 0, rw = 0;
    for (int i = 0; i < size; i++) {
      const double t = (double)((v[i][0] - cen[0]) * axis[0] + (v[i][1] - cen[1]) * axis[1] + (v[i][2] - cen[2]) * axis[2]);
      if (t < 0.0) { for (int k = 0; k < 3; k++) nl[k] += v[i][k] * (float)w[i]; lw += w[i]; }
      else { for (int k = 0; k < 3; k++) nr[k] += v[i][k] * (float)w[i]; rw += w[i]; }
    }
    if (lw > 0 && rw > 0)
      for (int k = 0; k < 3; k++) { L[k] = nl[k] * (float)(1.0 / lw); R[k] = nr[k] * (float)(1.0 / rw); }
  }
  float prev = 1e10f;
  for (int loop = 0; loop < 1024; loop++) {
    float nl[3] = {0, 0, 0}, nr[3] = {0, 0, 0};
    double lt = 0, rt = 0;
    uint64_t lw = 0, rw = 0;
    for (int i = 0; i < size; i++) {
      const float vv = (float)(v[i][0] * v[i][0] + v[i][1] * v[i][1] + v[i][2] * v[i][2]) * (float)w[i];
      if (d2(L, v[i]) < d2(R, v[i])) { for (int k = 0; k < 3; k++) nl[k] += v[i][k] * (float)w[i]; lt += vv; lw += w[i]; }
      else { for (int k = 0; k < 3; k++) nr[k] += v[i][k] * (float)w[i]; rt += vv; rw += w[i]; }
    }
    if (!lw || !rw) return;  // result stays at the centroid
    const float lv = (float)(lt - (double)(nl[0] * nl[0] + nl[1] * nl[1] + nl[2] * nl[2]) / (double)lw);
    const float rv = (float)(rt - (double)(nr[0] * nr[0] + nr[1] * nr[1] + nr[2] * nr[2]) / (double)rw);
    for (int k = 0; k < 3; k++) { L[k] = nl[k] * (1.0f / (float)lw); R[k] = nr[k] * (1.0f / (float)rw); }
    const float tv = lv + rv;
    if (tv < .00001f) break;
    if ((prev - tv) / tv < .00001f) break;
    prev = tv;
  }
  for (int k = 0; k < 3; k++) { res[k] = L[k]; res[3 + k] = R[k]; }
}

// ------------------------------------------------------------------------------------------
// Tiles: one thread per 2x2-block chunk.

// tile t of a chunk: offset into the 128-pixel chunk image and size (crn_dxt_hc.cpp:389-390)
#define HC_TILE_OFS {0, 16, 32, 48, 0, 32, 64, 96, 64}
// tiles of each layout, in layout order (crn_dxt_hc.cpp:390)
#define HC_LAYOUT_TILES {{8, 0, 0, 0}, {6, 7, 0, 0}, {4, 5, 0, 0}, {6, 1, 3, 0}, {7, 0, 2, 0}, {4, 2, 3, 0}, {5, 0, 1, 0}, {0, 2, 1, 3}}
#define HC_LAYOUT_NTILES {1, 2, 2, 3, 3, 3, 3, 4}
// tile (within the layout) covering each block of the chunk, [layout][by][bx] (g_tile_map, :36-45)
#define HC_TILE_MAP {{{0, 0}, {0, 0}}, {{0, 0}, {1, 1}}, {{0, 1}, {0, 1}}, {{0, 0}, {1, 2}}, \
                     {{1, 2}, {0, 0}}, {{0, 1}, {0, 2}}, {{1, 0}, {2, 0}}, {{0, 1}, {2, 3}}}
__constant__ uint8_t c_tile_ofs[9] = HC_TILE_OFS;

struct Chunk {
  uint32_t b;      // first (top-left) block
  uint32_t width;  // block width of the level
  uint32_t level;
};

// Tile record: the chunk it belongs to, which of the nine tiles it is, its weight and vec6.
struct Tile {
  uint32_t chunk;  // chunk index (chunk b = chunks[chunk].b)
  uint32_t kind;   // 0..8 (tile within the chunk image), 0xFF: unused slot
  float weight;    // pixels x level weight
  float v[6];      // palettize_color result
  float va[2][2];  // palettize_alpha result per alpha channel (low <= high)
};

// Which channels the clustered format carries (dxt_hc::compress, crn_dxt_hc.cpp:104-118).
struct TileCfg {
  int has_color;        // DXT1, DXT5
  int num_alpha;        // 0 (DXT1), 1 (DXT5, DXT5A), 2 (DXN)
  int comp[2];          // m_alpha_component_indices
  float ratio;          // m_adaptive_tile_color_alpha_weighting_ratio
  float alpha_derating[8];
  int qdxt;             // qdxt1::init's tiling (crnlib/crn_qdxt1.cpp:100-330) instead of dxt_hc's
};

// dxt_fast::compress_alpha_block (crnlib/crn_dxt_fast.cpp:788-826): endpoints max / min of the
// channel, selectors from the scaled distance to the minimum in three compare-and-subtract steps;
// returns the squared error against dxt5_block::get_block_values of (max, min), the tile error of
// qdxt5::init (crnlib/crn_qdxt5.cpp:180-200). sel48 (optional) gets the 16 3-bit selectors.
__host__ __device__ uint32_t fast_alpha_error(int n, const uint32_t* px, int comp, uint64_t* sel48 = nullptr) {
  auto chan = [&](int i) { return (int)((px[i] >> (8 * comp)) & 255u); };
  int mn = chan(0), mx = mn;
  for (int i = 1; i < n; i++) { mn = min(mn, chan(i)); mx = max(mx, chan(i)); }
  const int l = mx, h = mn;
  int c[8];
  c[0] = l; c[1] = h;
  if (l > h) {
    for (int k = 1; k <= 6; k++) c[1 + k] = (l * (7 - k) + h * k) / 7;
  } else {
    for (int k = 1; k <= 4; k++) c[1 + k] = (l * (5 - k) + h * k) / 5;
    c[6] = 0; c[7] = 255;
  }
  const int dist = mx - mn, bias = mn * 7 - (dist >> 1), dist4 = dist * 4, dist2 = dist * 2;
  uint32_t err = 0;
  uint64_t bits = 0;
  for (int i = 0; i < n; i++) {
    int a = chan(i) * 7 - bias, ind, t;
    t = (dist4 - a) >> 31; ind = t & 4; a -= dist4 & t;
    t = (dist2 - a) >> 31; ind += t & 2; a -= dist2 & t;
    t = (dist - a) >> 31; ind += t & 1;
    ind = -ind & 7;
    ind ^= (2 > ind) ? 1 : 0;
    const int d = chan(i) - c[ind];
    err += (uint32_t)(d * d);
    if (i < 16) bits |= (uint64_t)ind << (3 * i);
  }
  if (sel48) *sel48 = bits;
  return err;
}

// dxt5_endpoint_optimizer::compute at quality Normal with 8-value blocks only, for the tile
// decision (crn_dxt_hc.cpp:475-490): the smallest error over all pairs of the tile's unique
// values (crnlib/crn_dxt5a.cpp:40-100, 198-262).
__host__ __device__ uint32_t alpha_tile_error(int n, const uint32_t* px, int comp) {
  uint8_t uv[64];
  uint32_t uw[64];
  int U = 0;
  for (int i = 0; i < n; i++) {
    const uint8_t a = (uint8_t)((px[i] >> (8 * comp)) & 255u);
    int k = 0;
    while (k < U && uv[k] != a) k++;
    if (k == U) { uv[U] = a; uw[U] = 0; U++; }
    uw[k]++;
  }
  if (U == 1) return 0;
  unsigned long long best = ~0ull;
  for (int i = 0; i < U - 1; i++) {
    for (int j = i + 1; j < U; j++) {
      const int l = uv[i], h = uv[j];
      const int v[8] = {l, h, (l * 6 + h) / 7, (l * 5 + h * 2) / 7, (l * 4 + h * 3) / 7, (l * 3 + h * 4) / 7,
                        (l * 2 + h * 5) / 7, (l + h * 6) / 7};
      unsigned long long e = 0;
      for (int u = 0; u < U && e <= best; u++) {
        int bd = 0x7FFFFFFF;
        for (int k = 0; k < 8; k++) {
          const int d = (int)uv[u] - v[k];
          bd = min(bd, d * d);
        }
        e += (unsigned long long)bd * uw[u];
      }
      if (e < best) best = e;
    }
  }
  return (uint32_t)best;
}

// split_vectors<vec1F> (crn_tree_clusterizer.h:573-753) for up to 64 weighted values: the two
// centroids of a 1-D 2-means split seeded by the furthest/opposite values.
__host__ __device__ void split_vec1(const float* v, const uint32_t* w, int size, float* res) {
  float cen = 0.f;
  double ttsum = 0;
  uint64_t tw = 0;
  for (int i = 0; i < size; i++) { cen += v[i] * (float)w[i]; tw += w[i]; ttsum += (double)(v[i] * v[i]) * w[i]; }
  const float variance = (float)(ttsum - (double)(cen * cen) / (double)tw);
  cen *= 1.0f / (float)tw;
  res[0] = res[1] = cen;
  if (variance <= 0.0f || size == 1) return;
  int fi = 0, oi = 0;
  float fd = -1.f, od = -1.f;
  for (int i = 0; i < size; i++) { const float d = (v[i] - cen) * (v[i] - cen); if (d > fd) { fd = d; fi = i; } }
  for (int i = 0; i < size; i++) { const float d = (v[i] - v[fi]) * (v[i] - v[fi]); if (d > od) { od = d; oi = i; } }
  float L = (v[fi] + cen) * .5f, R = (v[oi] + cen) * .5f;
  if (size > 2) {
    // the 1-D principal axis is +1: split at the centroid
    float nl = 0.f, nr = 0.f;
    double lw = 0, rw = 0;
    for (int i = 0; i < size; i++) {
      if ((double)(v[i] - cen) < 0.0) { nl += v[i] * (float)w[i]; lw += w[i]; }
      else { nr += v[i] * (float)w[i]; rw += w[i]; }
    }
    if (lw > 0 && rw > 0) { L = nl * (float)(1.0 / lw); R = nr * (float)(1.0 / rw); }
  }
  float prev = 1e10f;
  for (int loop = 0; loop < 1024; loop++) {
    float nl = 0.f, nr = 0.f;
    double lt = 0, rt = 0;
    uint64_t lw = 0, rw = 0;
    for (int i = 0; i < size; i++) {
      const float vv = v[i] * v[i] * (float)w[i];
      if ((L - v[i]) * (L - v[i]) < (R - v[i]) * (R - v[i])) { nl += v[i] * (float)w[i]; lt += vv; lw += w[i]; }
      else { nr += v[i] * (float)w[i]; rt += vv; rw += w[i]; }
    }
    if (!lw || !rw) return;
    const float lv = (float)(lt - (double)(nl * nl) / (double)lw), rv = (float)(rt - (double)(nr * nr) / (double)rw);
    L = nl * (1.0f / (float)lw);
    R = nr * (1.0f / (float)rw);
    const float tv = lv + rv;
    if (tv < .00001f) break;
    if ((prev - tv) / tv < .00001f) break;
    prev = tv;
  }
  res[0] = L;
  res[1] = R;
}

// palettize_alpha (crn_dxt_hc.cpp:353-384): the tile's values of one channel split in two, sorted
__host__ __device__ void palettize_alpha(const uint32_t* px, int n, int comp, float* out2) {
  uint8_t a[64];
  for (int i = 0; i < n; i++) a[i] = (uint8_t)((px[i] >> (8 * comp)) & 255u);
  for (int i = 1; i < n; i++) {
    const uint8_t x = a[i];
    int j = i - 1;
    while (j >= 0 && a[j] > x) { a[j + 1] = a[j]; j--; }
    a[j + 1] = x;
  }
  float v[64];
  uint32_t w[64];
  int size = 0;
  for (int i = 0; i < n; i++) {
    if (!i || a[i] != a[i - 1]) { v[size] = (float)a[i] * (1.0f / 255.0f); w[size] = 1; size++; }
    else w[size - 1]++;
  }
  float r[2];
  split_vec1(v, w, size, r);
  if (r[0] > r[1]) { const float t = r[0]; r[0] = r[1]; r[1] = t; }
  out2[0] = r[0];
  out2[1] = r[1];
}

__host__ __device__ __forceinline__ uint32_t ld_px(const uint32_t* p) {
#ifdef __CUDA_ARCH__
  return __ldg(p);
#else
  return *p;
#endif
}

__host__ __device__ __forceinline__ void chunk_pixels(const uint32_t* __restrict__ blocks, uint32_t b, uint32_t width,
                                                      uint32_t* px /* 128 */) {
  const uint32_t bl[4] = {b, b + width, b + 1, b + width + 1};  // [0..63]: TL, BL, TR, BR blocks
  for (int q = 0; q < 4; q++)
    for (int i = 0; i < 16; i++) px[q * 16 + i] = ld_px(blocks + (size_t)bl[q] * 16 + i);
  // [64..127]: top 8x4 then bottom 8x4, row-major (t & 32: lower blocks, t & 4: right block)
  for (int t = 0; t < 64; t += 4) {
    const uint32_t blk = b + ((t & 32) ? width : 0) + ((t & 4) ? 1 : 0);
    const int row = (t >> 1) & 12;
    for (int i = 0; i < 4; i++) px[64 + t + i] = ld_px(blocks + (size_t)blk * 16 + row + i);
  }
}

// palettize_color (crn_dxt_hc.cpp:318-351): unique colours (perceptual: r * 0.5, b * 0.25) split in two
__host__ __device__ void palettize(const uint32_t* px, int n, bool perc, float* out6) {
  uint32_t col[64];
  for (int i = 0; i < n; i++) col[i] = (px_r(px[i]) << 16) | (px_g(px[i]) << 8) | px_b(px[i]);
  for (int i = 1; i < n; i++) {  // insertion sort (n <= 64)
    const uint32_t x = col[i];
    int j = i - 1;
    while (j >= 0 && col[j] > x) { col[j + 1] = col[j]; j--; }
    col[j + 1] = x;
  }
  float v[64][3];
  uint32_t w[64];
  int size = 0;
  for (int i = 0; i < n; i++) {
    if (!i || col[i] != col[i - 1]) {
      const float r = (float)(col[i] >> 16) * (1.0f / 255.0f), g = (float)((col[i] >> 8) & 255) * (1.0f / 255.0f),
                  b = (float)(col[i] & 255) * (1.0f / 255.0f);
      v[size][0] = perc ? r * 0.5f : r;
      v[size][1] = g;
      v[size][2] = perc ? b * 0.25f : b;
      w[size] = 1;
      size++;
    } else {
      w[size - 1]++;
    }
  }
  float res[6];
  split_vec3(v, w, size, res);
  const float l0 = res[0] * res[0] + res[1] * res[1] + res[2] * res[2];
  const float l1 = res[3] * res[3] + res[4] * res[4] + res[5] * res[5];
  if (sqrtf(l0) > sqrtf(l1)) {
    for (int k = 0; k < 3; k++) { const float t = res[k]; res[k] = res[3 + k]; res[3 + k] = t; }
  }
  for (int k = 0; k < 6; k++) out6[k] = res[k];
}

// One chunk of determine_tiles_task (crn_dxt_hc.cpp:386-561): tile errors, layout choice, the
// chosen tiles' colour vec6 / alpha vec2, and each block's tile slot and layout. Returns the layout.
__host__ __device__ int hc_tile_chunk(const uint32_t* __restrict__ blocks, uint32_t c, const Chunk& ch,
                                      const float* __restrict__ derating, const float* __restrict__ level_weight,
                                      bool perceptual, const SolidTables* __restrict__ st, const TileCfg& cfg,
                                      Tile* __restrict__ tiles, uint32_t* __restrict__ block_tile,
                                      uint8_t* __restrict__ block_enc) {
  const uint8_t tile_ofs[9] = HC_TILE_OFS;
  const uint8_t layout_tiles[8][4] = HC_LAYOUT_TILES;
  const uint8_t layout_ntiles[8] = HC_LAYOUT_NTILES;
  const uint8_t tile_map[8][2][2] = HC_TILE_MAP;
  uint32_t px[128];
  chunk_pixels(blocks, ch.b, ch.width, px);
  uint32_t terr[3][9];
  for (int t = 0; t < 9; t++) {
    const int n = 16 << (t >> 2);
    if (cfg.has_color) terr[0][t] = fast_tile_error(n, px + tile_ofs[t], st);
    for (int a = 0; a < cfg.num_alpha; a++)
      terr[1 + a][t] = cfg.qdxt ? fast_alpha_error(n, px + tile_ofs[t], cfg.comp[a])
                                : alpha_tile_error(n, px + tile_ofs[t], cfg.comp[a]);
  }
  float best_q = 0.0f;
  int best_e = 0;
  if (cfg.qdxt && !cfg.has_color) {
    // qdxt5::init (crnlib/crn_qdxt5.cpp:202-240): the same choice over the channel's 64 values
    double best = -1.0;
    for (int e = 0; e < 8; e++) {
      uint32_t tot = 0;
      for (int k = 0; k < layout_ntiles[e]; k++) tot += terr[1][layout_tiles[e][k]];
      const double ms = tot * (1.0f / 64.0f);
      double psnr = 999999.0f;
      if (ms) psnr = fmin(fmax(log10(255.0f / sqrt(ms)) * 20.0f, 0.0), 500.0);
      psnr = psnr - (double)derating[ch.level * 8 + e];
      if (psnr > best) { best = psnr; best_e = e; }
    }
  } else if (cfg.qdxt) {
    // qdxt1::init: PSNR clamped to [0, 500] (999999 for no error) minus the layout's derating,
    // the largest wins
    double best = -1.0;
    for (int e = 0; e < 8; e++) {
      uint32_t tot = 0;
      for (int k = 0; k < layout_ntiles[e]; k++) tot += terr[0][layout_tiles[e][k]];
      const double ms = tot * (1.0f / (64.0f * 3.0f));
      double psnr = 999999.0f;
      if (ms) psnr = fmin(fmax(log10(255.0f / sqrt(ms)) * 20.0f, 0.0), 500.0);
      psnr = psnr - (double)derating[ch.level * 8 + e];
      if (psnr > best) { best = psnr; best_e = e; }
    }
  }
  for (int e = 0; e < 8 && !cfg.qdxt; e++) {
    float q = 0.0f;
    if (cfg.has_color) {
      uint32_t tot = 0;
      for (int k = 0; k < layout_ntiles[e]; k++) tot += terr[0][layout_tiles[e][k]];
      const double psnr = tot ? log10((double)255.0f / sqrt(tot / 192.0)) * (double)20.0f : (double)999999.0f;
      q = (float)fmax(psnr - (double)derating[ch.level * 8 + e], 0.0);
      if (cfg.num_alpha) q *= cfg.ratio;
    }
    for (int a = 0; a < cfg.num_alpha; a++) {
      uint32_t tot = 0;
      for (int k = 0; k < layout_ntiles[e]; k++) tot += terr[1 + a][layout_tiles[e][k]];
      const double psnr = tot ? log10((double)255.0f / sqrt(tot / 64.0)) * (double)20.0f : (double)999999.0f;
      q += (float)fmax(psnr - (double)cfg.alpha_derating[e], 0.0);
    }
    if (q > best_q) { best_q = q; best_e = e; }
  }
  const float lw = level_weight[ch.level];
  for (int k = 0; k < 4; k++) {
    Tile& T = tiles[4 * c + k];
    if (k >= layout_ntiles[best_e]) { T.kind = 0xFFu; T.chunk = c; T.weight = 0; continue; }
    const int t = layout_tiles[best_e][k];
    const int n = 16 << (t >> 2);
    T.chunk = c;
    T.kind = (uint32_t)t;
    T.weight = (float)n * lw;
    if (cfg.qdxt && !cfg.has_color) {
      // qdxt5: the representative pair of the channel's values (as grey pixels), weighted by the
      // squared distance / 8, 1..8
      uint32_t grey[64];
      for (int i = 0; i < n; i++) grey[i] = ((px[tile_ofs[t] + i] >> (8 * cfg.comp[0])) & 255u) * 0x010101u;
      int lo[3], hi[3];
      find_rep_colors(n, grey, lo, hi);
      const uint32_t dist = (uint32_t)((lo[0] - hi[0]) * (lo[0] - hi[0]));
      const uint32_t w = dist / 8u < 1u ? 1u : dist / 8u > 8u ? 8u : dist / 8u;
      T.va[0][0] = (float)lo[0];
      T.va[0][1] = (float)hi[0];
      T.weight = (float)(w * (uint32_t)(n / 16));
      continue;
    }
    if (cfg.qdxt) {
      // representative colours as the training vector of each of the tile's blocks, weighted by
      // their distance (squared RGB / 5000, 1..8)
      int lo[3], hi[3];
      find_rep_colors(n, px + tile_ofs[t], lo, hi);
      const int d0 = lo[0] - hi[0], d1 = lo[1] - hi[1], d2 = lo[2] - hi[2];
      const uint32_t dist = (uint32_t)(d0 * d0 + d1 * d1 + d2 * d2);
      const uint32_t w = dist / 5000u < 1u ? 1u : dist / 5000u > 8u ? 8u : dist / 5000u;
      for (int k2 = 0; k2 < 3; k2++) { T.v[k2] = (float)lo[k2]; T.v[3 + k2] = (float)hi[k2]; }
      T.weight = (float)(w * (uint32_t)(n / 16));
      continue;
    }
    if (cfg.has_color) palettize(px + tile_ofs[t], n, perceptual, T.v);
    for (int a = 0; a < cfg.num_alpha; a++) palettize_alpha(px + tile_ofs[t], n, cfg.comp[a], T.va[a]);
  }
  for (int by = 0; by < 2; by++)
    for (int bx = 0; bx < 2; bx++) {
      const uint32_t blk = ch.b + (by ? ch.width : 0) + bx;
      block_tile[blk] = 4 * c + tile_map[best_e][by][bx];
      block_enc[blk] = (uint8_t)best_e;
    }
  return best_e;
}

// the dxt_fast alpha selectors of every block's channel comp (qdxt5::init's distinct-selector
// count, crnlib/crn_qdxt5.cpp:400-422)
__global__ void k_fast_alpha_selector_words(const uint32_t* __restrict__ blocks, uint32_t n, int comp,
                                            unsigned long long* __restrict__ words) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n) return;
  uint32_t px[16];
  for (int i = 0; i < 16; i++) px[i] = blocks[(size_t)b * 16 + i];
  uint64_t w = 0;
  fast_alpha_error(16, px, comp, &w);
  words[b] = (unsigned long long)w;
}

// the dxt_fast selector word of every block (qdxt1::init's distinct-selector count)
__global__ void k_fast_selector_words(const uint32_t* __restrict__ blocks, uint32_t n,
                                      const SolidTables* __restrict__ st, uint32_t* __restrict__ words) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n) return;
  uint32_t px[16];
  for (int i = 0; i < 16; i++) px[i] = blocks[(size_t)b * 16 + i];
  uint8_t sel[16];
  uint32_t lo16, hi16;
  fast_compress(16, px, st, lo16, hi16, sel);
  uint32_t w = 0;
  for (int i = 0; i < 16; i++) w |= (uint32_t)sel[i] << (2 * i);
  words[b] = w;
}

__global__ void __launch_bounds__(64) k_hc_tiles(const uint32_t* __restrict__ blocks, const Chunk* __restrict__ chunks,
                                                 uint32_t nchunks, const float* __restrict__ derating /* [level][8] */,
                                                 const float* __restrict__ level_weight, int perceptual,
                                                 const SolidTables* __restrict__ st, TileCfg cfg, Tile* __restrict__ tiles,
                                                 uint32_t* __restrict__ block_tile, uint8_t* __restrict__ block_enc) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nchunks) return;
  hc_tile_chunk(blocks, c, chunks[c], derating, level_weight, perceptual != 0, st, cfg, tiles, block_tile, block_enc);
}

// ------------------------------------------------------------------------------------------
// Tree clusterizer, batched: one thread-block cluster per node to split. The node's vectors lie
// contiguously (a split moves them, with their weights, into the other of two buffers: lefts, then
// rights, each in their previous order), so every pass over a node is a coalesced stream; large
// nodes get up to 16 CTAs on as many SMs, whose partial sums meet through distributed shared
// memory.

constexpr int kVqThreads = 512;
constexpr uint32_t kDefaultRoundFraction = 4;  // a VQ round splits at most leaves / 4 nodes
constexpr uint32_t kVqPerCta = 2048;            // vectors per CTA below which a node gets fewer CTAs

template <int D>
struct VqNode {
  float c[D];         // centroid
  double weight;      // total weight
  float variance;     // weighted variance (sum of squared deviations)
  uint32_t begin, end;
  int32_t left, right;  // children (-1: leaf)
  uint32_t unsplittable;  // 1: this node cannot be split; 2 (on a left child): its parent could not
  uint32_t buf;           // which of the two vector buffers holds this node's range
};

struct SplitJob { int32_t parent, left, right; };

// block-wide sum of `n` floats held per thread (in-place result in vals on every thread)
template <int N>
__device__ __forceinline__ void block_sum(float* vals, float* red /* smem [N * 16] */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < N; k++)
    for (int o = 16; o > 0; o >>= 1) vals[k] += __shfl_xor_sync(0xFFFFFFFFu, vals[k], o);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < N; k++) red[k * 16 + warp] = vals[k];
  __syncthreads();
#pragma unroll
  for (int k = 0; k < N; k++) {
    float s = 0.f;
    for (int w = 0; w < nw; w++) s += red[k * 16 + w];
    vals[k] = s;
  }
}

// block-wide argmax of (value, position): largest value, then smallest position
__device__ __forceinline__ void block_argmax(float& v, uint32_t& pos, float* rv, uint32_t* rp) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    const float ov = __shfl_xor_sync(0xFFFFFFFFu, v, o);
    const uint32_t op = __shfl_xor_sync(0xFFFFFFFFu, pos, o);
    if (ov > v || (ov == v && op < pos)) { v = ov; pos = op; }
  }
  __syncthreads();
  if (lane == 0) { rv[warp] = v; rp[warp] = pos; }
  __syncthreads();
  v = rv[0]; pos = rp[0];
  for (int w = 1; w < nw; w++)
    if (rv[w] > v || (rv[w] == v && rp[w] < pos)) { v = rv[w]; pos = rp[w]; }
}

// Cluster-wide exchange slots: each reduction writes its CTA's partial into slot[phase] and flips
// the phase, so a slot is rewritten only after a later cluster barrier, by which time every CTA has
// read it.
constexpr int kVqSlot = 40;
struct VqShared {
  float red[kVqSlot * 16];
  float rv[16];
  uint32_t rp[16];
  float part[2][kVqSlot];
  uint32_t upart[2][2];
  float tot[kVqSlot];
  float stage[16][kVqSlot];
  uint32_t ustage[16][2];
  uint32_t scan[2][kVqThreads / 32 + 1];
};

// cluster-wide sum of N floats per thread; every CTA adds the partials in rank order, so all of
// them hold bit-identical totals and take the same branches. Warps reduce by shuffles; N threads
// add the warps' partials; the CTAs' partials are fetched through distributed shared memory in one
// parallel round trip and added by N threads.
template <int N>
__device__ __forceinline__ void cluster_sum(float* vals, VqShared& sh, int& phase, cg::cluster_group& cl) {
  static_assert(N <= kVqSlot, "cluster_sum slot");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < N; k++)
    for (int o = 16; o > 0; o >>= 1) vals[k] += __shfl_xor_sync(0xFFFFFFFFu, vals[k], o);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < N; k++) sh.red[k * 16 + warp] = vals[k];
  __syncthreads();
  if (threadIdx.x < N) {
    float t = 0.f;
    for (int wi = 0; wi < nw; wi++) t += sh.red[threadIdx.x * 16 + wi];
    sh.part[phase][threadIdx.x] = t;
  }
  cl.sync();
  const unsigned C = cl.num_blocks();
  for (unsigned t = threadIdx.x; t < N * C; t += blockDim.x)
    sh.stage[t / N][t % N] = cl.map_shared_rank(&sh.part[phase][0], t / N)[t % N];
  __syncthreads();
  if (threadIdx.x < N) {
    float t = 0.f;
    for (unsigned q = 0; q < C; q++) t += sh.stage[q][threadIdx.x];
    sh.tot[threadIdx.x] = t;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < N; k++) vals[k] = sh.tot[k];
  phase ^= 1;
}

__device__ __forceinline__ void cluster_argmax(float& v, uint32_t& pos, VqShared& sh, int& phase, cg::cluster_group& cl) {
  block_argmax(v, pos, sh.rv, sh.rp);
  if (threadIdx.x == 0) { sh.part[phase][0] = v; sh.upart[phase][0] = pos; }
  cl.sync();
  const unsigned C = cl.num_blocks();
  if (threadIdx.x < C) {
    sh.stage[threadIdx.x][0] = cl.map_shared_rank(&sh.part[phase][0], threadIdx.x)[0];
    sh.ustage[threadIdx.x][0] = cl.map_shared_rank(&sh.upart[phase][0], threadIdx.x)[0];
  }
  __syncthreads();
  for (unsigned q = 0; q < C; q++) {
    const float qv = sh.stage[q][0];
    const uint32_t qp = sh.ustage[q][0];
    if (qv > v || (qv == v && qp < pos)) { v = qv; pos = qp; }
  }
  __syncthreads();
  phase ^= 1;
}

template <int D>
__device__ __forceinline__ void load_vec(const float* __restrict__ p, float* v) {
  if constexpr (D % 4 == 0) {
#pragma unroll
    for (int k = 0; k < D; k += 4) {
      const float4 q = __ldg(reinterpret_cast<const float4*>(p + k));
      v[k] = q.x; v[k + 1] = q.y; v[k + 2] = q.z; v[k + 3] = q.w;
    }
  } else if constexpr (D % 2 == 0) {
#pragma unroll
    for (int k = 0; k < D; k += 2) {
      const float2 q = __ldg(reinterpret_cast<const float2*>(p + k));
      v[k] = q.x; v[k + 1] = q.y;
    }
  } else {
#pragma unroll
    for (int k = 0; k < D; k++) v[k] = __ldg(p + k);
  }
}

template <int D>
__device__ __forceinline__ float dist2(const float* a, const float* b) {
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < D; k++) { const float d = a[k] - b[k]; s += d * d; }
  return s;
}

// Splits each job's parent node into two children (tree_clusterizer::split_node,
// crn_tree_clusterizer.h:265-570): furthest / opposite seeds, the principal axis by 10 steps of
// power iteration on the weighted covariance, the axis split as the 2-means start, then 2-means
// until the variance stops falling. vec[2] / w[2]: the two buffers (N x D floats, N weights).
// One cluster of CTAs per job; CTA r of C works on the r-th contiguous slice of the node's range.
template <int D>
__global__ void __launch_bounds__(kVqThreads) k_vq_split(float* __restrict__ vec0, float* __restrict__ vec1,
                                                         float* __restrict__ w0, float* __restrict__ w1,
                                                         VqNode<D>* __restrict__ nodes, const SplitJob* __restrict__ jobs) {
  __shared__ VqShared sh;
  __shared__ float s_c[D];
  cg::cluster_group cl = cg::this_cluster();
  const unsigned C = cl.num_blocks(), r = cl.block_rank();
  int phase = 0;
  const SplitJob job = jobs[blockIdx.x / C];
  VqNode<D>& P = nodes[job.parent];
  const uint32_t b0 = P.begin, b1 = P.end, src = P.buf;
  const float* __restrict__ vec = src ? vec1 : vec0;
  const float* __restrict__ w = src ? w1 : w0;
  float* __restrict__ dvec = src ? vec0 : vec1;
  float* __restrict__ dw = src ? w0 : w1;
  const uint32_t per = (b1 - b0 + C - 1) / C;
  const uint32_t s0 = min(b1, b0 + r * per), s1 = min(b1, s0 + per);  // this CTA's slice
  if (threadIdx.x < D) s_c[threadIdx.x] = P.c[threadIdx.x];
  __syncthreads();
  float c[D];
#pragma unroll
  for (int k = 0; k < D; k++) c[k] = s_c[k];
  // furthest from the centroid, then the point furthest from that
  float fv = -1.f;
  uint32_t fp = 0xFFFFFFFFu;
  for (uint32_t i = s0 + threadIdx.x; i < s1; i += blockDim.x) {
    float v[D];
    load_vec<D>(vec + (size_t)i * D, v);
    const float d = dist2<D>(v, c);
    if (d > fv) { fv = d; fp = i; }
  }
  cluster_argmax(fv, fp, sh, phase, cl);
  if (fp >= b1) fp = b0;  // only if every distance were NaN
  float fur[D];
  load_vec<D>(vec + (size_t)fp * D, fur);
  float ov = -1.f;
  uint32_t op = 0xFFFFFFFFu;
  for (uint32_t i = s0 + threadIdx.x; i < s1; i += blockDim.x) {
    float v[D];
    load_vec<D>(vec + (size_t)i * D, v);
    const float d = dist2<D>(v, fur);
    if (d > ov) { ov = d; op = i; }
  }
  cluster_argmax(ov, op, sh, phase, cl);
  if (op >= b1) op = b0;
  float L[D], R[D];
  {
    float opp[D];
    load_vec<D>(vec + (size_t)op * D, opp);
#pragma unroll
    for (int k = 0; k < D; k++) {
      L[k] = (fur[k] + c[k]) * 0.5f;
      R[k] = (opp[k] + c[k]) * 0.5f;
    }
  }
  if (b0 + 2 < b1) {
    // principal axis by power iteration on the weighted covariance, applied implicitly:
    // x = Cov a = sum_i w_i (v_i - c) ((v_i - c) . a) / W, normalised by its largest component
    float axis[D];
#pragma unroll
    for (int k = 0; k < D; k++) axis[k] = 1.0f;
    for (int it = 0; it < 10; it++) {
      float acc[D];
#pragma unroll
      for (int k = 0; k < D; k++) acc[k] = 0.f;
      for (uint32_t i = s0 + threadIdx.x; i < s1; i += blockDim.x) {
        float d[D], dot = 0.f;
        load_vec<D>(vec + (size_t)i * D, d);
#pragma unroll
        for (int k = 0; k < D; k++) { d[k] -= c[k]; dot += d[k] * axis[k]; }
        const float ww = w[i] * dot;
#pragma unroll
        for (int k = 0; k < D; k++) acc[k] += d[k] * ww;
      }
      cluster_sum<D>(acc, sh, phase, cl);
      float mx = acc[0];
#pragma unroll
      for (int k = 1; k < D; k++) mx = fmaxf(mx, acc[k]);
      if (mx != 0.f) {
#pragma unroll
        for (int k = 0; k < D; k++) axis[k] = acc[k] * (1.0f / mx);
      } else {
#pragma unroll
        for (int k = 0; k < D; k++) axis[k] = acc[k];
      }
    }
    float len = 0.f;
#pragma unroll
    for (int k = 0; k < D; k++) len += axis[k] * axis[k];
    len = sqrtf(len);
    if (len > 0.f) {
#pragma unroll
      for (int k = 0; k < D; k++) axis[k] /= len;
    }
    float acc[2 * D + 2];
#pragma unroll
    for (int k = 0; k < 2 * D + 2; k++) acc[k] = 0.f;
    for (uint32_t i = s0 + threadIdx.x; i < s1; i += blockDim.x) {
      float v[D];
      load_vec<D>(vec + (size_t)i * D, v);
      float t = 0.f;
#pragma unroll
      for (int k = 0; k < D; k++) t += (v[k] - c[k]) * axis[k];
      const float ww = w[i];
      const float wl = t < 0.f ? ww : 0.f, wr = t < 0.f ? 0.f : ww;
#pragma unroll
      for (int k = 0; k < D; k++) { acc[k] += v[k] * wl; acc[D + k] += v[k] * wr; }
      acc[2 * D] += wl;
      acc[2 * D + 1] += wr;
    }
    cluster_sum<2 * D + 2>(acc, sh, phase, cl);
    if (acc[2 * D] > 0.f && acc[2 * D + 1] > 0.f) {
#pragma unroll
      for (int k = 0; k < D; k++) { L[k] = acc[k] / acc[2 * D]; R[k] = acc[D + k] / acc[2 * D + 1]; }
    }
  }
  // 2-means; the partition is the last assignment (made with the centroids before their update).
  // The updated centroids live in shared memory; the assignment centroids in registers.
  __shared__ float s_L[D], s_R[D];
#pragma unroll
  for (int k = 0; k < D; k++)
    if (threadIdx.x == k) { s_L[k] = L[k]; s_R[k] = R[k]; }
  float prev = 1e10f, lvar = 0.f, rvar = 0.f, lw = 0.f, rw = 0.f;
  float AL[D], AR[D];  // centroids of the last assignment
  for (int loop = 0; loop < 1024; loop++) {
    __syncthreads();
#pragma unroll
    for (int k = 0; k < D; k++) { AL[k] = s_L[k]; AR[k] = s_R[k]; }
    float acc[2 * D + 4];
#pragma unroll
    for (int k = 0; k < 2 * D + 4; k++) acc[k] = 0.f;
    for (uint32_t i = s0 + threadIdx.x; i < s1; i += blockDim.x) {
      float vv[D];
      load_vec<D>(vec + (size_t)i * D, vv);
      const float ww = w[i];
      const bool left = dist2<D>(AL, vv) < dist2<D>(AR, vv);
      const float wl = left ? ww : 0.f, wr = left ? 0.f : ww;
      float sq = 0.f;
#pragma unroll
      for (int k = 0; k < D; k++) { acc[k] += vv[k] * wl; acc[D + k] += vv[k] * wr; sq += vv[k] * vv[k]; }
      acc[2 * D] += wl;
      acc[2 * D + 1] += wr;
      acc[2 * D + 2] += sq * wl;
      acc[2 * D + 3] += sq * wr;
    }
    cluster_sum<2 * D + 4>(acc, sh, phase, cl);
    lw = acc[2 * D]; rw = acc[2 * D + 1];
    if (!(lw > 0.f) || !(rw > 0.f)) break;
    float ll = 0.f, rr = 0.f;
#pragma unroll
    for (int k = 0; k < D; k++) { ll += acc[k] * acc[k]; rr += acc[D + k] * acc[D + k]; }
    lvar = acc[2 * D + 2] - ll / lw;
    rvar = acc[2 * D + 3] - rr / rw;
    // every thread read s_L / s_R before cluster_sum's barriers
#pragma unroll
    for (int k = 0; k < D; k++)
      if (threadIdx.x == k) { s_L[k] = acc[k] / lw; s_R[k] = acc[D + k] / rw; }
    const float tv = lvar + rvar;
    if (tv < .00001f) break;
    if ((prev - tv) / tv < .00001f) break;
    prev = tv;
  }
  __syncthreads();
  if (!(lw > 0.f) || !(rw > 0.f)) {
    if (r == 0 && threadIdx.x == 0) {
      P.unsplittable = 1;
      nodes[job.left].unsplittable = 2;
    }
    cl.sync();  // no CTA leaves while another may still read its shared memory
    return;
  }
  // stable partition of the node by the last assignment into the other buffer: lefts first, then
  // rights, each keeping its order. Count this slice's lefts, exchange the counts, then place.
  uint32_t my_left = 0;
  for (uint32_t base = s0; base < s1; base += blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    bool left = false;
    if (i < s1) {
      float vv[D];
      load_vec<D>(vec + (size_t)i * D, vv);
      left = dist2<D>(AL, vv) < dist2<D>(AR, vv);
    }
    my_left += (uint32_t)__syncthreads_count(left);
  }
  if (threadIdx.x == 0) { sh.upart[phase][0] = my_left; sh.upart[phase][1] = s1 - s0; }
  cl.sync();
  if (threadIdx.x < 2 * C) sh.ustage[threadIdx.x >> 1][threadIdx.x & 1] = cl.map_shared_rank(&sh.upart[phase][0], threadIdx.x >> 1)[threadIdx.x & 1];
  __syncthreads();
  uint32_t left_before = 0, right_before = 0, left_total = 0;
  for (unsigned q = 0; q < C; q++) {
    const uint32_t ql = sh.ustage[q][0], qn = sh.ustage[q][1];
    left_total += ql;
    if (q < r) { left_before += ql; right_before += qn - ql; }
  }
  phase ^= 1;
  uint32_t lrun = b0 + left_before, rrun = b0 + left_total + right_before;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int sb = 0;
  for (uint32_t base = s0; base < s1; base += blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    const bool live = i < s1;
    float vv[D];
    bool left = false;
    if (live) {
      load_vec<D>(vec + (size_t)i * D, vv);
      left = dist2<D>(AL, vv) < dist2<D>(AR, vv);
    }
    const uint32_t bl = __ballot_sync(0xFFFFFFFFu, live && left), br = __ballot_sync(0xFFFFFFFFu, live && !left);
    if (lane == 0) { sh.scan[sb][warp] = __popc(bl); sh.scan[sb][warp] |= (uint32_t)__popc(br) << 16; }
    __syncthreads();
    uint32_t lpre = 0, rpre = 0, ltot = 0, rtot = 0;
    for (int wi = 0; wi < nw; wi++) {
      const uint32_t t = sh.scan[sb][wi];
      if (wi < warp) { lpre += t & 0xFFFFu; rpre += t >> 16; }
      ltot += t & 0xFFFFu;
      rtot += t >> 16;
    }
    if (live) {
      const uint32_t dst = left ? lrun + lpre + __popc(bl & ((1u << lane) - 1u)) : rrun + rpre + __popc(br & ((1u << lane) - 1u));
#pragma unroll
      for (int k = 0; k < D; k++) dvec[(size_t)dst * D + k] = vv[k];
      dw[dst] = w[i];
    }
    lrun += ltot;
    rrun += rtot;
    sb ^= 1;  // the next window's counts go to the other slot; this one is rewritten after a barrier
  }
  if (r == 0 && threadIdx.x == 0) {
    VqNode<D>& A = nodes[job.left];
    VqNode<D>& B = nodes[job.right];
    for (int k = 0; k < D; k++) { A.c[k] = s_L[k]; B.c[k] = s_R[k]; }
    A.weight = lw; B.weight = rw;
    A.variance = lvar; B.variance = rvar;
    A.begin = b0; A.end = b0 + left_total;
    B.begin = b0 + left_total; B.end = b1;
    A.left = A.right = B.left = B.right = -1;
    A.unsplittable = B.unsplittable = 0;
    A.buf = B.buf = src ^ 1u;
    P.left = job.left;
    P.right = job.right;
  }
  cl.sync();  // no CTA leaves while another may still read its shared memory
}

// The same split for small nodes, one warp per job (8 jobs per CTA): the reductions are warp
// butterflies, which leave bit-identical totals in every lane, and no CTA-wide barrier is needed.
constexpr uint32_t kVqWarpMax = 256;  // nodes up to this many vectors take the warp kernel

template <int N>
__device__ __forceinline__ void warp_sum(float* vals) {
#pragma unroll
  for (int k = 0; k < N; k++)
    for (int o = 16; o > 0; o >>= 1) vals[k] += __shfl_xor_sync(0xFFFFFFFFu, vals[k], o);
}

__device__ __forceinline__ void warp_argmax(float& v, uint32_t& pos) {
  for (int o = 16; o > 0; o >>= 1) {
    const float ov = __shfl_xor_sync(0xFFFFFFFFu, v, o);
    const uint32_t op = __shfl_xor_sync(0xFFFFFFFFu, pos, o);
    if (ov > v || (ov == v && op < pos)) { v = ov; pos = op; }
  }
}

template <int D>
__global__ void __launch_bounds__(256, 2) k_vq_split_warp(float* __restrict__ vec0, float* __restrict__ vec1,
                                                       float* __restrict__ w0, float* __restrict__ w1,
                                                       VqNode<D>* __restrict__ nodes, const SplitJob* __restrict__ jobs,
                                                       uint32_t njobs) {
  const uint32_t jid = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (jid >= njobs) return;  // whole warps only
  const uint32_t lane = threadIdx.x & 31;
  const SplitJob job = jobs[jid];
  VqNode<D>& P = nodes[job.parent];
  const uint32_t b0 = P.begin, b1 = P.end, src = P.buf;
  const float* __restrict__ vec = src ? vec1 : vec0;
  const float* __restrict__ w = src ? w1 : w0;
  float* __restrict__ dvec = src ? vec0 : vec1;
  float* __restrict__ dw = src ? w0 : w1;
  float c[D];
#pragma unroll
  for (int k = 0; k < D; k++) c[k] = P.c[k];
  float fv = -1.f;
  uint32_t fp = 0xFFFFFFFFu;
  for (uint32_t i = b0 + lane; i < b1; i += 32) {
    float v[D];
    load_vec<D>(vec + (size_t)i * D, v);
    const float d = dist2<D>(v, c);
    if (d > fv) { fv = d; fp = i; }
  }
  warp_argmax(fv, fp);
  if (fp >= b1) fp = b0;  // only if every distance were NaN
  float fur[D];
  load_vec<D>(vec + (size_t)fp * D, fur);
  float ov = -1.f;
  uint32_t op = 0xFFFFFFFFu;
  for (uint32_t i = b0 + lane; i < b1; i += 32) {
    float v[D];
    load_vec<D>(vec + (size_t)i * D, v);
    const float d = dist2<D>(v, fur);
    if (d > ov) { ov = d; op = i; }
  }
  warp_argmax(ov, op);
  if (op >= b1) op = b0;
  float L[D], R[D];
  {
    float opp[D];
    load_vec<D>(vec + (size_t)op * D, opp);
#pragma unroll
    for (int k = 0; k < D; k++) {
      L[k] = (fur[k] + c[k]) * 0.5f;
      R[k] = (opp[k] + c[k]) * 0.5f;
    }
  }
  if (b0 + 2 < b1) {
    float axis[D];
#pragma unroll
    for (int k = 0; k < D; k++) axis[k] = 1.0f;
    for (int it = 0; it < 10; it++) {
      float acc[D];
#pragma unroll
      for (int k = 0; k < D; k++) acc[k] = 0.f;
      for (uint32_t i = b0 + lane; i < b1; i += 32) {
        float d[D], dot = 0.f;
        load_vec<D>(vec + (size_t)i * D, d);
#pragma unroll
        for (int k = 0; k < D; k++) { d[k] -= c[k]; dot += d[k] * axis[k]; }
        const float ww = w[i] * dot;
#pragma unroll
        for (int k = 0; k < D; k++) acc[k] += d[k] * ww;
      }
      warp_sum<D>(acc);
      float mx = acc[0];
#pragma unroll
      for (int k = 1; k < D; k++) mx = fmaxf(mx, acc[k]);
      if (mx != 0.f) {
#pragma unroll
        for (int k = 0; k < D; k++) axis[k] = acc[k] * (1.0f / mx);
      } else {
#pragma unroll
        for (int k = 0; k < D; k++) axis[k] = acc[k];
      }
    }
    float len = 0.f;
#pragma unroll
    for (int k = 0; k < D; k++) len += axis[k] * axis[k];
    len = sqrtf(len);
    if (len > 0.f) {
#pragma unroll
      for (int k = 0; k < D; k++) axis[k] /= len;
    }
    float acc[2 * D + 2];
#pragma unroll
    for (int k = 0; k < 2 * D + 2; k++) acc[k] = 0.f;
    for (uint32_t i = b0 + lane; i < b1; i += 32) {
      float v[D];
      load_vec<D>(vec + (size_t)i * D, v);
      float t = 0.f;
#pragma unroll
      for (int k = 0; k < D; k++) t += (v[k] - c[k]) * axis[k];
      const float ww = w[i];
      const float wl = t < 0.f ? ww : 0.f, wr = t < 0.f ? 0.f : ww;
#pragma unroll
      for (int k = 0; k < D; k++) { acc[k] += v[k] * wl; acc[D + k] += v[k] * wr; }
      acc[2 * D] += wl;
      acc[2 * D + 1] += wr;
    }
    warp_sum<2 * D + 2>(acc);
    if (acc[2 * D] > 0.f && acc[2 * D + 1] > 0.f) {
#pragma unroll
      for (int k = 0; k < D; k++) { L[k] = acc[k] / acc[2 * D]; R[k] = acc[D + k] / acc[2 * D + 1]; }
    }
  }
  float prev = 1e10f, lvar = 0.f, rvar = 0.f, lw = 0.f, rw = 0.f;
  float AL[D], AR[D];
  for (int loop = 0; loop < 1024; loop++) {
#pragma unroll
    for (int k = 0; k < D; k++) { AL[k] = L[k]; AR[k] = R[k]; }
    float acc[2 * D + 4];
#pragma unroll
    for (int k = 0; k < 2 * D + 4; k++) acc[k] = 0.f;
    for (uint32_t i = b0 + lane; i < b1; i += 32) {
      float vv[D];
      load_vec<D>(vec + (size_t)i * D, vv);
      const float ww = w[i];
      const bool left = dist2<D>(AL, vv) < dist2<D>(AR, vv);
      const float wl = left ? ww : 0.f, wr = left ? 0.f : ww;
      float sq = 0.f;
#pragma unroll
      for (int k = 0; k < D; k++) { acc[k] += vv[k] * wl; acc[D + k] += vv[k] * wr; sq += vv[k] * vv[k]; }
      acc[2 * D] += wl;
      acc[2 * D + 1] += wr;
      acc[2 * D + 2] += sq * wl;
      acc[2 * D + 3] += sq * wr;
    }
    warp_sum<2 * D + 4>(acc);
    lw = acc[2 * D]; rw = acc[2 * D + 1];
    if (!(lw > 0.f) || !(rw > 0.f)) break;
    float ll = 0.f, rr = 0.f;
#pragma unroll
    for (int k = 0; k < D; k++) { ll += acc[k] * acc[k]; rr += acc[D + k] * acc[D + k]; }
    lvar = acc[2 * D + 2] - ll / lw;
    rvar = acc[2 * D + 3] - rr / rw;
#pragma unroll
    for (int k = 0; k < D; k++) { L[k] = acc[k] / lw; R[k] = acc[D + k] / rw; }
    const float tv = lvar + rvar;
    if (tv < .00001f) break;
    if ((prev - tv) / tv < .00001f) break;
    prev = tv;
  }
  if (!(lw > 0.f) || !(rw > 0.f)) {
    if (lane == 0) {
      P.unsplittable = 1;
      nodes[job.left].unsplittable = 2;
    }
    return;
  }
  uint32_t left_total = 0;
  for (uint32_t base = b0; base < b1; base += 32) {
    const uint32_t i = base + lane;
    bool left = false;
    if (i < b1) {
      float vv[D];
      load_vec<D>(vec + (size_t)i * D, vv);
      left = dist2<D>(AL, vv) < dist2<D>(AR, vv);
    }
    left_total += (uint32_t)__popc(__ballot_sync(0xFFFFFFFFu, left));
  }
  uint32_t lrun = b0, rrun = b0 + left_total;
  for (uint32_t base = b0; base < b1; base += 32) {
    const uint32_t i = base + lane;
    const bool live = i < b1;
    float vv[D];
    bool left = false;
    if (live) {
      load_vec<D>(vec + (size_t)i * D, vv);
      left = dist2<D>(AL, vv) < dist2<D>(AR, vv);
    }
    const uint32_t bl = __ballot_sync(0xFFFFFFFFu, live && left), br = __ballot_sync(0xFFFFFFFFu, live && !left);
    if (live) {
      const uint32_t below = (1u << lane) - 1u;
      const uint32_t dst = left ? lrun + __popc(bl & below) : rrun + __popc(br & below);
#pragma unroll
      for (int k = 0; k < D; k++) dvec[(size_t)dst * D + k] = vv[k];
      dw[dst] = w[i];
    }
    lrun += __popc(bl);
    rrun += __popc(br);
  }
  if (lane == 0) {
    VqNode<D>& A = nodes[job.left];
    VqNode<D>& B = nodes[job.right];
    for (int k = 0; k < D; k++) { A.c[k] = L[k]; B.c[k] = R[k]; }
    A.weight = lw; B.weight = rw;
    A.variance = lvar; B.variance = rvar;
    A.begin = b0; A.end = b0 + left_total;
    B.begin = b0 + left_total; B.end = b1;
    A.left = A.right = B.left = B.right = -1;
    A.unsplittable = B.unsplittable = 0;
    A.buf = B.buf = src ^ 1u;
    P.left = job.left;
    P.right = job.right;
  }
}

// Root node statistics (centroid, weight, variance of all vectors) and the first buffer: the
// caller's vectors and integer weights copied as floats. One cluster over all vectors.
template <int D>
__global__ void __launch_bounds__(kVqThreads) k_vq_root(const float* __restrict__ vec, const uint32_t* __restrict__ w,
                                                        uint32_t n, float* __restrict__ vec0, float* __restrict__ w0,
                                                        VqNode<D>* __restrict__ nodes) {
  __shared__ VqShared sh;
  cg::cluster_group cl = cg::this_cluster();
  const unsigned C = cl.num_blocks(), r = cl.block_rank();
  int phase = 0;
  const uint32_t per = (n + C - 1) / C;
  const uint32_t s0 = min(n, r * per), s1 = min(n, s0 + per);
  float acc[D + 2];
#pragma unroll
  for (int k = 0; k < D + 2; k++) acc[k] = 0.f;
  for (uint32_t i = s0 + threadIdx.x; i < s1; i += blockDim.x) {
    const float ww = (float)w[i];
    float v[D];
    load_vec<D>(vec + (size_t)i * D, v);
    float sq = 0.f;
#pragma unroll
    for (int k = 0; k < D; k++) { acc[k] += v[k] * ww; sq += v[k] * v[k]; vec0[(size_t)i * D + k] = v[k]; }
    w0[i] = ww;
    acc[D] += ww;
    acc[D + 1] += sq * ww;
  }
  cluster_sum<D + 2>(acc, sh, phase, cl);
  if (r == 0 && threadIdx.x == 0) {
    VqNode<D>& rt = nodes[0];
    float cc = 0.f;
    for (int k = 0; k < D; k++) cc += acc[k] * acc[k];
    rt.variance = acc[D] > 0.f ? acc[D + 1] - cc / acc[D] : 0.f;
    for (int k = 0; k < D; k++) rt.c[k] = acc[D] > 0.f ? acc[k] / acc[D] : 0.f;
    rt.weight = acc[D];
    rt.begin = 0; rt.end = n;
    rt.left = rt.right = -1;
    rt.unsplittable = 0;
    rt.buf = 0;
  }
  cl.sync();
}

// CTAs per cluster for nodes of up to `size` vectors: one CTA per kVqPerCta vectors, a power of
// two, at most 16 (8 where the device cannot co-schedule 16-CTA clusters of this kernel).
inline unsigned vq_cluster_size(uint32_t size, unsigned max_cluster) {
  unsigned c = 1;
  while (c < max_cluster && (uint64_t)c * kVqPerCta < size) c <<= 1;
  return c;
}

template <class K, class... Args>
cudaError_t launch_clustered(K kernel, unsigned grid, unsigned cluster, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kVqThreads);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// Largest cluster (16 or 8) the device co-schedules for this kernel.
template <class K>
unsigned max_vq_cluster(K kernel) {
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
    cudaGetLastError();
    return 8;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(16);
  cfg.blockDim = dim3(kVqThreads);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 16;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int nclusters = 0;
  if (cudaOccupancyMaxActiveClusters(&nclusters, kernel, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 8;
  }
  return nclusters >= 1 ? 16u : 8u;
}

// Device scratch of the tree clusterizer (nodes, the two vector / weight buffers, the job list),
// kept across calls by the caller's workspace.
struct VqScratch {
  DevBuf nodes, v[2], wt[2], jobs;
};

// Host driver of the batched tree clusterizer: returns the codebook (leaf centroids) on the device
// as K x D floats in `codebook` and the leaf count in *k_out.
template <int D>
int tree_vq(const float* d_vec, const uint32_t* d_w, uint32_t n, uint32_t max_entries, uint32_t round_fraction,
            DevBuf& codebook, uint32_t* k_out, cudaStream_t s, VqScratch& scr) {
  using Node = VqNode<D>;
  *k_out = 0;
  if (!n) return CRNGPU_OK;
  max_entries = std::max<uint32_t>(1, std::min(max_entries, n));
  // every split attempt takes two node slots; a node fails at most once (it is then marked
  // unsplittable), so attempts <= (max_entries - 1) successes + at most 2 * max_entries failures
  const size_t max_nodes = 6 * (size_t)max_entries + 8;
  static const unsigned max_split_cluster = max_vq_cluster(k_vq_split<D>);
  static const unsigned max_root_cluster = max_vq_cluster(k_vq_root<D>);
  DevBuf& d_nodes = scr.nodes;
  DevBuf* d_v = scr.v;
  DevBuf* d_wt = scr.wt;
  DevBuf& d_jobs = scr.jobs;
  cudaError_t e;
  if ((e = d_nodes.ensure(sizeof(Node) * max_nodes)) != cudaSuccess) return cuda_check(e, "alloc vq nodes");
  for (int b = 0; b < 2; b++) {
    if ((e = d_v[b].ensure(sizeof(float) * D * (size_t)n)) != cudaSuccess) return cuda_check(e, "alloc vq vectors");
    if ((e = d_wt[b].ensure(sizeof(float) * (size_t)n)) != cudaSuccess) return cuda_check(e, "alloc vq weights");
  }
  if ((e = d_jobs.ensure(sizeof(SplitJob) * max_entries)) != cudaSuccess) return cuda_check(e, "alloc vq jobs");
  Node* nodes = static_cast<Node*>(d_nodes.ptr);
  float* v0 = static_cast<float*>(d_v[0].ptr);
  float* v1 = static_cast<float*>(d_v[1].ptr);
  float* w0 = static_cast<float*>(d_wt[0].ptr);
  float* w1 = static_cast<float*>(d_wt[1].ptr);
  {
    const unsigned C = vq_cluster_size(n, max_root_cluster);
    if ((e = launch_clustered(k_vq_root<D>, C, C, s, d_vec, d_w, n, v0, w0, nodes)) != cudaSuccess)
      return cuda_check(e, "launch k_vq_root");
  }
  std::vector<Node> h(max_nodes);
  if ((e = cudaMemcpyAsync(h.data(), nodes, sizeof(Node), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
    return cuda_check(e, "read vq root");
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_check(e, "sync");
  std::vector<int> leaves{0};
  size_t used = 1;
  while (leaves.size() < max_entries) {
    // candidates: splittable leaves, highest variance first (the reference's priority queue order)
    std::vector<int> cand;
    for (int l : leaves) {
      const Node& nd = h[l];
      if (!nd.unsplittable && nd.variance > 0.0f && nd.end - nd.begin > 1) cand.push_back(l);
    }
    if (cand.empty()) break;
    std::stable_sort(cand.begin(), cand.end(), [&](int a, int b) { return h[a].variance > h[b].variance; });
    // the reference splits one node at a time, always the leaf of largest variance; a round here
    // splits the top 1/round_fraction of the splittable leaves by variance (at least one), which
    // keeps the greedy order's preference for high-variance regions while giving the GPU a batch
    size_t take = std::min(cand.size(), (size_t)max_entries - leaves.size());
    take = std::min(take, std::max<size_t>(1, leaves.size() / round_fraction));
    take = std::min(take, (max_nodes - used) / 2);
    if (!take) break;
    // large nodes first in the job list (one CTA cluster each), then small ones (a warp each)
    std::vector<SplitJob> jobs;
    jobs.reserve(take);
    uint32_t largest = 0;
    const size_t first_new = used;
    for (int pass = 0; pass < 2; pass++)
      for (size_t i = 0; i < take; i++) {
        const uint32_t size = h[cand[i]].end - h[cand[i]].begin;
        if ((size > kVqWarpMax) != (pass == 0)) continue;
        jobs.push_back(SplitJob{cand[i], (int)used, (int)used + 1});
        used += 2;
        if (!pass) largest = std::max(largest, size);
      }
    size_t nbig = 0;
    while (nbig < jobs.size() && h[jobs[nbig].parent].end - h[jobs[nbig].parent].begin > kVqWarpMax) nbig++;
    if ((e = cudaMemcpyAsync(d_jobs.ptr, jobs.data(), sizeof(SplitJob) * take, cudaMemcpyHostToDevice, s)) != cudaSuccess)
      return cuda_check(e, "copy vq jobs");
    const SplitJob* dj = static_cast<const SplitJob*>(d_jobs.ptr);
    if (nbig) {
      const unsigned C = vq_cluster_size(largest, max_split_cluster);
      if ((e = launch_clustered(k_vq_split<D>, (unsigned)nbig * C, C, s, v0, v1, w0, w1, nodes, dj)) != cudaSuccess)
        return cuda_check(e, "launch k_vq_split");
    }
    if (nbig < take) {
      const uint32_t nsmall = (uint32_t)(take - nbig);
      k_vq_split_warp<D><<<(nsmall + 7) / 8, 256, 0, s>>>(v0, v1, w0, w1, nodes, dj + nbig, nsmall);
      if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(e, "launch k_vq_split_warp");
    }
    // only the new children are read back; a failed split is flagged on its left child
    if ((e = cudaMemcpyAsync(h.data() + first_new, nodes + first_new, sizeof(Node) * (used - first_new),
                             cudaMemcpyDeviceToHost, s)) != cudaSuccess)
      return cuda_check(e, "read vq nodes");
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_check(e, "sync");
    std::vector<int> next;
    bool progressed = false;
    std::vector<char> split(used, 0);
    for (const SplitJob& j : jobs) {
      if (h[j.left].unsplittable == 2) {
        h[j.parent].unsplittable = 1;
      } else {
        h[j.parent].left = j.left;
        h[j.parent].right = j.right;
        split[j.parent] = 1;
        progressed = true;
      }
    }
    for (int l : leaves) {
      if (split[l]) { next.push_back(h[l].left); next.push_back(h[l].right); }
      else next.push_back(l);
    }
    leaves.swap(next);
    if (!progressed) {
      // every candidate proved unsplittable this round; they are marked, try the rest next round
      bool any = false;
      for (int l : leaves) if (!h[l].unsplittable && h[l].variance > 0.0f && h[l].end - h[l].begin > 1) any = true;
      if (!any) break;
    }
  }
  // codebook in leaf order
  std::vector<float> cb((size_t)leaves.size() * D);
  for (size_t i = 0; i < leaves.size(); i++)
    for (int k = 0; k < D; k++) cb[i * D + k] = h[leaves[i]].c[k];
  if ((e = codebook.ensure(cb.size() * sizeof(float) + 16)) != cudaSuccess) return cuda_check(e, "alloc codebook");
  if ((e = cudaMemcpyAsync(codebook.ptr, cb.data(), cb.size() * sizeof(float), cudaMemcpyHostToDevice, s)) != cudaSuccess)
    return cuda_check(e, "copy codebook");
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_check(e, "sync");
  *k_out = (uint32_t)leaves.size();
  return CRNGPU_OK;
}

// ------------------------------------------------------------------------------------------
// Tile -> endpoint cluster (exact nearest codebook vec6, first index on ties); one thread per tile,
// codebook streamed through shared memory.
__global__ void __launch_bounds__(256) k_nearest_vec6(const Tile* __restrict__ tiles, uint32_t ntiles,
                                                      const float* __restrict__ cb, uint32_t K,
                                                      uint32_t* __restrict__ tile_cluster) {
  __shared__ float s_cb[1024 * 6];
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = t < ntiles && tiles[t].kind != 0xFFu;
  float v[6];
  if (live)
    for (int k = 0; k < 6; k++) v[k] = tiles[t].v[k];
  float best = 3.4e38f;
  uint32_t bi = 0;
  for (uint32_t base = 0; base < K; base += 1024) {
    const uint32_t cnt = min(1024u, K - base);
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < cnt * 6; i += blockDim.x) s_cb[i] = cb[(size_t)base * 6 + i];
    __syncthreads();
    if (live) {
      for (uint32_t j = 0; j < cnt; j++) {
        const float* c = s_cb + j * 6;
        float d = 0.f;
#pragma unroll
        for (int k = 0; k < 6; k++) { const float x = c[k] - v[k]; d += x * x; }
        if (d < best) { best = d; bi = base + j; }
      }
    }
  }
  if (t < ntiles) tile_cluster[t] = live ? bi : 0xFFFFFFFFu;
}

// ------------------------------------------------------------------------------------------
// Per-cluster endpoint fit over all pixels of the cluster's tiles (one CTA per cluster).

constexpr int kFitThreads = 128;

struct ClusterOut {
  uint32_t first, second;  // 565 endpoints, first > second (4-colour order)
  int col[4][3];           // linear-order colours: first, 2/3 first + 1/3 second, ..., second
};

// pixel j of tile T (chunk image coordinates as in chunk_pixels)
__device__ __forceinline__ uint32_t tile_pixel(const uint32_t* __restrict__ blocks, const Chunk& ch, uint32_t kind,
                                               uint32_t j) {
  const uint32_t idx = c_tile_ofs[kind] + j;  // position in the 128-pixel chunk image
  if (idx < 64) {
    const uint32_t q = idx >> 4;  // TL, BL, TR, BR
    const uint32_t blk = ch.b + ((q & 1) ? ch.width : 0) + ((q & 2) ? 1 : 0);
    return __ldg(blocks + (size_t)blk * 16 + (idx & 15));
  }
  const uint32_t t = idx - 64;  // row-major 8-wide, 8 rows: row r = t >> 3, column x = t & 7
  const uint32_t r = t >> 3, x = t & 7;
  const uint32_t blk = ch.b + ((r & 4) ? ch.width : 0) + ((x & 4) ? 1 : 0);
  return __ldg(blocks + (size_t)blk * 16 + (r & 3) * 4 + (x & 3));
}

__device__ __forceinline__ uint32_t tile_npix(uint32_t kind) { return 16u << (kind >> 2); }

// error of (first, second) over selectors chosen per pixel, plus the least-squares statistics
struct FitAcc {
  float aa, ab, bb, ax[3], bx[3];
  float err;
};


// Unique colours of a cluster in shared memory (open addressing on the packed RGB, count per
// colour); a cluster with more than kUniqCap / 2 distinct colours skips the probe search.
constexpr int kUniqCap = 4096;
constexpr int kMaxCand = 1024;
__constant__ int16_t c_probe[15] = {0, 1, 2, 3, 5, 7, 9, 10, 13, 15, 19, 27, 43, 59, 91};  // g_uber_probe_table

// The probe search's colour table: per unique colour u, {-2 w_r r, -2 w_g g, -2 w_b b, xx} with
// xx = w_r r^2 + w_g g^2 + w_b b^2 (w = 8, 25, 1 perceptual, else 1), and its pixel count. For a
// palette colour p with pp = sum w p^2, the weighted squared distance is xx + pp + a . p, so a
// pixel's error against the 4-colour palette is xx + min_k (pp_k + a . p_k): three multiply-adds
// per palette colour, exactly the integer error of cdist.
__device__ __forceinline__ int4 probe_entry(uint32_t rgb, bool perc) {
  const int r = (int)(rgb & 255), g = (int)((rgb >> 8) & 255), b = (int)((rgb >> 16) & 255);
  const int wr = perc ? 8 : 1, wg = perc ? 25 : 1;
  return make_int4(-2 * wr * r, -2 * wg * g, -2 * b, wr * r * r + wg * g * g + b * b);
}

// Error of the 4-colour block (lo, hi) over the unique colours, abandoned (returning ~0) as soon as
// its running sum reaches `bound` (a candidate that cannot win); one thread.
__device__ __forceinline__ unsigned long long pair_error(uint32_t lo, uint32_t hi, const int4* ut, const uint32_t* uc,
                                                        int U, bool perc, unsigned long long bound) {
  int col[4][3];
  colors4(lo, hi, col);
  const int wr = perc ? 8 : 1, wg = perc ? 25 : 1;
  int pp[4];
#pragma unroll
  for (int k = 0; k < 4; k++) pp[k] = wr * col[k][0] * col[k][0] + wg * col[k][1] * col[k][1] + col[k][2] * col[k][2];
  unsigned long long e = 0;
  for (int i = 0; i < U; i++) {
    const int4 t = ut[i];
    int m = pp[0] + t.x * col[0][0] + t.y * col[0][1] + t.z * col[0][2];
#pragma unroll
    for (int k = 1; k < 4; k++) m = min(m, pp[k] + t.x * col[k][0] + t.y * col[k][1] + t.z * col[k][2]);
    e += (unsigned long long)(uint32_t)(t.w + m) * uc[i];
    if ((i & 15) == 15 && e >= bound) return ~0ull;
  }
  return e < bound ? e : ~0ull;
}

// Evaluates the candidate pairs cand[0..n) (lo | hi << 16), one thread per candidate, and returns
// to every thread the best (lowest error, then lowest index) among those below `bound`; err = ~0
// and pair = 0 when none is.
__device__ void best_candidate(const uint32_t* cand, int n, const int4* ut, const uint32_t* uc, int U, bool perc,
                               unsigned long long bound, unsigned long long* s_be, uint32_t* s_bi,
                               unsigned long long& err, uint32_t& pair) {
  const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  unsigned long long be = ~0ull;
  uint32_t bi = 0xFFFFFFFFu;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    // a later candidate must beat this thread's best strictly (ties go to the lower index)
    const unsigned long long e = pair_error(cand[i] & 0xFFFFu, cand[i] >> 16, ut, uc, U, perc, min(bound, be));
    if (e < be) { be = e; bi = (uint32_t)i; }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long oe = __shfl_xor_sync(0xFFFFFFFFu, be, o);
    const uint32_t oi = __shfl_xor_sync(0xFFFFFFFFu, bi, o);
    if (oe < be || (oe == be && oi < bi)) { be = oe; bi = oi; }
  }
  __syncthreads();
  if ((threadIdx.x & 31) == 0) { s_be[warp] = be; s_bi[warp] = bi; }
  __syncthreads();
  be = s_be[0]; bi = s_bi[0];
  for (int w = 1; w < nw; w++)
    if (s_be[w] < be || (s_be[w] == be && s_bi[w] < bi)) { be = s_be[w]; bi = s_bi[w]; }
  err = be;
  pair = bi < (uint32_t)n ? cand[bi] : 0;
  __syncthreads();
}

__global__ void __launch_bounds__(kFitThreads) k_cluster_fit(const uint32_t* __restrict__ blocks,
                                                             const Chunk* __restrict__ chunks,
                                                             const Tile* __restrict__ tiles,
                                                             const uint32_t* __restrict__ ctile_start,
                                                             const uint32_t* __restrict__ ctile_list, int perceptual,
                                                             ClusterOut* __restrict__ out) {
  __shared__ float red[24 * 16];
  __shared__ uint32_t s_tiles[256];
  const uint32_t k = blockIdx.x;
  const uint32_t t0 = ctile_start[k], t1 = ctile_start[k + 1];
  const bool perc = perceptual != 0;
  ClusterOut& O = out[k];
  if (t0 == t1) {
    if (threadIdx.x == 0) { O.first = 0xFFFFu; O.second = 0; }
    return;
  }
  // pass over the cluster's pixels: thread handles (tile, pixel) pairs; tiles staged 256 at a time
  auto for_pixels = [&](auto&& fn) {
    for (uint32_t base = t0; base < t1; base += 256) {
      const uint32_t cnt = min(256u, t1 - base);
      __syncthreads();
      for (uint32_t i = threadIdx.x; i < cnt; i += blockDim.x) s_tiles[i] = ctile_list[base + i];
      __syncthreads();
      // each tile contributes up to 64 pixels: thread pairs (i, j) strided over cnt x 64
      for (uint32_t q = threadIdx.x; q < cnt * 64; q += blockDim.x) {
        const uint32_t ti = s_tiles[q >> 6], j = q & 63;
        const Tile& T = tiles[ti];
        if (j >= tile_npix(T.kind)) continue;
        fn(tile_pixel(blocks, chunks[T.chunk], T.kind, j));
      }
    }
  };
  // 1. mean and (perceptually weighted) covariance
  float acc[10];
  for (int i = 0; i < 10; i++) acc[i] = 0.f;
  for_pixels([&](uint32_t p) {
    const float r = (float)px_r(p), g = (float)px_g(p), b = (float)px_b(p);
    acc[0] += r; acc[1] += g; acc[2] += b; acc[3] += 1.f;
    acc[4] += r * r; acc[5] += r * g; acc[6] += r * b; acc[7] += g * g; acc[8] += g * b; acc[9] += b * b;
  });
  block_sum<10>(acc, red);
  const float cnt = acc[3];
  const float mean[3] = {acc[0] / cnt, acc[1] / cnt, acc[2] / cnt};
  // perceptual weights (crnlib/crn_dxt1.cpp:1074-1108 start from luma-like weights)
  const float pw[3] = {perc ? 0.212f : 1.f, perc ? 0.72f : 1.f, perc ? 0.072f : 1.f};
  double cov[6] = {acc[4] / cnt - mean[0] * mean[0], acc[5] / cnt - mean[0] * mean[1], acc[6] / cnt - mean[0] * mean[2],
                   acc[7] / cnt - mean[1] * mean[1], acc[8] / cnt - mean[1] * mean[2], acc[9] / cnt - mean[2] * mean[2]};
  cov[0] *= pw[0] * pw[0]; cov[1] *= pw[0] * pw[1]; cov[2] *= pw[0] * pw[2];
  cov[3] *= pw[1] * pw[1]; cov[4] *= pw[1] * pw[2]; cov[5] *= pw[2] * pw[2];
  double ar = .9, ag = 1.0, ab = .7;
  for (int it = 0; it < 8; it++) {
    const double r = ar * cov[0] + ag * cov[1] + ab * cov[2];
    const double g = ar * cov[1] + ag * cov[3] + ab * cov[4];
    const double b = ar * cov[2] + ag * cov[4] + ab * cov[5];
    const double m = fmax(fabs(r), fmax(fabs(g), fabs(b)));
    if (m > 1e-10) { ar = r / m; ag = g / m; ab = b / m; } else { ar = r; ag = g; ab = b; }
  }
  float axis[3] = {(float)(ar / pw[0]), (float)(ag / pw[1]), (float)(ab / pw[2])};
  {
    const float len = sqrtf(axis[0] * axis[0] + axis[1] * axis[1] + axis[2] * axis[2]);
    if (len < 1e-10f) { axis[0] = .2837149f; axis[1] = .9540631f; axis[2] = .096277453f; }
    else for (int i = 0; i < 3; i++) axis[i] /= len;
  }
  // 2. projection bounds
  float pr[2] = {3.4e38f, -3.4e38f};
  for_pixels([&](uint32_t p) {
    const float d = ((float)px_r(p) - mean[0]) * axis[0] + ((float)px_g(p) - mean[1]) * axis[1] + ((float)px_b(p) - mean[2]) * axis[2];
    pr[0] = fminf(pr[0], d);
    pr[1] = fmaxf(pr[1], d);
  });
  {
    float mn = -pr[0], mx = pr[1];
    for (int o = 16; o > 0; o >>= 1) { mn = fmaxf(mn, __shfl_xor_sync(0xFFFFFFFFu, mn, o)); mx = fmaxf(mx, __shfl_xor_sync(0xFFFFFFFFu, mx, o)); }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) { red[threadIdx.x >> 5] = mn; red[16 + (threadIdx.x >> 5)] = mx; }
    __syncthreads();
    mn = red[0]; mx = red[16];
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) { mn = fmaxf(mn, red[w]); mx = fmaxf(mx, red[16 + w]); }
    pr[0] = -mn; pr[1] = mx;
  }
  auto q565 = [](float r, float g, float b) -> uint32_t {
    const int ri = clampi((int)floorf(r * 31.f / 255.f + .5f), 0, 31), gi = clampi((int)floorf(g * 63.f / 255.f + .5f), 0, 63),
              bi = clampi((int)floorf(b * 31.f / 255.f + .5f), 0, 31);
    return (uint32_t)((ri << 11) | (gi << 5) | bi);
  };
  // spread of the pixels along the axis (unweighted covariance projected on it)
  const double c_rr = acc[4] / cnt - mean[0] * mean[0], c_rg = acc[5] / cnt - mean[0] * mean[1],
               c_rb = acc[6] / cnt - mean[0] * mean[2], c_gg = acc[7] / cnt - mean[1] * mean[1],
               c_gb = acc[8] / cnt - mean[1] * mean[2], c_bb = acc[9] / cnt - mean[2] * mean[2];
  const double var_ax = axis[0] * axis[0] * c_rr + axis[1] * axis[1] * c_gg + axis[2] * axis[2] * c_bb +
                        2 * (axis[0] * axis[1] * c_rg + axis[0] * axis[2] * c_rb + axis[1] * axis[2] * c_gb);
  const float sd = (float)sqrt(fmax(var_ax, 0.0)) * 1.25f;
  // 3. two starts -- the extreme projections and mean +- 1.25 sigma -- each refined by alternating
  // nearest-colour selectors and least-squares endpoints; keep the lowest (perceptual) error
  uint32_t best0 = 0, best1 = 0;
  float best_err = 3.4e38f;
  for (int start = 0; start < 2; start++) {
    const float hi_t = start ? fminf(pr[1], sd) : pr[1], lo_t = start ? fmaxf(pr[0], -sd) : pr[0];
    uint32_t e0 = q565(mean[0] + hi_t * axis[0], mean[1] + hi_t * axis[1], mean[2] + hi_t * axis[2]);
    uint32_t e1 = q565(mean[0] + lo_t * axis[0], mean[1] + lo_t * axis[1], mean[2] + lo_t * axis[2]);
    for (int it = 0; it < 8; it++) {
      int col[4][3];
      colors4(e0, e1, col);  // DXT order
      float a[10];
      for (int i = 0; i < 10; i++) a[i] = 0.f;
      for_pixels([&](uint32_t p) {
        const int r = px_r(p), g = px_g(p), b = px_b(p);
        uint32_t bd = 0xFFFFFFFFu;
        int bs = 0;
        for (int q = 0; q < 4; q++) {
          const uint32_t d = cdist(perc, r, g, b, col[q][0], col[q][1], col[q][2]);
          if (d < bd) { bd = d; bs = q; }
        }
        // weight of the first endpoint at DXT selector q: 1, 0, 2/3, 1/3
        const float wa = bs == 0 ? 1.f : bs == 1 ? 0.f : bs == 2 ? (2.f / 3.f) : (1.f / 3.f), wb = 1.f - wa;
        a[0] += wa * wa; a[1] += wa * wb; a[2] += wb * wb;
        a[3] += wa * r; a[4] += wa * g; a[5] += wa * b;
        a[6] += wb * r; a[7] += wb * g; a[8] += wb * b;
        a[9] += (float)bd;
      });
      block_sum<10>(a, red);
      if (a[9] < best_err) { best_err = a[9]; best0 = e0; best1 = e1; }
      const float det = a[0] * a[2] - a[1] * a[1];
      if (fabsf(det) < 1e-6f) break;
      const float inv = 1.f / det;
      float f0[3], f1[3];
      for (int c = 0; c < 3; c++) {
        f0[c] = (a[3 + c] * a[2] - a[6 + c] * a[1]) * inv;
        f1[c] = (a[6 + c] * a[0] - a[3 + c] * a[1]) * inv;
      }
      const uint32_t n0 = q565(f0[0], f0[1], f0[2]), n1 = q565(f1[0], f1[1], f1[2]);
      if (n0 == e0 && n1 == e1) break;
      e0 = n0; e1 = n1;
    }
  }
  // 3b. the uber probe search of dxt1_endpoint_optimizer::optimize_endpoints (crnlib/crn_dxt1.cpp:703-1028)
  // over the cluster's unique colours: low and high endpoints probed along the principal axis
  // (g_uber_probe_table steps of 1/64), every low x high pair, then the 26 lattice neighbours and
  // +-2 axis moves of each endpoint of the best pair; up to four passes.
  {
    // hashing: keys in s_raw[0, kUniqCap), counts in s_raw[kUniqCap, 2 kUniqCap); once compacted (at
    // most kUniqCap / 2 colours): the int4 probe table in s_raw[0, 2 kUniqCap), counts after it
    __shared__ __align__(16) uint32_t s_raw[2 * kUniqCap + kUniqCap / 2];
    uint32_t* s_key = s_raw;
    uint32_t* s_cnt = s_raw + kUniqCap;
    int4* s_ut = reinterpret_cast<int4*>(s_raw);
    uint32_t* s_uc = s_raw + 2 * kUniqCap;
    __shared__ uint32_t s_cand[kMaxCand];
    __shared__ unsigned long long s_be[kFitThreads / 32];
    __shared__ uint32_t s_bi[kFitThreads / 32];
    __shared__ uint32_t s_nu, s_overflow;
    __syncthreads();
    for (int i = threadIdx.x; i < kUniqCap; i += blockDim.x) { s_key[i] = 0; s_cnt[i] = 0; }
    if (threadIdx.x == 0) { s_nu = 0; s_overflow = 0; }
    __syncthreads();
    for_pixels([&](uint32_t p) {
      const uint32_t key = (p & 0xFFFFFFu) + 1u;  // 0 marks an empty slot
      uint32_t h = (key * 2654435761u) >> 20;      // 12-bit slot
      for (int probe_n = 0; probe_n < kUniqCap; probe_n++) {
        const uint32_t prev = atomicCAS(&s_key[h], 0u, key);
        if (prev == 0u || prev == key) { atomicAdd(&s_cnt[h], 1u); return; }
        h = (h + 1) & (kUniqCap - 1);
      }
      s_overflow = 1;
    });
    __syncthreads();
    // compact the table in place (slot order); count distinct colours
    __shared__ uint32_t s_wcnt[kFitThreads / 32 + 1];
    uint32_t mine_key[kUniqCap / kFitThreads], mine_cnt[kUniqCap / kFitThreads];
    int nm = 0;
    for (int i = threadIdx.x * (kUniqCap / kFitThreads); i < (int)((threadIdx.x + 1) * (kUniqCap / kFitThreads)); i++)
      if (s_key[i]) { mine_key[nm] = s_key[i] - 1u; mine_cnt[nm] = s_cnt[i]; nm++; }
    {
      // exclusive scan of nm over the CTA
      int incl = nm;
      for (int o = 1; o < 32; o <<= 1) { const int v = __shfl_up_sync(0xFFFFFFFFu, incl, o); if ((threadIdx.x & 31) >= o) incl += v; }
      if ((threadIdx.x & 31) == 31) s_wcnt[threadIdx.x >> 5] = incl;
      __syncthreads();
      int base = 0;
      for (int w = 0; w < (int)(threadIdx.x >> 5); w++) base += s_wcnt[w];
      const int at = base + incl - nm;
      __syncthreads();
      for (int j = 0; j < nm; j++)
        if (at + j < kUniqCap / 2) { s_ut[at + j] = probe_entry(mine_key[j], perc); s_uc[at + j] = mine_cnt[j]; }
      if (threadIdx.x == blockDim.x - 1) s_nu = (uint32_t)(at + nm);
    }
    __syncthreads();
    const int U = (int)s_nu;
    if (!s_overflow && U > 0 && U <= kUniqCap / 2) {
      // best so far: the least-squares fit
      uint32_t bl = best0, bh = best1;
      unsigned long long berr;
      {
        uint32_t pair;
        if (threadIdx.x == 0) s_cand[0] = bl | (bh << 16);
        __syncthreads();
        best_candidate(s_cand, 1, s_ut, s_uc, U, perc, ~0ull, s_be, s_bi, berr, pair);
      }
      // low / high colours from the axis projection bounds, in 565 units
      float lowc[3], highc[3];
      const float lim[3] = {31.f, 63.f, 31.f};
      for (int c = 0; c < 3; c++) {
        lowc[c] = fminf(fmaxf((mean[c] + pr[0] * axis[c]) / 255.f * lim[c], 0.f), lim[c]);
        highc[c] = fminf(fmaxf((mean[c] + pr[1] * axis[c]) / 255.f * lim[c], 0.f), lim[c]);
      }
      float sax[3];
      for (int c = 0; c < 3; c++) sax[c] = axis[c] * .015625f * lim[c];
      for (int pass = 0; pass < 4 && berr; pass++) {
        const unsigned long long prev_err = berr;
        if (pass) {
          int cl[3], ch[3];
          unpack565(bl, cl);
          unpack565(bh, ch);
          for (int c = 0; c < 3; c++) { lowc[c] = (float)cl[c] / 255.f * lim[c]; highc[c] = (float)ch[c] / 255.f * lim[c]; }
        }
        // probe lists (thread 0), then every low x high pair
        __shared__ uint32_t s_pl[32], s_ph[32], s_npl, s_nph;
        if (threadIdx.x == 0) {
          for (int which = 0; which < 2; which++) {
            const float* base = which ? highc : lowc;
            uint32_t* outp = which ? s_ph : s_pl;
            int prev[2] = {-1, -1}, n = 0;
            for (int i = 0; i < 15; i++) {
              const int x = c_probe[i];
              for (int sg = i ? 0 : 1; sg < 2; sg++) {
                const float f = sg ? 1.f : -1.f;
                const int r = clampi((int)floorf(base[0] + .5f + f * sax[0] * (float)x), 0, 31);
                const int g = clampi((int)floorf(base[1] + .5f + f * sax[1] * (float)x), 0, 63);
                const int b = clampi((int)floorf(base[2] + .5f + f * sax[2] * (float)x), 0, 31);
                const int pc = b | (g << 5) | (r << 11);
                if (pc != prev[sg]) { outp[n++] = (uint32_t)pc; prev[sg] = pc; }
              }
            }
            if (which) s_nph = (uint32_t)n; else s_npl = (uint32_t)n;
          }
        }
        __syncthreads();
        const int npl = (int)s_npl, nph = (int)s_nph;
        for (int i = threadIdx.x; i < npl * nph; i += blockDim.x) s_cand[i] = s_pl[i / nph] | (s_ph[i % nph] << 16);
        __syncthreads();
        {
          unsigned long long e;
          uint32_t pair;
          best_candidate(s_cand, npl * nph, s_ut, s_uc, U, perc, berr, s_be, s_bi, e, pair);
          if (e < berr) { berr = e; bl = pair & 0xFFFFu; bh = pair >> 16; }
        }
        // lattice neighbours (26) and +-2 axis moves of the low endpoint, then of the high one
        for (int which = 0; which < 2; which++) {
          if (threadIdx.x == 0) {
            int n = 0;
            const uint32_t E = which ? bh : bl, O2 = which ? bl : bh;
            const int r0 = (E >> 11) & 31, g0 = (E >> 5) & 63, b0 = E & 31;
            for (int dr = -1; dr <= 1; dr++)
              for (int dg = -1; dg <= 1; dg++)
                for (int db = -1; db <= 1; db++) {
                  if (!dr && !dg && !db) continue;
                  const int r = r0 + dr, g = g0 + dg, b = b0 + db;
                  if (r < 0 || r > 31 || g < 0 || g > 63 || b < 0 || b > 31) continue;
                  const uint32_t X = (uint32_t)((r << 11) | (g << 5) | b);
                  s_cand[n++] = which ? (O2 | (X << 16)) : (X | (O2 << 16));
                }
            const int d6[6][3] = {{-2, 0, 0}, {2, 0, 0}, {0, -2, 0}, {0, 2, 0}, {0, 0, -2}, {0, 0, 2}};
            for (int q = 0; q < 6; q++) {
              const int r = r0 + d6[q][0], g = g0 + d6[q][1], b = b0 + d6[q][2];
              if (r < 0 || r > 31 || g < 0 || g > 63 || b < 0 || b > 31) continue;
              const uint32_t X = (uint32_t)((r << 11) | (g << 5) | b);
              s_cand[n++] = which ? (O2 | (X << 16)) : (X | (O2 << 16));
            }
            s_npl = (uint32_t)n;
          }
          __syncthreads();
          const int n = (int)s_npl;
          unsigned long long e;
          uint32_t pair;
          best_candidate(s_cand, n, s_ut, s_uc, U, perc, berr, s_be, s_bi, e, pair);
          if (e < berr) { berr = e; bl = pair & 0xFFFFu; bh = pair >> 16; }
        }
        if (pass && berr == prev_err) break;
      }
      best0 = bl;
      best1 = bh;
    }
    __syncthreads();
  }
  // 4. dxt_endpoint_refiner::optimize_dxt1 (crn_dxt_endpoint_refiner.cpp:203-302): histogram
  // statistics of the current selectors and a lattice walk on both endpoints; repeated with the
  // selectors re-chosen for the walk's result while the true error keeps falling
  __shared__ unsigned long long s_stat[29];  // hist[4], D2[4][3], DD[4][3] (exact integers), error
  __shared__ uint32_t s_LH[2];
  __shared__ uint32_t s_sol[54], s_nsol;
  uint32_t L0 = best0 > best1 ? best0 : best1, H0 = best0 > best1 ? best1 : best0;
  if (L0 == H0) { if (L0 < 0xFFFFu) L0++; else H0--; }
  uint32_t keepL = L0, keepH = H0;
  unsigned long long keep_err = ~0ull;
  for (int outer = 0; outer < 4; outer++) {
    int col[4][3];
    colors4(L0, H0, col);
    __syncthreads();
    if (threadIdx.x < 29) s_stat[threadIdx.x] = 0;
    __syncthreads();
    for_pixels([&](uint32_t p) {
      const int r = px_r(p), g = px_g(p), b = px_b(p);
      uint32_t bd = 0xFFFFFFFFu;
      int bs = 0;
      for (int t = 0; t < 4; t++) {
        const uint32_t d = cdist(perc, r, g, b, col[t][0], col[t][1], col[t][2]);
        if (d < bd) { bd = d; bs = t; }
      }
      atomicAdd(&s_stat[bs], 1ull);
      const int rgb[3] = {r, g, b};
      for (int c = 0; c < 3; c++) {
        atomicAdd(&s_stat[4 + bs * 3 + c], (unsigned long long)(2 * rgb[c]));
        atomicAdd(&s_stat[16 + bs * 3 + c], (unsigned long long)(rgb[c] * rgb[c]));
      }
      atomicAdd(&s_stat[28], (unsigned long long)bd);
    });
    __syncthreads();
    const unsigned long long true_err = s_stat[28];
    if (true_err >= keep_err) break;  // uniform: every thread reads the same shared value
    keep_err = true_err;
    keepL = L0;
    keepH = H0;
    if (threadIdx.x < 32) {
      // the walk runs on warp 0: lane 0 lists the moves, the lanes score them, exactly in 64-bit
      // integers (the histogram sums are exact, so the reference's double sums are these values)
      const int lane = threadIdx.x;
      long long hist[4], D2[4][3], DD[4][3];
      for (int q = 0; q < 4; q++) {
        hist[q] = (long long)s_stat[q];
        for (int c = 0; c < 3; c++) { D2[q][c] = (long long)s_stat[4 + q * 3 + c]; DD[q][c] = (long long)s_stat[16 + q * 3 + c]; }
      }
      auto err_of = [&](uint32_t L, uint32_t H) {
        int cc[4][3];
        colors4(L, H, cc);
        long long er = 0;
        for (int q = 0; q < 4; q++) {
          long long d[3];
          for (int c = 0; c < 3; c++) d[c] = hist[q] * cc[q][c] * cc[q][c] - D2[q][c] * cc[q][c] + DD[q][c];
          er += perc ? d[0] * 8 + d[1] * 25 + d[2] : d[0] + d[1] + d[2];
        }
        return er;
      };
      uint32_t wL = L0, wH = H0;
      long long best = err_of(wL, wH);
      const bool preserveL = hist[0] + hist[2] > hist[1] + hist[3];
      bool improved = true;
      for (int iters = 8; improved && iters; iters--) {
        improved = false;
        if (lane == 0) {
          int ns = 0;
          for (int which = 0; which < 2; which++) {
            const uint32_t E = which ? wH : wL, O2 = which ? wL : wH;
            const int b0 = E & 31, g0 = (E >> 5) & 63, r0 = (E >> 11) & 31;
            for (int b = b0 ? b0 - 1 : b0; b <= b0 + 1 && b <= 31; b++)
              for (int g = g0 ? g0 - 1 : g0; g <= g0 + 1 && g <= 63; g++)
                for (int r = r0 ? r0 - 1 : r0; r <= r0 + 1 && r <= 31; r++) {
                  const uint32_t X = (uint32_t)((r << 11) | (g << 5) | b);
                  if (X != E) s_sol[ns++] = X > O2 ? (X | (O2 << 16)) : (O2 | (X << 16));
                }
          }
          for (int i = 1; i < ns; i++) {  // sorted, as the reference evaluates them
            const uint32_t x = s_sol[i];
            int j = i - 1;
            while (j >= 0 && s_sol[j] > x) { s_sol[j + 1] = s_sol[j]; j--; }
            s_sol[j + 1] = x;
          }
          s_nsol = (uint32_t)ns;
        }
        __syncwarp();
        const int ns = (int)s_nsol;
        // the first strictly better move in sorted order wins ties: (error, index) minimum
        long long le = LLONG_MAX;
        int li = 0x7FFFFFFF;
        for (int i = lane; i < ns; i += 32) {
          if (i && s_sol[i] == s_sol[i - 1]) continue;
          uint32_t L = s_sol[i] & 0xFFFFu, H = s_sol[i] >> 16;
          if (L == H) {
            L += !preserveL ? ((~L & 0x1F) ? 0x1 : (~L & 0xF800) ? 0x800 : (~L & 0x7E0) ? 0x20 : 0) : (!L ? 0x1 : 0);
            H -= preserveL ? ((H & 0x1F) ? 0x1 : (H & 0xF800) ? 0x800 : (H & 0x7E0) ? 0x20 : 0) : (H == 0xFFFF ? 0x1 : 0);
            L &= 0xFFFFu; H &= 0xFFFFu;
          }
          const long long er = err_of(L, H);
          if (er < le) { le = er; li = i; }
        }
        for (int o = 16; o > 0; o >>= 1) {
          const long long oe = __shfl_xor_sync(0xFFFFFFFFu, le, o);
          const int oi = __shfl_xor_sync(0xFFFFFFFFu, li, o);
          if (oe < le || (oe == le && oi < li)) { le = oe; li = oi; }
        }
        if (le < best) {
          best = le;
          uint32_t L = s_sol[li] & 0xFFFFu, H = s_sol[li] >> 16;
          if (L == H) {
            L += !preserveL ? ((~L & 0x1F) ? 0x1 : (~L & 0xF800) ? 0x800 : (~L & 0x7E0) ? 0x20 : 0) : (!L ? 0x1 : 0);
            H -= preserveL ? ((H & 0x1F) ? 0x1 : (H & 0xF800) ? 0x800 : (H & 0x7E0) ? 0x20 : 0) : (H == 0xFFFF ? 0x1 : 0);
            L &= 0xFFFFu; H &= 0xFFFFu;
          }
          wL = L; wH = H;
          improved = true;
        }
        __syncwarp();  // s_sol is rewritten by lane 0 in the next step
        if (best == 0) break;
      }
      if (wL <= wH) {  // keep 4-colour order (first > second)
        if (wL == wH) { if (wL < 0xFFFFu) wL++; else wH--; }
        else { const uint32_t t = wL; wL = wH; wH = t; }
      }
      if (lane == 0) {
        s_LH[0] = wL;
        s_LH[1] = wH;
      }
    }
    __syncthreads();
    if (s_LH[0] == L0 && s_LH[1] == H0) break;
    L0 = s_LH[0];
    H0 = s_LH[1];
  }
  if (threadIdx.x == 0) {
    O.first = keepL;
    O.second = keepH;
    int col[4][3];
    colors4(keepL, keepH, col);
    for (int i = 0; i < 4; i++)
      for (int c = 0; c < 3; c++) O.col[i][c] = col[c_from_linear[i]][c];
  }
}

// ------------------------------------------------------------------------------------------
// Per-block selectors (linear order) against the cluster's colours and selector-codebook weights
// (crn_dxt_hc.cpp:699-733). key = selector << 32 | weight (the reference's m_block_selectors).
__global__ void k_block_selectors(const uint32_t* __restrict__ blocks, uint32_t nblocks,
                                  const uint32_t* __restrict__ block_tile, const uint32_t* __restrict__ tile_cluster,
                                  const uint8_t* __restrict__ block_enc, const float* __restrict__ block_weight,
                                  const ClusterOut* __restrict__ cl, int perceptual, uint32_t* __restrict__ block_cluster,
                                  float* __restrict__ sel_vec /* n x 16 */, uint32_t* __restrict__ sel_w,
                                  unsigned long long* __restrict__ sse) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nblocks) return;
  const bool perc = perceptual != 0;
  const uint32_t k = tile_cluster[block_tile[b]];
  block_cluster[b] = k;
  const ClusterOut& C = cl[k];
  const uint32_t ew = cdist(perc, C.col[0][0], C.col[0][1], C.col[0][2], C.col[3][0], C.col[3][1], C.col[3][2]) / 2000;
  const float enc_w = 1.15f + (1.0f - 1.15f) * ((float)block_enc[b] / 7.0f);
  float wf = (float)ew * block_weight[b];
  wf = wf < 1.f ? 1.f : (wf > 2048.f ? 2048.f : wf);
  const uint32_t weight = (uint32_t)((float)(uint32_t)wf * enc_w);
  uint32_t rgb_sse = 0;
  for (int p = 0; p < 16; p++) {
    const uint32_t px = __ldg(blocks + (size_t)b * 16 + p);
    uint32_t bd = 0xFFFFFFFFu;
    int bs = 0;
    for (int t = 0; t < 4; t++) {
      const int s = c_to_linear[t];
      const uint32_t d = cdist(perc, px_r(px), px_g(px), px_b(px), C.col[s][0], C.col[s][1], C.col[s][2]);
      if (d < bd) { bd = d; bs = s; }
    }
    sel_vec[(size_t)b * 16 + p] = ((float)bs + 0.5f) * 0.25f;  // vector component v[s] = (s + 0.5) / 4
    rgb_sse += cdist(false, px_r(px), px_g(px), px_b(px), C.col[bs][0], C.col[bs][1], C.col[bs][2]);
  }
  sel_w[b] = weight;
  atomicAdd(sse, (unsigned long long)rgb_sse);
}

// codebook vectors -> 2-bit linear selectors (crn_dxt_hc.cpp:1468-1476)
__global__ void k_selector_quantise(const float* __restrict__ cb, uint32_t K, uint32_t* __restrict__ sel) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K) return;
  uint32_t s = 0;
  for (int j = 0; j < 16; j++) s |= (uint32_t)min(3, max(0, (int)(cb[(size_t)i * 16 + j] * 4.0f))) << (2 * j);
  sel[i] = s;
}

// Best selector-codebook entry per block through the E2/E4/E8 tables (crn_dxt_hc.cpp:1306-1360),
// one warp per block; per-entry error tables accumulate (for the re-optimisation) in 64 bits.
constexpr int kSelWarps = 8;
__global__ void __launch_bounds__(kSelWarps * 32) k_selector_assign(const uint32_t* __restrict__ blocks, uint32_t nblocks,
                                                                     const uint32_t* __restrict__ block_cluster,
                                                                     const ClusterOut* __restrict__ cl, int perceptual,
                                                                     const uint32_t* __restrict__ cbsel, uint32_t K,
                                                                     uint32_t* __restrict__ block_sel,
                                                                     unsigned long long* __restrict__ entry_err /* K x 64 */,
                                                                     uint32_t* __restrict__ entry_used) {
  __shared__ uint32_t s_E8[kSelWarps][4][256];
  __shared__ uint32_t s_E2[kSelWarps][16][4];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t b = blockIdx.x * kSelWarps + warp;
  if (b >= nblocks) return;
  const bool perc = perceptual != 0;
  const ClusterOut& C = cl[block_cluster[b]];
  for (int q = lane; q < 64; q += 32) {
    const int p = q >> 2, s = q & 3;
    const uint32_t px = __ldg(blocks + (size_t)b * 16 + p);
    s_E2[warp][p][s] = cdist(perc, px_r(px), px_g(px), px_b(px), C.col[s][0], C.col[s][1], C.col[s][2]);
  }
  __syncwarp();
  // E8[p][s]: pixels 4p..4p+3 with selectors s (2 bits each, pixel 4p in the low bits)
  for (int q = lane; q < 1024; q += 32) {
    const int p = q >> 8, s = q & 255;
    s_E8[warp][p][s] = s_E2[warp][4 * p][s & 3] + s_E2[warp][4 * p + 1][(s >> 2) & 3] + s_E2[warp][4 * p + 2][(s >> 4) & 3] +
                       s_E2[warp][4 * p + 3][s >> 6];
  }
  __syncwarp();
  uint32_t best = 0xFFFFFFFFu, bi = 0;
  for (uint32_t i = lane; i < K; i += 32) {
    const uint32_t sel = __ldg(cbsel + i);
    const uint32_t er = s_E8[warp][0][sel & 255] + s_E8[warp][1][(sel >> 8) & 255] + s_E8[warp][2][(sel >> 16) & 255] +
                        s_E8[warp][3][sel >> 24];
    if (er < best) { best = er; bi = i; }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const uint32_t ob = __shfl_xor_sync(0xFFFFFFFFu, best, o), oi = __shfl_xor_sync(0xFFFFFFFFu, bi, o);
    if (ob < best || (ob == best && oi < bi)) { best = ob; bi = oi; }
  }
  if (lane == 0) { block_sel[b] = bi; entry_used[bi] = 1; }
  for (int q = lane; q < 64; q += 32) atomicAdd(entry_err + (size_t)bi * 64 + q, (unsigned long long)s_E2[warp][q >> 2][q & 3]);
}

// per entry: the selector of each pixel minimising the accumulated error (crn_dxt_hc.cpp:1491-1503)
__global__ void k_selector_finalise(const unsigned long long* __restrict__ entry_err, uint32_t K, uint32_t* __restrict__ sel) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K) return;
  uint32_t s = 0;
  for (int p = 0; p < 16; p++) {
    const unsigned long long* e = entry_err + (size_t)i * 64 + p * 4;
    const int s03 = e[3] < e[0] ? 3 : 0, s12 = e[2] < e[1] ? 2 : 1;
    s |= (uint32_t)(e[s12] < e[s03] ? s12 : s03) << (2 * p);
  }
  sel[i] = s;
}

// finished DXT1 blocks: cluster endpoints + codebook selectors (linear -> DXT order)
__global__ void k_hc_emit(const uint32_t* __restrict__ blocks, uint32_t nblocks, const uint32_t* __restrict__ block_cluster,
                          const ClusterOut* __restrict__ cl, const uint32_t* __restrict__ block_sel,
                          const uint32_t* __restrict__ cbsel, uint8_t* __restrict__ out, uint32_t bpb, uint32_t ofs,
                          unsigned long long* __restrict__ sse) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nblocks) return;
  const ClusterOut& C = cl[block_cluster[b]];
  const uint32_t lin = cbsel[block_sel[b]];
  uint32_t dxt = 0, rgb_sse = 0;
  for (int p = 0; p < 16; p++) {
    const uint32_t l = (lin >> (2 * p)) & 3;
    dxt |= (uint32_t)c_from_linear[l] << (2 * p);
    const uint32_t px = __ldg(blocks + (size_t)b * 16 + p);
    rgb_sse += cdist(false, px_r(px), px_g(px), px_b(px), C.col[l][0], C.col[l][1], C.col[l][2]);
  }
  *reinterpret_cast<uint2*>(out + (size_t)b * bpb + ofs) = make_uint2(C.first | (C.second << 16), dxt);
  atomicAdd(sse, (unsigned long long)rgb_sse);
}

// cluster membership: count tiles per cluster (CSR built on the host from the counts)
__global__ void k_count_clusters(const uint32_t* __restrict__ tile_cluster, uint32_t ntiles, uint32_t* __restrict__ counts) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < ntiles && tile_cluster[t] != 0xFFFFFFFFu) atomicAdd(counts + tile_cluster[t], 1u);
}

// used-tile flags (for the ordered compaction) and the identity permutation
__global__ void k_tile_flags(const Tile* __restrict__ tiles, uint32_t ntiles, uint8_t* __restrict__ flag,
                             uint32_t* __restrict__ iota) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntiles) return;
  flag[t] = tiles[t].kind != 0xFFu ? 1 : 0;
  iota[t] = t;
}
// tile vectors and weights of the used tiles, in tile order, for the endpoint VQ
__global__ void k_tile_vectors(const Tile* __restrict__ tiles, const uint32_t* __restrict__ used, uint32_t nused,
                               float* __restrict__ vec, uint32_t* __restrict__ w) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nused) return;
  const Tile& T = tiles[used[i]];
  for (int k = 0; k < 6; k++) vec[(size_t)i * 6 + k] = T.v[k];
  w[i] = (uint32_t)T.weight;
}
// cluster of each used tile (sort key) and the tile index (value)
__global__ void k_used_clusters(const uint32_t* __restrict__ used, uint32_t nused, const uint32_t* __restrict__ tile_cluster,
                                uint32_t* __restrict__ key) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nused) key[i] = tile_cluster[used[i]];
}

__global__ void k_block_weights(const Level* __restrict__ lv, uint32_t nlev, uint32_t nblocks, float* __restrict__ bw) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nblocks) return;
  float w = 1.f;
  for (uint32_t l = 0; l < nlev; l++)
    if (b >= lv[l].first_block && b < lv[l].first_block + lv[l].num_blocks) w = lv[l].weight;
  bw[b] = w;
}


// ------------------------------------------------------------------------------------------
// Alpha channels (DXT5 alpha, DXT5A, the two DXN channels): vec2 endpoint VQ over the tiles'
// palettize_alpha pairs, per-cluster dxt5_endpoint_optimizer + dxt_endpoint_refiner::optimize_dxt5,
// 3-bit selector codebook (crn_dxt_hc.cpp:1014-1300, 1506-1720).

__constant__ uint8_t c_from_linear8[8] = {0, 2, 3, 4, 5, 6, 7, 1};  // g_dxt5_from_linear
__constant__ uint8_t c_to_linear8[8] = {0, 7, 1, 2, 3, 4, 5, 6};    // g_dxt5_to_linear

// dxt5_block::get_block_values8 / 6 (crnlib/crn_dxt.cpp:369-431)
__host__ __device__ __forceinline__ void alpha_values8(int l, int h, int* v) {
  v[0] = l; v[1] = h;
  v[2] = (l * 6 + h) / 7; v[3] = (l * 5 + h * 2) / 7; v[4] = (l * 4 + h * 3) / 7;
  v[5] = (l * 3 + h * 4) / 7; v[6] = (l * 2 + h * 5) / 7; v[7] = (l + h * 6) / 7;
}
__host__ __device__ __forceinline__ void alpha_values(int l, int h, int* v) {
  if (l > h) { alpha_values8(l, h, v); return; }
  v[0] = l; v[1] = h;
  v[2] = (l * 4 + h) / 5; v[3] = (l * 3 + h * 2) / 5; v[4] = (l * 2 + h * 3) / 5; v[5] = (l + h * 4) / 5;
  v[6] = 0; v[7] = 255;
}

struct AlphaCluster {
  uint32_t first, second;  // final endpoints (first > second: 8-value block), after the refiner
  int vals[8];             // linear-order values of the optimizer's endpoints (block selectors, search)
  int rvals[8];            // linear-order values of the final endpoints (error accumulation)
  uint32_t endpoint_weight;
};

// tile -> nearest alpha codebook entry per channel (determine_alpha_endpoint_clusters_task, :1132-1163)
__global__ void k_nearest_vec2(const Tile* __restrict__ tiles, const uint32_t* __restrict__ used, uint32_t nused,
                               int num_alpha, const float* __restrict__ cb, uint32_t K, uint32_t* __restrict__ tile_ac) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nused * (uint32_t)num_alpha) return;
  const uint32_t a = i / nused, t = used[i - a * nused];
  const float v0 = tiles[t].va[a][0], v1 = tiles[t].va[a][1];
  float best = 3.4e38f;
  uint32_t bi = 0;
  for (uint32_t k = 0; k < K; k++) {
    const float d = (cb[2 * k] - v0) * (cb[2 * k] - v0) + (cb[2 * k + 1] - v1) * (cb[2 * k + 1] - v1);
    if (d < best) { best = d; bi = k; if (best == 0.0f) break; }
  }
  tile_ac[2 * t + a] = bi;
}

// alpha VQ input: (channel-major) the used tiles' vec2 with their pixel counts as weights
// qdxt: the tile's training weight (qdxt5's distance weight x its blocks); else its pixel count
__global__ void k_alpha_vectors(const Tile* __restrict__ tiles, const uint32_t* __restrict__ used, uint32_t nused,
                                int num_alpha, int qdxt, float* __restrict__ vec, uint32_t* __restrict__ w,
                                uint32_t* __restrict__ key_item) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nused * (uint32_t)num_alpha) return;
  const uint32_t a = i / nused, t = used[i - a * nused];
  vec[2 * i] = tiles[t].va[a][0];
  vec[2 * i + 1] = tiles[t].va[a][1];
  w[i] = qdxt ? (uint32_t)tiles[t].weight : tile_npix(tiles[t].kind);
  key_item[i] = 2 * t + a;
}
__global__ void k_alpha_keys(const uint32_t* __restrict__ items, uint32_t n, const uint32_t* __restrict__ tile_ac,
                             uint32_t* __restrict__ key, uint32_t* __restrict__ counts) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  key[i] = tile_ac[items[i]];
  atomicAdd(counts + key[i], 1u);
}

constexpr int kAFitThreads = 256;

// error of the 8-value block (l, h) over a value histogram, each value on its nearest palette
// value, from prefix sums P0 (count), P1 (sum v), P2 (sum v^2) of 257 entries
__device__ __forceinline__ unsigned long long alpha_pair_error(int l, int h, const unsigned long long* P0,
                                                               const unsigned long long* P1, const unsigned long long* P2) {
  int q[8];
  alpha_values8(l, h, q);
  for (int i = 1; i < 8; i++) {  // sort the 8 values ascending
    const int x = q[i];
    int j = i - 1;
    while (j >= 0 && q[j] > x) { q[j + 1] = q[j]; j--; }
    q[j + 1] = x;
  }
  long long e = 0;
  int lo = 0;
  for (int k = 0; k < 8; k++) {
    const int hi = k < 7 ? (q[k] + q[k + 1]) >> 1 : 255;
    if (hi >= lo) {
      const long long s0 = (long long)(P0[hi + 1] - P0[lo]), s1 = (long long)(P1[hi + 1] - P1[lo]),
                      s2 = (long long)(P2[hi + 1] - P2[lo]);
      e += s2 - 2 * (long long)q[k] * s1 + (long long)q[k] * q[k] * s0;
      lo = hi + 1;
    }
  }
  return (unsigned long long)e;
}

// CTA-wide minimum of (error, key)
__device__ __forceinline__ void block_min_pair(unsigned long long& e, uint32_t& key, unsigned long long* se, uint32_t* sk) {
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long oe = __shfl_xor_sync(0xFFFFFFFFu, e, o);
    const uint32_t ok = __shfl_xor_sync(0xFFFFFFFFu, key, o);
    if (oe < e || (oe == e && ok < key)) { e = oe; key = ok; }
  }
  __syncthreads();
  if ((threadIdx.x & 31) == 0) { se[threadIdx.x >> 5] = e; sk[threadIdx.x >> 5] = key; }
  __syncthreads();
  e = se[0]; key = sk[0];
  for (int w = 1; w < (int)(blockDim.x >> 5); w++)
    if (se[w] < e || (se[w] == e && sk[w] < key)) { e = se[w]; key = sk[w]; }
  __syncthreads();
}

// Per alpha cluster (determine_alpha_endpoint_codebook_task, :1014-1130): the histogram of the
// cluster's values, dxt5_endpoint_optimizer at uber quality with 8-value blocks (all pairs of
// unique values, then the +-16 grid around the best, crnlib/crn_dxt5a.cpp:40-196) evaluated
// exactly through prefix sums, then dxt_endpoint_refiner::optimize_dxt5
// (crnlib/crn_dxt_endpoint_refiner.cpp:36-201).
__global__ void __launch_bounds__(kAFitThreads) k_alpha_cluster_fit(const uint32_t* __restrict__ blocks,
                                                                     const Chunk* __restrict__ chunks,
                                                                     const Tile* __restrict__ tiles, TileCfg cfg,
                                                                     const uint32_t* __restrict__ start,
                                                                     const uint32_t* __restrict__ members,
                                                                     AlphaCluster* __restrict__ out) {
  __shared__ uint32_t hist[256];
  __shared__ unsigned long long P0[257], P1[257], P2[257];
  __shared__ uint8_t uv[256];
  __shared__ uint32_t s_nu;
  __shared__ unsigned long long se[kAFitThreads / 32];
  __shared__ uint32_t sk[kAFitThreads / 32];
  const uint32_t k = blockIdx.x;
  const uint32_t m0 = start[k], m1 = start[k + 1];
  AlphaCluster& O = out[k];
  if (m0 == m1) {
    if (threadIdx.x == 0) { O.first = O.second = 0; for (int i = 0; i < 8; i++) O.vals[i] = O.rvals[i] = 0; O.endpoint_weight = 1; }
    return;
  }
  for (int i = threadIdx.x; i < 256; i += blockDim.x) hist[i] = 0;
  __syncthreads();
  for (uint32_t m = m0 + (threadIdx.x >> 6); m < m1; m += blockDim.x >> 6) {  // 64 threads per member tile
    const uint32_t item = members[m], t = item >> 1, a = item & 1;
    const Tile& T = tiles[t];
    const uint32_t j = threadIdx.x & 63;
    if (j < tile_npix(T.kind)) {
      const uint32_t v = (tile_pixel(blocks, chunks[T.chunk], T.kind, j) >> (8 * cfg.comp[a])) & 255u;
      atomicAdd(&hist[v], 1u);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    P0[0] = P1[0] = P2[0] = 0;
    uint32_t nu = 0;
    for (int v = 0; v < 256; v++) {
      P0[v + 1] = P0[v] + hist[v];
      P1[v + 1] = P1[v] + (unsigned long long)hist[v] * v;
      P2[v + 1] = P2[v] + (unsigned long long)hist[v] * v * v;
      if (hist[v]) uv[nu++] = (uint8_t)v;
    }
    s_nu = nu;
  }
  __syncthreads();
  const int U = (int)s_nu;
  int first, second;
  unsigned long long best;
  if (U == 1) {
    first = second = uv[0];
    best = 0;
  } else {
    // all pairs of unique values
    unsigned long long be = ~0ull;
    uint32_t bk = 0xFFFFFFFFu;
    for (int i = threadIdx.x; i < U - 1; i += blockDim.x)
      for (int j = i + 1; j < U; j++) {
        const unsigned long long e = alpha_pair_error(uv[i], uv[j], P0, P1, P2);
        const uint32_t key = (uint32_t)(i * 256 + j);
        if (e < be || (e == be && key < bk)) { be = e; bk = key; }
      }
    block_min_pair(be, bk, se, sk);
    first = uv[bk >> 8];
    second = uv[bk & 255];
    best = be;
    if (best) {
      // +-16 probe grid around the best pair
      unsigned long long ge = best;
      uint32_t gk = 0xFFFFFFFFu;
      for (int i = threadIdx.x; i < 33 * 33; i += blockDim.x) {
        const int l = first + i / 33 - 16, h = second + i % 33 - 16;
        if (l < 0 || l > 255 || h < 0 || h > 255) continue;
        const unsigned long long e = alpha_pair_error(l, h, P0, P1, P2);
        if (e < ge || (e == ge && (uint32_t)i < gk)) { ge = e; gk = (uint32_t)i; }
      }
      block_min_pair(ge, gk, se, sk);
      if (gk != 0xFFFFFFFFu && ge < best) {
        best = ge;
        const int l = first + (int)(gk / 33) - 16, h = second + (int)(gk % 33) - 16;
        first = l;
        second = h;
      }
    }
  }
  // 8-value blocks need first > second (the reference swaps and inverts the selectors)
  if (first <= second) { const int t = first; first = second; second = t; }
  if (threadIdx.x == 0) {
    int bv[8];
    alpha_values(first, second, bv);
    for (int i = 0; i < 8; i++) O.vals[i] = bv[c_from_linear8[i]];
    const int delta = first - second;
    O.endpoint_weight = (uint32_t)min(max((delta * delta) >> 3, 1), 2048);
    // refiner: least squares from the DXT-order selectors of every value, then the +-11 grid
    uint32_t L = (uint32_t)first, H = (uint32_t)second;
    if (U > 1 && best) {
      double a2 = 0, b2 = 0, ab = 0, ax = 0, bx = 0;
      double hs[8] = {0, 0, 0, 0, 0, 0, 0, 0}, d2[8] = {0, 0, 0, 0, 0, 0, 0, 0}, dd[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      double first_x = uv[0] / 255.0;
      for (int u = 0; u < U; u++) {
        const int v = uv[u];
        const double c = hist[v];
        int bs = 0, bd = 0x7FFFFFFF;
        for (int j = 0; j < 8; j++) { const int d = (v - bv[j]) * (v - bv[j]); if (d < bd) { bd = d; bs = j; } }
        const double kk = (double)c_to_linear8[bs] * (double)(1.0f / 7.0f);
        const double al = 1.0 - kk, be2 = kk, x = (double)((float)v * (1.0f / 255.0f));
        a2 += c * al * al; b2 += c * be2 * be2; ab += c * al * be2; ax += c * al * x; bx += c * be2 * x;
        hs[bs] += c; d2[bs] += c * 2 * v; dd[bs] += c * v * v;
      }
      double ea, eb;
      if (b2 == 0.0) { ea = ax / a2; eb = 0; }
      else if (a2 == 0.0) { ea = 0; eb = bx / b2; }
      else {
        const double f = a2 * b2 - ab * ab;
        if (f != 0.0) { ea = (ax * b2 - bx * ab) / f; eb = (bx * a2 - ax * ab) / f; }
        else { ea = eb = first_x; }
      }
      const float lf = fminf(fmaxf((float)ea, 0.f), 1.f), hf = fminf(fmaxf((float)eb, 0.f), 1.f);
      const int L0 = clampi((int)(lf * 256.0f), 0, 255), H0 = clampi((int)(hf * 256.0f), 0, 255);
      auto norm = [](int l, int h) -> uint32_t {
        return l == h ? (h ? ((uint32_t)(h - 1) << 8 | (uint32_t)l) : 1u) : (l > h ? ((uint32_t)h << 8 | (uint32_t)l) : ((uint32_t)l << 8 | (uint32_t)h));
      };
      unsigned long long rbest = ~0ull;
      uint32_t rsol = 0;
      auto eval = [&](uint32_t sol) {
        int v[8];
        alpha_values8((int)(sol & 255), (int)(sol >> 8), v);
        double er = 0;
        for (int q = 0; q < 8; q++) er += hs[q] * v[q] * v[q] - d2[q] * v[q] + dd[q];
        const unsigned long long e = (unsigned long long)(er + 0.5);
        if (e < rbest) { rbest = e; rsol = sol; }
      };
      eval(norm(L0, H0));
      const int minL = L0 <= 11 ? 0 : L0 - 11, maxL = L0 >= 244 ? 255 : L0 + 11;
      const int minH = H0 <= 11 ? 0 : H0 - 11, maxH = H0 >= 244 ? 255 : H0 + 11;
      for (int l = minL; l <= maxL && rbest; l++)
        for (int h = minH; h <= maxH && rbest; h++)
          if ((maxH < l || l <= h || h < minL) && (l != L0 || h != H0) && (l != H0 || h != L0)) eval(norm(l, h));
      if (rbest < best) { L = rsol & 255; H = rsol >> 8; }
    }
    O.first = L;
    O.second = H;
    int rv[8];
    alpha_values((int)L, (int)H, rv);
    for (int i = 0; i < 8; i++) O.rvals[i] = rv[c_from_linear8[i]];
  }
}

// Per (block, channel): 3-bit linear selectors against the cluster's values (absolute error, DXT
// order first-min) and the selector codebook weight (crn_dxt_hc.cpp:1076-1100); item = a * N + b.
__global__ void k_alpha_block_selectors(const uint32_t* __restrict__ blocks, uint32_t N, int num_alpha, TileCfg cfg,
                                        const uint32_t* __restrict__ block_tile, const uint32_t* __restrict__ tile_ac,
                                        const uint8_t* __restrict__ block_enc, const AlphaCluster* __restrict__ ac,
                                        uint32_t* __restrict__ item_cluster, float* __restrict__ sel_vec,
                                        uint32_t* __restrict__ sel_w) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N * (uint32_t)num_alpha) return;
  const uint32_t a = i / N, b = i - a * N;
  const uint32_t k = tile_ac[2 * block_tile[b] + a];
  item_cluster[i] = k;
  const AlphaCluster& C = ac[k];
  const float ew = 1.15f + (1.0f - 1.15f) * ((float)block_enc[b] / 7.0f);
  sel_w[i] = (uint32_t)((float)C.endpoint_weight * ew);
  for (int p = 0; p < 16; p++) {
    const int v = (int)((__ldg(blocks + (size_t)b * 16 + p) >> (8 * cfg.comp[a])) & 255u);
    int bd = 0x7FFFFFFF, bs = 0;
    for (int t = 0; t < 8; t++) {
      const int s = c_to_linear8[t];
      const int d = abs(v - C.vals[s]);
      if (d < bd) { bd = d; bs = s; }
    }
    sel_vec[(size_t)i * 16 + p] = ((float)bs + 0.5f) * 0.125f;
  }
}

__global__ void k_alpha_selector_quantise(const float* __restrict__ cb, uint32_t K, unsigned long long* __restrict__ sel) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K) return;
  unsigned long long s = 0;
  for (int j = 0; j < 16; j++) s |= (unsigned long long)min(7, max(0, (int)(cb[(size_t)i * 16 + j] * 8.0f))) << (3 * j);
  sel[i] = s;
}

// Best alpha selector-codebook entry per (block, channel) through E3/E6 tables
// (create_alpha_selector_codebook_task, :1516-1580); per-entry tables accumulate with the final
// (refined) values. One warp per item.
constexpr int kASelWarps = 8;
__global__ void __launch_bounds__(kASelWarps * 32) k_alpha_selector_assign(
    const uint32_t* __restrict__ blocks, uint32_t N, int num_alpha, TileCfg cfg, const uint32_t* __restrict__ item_cluster,
    const AlphaCluster* __restrict__ ac, const unsigned long long* __restrict__ cbsel, uint32_t K,
    uint32_t* __restrict__ item_sel, unsigned long long* __restrict__ entry_err /* K x 128 */) {
  __shared__ uint32_t s_E6[kASelWarps][8][64];
  __shared__ uint32_t s_E3[kASelWarps][16][8];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t i = blockIdx.x * kASelWarps + warp;
  if (i >= N * (uint32_t)num_alpha) return;
  const uint32_t a = i / N, b = i - a * N;
  const AlphaCluster& C = ac[item_cluster[i]];
  for (int q = lane; q < 128; q += 32) {
    const int p = q >> 3, sidx = q & 7;
    const int v = (int)((__ldg(blocks + (size_t)b * 16 + p) >> (8 * cfg.comp[a])) & 255u);
    s_E3[warp][p][sidx] = (uint32_t)((v - C.vals[sidx]) * (v - C.vals[sidx]));
  }
  __syncwarp();
  for (int q = lane; q < 512; q += 32) {
    const int p = q >> 6, sv = q & 63;
    s_E6[warp][p][sv] = s_E3[warp][2 * p][sv & 7] + s_E3[warp][2 * p + 1][sv >> 3];
  }
  __syncwarp();
  uint32_t best = 0xFFFFFFFFu, bi = 0;
  for (uint32_t e = lane; e < K; e += 32) {
    const unsigned long long sel = __ldg(cbsel + e);
    uint32_t er = 0;
#pragma unroll
    for (int p = 0; p < 8; p++) er += s_E6[warp][p][(sel >> (6 * p)) & 63];
    if (er < best) { best = er; bi = e; }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const uint32_t ob = __shfl_xor_sync(0xFFFFFFFFu, best, o), oi = __shfl_xor_sync(0xFFFFFFFFu, bi, o);
    if (ob < best || (ob == best && oi < bi)) { best = ob; bi = oi; }
  }
  if (lane == 0) item_sel[i] = bi;
  for (int q = lane; q < 128; q += 32) {
    const int p = q >> 3, sidx = q & 7;
    const int v = (int)((__ldg(blocks + (size_t)b * 16 + p) >> (8 * cfg.comp[a])) & 255u);
    atomicAdd(entry_err + (size_t)bi * 128 + q, (unsigned long long)((v - C.rvals[sidx]) * (v - C.rvals[sidx])));
  }
}

// per entry: each pixel's selector minimising the accumulated error (crn_dxt_hc.cpp:1700-1715)
__global__ void k_alpha_selector_finalise(const unsigned long long* __restrict__ entry_err, uint32_t K,
                                          unsigned long long* __restrict__ sel) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K) return;
  unsigned long long s = 0;
  for (int p = 0; p < 16; p++) {
    const unsigned long long* e = entry_err + (size_t)i * 128 + p * 8;
    const int s07 = e[7] < e[0] ? 7 : 0, s12 = e[2] < e[1] ? 2 : 1, s34 = e[4] < e[3] ? 4 : 3, s56 = e[6] < e[5] ? 6 : 5;
    const int s02 = e[s12] < e[s07] ? s12 : s07, s36 = e[s56] < e[s34] ? s56 : s34;
    s |= (unsigned long long)(e[s36] < e[s02] ? s36 : s02) << (3 * p);
  }
  sel[i] = s;
}

// finished alpha blocks: endpoints + codebook selectors (linear -> DXT5 order) at byte offset
// 8 * slot of each output block; squared error of the result into *sse
__global__ void k_alpha_emit(const uint32_t* __restrict__ blocks, uint32_t N, int num_alpha, TileCfg cfg,
                             const uint32_t* __restrict__ item_cluster, const AlphaCluster* __restrict__ ac,
                             const uint32_t* __restrict__ item_sel, const unsigned long long* __restrict__ cbsel,
                             uint8_t* __restrict__ out, uint32_t bpb, int slot0, unsigned long long* __restrict__ sse) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N * (uint32_t)num_alpha) return;
  const uint32_t a = i / N, b = i - a * N;
  const AlphaCluster& C = ac[item_cluster[i]];
  const unsigned long long lin = cbsel[item_sel[i]];
  unsigned long long dxt = 0;
  uint32_t err = 0;
  for (int p = 0; p < 16; p++) {
    const uint32_t l = (uint32_t)((lin >> (3 * p)) & 7);
    dxt |= (unsigned long long)c_from_linear8[l] << (3 * p);
    const int v = (int)((__ldg(blocks + (size_t)b * 16 + p) >> (8 * cfg.comp[a])) & 255u);
    err += (uint32_t)((v - C.rvals[l]) * (v - C.rvals[l]));
  }
  uint8_t* o = out + (size_t)b * bpb + 8 * (slot0 + (int)a);
  o[0] = (uint8_t)C.first;
  o[1] = (uint8_t)C.second;
  for (int k = 0; k < 6; k++) o[2 + k] = (uint8_t)(dxt >> (8 * k));
  atomicAdd(sse, (unsigned long long)err);
}

}  // namespace hc

const void* single_colour_tables_host();

namespace {

struct HcBuffers {
  DevBuf chunks, derating, lweight, st, tiles, block_tile, block_enc, vec6, w6, count, cb6, tile_cluster, ccount,
      cstart, clist, clusters, bweight, block_cluster, selvec, selw, cb16, cbsel, block_sel, entry_err, entry_used,
      levels, flags, iota, used, keys, keys2, cub_tmp, sse, avec, aw, aitems, tile_ac, cb2, acount, alist, astart,
      aclusters, aitem_cluster, aselvec, aselw, acb16, acbsel, aitem_sel, aentry_err;
  hc::VqScratch vq;
  bool clean = true;  // the last call ended with its stream synchronised
};

// The clustered encoder's device buffers, one set per host thread and device, kept between calls
// (they only grow): a call then allocates nothing once the texture sizes have been seen. Every
// successful call ends by synchronising its stream, so the next call may reuse them on any stream;
// after a failed call the device is synchronised first.
HcBuffers& hc_workspace() {
  static thread_local std::unique_ptr<HcBuffers> ws[64];
  int dev = 0;
  cudaGetDevice(&dev);
  std::unique_ptr<HcBuffers>& w = ws[dev & 63];
  if (!w) w.reset(new HcBuffers);
  if (!w->clean) {
    cudaDeviceSynchronize();
    w->clean = true;
  }
  return *w;
}

}  // namespace

}  // namespace crngpu

using namespace crngpu;
using namespace crngpu::hc;

namespace crngpu {
namespace {

// dxt_hc::compress (crnlib/crn_dxt_hc.cpp:97-316) for DXT1, DXT5, DXN_XY/YX and DXT5A.
// Variant of the clustered encode: dxt_hc's (the .crn path) or qdxt1's (clustered DDS): its
// tiling, training vectors and codebook sizes from the full codebook and selector counts.
struct HcMode {
  bool qdxt = false;
  float quality = 1.0f;        // qdxt: quality level / 255
  float power_mul = 1.0f;      // qdxt: codebook-size curve exponent multiplier
  uint32_t selector_base = 0;  // qdxt: distinct dxt_fast selector words + 128
  float derate_div = 3.1f;     // qdxt: per-level derating divisor (qdxt1 3.1, qdxt5 3.0)
};

// The number of distinct D-float training vectors (the size of the full codebook qdxt's tree
// clusterizer reaches before it runs out of splits, crnlib/crn_qdxt1.cpp:335-345,
// crnlib/crn_qdxt5.cpp:384-392); at most 65535 (cMaxEndpointClusters).
uint32_t distinct_vectors(const float* d_vec, uint32_t n, int D, cudaStream_t s) {
  std::vector<float> v((size_t)n * D);
  if (!n || cudaMemcpyAsync(v.data(), d_vec, v.size() * sizeof(float), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return n;
  // qdxt's training vectors are 8-bit endpoint components: packed into one 64-bit key each
  bool bytes = D <= 8;
  for (size_t i = 0; i < v.size() && bytes; i++) bytes = v[i] >= 0.0f && v[i] <= 255.0f && v[i] == (float)(int)v[i];
  if (bytes) {
    std::vector<uint64_t> keys(n);
    for (uint32_t i = 0; i < n; i++) {
      uint64_t k = 0;
      for (int c = 0; c < D; c++) k = (k << 8) | (uint64_t)(int)v[(size_t)i * D + c];
      keys[i] = k;
    }
    std::sort(keys.begin(), keys.end());
    return std::min<uint32_t>((uint32_t)(std::unique(keys.begin(), keys.end()) - keys.begin()), 65535u);
  }
  std::vector<uint32_t> idx(n);
  for (uint32_t i = 0; i < n; i++) idx[i] = i;
  auto less = [&](uint32_t a, uint32_t b) {
    return std::lexicographical_compare(&v[(size_t)a * D], &v[(size_t)a * D + D], &v[(size_t)b * D], &v[(size_t)b * D + D]);
  };
  std::sort(idx.begin(), idx.end(), less);
  uint32_t d = n ? 1 : 0;
  for (uint32_t i = 1; i < n; i++)
    if (less(idx[i - 1], idx[i])) d++;
  return std::min<uint32_t>(d, 65535u);
}

int hc_compress_impl(const uint8_t* d_blocks, const crngpu_hc_params& P, uint32_t format, uint8_t* d_out,
                     uint16_t* d_endpoint_idx, uint16_t* d_selector_idx, uint32_t* d_endpoints, uint32_t* d_selectors,
                     crngpu_hc_stats* stats, cudaStream_t s, const HcMode& mode = HcMode()) {
  const uint32_t N = P.num_blocks;
  cudaError_t e;
  HcBuffers& B = hc_workspace();
  B.clean = false;
  TileCfg cfg{};
  uint32_t bpb = 8, color_ofs = 0;
  int alpha_slot0 = 0;
  switch (format) {
    case CRNGPU_FMT_DXT1: cfg.has_color = 1; cfg.num_alpha = 0; break;
    case CRNGPU_FMT_DXT5: cfg.has_color = 1; cfg.num_alpha = 1; cfg.comp[0] = (int)(P.alpha_component & 3); bpb = 16; color_ofs = 8; break;
    case CRNGPU_FMT_DXN_XY: cfg.num_alpha = 2; cfg.comp[0] = 0; cfg.comp[1] = 1; bpb = 16; break;
    case CRNGPU_FMT_DXN_YX: cfg.num_alpha = 2; cfg.comp[0] = 1; cfg.comp[1] = 0; bpb = 16; break;
    case CRNGPU_FMT_DXT5A: cfg.num_alpha = 1; cfg.comp[0] = (int)(P.alpha_component & 3); break;
    default: set_error("clustered compression supports DXT1, DXT5, DXN_XY/YX and DXT5A"); return CRNGPU_E_UNSUPPORTED;
  }
  cfg.ratio = P.color_alpha_weighting_ratio > 0.f ? P.color_alpha_weighting_ratio : 3.0f;
  cfg.qdxt = mode.qdxt ? 1 : 0;
  // codebook sizes: the caller's (dxt_hc), or qdxt1::pack's curves (crnlib/crn_qdxt1.cpp:925-935):
  // the full endpoint codebook (one entry per distinct training vector, at most 65535) scaled by
  // quality^(1.8 m), at least 96; the selector base scaled by quality^(1.65 m), at least 128
  auto ce_request = [&](uint32_t nvec) -> uint32_t {
    if (!mode.qdxt) return std::min(nvec, P.color_endpoint_codebook_size);
    const uint32_t cb = std::min<uint32_t>(nvec, 65535u);
    const uint32_t k = (uint32_t)(cb * powf(mode.quality, 1.8f * mode.power_mul));
    return std::max(std::min(k, cb), std::min(96u, cb));
  };
  auto cs_request = [&](uint32_t nvec) -> uint32_t {
    if (!mode.qdxt) return std::min(nvec, P.color_selector_codebook_size);
    const uint32_t sb = mode.selector_base;
    const uint32_t k = (uint32_t)(sb * powf(mode.quality, 1.65f * mode.power_mul));
    return std::min(nvec, std::max(std::min(k, sb), std::min(128u, sb)));
  };
  // qdxt5::pack (crnlib/crn_qdxt5.cpp:845-850): endpoints quality^2.1 of the full codebook, at
  // least 16; selectors quality^1.65 of the distinct dxt_fast alpha selectors + 128, at least 32
  auto ae_request = [&](uint32_t nvec) -> uint32_t {
    if (!mode.qdxt) return std::min(nvec, P.alpha_endpoint_codebook_size);
    const uint32_t cb = std::min<uint32_t>(nvec, 65535u);
    const uint32_t k = (uint32_t)(cb * powf(mode.quality, 2.1f));
    return std::max(std::min(k, cb), std::min(16u, cb));
  };
  auto as_request = [&](uint32_t nvec) -> uint32_t {
    if (!mode.qdxt) return std::min(nvec, P.alpha_selector_codebook_size);
    const uint32_t sb = mode.selector_base;
    const uint32_t k = (uint32_t)(sb * powf(mode.quality, 1.65f));
    return std::min(nvec, std::max(std::min(k, sb), std::min(32u, sb)));
  };
  const int tile_derating[8] = {0, 1, 1, 2, 2, 2, 2, 3};
  for (int k = 0; k < 8; k++) cfg.alpha_derating[k] = P.adaptive_tile_alpha_psnr_derating * ((float)tile_derating[k] / 3.0f);
  // chunks of every level (block rows are processed in pairs; widths and heights are even)
  std::vector<Chunk> chunks;
  std::vector<float> derating(16 * 8), lweight(16);
  std::vector<Level> lv(P.num_levels);
  for (uint32_t l = 0; l < P.num_levels; l++) {
    const auto& L = P.levels[l];
    if (!L.block_width || (L.block_width & 1) || L.num_blocks % (2 * L.block_width) || L.first_block + L.num_blocks > N) {
      set_error("clustered compression: level " + std::to_string(l) + " is not a whole number of 2x2 chunks");
      return CRNGPU_E_PARAM;
    }
    lv[l] = Level{L.first_block, L.num_blocks, L.block_width, L.weight};
    lweight[l] = L.weight;
    // crn_dxt_hc.cpp:121-134: colour derating per level and layout
    float d = P.adaptive_tile_color_psnr_derating;
    if (l && d > .25f) d = std::max(.25f, d / powf(mode.qdxt ? mode.derate_div : 3.0f, (float)l));
    for (int k = 0; k < 8; k++) derating[l * 8 + k] = 0.0f + (d - 0.0f) * ((float)tile_derating[k] / 3.0f);
    const uint32_t rows = L.num_blocks / L.block_width;
    for (uint32_t y = 0; y < rows; y += 2)
      for (uint32_t x = 0; x < L.block_width; x += 2) chunks.push_back(Chunk{L.first_block + y * L.block_width + x, L.block_width, l});
  }
  const uint32_t nchunks = (uint32_t)chunks.size(), ntiles = 4 * nchunks;
  auto up = [&](DevBuf& b, const void* src, size_t bytes) -> cudaError_t {
    cudaError_t r = b.ensure(bytes + 16);
    if (r != cudaSuccess) return r;
    return cudaMemcpyAsync(b.ptr, src, bytes, cudaMemcpyHostToDevice, s);
  };
  const void* st_host = single_colour_tables_host();
  if ((e = up(B.chunks, chunks.data(), sizeof(Chunk) * nchunks)) != cudaSuccess ||
      (e = up(B.derating, derating.data(), derating.size() * 4)) != cudaSuccess ||
      (e = up(B.lweight, lweight.data(), lweight.size() * 4)) != cudaSuccess ||
      (e = up(B.st, st_host, sizeof(SolidTables))) != cudaSuccess ||
      (e = up(B.levels, lv.data(), sizeof(Level) * lv.size())) != cudaSuccess)
    return cuda_check(e, "upload hc tables");
  if ((e = B.tiles.ensure(sizeof(Tile) * ntiles)) != cudaSuccess || (e = B.block_tile.ensure(4 * N)) != cudaSuccess ||
      (e = B.block_enc.ensure(N)) != cudaSuccess)
    return cuda_check(e, "alloc tiles");
  const uint32_t* blocks = reinterpret_cast<const uint32_t*>(d_blocks);
  Tile* tiles = static_cast<Tile*>(B.tiles.ptr);
  k_hc_tiles<<<(nchunks + 63) / 64, 64, 0, s>>>(blocks, static_cast<Chunk*>(B.chunks.ptr), nchunks,
                                                 static_cast<float*>(B.derating.ptr), static_cast<float*>(B.lweight.ptr),
                                                 P.perceptual, static_cast<SolidTables*>(B.st.ptr), cfg, tiles,
                                                 static_cast<uint32_t*>(B.block_tile.ptr), static_cast<uint8_t*>(B.block_enc.ptr));
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(e, "launch k_hc_tiles");
  // the used tiles, compacted in tile order (so the result is reproducible)
  if ((e = B.count.ensure(16)) != cudaSuccess || (e = B.flags.ensure(ntiles)) != cudaSuccess ||
      (e = B.iota.ensure(4 * ntiles)) != cudaSuccess || (e = B.used.ensure(4 * ntiles)) != cudaSuccess ||
      (e = B.keys.ensure(8 * ntiles)) != cudaSuccess || (e = B.keys2.ensure(8 * ntiles)) != cudaSuccess)
    return cuda_check(e, "alloc tile lists");
  k_tile_flags<<<(ntiles + 255) / 256, 256, 0, s>>>(tiles, ntiles, static_cast<uint8_t*>(B.flags.ptr),
                                                     static_cast<uint32_t*>(B.iota.ptr));
  size_t tmp_bytes = 0;
  cub::DeviceSelect::Flagged(nullptr, tmp_bytes, static_cast<uint32_t*>(B.iota.ptr), static_cast<uint8_t*>(B.flags.ptr),
                             static_cast<uint32_t*>(B.used.ptr), static_cast<uint32_t*>(B.count.ptr), (int)ntiles, s);
  if ((e = B.cub_tmp.ensure(tmp_bytes + 256)) != cudaSuccess) return cuda_check(e, "alloc cub scratch");
  tmp_bytes = B.cub_tmp.cap;
  if ((e = cub::DeviceSelect::Flagged(B.cub_tmp.ptr, tmp_bytes, static_cast<uint32_t*>(B.iota.ptr),
                                      static_cast<uint8_t*>(B.flags.ptr), static_cast<uint32_t*>(B.used.ptr),
                                      static_cast<uint32_t*>(B.count.ptr), (int)ntiles, s)) != cudaSuccess)
    return cuda_check(e, "select used tiles");
  uint32_t nused = 0;
  if ((e = cudaMemcpyAsync(&nused, B.count.ptr, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return cuda_check(e, "read count");
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_check(e, "sync");
  const uint32_t frac = P.vq_round_fraction ? P.vq_round_fraction : kDefaultRoundFraction;
  if ((e = B.sse.ensure(32)) != cudaSuccess) return cuda_check(e, "alloc sse");
  cudaMemsetAsync(B.sse.ptr, 0, 32, s);
  // sorts `n` (key, value) pairs with keys below 2^bits (stable: equal keys keep value order)
  auto sort_pairs = [&](uint32_t* keys, uint32_t* keys_out, uint32_t* vals, uint32_t* vals_out, uint32_t n,
                        int bits) -> int {
    size_t need = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, need, keys, keys_out, vals, vals_out, (int)n, 0, bits, s);
    cudaError_t r = B.cub_tmp.ensure(need + 256);
    if (r != cudaSuccess) return cuda_check(r, "alloc cub scratch");
    size_t have = B.cub_tmp.cap;
    r = cub::DeviceRadixSort::SortPairs(B.cub_tmp.ptr, have, keys, keys_out, vals, vals_out, (int)n, 0, bits, s);
    return r == cudaSuccess ? CRNGPU_OK : cuda_check(r, "radix sort");
  };
  // CSR starts from per-cluster counts (device) -> start (device), host round trip of K words
  auto csr_starts = [&](DevBuf& counts, DevBuf& starts, uint32_t K) -> int {
    std::vector<uint32_t> cnt(K + 1), st(K + 1);
    cudaError_t r = cudaMemcpyAsync(cnt.data(), counts.ptr, 4 * K, cudaMemcpyDeviceToHost, s);
    if (r != cudaSuccess) return cuda_check(r, "read counts");
    if ((r = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_check(r, "sync");
    uint32_t run = 0;
    for (uint32_t k = 0; k < K; k++) { st[k] = run; run += cnt[k]; }
    st[K] = run;
    if ((r = starts.ensure(4 * (K + 1))) != cudaSuccess) return cuda_check(r, "alloc starts");
    r = cudaMemcpyAsync(starts.ptr, st.data(), 4 * (K + 1), cudaMemcpyHostToDevice, s);
    return r == cudaSuccess ? CRNGPU_OK : cuda_check(r, "copy starts");
  };
  uint32_t K = 0, KS = 0, KA = 0, KAS = 0;
  int rc;
  if ((e = B.bweight.ensure(4 * N)) != cudaSuccess) return cuda_check(e, "alloc block weights");
  k_block_weights<<<(N + 255) / 256, 256, 0, s>>>(static_cast<Level*>(B.levels.ptr), P.num_levels, N, static_cast<float*>(B.bweight.ptr));
  if (cfg.has_color) {
    // colour endpoint VQ over the used tiles' vec6
    if ((e = B.vec6.ensure(sizeof(float) * 6 * ntiles)) != cudaSuccess || (e = B.w6.ensure(4 * ntiles)) != cudaSuccess)
      return cuda_check(e, "alloc vq input");
    k_tile_vectors<<<(nused + 255) / 256, 256, 0, s>>>(tiles, static_cast<uint32_t*>(B.used.ptr), nused,
                                                        static_cast<float*>(B.vec6.ptr), static_cast<uint32_t*>(B.w6.ptr));
    const uint32_t ce_base = mode.qdxt ? distinct_vectors(static_cast<float*>(B.vec6.ptr), nused, 6, s) : nused;
    if ((rc = tree_vq<6>(static_cast<float*>(B.vec6.ptr), static_cast<uint32_t*>(B.w6.ptr), nused,
                         ce_request(ce_base), frac, B.cb6, &K, s, B.vq)) != CRNGPU_OK)
      return rc;
    if ((e = B.tile_cluster.ensure(4 * ntiles)) != cudaSuccess) return cuda_check(e, "alloc tile clusters");
    k_nearest_vec6<<<(ntiles + 255) / 256, 256, 0, s>>>(tiles, ntiles, static_cast<float*>(B.cb6.ptr), K,
                                                         static_cast<uint32_t*>(B.tile_cluster.ptr));
    // cluster -> tiles (CSR): used tiles sorted by cluster (stable radix sort keeps tile order)
    if ((e = B.ccount.ensure(4 * (K + 1))) != cudaSuccess || (e = B.clist.ensure(4 * ntiles)) != cudaSuccess)
      return cuda_check(e, "alloc cluster lists");
    cudaMemsetAsync(B.ccount.ptr, 0, 4 * (K + 1), s);
    k_count_clusters<<<(ntiles + 255) / 256, 256, 0, s>>>(static_cast<uint32_t*>(B.tile_cluster.ptr), ntiles,
                                                           static_cast<uint32_t*>(B.ccount.ptr));
    k_used_clusters<<<(nused + 255) / 256, 256, 0, s>>>(static_cast<uint32_t*>(B.used.ptr), nused,
                                                         static_cast<uint32_t*>(B.tile_cluster.ptr), static_cast<uint32_t*>(B.keys.ptr));
    int key_bits = 1;
    while ((1u << key_bits) < K) key_bits++;
    if ((rc = sort_pairs(static_cast<uint32_t*>(B.keys.ptr), static_cast<uint32_t*>(B.keys2.ptr),
                         static_cast<uint32_t*>(B.used.ptr), static_cast<uint32_t*>(B.clist.ptr), nused, key_bits)) != CRNGPU_OK)
      return rc;
    if ((rc = csr_starts(B.ccount, B.cstart, K)) != CRNGPU_OK) return rc;
    if ((e = B.clusters.ensure(sizeof(ClusterOut) * K)) != cudaSuccess) return cuda_check(e, "alloc clusters");
    ClusterOut* cl = static_cast<ClusterOut*>(B.clusters.ptr);
    k_cluster_fit<<<K, kFitThreads, 0, s>>>(blocks, static_cast<Chunk*>(B.chunks.ptr), tiles,
                                             static_cast<uint32_t*>(B.cstart.ptr), static_cast<uint32_t*>(B.clist.ptr),
                                             P.perceptual, cl);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(e, "launch k_cluster_fit");
    // per-block selectors and weights -> selector VQ
    if ((e = B.block_cluster.ensure(4 * N)) != cudaSuccess || (e = B.selvec.ensure(sizeof(float) * 16 * N)) != cudaSuccess ||
        (e = B.selw.ensure(4 * N)) != cudaSuccess)
      return cuda_check(e, "alloc selectors");
    k_block_selectors<<<(N + 127) / 128, 128, 0, s>>>(blocks, N, static_cast<uint32_t*>(B.block_tile.ptr),
                                                       static_cast<uint32_t*>(B.tile_cluster.ptr),
                                                       static_cast<uint8_t*>(B.block_enc.ptr), static_cast<float*>(B.bweight.ptr),
                                                       cl, P.perceptual, static_cast<uint32_t*>(B.block_cluster.ptr),
                                                       static_cast<float*>(B.selvec.ptr), static_cast<uint32_t*>(B.selw.ptr),
                                                       static_cast<unsigned long long*>(B.sse.ptr));
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(e, "launch k_block_selectors");
    if ((rc = tree_vq<16>(static_cast<float*>(B.selvec.ptr), static_cast<uint32_t*>(B.selw.ptr), N,
                          cs_request(N), frac, B.cb16, &KS, s, B.vq)) != CRNGPU_OK)
      return rc;
    if ((e = B.cbsel.ensure(4 * KS)) != cudaSuccess || (e = B.block_sel.ensure(4 * N)) != cudaSuccess ||
        (e = B.entry_err.ensure(8 * 64 * (size_t)KS)) != cudaSuccess || (e = B.entry_used.ensure(4 * KS)) != cudaSuccess)
      return cuda_check(e, "alloc selector codebook");
    uint32_t* cbsel = static_cast<uint32_t*>(B.cbsel.ptr);
    k_selector_quantise<<<(KS + 255) / 256, 256, 0, s>>>(static_cast<float*>(B.cb16.ptr), KS, cbsel);
    cudaMemsetAsync(B.entry_err.ptr, 0, 8 * 64 * (size_t)KS, s);
    cudaMemsetAsync(B.entry_used.ptr, 0, 4 * KS, s);
    k_selector_assign<<<(N + kSelWarps - 1) / kSelWarps, kSelWarps * 32, 0, s>>>(
        blocks, N, static_cast<uint32_t*>(B.block_cluster.ptr), cl, P.perceptual, cbsel, KS,
        static_cast<uint32_t*>(B.block_sel.ptr), static_cast<unsigned long long*>(B.entry_err.ptr),
        static_cast<uint32_t*>(B.entry_used.ptr));
    k_selector_finalise<<<(KS + 255) / 256, 256, 0, s>>>(static_cast<unsigned long long*>(B.entry_err.ptr), KS, cbsel);
    k_hc_emit<<<(N + 255) / 256, 256, 0, s>>>(blocks, N, static_cast<uint32_t*>(B.block_cluster.ptr), cl,
                                              static_cast<uint32_t*>(B.block_sel.ptr), cbsel, d_out, bpb, color_ofs,
                                              static_cast<unsigned long long*>(B.sse.ptr) + 1);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(e, "launch hc selector kernels");
    // optional index outputs (colour)
    if (d_endpoint_idx || d_selector_idx || d_endpoints || d_selectors) {
      std::vector<uint32_t> bc(N), bs(N);
      std::vector<ClusterOut> hcl(K);
      if ((e = cudaMemcpyAsync(bc.data(), B.block_cluster.ptr, 4 * N, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
          (e = cudaMemcpyAsync(bs.data(), B.block_sel.ptr, 4 * N, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
          (e = cudaMemcpyAsync(hcl.data(), cl, sizeof(ClusterOut) * K, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return cuda_check(e, "read indices");
      if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_check(e, "sync");
      std::vector<uint16_t> ei(N), si(N);
      std::vector<uint32_t> eps(K);
      for (uint32_t k = 0; k < K; k++) eps[k] = hcl[k].first | (hcl[k].second << 16);
      for (uint32_t b = 0; b < N; b++) { ei[b] = (uint16_t)bc[b]; si[b] = (uint16_t)bs[b]; }
      if (d_endpoint_idx) cudaMemcpyAsync(d_endpoint_idx, ei.data(), 2 * N, cudaMemcpyHostToDevice, s);
      if (d_selector_idx) cudaMemcpyAsync(d_selector_idx, si.data(), 2 * N, cudaMemcpyHostToDevice, s);
      if (d_endpoints) cudaMemcpyAsync(d_endpoints, eps.data(), 4 * K, cudaMemcpyHostToDevice, s);
      if (d_selectors) cudaMemcpyAsync(d_selectors, cbsel, 4 * KS, cudaMemcpyDeviceToDevice, s);
      if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_check(e, "sync");
    }
  }
  if (cfg.num_alpha) {
    const uint32_t na = (uint32_t)cfg.num_alpha, nitem_t = nused * na, nitem_b = N * na;
    // alpha endpoint VQ over the tiles' vec2 (both DXN channels share one codebook)
    if ((e = B.avec.ensure(sizeof(float) * 2 * nitem_t)) != cudaSuccess || (e = B.aw.ensure(4 * nitem_t)) != cudaSuccess ||
        (e = B.aitems.ensure(4 * nitem_t)) != cudaSuccess || (e = B.tile_ac.ensure(8 * ntiles)) != cudaSuccess)
      return cuda_check(e, "alloc alpha vq input");
    k_alpha_vectors<<<(nitem_t + 255) / 256, 256, 0, s>>>(tiles, static_cast<uint32_t*>(B.used.ptr), nused, cfg.num_alpha,
                                                          cfg.qdxt, static_cast<float*>(B.avec.ptr), static_cast<uint32_t*>(B.aw.ptr),
                                                          static_cast<uint32_t*>(B.aitems.ptr));
    if ((rc = tree_vq<2>(static_cast<float*>(B.avec.ptr), static_cast<uint32_t*>(B.aw.ptr), nitem_t,
                         ae_request(mode.qdxt ? distinct_vectors(static_cast<float*>(B.avec.ptr), nitem_t, 2, s) : nused),
                         frac, B.cb2, &KA, s, B.vq)) != CRNGPU_OK)
      return rc;
    k_nearest_vec2<<<(nitem_t + 255) / 256, 256, 0, s>>>(tiles, static_cast<uint32_t*>(B.used.ptr), nused, cfg.num_alpha,
                                                          static_cast<float*>(B.cb2.ptr), KA, static_cast<uint32_t*>(B.tile_ac.ptr));
    // alpha cluster -> (tile, channel) members
    if ((e = B.acount.ensure(4 * (KA + 1))) != cudaSuccess || (e = B.alist.ensure(4 * nitem_t)) != cudaSuccess)
      return cuda_check(e, "alloc alpha lists");
    cudaMemsetAsync(B.acount.ptr, 0, 4 * (KA + 1), s);
    k_alpha_keys<<<(nitem_t + 255) / 256, 256, 0, s>>>(static_cast<uint32_t*>(B.aitems.ptr), nitem_t,
                                                       static_cast<uint32_t*>(B.tile_ac.ptr), static_cast<uint32_t*>(B.keys.ptr),
                                                       static_cast<uint32_t*>(B.acount.ptr));
    int key_bits = 1;
    while ((1u << key_bits) < KA) key_bits++;
    if ((rc = sort_pairs(static_cast<uint32_t*>(B.keys.ptr), static_cast<uint32_t*>(B.keys2.ptr),
                         static_cast<uint32_t*>(B.aitems.ptr), static_cast<uint32_t*>(B.alist.ptr), nitem_t, key_bits)) != CRNGPU_OK)
      return rc;
    if ((rc = csr_starts(B.acount, B.astart, KA)) != CRNGPU_OK) return rc;
    if ((e = B.aclusters.ensure(sizeof(AlphaCluster) * KA)) != cudaSuccess) return cuda_check(e, "alloc alpha clusters");
    AlphaCluster* ac = static_cast<AlphaCluster*>(B.aclusters.ptr);
    k_alpha_cluster_fit<<<KA, kAFitThreads, 0, s>>>(blocks, static_cast<Chunk*>(B.chunks.ptr), tiles, cfg,
                                                     static_cast<uint32_t*>(B.astart.ptr), static_cast<uint32_t*>(B.alist.ptr), ac);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(e, "launch k_alpha_cluster_fit");
    // block selectors -> alpha selector VQ -> assignment -> finalise -> emit
    if ((e = B.aitem_cluster.ensure(4 * nitem_b)) != cudaSuccess || (e = B.aselvec.ensure(sizeof(float) * 16 * nitem_b)) != cudaSuccess ||
        (e = B.aselw.ensure(4 * nitem_b)) != cudaSuccess)
      return cuda_check(e, "alloc alpha selectors");
    k_alpha_block_selectors<<<(nitem_b + 127) / 128, 128, 0, s>>>(
        blocks, N, cfg.num_alpha, cfg, static_cast<uint32_t*>(B.block_tile.ptr), static_cast<uint32_t*>(B.tile_ac.ptr),
        static_cast<uint8_t*>(B.block_enc.ptr), ac, static_cast<uint32_t*>(B.aitem_cluster.ptr),
        static_cast<float*>(B.aselvec.ptr), static_cast<uint32_t*>(B.aselw.ptr));
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(e, "launch k_alpha_block_selectors");
    if ((rc = tree_vq<16>(static_cast<float*>(B.aselvec.ptr), static_cast<uint32_t*>(B.aselw.ptr), nitem_b,
                          as_request(nitem_b), frac, B.acb16, &KAS, s, B.vq)) != CRNGPU_OK)
      return rc;
    if ((e = B.acbsel.ensure(8 * KAS)) != cudaSuccess || (e = B.aitem_sel.ensure(4 * nitem_b)) != cudaSuccess ||
        (e = B.aentry_err.ensure(8 * 128 * (size_t)KAS)) != cudaSuccess)
      return cuda_check(e, "alloc alpha selector codebook");
    unsigned long long* acbsel = static_cast<unsigned long long*>(B.acbsel.ptr);
    k_alpha_selector_quantise<<<(KAS + 255) / 256, 256, 0, s>>>(static_cast<float*>(B.acb16.ptr), KAS, acbsel);
    cudaMemsetAsync(B.aentry_err.ptr, 0, 8 * 128 * (size_t)KAS, s);
    k_alpha_selector_assign<<<(nitem_b + kASelWarps - 1) / kASelWarps, kASelWarps * 32, 0, s>>>(
        blocks, N, cfg.num_alpha, cfg, static_cast<uint32_t*>(B.aitem_cluster.ptr), ac, acbsel, KAS,
        static_cast<uint32_t*>(B.aitem_sel.ptr), static_cast<unsigned long long*>(B.aentry_err.ptr));
    k_alpha_selector_finalise<<<(KAS + 255) / 256, 256, 0, s>>>(static_cast<unsigned long long*>(B.aentry_err.ptr), KAS, acbsel);
    k_alpha_emit<<<(nitem_b + 255) / 256, 256, 0, s>>>(blocks, N, cfg.num_alpha, cfg,
                                                       static_cast<uint32_t*>(B.aitem_cluster.ptr), ac,
                                                       static_cast<uint32_t*>(B.aitem_sel.ptr), acbsel, d_out, bpb,
                                                       alpha_slot0, static_cast<unsigned long long*>(B.sse.ptr) + 2);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(e, "launch alpha selector kernels");
  }
  unsigned long long sse[3] = {0, 0, 0};
  if ((e = cudaMemcpyAsync(sse, B.sse.ptr, 24, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return cuda_check(e, "read sse");
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_check(e, "sync");
  B.clean = true;
  if (stats) {
    stats->color_endpoints = K;
    stats->color_selectors = KS;
    stats->tiles = nused;
    stats->alpha_endpoints = KA;
    stats->alpha_selectors = KAS;
    stats->sse_endpoints = (double)sse[0];
    stats->sse_final = (double)sse[1];
    stats->sse_alpha = (double)sse[2];
  }
  return CRNGPU_OK;
}

bool hc_params_ok(const crngpu_hc_params* params) {
  return params && params->struct_size == sizeof(crngpu_hc_params) && params->num_blocks && params->num_levels >= 1 &&
         params->num_levels <= 16;
}

}  // namespace
}  // namespace crngpu

// Clustered DXT1 encode with the colour codebooks and indices (dxt_hc::compress for cDXT1).
extern "C" int crngpu_hc_compress_dxt1(const uint8_t* d_blocks, const crngpu_hc_params* params, uint8_t* d_out,
                                       uint16_t* d_endpoint_idx, uint16_t* d_selector_idx, uint32_t* d_endpoints,
                                       uint32_t* d_selectors, crngpu_hc_stats* stats, void* stream) try {
  clear_error();
  if (!d_blocks || !d_out || !hc_params_ok(params)) {
    set_error("crngpu_hc_compress_dxt1: bad arguments");
    return CRNGPU_E_PARAM;
  }
  return hc_compress_impl(d_blocks, *params, CRNGPU_FMT_DXT1, d_out, d_endpoint_idx, d_selector_idx, d_endpoints,
                          d_selectors, stats, as_stream(stream));
} catch (...) {
  return crngpu::exception_status();
}

// Clustered encode of any supported format (dxt_hc::compress). See include/crngpu.h.
extern "C" int crngpu_hc_compress(const uint8_t* d_blocks, const crngpu_hc_params* params, uint32_t format,
                                  uint8_t* d_out, crngpu_hc_stats* stats, void* stream) try {
  clear_error();
  if (!d_blocks || !d_out || !hc_params_ok(params)) {
    set_error("crngpu_hc_compress: bad arguments");
    return CRNGPU_E_PARAM;
  }
  return hc_compress_impl(d_blocks, *params, format, d_out, nullptr, nullptr, nullptr, nullptr, stats, as_stream(stream));
} catch (...) {
  return crngpu::exception_status();
}

// Codebook sizes of crn_comp::quantize_images (crnlib/crn_comp.cpp:541-577) for a quality level.
extern "C" int crngpu_hc_codebook_sizes(uint32_t width, uint32_t height, uint32_t quality_level, uint32_t format,
                                        uint32_t* sizes4) try {
  if (!sizes4 || !width || !height) return CRNGPU_E_PARAM;
  const uint32_t kMin = 8, kMax = 8192;  // cCRNMinPaletteSize, cCRNMaxPaletteSize (inc/crnlib.h:118-119)
  uint32_t max_entries = ((width + 3) / 4) * ((height + 3) / 4);
  max_entries = std::min(std::max(max_entries, kMin), kMax);
  const float quality = std::min(std::max((float)quality_level / 255.0f, 0.0f), 1.0f);
  float cmul = 1.0f, amul = 1.0f;
  if (format == CRNGPU_FMT_DXT5_CCXY) { cmul = 3.5f; amul = .35f; }
  else if (format == CRNGPU_FMT_DXT5) cmul = .75f;
  auto lerp = [](float a, float b, float t) { return a + (b - a) * t; };
  auto size = [&](float lo, float q) {
    const float v = .5f + lerp(std::max(lo, (float)kMin), (float)max_entries, q);
    const uint32_t u = v <= 0.0f ? 0u : (uint32_t)v;  // math::float_to_uint
    return std::min(std::max(u, kMin), kMax);
  };
  sizes4[0] = size(64, powf(quality, 1.8f * cmul));   // colour endpoints
  sizes4[1] = size(96, powf(quality, 1.65f * cmul));  // colour selectors
  sizes4[2] = size(24, powf(quality, 2.1f * amul));   // alpha endpoints
  sizes4[3] = size(48, powf(quality, 1.65f * amul));  // alpha selectors
  return CRNGPU_OK;
} catch (...) {
  return crngpu::exception_status();
}

// crn_compress with m_file_type = cCRNFileTypeCRN and source mips (inc/crnlib.h:614,
// crnlib/crnlib.cpp:242-267 -> crn_comp::compress_internal, crnlib/crn_comp.cpp:1515-1611):
// crn_comp's block gather (edge clamped, levels padded to 8 texels, crn_comp.cpp:717-741) and the
// clustered encode on the GPU, then the .crn writer on the host.
namespace crngpu {
namespace {

// The quality-independent part of crn_compress: the blocks of every level and face in crn_comp's
// layout (crn_comp::alias_images / quantize_images, crnlib/crn_comp.cpp:454-463, 717-741): the
// host chain uploaded once and gathered on the GPU with edge clamping (k_gather_chain); a pass per
// quality level then runs the clustered encode and the writer.
// per host thread: the uploaded chain, the gathered blocks and the encoded blocks on the device,
// kept between calls
struct CrnDeviceBuffers {
  DevBuf in, out, st, words, chain, images;
};
CrnDeviceBuffers& crn_buffers() {
  static thread_local std::unique_ptr<CrnDeviceBuffers> b[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (!b[dev & 63]) b[dev & 63].reset(new CrnDeviceBuffers);
  return *b[dev & 63];
}

struct CrnSource {
  crngpu_hc_params P;
  // crn_comp_params fields beyond quality (crnlib/crn_comp.cpp:527-577): deratings, alpha
  // channel and, when palette_sizes[0] is nonzero, manual palette sizes
  crngpu_crn_options opt = {sizeof(crngpu_crn_options), 2.0f, 2.0f, 3u, {0u, 0u, 0u, 0u}};
  uint32_t width = 0, height = 0, levels = 0, faces = 0, format = 0, bpb = 0;
  uint64_t texels = 0;
  cudaStream_t stream = nullptr;
  DevBuf& d_in = crn_buffers().in;
  DevBuf& d_out = crn_buffers().out;

  int prepare(const uint8_t* rgba_levels, uint32_t w, uint32_t h, uint32_t nl, uint32_t nf, uint32_t fmt,
              uint32_t flags, const char* who) {
    if (!rgba_levels || !w || !h || w > 4096 || h > 4096 || !nl || nl > 16 || (nf != 1 && nf != 6)) {
      set_error(std::string(who) + ": bad dimensions, level or face count");
      return CRNGPU_E_PARAM;
    }
    uint32_t full = 1;
    while ((w >> full) || (h >> full)) full++;
    if (nl > full) { set_error(std::string(who) + ": more levels than the mip chain has"); return CRNGPU_E_PARAM; }
    width = w; height = h; levels = nl; faces = nf; format = fmt;
    std::memset(&P, 0, sizeof(P));
    P.struct_size = sizeof(P);
    // the host chain (face after face, level after level) is uploaded as it is; the gather into
    // crn_comp's layout (levels in order, a level's faces one after another) runs on the GPU
    std::vector<size_t> img_ofs((size_t)faces * levels);
    size_t ofs = 0;
    for (uint32_t f = 0; f < faces; f++)
      for (uint32_t l = 0; l < levels; l++) {
        img_ofs[(size_t)f * levels + l] = ofs;
        ofs += (size_t)std::max(1u, width >> l) * std::max(1u, height >> l) * 4;
        texels += (uint64_t)std::max(1u, width >> l) * std::max(1u, height >> l);
      }
    std::vector<GatherImage> imgs;
    uint32_t nblocks = 0;
    for (uint32_t l = 0; l < levels; l++) {
      const uint32_t lw = std::max(1u, width >> l), lh = std::max(1u, height >> l);
      const uint32_t W = ((lw + 7) & ~7u) >> 2, H = ((lh + 7) & ~7u) >> 2;
      P.levels[l].first_block = nblocks;
      P.levels[l].num_blocks = W * H * faces;
      P.levels[l].block_width = W;
      P.levels[l].weight = std::min(12.0f, powf(1.3f, (float)l));
      for (uint32_t f = 0; f < faces; f++) {
        imgs.push_back(GatherImage{(uint64_t)img_ofs[(size_t)f * levels + l], lw, lh, W, nblocks});
        nblocks += W * H;
      }
    }
    P.num_blocks = nblocks;
    P.num_levels = levels;
    P.num_faces = faces;
    const bool colour_fmt = format == CRNGPU_FMT_DXT1 || format == CRNGPU_FMT_DXT5;
    P.perceptual = colour_fmt && (flags & CRNGPU_FLAG_PERCEPTUAL) ? 1 : 0;
    P.adaptive_tile_color_psnr_derating = opt.colour_psnr_derating;
    P.adaptive_tile_alpha_psnr_derating = opt.alpha_psnr_derating;
    if (format == CRNGPU_FMT_DXT5_CCXY && !opt.palette_sizes[0])
      P.adaptive_tile_color_psnr_derating = 5.0f;  // crn_comp.cpp:553-558
    P.color_alpha_weighting_ratio = 3.0f;
    P.alpha_component = opt.alpha_component;
    bpb = (format == CRNGPU_FMT_DXT1 || format == CRNGPU_FMT_DXT5A) ? 8 : 16;
    cudaError_t e;
    CrnDeviceBuffers& cb = crn_buffers();
    if ((e = d_in.ensure((size_t)nblocks * 64)) != cudaSuccess ||
        (e = d_out.ensure((size_t)P.num_blocks * bpb)) != cudaSuccess || (e = cb.chain.ensure(ofs)) != cudaSuccess ||
        (e = cb.images.ensure(sizeof(GatherImage) * imgs.size())) != cudaSuccess)
      return cuda_check(e, "alloc blocks");
    if ((e = cudaMemcpyAsync(cb.chain.ptr, rgba_levels, ofs, cudaMemcpyHostToDevice, stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(cb.images.ptr, imgs.data(), sizeof(GatherImage) * imgs.size(), cudaMemcpyHostToDevice,
                             stream)) != cudaSuccess)
      return cuda_check(e, "upload chain");
    int rc = launch_gather_chain(static_cast<const uint8_t*>(cb.chain.ptr), static_cast<const GatherImage*>(cb.images.ptr),
                                 (uint32_t)imgs.size(), nblocks, format, static_cast<uint32_t*>(d_in.ptr), stream);
    if (rc != CRNGPU_OK) return rc;
    if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return cuda_check(e, "sync");  // `imgs` is freed next
    return CRNGPU_OK;
  }

  // One compress pass at `quality`: the .crn bytes into `file`.
  int pass(uint32_t quality, std::vector<uint8_t>& file) {
    uint32_t sizes[4];
    if (opt.palette_sizes[0]) {
      for (int k = 0; k < 4; k++) sizes[k] = std::min(std::max(opt.palette_sizes[k], 8u), 8192u);  // crn_comp.cpp:532-538
    } else if (crngpu_hc_codebook_sizes(width, height, quality, format, sizes) != CRNGPU_OK) {
      return CRNGPU_E_PARAM;
    }
    P.color_endpoint_codebook_size = sizes[0];
    P.color_selector_codebook_size = sizes[1];
    P.alpha_endpoint_codebook_size = sizes[2];
    P.alpha_selector_codebook_size = sizes[3];
    int rc = crngpu_hc_compress(static_cast<const uint8_t*>(d_in.ptr), &P, format, static_cast<uint8_t*>(d_out.ptr),
                                nullptr, stream);
    if (rc != CRNGPU_OK) return rc;
    std::vector<uint8_t> dxt((size_t)P.num_blocks * bpb);
    cudaError_t e;
    if ((e = cudaMemcpyAsync(dxt.data(), d_out.ptr, dxt.size(), cudaMemcpyDeviceToHost, stream)) != cudaSuccess)
      return cuda_check(e, "copy result");
    if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return cuda_check(e, "sync");
    // a .crn is smaller than its DXT blocks plus palettes (8192 entries of at most 8 bytes each,
    // twice) and the models; grow once if not
    file.resize(dxt.size() + (1u << 18));
    int64_t n = crngpu_crn_pack(dxt.data(), width, height, levels, faces, format, file.data(), file.size());
    if (n > (int64_t)file.size()) {
      file.resize((size_t)n);
      n = crngpu_crn_pack(dxt.data(), width, height, levels, faces, format, file.data(), file.size());
    }
    if (n < 0) return (int)n;
    file.resize((size_t)n);
    return CRNGPU_OK;
  }
};

int64_t deliver(const std::vector<uint8_t>& file, void* out, uint64_t out_capacity) {
  if (out && out_capacity >= file.size()) std::memcpy(out, file.data(), file.size());
  return (int64_t)file.size();
}

}  // namespace
}  // namespace crngpu

extern "C" int64_t crngpu_compress_crn(const uint8_t* rgba_levels, uint32_t width, uint32_t height, uint32_t levels,
                                       uint32_t faces, uint32_t format, uint32_t quality_level, uint32_t flags,
                                       void* out, uint64_t out_capacity) try {
  using namespace crngpu;
  clear_error();
  if (quality_level > 255) { set_error("crngpu_compress_crn: quality above 255"); return CRNGPU_E_PARAM; }
  CrnSource src;
  int rc = src.prepare(rgba_levels, width, height, levels, faces, format, flags, "crngpu_compress_crn");
  if (rc != CRNGPU_OK) return rc;
  std::vector<uint8_t> file;
  if ((rc = src.pass(quality_level, file)) != CRNGPU_OK) return rc;
  return deliver(file, out, out_capacity);
} catch (...) {
  return crngpu::exception_status();
}

extern "C" int64_t crngpu_compress_dds_clustered(const uint8_t* rgba_levels, uint32_t width, uint32_t height,
                                                 uint32_t levels, uint32_t faces, uint32_t format,
                                                 uint32_t quality_level, uint32_t flags, void* out,
                                                 uint64_t out_capacity) try {
  return crngpu_compress_dds_clustered_ex(rgba_levels, width, height, levels, faces, format, quality_level, flags,
                                          nullptr, out, out_capacity);
} catch (...) {
  return crngpu::exception_status();
}

extern "C" int64_t crngpu_compress_dds_clustered_ex(const uint8_t* rgba_levels, uint32_t width, uint32_t height,
                                                    uint32_t levels, uint32_t faces, uint32_t format,
                                                    uint32_t quality_level, uint32_t flags,
                                                    const crngpu_block_options* options, void* out,
                                                    uint64_t out_capacity) try {
  using namespace crngpu;
  using namespace crngpu::hc;
  clear_error();
  if (quality_level > 255) { set_error("crngpu_compress_dds_clustered: quality above 255"); return CRNGPU_E_PARAM; }
  if (format_is_non_srgb(format)) flags &= ~CRNGPU_FLAG_PERCEPTUAL;
  // dds_comp::compress_init (crnlib/crn_dds_comp.cpp:244-247): DXT1 becomes DXT1A when the flag
  // is set, both block types are allowed and some source texel has alpha below 255
  if (format == CRNGPU_FMT_DXT1 && (flags & CRNGPU_FLAG_DXT1A) && (flags & CRNGPU_FLAG_USE_BOTH_BLOCK_TYPES) &&
      rgba_levels) {
    bool has_alpha = false;
    uint64_t texels = 0;
    for (uint32_t l = 0; l < levels; l++)
      texels += (uint64_t)std::max(1u, width >> l) * std::max(1u, height >> l) * faces;
    for (uint64_t t = 0; t < texels && !has_alpha; t++) has_alpha = rgba_levels[t * 4 + 3] < 255;
    if (!has_alpha) flags &= ~CRNGPU_FLAG_DXT1A;
  } else {
    flags &= ~CRNGPU_FLAG_DXT1A;
  }
  if ((flags & CRNGPU_FLAG_DXT1A) && quality_level < 255) {
    set_error("crngpu_compress_dds_clustered: DXT1A transparency below quality 255 (qdxt1 with alpha) is not built");
    return CRNGPU_E_UNSUPPORTED;
  }
  if (quality_level >= 255) {
    // dds_comp at quality 255 (crnlib/crn_dds_comp.cpp:150-157): the plain encoder on every block
    // of the cooked source -- uploaded once, gathered on the GPU, one encoder launch for the chain
    uint32_t q = kDxtQualityUber, thr = 128;
    if (options) {
      if (options->struct_size != sizeof(crngpu_block_options) || options->dxt_quality > kDxtQualityUber ||
          options->dxt1a_alpha_threshold > 255) {
        set_error("bad crngpu_block_options");
        return CRNGPU_E_PARAM;
      }
      q = options->dxt_quality;
      thr = options->dxt1a_alpha_threshold;
    }
    return dds_plain_chain(rgba_levels, width, height, levels, faces, format, flags, q, thr, out, out_capacity);
  }
  CrnSource src;
  int rc = src.prepare(rgba_levels, width, height, levels, faces, format, flags, "crngpu_compress_dds_clustered");
  if (rc != CRNGPU_OK) return rc;
  const uint32_t bpb = src.bpb;
  uint64_t need = 0;
  for (uint32_t l = 0; l < levels; l++)
    need += (uint64_t)((std::max(1u, width >> l) + 3) / 4) * ((std::max(1u, height >> l) + 3) / 4) * bpb * faces;
  const uint32_t N = src.P.num_blocks;
  cudaError_t e;
  // elements of a block, each an 8-byte DXT1 or DXT5A element: (kind, channel, byte offset)
  struct Element { uint32_t fmt; int comp; uint32_t ofs; };
  std::vector<Element> elems;
  switch (format) {
    case CRNGPU_FMT_DXT1: elems = {{CRNGPU_FMT_DXT1, 0, 0}}; break;
    case CRNGPU_FMT_DXT5A: elems = {{CRNGPU_FMT_DXT5A, 3, 0}}; break;
    case CRNGPU_FMT_DXN_XY: elems = {{CRNGPU_FMT_DXT5A, 0, 0}, {CRNGPU_FMT_DXT5A, 1, 8}}; break;
    case CRNGPU_FMT_DXN_YX: elems = {{CRNGPU_FMT_DXT5A, 1, 0}, {CRNGPU_FMT_DXT5A, 0, 8}}; break;
    default: elems = {{CRNGPU_FMT_DXT5A, 3, 0}, {CRNGPU_FMT_DXT1, 0, 8}}; break;  // the DXT5 family
  }
  {
    // mipmapped_texture::qdxt_pack (crnlib/crn_mipmapped_texture.cpp:2330-2560): qdxt1 on the
    // colour element, qdxt5 on each alpha / DXN element, each with its own tiling and codebooks;
    // element k is written to d_out + k * N * 8 and interleaved below
    CrnDeviceBuffers& cb = crn_buffers();
    if ((e = cb.st.ensure(sizeof(SolidTables))) != cudaSuccess || (e = cb.words.ensure(8ull * N)) != cudaSuccess)
      return cuda_check(e, "alloc selector words");
    if ((e = cudaMemcpy(cb.st.ptr, single_colour_tables_host(), sizeof(SolidTables), cudaMemcpyHostToDevice)) != cudaSuccess)
      return cuda_check(e, "upload tables");
    for (size_t k = 0; k < elems.size(); k++) {
      const Element& el = elems[k];
      const bool colour = el.fmt == CRNGPU_FMT_DXT1;
      // the distinct dxt_fast selector words of the blocks, plus 128 (qdxt1::init / qdxt5::init)
      uint32_t distinct = 0;
      if (colour) {
        k_fast_selector_words<<<(N + 255) / 256, 256>>>(static_cast<const uint32_t*>(src.d_in.ptr), N,
                                                        static_cast<const SolidTables*>(cb.st.ptr),
                                                        static_cast<uint32_t*>(cb.words.ptr));
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(e, "k_fast_selector_words");
        std::vector<uint32_t> words(N);
        if ((e = cudaMemcpy(words.data(), cb.words.ptr, 4ull * N, cudaMemcpyDeviceToHost)) != cudaSuccess)
          return cuda_check(e, "read selector words");
        std::sort(words.begin(), words.end());
        distinct = (uint32_t)(std::unique(words.begin(), words.end()) - words.begin());
      } else {
        k_fast_alpha_selector_words<<<(N + 255) / 256, 256>>>(static_cast<const uint32_t*>(src.d_in.ptr), N, el.comp,
                                                              static_cast<unsigned long long*>(cb.words.ptr));
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(e, "k_fast_alpha_selector_words");
        std::vector<unsigned long long> words(N);
        if ((e = cudaMemcpy(words.data(), cb.words.ptr, 8ull * N, cudaMemcpyDeviceToHost)) != cudaSuccess)
          return cuda_check(e, "read selector words");
        std::sort(words.begin(), words.end());
        distinct = (uint32_t)(std::unique(words.begin(), words.end()) - words.begin());
      }
      HcMode mode;
      mode.qdxt = true;
      mode.quality = quality_level / 255.0f;
      // codebook curves of the colour element: deeper for DXT5's colour (favoured over alpha) and
      // shallower for DXT5_CCxY's chroma (crnlib/crn_mipmapped_texture.cpp:2530-2544)
      mode.power_mul = !colour ? 1.0f : format == CRNGPU_FMT_DXT5 ? .75f : format == CRNGPU_FMT_DXT5_CCXY ? 1.5f : 1.0f;
      mode.selector_base = distinct + 128;
      mode.derate_div = colour ? 3.1f : 3.0f;
      crngpu_hc_params P = src.P;
      // qdxt1::init derates colour layouts by 1.5, qdxt5::init alpha layouts by 2.4
      P.adaptive_tile_color_psnr_derating = colour ? 1.5f : 2.4f;
      P.color_endpoint_codebook_size = P.color_selector_codebook_size = 65535;
      P.alpha_endpoint_codebook_size = P.alpha_selector_codebook_size = 65535;
      P.alpha_component = (uint32_t)el.comp;
      P.perceptual = colour ? src.P.perceptual : 0;
      if ((rc = hc_compress_impl(static_cast<const uint8_t*>(src.d_in.ptr), P, el.fmt,
                                 static_cast<uint8_t*>(src.d_out.ptr) + k * (size_t)N * 8, nullptr, nullptr, nullptr,
                                 nullptr, nullptr, nullptr, mode)) != CRNGPU_OK)
        return rc;
    }
  }
  if (!out || out_capacity < need) return (int64_t)need;
  std::vector<uint8_t> dxt((size_t)N * bpb);
  if ((e = cudaMemcpy(dxt.data(), src.d_out.ptr, dxt.size(), cudaMemcpyDeviceToHost)) != cudaSuccess)
    return cuda_check(e, "copy result");
  if (elems.size() == 2) {  // element planes -> 16-byte blocks
    std::vector<uint8_t> planes(dxt);
    for (uint32_t b = 0; b < N; b++)
      for (size_t k = 0; k < 2; k++)
        std::memcpy(dxt.data() + (size_t)b * 16 + elems[k].ofs, planes.data() + (k * (size_t)N + b) * 8, 8);
  }
  // DDS order: every face's mip chain, each level's visible blocks row by row
  uint8_t* o = static_cast<uint8_t*>(out);
  for (uint32_t f = 0; f < faces; f++)
    for (uint32_t l = 0; l < levels; l++) {
      const uint32_t lw = std::max(1u, width >> l), lh = std::max(1u, height >> l);
      const uint32_t bx = (lw + 3) / 4, by = (lh + 3) / 4;
      const auto& L = src.P.levels[l];
      const uint32_t H = L.num_blocks / (L.block_width * faces);
      for (uint32_t y = 0; y < by; y++) {
        const size_t row = (size_t)L.first_block + ((size_t)f * H + y) * L.block_width;
        std::memcpy(o, dxt.data() + row * bpb, (size_t)bx * bpb);
        o += (size_t)bx * bpb;
      }
    }
  return (int64_t)need;
} catch (...) {
  return crngpu::exception_status();
}

extern "C" int crngpu_compress_crn_batch(crngpu_crn_batch_item* items, uint32_t n, uint32_t threads) try {
  using namespace crngpu;
  clear_error();
  if (!items && n) { set_error("crngpu_compress_crn_batch: no items"); return CRNGPU_E_PARAM; }
  if (!n) return CRNGPU_OK;
  int dev = 0;
  cudaGetDevice(&dev);
  threads = std::max(1u, std::min(threads ? threads : 4u, std::min(n, 32u)));
  std::atomic<uint32_t> next{0};
  std::atomic<int> failed{0};
  auto worker = [&]() {
    cudaSetDevice(dev);
    cudaStream_t s = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) { failed = 1; return; }
    std::vector<uint8_t> file;
    for (uint32_t i = next++; i < n; i = next++) {
      crngpu_crn_batch_item& it = items[i];
      CrnSource src;
      src.stream = s;
      int rc = it.quality_level > 255 ? (int)CRNGPU_E_PARAM
                                      : src.prepare(it.rgba_levels, it.width, it.height, it.levels, it.faces,
                                                    it.format, it.flags, "crngpu_compress_crn_batch");
      if (rc == CRNGPU_OK) rc = src.pass(it.quality_level, file);
      it.result = rc == CRNGPU_OK ? deliver(file, it.out, it.out_capacity) : (int64_t)rc;
      if (rc != CRNGPU_OK) failed = 1;
    }
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
  };
  std::vector<std::thread> pool;
  for (uint32_t t = 1; t < threads; t++) pool.emplace_back(worker);
  worker();
  for (auto& t : pool) t.join();
  if (failed) set_error("crngpu_compress_crn_batch: some items failed (see their result)");
  return failed ? CRNGPU_E_PARAM : CRNGPU_OK;
} catch (...) {
  return crngpu::exception_status();
}

namespace crngpu {
namespace {

// The interpolative search over quality levels of create_compressed_texture
// (crnlib/crn_texture_comp.cpp:120-245): each trial's bitrate is cached; after the first trial the
// next quality is interpolated between the nearest tried levels that bracket the target (or taken
// a third of the way up the open range); after 8 trials the search is a plain bisection. The
// closest bitrate at or below the target wins, else the closest above; a result within 0.005 bpp
// below the target ends the search.
int bitrate_search(CrnSource& src, float target_bitrate, std::vector<uint8_t>& best_file, uint32_t* quality_out,
                   float* bitrate_out) {
  const int kLowest = 0, kHighest = 255, kMaxIterations = 8;
  float cached[256];
  for (float& c : cached) c = -1.0f;
  int low = kLowest, high = kHighest, best_q = -1, rc;
  float best_rate = 1e10f;
  std::vector<uint8_t> file;
  bool force_bisection = false;
  for (int iter = 0; low <= high; iter++) {
    int trial = (low + high) / 2;
    if (iter && !force_bisection) {
      int bl = trial;
      while (cached[bl] < 0 && bl > kLowest) bl--;
      if (cached[bl] < 0) {
        trial = (int)((float)low + ((float)high - (float)low) * .33f);
      } else {
        int bh = trial + 1;
        if (bh <= kHighest) {
          while (cached[bh] < 0 && bh < kHighest) bh++;
          if (cached[bh] >= 0) {
            const float lr = cached[bl], hr = cached[bh];
            if (lr < hr && lr < target_bitrate && hr >= target_bitrate) {
              const int q = low + (int)(((target_bitrate - lr) * (float)(high - low)) / (hr - lr));
              if (q >= low && q <= high) trial = q;
            }
          }
        }
      }
    }
    if ((rc = src.pass((uint32_t)trial, file)) != CRNGPU_OK) return rc;
    const float rate = (float)file.size() * 8.0f / (float)src.texels;
    cached[trial] = rate;
    if (best_q < 0 || (rate <= target_bitrate && best_rate > target_bitrate) ||
        ((rate <= target_bitrate || best_rate > target_bitrate) &&
         std::fabs(rate - target_bitrate) < std::fabs(best_rate - target_bitrate))) {
      best_rate = rate;
      best_q = trial;
      best_file.swap(file);
      if (best_rate <= target_bitrate && std::fabs(best_rate - target_bitrate) < .005f) break;
    }
    if (rate > target_bitrate) high = trial - 1;
    else low = trial + 1;
    if (iter + 1 > kMaxIterations) force_bisection = true;
  }
  if (quality_out) *quality_out = (uint32_t)best_q;
  if (bitrate_out) *bitrate_out = best_rate;
  return CRNGPU_OK;
}

}  // namespace
}  // namespace crngpu

extern "C" int64_t crngpu_compress_crn_bitrate(const uint8_t* rgba_levels, uint32_t width, uint32_t height,
                                               uint32_t levels, uint32_t faces, uint32_t format, float target_bitrate,
                                               uint32_t flags, void* out, uint64_t out_capacity,
                                               uint32_t* quality_out, float* bitrate_out) try {
  if (!(target_bitrate > 0.0f)) {
    crngpu::set_error("crngpu_compress_crn_bitrate: target bitrate must be positive");
    return CRNGPU_E_PARAM;
  }
  return crngpu_compress_crn_ex(rgba_levels, width, height, levels, faces, format, 0, target_bitrate, flags, nullptr,
                                out, out_capacity, quality_out, bitrate_out);
} catch (...) {
  return crngpu::exception_status();
}

extern "C" int64_t crngpu_compress_crn_ex(const uint8_t* rgba_levels, uint32_t width, uint32_t height,
                                          uint32_t levels, uint32_t faces, uint32_t format, uint32_t quality_level,
                                          float target_bitrate, uint32_t flags, const crngpu_crn_options* options,
                                          void* out, uint64_t out_capacity, uint32_t* quality_out,
                                          float* bitrate_out) try {
  using namespace crngpu;
  clear_error();
  if (quality_out) *quality_out = 0;
  if (bitrate_out) *bitrate_out = 0.0f;
  if (target_bitrate < 0.0f || target_bitrate != target_bitrate) {
    set_error("crngpu_compress_crn_ex: negative target bitrate");
    return CRNGPU_E_PARAM;
  }
  if (quality_level > 255) { set_error("crngpu_compress_crn_ex: quality above 255"); return CRNGPU_E_PARAM; }
  CrnSource src;
  if (options) {
    if (options->struct_size != sizeof(crngpu_crn_options) || options->alpha_component > 3 ||
        !(options->colour_psnr_derating >= 0.0f) || !(options->alpha_psnr_derating >= 0.0f)) {
      set_error("crngpu_compress_crn_ex: bad options");
      return CRNGPU_E_PARAM;
    }
    src.opt = *options;
  }
  int rc = src.prepare(rgba_levels, width, height, levels, faces, format, flags, "crngpu_compress_crn_ex");
  if (rc != CRNGPU_OK) return rc;
  std::vector<uint8_t> file;
  // manual palette sizes turn the bitrate search off (crnlib/crn_texture_comp.cpp:85)
  if (target_bitrate > 0.0f && !src.opt.palette_sizes[0]) {
    if ((rc = bitrate_search(src, target_bitrate, file, quality_out, bitrate_out)) != CRNGPU_OK) return rc;
  } else {
    if ((rc = src.pass(quality_level, file)) != CRNGPU_OK) return rc;
    if (quality_out && !(target_bitrate > 0.0f)) *quality_out = quality_level;
    if (bitrate_out) *bitrate_out = (float)file.size() * 8.0f / (float)src.texels;
  }
  return deliver(file, out, out_capacity);
} catch (...) {
  return crngpu::exception_status();
}

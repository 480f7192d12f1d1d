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
// clusterizer result depends on the thread count), so this path is judged on quality.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_select.cuh>

#include "crngpu_internal.h"

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
__host__ __device__ uint32_t fast_tile_error(int n, const uint32_t* px, const SolidTables* __restrict__ st) {
  uint8_t sel[64];
  uint32_t lo16, hi16;
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
};

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
// chosen tiles' vec6, and each block's tile slot and layout. Returns the layout.
__host__ __device__ int hc_tile_chunk(const uint32_t* __restrict__ blocks, uint32_t c, const Chunk& ch,
                                      const float* __restrict__ derating, const float* __restrict__ level_weight,
                                      bool perceptual, const SolidTables* __restrict__ st, Tile* __restrict__ tiles,
                                      uint32_t* __restrict__ block_tile, uint8_t* __restrict__ block_enc) {
  const uint8_t tile_ofs[9] = HC_TILE_OFS;
  const uint8_t layout_tiles[8][4] = HC_LAYOUT_TILES;
  const uint8_t layout_ntiles[8] = HC_LAYOUT_NTILES;
  const uint8_t tile_map[8][2][2] = HC_TILE_MAP;
  uint32_t px[128];
  chunk_pixels(blocks, ch.b, ch.width, px);
  uint32_t terr[9];
  for (int t = 0; t < 9; t++) terr[t] = fast_tile_error(16 << (t >> 2), px + tile_ofs[t], st);
  float best_q = 0.0f;
  int best_e = 0;
  for (int e = 0; e < 8; e++) {
    uint32_t tot = 0;
    for (int k = 0; k < layout_ntiles[e]; k++) tot += terr[layout_tiles[e][k]];
    const double psnr = tot ? log10((double)255.0f / sqrt(tot / 192.0)) * (double)20.0f : (double)999999.0f;
    const float q = (float)fmax(psnr - (double)derating[ch.level * 8 + e], 0.0);
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
    palettize(px + tile_ofs[t], n, perceptual, T.v);
  }
  for (int by = 0; by < 2; by++)
    for (int bx = 0; bx < 2; bx++) {
      const uint32_t blk = ch.b + (by ? ch.width : 0) + bx;
      block_tile[blk] = 4 * c + tile_map[best_e][by][bx];
      block_enc[blk] = (uint8_t)best_e;
    }
  return best_e;
}

__global__ void __launch_bounds__(64) k_hc_tiles(const uint32_t* __restrict__ blocks, const Chunk* __restrict__ chunks,
                                                 uint32_t nchunks, const float* __restrict__ derating /* [level][8] */,
                                                 const float* __restrict__ level_weight, int perceptual,
                                                 const SolidTables* __restrict__ st, Tile* __restrict__ tiles,
                                                 uint32_t* __restrict__ block_tile, uint8_t* __restrict__ block_enc) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nchunks) return;
  hc_tile_chunk(blocks, c, chunks[c], derating, level_weight, perceptual != 0, st, tiles, block_tile, block_enc);
}

// ------------------------------------------------------------------------------------------
// Tree clusterizer, batched: one CTA per node to split.

constexpr int kVqThreads = 512;
constexpr uint32_t kDefaultRoundFraction = 4;  // a VQ round splits at most leaves / 4 nodes

template <int D>
struct VqNode {
  float c[D];         // centroid
  double weight;      // total weight
  float variance;     // weighted variance (sum of squared deviations)
  uint32_t begin, end;
  int32_t left, right;  // children (-1: leaf)
  uint32_t unsplittable;
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

template <int D>
__device__ __forceinline__ float dist2(const float* a, const float* b) {
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < D; k++) { const float d = a[k] - b[k]; s += d * d; }
  return s;
}

// Splits node `parent` of the perm range [begin, end) into two children (tree_clusterizer::split_node,
// crn_tree_clusterizer.h:265-570). vec: N x D floats, w: weights, perm/tmp: index permutations.
template <int D>
__global__ void __launch_bounds__(kVqThreads) k_vq_split(const float* __restrict__ vec, const uint32_t* __restrict__ w,
                                                         uint32_t* __restrict__ perm, uint32_t* __restrict__ tmp,
                                                         VqNode<D>* __restrict__ nodes, const SplitJob* __restrict__ jobs) {
  __shared__ float red[(2 * D + 4) * 16];
  __shared__ float rv[16];
  __shared__ uint32_t rp[16];
  __shared__ float s_c[D];
  __shared__ uint32_t s_scan[kVqThreads / 32 + 1];
  const SplitJob job = jobs[blockIdx.x];
  VqNode<D>& P = nodes[job.parent];
  const uint32_t b0 = P.begin, b1 = P.end;
  if (threadIdx.x < D) s_c[threadIdx.x] = P.c[threadIdx.x];
  __syncthreads();
  float c[D];
#pragma unroll
  for (int k = 0; k < D; k++) c[k] = s_c[k];
  // furthest from the centroid, then the point furthest from that
  float fv = -1.f;
  uint32_t fp = 0xFFFFFFFFu;
  for (uint32_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
    const float d = dist2<D>(vec + (size_t)perm[i] * D, c);
    if (d > fv) { fv = d; fp = i; }
  }
  block_argmax(fv, fp, rv, rp);
  float fur[D];
#pragma unroll
  for (int k = 0; k < D; k++) fur[k] = vec[(size_t)perm[fp] * D + k];
  float ov = -1.f;
  uint32_t op = 0xFFFFFFFFu;
  for (uint32_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
    const float d = dist2<D>(vec + (size_t)perm[i] * D, fur);
    if (d > ov) { ov = d; op = i; }
  }
  block_argmax(ov, op, rv, rp);
  float L[D], R[D];
#pragma unroll
  for (int k = 0; k < D; k++) {
    L[k] = (fur[k] + c[k]) * 0.5f;
    R[k] = (vec[(size_t)perm[op] * D + k] + c[k]) * 0.5f;
  }
  const double tw = P.weight;
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
      for (uint32_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
        const float* v = vec + (size_t)perm[i] * D;
        float d[D], dot = 0.f;
#pragma unroll
        for (int k = 0; k < D; k++) { d[k] = v[k] - c[k]; dot += d[k] * axis[k]; }
        const float ww = (float)w[perm[i]] * dot;
#pragma unroll
        for (int k = 0; k < D; k++) acc[k] += d[k] * ww;
      }
      block_sum<D>(acc, red);
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
    for (uint32_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
      const float* v = vec + (size_t)perm[i] * D;
      float t = 0.f;
#pragma unroll
      for (int k = 0; k < D; k++) t += (v[k] - c[k]) * axis[k];
      const float ww = (float)w[perm[i]];
      const int side = t < 0.f ? 0 : 1;
#pragma unroll
      for (int k = 0; k < D; k++) acc[side * D + k] += v[k] * ww;
      acc[2 * D + side] += ww;
    }
    block_sum<2 * D + 2>(acc, red);
    if (acc[2 * D] > 0.f && acc[2 * D + 1] > 0.f) {
#pragma unroll
      for (int k = 0; k < D; k++) { L[k] = acc[k] / acc[2 * D]; R[k] = acc[D + k] / acc[2 * D + 1]; }
    }
  }
  // 2-means; the partition is the last assignment (made with the centroids before their update)
  float prev = 1e10f, lvar = 0.f, rvar = 0.f, lw = 0.f, rw = 0.f;
  float AL[D], AR[D];  // centroids of the last assignment
  for (int loop = 0; loop < 1024; loop++) {
    float acc[2 * D + 4];
#pragma unroll
    for (int k = 0; k < 2 * D + 4; k++) acc[k] = 0.f;
#pragma unroll
    for (int k = 0; k < D; k++) { AL[k] = L[k]; AR[k] = R[k]; }
    for (uint32_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
      const float* v = vec + (size_t)perm[i] * D;
      float vv[D];
#pragma unroll
      for (int k = 0; k < D; k++) vv[k] = v[k];
      const float ww = (float)w[perm[i]];
      const int side = dist2<D>(AL, vv) < dist2<D>(AR, vv) ? 0 : 1;
      float sq = 0.f;
#pragma unroll
      for (int k = 0; k < D; k++) { acc[side * D + k] += vv[k] * ww; sq += vv[k] * vv[k]; }
      acc[2 * D + side] += ww;
      acc[2 * D + 2 + side] += sq * ww;
    }
    block_sum<2 * D + 4>(acc, red);
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
    if (threadIdx.x == 0) P.unsplittable = 1;
    return;
  }
  // stable partition of perm[b0, b1) by the last assignment: lefts first (pass 0), then rights (pass 1)
  uint32_t nleft_total = 0, nright_done = 0;
  for (int pass = 0; pass < 2; pass++) {
    for (uint32_t base = b0; base < b1; base += blockDim.x) {
      const uint32_t i = base + threadIdx.x;
      bool take = false;
      uint32_t pi = 0;
      if (i < b1) {
        pi = perm[i];
        float vv[D];
#pragma unroll
        for (int k = 0; k < D; k++) vv[k] = vec[(size_t)pi * D + k];
        const bool left = dist2<D>(AL, vv) < dist2<D>(AR, vv);
        take = pass == 0 ? left : !left;
      }
      const uint32_t ballot = __ballot_sync(0xFFFFFFFFu, take);
      const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
      __syncthreads();
      if (lane == 0) s_scan[warp] = __popc(ballot);
      __syncthreads();
      if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (int wi = 0; wi < (int)(blockDim.x >> 5); wi++) { const uint32_t t = s_scan[wi]; s_scan[wi] = run; run += t; }
        s_scan[kVqThreads / 32] = run;
      }
      __syncthreads();
      const uint32_t rank = s_scan[warp] + __popc(ballot & ((1u << lane) - 1u));
      if (take) tmp[b0 + (pass == 0 ? nleft_total : nleft_total + nright_done) + rank] = pi;
      if (pass == 0) nleft_total += s_scan[kVqThreads / 32];
      else nright_done += s_scan[kVqThreads / 32];
    }
  }
  __syncthreads();
  for (uint32_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) perm[i] = tmp[i];
  if (threadIdx.x == 0) {
    VqNode<D>& A = nodes[job.left];
    VqNode<D>& B = nodes[job.right];
    for (int k = 0; k < D; k++) { A.c[k] = L[k]; B.c[k] = R[k]; }
    A.weight = lw; B.weight = rw;
    A.variance = lvar; B.variance = rvar;
    A.begin = b0; A.end = b0 + nleft_total;
    B.begin = b0 + nleft_total; B.end = b1;
    A.left = A.right = B.left = B.right = -1;
    A.unsplittable = B.unsplittable = 0;
    P.left = job.left;
    P.right = job.right;
  }
  (void)tw;
}

// Root node statistics: centroid, weight and variance of all vectors (one CTA).
template <int D>
__global__ void __launch_bounds__(kVqThreads) k_vq_root(const float* __restrict__ vec, const uint32_t* __restrict__ w,
                                                        uint32_t n, VqNode<D>* __restrict__ nodes) {
  __shared__ float red[(D + 2) * 16];
  float acc[D + 2];
#pragma unroll
  for (int k = 0; k < D + 2; k++) acc[k] = 0.f;
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
    const float ww = (float)w[i];
    float sq = 0.f;
#pragma unroll
    for (int k = 0; k < D; k++) { const float v = vec[(size_t)i * D + k]; acc[k] += v * ww; sq += v * v; }
    acc[D] += ww;
    acc[D + 1] += sq * ww;
  }
  block_sum<D + 2>(acc, red);
  if (threadIdx.x == 0) {
    VqNode<D>& r = nodes[0];
    float cc = 0.f;
    for (int k = 0; k < D; k++) cc += acc[k] * acc[k];
    r.variance = acc[D] > 0.f ? acc[D + 1] - cc / acc[D] : 0.f;
    for (int k = 0; k < D; k++) r.c[k] = acc[D] > 0.f ? acc[k] / acc[D] : 0.f;
    r.weight = acc[D];
    r.begin = 0; r.end = n;
    r.left = r.right = -1;
    r.unsplittable = 0;
  }
}

__global__ void k_iota(uint32_t* p, uint32_t n) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = i;
}

// Host driver of the batched tree clusterizer: returns the codebook (leaf centroids) on the device
// as K x D floats in `codebook` and the leaf count in *k_out.
template <int D>
int tree_vq(const float* d_vec, const uint32_t* d_w, uint32_t n, uint32_t max_entries, uint32_t round_fraction,
            DevBuf& codebook, uint32_t* k_out, cudaStream_t s) {
  using Node = VqNode<D>;
  *k_out = 0;
  if (!n) return CRNGPU_OK;
  max_entries = std::max<uint32_t>(1, std::min(max_entries, n));
  // every split attempt takes two node slots; a node fails at most once (it is then marked
  // unsplittable), so attempts <= (max_entries - 1) successes + at most 2 * max_entries failures
  const size_t max_nodes = 6 * (size_t)max_entries + 8;
  DevBuf d_nodes, d_perm, d_tmp, d_jobs;
  cudaError_t e;
  if ((e = d_nodes.ensure(sizeof(Node) * max_nodes)) != cudaSuccess) return cuda_check(e, "alloc vq nodes");
  if ((e = d_perm.ensure(sizeof(uint32_t) * n)) != cudaSuccess) return cuda_check(e, "alloc vq perm");
  if ((e = d_tmp.ensure(sizeof(uint32_t) * n)) != cudaSuccess) return cuda_check(e, "alloc vq tmp");
  if ((e = d_jobs.ensure(sizeof(SplitJob) * max_entries)) != cudaSuccess) return cuda_check(e, "alloc vq jobs");
  Node* nodes = static_cast<Node*>(d_nodes.ptr);
  k_iota<<<256, 256, 0, s>>>(static_cast<uint32_t*>(d_perm.ptr), n);
  k_vq_root<D><<<1, kVqThreads, 0, s>>>(d_vec, d_w, n, nodes);
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
    std::vector<SplitJob> jobs(take);
    for (size_t i = 0; i < take; i++) {
      jobs[i].parent = cand[i];
      jobs[i].left = (int)used++;
      jobs[i].right = (int)used++;
    }
    if ((e = cudaMemcpyAsync(d_jobs.ptr, jobs.data(), sizeof(SplitJob) * take, cudaMemcpyHostToDevice, s)) != cudaSuccess)
      return cuda_check(e, "copy vq jobs");
    k_vq_split<D><<<(unsigned)take, kVqThreads, 0, s>>>(d_vec, d_w, static_cast<uint32_t*>(d_perm.ptr),
                                                         static_cast<uint32_t*>(d_tmp.ptr), nodes,
                                                         static_cast<const SplitJob*>(d_jobs.ptr));
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(e, "launch k_vq_split");
    if ((e = cudaMemcpyAsync(h.data(), nodes, sizeof(Node) * used, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
      return cuda_check(e, "read vq nodes");
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_check(e, "sync");
    std::vector<int> next;
    bool progressed = false;
    std::vector<char> split(used, 0);
    for (const SplitJob& j : jobs)
      if (!h[j.parent].unsplittable) { split[j.parent] = 1; progressed = true; }
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

// Squared error (perceptual or RGB weights) of the 4-colour block (lo, hi) over the unique colours,
// each pixel on its nearest colour; one warp, result on every lane.
__device__ __forceinline__ unsigned long long warp_pair_error(uint32_t lo, uint32_t hi, const uint32_t* ucol,
                                                               const uint32_t* ucnt, int U, bool perc) {
  int col[4][3];
  colors4(lo, hi, col);
  unsigned long long e = 0;
  for (int i = (int)(threadIdx.x & 31); i < U; i += 32) {
    const uint32_t c = ucol[i];
    const int r = (int)(c & 255), g = (int)((c >> 8) & 255), b = (int)((c >> 16) & 255);
    uint32_t bd = cdist(perc, r, g, b, col[0][0], col[0][1], col[0][2]);
    bd = min(bd, cdist(perc, r, g, b, col[1][0], col[1][1], col[1][2]));
    bd = min(bd, cdist(perc, r, g, b, col[2][0], col[2][1], col[2][2]));
    bd = min(bd, cdist(perc, r, g, b, col[3][0], col[3][1], col[3][2]));
    e += (unsigned long long)bd * ucnt[i];
  }
  for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xFFFFFFFFu, e, o);
  return e;
}

// Evaluates the candidate pairs cand[0..n) (lo | hi << 16), warp per candidate; returns the best
// (lowest error, then lowest index) to every thread through shared memory.
__device__ void best_candidate(const uint32_t* cand, int n, const uint32_t* ucol, const uint32_t* ucnt, int U, bool perc,
                               unsigned long long* s_be, uint32_t* s_bi, unsigned long long& err, uint32_t& pair) {
  const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  unsigned long long be = ~0ull;
  uint32_t bi = 0xFFFFFFFFu;
  for (int i = warp; i < n; i += nw) {
    const unsigned long long e = warp_pair_error(cand[i] & 0xFFFFu, cand[i] >> 16, ucol, ucnt, U, perc);
    if (e < be) { be = e; bi = (uint32_t)i; }
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
    __shared__ uint32_t s_key[kUniqCap], s_cnt[kUniqCap];
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
      for (int j = 0; j < nm; j++) { s_key[at + j] = mine_key[j]; s_cnt[at + j] = mine_cnt[j]; }
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
        best_candidate(s_cand, 1, s_key, s_cnt, U, perc, s_be, s_bi, berr, pair);
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
          best_candidate(s_cand, npl * nph, s_key, s_cnt, U, perc, s_be, s_bi, e, pair);
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
          best_candidate(s_cand, n, s_key, s_cnt, U, perc, s_be, s_bi, e, pair);
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
    if (threadIdx.x == 0) {
      double hist[4], D2[4][3], DD[4][3];
      for (int q = 0; q < 4; q++) {
        hist[q] = (double)s_stat[q];
        for (int c = 0; c < 3; c++) { D2[q][c] = (double)s_stat[4 + q * 3 + c]; DD[q][c] = (double)s_stat[16 + q * 3 + c]; }
      }
      auto err_of = [&](uint32_t L, uint32_t H) {
        int cc[4][3];
        colors4(L, H, cc);
        double er = 0;
        for (int q = 0; q < 4; q++) {
          double d[3];
          for (int c = 0; c < 3; c++) d[c] = hist[q] * cc[q][c] * cc[q][c] - D2[q][c] * cc[q][c] + DD[q][c];
          er += perc ? d[0] * 8 + d[1] * 25 + d[2] : d[0] + d[1] + d[2];
        }
        return er;
      };
      uint32_t wL = L0, wH = H0;
      double best = err_of(wL, wH);
      const bool preserveL = hist[0] + hist[2] > hist[1] + hist[3];
      bool improved = true;
      for (int iters = 8; improved && iters; iters--) {
        improved = false;
        uint32_t sol[54];
        int ns = 0;
        for (int which = 0; which < 2; which++) {
          const uint32_t E = which ? wH : wL, O2 = which ? wL : wH;
          const int b0 = E & 31, g0 = (E >> 5) & 63, r0 = (E >> 11) & 31;
          for (int b = b0 ? b0 - 1 : b0; b <= b0 + 1 && b <= 31; b++)
            for (int g = g0 ? g0 - 1 : g0; g <= g0 + 1 && g <= 63; g++)
              for (int r = r0 ? r0 - 1 : r0; r <= r0 + 1 && r <= 31; r++) {
                const uint32_t X = (uint32_t)((r << 11) | (g << 5) | b);
                if (X != E) sol[ns++] = X > O2 ? (X | (O2 << 16)) : (O2 | (X << 16));
              }
        }
        for (int i = 1; i < ns; i++) {  // sorted, as the reference evaluates them
          const uint32_t x = sol[i];
          int j = i - 1;
          while (j >= 0 && sol[j] > x) { sol[j + 1] = sol[j]; j--; }
          sol[j + 1] = x;
        }
        for (int i = 0; i < ns; i++) {
          if (i && sol[i] == sol[i - 1]) continue;
          uint32_t L = sol[i] & 0xFFFFu, H = sol[i] >> 16;
          if (L == H) {
            L += !preserveL ? ((~L & 0x1F) ? 0x1 : (~L & 0xF800) ? 0x800 : (~L & 0x7E0) ? 0x20 : 0) : (!L ? 0x1 : 0);
            H -= preserveL ? ((H & 0x1F) ? 0x1 : (H & 0xF800) ? 0x800 : (H & 0x7E0) ? 0x20 : 0) : (H == 0xFFFF ? 0x1 : 0);
            L &= 0xFFFFu; H &= 0xFFFFu;
          }
          const double er = err_of(L, H);
          if (er < best) { best = er; wL = L; wH = H; improved = true; }
        }
        if (best == 0) break;
      }
      if (wL <= wH) {  // keep 4-colour order (first > second)
        if (wL == wH) { if (wL < 0xFFFFu) wL++; else wH--; }
        else { const uint32_t t = wL; wL = wH; wH = t; }
      }
      s_LH[0] = wL;
      s_LH[1] = wH;
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
                          const uint32_t* __restrict__ cbsel, uint2* __restrict__ out, unsigned long long* __restrict__ sse) {
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
  out[b] = make_uint2(C.first | (C.second << 16), dxt);
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

}  // namespace hc

const void* single_colour_tables_host();

namespace {

struct HcBuffers {
  DevBuf chunks, derating, lweight, st, tiles, block_tile, block_enc, vec6, w6, count, cb6, tile_cluster, ccount,
      cstart, clist, clusters, bweight, block_cluster, selvec, selw, cb16, cbsel, block_sel, entry_err, entry_used,
      levels, flags, iota, used, keys, keys2, cub_tmp, sse;
};

}  // namespace

}  // namespace crngpu

using namespace crngpu;
using namespace crngpu::hc;

// Clustered DXT1 encode (dxt_hc::compress for cDXT1). See include/crngpu.h.
extern "C" int crngpu_hc_compress_dxt1(const uint8_t* d_blocks, const crngpu_hc_params* params, uint8_t* d_out,
                                       uint16_t* d_endpoint_idx, uint16_t* d_selector_idx, uint32_t* d_endpoints,
                                       uint32_t* d_selectors, crngpu_hc_stats* stats, void* stream) {
  clear_error();
  if (!d_blocks || !params || !d_out || params->struct_size != sizeof(crngpu_hc_params) || !params->num_blocks ||
      params->num_levels < 1 || params->num_levels > 16) {
    set_error("crngpu_hc_compress_dxt1: bad arguments");
    return CRNGPU_E_PARAM;
  }
  const crngpu_hc_params& P = *params;
  const uint32_t N = P.num_blocks;
  cudaStream_t s = as_stream(stream);
  cudaError_t e;
  HcBuffers B;
  // chunks of every level (block rows are processed in pairs; widths and heights are even)
  std::vector<Chunk> chunks;
  std::vector<float> derating(16 * 8), lweight(16);
  const int tile_derating[8] = {0, 1, 1, 2, 2, 2, 2, 3};
  std::vector<Level> lv(P.num_levels);
  for (uint32_t l = 0; l < P.num_levels; l++) {
    const auto& L = P.levels[l];
    if (!L.block_width || (L.block_width & 1) || L.num_blocks % (2 * L.block_width) || L.first_block + L.num_blocks > N) {
      set_error("crngpu_hc_compress_dxt1: level " + std::to_string(l) + " is not a whole number of 2x2 chunks");
      return CRNGPU_E_PARAM;
    }
    lv[l] = Level{L.first_block, L.num_blocks, L.block_width, L.weight};
    lweight[l] = L.weight;
    // crn_dxt_hc.cpp:121-134: colour derating per level and layout
    float d = P.adaptive_tile_color_psnr_derating;
    if (l && d > .25f) d = std::max(.25f, d / powf(3.0f, (float)l));
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
                                                 P.perceptual, static_cast<SolidTables*>(B.st.ptr), tiles,
                                                 static_cast<uint32_t*>(B.block_tile.ptr), static_cast<uint8_t*>(B.block_enc.ptr));
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(e, "launch k_hc_tiles");
  // endpoint VQ over the used tiles' vec6 (compacted in tile order, so the result is reproducible)
  if ((e = B.vec6.ensure(sizeof(float) * 6 * ntiles)) != cudaSuccess || (e = B.w6.ensure(4 * ntiles)) != cudaSuccess ||
      (e = B.count.ensure(16)) != cudaSuccess || (e = B.flags.ensure(ntiles)) != cudaSuccess ||
      (e = B.iota.ensure(4 * ntiles)) != cudaSuccess || (e = B.used.ensure(4 * ntiles)) != cudaSuccess ||
      (e = B.keys.ensure(4 * ntiles)) != cudaSuccess || (e = B.keys2.ensure(4 * ntiles)) != cudaSuccess)
    return cuda_check(e, "alloc vq input");
  k_tile_flags<<<(ntiles + 255) / 256, 256, 0, s>>>(tiles, ntiles, static_cast<uint8_t*>(B.flags.ptr),
                                                     static_cast<uint32_t*>(B.iota.ptr));
  size_t tmp_bytes = 0, tmp2 = 0;
  cub::DeviceSelect::Flagged(nullptr, tmp_bytes, static_cast<uint32_t*>(B.iota.ptr), static_cast<uint8_t*>(B.flags.ptr),
                             static_cast<uint32_t*>(B.used.ptr), static_cast<uint32_t*>(B.count.ptr), (int)ntiles, s);
  cub::DeviceRadixSort::SortPairs(nullptr, tmp2, static_cast<uint32_t*>(B.keys.ptr), static_cast<uint32_t*>(B.keys2.ptr),
                                  static_cast<uint32_t*>(B.used.ptr), static_cast<uint32_t*>(B.iota.ptr), (int)ntiles, 0, 32, s);
  if ((e = B.cub_tmp.ensure(std::max(tmp_bytes, tmp2) + 256)) != cudaSuccess) return cuda_check(e, "alloc cub scratch");
  tmp_bytes = B.cub_tmp.cap;
  if ((e = cub::DeviceSelect::Flagged(B.cub_tmp.ptr, tmp_bytes, static_cast<uint32_t*>(B.iota.ptr),
                                      static_cast<uint8_t*>(B.flags.ptr), static_cast<uint32_t*>(B.used.ptr),
                                      static_cast<uint32_t*>(B.count.ptr), (int)ntiles, s)) != cudaSuccess)
    return cuda_check(e, "select used tiles");
  uint32_t nused = 0;
  if ((e = cudaMemcpyAsync(&nused, B.count.ptr, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return cuda_check(e, "read count");
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_check(e, "sync");
  k_tile_vectors<<<(nused + 255) / 256, 256, 0, s>>>(tiles, static_cast<uint32_t*>(B.used.ptr), nused,
                                                      static_cast<float*>(B.vec6.ptr), static_cast<uint32_t*>(B.w6.ptr));
  uint32_t K = 0;
  const uint32_t frac = P.vq_round_fraction ? P.vq_round_fraction : kDefaultRoundFraction;
  int rc = tree_vq<6>(static_cast<float*>(B.vec6.ptr), static_cast<uint32_t*>(B.w6.ptr), nused,
                      std::min(nused, P.color_endpoint_codebook_size), frac, B.cb6, &K, s);
  if (rc != CRNGPU_OK) return rc;
  if ((e = B.tile_cluster.ensure(4 * ntiles)) != cudaSuccess) return cuda_check(e, "alloc tile clusters");
  k_nearest_vec6<<<(ntiles + 255) / 256, 256, 0, s>>>(tiles, ntiles, static_cast<float*>(B.cb6.ptr), K,
                                                       static_cast<uint32_t*>(B.tile_cluster.ptr));
  // cluster -> tiles (CSR): used tiles sorted by cluster (stable radix sort keeps tile order)
  if ((e = B.ccount.ensure(4 * (K + 1))) != cudaSuccess || (e = B.cstart.ensure(4 * (K + 1))) != cudaSuccess ||
      (e = B.clist.ensure(4 * ntiles)) != cudaSuccess)
    return cuda_check(e, "alloc cluster lists");
  cudaMemsetAsync(B.ccount.ptr, 0, 4 * (K + 1), s);
  k_count_clusters<<<(ntiles + 255) / 256, 256, 0, s>>>(static_cast<uint32_t*>(B.tile_cluster.ptr), ntiles,
                                                         static_cast<uint32_t*>(B.ccount.ptr));
  k_used_clusters<<<(nused + 255) / 256, 256, 0, s>>>(static_cast<uint32_t*>(B.used.ptr), nused,
                                                       static_cast<uint32_t*>(B.tile_cluster.ptr), static_cast<uint32_t*>(B.keys.ptr));
  int key_bits = 1;
  while ((1u << key_bits) < K) key_bits++;
  tmp_bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, static_cast<uint32_t*>(B.keys.ptr), static_cast<uint32_t*>(B.keys2.ptr),
                                  static_cast<uint32_t*>(B.used.ptr), static_cast<uint32_t*>(B.clist.ptr), (int)nused, 0,
                                  key_bits, s);
  if ((e = B.cub_tmp.ensure(tmp_bytes + 256)) != cudaSuccess) return cuda_check(e, "alloc cub scratch");
  tmp_bytes = B.cub_tmp.cap;
  if ((e = cub::DeviceRadixSort::SortPairs(B.cub_tmp.ptr, tmp_bytes, static_cast<uint32_t*>(B.keys.ptr),
                                           static_cast<uint32_t*>(B.keys2.ptr), static_cast<uint32_t*>(B.used.ptr),
                                           static_cast<uint32_t*>(B.clist.ptr), (int)nused, 0, key_bits, s)) != cudaSuccess)
    return cuda_check(e, "sort tiles by cluster");
  std::vector<uint32_t> cnt(K + 1), start(K + 1);
  if ((e = cudaMemcpyAsync(cnt.data(), B.ccount.ptr, 4 * K, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return cuda_check(e, "read counts");
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_check(e, "sync");
  uint32_t run = 0;
  for (uint32_t k = 0; k < K; k++) { start[k] = run; run += cnt[k]; }
  start[K] = run;
  if ((e = cudaMemcpyAsync(B.cstart.ptr, start.data(), 4 * (K + 1), cudaMemcpyHostToDevice, s)) != cudaSuccess)
    return cuda_check(e, "copy cluster starts");
  if ((e = B.clusters.ensure(sizeof(ClusterOut) * K)) != cudaSuccess) return cuda_check(e, "alloc clusters");
  ClusterOut* cl = static_cast<ClusterOut*>(B.clusters.ptr);
  k_cluster_fit<<<K, kFitThreads, 0, s>>>(blocks, static_cast<Chunk*>(B.chunks.ptr), tiles,
                                           static_cast<uint32_t*>(B.cstart.ptr), static_cast<uint32_t*>(B.clist.ptr),
                                           P.perceptual, cl);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(e, "launch k_cluster_fit");
  // per-block selectors and weights -> selector VQ
  if ((e = B.bweight.ensure(4 * N)) != cudaSuccess || (e = B.block_cluster.ensure(4 * N)) != cudaSuccess ||
      (e = B.selvec.ensure(sizeof(float) * 16 * N)) != cudaSuccess || (e = B.selw.ensure(4 * N)) != cudaSuccess)
    return cuda_check(e, "alloc selectors");
  if ((e = B.sse.ensure(16)) != cudaSuccess) return cuda_check(e, "alloc sse");
  cudaMemsetAsync(B.sse.ptr, 0, 16, s);
  k_block_weights<<<(N + 255) / 256, 256, 0, s>>>(static_cast<Level*>(B.levels.ptr), P.num_levels, N, static_cast<float*>(B.bweight.ptr));
  k_block_selectors<<<(N + 127) / 128, 128, 0, s>>>(blocks, N, static_cast<uint32_t*>(B.block_tile.ptr),
                                                     static_cast<uint32_t*>(B.tile_cluster.ptr),
                                                     static_cast<uint8_t*>(B.block_enc.ptr), static_cast<float*>(B.bweight.ptr),
                                                     cl, P.perceptual, static_cast<uint32_t*>(B.block_cluster.ptr),
                                                     static_cast<float*>(B.selvec.ptr), static_cast<uint32_t*>(B.selw.ptr),
                                                     static_cast<unsigned long long*>(B.sse.ptr));
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(e, "launch k_block_selectors");
  uint32_t KS = 0;
  rc = tree_vq<16>(static_cast<float*>(B.selvec.ptr), static_cast<uint32_t*>(B.selw.ptr), N,
                   std::min(N, P.color_selector_codebook_size), frac, B.cb16, &KS, s);
  if (rc != CRNGPU_OK) return rc;
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
                                            static_cast<uint32_t*>(B.block_sel.ptr), cbsel, reinterpret_cast<uint2*>(d_out),
                                            static_cast<unsigned long long*>(B.sse.ptr) + 1);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(e, "launch hc selector kernels");
  // optional index outputs
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
  }
  if (stats) {
    unsigned long long sse[2] = {0, 0};
    if ((e = cudaMemcpyAsync(sse, B.sse.ptr, 16, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return cuda_check(e, "read sse");
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_check(e, "sync");
    stats->color_endpoints = K;
    stats->color_selectors = KS;
    stats->tiles = nused;
    stats->sse_endpoints = (double)sse[0];
    stats->sse_final = (double)sse[1];
  }
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_check(e, "sync");
  return CRNGPU_OK;
}

// Codebook sizes of crn_comp::quantize_images (crnlib/crn_comp.cpp:541-577) for a quality level.
extern "C" int crngpu_hc_codebook_sizes(uint32_t width, uint32_t height, uint32_t quality_level, uint32_t format,
                                        uint32_t* sizes4) {
  if (!sizes4 || !width || !height) return CRNGPU_E_PARAM;
  const uint32_t kMin = 32, kMax = 8192;  // cCRNMinPaletteSize, cCRNMaxPaletteSize (inc/crnlib.h:117-118)
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
}

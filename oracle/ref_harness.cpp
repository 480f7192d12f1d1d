// Golden-vector harness around the reference crnlib (test infrastructure only).
//
// This file is compiled together with the reference's own sources by oracle/Makefile into
// oracle/_ref/libcrnref.so. It exposes a small extern "C" surface that the golden-fixture
// generator (tests/golden/make_golden.py) drives through ctypes. Nothing in the product
// links or loads this library.
//
// Entry points used (reference file:line):
//   crn_create_block_compressor / crn_compress_block / crn_free_block_compressor
//       inc/crnlib.h:674-682, crnlib/crnlib.cpp:351-418 (dxt_image::set_block_pixels stack)
//   crn_compress (comp params + mip params)   inc/crnlib.h:614, crnlib/crnlib.cpp:242-267
//   crnd_unpack_begin / crnd_unpack_level / crnd_unpack_end   inc/crn_defs.h:174-205
//   crnd_get_texture_info / crnd_get_level_info              inc/crn_defs.h:152-160
//   crnlib::dxt_hc::compress (clustered DXT1)                 crnlib/crn_dxt_hc.cpp:97-316
//   crnlib::image_utils::resample_multithreaded (mip levels)   crnlib/crn_image_utils.cpp:662-874
//   crn_compress with crn_mipmap_params, crn_decompress_crn_to_dds   inc/crnlib.h:614-620
//   crnd_validate_file / _get_level_data / segmented files        inc/crn_defs.h:153-221
#include <cstdint>
#include <cstring>
#include <cstdlib>
#include <vector>
#include <thread>
#include <atomic>
#include <chrono>

#include "crnlib.h"
#include "crn_defs.h"
#include "crn_dxt_hc.h"
#include "crn_dxt_fast.h"
#include "crn_threading.h"
#include "crn_image.h"
#include "crn_image_utils.h"

namespace {

crn_comp_params make_params(uint32_t fmt, uint32_t flags, uint32_t dxt_quality) {
  crn_comp_params p;
  p.m_format = static_cast<crn_format>(fmt);
  p.m_flags = flags;
  p.m_dxt_quality = static_cast<crn_dxt_quality>(dxt_quality);
  p.m_width = 4;
  p.m_height = 4;
  return p;
}

}  // namespace

extern "C" {

// Compresses n independent 4x4 blocks (n x 16 RGBA8 pixels, row-major inside the block)
// with one reference block-compressor context. flags are crn_comp_flags; pass
// cCRNCompFlagDisableEndpointCaching (32) for thread-count-independent results.
// out receives n x bytes_per_block. Returns bytes per block, or 0 on failure.
int ref_compress_blocks(const uint8_t* rgba, uint32_t n, uint32_t fmt, uint32_t flags,
                        uint32_t dxt_quality, uint8_t* out) {
  crn_comp_params p = make_params(fmt, flags, dxt_quality);
  crn_block_compressor_context_t ctx = crn_create_block_compressor(p);
  if (!ctx) return 0;
  const uint32_t bpb = crnd::crnd_get_bytes_per_dxt_block(p.m_format);
  for (uint32_t i = 0; i < n; i++) {
    crn_compress_block(ctx, reinterpret_cast<const crn_uint32*>(rgba + (size_t)i * 64), out + (size_t)i * bpb);
  }
  crn_free_block_compressor(ctx);
  return (int)bpb;
}

// Same as ref_compress_blocks but splits the blocks over `threads` OS threads, one
// block-compressor context per thread (the way the reference's block API is meant to
// be used from several threads). Returns elapsed wall seconds through *seconds.
int ref_compress_blocks_mt(const uint8_t* rgba, uint32_t n, uint32_t fmt, uint32_t flags,
                           uint32_t dxt_quality, uint8_t* out, uint32_t threads, double* seconds) {
  if (threads < 1) threads = 1;
  crn_comp_params p = make_params(fmt, flags, dxt_quality);
  const uint32_t bpb = crnd::crnd_get_bytes_per_dxt_block(p.m_format);
  std::atomic<uint32_t> next(0);
  auto t0 = std::chrono::steady_clock::now();
  std::vector<std::thread> pool;
  for (uint32_t t = 0; t < threads; t++) {
    pool.emplace_back([&]() {
      crn_block_compressor_context_t ctx = crn_create_block_compressor(p);
      if (!ctx) return;
      for (;;) {
        uint32_t i0 = next.fetch_add(64);
        if (i0 >= n) break;
        uint32_t i1 = i0 + 64 < n ? i0 + 64 : n;
        for (uint32_t i = i0; i < i1; i++)
          crn_compress_block(ctx, reinterpret_cast<const crn_uint32*>(rgba + (size_t)i * 64), out + (size_t)i * bpb);
      }
      crn_free_block_compressor(ctx);
    });
  }
  for (auto& th : pool) th.join();
  auto t1 = std::chrono::steady_clock::now();
  if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
  return (int)bpb;
}

// Compresses a texture given as faces x levels RGBA8 mip images (face-major; level l is
// max(1,w>>l) x max(1,h>>l), tightly packed, concatenated) to a .crn (file_type 0) or .dds
// (file_type 1) file in memory.
// quality is m_quality_level (0..255). Returns the file size (0 on failure); the file is copied
// to out when it fits in out_cap.
uint32_t ref_compress_texture(const uint8_t* rgba_levels, uint32_t width, uint32_t height, uint32_t levels, uint32_t faces,
                              uint32_t fmt, uint32_t file_type, uint32_t quality, uint32_t flags,
                              uint32_t dxt_quality, uint32_t helper_threads, uint8_t* out, uint32_t out_cap) {
  crn_comp_params p;
  p.m_file_type = file_type ? cCRNFileTypeDDS : cCRNFileTypeCRN;
  p.m_width = width;
  p.m_height = height;
  p.m_levels = levels;
  p.m_faces = faces;
  p.m_format = static_cast<crn_format>(fmt);
  p.m_flags = flags;
  p.m_quality_level = quality;
  p.m_dxt_quality = static_cast<crn_dxt_quality>(dxt_quality);
  p.m_num_helper_threads = helper_threads;
  size_t ofs = 0;
  for (uint32_t f = 0; f < faces; f++) {
    for (uint32_t l = 0; l < levels; l++) {
      uint32_t w = width >> l ? width >> l : 1, h = height >> l ? height >> l : 1;
      p.m_pImages[f][l] = reinterpret_cast<const crn_uint32*>(rgba_levels + ofs);
      ofs += (size_t)w * h * 4;
    }
  }
  crn_mipmap_params mp;
  mp.m_mode = cCRNMipModeUseSourceMips;
  crn_uint32 size = 0;
  void* data = crn_compress(p, mp, size);
  if (!data) return 0;
  if (size <= out_cap && out) memcpy(out, data, size);
  crn_free_block(data);
  return size;
}

// crn_compress to .crn with m_target_bitrate set (the interpolative quality search of
// create_compressed_texture, crnlib/crn_texture_comp.cpp:143-260): returns the file size (0 on
// failure) and the chosen quality level and the bitrate crn_compress reports.
uint32_t ref_compress_texture_bitrate(const uint8_t* rgba_levels, uint32_t width, uint32_t height, uint32_t levels,
                                      uint32_t fmt, uint32_t flags, float target_bitrate, uint32_t helper_threads,
                                      uint32_t* actual_quality, float* actual_bitrate) {
  crn_comp_params p;
  p.m_file_type = cCRNFileTypeCRN;
  p.m_width = width;
  p.m_height = height;
  p.m_levels = levels;
  p.m_faces = 1;
  p.m_format = static_cast<crn_format>(fmt);
  p.m_flags = flags;
  p.m_target_bitrate = target_bitrate;
  p.m_num_helper_threads = helper_threads;
  size_t ofs = 0;
  for (uint32_t l = 0; l < levels; l++) {
    uint32_t w = width >> l ? width >> l : 1, h = height >> l ? height >> l : 1;
    p.m_pImages[0][l] = reinterpret_cast<const crn_uint32*>(rgba_levels + ofs);
    ofs += (size_t)w * h * 4;
  }
  crn_mipmap_params mp;
  mp.m_mode = cCRNMipModeUseSourceMips;
  crn_uint32 size = 0, q = 0;
  float rate = 0.0f;
  void* data = crn_compress(p, mp, size, &q, &rate);
  if (!data) return 0;
  crn_free_block(data);
  if (actual_quality) *actual_quality = q;
  if (actual_bitrate) *actual_bitrate = rate;
  return size;
}

// Transcodes one level of a .crn file with the reference crnd unpacker into out
// (faces x blocks_y x row_pitch bytes, row_pitch = minimal). Returns bytes written or 0.
uint32_t ref_unpack_level(const uint8_t* crn, uint32_t crn_size, uint32_t level, uint8_t* out, uint32_t out_cap) {
  crnd::crn_texture_info ti;
  if (!crnd::crnd_get_texture_info(crn, crn_size, &ti)) return 0;
  crnd::crn_level_info li;
  if (!crnd::crnd_get_level_info(crn, crn_size, level, &li)) return 0;
  const uint32_t pitch = li.m_blocks_x * li.m_bytes_per_block;
  const uint32_t face_size = pitch * li.m_blocks_y;
  if ((uint64_t)face_size * ti.m_faces > out_cap) return 0;
  crnd::crnd_unpack_context ctx = crnd::crnd_unpack_begin(crn, crn_size);
  if (!ctx) return 0;
  void* faces[6];
  for (uint32_t f = 0; f < ti.m_faces; f++) faces[f] = out + (size_t)f * face_size;
  bool ok = crnd::crnd_unpack_level(ctx, faces, face_size, pitch, level);
  crnd::crnd_unpack_end(ctx);
  return ok ? face_size * ti.m_faces : 0;
}

// Times `reps` full transcodes (every level) of a .crn file on one thread; returns seconds.
double ref_time_unpack(const uint8_t* crn, uint32_t crn_size, uint32_t reps, uint8_t* scratch, uint32_t scratch_cap) {
  crnd::crn_texture_info ti;
  if (!crnd::crnd_get_texture_info(crn, crn_size, &ti)) return -1.0;
  auto t0 = std::chrono::steady_clock::now();
  for (uint32_t r = 0; r < reps; r++) {
    crnd::crnd_unpack_context ctx = crnd::crnd_unpack_begin(crn, crn_size);
    if (!ctx) return -1.0;
    for (uint32_t l = 0; l < ti.m_levels; l++) {
      crnd::crn_level_info li;
      crnd::crnd_get_level_info(crn, crn_size, l, &li);
      const uint32_t pitch = li.m_blocks_x * li.m_bytes_per_block;
      const uint32_t face_size = pitch * li.m_blocks_y;
      if ((uint64_t)face_size * ti.m_faces > scratch_cap) return -1.0;
      void* faces[6];
      for (uint32_t f = 0; f < ti.m_faces; f++) faces[f] = scratch + (size_t)f * face_size;
      crnd::crnd_unpack_level(ctx, faces, face_size, pitch, l);
    }
    crnd::crnd_unpack_end(ctx);
  }
  auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double>(t1 - t0).count();
}

// The reference's clustered DXT1 compressor (crnlib::dxt_hc::compress, crnlib/crn_dxt_hc.cpp:97-316)
// run directly on blocks in crn_comp's layout (crnlib/crn_comp.cpp:717-741), with crn_comp's level
// weights. level_info: first_block, num_blocks, block_width per level. Writes the DXT1 blocks the
// returned codebooks and indices describe (endpoints as stored, linear selectors converted to DXT
// order) to out (n x 8) and stats[0..2] = tiles, endpoint entries, selector entries. Returns 1.
int ref_dxt_hc_dxt1(const uint8_t* rgba_blocks, uint32_t n, uint32_t nlevels, const uint32_t* level_info,
                    uint32_t faces, uint32_t endpoint_codebook, uint32_t selector_codebook, int perceptual,
                    uint32_t threads, uint8_t* out, uint32_t* stats) {
  crnlib::task_pool pool;
  if (!pool.init(threads > 1 ? threads - 1 : 0)) return 0;
  crnlib::dxt_hc::params p;
  p.m_num_blocks = n;
  p.m_num_levels = nlevels;
  p.m_num_faces = faces;
  p.m_format = crnlib::cDXT1;
  p.m_perceptual = perceptual != 0;
  p.m_hierarchical = true;
  p.m_color_endpoint_codebook_size = endpoint_codebook;
  p.m_color_selector_codebook_size = selector_codebook;
  p.m_pTask_pool = &pool;
  for (uint32_t l = 0; l < nlevels; l++) {
    p.m_levels[l].m_first_block = level_info[3 * l];
    p.m_levels[l].m_num_blocks = level_info[3 * l + 1];
    p.m_levels[l].m_block_width = level_info[3 * l + 2];
    p.m_levels[l].m_weight = crnlib::math::minimum(12.0f, powf(1.3f, (float)l));
  }
  std::vector<uint8_t> copy(rgba_blocks, rgba_blocks + (size_t)n * 64);
  crnlib::vector<crnlib::dxt_hc::endpoint_indices_details> ei;
  crnlib::vector<crnlib::dxt_hc::selector_indices_details> si;
  crnlib::vector<crnlib::uint32> ce, ae, cs;
  crnlib::vector<crnlib::uint64> as;
  crnlib::dxt_hc hc;
  if (!hc.compress(reinterpret_cast<crnlib::color_quad_u8(*)[16]>(copy.data()), ei, si, ce, ae, cs, as, p)) return 0;
  static const uint8_t from_linear[4] = {0, 2, 3, 1};
  for (uint32_t b = 0; b < n; b++) {
    const uint32_t ep = ce[ei[b].color], lin = cs[si[b].color];
    uint32_t dxt = 0;
    for (int q = 0; q < 16; q++) dxt |= (uint32_t)from_linear[(lin >> (2 * q)) & 3] << (2 * q);
    memcpy(out + (size_t)b * 8, &ep, 4);
    memcpy(out + (size_t)b * 8 + 4, &dxt, 4);
  }
  stats[0] = hc.m_num_tiles;
  stats[1] = ce.size();
  stats[2] = cs.size();
  pool.deinit();
  return 1;
}

// The reference's clustered compressor for an alpha-carrying format (fmt: 0 DXT5 with alpha
// channel 3, 1 DXN_XY, 2 DXN_YX, 3 DXT5A on channel 3), same layout and weights as
// ref_dxt_hc_dxt1. codebooks: colour endpoints, colour selectors, alpha endpoints, alpha selectors.
// Writes n x 16 bytes (DXT5, DXN) or n x 8 (DXT5A): alpha blocks are endpoints (first, second)
// then 16 3-bit selectors converted from linear to DXT5 order. stats[0..4] = tiles, colour
// endpoints, colour selectors, alpha endpoints, alpha selectors. Returns bytes per block.
int ref_dxt_hc_alpha(const uint8_t* rgba_blocks, uint32_t n, uint32_t nlevels, const uint32_t* level_info,
                     uint32_t faces, uint32_t fmt, const uint32_t* codebooks, int perceptual, uint32_t threads,
                     uint8_t* out, uint32_t* stats) {
  crnlib::task_pool pool;
  if (!pool.init(threads > 1 ? threads - 1 : 0)) return 0;
  crnlib::dxt_hc::params p;
  p.m_num_blocks = n;
  p.m_num_levels = nlevels;
  p.m_num_faces = faces;
  p.m_format = fmt == 0 ? crnlib::cDXT5 : fmt == 1 ? crnlib::cDXN_XY : fmt == 2 ? crnlib::cDXN_YX : crnlib::cDXT5A;
  p.m_perceptual = perceptual != 0;
  p.m_hierarchical = true;
  p.m_color_endpoint_codebook_size = codebooks[0];
  p.m_color_selector_codebook_size = codebooks[1];
  p.m_alpha_endpoint_codebook_size = codebooks[2];
  p.m_alpha_selector_codebook_size = codebooks[3];
  if (fmt == 0 || fmt == 3) p.m_alpha_component_indices[0] = 3;
  else if (fmt == 1) { p.m_alpha_component_indices[0] = 0; p.m_alpha_component_indices[1] = 1; }
  else { p.m_alpha_component_indices[0] = 1; p.m_alpha_component_indices[1] = 0; }
  p.m_pTask_pool = &pool;
  for (uint32_t l = 0; l < nlevels; l++) {
    p.m_levels[l].m_first_block = level_info[3 * l];
    p.m_levels[l].m_num_blocks = level_info[3 * l + 1];
    p.m_levels[l].m_block_width = level_info[3 * l + 2];
    p.m_levels[l].m_weight = crnlib::math::minimum(12.0f, powf(1.3f, (float)l));
  }
  std::vector<uint8_t> copy(rgba_blocks, rgba_blocks + (size_t)n * 64);
  crnlib::vector<crnlib::dxt_hc::endpoint_indices_details> ei;
  crnlib::vector<crnlib::dxt_hc::selector_indices_details> si;
  crnlib::vector<crnlib::uint32> ce, ae, cs;
  crnlib::vector<crnlib::uint64> as;
  crnlib::dxt_hc hc;
  if (!hc.compress(reinterpret_cast<crnlib::color_quad_u8(*)[16]>(copy.data()), ei, si, ce, ae, cs, as, p)) return 0;
  static const uint8_t from_linear[4] = {0, 2, 3, 1};
  static const uint8_t from_linear8[8] = {0, 2, 3, 4, 5, 6, 7, 1};
  const uint32_t nalpha = (fmt == 1 || fmt == 2) ? 2 : 1;
  const uint32_t bpb = fmt == 3 ? 8 : 16;
  for (uint32_t b = 0; b < n; b++) {
    uint8_t* o = out + (size_t)b * bpb;
    for (uint32_t a = 0; a < nalpha; a++) {
      const uint32_t ep = ae[ei[b].component[1 + a]];
      const uint64_t lin = as[si[b].component[1 + a]];
      uint64_t dxt = 0;
      for (int q = 0; q < 16; q++) dxt |= (uint64_t)from_linear8[(lin >> (3 * q)) & 7] << (3 * q);
      o[8 * a] = (uint8_t)(ep & 255);
      o[8 * a + 1] = (uint8_t)((ep >> 8) & 255);
      for (int k = 0; k < 6; k++) o[8 * a + 2 + k] = (uint8_t)(dxt >> (8 * k));
    }
    if (fmt == 0) {
      const uint32_t ep = ce[ei[b].color], lin = cs[si[b].color];
      uint32_t dxt = 0;
      for (int q = 0; q < 16; q++) dxt |= (uint32_t)from_linear[(lin >> (2 * q)) & 3] << (2 * q);
      memcpy(o + 8, &ep, 4);
      memcpy(o + 12, &dxt, 4);
    }
  }
  stats[0] = hc.m_num_tiles;
  stats[1] = ce.size();
  stats[2] = cs.size();
  stats[3] = ae.size();
  stats[4] = as.size();
  pool.deinit();
  return (int)bpb;
}

// Squared RGB error of dxt_fast::compress_color_block on n pixels (n = 16, 32 or 64), measured
// against the 4-colour palette as dxt_hc::determine_tiles_task does (crnlib/crn_dxt_hc.cpp:459-472).
uint32_t ref_dxt_fast_tile_error(const uint8_t* rgba, uint32_t n) {
  uint8_t sel[64];
  crnlib::uint low16, high16;
  const crnlib::color_quad_u8* px = reinterpret_cast<const crnlib::color_quad_u8*>(rgba);
  crnlib::dxt_fast::compress_color_block(n, px, low16, high16, sel);
  crnlib::color_quad_u8 colors[4];
  crnlib::dxt1_block::get_block_colors4(colors, (crnlib::uint16)low16, (crnlib::uint16)high16);
  uint32_t err = 0;
  for (uint32_t p = 0; p < n; p++)
    for (int c = 0; c < 3; c++) {
      const uint32_t d = px[p][c] - colors[sel[p]][c];
      err += d * d;
    }
  return err;
}

// crnlib::image_utils::resample_multithreaded (crnlib/crn_image_utils.cpp:662-874), the resampler
// mipmapped_texture::generate_mipmaps (crnlib/crn_mipmapped_texture.cpp:2140-2215) runs for every
// mip level from the level-0 image: the filter by name, filter scale (the mip "blurriness"), sRGB
// gamma filtering, wrap or clamp addressing, 3 or 4 components. Returns 1 on success.
int ref_resample(const uint8_t* rgba, uint32_t w, uint32_t h, uint32_t dst_w, uint32_t dst_h, const char* filter,
                 float filter_scale, int srgb, int wrap, uint32_t num_comps, uint8_t* out) {
  crnlib::image_u8 src(w, h);
  for (uint32_t y = 0; y < h; y++) std::memcpy(src.get_scanline(y), rgba + (size_t)y * w * 4, (size_t)w * 4);
  crnlib::image_u8 dst;
  crnlib::image_utils::resample_params rp;
  rp.m_dst_width = dst_w;
  rp.m_dst_height = dst_h;
  rp.m_pFilter = filter;
  rp.m_filter_scale = filter_scale;
  rp.m_srgb = srgb != 0;
  rp.m_wrapping = wrap != 0;
  rp.m_first_comp = 0;
  rp.m_num_comps = num_comps;
  rp.m_multithreaded = true;
  if (!crnlib::image_utils::resample_multithreaded(src, dst, rp)) return 0;
  for (uint32_t y = 0; y < dst_h; y++) std::memcpy(out + (size_t)y * dst_w * 4, dst.get_scanline(y), (size_t)dst_w * 4);
  return 1;
}

// crn_compress with mip parameters (inc/crnlib.h:614, crnlib/crn_texture_comp.cpp:580-613):
// faces top-level RGBA8 images (w x h each, face after face) and the crn_mipmap_params fields that
// mip generation reads. Returns the file size (0 on failure); copied to out when it fits.
uint32_t ref_compress_mips(const uint8_t* rgba_faces, uint32_t width, uint32_t height, uint32_t faces, uint32_t fmt,
                           uint32_t file_type, uint32_t quality, uint32_t flags, uint32_t mip_mode, uint32_t filter,
                           float blurriness, uint32_t gamma_filtering, uint32_t tiled, uint32_t max_levels,
                           uint32_t min_mip_size, uint8_t* out, uint32_t out_cap) {
  crn_comp_params p;
  p.m_file_type = file_type ? cCRNFileTypeDDS : cCRNFileTypeCRN;
  p.m_width = width;
  p.m_height = height;
  p.m_levels = 1;
  p.m_faces = faces;
  p.m_format = static_cast<crn_format>(fmt);
  p.m_flags = flags;
  p.m_quality_level = quality;
  for (uint32_t f = 0; f < faces; f++)
    p.m_pImages[f][0] = reinterpret_cast<const crn_uint32*>(rgba_faces + (size_t)f * width * height * 4);
  crn_mipmap_params mp;
  mp.m_mode = static_cast<crn_mip_mode>(mip_mode);
  mp.m_filter = static_cast<crn_mip_filter>(filter);
  mp.m_blurriness = blurriness;
  mp.m_gamma_filtering = gamma_filtering;
  mp.m_tiled = tiled;
  mp.m_max_levels = max_levels;
  mp.m_min_mip_size = min_mip_size;
  crn_uint32 size = 0;
  void* data = crn_compress(p, mp, size);
  if (!data) return 0;
  if (size <= out_cap && out) memcpy(out, data, size);
  crn_free_block(data);
  return size;
}

// crn_decompress_crn_to_dds (inc/crnlib.h:620, crnlib/crnlib.cpp:269-292). Returns the .dds size
// (0 on failure); copied to out when it fits.
uint32_t ref_crn_to_dds(const uint8_t* crn, uint32_t crn_size, uint8_t* out, uint32_t out_cap) {
  crn_uint32 size = crn_size;
  void* data = crn_decompress_crn_to_dds(crn, size);
  if (!data) return 0;
  if (size <= out_cap && out) memcpy(out, data, size);
  crn_free_block(data);
  return size;
}

// The crnd header API on one file (inc/crn_defs.h:139-221): writes to info[] the validate result
// and every crn_file_info field, every crn_texture_info field, each level's crn_level_info fields
// and crnd_get_level_data size, crnd_get_segmented_file_size and the crnd_create_segmented_file
// result; the segmented base file goes to seg (when it fits in seg_cap). Returns the number of
// values written.
uint32_t ref_crnd_probe(const uint8_t* crn, uint32_t crn_size, uint32_t* info, uint8_t* seg, uint32_t seg_cap) {
  uint32_t n = 0;
  crnd::crn_file_info fi;
  info[n++] = crnd::crnd_validate_file(crn, crn_size, &fi) ? 1u : 0u;
  const uint32_t* f = reinterpret_cast<const uint32_t*>(&fi);
  for (size_t k = 0; k < sizeof(fi) / 4; k++) info[n++] = f[k];
  crnd::crn_texture_info ti;
  info[n++] = crnd::crnd_get_texture_info(crn, crn_size, &ti) ? 1u : 0u;
  info[n++] = ti.m_width;
  info[n++] = ti.m_height;
  info[n++] = ti.m_levels;
  info[n++] = ti.m_faces;
  info[n++] = ti.m_bytes_per_block;
  info[n++] = ti.m_userdata0;
  info[n++] = ti.m_userdata1;
  info[n++] = (uint32_t)ti.m_format;
  for (uint32_t l = 0; l < ti.m_levels; l++) {
    crnd::crn_level_info li;
    info[n++] = crnd::crnd_get_level_info(crn, crn_size, l, &li) ? 1u : 0u;
    info[n++] = li.m_width;
    info[n++] = li.m_height;
    info[n++] = li.m_faces;
    info[n++] = li.m_blocks_x;
    info[n++] = li.m_blocks_y;
    info[n++] = li.m_bytes_per_block;
    info[n++] = (uint32_t)li.m_format;
    crn_uint32 sz = 0;
    const void* p = crnd::crnd_get_level_data(crn, crn_size, l, &sz);
    info[n++] = p ? (uint32_t)(static_cast<const uint8_t*>(p) - crn) : 0xFFFFFFFFu;
    info[n++] = sz;
  }
  const uint32_t base = crnd::crnd_get_segmented_file_size(crn, crn_size);
  info[n++] = base;
  info[n++] = (base <= seg_cap && crnd::crnd_create_segmented_file(crn, crn_size, seg, seg_cap)) ? 1u : 0u;
  return n;
}

}  // extern "C"

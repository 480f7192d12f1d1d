// crnlib's public C++ API (inc/crnlib.h, inc/crn_defs.h) with the reference's own signatures,
// over this library's C ABI, so that a program built against the reference's headers links
// against libcrngpu.so unchanged. Every compress and transcode call runs on the GPU; what runs on
// the host here is argument checking, the DDS header and the copies between the caller's
// buffers and the returned blocks.
//
// Entry points and the reference behaviour each one keeps (reference file:line):
//   crn_compress                 crnlib/crnlib.cpp:215-240 -> create_compressed_texture,
//                                crnlib/crn_texture_comp.cpp:48-245 (CRN: crn_comp, DDS: dds_comp)
//   crn_compress (mip params)    crnlib/crnlib.cpp:242-267, crnlib/crn_texture_comp.cpp:348-578
//   crn_decompress_crn_to_dds    crnlib/crnlib.cpp:269-292 (read_crn_from_memory + write_dds,
//                                crnlib/crn_mipmapped_texture.cpp:921-1130)
//   block compressor             crnlib/crnlib.cpp:351-418
//   format helpers, strings      crnlib/crnlib.cpp:70-198, inc/crn_decomp.h:2567-2654
//   crnd_* (transcoder API)      inc/crn_decomp.h:2657-2880, 4404-4487
//   emscripten C exports         emscripten/crunch_lib.cpp:32-120
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/crnlib_compat.h"
#include "crn_file.h"
#include "host_alloc.h"
#include "crngpu_internal.h"

namespace {

using crngpu::set_error;

// ---------------------------------------------------------------------------------------------
// Memory hooks for returned blocks (crn_set_memory_callbacks, inc/crnlib.h:584-586).

struct Hooks {
  crn_realloc_func realloc_fn = nullptr;
  crn_msize_func msize_fn = nullptr;
  void* user = nullptr;
};
std::mutex g_hooks_mu;
Hooks g_hooks;

Hooks hooks() {
  std::lock_guard<std::mutex> lock(g_hooks_mu);
  return g_hooks;
}

void* block_alloc(size_t n) {
  const Hooks h = hooks();
  if (h.realloc_fn) {
    size_t actual = 0;
    return h.realloc_fn(nullptr, n ? n : 1, &actual, true, h.user);
  }
  return std::malloc(n ? n : 1);
}

void block_free(void* p) {
  if (!p) return;
  const Hooks h = hooks();
  if (h.realloc_fn) h.realloc_fn(p, 0, nullptr, true, h.user);
  else std::free(p);
}

void* to_block(const std::vector<uint8_t>& v, crn_uint32& size) {
  void* p = block_alloc(v.size());
  if (!p) {
    size = 0;
    return nullptr;
  }
  if (!v.empty()) std::memcpy(p, v.data(), v.size());
  size = (crn_uint32)v.size();
  return p;
}

// ---------------------------------------------------------------------------------------------
// Formats

uint32_t fourcc(char a, char b, char c, char d) {
  return (uint32_t)(uint8_t)a | ((uint32_t)(uint8_t)b << 8) | ((uint32_t)(uint8_t)c << 16) |
         ((uint32_t)(uint8_t)d << 24);
}

uint32_t format_fourcc(crn_format fmt) {
  switch (fmt) {
    case cCRNFmtDXT1: return fourcc('D', 'X', 'T', '1');
    case cCRNFmtDXT3: return fourcc('D', 'X', 'T', '3');
    case cCRNFmtDXT5: return fourcc('D', 'X', 'T', '5');
    case cCRNFmtDXN_XY: return fourcc('A', '2', 'X', 'Y');
    case cCRNFmtDXN_YX: return fourcc('A', 'T', 'I', '2');
    case cCRNFmtDXT5A: return fourcc('A', 'T', 'I', '1');
    case cCRNFmtDXT5_CCxY: return fourcc('C', 'C', 'x', 'Y');
    case cCRNFmtDXT5_xGxR: return fourcc('x', 'G', 'x', 'R');
    case cCRNFmtDXT5_xGBR: return fourcc('x', 'G', 'B', 'R');
    case cCRNFmtDXT5_AGBR: return fourcc('A', 'G', 'B', 'R');
    case cCRNFmtETC1: return fourcc('E', 'T', 'C', '1');
    case cCRNFmtETC2: return fourcc('E', 'T', 'C', '2');
    case cCRNFmtETC2A: return fourcc('E', 'T', '2', 'A');
    case cCRNFmtETC1S: return fourcc('E', 'T', '1', 'S');
    case cCRNFmtETC2AS: return fourcc('E', '2', 'A', 'S');
    default: return 0;
  }
}

uint32_t format_bits_per_texel(crn_format fmt) {
  switch (fmt) {
    case cCRNFmtDXT1: case cCRNFmtDXT5A: case cCRNFmtETC1: case cCRNFmtETC2: case cCRNFmtETC1S: return 4;
    case cCRNFmtDXT3: case cCRNFmtDXT5: case cCRNFmtDXN_XY: case cCRNFmtDXN_YX: case cCRNFmtDXT5_CCxY:
    case cCRNFmtDXT5_xGxR: case cCRNFmtDXT5_xGBR: case cCRNFmtDXT5_AGBR: case cCRNFmtETC2A: case cCRNFmtETC2AS:
      return 8;
    default: return 0;
  }
}

// Formats this library encodes and transcodes (ETC and DXT3 are not built).
bool format_supported(crn_format fmt) {
  switch (fmt) {
    case cCRNFmtDXT1: case cCRNFmtDXT5: case cCRNFmtDXT5_CCxY: case cCRNFmtDXT5_xGxR: case cCRNFmtDXT5_xGBR:
    case cCRNFmtDXT5_AGBR: case cCRNFmtDXN_XY: case cCRNFmtDXN_YX: case cCRNFmtDXT5A:
      return true;
    default: return false;
  }
}

// The 128-byte DDS header mipmapped_texture::write_dds writes for a compressed texture
// (crnlib/crn_mipmapped_texture.cpp:929-1027; field layout of DDSURFACEDESC2, inc/dds_defs.h).
// The DDS pixel format of a crn format follows read_crn_from_memory's mapping: DXN_XY is stored
// as ATI2 tagged 'A2XY' in the RGB bit count, the swizzled DXT5 formats as DXT5 tagged with
// their own code there.
void dds_header(uint8_t* h, uint32_t width, uint32_t height, uint32_t levels, uint32_t faces, crn_format fmt) {
  std::memset(h, 0, 128);
  auto put = [&](uint32_t ofs, uint32_t v) { std::memcpy(h + ofs, &v, 4); };
  constexpr uint32_t kCaps = 0x1, kHeight = 0x2, kWidth = 0x4, kPixelFormat = 0x1000, kMipCount = 0x20000,
                     kLinearSize = 0x80000;
  constexpr uint32_t kFourCC = 0x4, kComplex = 0x8, kTexture = 0x1000, kMipmap = 0x400000;
  constexpr uint32_t kCubeAllFaces = 0x200 | 0x400 | 0x800 | 0x1000 | 0x2000 | 0x4000 | 0x8000;
  std::memcpy(h, "DDS ", 4);
  uint32_t flags = kWidth | kHeight | kPixelFormat | kCaps | kLinearSize;
  uint32_t caps = kTexture, caps2 = 0;
  if (levels > 1) {
    flags |= kMipCount;
    caps |= kMipmap | kComplex;
    put(4 + 24, levels);  // dwMipMapCount
  }
  if (faces > 1) {
    caps |= kComplex;
    caps2 |= kCubeAllFaces;
  }
  uint32_t code = format_fourcc(fmt), bitcount = 0;
  switch (fmt) {
    case cCRNFmtDXN_XY: code = fourcc('A', 'T', 'I', '2'); bitcount = fourcc('A', '2', 'X', 'Y'); break;
    case cCRNFmtDXT5_CCxY: case cCRNFmtDXT5_xGxR: case cCRNFmtDXT5_xGBR: case cCRNFmtDXT5_AGBR:
      bitcount = code;
      code = fourcc('D', 'X', 'T', '5');
      break;
    default: break;
  }
  const uint32_t bpp = format_bits_per_texel(fmt);
  put(4 + 0, 124);                                              // dwSize
  put(4 + 4, flags);                                            // dwFlags
  put(4 + 8, height);                                           // dwHeight
  put(4 + 12, width);                                           // dwWidth
  put(4 + 16, (((width + 3) & ~3u) * ((height + 3) & ~3u) * bpp) >> 3);  // linear size
  put(4 + 72, 32);                                              // ddpfPixelFormat.dwSize
  put(4 + 76, kFourCC);                                         // ddpfPixelFormat.dwFlags
  put(4 + 80, code);                                            // ddpfPixelFormat.dwFourCC
  put(4 + 84, bitcount);                                        // ddpfPixelFormat.dwRGBBitCount
  put(4 + 104, caps);                                           // ddsCaps.dwCaps
  put(4 + 108, caps2);                                          // ddsCaps.dwCaps2
}

// ---------------------------------------------------------------------------------------------
// Compression

uint32_t max_mips(uint32_t w, uint32_t h) {
  uint32_t n = 1;
  while (w > 1 || h > 1) {
    w >>= 1;
    h >>= 1;
    n++;
  }
  return n;
}

bool progress(const crn_comp_params& p, crn_uint32 phase, crn_uint32 phases) {
  return !p.m_pProgress_func || p.m_pProgress_func(phase, phases, 0, 1, p.m_pProgress_func_data) != 0;
}

// The images of m_pImages[face][level] packed face-major, level after level.
bool gather_images(const crn_comp_params& p, std::vector<uint8_t>& out) {
  size_t total = 0;
  for (crn_uint32 l = 0; l < p.m_levels; l++)
    total += (size_t)std::max(1u, p.m_width >> l) * std::max(1u, p.m_height >> l) * 4 * p.m_faces;
  out.resize(total);
  uint8_t* o = out.data();
  for (crn_uint32 f = 0; f < p.m_faces; f++)
    for (crn_uint32 l = 0; l < p.m_levels; l++) {
      if (!p.m_pImages[f][l]) {
        set_error("crn_compress: m_pImages[" + std::to_string(f) + "][" + std::to_string(l) + "] is NULL");
        return false;
      }
      const size_t n = (size_t)std::max(1u, p.m_width >> l) * std::max(1u, p.m_height >> l) * 4;
      std::memcpy(o, p.m_pImages[f][l], n);
      o += n;
    }
  return true;
}

void* compress(const crn_comp_params& p, crn_uint32& compressed_size, crn_uint32* pActual_quality_level,
               float* pActual_bitrate) {
  compressed_size = 0;
  if (pActual_quality_level) *pActual_quality_level = 0;
  if (pActual_bitrate) *pActual_bitrate = 0.0f;
  crngpu::clear_error();
  if (!p.check()) {
    set_error("crn_compress: parameters out of range (crn_comp_params::check)");
    return nullptr;
  }
  if (!format_supported(p.m_format)) {
    set_error("crn_compress: ETC and DXT3 output are not built");
    return nullptr;
  }
  std::vector<uint8_t> images;
  if (!gather_images(p, images)) return nullptr;
  const uint32_t fmt = (uint32_t)p.m_format;
  // crn_comp reads only the perceptual and block-type flags (.crn files never hold 3-colour
  // blocks); dds_comp's plain encoder also honours DXT1A, grayscale sampling and transparent
  // indices for black, with m_dxt_quality and m_dxt1a_alpha_threshold (dxt_image::pack_params::init,
  // crnlib/crn_dxt_image.h:197-207)
  const uint32_t crn_flags = p.m_flags & (CRNGPU_FLAG_PERCEPTUAL | CRNGPU_FLAG_USE_BOTH_BLOCK_TYPES);
  const uint32_t dds_flags =
      p.m_flags & (CRNGPU_FLAG_PERCEPTUAL | CRNGPU_FLAG_USE_BOTH_BLOCK_TYPES | CRNGPU_FLAG_TRANSPARENT_BLACK |
                   CRNGPU_FLAG_DXT1A | CRNGPU_FLAG_GRAYSCALE);
  const uint32_t flags = crn_flags;
  if (!progress(p, 0, 2)) {
    set_error("crn_compress: cancelled by the progress callback");
    return nullptr;
  }
  std::vector<uint8_t> file;
  float bitrate = 0.0f;
  uint32_t quality = 0;
  if (p.m_file_type == cCRNFileTypeCRN) {
    crngpu_crn_options o;
    o.struct_size = sizeof(o);
    o.colour_psnr_derating = p.m_crn_adaptive_tile_color_psnr_derating;
    o.alpha_psnr_derating = p.m_crn_adaptive_tile_alpha_psnr_derating;
    o.alpha_component = p.m_alpha_component;
    const bool manual = (p.m_flags & cCRNCompFlagManualPaletteSizes) != 0;
    o.palette_sizes[0] = manual ? std::max(p.m_crn_color_endpoint_palette_size, 8u) : 0u;
    o.palette_sizes[1] = manual ? std::max(p.m_crn_color_selector_palette_size, 8u) : 0u;
    o.palette_sizes[2] = manual ? std::max(p.m_crn_alpha_endpoint_palette_size, 8u) : 0u;
    o.palette_sizes[3] = manual ? std::max(p.m_crn_alpha_selector_palette_size, 8u) : 0u;
    uint64_t blocks = 0;
    for (crn_uint32 l = 0; l < p.m_levels; l++)
      blocks += (uint64_t)((std::max(1u, p.m_width >> l) + 7) / 4) * ((std::max(1u, p.m_height >> l) + 7) / 4);
    file.resize((size_t)(blocks * p.m_faces * 16 + (1u << 20)));
    int64_t n = 0;
    for (int attempt = 0; attempt < 2; attempt++) {
      n = crngpu_compress_crn_ex(images.data(), p.m_width, p.m_height, p.m_levels, p.m_faces, fmt,
                                 p.m_quality_level, p.m_target_bitrate, flags, &o, file.data(), file.size(), &quality,
                                 &bitrate);
      if (n < 0 || (uint64_t)n <= file.size()) break;
      file.resize((size_t)n);
    }
    if (n < 0) return nullptr;
    file.resize((size_t)n);
  } else {
    if (p.m_target_bitrate > 0.0f) {
      set_error("crn_compress: a target bitrate for DDS output needs crnlib's LZMA estimate, which is not built");
      return nullptr;
    }
    const uint32_t bpb = format_bits_per_texel(p.m_format) * 2;
    uint64_t data = 0;
    for (crn_uint32 l = 0; l < p.m_levels; l++)
      data += (uint64_t)((std::max(1u, p.m_width >> l) + 3) / 4) * ((std::max(1u, p.m_height >> l) + 3) / 4) * bpb;
    data *= p.m_faces;
    file.resize((size_t)(128 + data));
    crngpu_block_options bo;
    bo.struct_size = sizeof(bo);
    bo.dxt_quality = (uint32_t)p.m_dxt_quality;
    bo.dxt1a_alpha_threshold = p.m_dxt1a_alpha_threshold;
    const int64_t n = crngpu_compress_dds_clustered_ex(images.data(), p.m_width, p.m_height, p.m_levels, p.m_faces,
                                                       fmt, p.m_quality_level, dds_flags, &bo, file.data() + 128, data);
    if (n < 0) return nullptr;
    dds_header(file.data(), p.m_width, p.m_height, p.m_levels, p.m_faces, p.m_format);
    quality = p.m_quality_level;
  }
  if (!progress(p, 1, 2)) {
    set_error("crn_compress: cancelled by the progress callback");
    return nullptr;
  }
  if (pActual_quality_level) *pActual_quality_level = quality;
  if (pActual_bitrate) *pActual_bitrate = bitrate;
  return to_block(file, compressed_size);
}

// Mip handling of create_texture_mipmaps (crnlib/crn_texture_comp.cpp:348-578) and
// mipmapped_texture::generate_mipmaps (crnlib/crn_mipmapped_texture.cpp:2140-2215): source mips,
// none, or a chain resampled from level 0 on the GPU. The level count stops where both sides
// reach m_min_mip_size and is capped at m_max_levels; alpha is filtered only if some source
// texel has alpha below 255 (create_dds_tex's has_alpha scan).
void* compress_with_mips(const crn_comp_params& cp, const crn_mipmap_params& mp, crn_uint32& compressed_size,
                         crn_uint32* pActual_quality_level, float* pActual_bitrate) {
  compressed_size = 0;
  if (pActual_quality_level) *pActual_quality_level = 0;
  if (pActual_bitrate) *pActual_bitrate = 0.0f;
  crngpu::clear_error();
  if (!cp.check() || !mp.check()) {
    set_error("crn_compress: parameters out of range");
    return nullptr;
  }
  const bool window = mp.m_window_right > mp.m_window_left && mp.m_window_bottom > mp.m_window_top;
  if (mp.m_scale_mode != cCRNSMDisabled || window || (mp.m_clamp_width && mp.m_clamp_height) || mp.m_renormalize ||
      mp.m_rtopmip) {
    set_error("crn_compress: rescaling, cropping, clamping and renormalisation of the source are not built");
    return nullptr;
  }
  if (mp.m_gamma_filtering && mp.m_gamma != 2.2f) {
    set_error("crn_compress: mip filtering in linear light is built for gamma 2.2 only");
    return nullptr;
  }
  if ((uint32_t)mp.m_filter > (uint32_t)cCRNMipFilterKaiser || (uint32_t)mp.m_mode >= (uint32_t)cCRNMipModeTotal) {
    set_error("crn_compress: bad mip filter or mode");
    return nullptr;
  }
  bool generate = mp.m_mode == cCRNMipModeGenerateMips ||
                  (mp.m_mode == cCRNMipModeUseSourceOrGenerateMips && cp.m_levels == 1);
  crn_comp_params np(cp);
  if (mp.m_mode == cCRNMipModeNoMips) np.m_levels = 1;
  if (!generate) return compress(np, compressed_size, pActual_quality_level, pActual_bitrate);

  uint32_t levels = 1;
  for (uint32_t w = cp.m_width, h = cp.m_height; w > mp.m_min_mip_size || h > mp.m_min_mip_size; w >>= 1, h >>= 1)
    levels++;
  if (mp.m_max_levels > 0 && levels > mp.m_max_levels) levels = mp.m_max_levels;
  levels = std::min(levels, max_mips(cp.m_width, cp.m_height));  // a minimum size of 0 stops at 1x1
  bool has_alpha = false;
  for (crn_uint32 f = 0; f < cp.m_faces && !has_alpha; f++)
    for (crn_uint32 l = 0; l < cp.m_levels && !has_alpha; l++) {
      const crn_uint32* img = cp.m_pImages[f][l];
      if (!img) {
        set_error("crn_compress: m_pImages is missing an image");
        return nullptr;
      }
      const size_t n = (size_t)std::max(1u, cp.m_width >> l) * std::max(1u, cp.m_height >> l);
      for (size_t i = 0; i < n && !has_alpha; i++) has_alpha = (img[i] >> 24) != 255u;
    }
  uint64_t chain = 0;
  for (uint32_t l = 0; l < levels; l++)
    chain += (uint64_t)std::max(1u, cp.m_width >> l) * std::max(1u, cp.m_height >> l) * 4;
  std::vector<uint8_t> mips((size_t)(chain * cp.m_faces));
  const uint32_t mflags = (mp.m_gamma_filtering ? CRNGPU_MIP_SRGB : 0u) | (mp.m_tiled ? CRNGPU_MIP_WRAP : 0u) |
                          (has_alpha ? CRNGPU_MIP_ALPHA : 0u);
  for (crn_uint32 f = 0; f < cp.m_faces; f++) {
    const int64_t n = crngpu_generate_mipmaps(reinterpret_cast<const uint8_t*>(cp.m_pImages[f][0]), cp.m_width,
                                              cp.m_height, levels, (uint32_t)mp.m_filter, mp.m_blurriness, mflags,
                                              mips.data() + chain * f, chain, CRNGPU_MEM_HOST, nullptr);
    if (n < 0) return nullptr;
  }
  np.m_levels = levels;
  std::memset(np.m_pImages, 0, sizeof(np.m_pImages));
  for (crn_uint32 f = 0; f < cp.m_faces; f++) {
    uint64_t ofs = chain * f;
    for (uint32_t l = 0; l < levels; l++) {
      np.m_pImages[f][l] = reinterpret_cast<const crn_uint32*>(mips.data() + ofs);
      ofs += (uint64_t)std::max(1u, cp.m_width >> l) * std::max(1u, cp.m_height >> l) * 4;
    }
  }
  return compress(np, compressed_size, pActual_quality_level, pActual_bitrate);
}

// ---------------------------------------------------------------------------------------------
// Transcoder contexts

struct CrndContext : crngpu::HostObject {
  uint32_t magic;
  crngpu_unpack_context ctx;
  const void* data;
  uint32_t size;
};
constexpr uint32_t kCrndMagic = 0x43524E44u;  // "CRND"

CrndContext* crnd_ctx(void* p) {
  CrndContext* c = static_cast<CrndContext*>(p);
  return (c && c->magic == kCrndMagic && c->ctx) ? c : nullptr;
}

// Host or device memory: the transcoder writes device buffers directly.
int memory_kind(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return CRNGPU_MEM_HOST;
  }
  return (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) ? CRNGPU_MEM_DEVICE : CRNGPU_MEM_HOST;
}

// Header fields (inc/crn_defs.h:299-330): big-endian packed integers.
uint32_t be(const uint8_t* p, int n) {
  uint32_t v = 0;
  for (int i = 0; i < n; i++) v = (v << 8) | p[i];
  return v;
}
void put_be(uint8_t* p, int n, uint32_t v) {
  for (int i = n - 1; i >= 0; i--, v >>= 8) p[i] = (uint8_t)v;
}

constexpr uint32_t kHeaderMin = 62;     // cCRNHeaderMinSize
constexpr uint32_t kHeaderStruct = 74;  // sizeof(crn_header) with one level offset

// crnd_get_header (inc/crn_decomp.h:2657-2670)
const uint8_t* crn_header_of(const void* data, uint32_t size) {
  const uint8_t* d = static_cast<const uint8_t*>(data);
  if (!d || size < kHeaderStruct) return nullptr;
  if (be(d, 2) != (('H' << 8) | 'x')) return nullptr;
  if (be(d + 2, 2) < kHeaderStruct || size < be(d + 6, 4)) return nullptr;
  return d;
}

}  // namespace

// =============================================================================================
// inc/crnlib.h

void crn_set_memory_callbacks(crn_realloc_func pRealloc, crn_msize_func pMSize, void* pUser_data) {
  std::lock_guard<std::mutex> lock(g_hooks_mu);
  if (!pRealloc || !pMSize) g_hooks = Hooks();
  else g_hooks = Hooks{pRealloc, pMSize, pUser_data};
}

void crn_free_block(void* pBlock) { block_free(pBlock); }

// No exception leaves these (the reference reports failure as NULL with a zero size): an
// allocation that fails, or that installed memory hooks refuse, ends the call that way.
void* crn_compress(const crn_comp_params& comp_params, crn_uint32& compressed_size, crn_uint32* pActual_quality_level,
                   float* pActual_bitrate) try {
  return compress(comp_params, compressed_size, pActual_quality_level, pActual_bitrate);
} catch (...) {
  crngpu::exception_status();
  compressed_size = 0;
  return nullptr;
}

void* crn_compress(const crn_comp_params& comp_params, const crn_mipmap_params& mip_params, crn_uint32& compressed_size,
                   crn_uint32* pActual_quality_level, float* pActual_bitrate) try {
  return compress_with_mips(comp_params, mip_params, compressed_size, pActual_quality_level, pActual_bitrate);
} catch (...) {
  crngpu::exception_status();
  compressed_size = 0;
  return nullptr;
}

namespace {
void* dds_of_context(crngpu_unpack_context ctx, crn_uint32& file_size);
}  // namespace

void* crn_decompress_crn_to_dds(const void* pCRN_file_data, crn_uint32& file_size) {
  const uint32_t crn_size = file_size;
  file_size = 0;
  crngpu_unpack_context ctx = crngpu_unpack_begin(pCRN_file_data, crn_size);
  if (!ctx) return nullptr;
  struct End {
    crngpu_unpack_context c;
    ~End() { crngpu_unpack_end(c); }
  } end{ctx};
  try {
    return dds_of_context(ctx, file_size);
  } catch (...) {
    crngpu::exception_status();
    file_size = 0;
    return nullptr;
  }
}

namespace {
// the DDS file of every level of an unpack context
void* dds_of_context(crngpu_unpack_context ctx, crn_uint32& file_size) {
  uint32_t w = 0, h = 0, levels = 0, faces = 0, fmt = 0, bpb = 0;
  crngpu_get_info(ctx, &w, &h, &levels, &faces, &fmt, &bpb);
  uint64_t data = 0;
  for (uint32_t l = 0; l < levels; l++)
    data += (uint64_t)((std::max(1u, w >> l) + 3) / 4) * ((std::max(1u, h >> l) + 3) / 4) * bpb * faces;
  std::vector<uint8_t> out((size_t)(128 + data));
  // transcode every level at minimal pitch (level-major, face after face), then lay the result
  // out face-major as DDS stores it
  std::vector<uint8_t> lv((size_t)data);
  const int64_t n = crngpu_unpack_levels(ctx, 0, levels, lv.data(), data, CRNGPU_MEM_HOST, nullptr);
  if (n < 0) return nullptr;
  uint8_t* o = out.data() + 128;
  for (uint32_t f = 0; f < faces; f++) {
    uint64_t ofs = 0;
    for (uint32_t l = 0; l < levels; l++) {
      const uint64_t face_bytes = (uint64_t)((std::max(1u, w >> l) + 3) / 4) * ((std::max(1u, h >> l) + 3) / 4) * bpb;
      std::memcpy(o, lv.data() + ofs + face_bytes * f, (size_t)face_bytes);
      o += face_bytes;
      ofs += face_bytes * faces;
    }
  }
  dds_header(out.data(), w, h, levels, faces, static_cast<crn_format>(fmt));
  return to_block(out, file_size);
}
}  // namespace

crn_uint32 crn_get_format_fourcc(crn_format fmt) { return format_fourcc(fmt); }
crn_uint32 crn_get_format_bits_per_texel(crn_format fmt) { return format_bits_per_texel(fmt); }
crn_uint32 crn_get_bytes_per_dxt_block(crn_format fmt) { return (format_bits_per_texel(fmt) << 4) >> 3; }
crn_format crn_get_fundamental_dxt_format(crn_format fmt) { return crnd::crnd_get_fundamental_dxt_format(fmt); }

const char* crn_get_file_type_ext(crn_file_type file_type) {
  return file_type == cCRNFileTypeDDS ? "dds" : (file_type == cCRNFileTypeCRN ? "crn" : "?");
}

const char* crn_get_format_string(crn_format fmt) {
  static const char* const kNames[] = {"DXT1",   "DXT3",   "DXT5", "DXT5_CCxY", "DXT5_xGxR",
                                       "DXT5_xGBR", "DXT5_AGBR", "DXN_XY", "DXN_YX", "DXT5A",
                                       "ETC1",   "ETC2",   "ETC2A", "ETC1S",    "ETC2AS"};
  const long f = (long)fmt;
  return (f >= 0 && f < (long)cCRNFmtTotal) ? kNames[f] : "?";
}

const char* crn_get_dxt_quality_string(crn_dxt_quality q) {
  static const char* const kNames[] = {"SuperFast", "Fast", "Normal", "Better", "Uber"};
  return (uint32_t)q < (uint32_t)cCRNDXTQualityTotal ? kNames[q] : "?";
}

const char* crn_get_mip_mode_desc(crn_mip_mode m) {
  static const char* const kDesc[] = {"Use source/generate if none", "Only use source MIP maps (if any)",
                                      "Always generate new MIP maps", "No MIP maps"};
  return (uint32_t)m < (uint32_t)cCRNMipModeTotal ? kDesc[m] : "?";
}

const char* crn_get_mip_mode_name(crn_mip_mode m) {
  static const char* const kNames[] = {"UseSourceOrGenerate", "UseSource", "Generate", "None"};
  return (uint32_t)m < (uint32_t)cCRNMipModeTotal ? kNames[m] : "?";
}

const char* crn_get_mip_filter_name(crn_mip_filter f) {
  static const char* const kNames[] = {"box", "tent", "lanczos4", "mitchell", "kaiser"};
  return (uint32_t)f < (uint32_t)cCRNMipFilterTotal ? kNames[f] : "?";
}

const char* crn_get_scale_mode_desc(crn_scale_mode sm) {
  static const char* const kNames[] = {"disabled", "absolute", "relative", "lowerpow2", "nearestpow2", "nextpow2"};
  return (uint32_t)sm < (uint32_t)cCRNSMTotal ? kNames[sm] : "?";
}

// The block compressor: one context per caller thread in the reference; here a context holds the
// format, flags, dxt quality and DXT1A threshold, and each call encodes its block on the GPU (no
// endpoint cache, so the output does not depend on the blocks compressed before). Each call is one
// launch and one synchronisation: callers with many blocks should use crngpu_compress_blocks_ex.
namespace {
struct BlockCompressor {
  uint32_t magic;
  uint32_t format, flags;
  crngpu_block_options options;
};
constexpr uint32_t kBlockMagic = 0x424C4B43u;  // "BLKC"
}  // namespace

crn_block_compressor_context_t crn_create_block_compressor(const crn_comp_params& params) {
  crngpu::clear_error();
  const crn_format fund = crnd::crnd_get_fundamental_dxt_format(params.m_format);
  if (!format_supported(params.m_format) || (uint32_t)params.m_dxt_quality > (uint32_t)cCRNDXTQualityUber ||
      params.m_dxt1a_alpha_threshold > 255) {
    set_error("crn_create_block_compressor: format not built or parameters out of range");
    return nullptr;
  }
  BlockCompressor* c = new (std::nothrow) BlockCompressor;
  if (!c) return nullptr;
  c->magic = kBlockMagic;
  // dxt_image::pack_params::init (crnlib/crn_dxt_image.h:197-207) takes the perceptual,
  // both-block-types, transparent-black and grayscale flags, the dxt quality and the DXT1A
  // threshold; crn_block_compressor::init encodes DXT1 as DXT1A when the DXT1A flag is set; the
  // swizzled DXT5 formats encode as plain DXT5 blocks (crnlib/crnlib.cpp:358-381)
  c->format = (uint32_t)fund;
  c->flags = params.m_flags & (CRNGPU_FLAG_PERCEPTUAL | CRNGPU_FLAG_USE_BOTH_BLOCK_TYPES |
                               CRNGPU_FLAG_TRANSPARENT_BLACK | CRNGPU_FLAG_GRAYSCALE);
  if ((params.m_flags & cCRNCompFlagDXT1AForTransparency) && fund == cCRNFmtDXT1) c->flags |= CRNGPU_FLAG_DXT1A;
  c->options.struct_size = sizeof(crngpu_block_options);
  c->options.dxt_quality = (uint32_t)params.m_dxt_quality;
  c->options.dxt1a_alpha_threshold = params.m_dxt1a_alpha_threshold;
  return c;
}

void crn_compress_block(crn_block_compressor_context_t pContext, const crn_uint32* pPixels, void* pDst_block) {
  BlockCompressor* c = static_cast<BlockCompressor*>(pContext);
  if (!c || c->magic != kBlockMagic || !pPixels || !pDst_block) return;
  crngpu_compress_blocks_ex(reinterpret_cast<const uint8_t*>(pPixels), 1, c->format, c->flags, &c->options,
                            static_cast<uint8_t*>(pDst_block), CRNGPU_MEM_HOST, nullptr);
}

void crn_free_block_compressor(crn_block_compressor_context_t pContext) {
  BlockCompressor* c = static_cast<BlockCompressor*>(pContext);
  if (!c || c->magic != kBlockMagic) return;
  c->magic = 0;
  delete c;
}

const char* crn_get_version() { return "1.04 (crngpu, sm_103a)"; }
int crn_get_version_number() { return 104; }
int crn_get_version_major() { return 1; }
int crn_get_version_minor() { return 4; }
int crn_get_version_patch() { return 0; }

// =============================================================================================
// inc/crn_defs.h (namespace crnd)

namespace crnd {

// The transcoder's host state (contexts, parsed files, palettes, launch plans, batches) is
// allocated through these hooks from then on, as crnd's is (inc/crn_decomp.h:2440-2459). Device
// memory is the CUDA runtime's; the reference has none.
void crnd_set_memory_callbacks(crnd_realloc_func pRealloc, crnd_msize_func pMSize, void* pUser_data) {
  crngpu::set_host_hooks(pRealloc, pMSize, pUser_data);
}

uint32 crnd_crn_format_to_fourcc(crn_format fmt) { return format_fourcc(fmt); }

crn_format crnd_get_fundamental_dxt_format(crn_format fmt) {
  switch (fmt) {
    case cCRNFmtDXT5_CCxY: case cCRNFmtDXT5_xGxR: case cCRNFmtDXT5_xGBR: case cCRNFmtDXT5_AGBR: return cCRNFmtDXT5;
    default: return fmt;
  }
}

uint32 crnd_get_crn_format_bits_per_texel(crn_format fmt) { return format_bits_per_texel(fmt); }
uint32 crnd_get_bytes_per_dxt_block(crn_format fmt) { return (format_bits_per_texel(fmt) << 4) >> 3; }

// crnd_validate_file (inc/crn_decomp.h:2672-2735): header and data CRC-16s, then the geometry.
bool crnd_validate_file(const void* pData, uint32 data_size, crn_file_info* pFile_info) {
  if (pFile_info) {
    if (pFile_info->m_struct_size != sizeof(crn_file_info)) return false;
    std::memset(&pFile_info->m_struct_size + 1, 0, sizeof(crn_file_info) - sizeof(pFile_info->m_struct_size));
  }
  if (!pData || data_size < kHeaderMin) return false;
  const uint8_t* d = crn_header_of(pData, data_size);
  if (!d) return false;
  const uint32_t header_size = be(d + 2, 2), file_size = be(d + 6, 4);
  if (crngpu::crc16(d + 6, header_size - 6) != be(d + 4, 2)) return false;
  if (file_size < header_size || crngpu::crc16(d + header_size, file_size - header_size) != be(d + 10, 2)) return false;
  const uint32_t w = be(d + 12, 2), h = be(d + 14, 2), levels = d[16], faces = d[17], fmt = d[18];
  if (faces != 1 && faces != 6) return false;
  if (w < 1 || w > cCRNMaxLevelResolution || h < 1 || h > cCRNMaxLevelResolution) return false;
  if (levels < 1 || levels > max_mips(w, h)) return false;
  if (fmt >= (uint32_t)cCRNFmtTotal) return false;
  if (pFile_info) {
    pFile_info->m_actual_data_size = file_size;
    pFile_info->m_header_size = header_size;
    uint32_t pal = 0;
    for (int k = 0; k < 4; k++) pal += be(d + 36 + 8 * k, 3);
    pFile_info->m_total_palette_size = pal;
    pFile_info->m_tables_size = be(d + 65, 2);
    pFile_info->m_levels = levels;
    for (uint32_t l = 0; l < levels && l < (uint32_t)cCRNMaxLevels; l++) {
      const uint32_t next = l + 1 < levels ? be(d + 70 + 4 * (l + 1), 4) : file_size;
      pFile_info->m_level_compressed_size[l] = next - be(d + 70 + 4 * l, 4);
    }
    pFile_info->m_color_endpoint_palette_entries = be(d + 39, 2);
    pFile_info->m_color_selector_palette_entries = be(d + 47, 2);
    pFile_info->m_alpha_endpoint_palette_entries = be(d + 55, 2);
    pFile_info->m_alpha_selector_palette_entries = be(d + 63, 2);
  }
  return true;
}

bool crnd_get_texture_info(const void* pData, uint32 data_size, crn_texture_info* pInfo) {
  if (!pData || data_size < kHeaderStruct || !pInfo || pInfo->m_struct_size != sizeof(crn_texture_info)) return false;
  const uint8_t* d = crn_header_of(pData, data_size);
  if (!d) return false;
  const uint32_t fmt = d[18];
  pInfo->m_width = be(d + 12, 2);
  pInfo->m_height = be(d + 14, 2);
  pInfo->m_levels = d[16];
  pInfo->m_faces = d[17];
  pInfo->m_format = static_cast<crn_format>(fmt);
  pInfo->m_bytes_per_block = (fmt == cCRNFmtDXT1 || fmt == cCRNFmtDXT5A || fmt == cCRNFmtETC1 || fmt == cCRNFmtETC2 ||
                              fmt == cCRNFmtETC1S) ? 8 : 16;
  pInfo->m_userdata0 = be(d + 25, 4);
  pInfo->m_userdata1 = be(d + 29, 4);
  return true;
}

bool crnd_get_level_info(const void* pData, uint32 data_size, uint32 level_index, crn_level_info* pLevel_info) {
  if (!pData || data_size < kHeaderMin || !pLevel_info || pLevel_info->m_struct_size != sizeof(crn_level_info))
    return false;
  const uint8_t* d = crn_header_of(pData, data_size);
  if (!d || level_index >= d[16]) return false;
  const uint32_t fmt = d[18];
  const uint32_t w = std::max(1u, be(d + 12, 2) >> level_index), h = std::max(1u, be(d + 14, 2) >> level_index);
  pLevel_info->m_width = w;
  pLevel_info->m_height = h;
  pLevel_info->m_faces = d[17];
  pLevel_info->m_blocks_x = (w + 3) >> 2;
  pLevel_info->m_blocks_y = (h + 3) >> 2;
  pLevel_info->m_bytes_per_block = (fmt == cCRNFmtDXT1 || fmt == cCRNFmtDXT5A) ? 8 : 16;
  pLevel_info->m_format = static_cast<crn_format>(fmt);
  return true;
}

crnd_unpack_context crnd_unpack_begin(const void* pData, uint32 data_size) {
  if (!pData || data_size < kHeaderMin) return nullptr;
  crngpu_unpack_context ctx = crngpu_unpack_begin(pData, data_size);
  if (!ctx) return nullptr;
  CrndContext* c = new (std::nothrow) CrndContext{{}, kCrndMagic, ctx, pData, data_size};
  if (!c) crngpu_unpack_end(ctx);
  return c;
}

bool crnd_get_data(crnd_unpack_context pContext, const void** ppData, uint32* pData_size) {
  CrndContext* c = crnd_ctx(pContext);
  if (!c) return false;
  if (ppData) *ppData = c->data;
  if (pData_size) *pData_size = c->size;
  return true;
}

bool crnd_unpack_level(crnd_unpack_context pContext, void** ppDst, uint32 dst_size_in_bytes, uint32 row_pitch_in_bytes,
                       uint32 level_index) {
  CrndContext* c = crnd_ctx(pContext);
  if (!c || !ppDst || !ppDst[0] || dst_size_in_bytes < 8 || level_index >= (uint32)cCRNMaxLevels) return false;
  const int mem = memory_kind(ppDst[0]);
  if (crngpu_unpack_level(c->ctx, ppDst, dst_size_in_bytes, row_pitch_in_bytes, level_index, mem, nullptr) != CRNGPU_OK)
    return false;
  return mem == CRNGPU_MEM_HOST || cudaStreamSynchronize(nullptr) == cudaSuccess;
}

bool crnd_unpack_level_segmented(crnd_unpack_context pContext, const void* pSrc, uint32 src_size_in_bytes, void** ppDst,
                                 uint32 dst_size_in_bytes, uint32 row_pitch_in_bytes, uint32 level_index) {
  CrndContext* c = crnd_ctx(pContext);
  if (!c || !pSrc || !ppDst || !ppDst[0] || dst_size_in_bytes < 8 || level_index >= (uint32)cCRNMaxLevels) return false;
  const int mem = memory_kind(ppDst[0]);
  if (memory_kind(pSrc) != mem) {
    set_error("crnd_unpack_level_segmented: the level data and the destination must both be host or both device memory");
    return false;
  }
  if (crngpu_unpack_level_segmented(c->ctx, pSrc, src_size_in_bytes, ppDst, dst_size_in_bytes, row_pitch_in_bytes,
                                    level_index, mem, nullptr) != CRNGPU_OK)
    return false;
  return mem == CRNGPU_MEM_HOST || cudaStreamSynchronize(nullptr) == cudaSuccess;
}

bool crnd_unpack_end(crnd_unpack_context pContext) {
  CrndContext* c = crnd_ctx(pContext);
  if (!c) return false;
  crngpu_unpack_end(c->ctx);
  c->magic = 0;
  delete c;
  return true;
}

const void* crnd_get_level_data(const void* pData, uint32 data_size, uint32 level_index, uint32* pSize) {
  if (pSize) *pSize = 0;
  if (!pData || data_size < kHeaderMin) return nullptr;
  const uint8_t* d = crn_header_of(pData, data_size);
  if (!d || level_index >= d[16]) return nullptr;
  const uint32_t ofs = be(d + 70 + 4 * level_index, 4);
  if (pSize) {
    const uint32_t next = level_index + 1 < d[16] ? be(d + 70 + 4 * (level_index + 1), 4) : data_size;
    *pSize = next - ofs;
  }
  return d + ofs;
}

// The header, palettes and tables without the level data (inc/crn_decomp.h:2819-2837).
uint32 crnd_get_segmented_file_size(const void* pData, uint32 data_size) {
  if (!pData || data_size < kHeaderMin) return 0;
  const uint8_t* d = crn_header_of(pData, data_size);
  if (!d) return 0;
  uint32_t size = be(d + 2, 2);
  for (int k = 0; k < 4; k++) size = std::max(size, be(d + 33 + 8 * k, 3) + be(d + 36 + 8 * k, 3));
  return std::max(size, be(d + 67, 3) + be(d + 65, 2));
}

// crnd_create_segmented_file (inc/crn_decomp.h:2839-2870): the base data with the segmented flag,
// its own data size and both CRCs recomputed.
bool crnd_create_segmented_file(const void* pData, uint32 data_size, void* pBase_data, uint base_data_size) {
  if (!pData || data_size < kHeaderMin || !pBase_data) return false;
  const uint8_t* d = crn_header_of(pData, data_size);
  if (!d || (be(d + 19, 2) & 1u)) return false;
  const uint32_t base = crnd_get_segmented_file_size(pData, data_size);
  if (!base || base_data_size < base || base > data_size) return false;
  uint8_t* b = static_cast<uint8_t*>(pBase_data);
  std::memmove(b, d, base);
  const uint32_t header_size = be(b + 2, 2);
  put_be(b + 19, 2, be(b + 19, 2) | 1u);
  put_be(b + 6, 4, base);
  put_be(b + 10, 2, crngpu::crc16(b + header_size, base - header_size));
  put_be(b + 4, 2, crngpu::crc16(b + 6, header_size - 6));
  return true;
}

}  // namespace crnd

// =============================================================================================
// emscripten/crunch_lib.cpp's C exports. Geometry comes from crnd_get_texture_info (zeros when
// the header is not a .crn); sizes use width >> level without the minimum of 1, as the wrapper
// does.

namespace {
crnd::crn_texture_info wrapper_info(void* src, unsigned int src_size) {
  crnd::crn_texture_info ti;
  if (!crnd::crnd_get_texture_info(src, src_size, &ti)) {
    ti.m_width = ti.m_height = ti.m_levels = ti.m_faces = ti.m_bytes_per_block = 0;
    ti.m_userdata0 = ti.m_userdata1 = 0;
    ti.m_format = static_cast<crn_format>(0);
  }
  return ti;
}
}  // namespace

extern "C" unsigned int crn_get_width(void* src, unsigned int src_size) { return wrapper_info(src, src_size).m_width; }
extern "C" unsigned int crn_get_height(void* src, unsigned int src_size) { return wrapper_info(src, src_size).m_height; }
extern "C" unsigned int crn_get_levels(void* src, unsigned int src_size) { return wrapper_info(src, src_size).m_levels; }
extern "C" unsigned int crn_get_dxt_format(void* src, unsigned int src_size) {
  return (unsigned int)wrapper_info(src, src_size).m_format;
}
extern "C" unsigned int crn_get_bytes_per_block(void* src, unsigned int src_size) {
  return crnd::crnd_get_bytes_per_dxt_block(wrapper_info(src, src_size).m_format);
}
extern "C" unsigned int crn_get_uncompressed_size(void* src, unsigned int src_size, unsigned int level) {
  const crnd::crn_texture_info ti = wrapper_info(src, src_size);
  const unsigned int w = level < 32 ? ti.m_width >> level : 0, h = level < 32 ? ti.m_height >> level : 0;
  return ((w + 3) >> 2) * ((h + 3) >> 2) * crnd::crnd_get_bytes_per_dxt_block(ti.m_format);
}
extern "C" void crn_decompress(void* src, unsigned int src_size, void* dst, unsigned int dst_size,
                               unsigned int firstLevel, unsigned int levelCount) {
  crngpu_crn_decompress(src, src_size, dst, dst_size, firstLevel, levelCount);
}

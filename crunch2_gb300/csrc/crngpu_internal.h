// Internal helpers shared by the crngpu translation units (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/crngpu.h"

namespace crngpu {

// The source "cooking" crn_comp and dds_comp apply before compressing to a swizzled DXT5 format
// (image_utils::get_image_conversion_type_from_crn_format, crnlib/crn_image_utils.cpp:1454-1470;
// the conversions :1267-1311). DXT5_CCxY stores luma in alpha and the JFIF chroma (biased by 123
// and 125, crnlib/crn_color.h:788-807) in red and green; xGxR / xGBR / AGBR move red to alpha.
// Texels are RGBA8 with red in the lowest byte. Other formats pass through.
inline uint32_t cook_texel(uint32_t format, uint32_t px) {
  const int r = (int)(px & 255u), g = (int)((px >> 8) & 255u), b = (int)((px >> 16) & 255u), a = (int)(px >> 24);
  auto pack = [](int c0, int c1, int c2, int c3) {
    return (uint32_t)c0 | ((uint32_t)c1 << 8) | ((uint32_t)c2 << 16) | ((uint32_t)c3 << 24);
  };
  auto clamp8 = [](int v) { return v < 0 ? 0 : (v > 255 ? 255 : v); };
  switch (format) {
    case CRNGPU_FMT_DXT5_CCXY: {
      const int y = (r * 19595 + g * 38470 + b * 7471 + 32768) >> 16;
      const int cb = clamp8(123 + ((r * -11059 + g * -21709 + b * 32768 + 32768) >> 16));
      const int cr = clamp8(125 + ((r * 32768 + g * -27439 + b * -5329 + 32768) >> 16));
      return pack(cb, cr, 0, y & 255);
    }
    case CRNGPU_FMT_DXT5_XGXR: return pack(0, g, 0, r);
    case CRNGPU_FMT_DXT5_XGBR: return pack(0, g, b, r);
    case CRNGPU_FMT_DXT5_AGBR: return pack(a, g, b, r);
    default: return px;
  }
}

// crn_compress turns the perceptual metric off for formats that are not sRGB colour
// (pixel_format_helpers::is_crn_format_non_srgb, crnlib/crn_pixel_format.h:258-273,
// crnlib/crn_texture_comp.cpp:52-61).
inline bool format_is_non_srgb(uint32_t format) {
  return format == CRNGPU_FMT_DXN_XY || format == CRNGPU_FMT_DXN_YX || format == CRNGPU_FMT_DXT5A ||
         format == CRNGPU_FMT_DXT5_CCXY || format == CRNGPU_FMT_DXT5_XGXR || format == CRNGPU_FMT_DXT5_XGBR ||
         format == CRNGPU_FMT_DXT5_AGBR;
}

// Thread-local last-error text behind crngpu_last_error().
void set_error(const std::string& msg);
void clear_error();
const char* last_error_cstr();

// Guards every lazily filled per-device cache of the library (function attributes, symbol
// addresses, uploaded tables, SM counts): first calls on one device from several host threads
// would otherwise race on them.
std::mutex& device_setup_mutex();

// Records `what` + the CUDA error string and returns CRNGPU_E_DEVICE when e != cudaSuccess.
int cuda_check(cudaError_t e, const char* what);

// A device buffer owned by the library; grows on demand, never shrinks.
struct DevBuf {
  void* ptr = nullptr;
  size_t cap = 0;
  int device = -1;
  cudaError_t ensure(size_t bytes);
  void release();
  ~DevBuf() { release(); }
};

// Per-thread scratch for host-memory calls (input/output staging), slots 0..7: 0-3 the encoders,
// 4-6 mip generation.
DevBuf& staging(int slot);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Batched block encoding (many textures, mixed formats). A segment is one element of one texture
// over its gathered blocks [first_block, first_block + count): the colour half of DXT1/DXT5, the
// alpha of DXT5/DXT5A or one DXN channel; block b's 8 bytes go to out + (b - first_block) * stride.
struct EncodeSegment {
  uint8_t* out;
  uint32_t first_block, count, stride, options;
};
constexpr uint32_t kSegPerceptual = 1u, kSegThreeColour = 2u, kSegBothTypes = 4u, kSegCompShift = 8u;
// a run of consecutive blocks of one segment, the unit a warp takes
struct EncodeChunk {
  uint32_t first, count, segment;
};
constexpr uint32_t kColourChunkBlocks = 8;  // blocks per DXT1 chunk (the encoder's blocks per warp)
int dxt1_chunks_max_grid();
int dxt5a_chunks_max_grid();
int launch_dxt1_chunks(const uint8_t* d_blocks, const EncodeChunk* d_chunks, uint32_t nchunks,
                       const EncodeSegment* d_segs, int grid, cudaStream_t s);
int launch_dxt5a_chunks(const uint8_t* d_blocks, const EncodeChunk* d_chunks, uint32_t nchunks,
                        const EncodeSegment* d_segs, int grid, cudaStream_t s);

}  // namespace crngpu

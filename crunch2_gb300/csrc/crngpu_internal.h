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
__host__ __device__ inline uint32_t cook_texel(uint32_t format, uint32_t px) {
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
// The status of the exception being handled, for the C-ABI entry points, which let none escape:
// CRNGPU_E_NOMEM for std::bad_alloc (host memory exhausted, or an allocation the installed memory
// hooks refused), CRNGPU_E_DEVICE for anything else; the last-error text says which.
int exception_status() noexcept;
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
// DXT1 encoder options (the options word of a launch, and of a colour segment): the parameters
// dxt_image::set_block_pixels gives dxt1_endpoint_optimizer (crnlib/crn_dxt_image.cpp:1436-1480)
constexpr uint32_t kD1Perceptual = 1u;      // m_perceptual (never set together with kD1Gray)
constexpr uint32_t kD1Three = 2u;           // m_use_alpha_blocks: 3-colour blocks allowed
constexpr uint32_t kD1Gray = 4u;            // m_grayscale_sampling: luma distance
constexpr uint32_t kD1Dxt1a = 8u;           // DXT1A: texels with alpha below the threshold are transparent
constexpr uint32_t kD1BlackTrial = 16u;     // the transparent-black trial of try_alpha_as_black_optimization
constexpr uint32_t kD1QualityShift = 8u;    // bits 8-10: crn_dxt_quality (0 superfast .. 4 uber)
constexpr uint32_t kD1ThresholdShift = 16u; // bits 16-23: m_dxt1a_alpha_threshold
// alpha segments: crn_dxt_quality in bits 12-14 (the probe grid of dxt5_endpoint_optimizer)
constexpr uint32_t kSegAlphaQualityShift = 12u;
constexpr uint32_t kDxtQualityUber = 4u, kDxtQualityBetter = 3u, kDxtQualityNormal = 2u;
inline uint32_t dxt1_options(bool perceptual, bool use_alpha_blocks, uint32_t quality, bool grayscale, bool dxt1a,
                             uint32_t alpha_threshold) {
  return (perceptual && !grayscale ? kD1Perceptual : 0u) | (use_alpha_blocks ? kD1Three : 0u) |
         (grayscale ? kD1Gray : 0u) | (dxt1a ? kD1Dxt1a : 0u) | ((quality & 7u) << kD1QualityShift) |
         ((alpha_threshold & 255u) << kD1ThresholdShift);
}
// a run of consecutive blocks of one segment, the unit a warp takes
struct EncodeChunk {
  uint32_t first, count, segment;
};
constexpr uint32_t kColourChunkBlocks = 8;  // blocks per DXT1 chunk (the encoder's blocks per warp)
int dxt1_chunks_max_grid();
int dxt5a_chunks_max_grid();
// DXT1 / DXT5A block encoders on device buffers (dxt_encode.cu). launch_dxt1: opts is a
// dxt1_options() word; d_err (optional) receives each block's error. launch_dxt1_black_trial: the
// transparent-black trial over blocks already encoded with the same options (d_err_io their
// errors): a block whose trial is better is rewritten in place, with its new error.
// launch_dxt5a: quality sets the probe grid (+-16 Uber, +-8 Better, none below).
int launch_dxt1(const uint8_t* d_blocks, uint32_t n, uint32_t opts, uint8_t* d_out, uint32_t out_stride,
                uint64_t* d_err, cudaStream_t s);
// One image of a host mip chain uploaded as a whole, gathered into 4x4 blocks of cooked texels
// (cook_texel) by launch_gather_chain: the image's blocks are [first, the next image's first),
// bx to a row, texels edge-clamped to w x h.
struct GatherImage {
  uint64_t src;      // byte offset of the image in the uploaded chain
  uint32_t w, h, bx;
  uint32_t first;    // first block of the image in the output
};
int launch_gather_chain(const uint8_t* d_chain, const GatherImage* d_imgs, uint32_t nimg, uint32_t blocks,
                        uint32_t format, uint32_t* d_out, cudaStream_t s);

// dds_comp at quality 255 for a whole texture (host RGBA8 levels, face after face, level after
// level, tightly packed): every block of every face and level through the plain encoder, output in
// DDS order at minimal pitch. Returns the output bytes (or the bytes needed when out is NULL or
// too small) or a CRNGPU_E_* code. `flags` / `quality` / `threshold` as encode_device takes them.
int64_t dds_plain_chain(const uint8_t* rgba_levels, uint32_t width, uint32_t height, uint32_t levels, uint32_t faces,
                        uint32_t format, uint32_t flags, uint32_t quality, uint32_t threshold, void* out,
                        uint64_t out_capacity);

// The same with the block count in device memory (*n_dev <= n_max), so that a caller need not
// read it back before the launch; the grids are sized for n_max.
int launch_dxt1_count(const uint8_t* d_blocks, uint32_t n_max, const uint32_t* n_dev, uint32_t opts, uint8_t* d_out,
                      uint32_t out_stride, cudaStream_t s);
int launch_dxt1_black_trial(const uint8_t* d_blocks, uint32_t n, uint32_t opts, uint8_t* d_out, uint32_t out_stride,
                            uint64_t* d_err_io, cudaStream_t s);
int launch_dxt5a(const uint8_t* d_blocks, uint32_t n, int comp, bool both, uint32_t quality, uint8_t* d_out,
                 uint32_t out_stride, cudaStream_t s);
// the batched colour encode: phase 1 writes one seed record of kDxt1SeedBytes per block to
// d_seeds (room for every gathered block of the batch), phase 2 reads them
constexpr size_t kDxt1SeedBytes = 64;
int launch_dxt1_chunks(const uint8_t* d_blocks, const EncodeChunk* d_chunks, uint32_t nchunks,
                       const EncodeSegment* d_segs, void* d_seeds, int grid, cudaStream_t s);
int launch_dxt5a_chunks(const uint8_t* d_blocks, const EncodeChunk* d_chunks, uint32_t nchunks,
                        const EncodeSegment* d_segs, int grid, cudaStream_t s);

}  // namespace crngpu

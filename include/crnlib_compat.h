/* crnlib-compatible C++ API of libcrngpu.so.
 *
 * libcrngpu.so exports, with C++ linkage and the reference's own signatures, the public functions
 * of crnlib's inc/crnlib.h (crn_compress, crn_decompress_crn_to_dds, the block compressor, the
 * format helpers, the memory hooks) and of inc/crn_defs.h (namespace crnd: crnd_unpack_begin /
 * _level / _level_segmented / _end, crnd_get_texture_info, crnd_validate_file and the rest). A
 * program written against the reference's headers links against libcrngpu.so instead of crnlib
 * without source changes; every call runs on the GPU.
 *
 * This header restates the types those functions take, for callers without the reference's
 * headers and for the library's own build: the names, enumerator values, member order and member
 * types are the reference's, because the link names (C++ mangling) and the struct layouts are the
 * binary interface. The member functions (defaults, validation) are this library's own.
 *
 * Not exported: crn_decompress_dds_to_images, crn_free_all_images and crn_decompress_block (DDS
 * reading and DXTn-to-RGBA decoding are outside this library's path).
 *
 * Behaviour that differs from crnlib (all reported by returning NULL / false):
 *   - ETC formats, DXT3 and cCRNCompFlagDXT1AForTransparency are not encoded;
 *   - a target bitrate with DDS output is refused (crnlib estimates DDS bitrates with LZMA);
 *   - mip generation: gamma 2.2 only; no rescaling, cropping, clamping or renormalisation.
 * Plain encodes are always uber quality without endpoint caching, so m_dxt_quality and
 * m_dxt_compressor_type do not lower the quality and results do not depend on call order. */
#ifndef CRNGPU_CRNLIB_COMPAT_H
#define CRNGPU_CRNLIB_COMPAT_H

#include <cstddef>

#ifndef CRN_EXPORT
#define CRN_EXPORT __attribute__((visibility("default")))
#endif

typedef unsigned char crn_uint8;
typedef unsigned short crn_uint16;
typedef unsigned int crn_uint32;
typedef signed char crn_int8;
typedef signed short crn_int16;
typedef signed int crn_int32;
typedef unsigned int crn_bool;

/* The 0xFFFFFFFF enumerators fix each enum's underlying type as the reference's: 32-bit unsigned,
 * and 64-bit for crn_format, whose range also holds -1. */
enum crn_file_type { cCRNFileTypeCRN = 0, cCRNFileTypeDDS, cCRNFileTypeForceDWORD = 0xFFFFFFFF };

enum crn_format {
  cCRNFmtInvalid = -1,
  cCRNFmtDXT1 = 0,
  cCRNFmtFirstValid = cCRNFmtDXT1,
  cCRNFmtDXT3,
  cCRNFmtDXT5,
  cCRNFmtDXT5_CCxY,
  cCRNFmtDXT5_xGxR,
  cCRNFmtDXT5_xGBR,
  cCRNFmtDXT5_AGBR,
  cCRNFmtDXN_XY,
  cCRNFmtDXN_YX,
  cCRNFmtDXT5A,
  cCRNFmtETC1,
  cCRNFmtETC2,
  cCRNFmtETC2A,
  cCRNFmtETC1S,
  cCRNFmtETC2AS,
  cCRNFmtTotal,
  cCRNFmtForceDWORD = 0xFFFFFFFF
};

enum crn_limits {
  cCRNMaxLevelResolution = 4096,
  cCRNMinPaletteSize = 8,
  cCRNMaxPaletteSize = 8192,
  cCRNMaxFaces = 6,
  cCRNMaxLevels = 16,
  cCRNMaxHelperThreads = 15,
  cCRNMinQualityLevel = 0,
  cCRNMaxQualityLevel = 255
};

enum crn_comp_flags {
  cCRNCompFlagPerceptual = 1,
  cCRNCompFlagHierarchical = 2,
  cCRNCompFlagQuick = 4,
  cCRNCompFlagUseBothBlockTypes = 8,
  cCRNCompFlagUseTransparentIndicesForBlack = 16,
  cCRNCompFlagDisableEndpointCaching = 32,
  cCRNCompFlagManualPaletteSizes = 64,
  cCRNCompFlagDXT1AForTransparency = 128,
  cCRNCompFlagGrayscaleSampling = 256,
  cCRNCompFlagDebugging = 0x80000000,
  cCRNCompFlagForceDWORD = 0xFFFFFFFF
};

enum crn_dxt_quality {
  cCRNDXTQualitySuperFast,
  cCRNDXTQualityFast,
  cCRNDXTQualityNormal,
  cCRNDXTQualityBetter,
  cCRNDXTQualityUber,
  cCRNDXTQualityTotal,
  cCRNDXTQualityForceDWORD = 0xFFFFFFFF
};

enum crn_dxt_compressor_type {
  cCRNDXTCompressorCRN,
  cCRNDXTCompressorCRNF,
  cCRNDXTCompressorRYG,
  cCRNTotalDXTCompressors,
  cCRNDXTCompressorForceDWORD = 0xFFFFFFFF
};

typedef crn_bool (*crn_progress_callback_func)(crn_uint32 phase_index, crn_uint32 total_phases,
                                               crn_uint32 subphase_index, crn_uint32 total_subphases,
                                               void* pUser_data_ptr);

struct crn_comp_params {
  crn_comp_params() { clear(); }

  /* crunch's defaults: .crn, one face, DXT1, perceptual + hierarchical + both block types,
   * quality 255, uber, deratings 2.0, automatic palette sizes */
  void clear() {
    m_size_of_obj = sizeof(*this);
    m_file_type = cCRNFileTypeCRN;
    m_faces = 1;
    m_width = m_height = 0;
    m_levels = 1;
    m_format = cCRNFmtDXT1;
    m_flags = cCRNCompFlagPerceptual | cCRNCompFlagHierarchical | cCRNCompFlagUseBothBlockTypes;
    for (crn_uint32 f = 0; f < cCRNMaxFaces; f++)
      for (crn_uint32 l = 0; l < cCRNMaxLevels; l++) m_pImages[f][l] = 0;
    m_target_bitrate = 0.0f;
    m_quality_level = cCRNMaxQualityLevel;
    m_dxt1a_alpha_threshold = 128;
    m_dxt_quality = cCRNDXTQualityUber;
    m_dxt_compressor_type = cCRNDXTCompressorCRN;
    m_alpha_component = 3;
    m_crn_adaptive_tile_color_psnr_derating = 2.0f;
    m_crn_adaptive_tile_alpha_psnr_derating = 2.0f;
    m_crn_color_endpoint_palette_size = m_crn_color_selector_palette_size = 0;
    m_crn_alpha_endpoint_palette_size = m_crn_alpha_selector_palette_size = 0;
    m_num_helper_threads = 0;
    m_userdata0 = m_userdata1 = 0;
    m_pProgress_func = 0;
    m_pProgress_func_data = 0;
  }

  /* the parameter ranges crn_compress accepts */
  bool check() const {
    auto palette_ok = [](crn_uint32 n) { return !n || (n >= cCRNMinPaletteSize && n <= cCRNMaxPaletteSize); };
    return m_file_type <= cCRNFileTypeDDS && m_quality_level <= (crn_uint32)cCRNMaxQualityLevel &&
           m_dxt1a_alpha_threshold <= 255 && (m_faces == 1 || m_faces == 6) && m_width >= 1 &&
           m_width <= cCRNMaxLevelResolution && m_height >= 1 && m_height <= cCRNMaxLevelResolution &&
           m_levels >= 1 && m_levels <= cCRNMaxLevels && (long)m_format >= (long)cCRNFmtDXT1 &&
           (long)m_format < (long)cCRNFmtTotal && palette_ok(m_crn_color_endpoint_palette_size) &&
           palette_ok(m_crn_color_selector_palette_size) && palette_ok(m_crn_alpha_endpoint_palette_size) &&
           palette_ok(m_crn_alpha_selector_palette_size) && m_alpha_component <= 3 &&
           m_num_helper_threads <= cCRNMaxHelperThreads && m_dxt_quality <= cCRNDXTQualityUber &&
           m_dxt_compressor_type < cCRNTotalDXTCompressors;
  }

  bool get_flag(crn_comp_flags flag) const { return (m_flags & flag) != 0; }
  void set_flag(crn_comp_flags flag, bool val) { m_flags = val ? (m_flags | flag) : (m_flags & ~(crn_uint32)flag); }

  crn_uint32 m_size_of_obj;
  crn_file_type m_file_type;
  crn_uint32 m_faces;
  crn_uint32 m_width;
  crn_uint32 m_height;
  crn_uint32 m_levels;
  crn_format m_format;
  crn_uint32 m_flags;
  const crn_uint32* m_pImages[cCRNMaxFaces][cCRNMaxLevels];  /* RGBA8 texels, R in the lowest byte */
  float m_target_bitrate;
  crn_uint32 m_quality_level;
  crn_uint32 m_dxt1a_alpha_threshold;
  crn_dxt_quality m_dxt_quality;
  crn_dxt_compressor_type m_dxt_compressor_type;
  crn_uint32 m_alpha_component;
  float m_crn_adaptive_tile_color_psnr_derating;
  float m_crn_adaptive_tile_alpha_psnr_derating;
  crn_uint32 m_crn_color_endpoint_palette_size;
  crn_uint32 m_crn_color_selector_palette_size;
  crn_uint32 m_crn_alpha_endpoint_palette_size;
  crn_uint32 m_crn_alpha_selector_palette_size;
  crn_uint32 m_num_helper_threads;
  crn_uint32 m_userdata0;
  crn_uint32 m_userdata1;
  crn_progress_callback_func m_pProgress_func;
  void* m_pProgress_func_data;
};

enum crn_mip_mode {
  cCRNMipModeUseSourceOrGenerateMips,
  cCRNMipModeUseSourceMips,
  cCRNMipModeGenerateMips,
  cCRNMipModeNoMips,
  cCRNMipModeTotal,
  cCRNModeForceDWORD = 0xFFFFFFFF
};

enum crn_mip_filter {
  cCRNMipFilterBox,
  cCRNMipFilterTent,
  cCRNMipFilterLanczos4,
  cCRNMipFilterMitchell,
  cCRNMipFilterKaiser,
  cCRNMipFilterTotal,
  cCRNMipFilterForceDWORD = 0xFFFFFFFF
};

enum crn_scale_mode {
  cCRNSMDisabled,
  cCRNSMAbsolute,
  cCRNSMRelative,
  cCRNSMLowerPow2,
  cCRNSMNearestPow2,
  cCRNSMNextPow2,
  cCRNSMTotal,
  cCRNSMForceDWORD = 0xFFFFFFFF
};

struct crn_mipmap_params {
  crn_mipmap_params() { clear(); }

  /* crunch's defaults: source mips if any, else a Kaiser chain (blurriness 0.9) filtered in
   * linear light (gamma 2.2), no rescaling */
  void clear() {
    m_size_of_obj = sizeof(*this);
    m_mode = cCRNMipModeUseSourceOrGenerateMips;
    m_filter = cCRNMipFilterKaiser;
    m_gamma_filtering = 1;
    m_gamma = 2.2f;
    m_blurriness = .9f;
    m_renormalize = m_rtopmip = m_tiled = 0;
    m_max_levels = cCRNMaxLevels;
    m_min_mip_size = 1;
    m_scale_mode = cCRNSMDisabled;
    m_scale_x = m_scale_y = 1.0f;
    m_window_left = m_window_top = m_window_right = m_window_bottom = 0;
    m_clamp_scale = 0;
    m_clamp_width = m_clamp_height = 0;
  }
  bool check() const { return true; }

  crn_uint32 m_size_of_obj;
  crn_mip_mode m_mode;
  crn_mip_filter m_filter;
  crn_bool m_gamma_filtering;
  float m_gamma;
  float m_blurriness;
  crn_uint32 m_max_levels;
  crn_uint32 m_min_mip_size;
  crn_bool m_renormalize;
  crn_bool m_rtopmip;
  crn_bool m_tiled;
  crn_scale_mode m_scale_mode;
  float m_scale_x;
  float m_scale_y;
  crn_uint32 m_window_left;
  crn_uint32 m_window_top;
  crn_uint32 m_window_right;
  crn_uint32 m_window_bottom;
  crn_bool m_clamp_scale;
  crn_uint32 m_clamp_width;
  crn_uint32 m_clamp_height;
};

typedef void* (*crn_realloc_func)(void* p, size_t size, size_t* pActual_size, bool movable, void* pUser_data);
typedef size_t (*crn_msize_func)(void* p, void* pUser_data);

struct crn_texture_desc {
  crn_uint32 m_faces;
  crn_uint32 m_width;
  crn_uint32 m_height;
  crn_uint32 m_levels;
  crn_uint32 m_fmt_fourcc;
};

typedef void* crn_block_compressor_context_t;

/* Memory hooks for the blocks this API returns (crn_compress, crn_decompress_crn_to_dds); NULL
 * restores malloc/free. */
CRN_EXPORT void crn_set_memory_callbacks(crn_realloc_func pRealloc, crn_msize_func pMSize, void* pUser_data);
CRN_EXPORT void crn_free_block(void* pBlock);

/* .crn (clustered) or .dds (plain at quality 255, clustered DXT1 below) from the images in
 * comp_params.m_pImages. NULL and compressed_size 0 on failure. */
CRN_EXPORT void* crn_compress(const crn_comp_params& comp_params, crn_uint32& compressed_size,
                              crn_uint32* pActual_quality_level = 0, float* pActual_bitrate = 0);
/* The same after mip handling by mip_params (source mips, or a chain generated on the GPU). */
CRN_EXPORT void* crn_compress(const crn_comp_params& comp_params, const crn_mipmap_params& mip_params,
                              crn_uint32& compressed_size, crn_uint32* pActual_quality_level = 0,
                              float* pActual_bitrate = 0);
/* .crn -> .dds (every face and level transcoded); file_size: in the .crn size, out the .dds size. */
CRN_EXPORT void* crn_decompress_crn_to_dds(const void* pCRN_file_data, crn_uint32& file_size);

CRN_EXPORT crn_uint32 crn_get_format_fourcc(crn_format fmt);
CRN_EXPORT crn_uint32 crn_get_format_bits_per_texel(crn_format fmt);
CRN_EXPORT crn_uint32 crn_get_bytes_per_dxt_block(crn_format fmt);
CRN_EXPORT crn_format crn_get_fundamental_dxt_format(crn_format fmt);
CRN_EXPORT const char* crn_get_file_type_ext(crn_file_type file_type);
CRN_EXPORT const char* crn_get_format_string(crn_format fmt);
CRN_EXPORT const char* crn_get_dxt_quality_string(crn_dxt_quality q);
CRN_EXPORT const char* crn_get_mip_mode_desc(crn_mip_mode m);
CRN_EXPORT const char* crn_get_mip_mode_name(crn_mip_mode m);
CRN_EXPORT const char* crn_get_mip_filter_name(crn_mip_filter f);
CRN_EXPORT const char* crn_get_scale_mode_desc(crn_scale_mode sm);

/* One 4x4 block at a time (16 RGBA8 texels in, one DXTn block out). */
CRN_EXPORT crn_block_compressor_context_t crn_create_block_compressor(const crn_comp_params& params);
CRN_EXPORT void crn_compress_block(crn_block_compressor_context_t pContext, const crn_uint32* pPixels,
                                   void* pDst_block);
CRN_EXPORT void crn_free_block_compressor(crn_block_compressor_context_t pContext);

CRN_EXPORT const char* crn_get_version();
CRN_EXPORT int crn_get_version_number();
CRN_EXPORT int crn_get_version_major();
CRN_EXPORT int crn_get_version_minor();
CRN_EXPORT int crn_get_version_patch();

/* The emscripten wrapper's C exports (emscripten/crunch_lib.cpp:32-41), for JavaScript / WASM
 * bindings and any other C FFI: texture geometry from the .crn header, and crn_decompress, which
 * transcodes levels firstLevel .. firstLevel + levelCount - 1 of face 0 back to back into dst. */
extern "C" {
CRN_EXPORT unsigned int crn_get_width(void* src, unsigned int src_size);
CRN_EXPORT unsigned int crn_get_height(void* src, unsigned int src_size);
CRN_EXPORT unsigned int crn_get_levels(void* src, unsigned int src_size);
CRN_EXPORT unsigned int crn_get_dxt_format(void* src, unsigned int src_size);
CRN_EXPORT unsigned int crn_get_bytes_per_block(void* src, unsigned int src_size);
CRN_EXPORT unsigned int crn_get_uncompressed_size(void* src, unsigned int src_size, unsigned int level);
CRN_EXPORT void crn_decompress(void* src, unsigned int src_size, void* dst, unsigned int dst_size,
                               unsigned int firstLevel, unsigned int levelCount);
}

namespace crnd {

typedef unsigned char uint8;
typedef unsigned short uint16;
typedef unsigned int uint32;
typedef unsigned int uint;
typedef signed int int32;

typedef void* (*crnd_realloc_func)(void* p, size_t size, size_t* pActual_size, bool movable, void* pUser_data);
typedef size_t (*crnd_msize_func)(void* p, void* pUser_data);
/* Accepted for compatibility: the transcoder keeps its tables on the GPU and allocates no host
 * blocks that the caller frees. */
CRN_EXPORT void crnd_set_memory_callbacks(crnd_realloc_func pRealloc, crnd_msize_func pMSize, void* pUser_data);

struct crn_file_info {
  crn_file_info() : m_struct_size(sizeof(crn_file_info)) {}
  uint32 m_struct_size;
  uint32 m_actual_data_size;
  uint32 m_header_size;
  uint32 m_total_palette_size;
  uint32 m_tables_size;
  uint32 m_levels;
  uint32 m_level_compressed_size[cCRNMaxLevels];
  uint32 m_color_endpoint_palette_entries;
  uint32 m_color_selector_palette_entries;
  uint32 m_alpha_endpoint_palette_entries;
  uint32 m_alpha_selector_palette_entries;
};

struct crn_texture_info {
  crn_texture_info() : m_struct_size(sizeof(crn_texture_info)) {}
  uint32 m_struct_size;
  uint32 m_width;
  uint32 m_height;
  uint32 m_levels;
  uint32 m_faces;
  uint32 m_bytes_per_block;
  uint32 m_userdata0;
  uint32 m_userdata1;
  crn_format m_format;
};

struct crn_level_info {
  crn_level_info() : m_struct_size(sizeof(crn_level_info)) {}
  uint32 m_struct_size;
  uint32 m_width;
  uint32 m_height;
  uint32 m_faces;
  uint32 m_blocks_x;
  uint32 m_blocks_y;
  uint32 m_bytes_per_block;
  crn_format m_format;
};

typedef void* crnd_unpack_context;

CRN_EXPORT uint32 crnd_crn_format_to_fourcc(crn_format fmt);
CRN_EXPORT crn_format crnd_get_fundamental_dxt_format(crn_format fmt);
CRN_EXPORT uint32 crnd_get_crn_format_bits_per_texel(crn_format fmt);
CRN_EXPORT uint32 crnd_get_bytes_per_dxt_block(crn_format fmt);
CRN_EXPORT bool crnd_validate_file(const void* pData, uint32 data_size, crn_file_info* pFile_info);
CRN_EXPORT bool crnd_get_texture_info(const void* pData, uint32 data_size, crn_texture_info* pTexture_info);
CRN_EXPORT bool crnd_get_level_info(const void* pData, uint32 data_size, uint32 level_index,
                                    crn_level_info* pLevel_info);
/* The context keeps pData (crnd_get_data returns it); decode tables and palettes live on the GPU. */
CRN_EXPORT crnd_unpack_context crnd_unpack_begin(const void* pData, uint32 data_size);
CRN_EXPORT bool crnd_get_data(crnd_unpack_context pContext, const void** ppData, uint32* pData_size);
/* ppDst: 1 or 6 face pointers, host or device memory (detected per call). */
CRN_EXPORT bool crnd_unpack_level(crnd_unpack_context pContext, void** ppDst, uint32 dst_size_in_bytes,
                                  uint32 row_pitch_in_bytes, uint32 level_index);
CRN_EXPORT bool crnd_unpack_level_segmented(crnd_unpack_context pContext, const void* pSrc, uint32 src_size_in_bytes,
                                            void** ppDst, uint32 dst_size_in_bytes, uint32 row_pitch_in_bytes,
                                            uint32 level_index);
CRN_EXPORT bool crnd_unpack_end(crnd_unpack_context pContext);
CRN_EXPORT const void* crnd_get_level_data(const void* pData, uint32 data_size, uint32 level_index, uint32* pSize);
CRN_EXPORT uint32 crnd_get_segmented_file_size(const void* pData, uint32 data_size);
CRN_EXPORT bool crnd_create_segmented_file(const void* pData, uint32 data_size, void* pBase_data,
                                           uint base_data_size);

}  // namespace crnd

#endif /* CRNGPU_CRNLIB_COMPAT_H */

/*
 * crngpu: GB300 (sm_103a) implementation of crnlib's DXTn hot path behind a plain C ABI.
 *
 * Every entry point takes plain pointers and sizes. Buffers are either host or device
 * memory, as each call's `mem` argument says; device pointers must live on the current
 * CUDA device. `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 * Calls are asynchronous on `stream` only when every buffer is device memory; with any host
 * buffer the call synchronizes before returning.
 *
 * Status codes: >= 0 success (some calls return a size), < 0 failure (CRNGPU_E_*).
 */
#ifndef CRNGPU_H
#define CRNGPU_H

#include <stdint.h>

#if defined(__GNUC__)
#define CRNGPU_API __attribute__((visibility("default")))
#else
#define CRNGPU_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define CRNGPU_OK 0
#define CRNGPU_E_PARAM (-1)        /* bad argument (size, pitch, level, format, NULL) */
#define CRNGPU_E_CORRUPT (-2)      /* malformed .crn data (header, tables or block stream) */
#define CRNGPU_E_DEVICE (-3)       /* CUDA error (allocation, launch, copy) */
#define CRNGPU_E_UNSUPPORTED (-4)  /* valid request outside this library's scope */
#define CRNGPU_E_NOMEM (-5)        /* host memory exhausted (or refused by the installed memory hooks) */

/* Memory kinds for the `mem` arguments. */
#define CRNGPU_MEM_HOST 0
#define CRNGPU_MEM_DEVICE 1

/* crn_format values (inc/crnlib.h:71-110). */
#define CRNGPU_FMT_DXT1 0
#define CRNGPU_FMT_DXT5 2
#define CRNGPU_FMT_DXT5_CCXY 3
#define CRNGPU_FMT_DXT5_XGXR 4
#define CRNGPU_FMT_DXT5_XGBR 5
#define CRNGPU_FMT_DXT5_AGBR 6
#define CRNGPU_FMT_DXN_XY 7
#define CRNGPU_FMT_DXN_YX 8
#define CRNGPU_FMT_DXT5A 9

/* crn_comp_flags bits that the block encoders honour (inc/crnlib.h:132-185). */
#define CRNGPU_FLAG_PERCEPTUAL 1u
#define CRNGPU_FLAG_USE_BOTH_BLOCK_TYPES 8u
#define CRNGPU_FLAG_TRANSPARENT_BLACK 16u  /* cCRNCompFlagUseTransparentIndicesForBlack (DXT1, with both
                                              block types: try_alpha_as_black_optimization) */
#define CRNGPU_FLAG_DXT1A 128u             /* cCRNCompFlagDXT1AForTransparency: DXT1 texels with alpha below
                                              the threshold become transparent (selector 3) */
#define CRNGPU_FLAG_GRAYSCALE 256u         /* cCRNCompFlagGrayscaleSampling: luma distance (DXT1 colour) */

/* crn_dxt_quality (inc/crnlib.h:188-199): the search effort of the block encoders. */
#define CRNGPU_DXT_QUALITY_SUPERFAST 0u
#define CRNGPU_DXT_QUALITY_FAST 1u
#define CRNGPU_DXT_QUALITY_NORMAL 2u
#define CRNGPU_DXT_QUALITY_BETTER 3u
#define CRNGPU_DXT_QUALITY_UBER 4u

/* Library version and last-error text (thread-local). */
CRNGPU_API const char* crngpu_version(void);
CRNGPU_API const char* crngpu_last_error(void);

/* Profiling hook (the counterpart of the reference's timing/statistics output, crn_timer.h:43-50):
 * when enabled, DXT1 encodes count candidate x unique-colour evaluations, the algorithmic work
 * unit of the endpoint search. Reads the count accumulated since the last call into
 * *dxt1_evaluations (if not NULL), then enables (1) or disables (0) counting and clears it. */
CRNGPU_API int crngpu_profile_counters(int enable, uint64_t* dxt1_evaluations, void* stream);

/* Bounded waits inside the kernels (no counterpart in the reference, whose code runs on the CPU).
 * Every wait on an mbarrier is bounded. A staging wait of the DXT1 encoders or of the TMA
 * expansion variants that runs out falls back to reading global memory (the output does not
 * change); a wait on a tcgen05 MMA of the MLP kernels that runs out makes the call return
 * CRNGPU_E_DEVICE. In-flight copies and MMAs are always drained, with a much longer bound, before
 * a CTA exits. crngpu_wait_counters reads how often each happened on the current device (and
 * clears the counts if reset != 0): a non-zero drain count means a CTA exited with a copy still
 * in flight. crngpu_force_wait_timeouts(1) makes every first wait give up at once (a test hook
 * for the fallback paths); crngpu_force_wait_timeouts(0) restores the normal bounds. */
typedef struct crngpu_wait_stats {
    uint32_t encode_stage_timeouts;   /* DXT1 encoders: staging waits that ran out */
    uint32_t encode_drain_failures;   /* DXT1 encoders: drains that ran out */
    uint32_t expand_stage_timeouts;   /* transcode expansion: staging waits that ran out */
    uint32_t expand_drain_failures;   /* transcode expansion: drains that ran out */
    uint32_t mma_wait_timeouts;       /* MLP kernels: MMA waits that ran out */
} crngpu_wait_stats;
CRNGPU_API int crngpu_wait_counters(crngpu_wait_stats* out, int reset);
CRNGPU_API int crngpu_force_wait_timeouts(int on);

/* ------------------------------------------------------------------------------------------
 * Block encoders (every crn_dxt_quality; endpoint caching is never used, so results do not
 * depend on how blocks are batched).
 * --------------------------------------------------------------------------------------- */

/* Parameters of dxt1_endpoint_optimizer::params (crnlib/crn_dxt1.h:168-201) that apply to
 * 16-texel blocks. A caller that fills only the first four fields (struct_size 16, the layout of
 * earlier versions) gets Uber quality without grayscale sampling, DXT1A or the black trial. */
typedef struct crngpu_dxt1_params {
    uint32_t struct_size;      /* sizeof(crngpu_dxt1_params), or 16 */
    int32_t perceptual;        /* m_perceptual */
    int32_t use_alpha_blocks;  /* m_use_alpha_blocks */
    int32_t reserved;
    uint32_t dxt_quality;      /* m_quality: CRNGPU_DXT_QUALITY_* */
    int32_t grayscale_sampling;            /* m_grayscale_sampling */
    int32_t dxt1a;                         /* m_pixels_have_alpha per block, as dxt_image sets it for
                                              DXT1A: some texel's alpha is below the threshold */
    uint32_t dxt1a_alpha_threshold;        /* m_dxt1a_alpha_threshold (128) */
    int32_t use_transparent_indices_for_black;  /* m_use_transparent_indices_for_black */
} crngpu_dxt1_params;

/* The crn_comp_params fields the block encoders read besides m_flags (crnlib.h:231-414). */
typedef struct crngpu_block_options {
    uint32_t struct_size;            /* sizeof(crngpu_block_options) */
    uint32_t dxt_quality;            /* m_dxt_quality: CRNGPU_DXT_QUALITY_* (Uber by default) */
    uint32_t dxt1a_alpha_threshold;  /* m_dxt1a_alpha_threshold (128 by default) */
} crngpu_block_options;

/* Batched replacement for dxt1_endpoint_optimizer::compute (crnlib/crn_dxt1.h:223,
 * crnlib/crn_dxt1.cpp:2234) plus the dxt1_block packing of dxt_image::set_block_pixels
 * (crnlib/crn_dxt_image.cpp:1436-1490).
 *   rgba_blocks: n x 64 bytes (16 RGBA8 texels, row-major within the block)
 *   out_blocks:  n x 8 bytes (dxt1_block: LE16 low colour, LE16 high colour, 4 selector bytes)
 *   out_error:   optional (NULL), n x uint64 squared error (results::m_error)
 * Returns CRNGPU_OK or an error code. */
CRNGPU_API int crngpu_dxt1_optimize_batch(const uint8_t* rgba_blocks, uint32_t n, const crngpu_dxt1_params* params,
                               uint8_t* out_blocks, uint64_t* out_error, int mem, void* stream);

/* Batched replacement for dxt5_endpoint_optimizer::compute (crnlib/crn_dxt5a.h:72,
 * crnlib/crn_dxt5a.cpp:40-196) plus dxt5_block packing (crnlib/crn_dxt_image.cpp:1491-1522).
 *   comp_index: channel (0..3) of each texel to encode; use_both_block_types: allow 6-value blocks
 *   out_blocks: n x 8 bytes (dxt5_block) */
CRNGPU_API int crngpu_dxt5a_optimize_batch(const uint8_t* rgba_blocks, uint32_t n, uint32_t comp_index,
                                int32_t use_both_block_types, uint8_t* out_blocks, int mem, void* stream);

/* Batched replacement for crn_compress_block (inc/crnlib.h:679, crnlib/crnlib.cpp:351-418):
 * encodes n 4x4 blocks to `format` (DXT1, DXT5 family, DXN_XY/YX, DXT5A) with the block
 * layout dxt_image produces. flags: CRNGPU_FLAG_* (crn_comp_params::m_flags).
 * Returns bytes per block (8 or 16) or an error code. */
CRNGPU_API int crngpu_compress_blocks(const uint8_t* rgba_blocks, uint32_t n, uint32_t format, uint32_t flags,
                           uint8_t* out_blocks, int mem, void* stream);

/* The same with crn_comp_params::m_dxt_quality and m_dxt1a_alpha_threshold (options NULL: Uber,
 * 128). Also honours CRNGPU_FLAG_GRAYSCALE, CRNGPU_FLAG_DXT1A (DXT1 only) and
 * CRNGPU_FLAG_TRANSPARENT_BLACK (DXT1 with both block types), as crn_compress_block does. */
CRNGPU_API int crngpu_compress_blocks_ex(const uint8_t* rgba_blocks, uint32_t n, uint32_t format, uint32_t flags,
                                         const crngpu_block_options* options, uint8_t* out_blocks, int mem,
                                         void* stream);

/* Plain (quality 255, no clustering) DXTn encode of one RGBA8 image, the dxt_image::init path
 * (crnlib/crn_dxt_image.cpp:283-349,447-493): 4x4 blocks with edge clamping, block-row-major
 * output, row pitch = blocks_x * bytes_per_block. pitch_bytes: source row pitch (0 = width*4).
 * Returns the number of output bytes or an error code. */
CRNGPU_API int64_t crngpu_compress_image(const uint8_t* rgba, uint32_t width, uint32_t height, uint32_t pitch_bytes,
                              uint32_t format, uint32_t flags, uint8_t* out, uint64_t out_size, int mem,
                              void* stream);

/* crngpu_compress_image with the options of crngpu_compress_blocks_ex. */
CRNGPU_API int64_t crngpu_compress_image_ex(const uint8_t* rgba, uint32_t width, uint32_t height,
                                            uint32_t pitch_bytes, uint32_t format, uint32_t flags,
                                            const crngpu_block_options* options, uint8_t* out, uint64_t out_size,
                                            int mem, void* stream);

/* ------------------------------------------------------------------------------------------
 * Clustered (CRN-style) DXT1 compression: dxt_hc::compress (crnlib/crn_dxt_hc.cpp:97-316) for
 * cDXT1 on the GPU -- adaptive tiles, endpoint codebook VQ, per-cluster endpoint optimisation,
 * selector codebook VQ. The reference's clusterizer is not thread-count deterministic, so this
 * path is compared on quality (RGB RMSE at the same codebook sizes), not bit-exactness.
 * --------------------------------------------------------------------------------------- */

/* dxt_hc::params (crnlib/crn_dxt_hc.h:113-173) for DXT1. Blocks are in the crn_comp layout
 * (crnlib/crn_comp.cpp:454-463, 717-741): per level, per face, rows of block_width blocks, each
 * level padded to a multiple of 8 texels so that block_width and the row count are even. */
typedef struct crngpu_hc_params {
    uint32_t struct_size;                   /* sizeof(crngpu_hc_params) */
    uint32_t num_blocks;                    /* m_num_blocks */
    uint32_t num_levels, num_faces;         /* m_num_levels (1..16), m_num_faces */
    int32_t perceptual;                     /* m_perceptual */
    uint32_t color_endpoint_codebook_size;  /* m_color_endpoint_codebook_size */
    uint32_t color_selector_codebook_size;  /* m_color_selector_codebook_size */
    float adaptive_tile_color_psnr_derating; /* m_adaptive_tile_color_psnr_derating (2.0) */
    uint32_t vq_round_fraction;             /* codebook tree: a round splits the top 1/this of the
                                               leaves by variance (0 = 4; larger = closer to the
                                               reference's one-at-a-time order, more rounds) */
    uint32_t alpha_endpoint_codebook_size;  /* m_alpha_endpoint_codebook_size */
    uint32_t alpha_selector_codebook_size;  /* m_alpha_selector_codebook_size */
    float adaptive_tile_alpha_psnr_derating; /* m_adaptive_tile_alpha_psnr_derating (2.0) */
    float color_alpha_weighting_ratio;      /* m_adaptive_tile_color_alpha_weighting_ratio (3.0) */
    uint32_t alpha_component;               /* DXT5 / DXT5A: the channel encoded as alpha (3) */
    struct {
        uint32_t first_block, num_blocks, block_width;
        float weight;                       /* min(12, 1.3^level) in crn_comp */
    } levels[16];
} crngpu_hc_params;

typedef struct crngpu_hc_stats {
    uint32_t color_endpoints;  /* endpoint codebook entries produced */
    uint32_t color_selectors;  /* selector codebook entries produced */
    uint32_t tiles;            /* tiles the adaptive tiling chose */
    uint32_t reserved;
    double sse_endpoints;      /* RGB squared error over all blocks with the codebook endpoints and
                                  each pixel's best selector (before the selector codebook) */
    double sse_final;          /* RGB squared error of the output blocks */
    uint32_t alpha_endpoints;  /* alpha endpoint codebook entries produced */
    uint32_t alpha_selectors;  /* alpha selector codebook entries produced */
    double sse_alpha;          /* squared error of the output alpha channels (all channels summed) */
} crngpu_hc_stats;

/* d_blocks: num_blocks x 64 bytes (device); d_out: num_blocks x 8 bytes of DXT1 (device).
 * Optional device outputs (NULL to skip): per-block endpoint / selector codebook indices
 * (uint16), the endpoint codebook (uint32 first | second << 16, first > second) and the selector
 * codebook (uint32, 2-bit linear selectors, pixel p at bits 2p). stats (host) may be NULL.
 * Synchronises `stream`. */
CRNGPU_API int crngpu_hc_compress_dxt1(const uint8_t* d_blocks, const crngpu_hc_params* params, uint8_t* d_out,
                                       uint16_t* d_endpoint_idx, uint16_t* d_selector_idx, uint32_t* d_endpoints,
                                       uint32_t* d_selectors, crngpu_hc_stats* stats, void* stream);

/* Clustered encode of DXT1, DXT5 (colour + alpha = params->alpha_component), DXN_XY/YX (two
 * alpha channels, X = red / Y = green) or DXT5A: dxt_hc::compress for those formats, including the
 * alpha endpoint VQ (vec2), the per-cluster dxt5_endpoint_optimizer + refiner and the 3-bit
 * selector codebook (crnlib/crn_dxt_hc.cpp:1014-1300, 1506-1720). d_out: num_blocks x 8 (DXT1,
 * DXT5A) or x 16 (DXT5: alpha then colour; DXN: X then Y) bytes. Synchronises `stream`. */
CRNGPU_API int crngpu_hc_compress(const uint8_t* d_blocks, const crngpu_hc_params* params, uint32_t format,
                                  uint8_t* d_out, crngpu_hc_stats* stats, void* stream);

/* .crn writer: the tail of crn_comp (crnlib/crn_comp.cpp:295-422, 1356-1611; palettes
 * crn_comp::pack_color_endpoints .. pack_alpha_selectors, block streams crn_comp::pack_blocks,
 * models crn_comp::pack_data_models, header crn_comp::create_comp_data). Host code, no GPU needed.
 * blocks: host memory, DXTn blocks of every level in crn_comp's layout (per level, per face, rows
 * of ((w + 7) & ~7) / 4 blocks, ((h + 7) & ~7) / 4 rows; the blocks outside the image are stored
 * but never output), 8 or 16 bytes each as `format` says. Palettes are the distinct endpoint
 * pairs and selector words (at most 8192 of each: cluster first, e.g. crngpu_hc_compress).
 * Returns the file size (the file is copied to `out` when out_capacity suffices) or an error. */
CRNGPU_API int64_t crngpu_crn_pack(const uint8_t* blocks, uint32_t width, uint32_t height, uint32_t levels,
                                   uint32_t faces, uint32_t format, void* out, uint64_t out_capacity);

/* Replaces crn_compress for .crn output with source mips (inc/crnlib.h:614, crnlib/crnlib.cpp:
 * 242-267, m_file_type = cCRNFileTypeCRN, cCRNMipModeUseSourceMips): rgba_levels holds faces x
 * levels RGBA8 images, face-major, level l being max(1, w >> l) x max(1, h >> l) texels, tightly
 * packed and concatenated (the order of crn_comp_params::m_pImages[face][level]). format: DXT1,
 * the DXT5 family (alpha = channel 3; the swizzled variants get the reference's source
 * conversions, crn_comp.cpp:440-452), DXN_XY/YX, DXT5A; quality_level 0..255 sets the codebook
 * sizes; flags: CRNGPU_FLAG_PERCEPTUAL for DXT1 / DXT5. Clustered encode on the GPU, .crn written
 * on the host. Returns the file size (copied to `out` when out_capacity suffices) or an error. */
CRNGPU_API int64_t crngpu_compress_crn(const uint8_t* rgba_levels, uint32_t width, uint32_t height, uint32_t levels,
                                       uint32_t faces, uint32_t format, uint32_t quality_level, uint32_t flags,
                                       void* out, uint64_t out_capacity);

/* crn_compress to DDS (m_file_type = cCRNFileTypeDDS; dds_comp, crnlib/crn_dds_comp.cpp:150-205).
 * quality_level 255: the plain encoder for every format (DXT1, the DXT5 family with the reference's
 * source swizzles, DXN_XY/YX, DXT5A; the perceptual flag is dropped for the non-sRGB formats, as
 * crn_compress does). Below 255, clustered DDS (mipmapped_texture::qdxt_pack,
 * crnlib/crn_mipmapped_texture.cpp:2300-2600): qdxt1 (crnlib/crn_qdxt1.cpp:81-1027) on the colour
 * element and qdxt5 (crnlib/crn_qdxt5.cpp:82-939) on each alpha / DXN element, each with its own
 * adaptive tiling (PSNR clamped to [0, 500]; derating 1.5 / 3.1^level for colour, 2.4 / 3^level
 * for alpha), representative-pair training vectors weighted by endpoint distance, and codebook
 * curves (endpoints: the distinct training vectors x (q/255)^(1.8 m) >= 96 for colour, ^2.1 >= 16
 * for alpha; selectors: the distinct dxt_fast selector words + 128, x (q/255)^(1.65 m) >= 128 for
 * colour, >= 32 for alpha; m = .75 for DXT5's colour, 1.5 for DXT5_CCxY's, else 1), on this
 * library's GPU clusterizer, cluster fit and selector codebooks. Output: the blocks of every
 * face's mip chain, each level's visible blocks row by row (the DDS data layout, without the
 * 128-byte header); returns their size (written when out_capacity suffices). */
CRNGPU_API int64_t crngpu_compress_dds_clustered(const uint8_t* rgba_levels, uint32_t width, uint32_t height,
                                                 uint32_t levels, uint32_t faces, uint32_t format,
                                                 uint32_t quality_level, uint32_t flags, void* out,
                                                 uint64_t out_capacity);

/* The same with crn_comp_params::m_dxt_quality and m_dxt1a_alpha_threshold (options NULL: Uber,
 * 128) for the plain encode at quality 255, where flags may also hold CRNGPU_FLAG_GRAYSCALE,
 * CRNGPU_FLAG_TRANSPARENT_BLACK and CRNGPU_FLAG_DXT1A (DXT1A when both block types are allowed and
 * some texel's alpha is below 255, dds_comp::compress_init, crnlib/crn_dds_comp.cpp:244-247).
 * Below 255 the clusterizer's per-cluster search is Uber's at every dxt quality (the output is
 * judged on quality, not bytes), grayscale and black trials are not used (qdxt1 has neither), and
 * DXT1A is refused with CRNGPU_E_UNSUPPORTED. */
CRNGPU_API int64_t crngpu_compress_dds_clustered_ex(const uint8_t* rgba_levels, uint32_t width, uint32_t height,
                                                    uint32_t levels, uint32_t faces, uint32_t format,
                                                    uint32_t quality_level, uint32_t flags,
                                                    const crngpu_block_options* options, void* out,
                                                    uint64_t out_capacity);

/* Many crn_compress calls at once (no counterpart in the reference, which compresses one texture
 * per call): `threads` host threads (0 = 4), each with its own CUDA stream and device buffers, take
 * items in turn, so one texture's host work (block gather, .crn writer) overlaps other textures'
 * GPU work. Each item is exactly crngpu_compress_crn's call; its `result` gets the file size (the
 * file is copied to `out` when out_capacity suffices) or an error code. Returns CRNGPU_OK when every
 * item succeeded. */
typedef struct crngpu_crn_batch_item {
    const uint8_t* rgba_levels;
    uint32_t width, height, levels, faces, format, quality_level, flags;
    void* out;
    uint64_t out_capacity;
    int64_t result;
} crngpu_crn_batch_item;
CRNGPU_API int crngpu_compress_crn_batch(crngpu_crn_batch_item* items, uint32_t n, uint32_t threads);

/* crn_compress with a target bitrate instead of a quality level (crn_comp_params::m_target_bitrate,
 * inc/crnlib.h:254; the search of create_compressed_texture, crnlib/crn_texture_comp.cpp:120-245):
 * the reference's interpolative search over quality levels 0..255, each trial a full clustered
 * encode and .crn write (bitrate = file bits / texels over all faces and levels), keeping the
 * closest bitrate at or below the target (else the closest above). The blocks are gathered and
 * uploaded once for all trials. The reference's retry without adaptive tiles is not made: its
 * clustered encoder ignores that flag (dxt_hc::params::m_hierarchical is never read), so the retry
 * repeats the same search. *quality_out / *bitrate_out (optional) get the chosen level and its
 * bitrate. Returns the chosen file's size (copied to `out` when out_capacity suffices) or an error. */
CRNGPU_API int64_t crngpu_compress_crn_bitrate(const uint8_t* rgba_levels, uint32_t width, uint32_t height,
                                               uint32_t levels, uint32_t faces, uint32_t format, float target_bitrate,
                                               uint32_t flags, void* out, uint64_t out_capacity,
                                               uint32_t* quality_out, float* bitrate_out);

/* crn_compress for .crn output with every crn_comp_params field this library honours
 * (crnlib/crn_texture_comp.cpp:48-245, crnlib/crn_comp.cpp:524-590): quality_level, or, when
 * target_bitrate > 0 and no manual palette sizes are given, the bitrate search of
 * crngpu_compress_crn_bitrate; options (NULL = crunch's defaults) carry the adaptive-tile PSNR
 * deratings (m_crn_adaptive_tile_color/alpha_psnr_derating, 2.0 each; DXT5_CCxY uses 5.0 for
 * colour unless palette sizes are manual), the alpha channel (m_alpha_component, 3) and manual
 * palette sizes (cCRNCompFlagManualPaletteSizes with m_crn_*_palette_size, clamped to [8, 8192];
 * palette_sizes[0] == 0 = sizes from the quality level). *quality_out gets the quality level of
 * the file (the search's choice when it ran; 0 when manual palette sizes overrode a target
 * bitrate, as in the reference), *bitrate_out the file's bits per texel. Returns the file size (copied to `out` when out_capacity
 * suffices) or an error. */
typedef struct crngpu_crn_options {
    uint32_t struct_size;        /* sizeof(crngpu_crn_options) */
    float colour_psnr_derating;  /* m_crn_adaptive_tile_color_psnr_derating */
    float alpha_psnr_derating;   /* m_crn_adaptive_tile_alpha_psnr_derating */
    uint32_t alpha_component;    /* m_alpha_component (0..3) */
    uint32_t palette_sizes[4];   /* colour endpoints, colour selectors, alpha endpoints, alpha selectors */
} crngpu_crn_options;
CRNGPU_API int64_t crngpu_compress_crn_ex(const uint8_t* rgba_levels, uint32_t width, uint32_t height,
                                          uint32_t levels, uint32_t faces, uint32_t format, uint32_t quality_level,
                                          float target_bitrate, uint32_t flags, const crngpu_crn_options* options,
                                          void* out, uint64_t out_capacity, uint32_t* quality_out,
                                          float* bitrate_out);

/* Codebook sizes for a quality level (crn_comp::quantize_images, crnlib/crn_comp.cpp:541-577):
 * sizes4 = colour endpoints, colour selectors, alpha endpoints, alpha selectors. */
CRNGPU_API int crngpu_hc_codebook_sizes(uint32_t width, uint32_t height, uint32_t quality_level, uint32_t format,
                                        uint32_t* sizes4);

/* ------------------------------------------------------------------------------------------
 * Learned DXT1 endpoint proposal (no counterpart in the reference). A 48 -> 256 -> 256 -> 8 MLP
 * (GELU, BF16 weights, FP32 accumulation on tcgen05 tensor cores) predicts the endpoints the
 * plain optimizer would choose and the error it would reach; the learned encode refines the
 * prediction (selector fit, least-squares endpoint refit, a short +-1 search on the six endpoint
 * components, the 3-colour block on the same endpoints) and keeps it unless its error exceeds
 * threshold x that predicted bound, in which case the block goes through
 * crngpu_dxt1_optimize_batch's exact search.
 * All block/target/output pointers are device memory.
 * --------------------------------------------------------------------------------------- */

/* Creates a network with seeded random weights on the current device; NULL on failure. */
CRNGPU_API void* crngpu_mlp_create(uint64_t seed);
CRNGPU_API int crngpu_mlp_destroy(void* net);

/* Reads (write = 0) or writes (write = 1) parameter `which` (0 W1[256x48], 1 b1[256], 2 W2[256x256],
 * 3 b2[256], 4 W3[16x256] (rows 7..15 stay zero), 5 b3[16]); what: 0 = weights, 1 = gradients. */
CRNGPU_API int crngpu_mlp_param(void* net, int which, int what, float* host, uint32_t count, int write);

/* Forward pass: n RGBA8 blocks (n x 64) -> outputs y (n x 16 fp32; columns 0..6 used). */
CRNGPU_API int crngpu_mlp_forward(void* net, const uint8_t* d_blocks, uint32_t n, float* d_y, void* stream);

/* Training targets from plain-optimizer results: blocks8 (n x 8) and errors (n) -> n x 8 fp32. */
CRNGPU_API int crngpu_mlp_make_targets(const uint8_t* d_blocks8, const uint64_t* d_err, uint32_t n,
                                       float* d_targets, void* stream);

/* Loss of the error-bound output y[6]: tau <= 0 squared error (the default); 0 < tau < 1 the
 * tau-quantile (pinball) loss times `weight`, so y[6] learns an upper bound of the plain
 * optimizer's error that holds for a fraction tau of blocks. Endpoint outputs keep squared error. */
CRNGPU_API int crngpu_mlp_set_bound_loss(void* net, float tau, float weight);

/* Loss gradients for a batch into the gradient buffers; *loss (host) gets the loss. */
CRNGPU_API int crngpu_mlp_gradients(void* net, const uint8_t* d_blocks, const float* d_targets, uint32_t n,
                                    float* loss, void* stream);

/* One AdamW step (betas 0.9/0.999, eps 1e-8, decoupled weight decay) on a batch. */
CRNGPU_API int crngpu_mlp_train_step(void* net, const uint8_t* d_blocks, const float* d_targets, uint32_t n,
                                     float lr, float weight_decay, float* loss, void* stream);

/* Learned DXT1 encode of n blocks (n <= 2^28; fallback blocks use the exact optimizer with both
 * block types). threshold <= 0 sends every block to the exact optimizer. *fallbacks (host,
 * optional) receives the number of blocks that fell back. Synchronises `stream` once, to read the
 * fallback count. */
CRNGPU_API int crngpu_dxt1_learned(void* net, const uint8_t* d_blocks, uint32_t n, int perceptual, float threshold,
                                   uint8_t* d_out, uint32_t* fallbacks, void* stream);

/* The same with the exact optimizer's search effort on the fallback blocks: fallback_quality is a
 * CRNGPU_DXT_QUALITY_* (crngpu_dxt1_learned uses CRNGPU_DXT_QUALITY_UBER). */
CRNGPU_API int crngpu_dxt1_learned_ex(void* net, const uint8_t* d_blocks, uint32_t n, int perceptual, float threshold,
                                      uint32_t fallback_quality, uint8_t* d_out, uint32_t* fallbacks, void* stream);

/* ------------------------------------------------------------------------------------------
 * CRN -> DXTn transcoder (crnd::crn_unpacker, inc/crn_decomp.h:3498-4223; API inc/crn_defs.h:
 * 174-205). Supported: DXT1, DXT5 family, DXN_XY/YX, DXT5A. ETC formats: CRNGPU_E_UNSUPPORTED.
 * --------------------------------------------------------------------------------------- */

typedef struct crngpu_unpack_context_s* crngpu_unpack_context;

/* Replaces crnd_unpack_begin (inc/crn_defs.h:174): parses the header, Huffman models and
 * palettes on the host and uploads the file, decode tables and palettes to the current device.
 * The caller's buffer may be freed after this returns. NULL on failure. */
CRNGPU_API crngpu_unpack_context crngpu_unpack_begin(const void* data, uint32_t data_size);

/* Texture geometry of an open context (crnd_get_texture_info, inc/crn_defs.h:152). */
CRNGPU_API int crngpu_get_info(crngpu_unpack_context ctx, uint32_t* width, uint32_t* height, uint32_t* levels,
                    uint32_t* faces, uint32_t* format, uint32_t* bytes_per_block);

/* Replaces crnd_unpack_level (inc/crn_defs.h:188-191, checks inc/crn_decomp.h:3569-3575):
 * writes level `level_index` of every face to dst_faces[f] (faces pointers), each
 * dst_size_in_bytes large, rows row_pitch_in_bytes apart (0 = minimal; else >= minimal and a
 * multiple of 4). Returns CRNGPU_OK or an error code. */
CRNGPU_API int crngpu_unpack_level(crngpu_unpack_context ctx, void** dst_faces, uint32_t dst_size_in_bytes,
                        uint32_t row_pitch_in_bytes, uint32_t level_index, int mem, void* stream);

/* Segmented variant (crnd_unpack_level_segmented, inc/crn_defs.h:196-200): the level's
 * compressed bytes come from `src` instead of the file passed to crngpu_unpack_begin. */
CRNGPU_API int crngpu_unpack_level_segmented(crngpu_unpack_context ctx, const void* src, uint32_t src_size_in_bytes,
                                  void** dst_faces, uint32_t dst_size_in_bytes, uint32_t row_pitch_in_bytes,
                                  uint32_t level_index, int mem, void* stream);

/* Transcodes levels [first_level, first_level + level_count) in one decode launch and one
 * expansion launch. dst: one buffer receiving the levels back to back, each level
 * faces x blocks_y x (blocks_x * bytes_per_block) bytes (minimal pitch). Returns the total number
 * of bytes written or an error code. */
CRNGPU_API int64_t crngpu_unpack_levels(crngpu_unpack_context ctx, uint32_t first_level, uint32_t level_count, void* dst,
                             uint64_t dst_size, int mem, void* stream);

/* Batched transcode (no single counterpart in the reference, which transcodes one level per
 * crnd_unpack_level call, inc/crn_decomp.h:3537-3619): many levels of many open contexts, of any
 * mix of sizes and formats, decoded by ONE persistent launch (one lane per level stream, streams
 * taken largest-first from a work counter) and expanded by one more. Each item writes levels
 * [first_level, first_level + level_count) of its context back to back into `dst` (device
 * memory), exactly as crngpu_unpack_levels does. Creation validates every item, uploads the job
 * tables and allocates the index-record buffer once; the contexts must stay open while the batch
 * exists. */
typedef struct crngpu_unpack_batch_item {
    crngpu_unpack_context ctx;
    uint32_t first_level;
    uint32_t level_count;
    void* dst;          /* device memory */
    uint64_t dst_size;  /* bytes available at dst */
} crngpu_unpack_batch_item;

typedef struct crngpu_unpack_batch_s* crngpu_unpack_batch;

/* NULL on failure (crngpu_last_error says which item). */
CRNGPU_API crngpu_unpack_batch crngpu_unpack_batch_create(const crngpu_unpack_batch_item* items, uint32_t n);

/* Enqueues the batch on `stream` without synchronising: a two-word memset and two kernels.
 * flags: CRNGPU_BATCH_GRAPH captures them into a CUDA graph on the first call and replays that
 * graph on later calls (one launch from the host per batch); CRNGPU_BATCH_EXPAND_ONLY re-runs
 * only the expansion kernel from the index records of the last decode (the destinations are
 * rewritten; used to time the HBM-bound expansion on its own). The first launch of a batch also
 * runs the expansion autotuner (see crngpu_unpack_batch_tuning) and synchronises once. */
#define CRNGPU_BATCH_GRAPH 1u
#define CRNGPU_BATCH_EXPAND_ONLY 2u
CRNGPU_API int crngpu_unpack_batch_launch(crngpu_unpack_batch batch, uint32_t flags, void* stream);

/* Synchronises `stream` and reports the last launch's outcome: CRNGPU_OK, or CRNGPU_E_CORRUPT if
 * a block stream held an invalid code or palette index (the reference's bool result). */
CRNGPU_API int crngpu_unpack_batch_status(crngpu_unpack_batch batch, void* stream);

/* Autotuner result: the first launch of a batch decodes, then times each expansion variant and
 * keeps the fastest for the batch and as the device's default for later single-texture calls.
 * Variants 0..11: tiles of 1024 << (v >> 1) blocks, DXT1 palettes staged in shared memory when v
 * is odd; 12..15: 8192- and 16384-block tiles whose next pass of index records is loaded before the
 * current pass's palette gathers (staged when v is odd); 16, 17: 16384- and 32768-block tiles,
 * pipelined, 4096-block passes; 18..20: 16384-block (palettes staged when v = 19) and 32768-block
 * tiles whose index records are brought into shared memory by double-buffered TMA bulk copies,
 * 2048-block passes. *variant (-1 before the first launch) and up to n measured times in ms;
 * returns the number of variants. */
CRNGPU_API int crngpu_unpack_batch_tuning(crngpu_unpack_batch batch, int32_t* variant, float* ms, uint32_t n);

/* Forces the expansion variant of later launches (0 .. number of variants - 1; -1 runs the
 * autotuner again at the next launch); drops a captured graph. Every variant writes the same
 * output: this exists to time and test them one by one. */
CRNGPU_API int crngpu_unpack_batch_set_variant(crngpu_unpack_batch batch, int32_t variant);

/* Total output bytes of the batch (sum of the items' level sizes). */
CRNGPU_API int64_t crngpu_unpack_batch_bytes(crngpu_unpack_batch batch);

/* Which decoder runs a level's block stream (no counterpart in the reference, which has one
 * serial decoder). The wide decoder gives one CTA to a level: per-bit-position step tables built
 * in parallel, a serial walk of chunk and block starts at one shared-memory load per step, then
 * parallel symbol decode and a scan of the endpoint indices. It has the lowest latency per level
 * but does more work per block. The lane decoder runs one level stream per lane, many streams per
 * warp: least work per block, the latency of a serial decode. Both give the same bytes.
 * min_blocks = 0 (the default): each plan sends its largest levels to the wide decoder as long as
 * that shortens the plan's decode (a cost model of both decoders and the device's resident wide
 * CTAs); a single texture's large levels go wide, a batch of many textures mostly stays on the
 * lane decoder. Otherwise levels of at least min_blocks blocks (all faces) go wide: 1 sends every
 * level with rows of at most 1024 blocks, 0xFFFFFFFF none. Applies to plans built after the call:
 * contexts' unpack calls and batches created afterwards. */
CRNGPU_API int crngpu_set_decode_split(uint32_t min_blocks);

CRNGPU_API int crngpu_unpack_batch_destroy(crngpu_unpack_batch batch);

/* Mip generation (mipmapped_texture::generate_mipmaps, crnlib/crn_mipmapped_texture.cpp:2140-2215,
 * with the resampler of image_utils::resample_multithreaded, crnlib/crn_image_utils.cpp:662-874):
 * level 0 (width x height RGBA8, tightly packed) is copied, and every further level l is resampled
 * from level 0 to max(1, width >> l) x max(1, height >> l). filter: the crn_mip_filter order
 * (CRNGPU_MIP_FILTER_BOX .. _KAISER; crunch's default is Kaiser); filter_scale: the mip
 * "blurriness" (crunch's default 0.9); flags: CRNGPU_MIP_SRGB filters R, G, B in linear light with
 * gamma 2.2 (crunch's default), CRNGPU_MIP_WRAP wraps at the edges instead of clamping (tiled
 * textures), CRNGPU_MIP_ALPHA filters alpha too (else alpha is 255, as for an image without an
 * alpha channel). levels: 0 = the full chain. out receives the levels back to back. Host or
 * device buffers (mem). Returns the bytes written or an error. */
#define CRNGPU_MIP_FILTER_BOX 0u
#define CRNGPU_MIP_FILTER_TENT 1u
#define CRNGPU_MIP_FILTER_LANCZOS4 2u
#define CRNGPU_MIP_FILTER_MITCHELL 3u
#define CRNGPU_MIP_FILTER_KAISER 4u
#define CRNGPU_MIP_SRGB 1u
#define CRNGPU_MIP_WRAP 2u
#define CRNGPU_MIP_ALPHA 4u
CRNGPU_API int64_t crngpu_generate_mipmaps(const uint8_t* rgba, uint32_t width, uint32_t height, uint32_t levels,
                                           uint32_t filter, float filter_scale, uint32_t flags, uint8_t* out,
                                           uint64_t out_size, int mem, void* stream);

/* Batched plain encode (no single counterpart in the reference, whose dxt_image::init encodes one
 * image at a time, crnlib/crn_dxt_image.cpp:447-493): the mip chains of many textures of any mix
 * of sizes and formats (DXT1, the DXT5 family, DXN_XY/YX, DXT5A) in one gather launch and two
 * persistent encoder launches (colour elements; alpha and DXN channel elements) running side by
 * side. Every block's result equals crngpu_compress_image's on its level with the same flags. */
typedef struct crngpu_encode_item {
    const uint8_t* rgba;  /* device: the levels' RGBA8 texels back to back, level l being
                             max(1, width >> l) x max(1, height >> l), tightly packed (4-byte aligned) */
    uint8_t* out;         /* device: every level's blocks back to back, row-major at minimal pitch
                             (8-byte aligned) */
    uint32_t width, height, levels, format;
} crngpu_encode_item;

typedef struct crngpu_encode_batch_s* crngpu_encode_batch;

/* flags: CRNGPU_FLAG_PERCEPTUAL, CRNGPU_FLAG_USE_BOTH_BLOCK_TYPES (as crngpu_compress_image).
 * Validates every item, uploads the gather and work tables and allocates the gathered-block
 * buffer (64 bytes per block) once. NULL on failure (crngpu_last_error says which item). */
CRNGPU_API crngpu_encode_batch crngpu_encode_batch_create(const crngpu_encode_item* items, uint32_t n, uint32_t flags);

/* Enqueues the batch on `stream` without synchronising. The first launch runs the autotuner (each
 * encoder timed at several CTAs-per-SM launch shapes on the real blocks; synchronises once).
 * flags: CRNGPU_BATCH_GRAPH captures the launches into a CUDA graph on the first call and replays
 * it on later calls. The items' input and output buffers must stay valid while the batch exists. */
CRNGPU_API int crngpu_encode_batch_launch(crngpu_encode_batch batch, uint32_t flags, void* stream);

/* grids[0], grids[1]: the tuned colour / alpha grid sizes (0 before the first launch); ms: the
 * measured times of the colour variants then the alpha variants. Returns the number of variants. */
CRNGPU_API int crngpu_encode_batch_tuning(crngpu_encode_batch batch, int32_t* grids, float* ms, uint32_t n);

/* Number of blocks in the batch; *texels (optional) gets the visible texels. */
CRNGPU_API int64_t crngpu_encode_batch_size(crngpu_encode_batch batch, uint64_t* texels);

CRNGPU_API int crngpu_encode_batch_destroy(crngpu_encode_batch batch);

/* Allocation-free transcode of one level. No counterpart in the reference: it exists for
 * callers that cannot allocate GPU memory while they run -- engines that reserve their whole
 * VRAM budget up front and forbid untracked allocations, and real-time loops in which
 * cudaMalloc/cudaFree would wait for the device to go idle and stall other work.
 * crn_data (crn_size bytes) is the .crn file in host memory; dst_faces holds one device
 * pointer per face; size, pitch and level rules are those of crngpu_unpack_level. Everything
 * else the kernels need lives in one fixed 16 MiB device array that every GPU loading this
 * library holds until the process exits; a level that needs more (tables + palettes + its
 * compressed bytes + 4 or 8 bytes per block) is rejected with CRNGPU_E_PARAM and a message.
 * The call makes no cudaMalloc/cudaFree or other device allocation. The first call on each
 * device looks up the array's device address (cudaGetSymbolAddress); make that first call
 * before any stream capture. All calls share the array and it keeps the last call's contents,
 * so calls that overlap on the GPU (from other threads or streams) race: serialise them.
 * The call returns after the level is written (it reads back a status word). */
CRNGPU_API int crngpu_unpack_level_noalloc(const void* crn_data, uint32_t crn_size, void** dst_faces,
                                           uint32_t dst_size_in_bytes, uint32_t row_pitch_in_bytes,
                                           uint32_t level_index, void* stream);

/* Replaces crnd_unpack_end (inc/crn_defs.h:205). Returns CRNGPU_OK, or CRNGPU_E_PARAM for NULL. */
CRNGPU_API int crngpu_unpack_end(crngpu_unpack_context ctx);

/* Same contract as the reference's extern "C" crn_decompress (emscripten/crunch_lib.cpp:40,
 * 91-120): transcodes levels firstLevel .. firstLevel+levelCount-1 of face 0 back to back into
 * dst (host memory), each level with minimal pitch; levels whose width or height shifts to 0
 * are skipped without advancing dst, as in the reference. */
CRNGPU_API void crngpu_crn_decompress(void* src, unsigned int src_size, void* dst, unsigned int dst_size,
                           unsigned int firstLevel, unsigned int levelCount);

#ifdef __cplusplus
}
#endif

#endif /* CRNGPU_H */

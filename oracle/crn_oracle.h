// CPU restatement of crnlib's DXTn hot path, used as the test oracle and as the CPU
// baseline ("port"). TEST INFRASTRUCTURE: only tests, the smoke check and bench.py's
// cpu_baseline leg load this; the product (crunch2_gb300) never links or calls it.
//
// Parity of this restatement with the reference itself is pinned by tests/golden/ fixtures
// that were produced by the reference compiled from its own sources (oracle/Makefile `ref`).
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

// DXT1 endpoint optimizer over 4x4 blocks (dxt1_endpoint_optimizer::compute,
// crnlib/crn_dxt1.cpp:2234, driven the way dxt_image::set_block_pixels does for cColorDXT1,
// crnlib/crn_dxt_image.cpp:1436-1490, endpoint caching off).
//   blocks: n x 64 bytes (16 RGBA8 texels, row-major in the block)
//   perceptual: 8/25/1 weighted distance (crn_color.h:724-745) when nonzero
//   use_alpha_blocks: allow 3-colour blocks (DXT1 DDS). 0 selects the reference's "hc"
//                     evaluation path (used for the colour half of DXT5)
//   out: n x 8 bytes (dxt1_block layout, crn_dxt.h:109-222); err (optional): n x uint64
// Quality is uber (cCRNDXTQualityUber). Returns 0 on success.
int oracle_dxt1_blocks(const uint8_t* blocks, uint32_t n, int perceptual, int use_alpha_blocks,
                       uint8_t* out, uint64_t* err, int threads);

// The DXT1 block encoder with every parameter the reference's block compressor passes to the
// optimizer (dxt_image::set_block_pixels, crn_dxt_image.cpp:1436-1490):
//   quality: crn_dxt_quality, 0 superfast .. 4 uber (crnlib.h:88-97)
//   grayscale: cCRNCompFlagGrayscaleSampling (luma distance, perceptual off)
//   dxt1a: DXT1A: a block with a texel whose alpha is below alpha_threshold has transparent texels
//   transparent_black: cCRNCompFlagUseTransparentIndicesForBlack (try_alpha_as_black_optimization)
typedef struct oracle_dxt1_opts {
  int perceptual, use_alpha_blocks, quality, grayscale, dxt1a, alpha_threshold, transparent_black;
} oracle_dxt1_opts;
int oracle_dxt1_blocks_ex(const uint8_t* blocks, uint32_t n, const oracle_dxt1_opts* o, uint8_t* out,
                          uint64_t* err, int threads);

// Candidate x unique-colour evaluations (colours visited by the reference's evaluate_solution
// loops, crn_dxt1.cpp:1370-1592, 1759-1835) of the Uber DXT1 search on n blocks: the encoder's
// algorithmic work count.
uint64_t oracle_dxt1_count_evaluations(const uint8_t* blocks, uint32_t n, int perceptual, int use_alpha_blocks,
                                       int threads);

// DXT5A (single channel) endpoint optimizer over 4x4 blocks
// (dxt5_endpoint_optimizer::compute, crnlib/crn_dxt5a.cpp:40-196), uber quality.
//   comp: channel index 0..3;  use_both_block_types: allow 6-value blocks
//   out: n x 8 bytes (dxt5_block layout, crn_dxt.h:266-406)
int oracle_dxt5a_blocks(const uint8_t* blocks, uint32_t n, int comp, int use_both_block_types,
                        uint8_t* out, int threads);

// The same at a given crn_dxt_quality (0 superfast .. 4 uber): the +-16 / +-8 probe grid runs at
// Uber / Better only (crn_dxt5a.cpp:105-141).
int oracle_dxt5a_blocks_q(const uint8_t* blocks, uint32_t n, int comp, int use_both_block_types, int quality,
                          uint8_t* out);

// Whole-format block encode the way dxt_image packs each element
// (crn_dxt_image.cpp:1430-1530): fmt 0 = DXT1 (8 B), 2 = DXT5 (alpha + colour, 16 B),
// 7 = DXN_XY (X then Y, 16 B), 8 = DXN_YX, 9 = DXT5A (8 B). Returns bytes per block or <= 0.
int oracle_encode_blocks(const uint8_t* blocks, uint32_t n, int fmt, int perceptual, int use_both_block_types,
                         uint8_t* out, int threads);

// CRN -> DXTn transcoder (crnd::crn_unpacker, inc/crn_decomp.h:3498-4223).
// Unpacks one level into `faces` output images of row_pitch bytes per block row
// (row_pitch 0 = minimal). Returns 1 on success, 0 on failure (bad file, bad pitch, size).
int oracle_unpack_level(const uint8_t* crn, uint32_t crn_size, uint32_t level, uint8_t* out,
                        uint32_t out_size, uint32_t row_pitch);

// Times `reps` transcodes of every level with `threads` host threads (one unpack
// context per thread, levels/textures distributed over threads). Returns seconds.
double oracle_time_unpack(const uint8_t* crn, uint32_t crn_size, uint32_t reps, int threads);

#ifdef __cplusplus
}
#endif

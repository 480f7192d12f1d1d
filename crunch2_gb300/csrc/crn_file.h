// Host-side .crn container parsing for the GPU transcoder: header, canonical Huffman models
// and palettes. The per-block symbol streams are decoded on the device (crn_transcode.cu).
#pragma once
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "host_alloc.h"

namespace crngpu {

// Canonical-prefix decode table in the layout the device decoder reads (one contiguous POD
// block per model so a context uploads all of them with one copy).
constexpr int kLutBits = 11;               // first-level table: codes up to 11 bits
constexpr int kMaxCodeLen = 16;            // crnd prefix_coding::cMaxExpectedCodeSize
constexpr int kMaxSyms = 8192;             // crnd prefix_coding::cMaxSupportedSyms
constexpr uint32_t kLutLong = 0xFFFFFFFFu; // prefix of a longer (or unused) code

struct DevModel {
  uint32_t lut[1 << kLutBits];   // sym | len << 16 for codes of length <= kLutBits
  uint32_t limit[kMaxCodeLen + 1];  // left-aligned 16-bit exclusive bound of codes with length <= len
  int32_t base[kMaxCodeLen + 1];    // sorted index = base[len] + (peek16 >> (16 - len))
  uint32_t num_syms;
  uint32_t used;                    // 0: the file sent an empty model
  uint16_t sorted[kMaxSyms];        // symbols ordered by (length, symbol)
};

// Host copy of a received model (code lengths) + the device table built from it.
struct Model {
  HVec<uint8_t> sizes;
  bool used = false;
  // host decode helpers (palettes are decoded on the host)
  uint32_t first[kMaxCodeLen + 1] = {}, count[kMaxCodeLen + 1] = {}, offset[kMaxCodeLen + 1] = {};
  HVec<uint16_t> sorted;
  bool build();
  void to_device(DevModel& d) const;
};

struct LevelInfo {
  uint32_t width, height, blocks_x, blocks_y;
  uint32_t ofs, size;  // compressed bytes within the file
};

enum class Kind { DXT1, DXT5, DXN, DXT5A };

// Parsed file: everything the device needs except the compressed level streams themselves.
struct CrnFile {
  uint32_t width = 0, height = 0, levels = 0, faces = 0, format = 0, bytes_per_block = 0;
  uint32_t data_size = 0;
  // cCRNHeaderFlagSegmented (inc/crn_defs.h:296): the level data is not in the file; each level
  // comes with its own buffer (crnd_unpack_level_segmented)
  bool segmented = false;
  Kind kind = Kind::DXT1;
  LevelInfo level[16];
  Model ref_dm, ep_dm[2], sel_dm[2];
  HVec<uint32_t> colour_ep, colour_sel;
  HVec<uint16_t> alpha_ep, alpha_sel;  // alpha_sel: 3 uint16 per entry
  std::string error;

  // Validates the header (crnd_get_header, inc/crn_decomp.h:2657-2670), receives the five
  // Huffman models (init_tables :3662-3692) and decodes the palettes (decode_palettes
  // :3694-3851). Returns false with `error` set on malformed or unsupported input.
  bool parse(const uint8_t* data, uint32_t size);
};

// crc16 of the reference container (inc/crn_decomp.h:2048-2069), used by validate().
uint16_t crc16(const uint8_t* p, uint32_t len, uint16_t crc = 0);

}  // namespace crngpu

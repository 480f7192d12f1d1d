// Host-side .crn parsing: header fields, Huffman model transmission, palette delta decoding.
// Follows the container definition of inc/crn_defs.h:286-339 and the decoder in
// inc/crn_decomp.h (cited per function). Malformed input is reported, never trusted.
#include "crn_file.h"

#include <algorithm>

namespace crngpu {

namespace {

inline uint32_t be(const uint8_t* p, int n) {
  uint32_t v = 0;
  for (int i = 0; i < n; i++) v = (v << 8) | p[i];
  return v;
}

// MSB-first reader; bits past the end read as zero (symbol_codec, inc/crn_decomp.h:3146-3214).
class BitReader {
 public:
  BitReader(const uint8_t* p, uint32_t n) : p_(p), n_(n) {}
  uint32_t get(uint32_t bits) {
    while (have_ < (int)bits) {
      uint32_t byte = pos_ < n_ ? p_[pos_] : 0;
      pos_++;
      acc_ |= (uint64_t)byte << (56 - have_);
      have_ += 8;
    }
    uint32_t v = bits ? (uint32_t)(acc_ >> (64 - bits)) : 0;
    acc_ <<= bits;
    have_ -= bits;
    return v;
  }
  uint32_t peek16() {
    while (have_ < 16) {
      uint32_t byte = pos_ < n_ ? p_[pos_] : 0;
      pos_++;
      acc_ |= (uint64_t)byte << (56 - have_);
      have_ += 8;
    }
    return (uint32_t)(acc_ >> 48);
  }
  void skip(uint32_t bits) { acc_ <<= bits; have_ -= bits; }

 private:
  const uint8_t* p_;
  uint32_t n_, pos_ = 0;
  uint64_t acc_ = 0;
  int have_ = 0;
};

// Decodes one symbol with a canonical model; -1 if the bits match no code.
int decode(const Model& m, BitReader& br) {
  const uint32_t v = br.peek16();
  for (int len = 1; len <= kMaxCodeLen; len++) {
    const uint32_t code = v >> (16 - len);
    if (m.count[len] && code - m.first[len] < m.count[len]) {
      br.skip(len);
      return m.sorted[m.offset[len] + code - m.first[len]];
    }
  }
  return -1;
}

// symbol_codec::decode_receive_static_data_model (inc/crn_decomp.h:3044-3123): the code
// lengths themselves are sent with a 21-symbol code-length code (zero runs and repeats).
bool receive_model(BitReader& br, Model& m) {
  static const uint8_t kOrder[21] = {17, 18, 19, 20, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15, 16};
  m = Model();
  const uint32_t total = br.get(14);
  if (!total) return true;  // empty model: legal to send, an error to use
  if (total > (uint32_t)kMaxSyms) return false;
  const uint32_t ncl = br.get(5);
  if (ncl < 1 || ncl > 21) return false;
  Model cl;
  cl.sizes.assign(21, 0);
  for (uint32_t i = 0; i < ncl; i++) cl.sizes[kOrder[i]] = (uint8_t)br.get(3);
  if (!cl.build()) return false;
  m.sizes.assign(total, 0);
  uint32_t ofs = 0;
  while (ofs < total) {
    const uint32_t left = total - ofs;
    const int c = decode(cl, br);
    if (c < 0) return false;
    if (c <= 16) {
      m.sizes[ofs++] = (uint8_t)c;
    } else if (c == 17 || c == 18) {
      const uint32_t run = c == 17 ? br.get(3) + 3 : br.get(7) + 11;
      if (run > left) return false;
      ofs += run;
    } else {
      const uint32_t run = c == 19 ? br.get(2) + 3 : br.get(6) + 7;
      if (!ofs || run > left || !m.sizes[ofs - 1]) return false;
      std::fill(m.sizes.begin() + ofs, m.sizes.begin() + ofs + run, m.sizes[ofs - 1]);
      ofs += run;
    }
  }
  return m.build();
}

}  // namespace

// decoder_tables::init (inc/crn_decomp.h:2150-2326): canonical codes, symbols sorted by
// (length, index), consecutive code values within a length.
bool Model::build() {
  std::memset(count, 0, sizeof(count));
  for (uint8_t s : sizes) {
    if (s > kMaxCodeLen) return false;
    if (s) count[s]++;
  }
  uint32_t code = 0, off = 0;
  for (int l = 1; l <= kMaxCodeLen; l++) {
    first[l] = code;
    offset[l] = off;
    code = (code + count[l]) << 1;
    off += count[l];
  }
  if (!off) return false;
  // over-subscribed code: some length's codes overflow its bit width
  for (int l = 1; l <= kMaxCodeLen; l++)
    if (count[l] && first[l] + count[l] > (1u << l)) return false;
  sorted.assign(off, 0);
  uint32_t pos[kMaxCodeLen + 1];
  std::memcpy(pos, offset, sizeof(pos));
  for (uint32_t s = 0; s < sizes.size(); s++)
    if (sizes[s]) sorted[pos[sizes[s]]++] = (uint16_t)s;
  used = true;
  return true;
}

void Model::to_device(DevModel& d) const {
  std::memset(&d, 0, sizeof(d));
  d.num_syms = (uint32_t)sizes.size();
  d.used = used ? 1u : 0u;
  for (uint32_t i = 0; i < (1u << kLutBits); i++) d.lut[i] = kLutLong;
  if (!used) return;
  for (int l = 1; l <= kMaxCodeLen; l++) {
    d.limit[l] = (first[l] + count[l]) << (16 - l);
    d.base[l] = (int32_t)offset[l] - (int32_t)first[l];
  }
  for (size_t i = 0; i < sorted.size(); i++) d.sorted[i] = sorted[i];
  for (int l = 1; l <= kLutBits; l++) {
    for (uint32_t k = 0; k < count[l]; k++) {
      const uint32_t c = first[l] + k;
      const uint32_t sym = sorted[offset[l] + k];
      const uint32_t lo = c << (kLutBits - l), hi = (c + 1) << (kLutBits - l);
      for (uint32_t e = lo; e < hi; e++) d.lut[e] = sym | ((uint32_t)l << 16);
    }
  }
}

uint16_t crc16(const uint8_t* p, uint32_t len, uint16_t crc) {
  // CCITT-style polynomial with the byte-wise shift/xor form of inc/crn_decomp.h:2048-2069
  crc = (uint16_t)~crc;
  while (len--) {
    const uint16_t q = (uint16_t)(*p++ ^ (crc >> 8));
    crc = (uint16_t)(crc << 8);
    uint16_t r = (uint16_t)((q >> 4) ^ q);
    crc ^= r;
    r = (uint16_t)(r << 5);
    crc ^= r;
    r = (uint16_t)(r << 7);
    crc ^= r;
  }
  return (uint16_t)~crc;
}

bool CrnFile::parse(const uint8_t* d, uint32_t size) {
  constexpr uint32_t kStructSize = 74;  // sizeof(crn_header) incl. one level offset
  constexpr uint32_t kLevelOfs = 70;
  if (!d || size < kStructSize) { error = "buffer smaller than a crn header"; return false; }
  if (be(d, 2) != (('H' << 8) | 'x')) { error = "bad crn signature"; return false; }
  const uint32_t header_size = be(d + 2, 2);
  data_size = be(d + 6, 4);
  if (header_size < kStructSize || size < data_size) { error = "bad header/data size"; return false; }
  width = be(d + 12, 2);
  height = be(d + 14, 2);
  levels = d[16];
  faces = d[17];
  format = d[18];
  segmented = (be(d + 19, 2) & 1u) != 0;
  if (!width || !height || width > 4096 || height > 4096) { error = "bad dimensions"; return false; }
  if (faces != 1 && faces != 6) { error = "bad face count"; return false; }
  if (!levels || levels > 16 || kLevelOfs + 4 * levels > header_size) { error = "bad level count"; return false; }
  switch (format) {
    case 0: kind = Kind::DXT1; bytes_per_block = 8; break;
    case 2: case 3: case 4: case 5: case 6: kind = Kind::DXT5; bytes_per_block = 16; break;
    case 7: case 8: kind = Kind::DXN; bytes_per_block = 16; break;
    case 9: kind = Kind::DXT5A; bytes_per_block = 8; break;
    default: error = "unsupported crn format (ETC family or invalid)"; return false;
  }
  uint32_t pal_ofs[4], pal_size[4], pal_num[4];
  for (int p = 0; p < 4; p++) {
    pal_ofs[p] = be(d + 33 + 8 * p, 3);
    pal_size[p] = be(d + 36 + 8 * p, 3);
    pal_num[p] = be(d + 39 + 8 * p, 2);
  }
  const uint32_t tables_size = be(d + 65, 2), tables_ofs = be(d + 67, 3);
  auto in_file = [&](uint32_t o, uint32_t n) { return (uint64_t)o + n <= size; };
  for (uint32_t l = 0; l < levels; l++) {
    LevelInfo& li = level[l];
    li.width = std::max(width >> l, 1u);
    li.height = std::max(height >> l, 1u);
    li.blocks_x = (li.width + 3) >> 2;
    li.blocks_y = (li.height + 3) >> 2;
    li.ofs = be(d + kLevelOfs + 4 * l, 4);
    if (segmented) { li.size = 0; continue; }  // level data lives outside this buffer
    const uint32_t next = l + 1 < levels ? be(d + kLevelOfs + 4 * (l + 1), 4) : size;
    if (next <= li.ofs || !in_file(li.ofs, next - li.ofs)) { error = "bad level offsets"; return false; }
    li.size = next - li.ofs;
  }
  const bool colour = kind == Kind::DXT1 || kind == Kind::DXT5;
  const bool alpha = kind != Kind::DXT1;
  if (!tables_size || !in_file(tables_ofs, tables_size)) { error = "bad tables range"; return false; }
  {
    BitReader br(d + tables_ofs, tables_size);
    if (!receive_model(br, ref_dm)) { error = "bad reference model"; return false; }
    if (!pal_num[0] && !pal_num[2]) { error = "no palettes"; return false; }
    if (pal_num[0] && (!receive_model(br, ep_dm[0]) || !receive_model(br, sel_dm[0]))) {
      error = "bad colour models"; return false;
    }
    if (pal_num[2] && (!receive_model(br, ep_dm[1]) || !receive_model(br, sel_dm[1]))) {
      error = "bad alpha models"; return false;
    }
  }
  if (!ref_dm.used || (colour && (!ep_dm[0].used || !sel_dm[0].used || !pal_num[0] || !pal_num[1])) ||
      (alpha && (!ep_dm[1].used || !sel_dm[1].used || !pal_num[2] || !pal_num[3]))) {
    error = "format needs a model or palette the file does not carry";
    return false;
  }
  if (pal_num[0]) {
    // colour endpoints: six running 5/6/5 deltas per entry (decode_color_endpoints :3715-3761)
    if (!pal_size[0] || !in_file(pal_ofs[0], pal_size[0])) { error = "bad colour endpoint range"; return false; }
    BitReader br(d + pal_ofs[0], pal_size[0]);
    Model dm[2];
    if (!receive_model(br, dm[0]) || !receive_model(br, dm[1]) || !dm[0].used || !dm[1].used) {
      error = "bad colour endpoint models"; return false;
    }
    colour_ep.resize(pal_num[0]);
    uint32_t v[6] = {0, 0, 0, 0, 0, 0};
    static const int kModel[6] = {0, 1, 0, 0, 1, 0};
    static const uint32_t kMask[6] = {31, 63, 31, 31, 63, 31};
    for (uint32_t i = 0; i < pal_num[0]; i++) {
      for (int k = 0; k < 6; k++) {
        const int s = decode(dm[kModel[k]], br);
        if (s < 0) { error = "corrupt colour endpoint palette"; return false; }
        v[k] = (v[k] + (uint32_t)s) & kMask[k];
      }
      colour_ep[i] = v[2] | (v[1] << 5) | (v[0] << 11) | (v[5] << 16) | (v[4] << 21) | (v[3] << 27);
    }
    // colour selectors: XOR-delta nibbles, linear order -> DXT1 index order
    // (decode_color_selectors :3763-3798)
    if (!in_file(pal_ofs[1], pal_size[1])) { error = "bad colour selector range"; return false; }
    BitReader bs(d + pal_ofs[1], pal_size[1]);
    Model sm;
    if (!receive_model(bs, sm) || !sm.used) { error = "bad colour selector model"; return false; }
    colour_sel.resize(pal_num[1]);
    uint32_t s = 0;
    for (uint32_t i = 0; i < pal_num[1]; i++) {
      for (uint32_t j = 0; j < 32; j += 4) {
        const int x = decode(sm, bs);
        if (x < 0) { error = "corrupt colour selector palette"; return false; }
        s ^= (uint32_t)x << j;
      }
      colour_sel[i] = ((s ^ (s << 1)) & 0xAAAAAAAAu) | ((s >> 1) & 0x55555555u);
    }
  }
  if (pal_num[2]) {
    // alpha endpoints: two running 8-bit deltas (decode_alpha_endpoints :3800-3827)
    if (!pal_size[2] || !in_file(pal_ofs[2], pal_size[2])) { error = "bad alpha endpoint range"; return false; }
    BitReader br(d + pal_ofs[2], pal_size[2]);
    Model dm;
    if (!receive_model(br, dm) || !dm.used) { error = "bad alpha endpoint model"; return false; }
    alpha_ep.resize(pal_num[2]);
    uint32_t a = 0, b = 0;
    for (uint32_t i = 0; i < pal_num[2]; i++) {
      const int s0 = decode(dm, br), s1 = decode(dm, br);
      if (s0 < 0 || s1 < 0) { error = "corrupt alpha endpoint palette"; return false; }
      a = (a + (uint32_t)s0) & 255;
      b = (b + (uint32_t)s1) & 255;
      alpha_ep[i] = (uint16_t)(a | (b << 8));
    }
    // alpha selectors: XOR-delta 6-bit pairs, linear -> DXT5 index order, 48 bits as 3 x u16
    // (decode_alpha_selectors :3829-3851)
    if (!in_file(pal_ofs[3], pal_size[3])) { error = "bad alpha selector range"; return false; }
    BitReader bs(d + pal_ofs[3], pal_size[3]);
    Model sm;
    if (!receive_model(bs, sm) || !sm.used) { error = "bad alpha selector model"; return false; }
    static const uint8_t kFromLinear[8] = {0, 2, 3, 4, 5, 6, 7, 1};
    uint8_t fl[64];
    for (int i = 0; i < 64; i++) fl[i] = (uint8_t)(kFromLinear[i & 7] | (kFromLinear[i >> 3] << 3));
    alpha_sel.resize((size_t)pal_num[3] * 3);
    uint32_t lin[2] = {0, 0};
    for (uint32_t i = 0; i < pal_num[3]; i++) {
      uint32_t s[2] = {0, 0};
      for (int h = 0; h < 2; h++) {
        for (uint32_t j = 0; j < 24; j += 6) {
          const int x = decode(sm, bs);
          if (x < 0) { error = "corrupt alpha selector palette"; return false; }
          lin[h] ^= (uint32_t)x << j;
          s[h] |= (uint32_t)fl[(lin[h] >> j) & 63] << j;
        }
      }
      alpha_sel[3 * i] = (uint16_t)s[0];
      alpha_sel[3 * i + 1] = (uint16_t)((s[0] >> 16) | (s[1] << 8));
      alpha_sel[3 * i + 2] = (uint16_t)(s[1] >> 8);
    }
  }
  return true;
}

}  // namespace crngpu

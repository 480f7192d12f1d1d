// CPU restatement of the reference CRN -> DXTn transcoder (crnd::crn_unpacker,
// inc/crn_decomp.h). TEST INFRASTRUCTURE ONLY: the oracle for the CUDA transcoder and the
// CPU baseline ("port"). Straight sequential code; each piece cites what it restates.
#include "crn_oracle.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <thread>
#include <vector>

namespace {

// Big-endian packed header fields (crn_packed_uint, inc/crn_defs.h:220-283; layout :301-339).
inline uint32_t be(const uint8_t* p, int n) {
  uint32_t v = 0;
  for (int i = 0; i < n; i++) v = (v << 8) | p[i];
  return v;
}

struct Header {
  uint32_t header_size, data_size, width, height, levels, faces, format;
  uint32_t pal_ofs[4], pal_size[4], pal_num[4];  // colour ep, colour sel, alpha ep, alpha sel
  uint32_t tables_size, tables_ofs;
  uint32_t level_ofs[16];
};
const uint32_t kHeaderFixed = 70;  // bytes before m_level_ofs[]
const uint32_t kHeaderStructSize = 74;  // sizeof(crn_header) with its one-element level array

// crnd_get_header (inc/crn_decomp.h:2657-2670)
bool parse_header(const uint8_t* d, uint32_t size, Header& h) {
  if (!d || size < kHeaderStructSize) return false;
  if (be(d, 2) != (('H' << 8) | 'x')) return false;
  h.header_size = be(d + 2, 2);
  h.data_size = be(d + 6, 4);
  if (h.header_size < kHeaderStructSize || size < h.data_size) return false;
  h.width = be(d + 12, 2);
  h.height = be(d + 14, 2);
  h.levels = d[16];
  h.faces = d[17];
  h.format = d[18];
  for (int p = 0; p < 4; p++) {
    h.pal_ofs[p] = be(d + 33 + 8 * p, 3);
    h.pal_size[p] = be(d + 36 + 8 * p, 3);
    h.pal_num[p] = be(d + 39 + 8 * p, 2);
  }
  h.tables_size = be(d + 65, 2);
  h.tables_ofs = be(d + 67, 3);
  if (h.levels > 16 || kHeaderFixed + 4 * h.levels > h.header_size) return false;
  for (uint32_t l = 0; l < h.levels; l++) h.level_ofs[l] = be(d + kHeaderFixed + 4 * l, 4);
  return true;
}

// MSB-first bit reader over a byte range; reads past the end return zero bits
// (symbol_codec::get_bits / decode refills, inc/crn_decomp.h:3162-3214).
struct Bits {
  const uint8_t* p = nullptr;
  uint64_t n_bits = 0, pos = 0;
  void start(const uint8_t* b, uint32_t size) { p = b; n_bits = (uint64_t)size * 8; pos = 0; }
  uint32_t bit() {
    uint32_t v = 0;
    if (pos < n_bits) v = (p[pos >> 3] >> (7 - (pos & 7))) & 1;
    pos++;
    return v;
  }
  uint32_t bits(uint32_t n) {
    uint32_t v = 0;
    for (uint32_t i = 0; i < n; i++) v = (v << 1) | bit();
    return v;
  }
};

// Canonical prefix code (decoder_tables::init, inc/crn_decomp.h:2150-2326): symbols sorted
// by (code length, symbol index); code values assigned consecutively per length.
struct Model {
  uint32_t n = 0;
  uint32_t first[17] = {}, count[17] = {}, offset[17] = {};
  std::vector<uint16_t> sorted;
  bool ok = false;
  bool build(const std::vector<uint8_t>& sizes) {
    n = (uint32_t)sizes.size();
    std::memset(count, 0, sizeof(count));
    for (uint8_t s : sizes) {
      if (s > 16) return false;
      if (s) count[s]++;
    }
    uint32_t code = 0, off = 0;
    for (int l = 1; l <= 16; l++) {
      first[l] = code;
      offset[l] = off;
      code = (code + count[l]) << 1;
      off += count[l];
    }
    if (!off) return false;
    sorted.assign(off, 0);
    uint32_t pos[17];
    std::memcpy(pos, offset, sizeof(pos));
    for (uint32_t s = 0; s < n; s++)
      if (sizes[s]) sorted[pos[sizes[s]]++] = (uint16_t)s;
    ok = true;
    return true;
  }
  // Returns the symbol, or -1 for a bit pattern that is no code of this model.
  int decode(Bits& br) const {
    uint32_t code = 0;
    for (int l = 1; l <= 16; l++) {
      code = (code << 1) | br.bit();
      if (count[l] && code - first[l] < count[l]) return sorted[offset[l] + code - first[l]];
    }
    return -1;
  }
};

// symbol_codec::decode_receive_static_data_model (inc/crn_decomp.h:3044-3123)
bool receive_model(Bits& br, Model& m) {
  static const uint8_t order[21] = {17, 18, 19, 20, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15, 16};
  const uint32_t total = br.bits(14);
  if (!total) { m = Model(); return true; }
  if (total > 8192) return false;
  std::vector<uint8_t> sizes(total, 0);
  const uint32_t ncl = br.bits(5);
  if (ncl < 1 || ncl > 21) return false;
  std::vector<uint8_t> cl(21, 0);
  for (uint32_t i = 0; i < ncl; i++) cl[order[i]] = (uint8_t)br.bits(3);
  Model clm;
  if (!clm.build(cl)) return false;
  uint32_t ofs = 0;
  while (ofs < total) {
    const uint32_t remaining = total - ofs;
    const int c = clm.decode(br);
    if (c < 0) return false;
    if (c <= 16) {
      sizes[ofs++] = (uint8_t)c;
    } else if (c == 17 || c == 18) {
      const uint32_t len = c == 17 ? br.bits(3) + 3 : br.bits(7) + 11;
      if (len > remaining) return false;
      ofs += len;
    } else {
      const uint32_t len = c == 19 ? br.bits(2) + 3 : br.bits(6) + 7;
      if (!ofs || len > remaining) return false;
      const uint8_t prev = sizes[ofs - 1];
      if (!prev) return false;
      for (uint32_t k = 0; k < len; k++) sizes[ofs++] = prev;
    }
  }
  return m.build(sizes);
}

struct Unpacker {
  const uint8_t* data = nullptr;
  uint32_t size = 0;
  Header h{};
  Model ref_dm, ep_dm[2], sel_dm[2];
  std::vector<uint32_t> colour_ep, colour_sel;
  std::vector<uint16_t> alpha_ep, alpha_sel;

  bool is_dxt5_family() const { return h.format >= 2 && h.format <= 6; }
  bool is_dxn() const { return h.format == 7 || h.format == 8; }
  bool is_dxt5a() const { return h.format == 9; }
  bool is_dxt1() const { return h.format == 0; }

  bool in_file(uint32_t ofs, uint32_t sz) const { return (uint64_t)ofs + sz <= size; }

  // crn_unpacker::init / init_tables / decode_palettes (inc/crn_decomp.h:3519-3851)
  bool init(const uint8_t* d, uint32_t sz) {
    if (!parse_header(d, sz, h)) return false;
    data = d;
    size = sz;
    if (!(is_dxt1() || is_dxt5_family() || is_dxn() || is_dxt5a())) return false;
    Bits br;
    if (!h.tables_size || !in_file(h.tables_ofs, h.tables_size)) return false;
    br.start(d + h.tables_ofs, h.tables_size);
    if (!receive_model(br, ref_dm)) return false;
    if (!h.pal_num[0] && !h.pal_num[2]) return false;
    if (h.pal_num[0]) {
      if (!receive_model(br, ep_dm[0]) || !receive_model(br, sel_dm[0])) return false;
    }
    if (h.pal_num[2]) {
      if (!receive_model(br, ep_dm[1]) || !receive_model(br, sel_dm[1])) return false;
    }
    if (h.pal_num[0]) {
      // decode_color_endpoints :3715-3761 (delta-coded 5/6/5 pairs)
      if (!h.pal_size[0] || !in_file(h.pal_ofs[0], h.pal_size[0])) return false;
      br.start(d + h.pal_ofs[0], h.pal_size[0]);
      Model dm[2];
      if (!receive_model(br, dm[0]) || !receive_model(br, dm[1])) return false;
      if (!dm[0].ok || !dm[1].ok) return false;
      uint32_t a = 0, b = 0, c = 0, e = 0, f = 0, g = 0;
      colour_ep.resize(h.pal_num[0]);
      for (uint32_t i = 0; i < h.pal_num[0]; i++) {
        int s0 = dm[0].decode(br), s1 = dm[1].decode(br), s2 = dm[0].decode(br);
        int s3 = dm[0].decode(br), s4 = dm[1].decode(br), s5 = dm[0].decode(br);
        if (s0 < 0 || s1 < 0 || s2 < 0 || s3 < 0 || s4 < 0 || s5 < 0) return false;
        a = (a + s0) & 31; b = (b + s1) & 63; c = (c + s2) & 31;
        e = (e + s3) & 31; f = (f + s4) & 63; g = (g + s5) & 31;
        colour_ep[i] = c | (b << 5) | (a << 11) | (g << 16) | (f << 21) | (e << 27);
      }
      // decode_color_selectors :3763-3798 (XOR-delta nibbles, linear -> DXT1 index order)
      if (!in_file(h.pal_ofs[1], h.pal_size[1])) return false;
      br.start(d + h.pal_ofs[1], h.pal_size[1]);
      Model sm;
      if (!receive_model(br, sm) || !sm.ok) return false;
      colour_sel.resize(h.pal_num[1]);
      uint32_t s = 0;
      for (uint32_t i = 0; i < h.pal_num[1]; i++) {
        for (uint32_t j = 0; j < 32; j += 4) {
          int v = sm.decode(br);
          if (v < 0) return false;
          s ^= (uint32_t)v << j;
        }
        colour_sel[i] = ((s ^ (s << 1)) & 0xAAAAAAAAu) | ((s >> 1) & 0x55555555u);
      }
    }
    if (h.pal_num[2]) {
      // decode_alpha_endpoints :3800-3827
      if (!h.pal_size[2] || !in_file(h.pal_ofs[2], h.pal_size[2])) return false;
      br.start(d + h.pal_ofs[2], h.pal_size[2]);
      Model dm;
      if (!receive_model(br, dm) || !dm.ok) return false;
      alpha_ep.resize(h.pal_num[2]);
      uint32_t a = 0, b = 0;
      for (uint32_t i = 0; i < h.pal_num[2]; i++) {
        int s0 = dm.decode(br), s1 = dm.decode(br);
        if (s0 < 0 || s1 < 0) return false;
        a = (a + s0) & 255;
        b = (b + s1) & 255;
        alpha_ep[i] = (uint16_t)(a | (b << 8));
      }
      // decode_alpha_selectors :3829-3851 (XOR-delta 6-bit pairs, linear -> DXT5 index order)
      if (!in_file(h.pal_ofs[3], h.pal_size[3])) return false;
      br.start(d + h.pal_ofs[3], h.pal_size[3]);
      Model sm;
      if (!receive_model(br, sm) || !sm.ok) return false;
      static const uint8_t from_linear[8] = {0, 2, 3, 4, 5, 6, 7, 1};
      uint8_t fl64[64];
      for (int i = 0; i < 64; i++) fl64[i] = (uint8_t)(from_linear[i & 7] | (from_linear[i >> 3] << 3));
      alpha_sel.resize((size_t)h.pal_num[3] * 3);
      uint32_t s0l = 0, s1l = 0;
      for (size_t i = 0; i < alpha_sel.size();) {
        uint32_t s0 = 0, s1 = 0;
        for (uint32_t j = 0; j < 24; j += 6) {
          int v = sm.decode(br);
          if (v < 0) return false;
          s0l ^= (uint32_t)v << j;
          s0 |= (uint32_t)fl64[(s0l >> j) & 63] << j;
        }
        for (uint32_t j = 0; j < 24; j += 6) {
          int v = sm.decode(br);
          if (v < 0) return false;
          s1l ^= (uint32_t)v << j;
          s1 |= (uint32_t)fl64[(s1l >> j) & 63] << j;
        }
        alpha_sel[i++] = (uint16_t)s0;
        alpha_sel[i++] = (uint16_t)((s0 >> 16) | (s1 << 8));
        alpha_sel[i++] = (uint16_t)(s1 >> 8);
      }
    }
    return true;
  }

  // crn_unpacker::unpack_level + unpack_dxt1/dxt5/dxn/dxt5a (inc/crn_decomp.h:3537-4223)
  bool unpack_level(uint32_t level, uint8_t* out, uint32_t out_size, uint32_t row_pitch) {
    if (level >= h.levels) return false;
    const uint32_t ofs = h.level_ofs[level];
    const uint32_t next = level + 1 < h.levels ? h.level_ofs[level + 1] : size;
    if (next <= ofs || next > size) return false;
    const uint32_t w = std::max(h.width >> level, 1u), ht = std::max(h.height >> level, 1u);
    const uint32_t bx = (w + 3) >> 2, by = (ht + 3) >> 2;
    const uint32_t bpb = (is_dxt1() || is_dxt5a()) ? 8 : 16;
    const uint32_t minimal = bpb * bx;
    if (!row_pitch) row_pitch = minimal;
    else if (row_pitch < minimal || (row_pitch & 3)) return false;
    const uint64_t face_bytes = (uint64_t)row_pitch * by;
    if ((uint64_t)out_size < face_bytes * h.faces) return false;
    Bits br;
    br.start(data + ofs, next - ofs);
    const bool colour = is_dxt1() || is_dxt5_family();
    const int alpha_channels = is_dxn() ? 2 : ((is_dxt5_family() || is_dxt5a()) ? 1 : 0);
    if (!ref_dm.ok) return false;
    if (colour && (!ep_dm[0].ok || !sel_dm[0].ok || colour_ep.empty())) return false;
    if (alpha_channels && (!ep_dm[1].ok || !sel_dm[1].ok || alpha_ep.empty())) return false;
    const uint32_t W = (bx + 1) & ~1u, H = (by + 1) & ~1u;
    struct Buf { uint32_t ref, cep, aep[2]; };
    std::vector<Buf> row(W, Buf{0, 0, {0, 0}});
    uint32_t cep = 0, aep[2] = {0, 0};
    uint32_t group = 0;
    const uint32_t ncep = (uint32_t)colour_ep.size(), naep = (uint32_t)alpha_ep.size();
    for (uint32_t f = 0; f < h.faces; f++) {
      uint8_t* face = out + face_bytes * f;
      for (uint32_t y = 0; y < H; y++) {
        for (uint32_t x = 0; x < W; x++) {
          const bool visible = y < by && x < bx;
          if (!(y & 1) && !(x & 1)) {
            int g = ref_dm.decode(br);
            if (g < 0) return false;
            group = (uint32_t)g;
          }
          Buf& b = row[x];
          uint32_t refv;
          if (y & 1) {
            refv = b.ref;
          } else {
            refv = group & 3;
            group >>= 2;
            b.ref = group & 3;
            group >>= 2;
          }
          if (refv == 0) {
            if (colour) {
              int dlt = ep_dm[0].decode(br);
              if (dlt < 0) return false;
              cep += (uint32_t)dlt;
              if (cep >= ncep) cep -= ncep;
              if (cep >= ncep) return false;
              b.cep = cep;
            }
            for (int k = 0; k < alpha_channels; k++) {
              int dlt = ep_dm[1].decode(br);
              if (dlt < 0) return false;
              aep[k] += (uint32_t)dlt;
              if (aep[k] >= naep) aep[k] -= naep;
              if (aep[k] >= naep) return false;
              b.aep[k] = aep[k];
            }
          } else if (refv == 1) {
            b.cep = cep;
            b.aep[0] = aep[0];
            b.aep[1] = aep[1];
          } else {
            cep = b.cep;
            aep[0] = b.aep[0];
            aep[1] = b.aep[1];
          }
          uint32_t csel = 0, asel[2] = {0, 0};
          if (colour) {
            int v = sel_dm[0].decode(br);
            if (v < 0 || (uint32_t)v >= colour_sel.size()) return false;
            csel = (uint32_t)v;
          }
          for (int k = 0; k < alpha_channels; k++) {
            int v = sel_dm[1].decode(br);
            if (v < 0 || (uint32_t)v * 3 >= alpha_sel.size()) return false;
            asel[k] = (uint32_t)v;
          }
          if (!visible) continue;
          uint32_t* o = reinterpret_cast<uint32_t*>(face + (size_t)y * row_pitch + (size_t)x * bpb);
          uint32_t words[4];
          int nw = 0;
          for (int k = 0; k < alpha_channels; k++) {
            const uint16_t* s = &alpha_sel[asel[k] * 3];
            words[nw++] = alpha_ep[aep[k]] | ((uint32_t)s[0] << 16);
            words[nw++] = s[1] | ((uint32_t)s[2] << 16);
          }
          if (colour) {
            words[nw++] = colour_ep[cep];
            words[nw++] = colour_sel[csel];
          }
          std::memcpy(o, words, 4 * nw);
        }
      }
    }
    return true;
  }
};

}  // namespace

extern "C" int oracle_unpack_level(const uint8_t* crn, uint32_t crn_size, uint32_t level, uint8_t* out,
                                   uint32_t out_size, uint32_t row_pitch) {
  Unpacker u;
  if (!u.init(crn, crn_size)) return 0;
  return u.unpack_level(level, out, out_size, row_pitch) ? 1 : 0;
}

extern "C" double oracle_time_unpack(const uint8_t* crn, uint32_t crn_size, uint32_t reps, int threads) {
  Unpacker probe;
  if (!probe.init(crn, crn_size)) return -1.0;
  const uint32_t levels = probe.h.levels;
  if (threads < 1) threads = 1;
  std::atomic<uint32_t> next(0);
  const uint32_t total = reps * levels;
  auto t0 = std::chrono::steady_clock::now();
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; t++) {
    pool.emplace_back([&]() {
      Unpacker u;
      if (!u.init(crn, crn_size)) return;
      std::vector<uint8_t> scratch;
      for (;;) {
        const uint32_t job = next.fetch_add(1);
        if (job >= total) break;
        const uint32_t l = job % levels;
        const uint32_t w = std::max(u.h.width >> l, 1u), ht = std::max(u.h.height >> l, 1u);
        const uint32_t bpb = (u.is_dxt1() || u.is_dxt5a()) ? 8 : 16;
        const size_t need = (size_t)((w + 3) >> 2) * ((ht + 3) >> 2) * bpb * u.h.faces;
        if (scratch.size() < need) scratch.resize(need);
        u.unpack_level(l, scratch.data(), (uint32_t)scratch.size(), 0);
      }
    });
  }
  for (auto& th : pool) th.join();
  auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double>(t1 - t0).count();
}

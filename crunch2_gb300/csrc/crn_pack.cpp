// .crn writer: the serial tail of crn_comp (crnlib/crn_comp.cpp:295-422, 1356-1611) after the
// clustered encode. It packs DXTn blocks in crn_comp's block layout into a .crn file that
// crnd::crn_unpacker (inc/crn_decomp.h) and this library's transcoder decode back to exactly
// those blocks:
//   * palettes = the distinct endpoint pairs and selector words of the blocks (at most 8192 of
//     each, the decoder's limit), in first-use order, delta coded as crn_comp::pack_color_endpoints /
//     pack_color_selectors / pack_alpha_endpoints / pack_alpha_selectors do;
//   * per level, the block stream of crn_comp::pack_blocks: one reference group per 2x2 blocks
//     (left / top endpoint reuse), endpoint index deltas modulo the palette size, selector
//     indices;
//   * static canonical Huffman models (code lengths limited to 16 bits), transmitted with the
//     21-symbol code-length code of symbol_codec (run-length codes 17-20);
//   * the header (inc/crn_defs.h:286-339) with its two CRC16s.
//   * palette order chosen as crn_comp::optimize_color / optimize_alpha do
//     (crnlib/crn_comp.cpp:767-1321): selectors as a nearest-neighbour chain under an XOR-delta
//     cost; endpoints by four trials (a nearest-neighbour chain, and three two-ended chains grown
//     from the most frequent endpoint by similarity times co-occurrence in the block stream),
//     keeping the trial whose palette plus index stream codes in the fewest bits.
// The order changes the file size only, never the decoded blocks.
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <exception>
#include <functional>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "crn_file.h"
#include "crngpu_internal.h"

namespace crngpu {
namespace {

// MSB-first bit writer. A code of up to 32 bits joins the fewer than 8 pending bits in a 64-bit
// accumulator, whose whole bytes are then appended; bits above the pending ones are stale and
// never read.
class BitWriter {
 public:
  void put(uint32_t v, uint32_t bits) {  // the low `bits` (<= 32) bits of v
    if (!bits) return;
    acc_ = (acc_ << bits) | ((uint64_t)v & ((1ull << bits) - 1ull));
    n_ += bits;
    while (n_ >= 8) {
      n_ -= 8;
      out_.push_back((uint8_t)(acc_ >> n_));
    }
  }
  std::vector<uint8_t> finish() {
    if (n_) { out_.push_back((uint8_t)(acc_ << (8 - n_))); acc_ = 0; n_ = 0; }
    return std::move(out_);
  }
  uint64_t bits() const { return (uint64_t)out_.size() * 8 + (uint64_t)n_; }

 private:
  std::vector<uint8_t> out_;
  uint64_t acc_ = 0;
  uint32_t n_ = 0;
};

// Huffman code lengths for a histogram, limited to `limit` bits (frequencies are halved until the
// tree fits). Unused symbols get 0; a single used symbol gets length 1. The two lightest nodes
// are merged first, ties to the lower node id (leaves 0..n-1 by symbol, then merged nodes in
// creation order). Merged nodes are created in non-decreasing weight, so the lightest node is at
// the front of either the (weight, symbol)-sorted leaves or the merged nodes: two queues instead
// of a heap, with the same merges.
std::vector<uint8_t> code_lengths(const std::vector<uint32_t>& freq_in, int limit) {
  const size_t n = freq_in.size();
  std::vector<uint8_t> len(n, 0);
  std::vector<uint64_t> freq(freq_in.begin(), freq_in.end());
  size_t used = 0, last = 0;
  for (size_t i = 0; i < n; i++)
    if (freq[i]) { used++; last = i; }
  if (!used) return len;
  if (used == 1) { len[last] = 1; return len; }
  std::vector<uint32_t> leaves;
  leaves.reserve(used);
  std::vector<uint64_t> mw(used - 1);             // merged node k: weight, parent
  std::vector<uint32_t> parent(n + used - 1);     // by node id: leaves 0..n-1, merged n + k
  std::vector<uint8_t> depth(used - 1);
  for (;;) {
    leaves.clear();
    for (size_t i = 0; i < n; i++)
      if (freq[i]) leaves.push_back((uint32_t)i);
    std::sort(leaves.begin(), leaves.end(),
              [&](uint32_t a, uint32_t b) { return freq[a] != freq[b] ? freq[a] < freq[b] : a < b; });
    size_t li = 0, mi = 0, made = 0;
    auto take = [&]() -> std::pair<uint64_t, size_t> {  // (weight, node id) of the lighter front
      if (li < leaves.size() && (mi == made || freq[leaves[li]] <= mw[mi])) {
        const uint32_t s = leaves[li++];
        return {freq[s], s};
      }
      const size_t k = mi++;
      return {mw[k], n + k};
    };
    while (made < used - 1) {
      const auto a = take();
      const auto b = take();
      parent[a.second] = (uint32_t)(n + made);
      parent[b.second] = (uint32_t)(n + made);
      mw[made++] = a.first + b.first;
    }
    // depths top-down: a merged node's parent was created after it
    int maxl = 0;
    depth[used - 2] = 0;
    for (size_t k = used - 1; k-- > 0;)
      if (k != used - 2) depth[k] = (uint8_t)std::min<int>(255, depth[parent[n + k] - n] + 1);
    for (uint32_t s : leaves) {
      const int d = depth[parent[s] - n] + 1;
      len[s] = (uint8_t)std::min(d, 255);
      maxl = std::max(maxl, d);
    }
    if (maxl <= limit) return len;
    for (auto& f : freq)
      if (f) f = (f + 1) >> 1;
  }
}

// Canonical codes (the decoder's convention, inc/crn_decomp.h:2150-2326): symbols ordered by
// (length, index), consecutive codes within a length.
std::vector<uint32_t> canonical_codes(const std::vector<uint8_t>& len) {
  uint32_t count[17] = {}, next_code[17] = {};
  for (uint8_t l : len)
    if (l) count[l]++;
  uint32_t code = 0;
  for (int l = 1; l <= 16; l++) {
    next_code[l] = code;
    code = (code + count[l]) << 1;
  }
  std::vector<uint32_t> codes(len.size(), 0);
  for (size_t s = 0; s < len.size(); s++)
    if (len[s]) codes[s] = next_code[len[s]]++;
  return codes;
}

struct Huff {
  std::vector<uint8_t> len;
  std::vector<uint32_t> code;
  void build(const std::vector<uint32_t>& freq, int limit) {
    len = code_lengths(freq, limit);
    code = canonical_codes(len);
  }
  void put(BitWriter& bw, uint32_t sym) const { bw.put(code[sym], len[sym]); }
};

// A symbol list (model << 16 | symbol) coded behind its models, MSB first, as BitWriter would
// write it: the accumulator in locals, whole 32-bit words stored into a buffer sized for the
// longest codes (16 bits a symbol).
std::vector<uint8_t> code_symbols(const std::vector<uint32_t>& syms, const Huff* models, int nmodels,
                                  uint64_t* bits = nullptr) {
  const uint32_t* code[8];
  const uint8_t* len[8];
  for (int k = 0; k < nmodels; k++) {
    code[k] = models[k].code.data();
    len[k] = models[k].len.data();
  }
  std::vector<uint8_t> out(syms.size() * 2 + 8);
  uint8_t* p = out.data();
  uint64_t acc = 0;
  uint32_t n = 0;
  for (uint32_t v : syms) {
    const uint32_t k = v >> 16, sym = v & 0xFFFFu, l = len[k][sym];
    acc = (acc << l) | code[k][sym];  // a canonical code of l bits is below 2^l
    n += l;
    if (n >= 32) {
      n -= 32;
      const uint32_t w = (uint32_t)(acc >> n);
      p[0] = (uint8_t)(w >> 24); p[1] = (uint8_t)(w >> 16); p[2] = (uint8_t)(w >> 8); p[3] = (uint8_t)w;
      p += 4;
    }
  }
  while (n >= 8) {
    n -= 8;
    *p++ = (uint8_t)(acc >> n);
  }
  if (bits) *bits = (uint64_t)(p - out.data()) * 8 + n;
  if (n) *p++ = (uint8_t)(acc << (8 - n));
  out.resize((size_t)(p - out.data()));
  return out;
}

// Appends `bits` bits of a zero-padded MSB-first bit string to an MSB-first stream of out_bits
// bits (whose last byte is zero-padded as well).
void append_bits(std::vector<uint8_t>& out, uint64_t& out_bits, const std::vector<uint8_t>& in, uint64_t bits) {
  const size_t nin = (size_t)((bits + 7) / 8);
  if (!nin) return;
  const uint32_t shift = (uint32_t)(out_bits & 7);
  out.resize((size_t)((out_bits + bits + 7) / 8) + 1);  // one byte of room for the shifted spill
  uint8_t* o = out.data() + out_bits / 8;
  if (!shift) {
    std::memcpy(o, in.data(), nin);
  } else {
    for (size_t k = 0; k < nin; k++) {
      o[k] |= (uint8_t)(in[k] >> shift);
      o[k + 1] = (uint8_t)(in[k] << (8 - shift));
    }
  }
  out_bits += bits;
  out.resize((size_t)((out_bits + 7) / 8));
}

// Runs fn(job, worker) for jobs 0 .. n-1 on up to `threads` threads (worker < threads), taking
// jobs in order as workers free up. An exception in a job is passed on to the caller once every
// worker has stopped.
template <class F>
void parallel_jobs(size_t n, unsigned threads, F fn) {
  threads = (unsigned)std::max<size_t>(1, std::min<size_t>(threads, n));
  if (threads == 1) {
    for (size_t j = 0; j < n; j++) fn(j, 0u);
    return;
  }
  std::atomic<size_t> next{0};
  std::exception_ptr error;
  std::mutex error_mu;
  auto work = [&](unsigned w) {
    try {
      for (size_t j = next++; j < n; j = next++) fn(j, w);
    } catch (...) {
      std::lock_guard<std::mutex> lock(error_mu);
      if (!error) error = std::current_exception();
      next = n;
    }
  };
  std::vector<std::thread> pool;
  try {
    for (unsigned w = 1; w < threads; w++) pool.emplace_back(work, w);
  } catch (...) {  // a thread that cannot start: the others take its jobs
  }
  work(0);
  for (auto& t : pool) t.join();
  if (error) std::rethrow_exception(error);
}

// worker threads for the writer's parallel steps
unsigned pack_threads(uint64_t nblocks) {
  if (nblocks < 16384) return 1;
  const unsigned hw = std::thread::hardware_concurrency();
  return std::max(1u, std::min(hw ? hw : 4u, 16u));
}

// symbol_codec's static model transmission, the inverse of
// decode_receive_static_data_model (inc/crn_decomp.h:3044-3123): 14-bit symbol count, the 21
// code-length-code lengths in transmission order (3 bits each), then the code lengths coded with
// literals 0-16, zero runs (17: 3-10, 18: 11-138) and repeats of the previous length (19: 3-6,
// 20: 7-70).
void send_model(BitWriter& bw, const Huff& h) {
  static const uint8_t kOrder[21] = {17, 18, 19, 20, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15, 16};
  const std::vector<uint8_t>& len = h.len;
  const uint32_t total = (uint32_t)len.size();
  bw.put(total, 14);
  if (!total) return;
  struct Sym { uint8_t s; uint32_t extra; int bits; };
  std::vector<Sym> syms;
  for (uint32_t i = 0; i < total;) {
    const uint8_t l = len[i];
    if (!l) {
      uint32_t r = 1;
      while (i + r < total && !len[i + r] && r < 138) r++;
      if (r >= 11) syms.push_back({18, r - 11, 7});
      else if (r >= 3) syms.push_back({17, r - 3, 3});
      else for (uint32_t k = 0; k < r; k++) syms.push_back({0, 0, 0});
      i += r;
    } else {
      syms.push_back({l, 0, 0});
      i++;
      uint32_t r = 0;
      while (i + r < total && len[i + r] == l && r < 70) r++;
      if (r >= 7) { syms.push_back({20, r - 7, 6}); i += r; }
      else if (r >= 3) { syms.push_back({19, r - 3, 2}); i += r; }
    }
  }
  std::vector<uint32_t> cf(21, 0);
  for (const Sym& s : syms) cf[s.s]++;
  Huff cl;
  cl.build(cf, 7);
  int ncl = 21;
  while (ncl > 1 && !cl.len[kOrder[ncl - 1]]) ncl--;
  bw.put((uint32_t)ncl, 5);
  for (int i = 0; i < ncl; i++) bw.put(cl.len[kOrder[i]], 3);
  for (const Sym& s : syms) {
    cl.put(bw, s.s);
    if (s.bits) bw.put(s.extra, (uint32_t)s.bits);
  }
}

// histogram with at least one used symbol (a model the format requires must not be empty)
void ensure_used(std::vector<uint32_t>& f) {
  for (uint32_t v : f)
    if (v) return;
  if (!f.empty()) f[0] = 1;
}

void put_be(std::vector<uint8_t>& d, size_t at, uint32_t v, int bytes) {
  for (int i = bytes - 1; i >= 0; i--) d[at + (size_t)(bytes - 1 - i)] = (uint8_t)(v >> (8 * i));
}

// Distinct values in first-use order, found through an open-addressing table (multiplicative
// hash, linear probing, at most half full).
struct Palette {
  std::vector<uint64_t> values;
  std::vector<uint64_t> keys;
  std::vector<uint32_t> slot;  // index into values + 1; 0 = empty
  uint32_t shift = 64;
  static size_t hash(uint64_t v, uint32_t shift) { return (size_t)((v * 0x9E3779B97F4A7C15ull) >> shift); }
  void grow() {
    const size_t size = slot.empty() ? 1024 : 2 * slot.size();
    shift = 64;
    for (size_t k = size; k > 1; k >>= 1) shift--;
    keys.assign(size, 0);
    slot.assign(size, 0);
    for (size_t i = 0; i < values.size(); i++) {
      size_t h = hash(values[i], shift);
      while (slot[h]) h = (h + 1) & (size - 1);
      keys[h] = values[i];
      slot[h] = (uint32_t)i + 1;
    }
  }
  uint64_t last_value = 0;
  uint32_t last_index = UINT32_MAX;  // the previous add's result: neighbouring blocks often repeat
  uint32_t add(uint64_t v) {
    if (last_index != UINT32_MAX && v == last_value) return last_index;
    last_value = v;
    return last_index = insert(v);
  }
  uint32_t insert(uint64_t v) {
    if (2 * (values.size() + 1) > slot.size()) grow();
    const size_t mask = slot.size() - 1;
    size_t h = hash(v, shift);
    for (; slot[h]; h = (h + 1) & mask)
      if (keys[h] == v) return slot[h] - 1;
    keys[h] = v;
    slot[h] = (uint32_t)values.size() + 1;
    values.push_back(v);
    return (uint32_t)values.size() - 1;
  }
};

// DXT order -> linear order selectors (g_dxt1_to_linear, g_dxt5_to_linear, crnlib/crn_dxt.cpp:35-39),
// four selectors per table lookup
struct SelectorTables {
  uint8_t d1[256];
  uint16_t d5[4096];
  SelectorTables() {
    static const uint8_t t1[4] = {0, 3, 1, 2}, t5[8] = {0, 7, 1, 2, 3, 4, 5, 6};
    for (uint32_t x = 0; x < 256; x++) {
      uint32_t v = 0;
      for (int p = 0; p < 4; p++) v |= (uint32_t)t1[(x >> (2 * p)) & 3] << (2 * p);
      d1[x] = (uint8_t)v;
    }
    for (uint32_t x = 0; x < 4096; x++) {
      uint32_t v = 0;
      for (int p = 0; p < 4; p++) v |= (uint32_t)t5[(x >> (3 * p)) & 7] << (3 * p);
      d5[x] = (uint16_t)v;
    }
  }
};
const SelectorTables kSelectorTables;
uint32_t dxt1_sel_to_linear(uint32_t dxt) {
  const uint8_t* t = kSelectorTables.d1;
  return (uint32_t)t[dxt & 255] | ((uint32_t)t[(dxt >> 8) & 255] << 8) | ((uint32_t)t[(dxt >> 16) & 255] << 16) |
         ((uint32_t)t[dxt >> 24] << 24);
}
uint64_t dxt5_sel_to_linear(uint64_t dxt) {
  const uint16_t* t = kSelectorTables.d5;
  return (uint64_t)t[dxt & 4095] | ((uint64_t)t[(dxt >> 12) & 4095] << 12) | ((uint64_t)t[(dxt >> 24) & 4095] << 24) |
         ((uint64_t)t[(dxt >> 36) & 4095] << 36);
}

// ---- palettes (crn_comp::pack_color_endpoints / pack_color_selectors / pack_alpha_endpoints /
// pack_alpha_selectors; the inverse of crn_unpacker::decode_palettes, inc/crn_decomp.h:3715-3851).
// Each codes its symbols twice: a histogram pass, then the Huffman-coded pass behind its model.

// colour endpoints: six running component deltas, a 5-bit model for red/blue, 6-bit for green
std::vector<uint8_t> pack_colour_endpoints(const std::vector<uint64_t>& values) {
  std::vector<uint32_t> f5(32, 0), f6(64, 0);
  static const uint32_t kMask[6] = {31, 63, 31, 31, 63, 31};
  static const int kModel[6] = {0, 1, 0, 0, 1, 0};
  static const int kShift[6] = {11, 5, 0, 27, 21, 16};
  std::vector<uint8_t> outb;
  for (int pass = 0; pass < 2; pass++) {
    Huff h5, h6;
    BitWriter bw;
    if (pass) {
      ensure_used(f5); ensure_used(f6);
      h5.build(f5, 16); h6.build(f6, 16);
      send_model(bw, h5);
      send_model(bw, h6);
    }
    uint32_t prev[6] = {0, 0, 0, 0, 0, 0};
    for (uint64_t v : values)
      for (int k = 0; k < 6; k++) {
        const uint32_t c = ((uint32_t)v >> kShift[k]) & kMask[k];
        const uint32_t d = (c - prev[k]) & kMask[k];
        prev[k] = c;
        if (pass) (kModel[k] ? h6 : h5).put(bw, d);
        else (kModel[k] ? f6 : f5)[d]++;
      }
    if (pass) outb = bw.finish();
  }
  return outb;
}

// colour selectors: XOR deltas of the linear words, 4 bits at a time
std::vector<uint8_t> pack_colour_selectors(const std::vector<uint64_t>& values) {
  std::vector<uint32_t> fs(16, 0);
  std::vector<uint8_t> outb;
  for (int pass = 0; pass < 2; pass++) {
    Huff hs;
    BitWriter bw;
    if (pass) { ensure_used(fs); hs.build(fs, 16); send_model(bw, hs); }
    uint32_t prev = 0;
    for (uint64_t v : values) {
      const uint32_t d = (uint32_t)v ^ prev;
      prev = (uint32_t)v;
      for (int j = 0; j < 32; j += 4) {
        const uint32_t x = (d >> j) & 15u;
        if (pass) hs.put(bw, x); else fs[x]++;
      }
    }
    if (pass) outb = bw.finish();
  }
  return outb;
}

// alpha endpoints: two running 8-bit deltas
std::vector<uint8_t> pack_alpha_endpoints(const std::vector<uint64_t>& values) {
  std::vector<uint32_t> fa(256, 0);
  std::vector<uint8_t> outb;
  for (int pass = 0; pass < 2; pass++) {
    Huff ha;
    BitWriter bw;
    if (pass) { ensure_used(fa); ha.build(fa, 16); send_model(bw, ha); }
    uint32_t pa = 0, pb = 0;
    for (uint64_t v : values) {
      const uint32_t a = (uint32_t)v & 255u, b = (uint32_t)(v >> 8) & 255u;
      const uint32_t d0 = (a - pa) & 255u, d1 = (b - pb) & 255u;
      pa = a; pb = b;
      if (pass) { ha.put(bw, d0); ha.put(bw, d1); } else { fa[d0]++; fa[d1]++; }
    }
    if (pass) outb = bw.finish();
  }
  return outb;
}

// alpha selectors: XOR deltas of the two 24-bit linear halves, 6 bits at a time
std::vector<uint8_t> pack_alpha_selectors(const std::vector<uint64_t>& values) {
  std::vector<uint32_t> fs(64, 0);
  std::vector<uint8_t> outb;
  for (int pass = 0; pass < 2; pass++) {
    Huff hs;
    BitWriter bw;
    if (pass) { ensure_used(fs); hs.build(fs, 16); send_model(bw, hs); }
    uint32_t prev[2] = {0, 0};
    for (uint64_t v : values)
      for (int h = 0; h < 2; h++) {
        const uint32_t half = (uint32_t)(v >> (24 * h)) & 0xFFFFFFu;
        const uint32_t d = half ^ prev[h];
        prev[h] = half;
        for (int j = 0; j < 24; j += 6) {
          const uint32_t x = (d >> j) & 63u;
          if (pass) hs.put(bw, x); else fs[x]++;
        }
      }
    if (pass) outb = bw.finish();
  }
  return outb;
}

// ---- palette ordering ----

// Estimated coded size of an XOR delta between two linear selector words (optimize_color_selectors
// and optimize_alpha_selectors, crnlib/crn_comp.cpp:921-975, 1236-1282): a per-field cost of the
// XOR of corresponding 2-bit (colour) or 3-bit (alpha) selectors, costs {0, 5, 14, 10} and
// {0, 2, 3, 3, 5, 5, 4, 4}.
// Colour: the 2-bit fields of the XOR, even and odd ones in separate nibbles, each nibble's cost
// 5 b0 + 14 b1 - 9 b0 b1 (exact in modular arithmetic: every nibble ends in 0..14), then the
// nibbles summed as bytes; plain integer operations, so the chain's scans vectorise.
inline uint32_t colour_selector_cost(uint32_t a, uint32_t b) {
  const uint32_t x = a ^ b;
  const uint32_t e = x & 0x33333333u, o = (x >> 2) & 0x33333333u;
  const uint32_t e0 = e & 0x11111111u, e1 = (e >> 1) & 0x11111111u;
  const uint32_t o0 = o & 0x11111111u, o1 = (o >> 1) & 0x11111111u;
  const uint32_t ce = 5u * e0 + 14u * e1 - 9u * (e0 & e1), co = 5u * o0 + 14u * o1 - 9u * (o0 & o1);
  const uint32_t bytes = (ce & 0x0F0F0F0Fu) + ((ce >> 4) & 0x0F0F0F0Fu) + (co & 0x0F0F0F0Fu) + ((co >> 4) & 0x0F0F0F0Fu);
  return (bytes * 0x01010101u) >> 24;
}
// the XOR-delta cost of four 3-bit selectors at once, {0, 2, 3, 3, 5, 5, 4, 4} per selector
struct AlphaCost4 {
  uint8_t t[4096];
  AlphaCost4() {
    static const uint8_t kCost[8] = {0, 2, 3, 3, 5, 5, 4, 4};
    for (uint32_t x = 0; x < 4096; x++) t[x] = (uint8_t)(kCost[x & 7] + kCost[(x >> 3) & 7] + kCost[(x >> 6) & 7] + kCost[x >> 9]);
  }
};
inline uint32_t alpha_selector_cost(uint64_t a, uint64_t b) {
  static const AlphaCost4 tab;
  const uint64_t x = a ^ b;
  return (uint32_t)tab.t[x & 4095] + tab.t[(x >> 12) & 4095] + tab.t[(x >> 24) & 4095] + tab.t[(x >> 36) & 4095];
}

// Nearest-neighbour chain over payload values: starting from the entry with the smallest
// start_cost (its distance from an all-zero entry), repeatedly take the remaining entry closest
// (cost) to the last one taken (sort_color_endpoints / sort_alpha_endpoints / the selector
// sorts). Returns each entry's rank. `floor` is the least cost two distinct entries can have: a
// scan that meets it has found its first minimum and stops there. Costs are computed a tile at a
// time into a buffer (a loop the compiler vectorises), then the tile is searched.
template <class T, class Start, class Cost>
std::vector<uint32_t> nearest_chain(const std::vector<T>& payload, Start start_cost, Cost cost, uint32_t floor) {
  // the remaining entries' ids and payloads are kept dense, in the order a swap-with-last removal
  // leaves them, so the scan (and its first-minimum tie-break) visits them in that order
  constexpr uint32_t kTile = 256;
  const uint32_t n = (uint32_t)payload.size();
  std::vector<uint32_t> rank(n), id(n);
  std::vector<T> val(payload);
  for (uint32_t i = 0; i < n; i++) id[i] = i;
  uint32_t c[kTile];
  T cur{};
  for (uint32_t left = n; left; left--) {
    uint32_t best = 0, best_cost = UINT32_MAX;
    const uint32_t stop = left == n ? 0u : floor;
    for (uint32_t t0 = 0; t0 < left && best_cost > stop; t0 += kTile) {
      const uint32_t m = std::min(kTile, left - t0);
      const T* v = val.data() + t0;
      if (left == n) {
        for (uint32_t i = 0; i < m; i++) c[i] = start_cost(v[i]);
      } else {
        for (uint32_t i = 0; i < m; i++) c[i] = cost(v[i], cur);
      }
      uint32_t tmin = UINT32_MAX;
      for (uint32_t i = 0; i < m; i++) tmin = std::min(tmin, c[i]);
      if (tmin < best_cost) {
        uint32_t i = 0;
        while (c[i] != tmin) i++;
        best_cost = tmin;
        best = t0 + i;
      }
    }
    cur = val[best];
    rank[id[best]] = n - left;
    id[best] = id[left - 1];
    val[best] = val[left - 1];
  }
  return rank;
}

// An endpoint as 8-bit components: (r, g, b) of both colour endpoints, or the two alphas.
struct Comps {
  int32_t c[6];
};

// nearest_chain over endpoints, the cost the squared distance of the six components (the start
// cost: the distance from the all-zero entry), with the components in one array each so that the
// distance loop vectorises; the same scan order, first-minimum tie-break and stop at `floor`.
std::vector<uint32_t> nearest_chain_comps(const std::vector<Comps>& u, uint32_t floor) {
  constexpr uint32_t kTile = 256;
  const uint32_t n = (uint32_t)u.size();
  std::vector<uint32_t> rank(n), id(n);
  std::vector<int32_t> cc[6];
  for (int k = 0; k < 6; k++) cc[k].resize(n);
  for (uint32_t i = 0; i < n; i++) {
    id[i] = i;
    for (int k = 0; k < 6; k++) cc[k][i] = u[i].c[k];
  }
  uint32_t c[kTile];
  int32_t cur[6] = {0, 0, 0, 0, 0, 0};
  for (uint32_t left = n; left; left--) {
    uint32_t best = 0, best_cost = UINT32_MAX;
    const uint32_t stop = left == n ? 0u : floor;
    for (uint32_t t0 = 0; t0 < left && best_cost > stop; t0 += kTile) {
      const uint32_t m = std::min(kTile, left - t0);
      const int32_t *c0 = cc[0].data() + t0, *c1 = cc[1].data() + t0, *c2 = cc[2].data() + t0,
                    *c3 = cc[3].data() + t0, *c4 = cc[4].data() + t0, *c5 = cc[5].data() + t0;
      for (uint32_t i = 0; i < m; i++) {
        const int32_t d0 = c0[i] - cur[0], d1 = c1[i] - cur[1], d2 = c2[i] - cur[2], d3 = c3[i] - cur[3],
                      d4 = c4[i] - cur[4], d5 = c5[i] - cur[5];
        c[i] = (uint32_t)(d0 * d0 + d1 * d1 + d2 * d2 + d3 * d3 + d4 * d4 + d5 * d5);
      }
      uint32_t tmin = UINT32_MAX;
      for (uint32_t i = 0; i < m; i++) tmin = std::min(tmin, c[i]);
      if (tmin < best_cost) {
        uint32_t i = 0;
        while (c[i] != tmin) i++;
        best_cost = tmin;
        best = t0 + i;
      }
    }
    for (int k = 0; k < 6; k++) {
      cur[k] = cc[k][best];
      cc[k][best] = cc[k][left - 1];
    }
    rank[id[best]] = n - left;
    id[best] = id[left - 1];
  }
  return rank;
}

// Symmetric counts of consecutive endpoint indices in the coded stream, as compressed rows.
struct Adjacency {
  std::vector<uint32_t> start, nb, count;
  std::vector<uint32_t> total;  // per entry: sum of its row
};

// Two-ended chain grown from `first` (remap_color_endpoints / remap_alpha_endpoints,
// crnlib/crn_comp.cpp:800-873, 1094-1158). Each remaining entry carries its accumulated
// co-occurrence with the entries taken so far and its similarity (base - min(cap, distance)) to
// the two ends of the chain; the entry with the largest max(similarity) * (co-occurrence +
// normaliser) is taken next, and joins the end whose half of the chain it co-occurs with more
// (weighted toward the ends). The normaliser is the taken entry's co-occurrence << shift.
std::vector<uint32_t> grow_chain(const std::vector<Comps>& u, const Adjacency& adj, uint32_t first, uint32_t base,
                                 uint32_t cap, int shift) {
  // per remaining entry (dense slots, swap-with-last removal): id, accumulated co-occurrence,
  // similarity to the front and to the back of the chain, components
  const uint32_t n = (uint32_t)u.size();
  std::vector<uint32_t> id, freq, slot_of(n, UINT32_MAX), pos(n, UINT32_MAX), chain(2 * n + 1);
  std::vector<uint16_t> sim_f, sim_b;
  std::vector<int16_t> cc[6];  // components, one array each, so the distance loops vectorise
  id.reserve(n);
  for (uint32_t i = 0; i < n; i++)
    if (i != first) {
      id.push_back(i);
      for (int k = 0; k < 6; k++) cc[k].push_back((int16_t)u[i].c[k]);
    }
  freq.assign(id.size(), 0);
  sim_f.assign(id.size(), 0);
  sim_b.assign(id.size(), 0);
  uint32_t lo = n, hi = n;
  chain[n] = first;
  pos[first] = n;
  // a taken entry's co-occurrences join the accumulated counts of the entries still remaining
  for (uint32_t i = 0; i < (uint32_t)id.size(); i++) slot_of[id[i]] = i;
  auto take_row = [&](uint32_t s) {
    for (uint32_t k = adj.start[s]; k < adj.start[s + 1]; k++) {
      const uint32_t sl = slot_of[adj.nb[k]];
      if (sl != UINT32_MAX) freq[sl] += adj.count[k];
    }
  };
  take_row(first);
  Comps front = u[first], back = u[first];
  bool front_new = true, back_new = true;
  uint64_t normaliser = 0;
  // similarity of every remaining entry to a new chain end, base - min(distance, cap), in 16-bit
  // lanes: a squared component difference (<= 255^2) is clamped to cap before the sum, so the sum
  // (<= 6 cap) cannot wrap and its minimum with cap is min(distance, cap). Needs cap <= 10922 and
  // base <= 65535 (the callers' units are 4000 and 1000, base at most 1.5 units).
  const uint16_t cap16 = (uint16_t)cap, base16 = (uint16_t)base;
  auto similarity = [&](const Comps& end, uint16_t* sim, size_t m) {
    const int16_t e0 = (int16_t)end.c[0], e1 = (int16_t)end.c[1], e2 = (int16_t)end.c[2], e3 = (int16_t)end.c[3],
                  e4 = (int16_t)end.c[4], e5 = (int16_t)end.c[5];
    const int16_t *c0 = cc[0].data(), *c1 = cc[1].data(), *c2 = cc[2].data(), *c3 = cc[3].data(), *c4 = cc[4].data(),
                  *c5 = cc[5].data();
    auto sq = [cap16](int16_t a, int16_t b) -> uint16_t {
      const uint16_t x = (uint16_t)(a - b);
      const uint16_t q = (uint16_t)((uint32_t)x * x);  // the square modulo 2^16: exact, at most 255^2
      return q < cap16 ? q : cap16;
    };
    for (size_t i = 0; i < m; i++) {
      const uint16_t d = (uint16_t)(sq(c0[i], e0) + sq(c1[i], e1) + sq(c2[i], e2) + sq(c3[i], e3) + sq(c4[i], e4) +
                                    sq(c5[i], e5));
      sim[i] = (uint16_t)(base16 - (d < cap16 ? d : cap16));
    }
  };
  while (!id.empty()) {
    const size_t m = id.size();
    if (front_new) similarity(front, sim_f.data(), m);
    if (back_new) similarity(back, sim_b.data(), m);
    // the best entry: the highest score, the lowest id among equal scores, found as the largest key
    // score << 13 | (8191 - id) in one pass the compiler vectorises. A score is below 2^46: a
    // similarity below 2^16 times a co-occurrence count plus normaliser below 2^30 (at most two
    // co-occurrences per block and component, at most 2^23 blocks of 3 components, a normaliser of
    // at most 8 counts); ids are below kMaxSyms = 2^13.
    const uint32_t norm = (uint32_t)normaliser;
    uint64_t top = 0;
    for (size_t i = 0; i < m; i++) {
      const uint64_t score = (uint64_t)std::max(sim_f[i], sim_b[i]) * (uint32_t)(freq[i] + norm) + 1;
      top = std::max(top, (score << 13) | (uint64_t)(8191u - id[i]));
    }
    const uint32_t s = 8191u - (uint32_t)(top & 8191u);
    const size_t best = slot_of[s];
    const uint32_t sf = sim_f[best], sb = sim_b[best], fs = freq[best];
    // co-occurrence of s with each half of the chain, weighted (L-1-2k) by distance k from that end
    const int64_t L = (int64_t)hi - lo + 1;
    uint64_t w_front = 0, w_back = 0;
    for (uint32_t k = adj.start[s]; k < adj.start[s + 1]; k++) {
      const uint32_t p = pos[adj.nb[k]];
      if (p == UINT32_MAX) continue;
      const int64_t wf = L - 1 - 2 * ((int64_t)p - lo), wb = L - 1 - 2 * ((int64_t)hi - p);
      if (wf > 0) w_front += (uint64_t)wf * adj.count[k];
      if (wb > 0) w_back += (uint64_t)wb * adj.count[k];
    }
    normaliser = (uint64_t)fs << shift;
    if ((uint64_t)sf * w_front > (uint64_t)sb * w_back) {
      chain[--lo] = s; pos[s] = lo; front = u[s]; front_new = true; back_new = false;
    } else {
      chain[++hi] = s; pos[s] = hi; back = u[s]; back_new = true; front_new = false;
    }
    id[best] = id.back(); id.pop_back();
    for (int k = 0; k < 6; k++) { cc[k][best] = cc[k].back(); cc[k].pop_back(); }
    freq[best] = freq[m - 1]; freq.pop_back();
    sim_f[best] = sim_f[m - 1]; sim_f.pop_back();
    sim_b[best] = sim_b[m - 1]; sim_b.pop_back();
    slot_of[s] = UINT32_MAX;
    if (best < id.size()) slot_of[id[best]] = (uint32_t)best;
    take_row(s);
  }
  std::vector<uint32_t> rank(n);
  for (uint32_t p = lo; p <= hi; p++) rank[chain[p]] = p - lo;
  return rank;
}

template <class T>
std::vector<T> permuted(const std::vector<T>& v, const std::vector<uint32_t>& rank) {
  std::vector<T> out(v.size());
  for (size_t i = 0; i < v.size(); i++) out[rank[i]] = v[i];
  return out;
}

}  // namespace
}  // namespace crngpu

using namespace crngpu;

extern "C" int64_t crngpu_crn_pack(const uint8_t* blocks, uint32_t width, uint32_t height, uint32_t levels,
                                   uint32_t faces, uint32_t format, void* out, uint64_t out_capacity) try {
  clear_error();
  if (!blocks || !width || !height || width > 4096 || height > 4096 || !levels || levels > 16 ||
      (faces != 1 && faces != 6)) {
    set_error("crngpu_crn_pack: bad dimensions, level or face count");
    return CRNGPU_E_PARAM;
  }
  int nalpha;
  bool colour;
  uint32_t bpb;
  switch (format) {
    case CRNGPU_FMT_DXT1: colour = true; nalpha = 0; bpb = 8; break;
    case CRNGPU_FMT_DXT5: case CRNGPU_FMT_DXT5_CCXY: case CRNGPU_FMT_DXT5_XGXR: case CRNGPU_FMT_DXT5_XGBR:
    case CRNGPU_FMT_DXT5_AGBR: colour = true; nalpha = 1; bpb = 16; break;
    case CRNGPU_FMT_DXN_XY: case CRNGPU_FMT_DXN_YX: colour = false; nalpha = 2; bpb = 16; break;
    case CRNGPU_FMT_DXT5A: colour = false; nalpha = 1; bpb = 8; break;
    default: set_error("crngpu_crn_pack: unsupported format"); return CRNGPU_E_UNSUPPORTED;
  }
  if (levels > 1) {
    uint32_t full = 1;
    while ((width >> full) || (height >> full)) full++;
    if (levels > full) { set_error("crngpu_crn_pack: more levels than the mip chain has"); return CRNGPU_E_PARAM; }
  }
  // level geometry (crn_comp::alias_images, crnlib/crn_comp.cpp:454-463)
  struct Lv { uint32_t W, H, first; };
  std::vector<Lv> lv(levels);
  uint64_t nblocks = 0;
  for (uint32_t l = 0; l < levels; l++) {
    const uint32_t w = std::max(1u, width >> l), h = std::max(1u, height >> l);
    lv[l] = Lv{((w + 7) & ~7u) >> 2, ((h + 7) & ~7u) >> 2, (uint32_t)nblocks};
    nblocks += (uint64_t)lv[l].W * lv[l].H * faces;
  }
  // endpoint / selector palette indices of each component (colour, alpha0, alpha1), component
  // after component
  Palette cep, csel, aep, asel;
  const int ncomp = (colour ? 1 : 0) + nalpha;
  std::vector<uint32_t> eidx((size_t)nblocks * ncomp), sidx((size_t)nblocks * ncomp);
  // the four palettes are independent (each in its own first-use order): one thread each on large
  // inputs
  auto colour_endpoints = [&] {
    for (uint64_t b = 0; b < nblocks; b++) {
      uint32_t ep;
      std::memcpy(&ep, blocks + b * bpb + (bpb == 16 ? 8 : 0), 4);
      eidx[b] = cep.add(ep);
    }
  };
  auto colour_selectors = [&] {
    for (uint64_t b = 0; b < nblocks; b++) {
      uint32_t sel;
      std::memcpy(&sel, blocks + b * bpb + (bpb == 16 ? 8 : 0) + 4, 4);
      sidx[b] = csel.add(dxt1_sel_to_linear(sel));
    }
  };
  const int c_alpha = colour ? 1 : 0;
  auto alpha_endpoints = [&] {
    for (uint64_t b = 0; b < nblocks; b++)
      for (int a = 0; a < nalpha; a++) {
        const uint8_t* ab = blocks + b * bpb + 8 * a;
        eidx[(size_t)(c_alpha + a) * nblocks + b] = aep.add((uint64_t)ab[0] | ((uint64_t)ab[1] << 8));
      }
  };
  auto alpha_selectors = [&] {
    for (uint64_t b = 0; b < nblocks; b++)
      for (int a = 0; a < nalpha; a++) {
        const uint8_t* ab = blocks + b * bpb + 8 * a;
        uint64_t sel = 0;
        for (int k = 0; k < 6; k++) sel |= (uint64_t)ab[2 + k] << (8 * k);
        sidx[(size_t)(c_alpha + a) * nblocks + b] = asel.add(dxt5_sel_to_linear(sel));
      }
  };
  {
    std::vector<std::function<void()>> jobs;
    if (colour) { jobs.emplace_back(colour_endpoints); jobs.emplace_back(colour_selectors); }
    if (nalpha) { jobs.emplace_back(alpha_endpoints); jobs.emplace_back(alpha_selectors); }
    parallel_jobs(jobs.size(), pack_threads(nblocks), [&](size_t j, unsigned) { jobs[j](); });
  }
  if (cep.values.size() > (size_t)kMaxSyms || csel.values.size() > (size_t)kMaxSyms ||
      aep.values.size() > (size_t)kMaxSyms || asel.values.size() > (size_t)kMaxSyms) {
    set_error("crngpu_crn_pack: more than 8192 distinct endpoints or selectors (cluster the blocks first)");
    return CRNGPU_E_PARAM;
  }
  // references of every block (crn_comp::pack_blocks, crnlib/crn_comp.cpp:295-422): 0 new (an
  // endpoint delta per component), 1 same endpoints as the previous block in decode order, 2 same
  // as the block above (the faces of a level are one tall image to the decoder's row buffer)
  std::vector<uint8_t> ref(nblocks, 0);
  // the block streams' work units: runs of whole row pairs (a reference group covers two rows; a
  // level's faces are one tall image, each face an even number of rows)
  struct RowRun {
    uint32_t level, row0, row1;
  };
  std::vector<RowRun> runs;
  for (uint32_t l = 0; l < levels; l++) {
    const uint32_t rows = faces * lv[l].H, step = std::max(2u, (16384u / lv[l].W) & ~1u);
    for (uint32_t r = 0; r < rows; r += step) runs.push_back(RowRun{l, r, std::min(rows, r + step)});
  }
  const unsigned threads = pack_threads(nblocks);
  // the per-block passes only pay for their threads on large inputs (a 2048 x 2048 mip chain)
  const unsigned block_threads = nblocks >= (1u << 18) ? threads : 1u;
  parallel_jobs(runs.size(), block_threads, [&](size_t j, unsigned) {
    const Lv& L = lv[runs[j].level];
    for (uint32_t row = runs[j].row0; row < runs[j].row1; row++)
      for (uint32_t x = 0; x < L.W; x++) {
        const uint64_t b = L.first + (uint64_t)row * L.W + x;
        bool left = row || x, top = row != 0;
        for (int c = 0; c < ncomp; c++) {
          const uint32_t e = eidx[(size_t)c * nblocks + b];
          if (left) left = e == eidx[(size_t)c * nblocks + b - 1];
          if (top) top = e == eidx[(size_t)c * nblocks + b - L.W];
        }
        ref[b] = left ? 1 : top ? 2 : 0;
      }
  });
  // palette order. Model 0 = colour (component 0 when present), model 1 = alpha (the rest).
  const int comp_lo[2] = {0, colour ? 1 : 0}, comp_hi[2] = {colour ? 1 : 0, ncomp};
  Palette* ep_pal[2] = {&cep, &aep};
  Palette* sel_pal[2] = {&csel, &asel};
  std::vector<uint32_t> ep_rank[2], sel_rank[2];
  {
    std::vector<std::function<void()>> workers;  // per model: the selector order, the endpoint order
    // the endpoint trials of model m: coded size of the palette plus the index deltas
    auto stream_bits = [&](int m, const std::vector<uint32_t>& rank) -> uint64_t {
      const uint32_t n = (uint32_t)rank.size();
      std::vector<uint32_t> h(n, 0);
      for (uint32_t l = 0; l < levels; l++) {
        uint32_t prev[3] = {0, 0, 0};
        const uint64_t end = lv[l].first + (uint64_t)lv[l].W * lv[l].H * faces;
        for (uint64_t b = lv[l].first; b < end; b++)
          for (int c = comp_lo[m]; c < comp_hi[m]; c++) {
            const uint32_t e = rank[eidx[(size_t)c * nblocks + b]];
            if (!ref[b]) h[e >= prev[c] ? e - prev[c] : e + n - prev[c]]++;
            prev[c] = e;
          }
      }
      ensure_used(h);
      Huff hf;
      hf.build(h, 16);
      uint64_t bits = 0;
      for (uint32_t k = 0; k < n; k++) bits += (uint64_t)h[k] * hf.len[k];
      BitWriter bw;
      send_model(bw, hf);
      const std::vector<uint64_t> vals = permuted(ep_pal[m]->values, rank);
      return bits + bw.bits() + 8 * (m ? pack_alpha_endpoints(vals) : pack_colour_endpoints(vals)).size();
    };
    for (int m = 0; m < 2; m++) {
      if (comp_lo[m] == comp_hi[m]) continue;
      const uint32_t n = (uint32_t)ep_pal[m]->values.size();
      // selectors: nearest-neighbour chain under the XOR-delta cost
      workers.emplace_back([&, m] {
        const std::vector<uint64_t>& v = sel_pal[m]->values;
        // least cost between distinct words: one selector off by one (5 colour, 2 alpha)
        if (m) {
          sel_rank[m] = nearest_chain(v, [](uint64_t a) { return alpha_selector_cost(a, 0); },
                                      [](uint64_t a, uint64_t b) { return alpha_selector_cost(a, b); }, 2u);
        } else {
          const std::vector<uint32_t> v32(v.begin(), v.end());
          sel_rank[m] = nearest_chain(v32, [](uint32_t a) { return colour_selector_cost(a, 0u); },
                                      [](uint32_t a, uint32_t b) { return colour_selector_cost(a, b); }, 5u);
        }
      });
      workers.emplace_back([&, m, n] {
        // endpoints, unpacked to 8-bit components: colour (r, g, b) of both endpoints, or the two alphas
        std::vector<Comps> u(n);
        for (uint32_t i = 0; i < n; i++) {
          const uint32_t v = (uint32_t)ep_pal[m]->values[i];
          int32_t* c = u[i].c;
          if (m) { c[0] = (int32_t)(v & 255u); c[1] = (int32_t)((v >> 8) & 255u); c[2] = c[3] = c[4] = c[5] = 0; continue; }
          for (int e = 0; e < 2; e++) {
            const uint32_t q = v >> (16 * e), r = (q >> 11) & 31, g = (q >> 5) & 63, bl = q & 31;
            c[3 * e + 0] = (int32_t)((r << 3) | (r >> 2));
            c[3 * e + 1] = (int32_t)((g << 2) | (g >> 4));
            c[3 * e + 2] = (int32_t)((bl << 3) | (bl >> 2));
          }
        }
        // co-occurrence of consecutive endpoints in the delta-coded blocks, both directions, as
        // (entry << 13 | neighbour) keys (indices < kMaxSyms = 2^13), sorted by two stable
        // counting passes over the 13-bit digits and run-length counted into rows
        static_assert(kMaxSyms <= (1 << 13), "pair keys hold two 13-bit indices");
        std::vector<uint32_t> pairs;
        for (uint32_t l = 0; l < levels; l++) {
          uint32_t prev[3] = {0, 0, 0};
          const uint64_t end = lv[l].first + (uint64_t)lv[l].W * lv[l].H * faces;
          for (uint64_t b = lv[l].first; b < end; b++)
            for (int c = comp_lo[m]; c < comp_hi[m]; c++) {
              const uint32_t e = eidx[(size_t)c * nblocks + b];
              if (!ref[b] && e != prev[c]) {
                pairs.push_back((e << 13) | prev[c]);
                pairs.push_back((prev[c] << 13) | e);
              }
              prev[c] = e;
            }
        }
        {
          std::vector<uint32_t> sorted(pairs.size()), cnt(8193);
          for (int shift = 0; shift <= 13; shift += 13) {
            std::fill(cnt.begin(), cnt.end(), 0u);
            for (uint32_t k : pairs) cnt[((k >> shift) & 8191u) + 1]++;
            for (int i = 0; i < 8192; i++) cnt[i + 1] += cnt[i];
            for (uint32_t k : pairs) sorted[cnt[(k >> shift) & 8191u]++] = k;
            pairs.swap(sorted);
          }
        }
        Adjacency adj;
        adj.start.assign(n + 1, 0);
        adj.total.assign(n, 0);
        for (size_t k = 0; k < pairs.size();) {
          size_t r = k + 1;
          while (r < pairs.size() && pairs[r] == pairs[k]) r++;
          const uint32_t i = pairs[k] >> 13;
          adj.nb.push_back(pairs[k] & 8191u);
          adj.count.push_back((uint32_t)(r - k));
          adj.start[i + 1]++;
          adj.total[i] += (uint32_t)(r - k);
          k = r;
        }
        for (uint32_t i = 0; i < n; i++) adj.start[i + 1] += adj.start[i];
        uint32_t first = 0;
        for (uint32_t i = 0; i < n; i++)
          if (adj.total[i] > adj.total[first]) first = i;
        // four trials, run side by side: the nearest-neighbour chain and three grown chains
        const uint32_t unit = m ? 1000u : 4000u;
        const float weights[3] = {0.0f, 1.0f / 6.0f, 0.5f};
        std::vector<uint32_t> trial[4];
        uint64_t bits[4];
        static_assert(4000u * 3 / 2 <= 65535u && 4000u <= 10922u, "grow_chain's 16-bit similarity");
        parallel_jobs(4, threads, [&](size_t t, unsigned) {
          if (t == 0) {
            // least distance between distinct endpoints: one 6-bit green step (4^2) or one alpha step
            trial[0] = nearest_chain_comps(u, m ? 1u : 16u);
          } else {
            trial[t] = grow_chain(u, adj, first, (uint32_t)((float)unit * (1.0f + weights[t - 1])), unit, m ? 0 : 3);
          }
          bits[t] = stream_bits(m, trial[t]);
        });
        int best = 0;
        for (int t = 1; t < 4; t++)
          if (bits[t] < bits[best]) best = t;
        ep_rank[m] = std::move(trial[best]);
      });
    }
    parallel_jobs(workers.size(), threads, [&](size_t j, unsigned) { workers[j](); });
  }
  for (int m = 0; m < 2; m++) {
    if (comp_lo[m] == comp_hi[m]) continue;
    ep_pal[m]->values = permuted(ep_pal[m]->values, ep_rank[m]);
    sel_pal[m]->values = permuted(sel_pal[m]->values, sel_rank[m]);
    for (uint64_t b = 0; b < nblocks; b++)
      for (int c = comp_lo[m]; c < comp_hi[m]; c++) {
        eidx[(size_t)c * nblocks + b] = ep_rank[m][eidx[(size_t)c * nblocks + b]];
        sidx[(size_t)c * nblocks + b] = sel_rank[m][sidx[(size_t)c * nblocks + b]];
      }
  }
  // block streams: each run of rows records its symbols (model << 16 | symbol) and counts them;
  // then every run is coded behind the finished models and a level's runs are joined. Models:
  // 0 reference groups, 1 / 2 colour endpoint deltas / selectors, 3 / 4 alpha endpoint deltas /
  // selectors. An endpoint delta is against the previous block of the level in decode order, so a
  // run starts from the indices of the block before it.
  size_t hist_size[5] = {256, 0, 0, 0, 0};
  if (colour) { hist_size[1] = cep.values.size(); hist_size[2] = csel.values.size(); }
  if (nalpha) { hist_size[3] = aep.values.size(); hist_size[4] = asel.values.size(); }
  std::vector<std::vector<uint32_t>> hists((size_t)block_threads * 5);
  for (unsigned w = 0; w < block_threads; w++)
    for (int k = 0; k < 5; k++) hists[(size_t)w * 5 + k].assign(hist_size[k], 0);
  const uint32_t pal_n[2] = {(uint32_t)cep.values.size(), (uint32_t)aep.values.size()};
  std::vector<std::vector<uint32_t>> run_syms(runs.size());
  parallel_jobs(runs.size(), block_threads, [&](size_t j, unsigned w) {
    const RowRun& R = runs[j];
    const Lv& L = lv[R.level];
    std::vector<uint32_t>* hist = &hists[(size_t)w * 5];
    std::vector<uint32_t>& out = run_syms[j];
    out.reserve((size_t)L.W * (R.row1 - R.row0) * (2 * ncomp + 1));
    uint32_t prev[3] = {0, 0, 0};
    const uint64_t start = L.first + (uint64_t)R.row0 * L.W;
    if (R.row0)
      for (int c = 0; c < ncomp; c++) prev[c] = eidx[(size_t)c * nblocks + start - 1];
    for (uint32_t y = R.row0; y < R.row1; y++) {
      const uint64_t row = L.first + (uint64_t)y * L.W;
      for (uint32_t x = 0; x < L.W; x++) {
        const uint64_t b = row + x;
        if (!(y & 1) && !(x & 1)) {
          const uint32_t g = ref[b] | (ref[b + L.W] << 2) | (ref[b + 1] << 4) | (ref[b + L.W + 1] << 6);
          out.push_back(g);
          hist[0][g]++;
        }
        for (int c = 0; c < ncomp; c++) {
          const int m = (colour && c == 0) ? 0 : 1;
          const uint32_t e = eidx[(size_t)c * nblocks + b];
          if (ref[b] == 0) {
            const uint32_t d = e >= prev[c] ? e - prev[c] : e + pal_n[m] - prev[c];
            out.push_back(((uint32_t)(1 + 2 * m) << 16) | d);
            hist[1 + 2 * m][d]++;
          }
          prev[c] = e;
        }
        for (int c = 0; c < ncomp; c++) {
          const int m = (colour && c == 0) ? 0 : 1;
          const uint32_t sel = sidx[(size_t)c * nblocks + b];
          out.push_back(((uint32_t)(2 + 2 * m) << 16) | sel);
          hist[2 + 2 * m][sel]++;
        }
      }
    }
  });
  Huff models[5];
  for (int k = 0; k < 5; k++) {
    if (!hist_size[k]) continue;
    std::vector<uint32_t>& h = hists[k];
    for (unsigned w = 1; w < block_threads; w++)
      for (size_t i = 0; i < h.size(); i++) h[i] += hists[(size_t)w * 5 + k][i];
    ensure_used(h);
    models[k].build(h, 16);
  }
  std::vector<std::vector<uint8_t>> run_code(runs.size());
  std::vector<uint64_t> run_bits(runs.size());
  parallel_jobs(runs.size(), block_threads, [&](size_t j, unsigned) {
    run_code[j] = code_symbols(run_syms[j], models, 5, &run_bits[j]);
    std::vector<uint32_t>().swap(run_syms[j]);
  });
  std::vector<std::vector<uint8_t>> level_data(levels);
  std::vector<uint64_t> level_bits(levels, 0);
  for (size_t j = 0; j < runs.size(); j++)
    append_bits(level_data[runs[j].level], level_bits[runs[j].level], run_code[j], run_bits[j]);
  std::vector<uint8_t> pal[4];
  if (colour) {
    pal[0] = pack_colour_endpoints(cep.values);
    pal[1] = pack_colour_selectors(csel.values);
  }
  if (nalpha) {
    pal[2] = pack_alpha_endpoints(aep.values);
    pal[3] = pack_alpha_selectors(asel.values);
  }
  // the block-stream models (crn_comp::pack_data_models)
  std::vector<uint8_t> tables;
  {
    BitWriter bw;
    send_model(bw, models[0]);
    if (colour) { send_model(bw, models[1]); send_model(bw, models[2]); }
    if (nalpha) { send_model(bw, models[3]); send_model(bw, models[4]); }
    tables = bw.finish();
  }
  if (tables.size() > 0xFFFF) { set_error("crngpu_crn_pack: model tables too large"); return CRNGPU_E_PARAM; }
  // file: header | palettes | tables | levels (crn_comp::create_comp_data, crnlib/crn_comp.cpp:1414-1496)
  const uint32_t header_size = 74 + 4 * (levels - 1);
  std::vector<uint8_t> d(header_size, 0);
  uint32_t pal_ofs[4] = {0, 0, 0, 0};
  for (int p = 0; p < 4; p++) {
    if (pal[p].empty()) continue;
    pal_ofs[p] = (uint32_t)d.size();
    d.insert(d.end(), pal[p].begin(), pal[p].end());
  }
  const uint32_t tables_ofs = (uint32_t)d.size();
  d.insert(d.end(), tables.begin(), tables.end());
  std::vector<uint32_t> level_ofs(levels);
  for (uint32_t l = 0; l < levels; l++) {
    level_ofs[l] = (uint32_t)d.size();
    d.insert(d.end(), level_data[l].begin(), level_data[l].end());
  }
  if (d.size() > 0xFFFFFFu) { set_error("crngpu_crn_pack: file larger than the format's 24-bit offsets"); return CRNGPU_E_PARAM; }
  put_be(d, 0, ('H' << 8) | 'x', 2);
  put_be(d, 2, header_size, 2);
  put_be(d, 6, (uint32_t)d.size(), 4);
  put_be(d, 12, width, 2);
  put_be(d, 14, height, 2);
  d[16] = (uint8_t)levels;
  d[17] = (uint8_t)faces;
  d[18] = (uint8_t)format;
  const size_t nums[4] = {cep.values.size(), csel.values.size(), aep.values.size(), asel.values.size()};
  for (int p = 0; p < 4; p++) {
    if (pal[p].empty()) continue;
    put_be(d, 33 + 8 * p, pal_ofs[p], 3);
    put_be(d, 36 + 8 * p, (uint32_t)pal[p].size(), 3);
    put_be(d, 39 + 8 * p, (uint32_t)nums[p], 2);
  }
  put_be(d, 65, (uint32_t)tables.size(), 2);
  put_be(d, 67, tables_ofs, 3);
  for (uint32_t l = 0; l < levels; l++) put_be(d, 70 + 4 * l, level_ofs[l], 4);
  put_be(d, 10, crc16(d.data() + header_size, (uint32_t)(d.size() - header_size)), 2);
  put_be(d, 4, crc16(d.data() + 6, header_size - 6), 2);
  if (out && out_capacity >= d.size()) std::memcpy(out, d.data(), d.size());
  return (int64_t)d.size();
} catch (...) {
  return crngpu::exception_status();
}

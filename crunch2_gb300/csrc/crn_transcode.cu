// CRN -> DXTn transcoder on the GPU.
//
// Restates crnd::crn_unpacker::unpack_level and unpack_dxt1/dxt5/dxn/dxt5a
// (inc/crn_decomp.h:3537-3619, 3944-4223) as two kernels:
//   k_crn_decode_textures - the serial part. Each level stream is a serial chain of prefix
//                   codes whose meaning depends on the symbols before it, so one lane owns one
//                   stream: it Huffman-decodes the reference-group / endpoint-delta / selector
//                   symbols, resolves the left/top endpoint references and the running (mod
//                   palette size) endpoint indices, and writes one index record per visible
//                   block. A warp takes one texture (its prefix tables staged in shared memory)
//                   and its lanes decode the texture's levels side by side; the decode is a
//                   per-lane state machine (one symbol per iteration) so the lanes stay in
//                   lockstep. The kernel is persistent: warps take textures largest-first from
//                   a work counter until none are left, so one launch decodes every level of
//                   every texture of a batch, whatever their sizes and formats.
//   k_crn_expand_tiles - the parallel part: every thread turns index records into finished
//                   DXT words (palette gathers from L2) and writes 16 bytes per store.
// The header, Huffman models and palettes are decoded once on the host (crn_file.cpp).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "crn_file.h"
#include "crngpu_internal.h"
#include "host_alloc.h"

namespace crngpu {

// Device status word values (written by k_crn_decode_textures, read back by the host).
enum : uint32_t { kStOk = 0, kStBadCode = 1, kStBadIndex = 2 };

// Model slots in a context's device model array.
enum { kMRef = 0, kMEp0 = 1, kMSel0 = 2, kMEp1 = 3, kMSel1 = 4, kNumModels = 5 };

// Block formats of a level stream (runtime, per job).
enum : uint32_t { kKDxt1 = 0, kKDxt5 = 1, kKDxn = 2, kKDxt5a = 3 };

struct DevPalettes {
  const uint32_t* colour_ep;
  const uint32_t* colour_sel;
  const uint16_t* alpha_ep;
  const uint64_t* alpha_sel;  // 48 bits of DXT5 alpha selectors per entry
  uint32_t n_cep, n_csel, n_aep, n_asel;
};

// One level stream for the decoder. Endpoint "A" is the colour endpoint (DXT1, DXT5) or the
// first alpha endpoint (DXN, DXT5A); "B" is the DXT5 alpha endpoint or the second DXN alpha.
struct StreamJob {
  const uint8_t* src;       // compressed level stream (device; readable 64 bytes past the end)
  const DevModel* models;   // the file's five prefix models
  uint8_t* rec;             // index records of the level: faces x by x bx, 4 or 8 bytes each
  uint32_t src_size;
  uint32_t bx, by, faces;
  uint32_t kind;
  uint32_t n_a, n_b, n_sa, n_sb;  // endpoint and selector palette sizes (A, B)
  uint32_t rb_ofs;                // the lane's row-buffer slice in shared memory (words)
};

// One texture for the decoder: the streams [first, first + nlev) of one file, one lane each.
struct TexJob {
  const DevModel* models;  // the file's five prefix models
  uint32_t first, nlev, kind, rb_words;  // rb_words: row-buffer words of all its lanes
  uint64_t work;           // blocks x streams-per-block, for the largest-first order
};

// One face of one level for the expansion kernel.
struct ExpandJob {
  uint8_t* dst;           // row 0 of the face (device)
  const uint8_t* rec;     // the face's index records
  DevPalettes pal;
  uint32_t bx, by, pitch, kind;
  uint32_t flat;          // pitch == bx * bytes per block: the face is one contiguous block array
  uint32_t vec;           // 16-byte stores are aligned (dst, and pitch unless flat)
};

constexpr uint32_t kExpandThreads = 256;
// Expansion variants: tile of 1024 << kTileShift[v] blocks, DXT1 palettes staged or not. The
// autotuner (crngpu_unpack_batch_launch, first launch) times all of them and keeps the fastest.
constexpr int kTileSizes = 6;           // 1024 .. 32768 blocks per tile, processed 2048 at a time
constexpr uint32_t kSubBlocks = 2048;   // blocks per pass of a CTA over its tile (8 per thread)
constexpr int kExpandVariants = 2 * kTileSizes + 9;  // + pipelined tiles, + TMA-staged records
constexpr uint32_t kTmaSub = 2048;      // blocks per pass of the TMA variants (records staged per pass)
constexpr uint32_t kStageMin = 1024;    // DXT1 tiles at least this large may stage their palettes
// Decoder shared memory per CTA: five first-level tables + the row buffers of one texture's
// levels (at most 2 x 1024 + 2 x 16 words for a 4096-texel-wide texture with 16 levels).
constexpr size_t kDecodeSmemMax = 64u << 10;

__host__ __device__ constexpr uint32_t record_bytes(uint32_t kind) {
  return (kind == kKDxt1 || kind == kKDxt5a) ? 4u : 8u;
}

// ------------------------------------------------------------------------------------------
// Bit reader: MSB-first 64-bit window; bytes past the end of the stream read as zero, as in
// symbol_codec::get_bits / decode (inc/crn_decomp.h:3162-3214). After a byte-wise head the
// stream is read as aligned 32-bit words (byte-swapped to MSB-first); the next word is always
// loaded one refill ahead so a refill never waits on memory, and an L1 prefetch runs 1 KB ahead.
struct Bits {
  const uint8_t* p;   // stream start
  uint32_t pos, end;  // byte offset of `next`, stream size
  uint32_t next;      // the word at pos (masked past the end)
  uint32_t hi, lo;    // the next n <= 64 stream bits, MSB first in hi:lo; the bits past them are zero
  int n;
  __device__ __forceinline__ uint32_t load_word(uint32_t at) const {
    if (at >= end) return 0u;
    uint32_t w = __byte_perm(__ldg(reinterpret_cast<const uint32_t*>(p + at)), 0, 0x0123);
    if (at + 4 > end) w &= 0xFFFFFFFFu << (8 * (4 - (end - at)));  // zero the bytes past the end
    return w;
  }
  __device__ __forceinline__ void init(const uint8_t* src, uint32_t size) {
    p = src; pos = 0; end = size; hi = 0; lo = 0; n = 0;
    while (((uintptr_t)(p + pos) & 3) && n <= 24) {  // at most 3 bytes up to word alignment
      const uint32_t v = pos < end ? (uint32_t)__ldg(p + pos) : 0u;
      hi |= v << (24 - n);
      n += 8;
      pos++;
    }
    next = load_word(pos);
  }
  __device__ __forceinline__ void refill() {
    if (n <= 32) {
      const uint64_t w = (uint64_t)next << (32 - n);  // the word's bits at positions n .. n + 31
      hi |= (uint32_t)(w >> 32);
      lo = (uint32_t)w;
      n += 32;
      pos += 4;
      if ((pos & 127) == 0 && pos + 1024 < end) asm volatile("prefetch.global.L1 [%0];" ::"l"(p + pos + 1024));
      next = load_word(pos);
    }
  }
  __device__ __forceinline__ uint32_t peek16() const { return hi >> 16; }
  __device__ __forceinline__ void consume(uint32_t len) {  // len <= 16
    hi = __funnelshift_l(lo, hi, len);
    lo <<= len;
    n -= (int)len;
  }
};

// Canonical prefix decode (symbol_codec::decode, inc/crn_decomp.h:3186-3253): 11-bit first-level
// table, then a walk over left-aligned per-length limits. -1: no such code.
__device__ __forceinline__ int decode_sym(Bits& b, const DevModel* __restrict__ m) {
  b.refill();
  const uint32_t v = b.peek16();
  const uint32_t e = __ldg(&m->lut[v >> (16 - kLutBits)]);
  uint32_t s, len;
  if (e != kLutLong) {
    s = e & 0xFFFFu;
    len = e >> 16;
  } else {
    len = kLutBits + 1;
    while (len <= (uint32_t)kMaxCodeLen && v >= __ldg(&m->limit[len])) len++;
    if (len > (uint32_t)kMaxCodeLen) return -1;
    const int idx = __ldg(&m->base[len]) + (int)(v >> (16 - len));
    if (idx < 0 || (uint32_t)idx >= __ldg(&m->num_syms)) return -1;
    s = __ldg(&m->sorted[idx]);
  }
  b.consume(len);
  return (int)s;
}

// Row buffer entry (block_buffer_element, inc/crn_decomp.h:3652-3658), packed:
// bits 0-1 endpoint reference for the odd row, 2-14 endpoint index A, 15-27 endpoint index B.
__device__ __forceinline__ uint32_t rb_pack(uint32_t ref, uint32_t a, uint32_t b) { return ref | (a << 2) | (b << 15); }
__device__ __forceinline__ uint32_t rb_a(uint32_t e) { return (e >> 2) & 0x1FFFu; }
__device__ __forceinline__ uint32_t rb_b(uint32_t e) { return (e >> 15) & 0x1FFFu; }

__host__ __device__ constexpr uint32_t models_used(uint32_t kind) { return kind == kKDxt5 ? 5u : 3u; }

// Decodes one symbol with a first-level table in shared memory (`lut`) and, for the rare codes
// longer than kLutBits, the device model `m`. An invalid code sets `bad` and yields symbol 0 after
// consuming kMaxCodeLen bits, so a corrupt stream still ends after its block count.
__device__ __forceinline__ uint32_t decode_sym(Bits& b, const uint32_t* __restrict__ lut,
                                               const DevModel* __restrict__ m, uint32_t& bad) {
  b.refill();
  const uint32_t v = b.peek16();
  const uint32_t e = lut[v >> (16 - kLutBits)];
  uint32_t s, len;
  if (e != kLutLong) {
    s = e & 0xFFFFu;
    len = e >> 16;
  } else {
    len = kLutBits + 1;
    while (len <= (uint32_t)kMaxCodeLen && v >= __ldg(&m->limit[len])) len++;
    s = 0;
    if (len > (uint32_t)kMaxCodeLen) {
      bad |= 1u;
      len = kMaxCodeLen;
    } else {
      const int idx = __ldg(&m->base[len]) + (int)(v >> (16 - len));
      if (idx < 0 || (uint32_t)idx >= __ldg(&m->num_syms)) bad |= 1u;
      else s = __ldg(&m->sorted[idx]);
    }
  }
  b.consume(len);
  return s;
}

// One level stream (all its faces), the loop of unpack_dxt1/dxt5/dxn/dxt5a
// (inc/crn_decomp.h:3944-4223). `luts` holds the first-level tables of the models this format
// reads (ref, then delta/selector of endpoint A, then of endpoint B for DXT5); `rb` is the lane's
// row buffer. Returns a kSt* status. Errors do not leave the loop: invalid codes are flagged as they
// occur, out-of-range palette indices through the largest index seen, and the stream runs to its
// block count, which keeps the loop free of early exits.
template <int KIND>
__device__ uint32_t decode_level(const StreamJob& J, const uint32_t* __restrict__ luts, uint32_t* __restrict__ rb) {
  constexpr bool colour = KIND == kKDxt1 || KIND == kKDxt5;
  constexpr bool two = KIND == kKDxt5 || KIND == kKDxn;
  const DevModel* mR = J.models + kMRef;
  const DevModel* mDA = J.models + (colour ? kMEp0 : kMEp1);
  const DevModel* mSA = J.models + (colour ? kMSel0 : kMSel1);
  const DevModel* mDB = J.models + kMEp1;
  const DevModel* mSB = J.models + kMSel1;
  const uint32_t* lR = luts;
  const uint32_t* lDA = luts + (1u << kLutBits);
  const uint32_t* lSA = luts + (2u << kLutBits);
  const uint32_t* lDB = KIND == kKDxt5 ? luts + (3u << kLutBits) : lDA;
  const uint32_t* lSB = KIND == kKDxt5 ? luts + (4u << kLutBits) : lSA;
  const uint32_t bx = J.bx, by = J.by, faces = J.faces;
  const uint32_t W = (bx + 1) & ~1u, H = (by + 1) & ~1u;
  const uint32_t nA = J.n_a, nB = J.n_b, nSA = J.n_sa, nSB = J.n_sb;
  for (uint32_t x = 0; x < W; x++) rb[x] = 0;
  Bits b;
  b.init(J.src, J.src_size);
  uint32_t iA = 0, iB = 0, bad = 0;
  // the largest endpoint / selector index seen: a stream is corrupt if it ever leaves a palette
  // (the expansion clamps every index, so the records of such a stream stay in bounds)
  uint32_t max_a = 0, max_b = 0, max_sa = 0, max_sb = 0;
  uint32_t* rec32 = reinterpret_cast<uint32_t*>(J.rec);
  uint64_t* rec64 = reinterpret_cast<uint64_t*>(J.rec);
  // one block given its reference kind and its row-buffer word (whose low bits are already the
  // reference of the block below, on even rows)
  auto block = [&](uint32_t ref, uint32_t e, uint32_t x, bool vis) {
    if (ref == 0) {
      iA += decode_sym(b, lDA, mDA, bad);
      iA -= iA >= nA ? nA : 0u;
      if (two) {
        iB += decode_sym(b, lDB, mDB, bad);
        iB -= iB >= nB ? nB : 0u;
      }
    }
    if (ref <= 1) {
      e = rb_pack(e & 3u, iA, iB);
    } else {
      iA = rb_a(e);
      iB = rb_b(e);
    }
    max_a = max(max_a, iA);
    rb[x] = e;
    const uint32_t sa = decode_sym(b, lSA, mSA, bad);
    max_sa = max(max_sa, sa);
    uint32_t sb = 0;
    if (two) {
      max_b = max(max_b, iB);
      sb = decode_sym(b, lSB, mSB, bad);
      max_sb = max(max_sb, sb);
    }
    if (vis) {
      const uint32_t lo = iA | (sa << 16);
      if (!two) *rec32++ = lo;
      else *rec64++ = (uint64_t)lo | ((uint64_t)(iB | (sb << 16)) << 32);
    }
  };
  for (uint32_t f = 0; f < faces; f++) {
    for (uint32_t y = 0; y < H; y += 2) {
      // even row: one reference group per 2x2 chunk gives this block's and the one below's
      // reference for the left and the right column
      const bool vis0 = y < by;
      for (uint32_t x = 0; x < W; x += 2) {
        const uint32_t g = decode_sym(b, lR, mR, bad) & 0xFFu;  // reference_group is a uint8
        block(g & 3u, (rb[x] & ~3u) | ((g >> 2) & 3u), x, vis0 && x < bx);
        block((g >> 4) & 3u, (rb[x + 1] & ~3u) | ((g >> 6) & 3u), x + 1, vis0 && x + 1 < bx);
      }
      // odd row: the references stored by the row above
      const bool vis1 = y + 1 < by;
      for (uint32_t x = 0; x < W; x++) {
        const uint32_t e = rb[x];
        block(e & 3u, e, x, vis1 && x < bx);
      }
    }
  }
  if (max_a >= nA || max_sa >= nSA || (two && (max_b >= nB || max_sb >= nSB))) bad |= 2u;
  return (bad & 1u) ? kStBadCode : (bad & 2u) ? kStBadIndex : kStOk;
}

// Persistent decoder: one warp per texture (one batch item: one file, up to 32 level streams),
// one lane per level. The warp stages the file's first-level prefix tables in shared memory, so
// every lane's symbol lookup is a shared-memory load; each lane keeps its row buffer (packed
// block_buffer_element entries) in a compact slice of shared memory.
// Dynamic shared memory: [lut_words table words][rb_total row-buffer words].
// `counter` must be zero at launch; items are ordered largest first.
constexpr uint32_t kDecodeWarps = 4;
__global__ void __launch_bounds__(kDecodeWarps * 32) k_crn_decode_textures(const TexJob* __restrict__ items,
                                                                          uint32_t nitems,
                                                                          const StreamJob* __restrict__ streams,
                                                                          uint32_t* __restrict__ counter,
                                                                          uint32_t lut_words, uint32_t rb_total,
                                                                          uint32_t* __restrict__ status) {
  extern __shared__ uint32_t smem[];
  __shared__ uint32_t s_item;
  uint32_t* luts = smem;
  uint32_t* rb_base = smem + lut_words;
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t err = kStOk;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1u);
    __syncthreads();
    const uint32_t it = s_item;
    __syncthreads();  // every thread has read s_item before it is rewritten
    if (it >= nitems) break;
    const TexJob T = items[it];
    const uint32_t kind = T.kind;
    const uint32_t nm = models_used(kind);
    if ((nm << kLutBits) > lut_words || T.rb_words > rb_total) { err = max(err, (uint32_t)kStBadCode); continue; }
    // stage the tables this format reads: ref, delta A, selector A (+ delta B, selector B for DXT5)
    {
      const bool colour = kind == kKDxt5 || kind == kKDxt1;
      const int srcm[5] = {kMRef, colour ? kMEp0 : kMEp1, colour ? kMSel0 : kMSel1, kMEp1, kMSel1};
      for (uint32_t t = 0; t < nm; t++) {
        const uint4* src = reinterpret_cast<const uint4*>(T.models[srcm[t]].lut);
        uint4* dst = reinterpret_cast<uint4*>(luts + (t << kLutBits));
        for (uint32_t k = threadIdx.x; k < (1u << kLutBits) / 4; k += blockDim.x) dst[k] = __ldg(src + k);
      }
    }
    __syncthreads();
    // level streams, largest first: stream w < kDecodeWarps - 1 alone on lane 0 of warp w, the
    // rest on the lanes of the last warp, so the longest streams share no warp with others
    const uint32_t si = warp + 1 < kDecodeWarps ? (lane == 0 ? warp : 0xFFFFFFFFu) : (kDecodeWarps - 1 + lane);
    if (si < T.nlev) {
      const StreamJob J = streams[T.first + si];
      const uint32_t W = (J.bx + 1) & ~1u;
      if (J.rb_ofs + W <= rb_total && J.kind == kind) {  // host validated; never false
        uint32_t* rb = rb_base + J.rb_ofs;
        uint32_t st;
        switch (kind) {
          case kKDxt1: st = decode_level<kKDxt1>(J, luts, rb); break;
          case kKDxt5: st = decode_level<kKDxt5>(J, luts, rb); break;
          case kKDxn: st = decode_level<kKDxn>(J, luts, rb); break;
          default: st = decode_level<kKDxt5a>(J, luts, rb); break;
        }
        err = max(err, st);
      }
    }
    __syncthreads();  // the texture's streams are done before its tables are replaced
  }
  if (err) atomicMax(status, err);
}

// ------------------------------------------------------------------------------------------
// Large levels: k_crn_decode_wide, one CTA per level stream.
//
// The lane decoder above spends about 430 cycles per block on one lane, because every symbol is
// a chain of dependent steps (bit-window refill, table lookup, shift) and a 1024 x 1024 level has
// 65,536 blocks in one chain. This decoder keeps only the part of that chain that is truly serial
// -- where the next chunk or block starts in the bit stream -- and makes each of its steps one
// shared-memory load:
//
//  * Step tables, per bit position. For every bit position p of a window of the stream, worker
//    warps decode, in parallel and without knowing whether a code starts at p, the code of every
//    model the format reads at p, and compose the lengths into three "where does the next item
//    start" tables: next0[p] (a block with no endpoint deltas: its selector code(s)), next1[p] (a
//    block with endpoint deltas: delta code(s) then selector code(s)), nextC[p] (a 2x2 chunk pair
//    of an even row: the reference-group code, then its two blocks, each as next0 or next1 as the
//    group says), and the reference group g[p] decoded at p.
//  * The chain. Lane 0 of warp 0 walks the level: on an even row it visits chunk starts
//    (p = nextC[p], keeping g[p] for the row below), on an odd row block starts (p = next0[p] or
//    next1[p] as the reference stored by the row above says). It records each item's bit position.
//  * Emission. With the positions known, worker threads decode the symbols of each recorded item
//    in parallel (one item per thread), then resolve the running endpoint indices of each row with
//    a scan: a block with endpoint deltas adds them (mod the palette size), a "left" reference
//    keeps the running index, an "up" reference sets it from the row above. The scan's operator
//    (set-or-add-mod-n) is associative as long as every delta is below the palette size, which
//    holds for every stream the reference writes (its delta models have one symbol per palette
//    entry); a row holding a larger delta is resolved sequentially with the reference's own rule.
//
// Windows are kWS bits apart and kWX = kWS + kWM bits long. The chain steps in pairs and tests
// the position of the last item it recorded once per pair, so that its loop branch never waits on
// a load in flight: its last items in a window may start up to 2 x 144 bits (two chunk pairs) past
// kWS, and a table entry reads at most 128 bits past its own position; the overlap kWM covers both. The CTA runs in
// phases: in phase t the chain
// walks window t - 1 while the workers build window t and emit the items the chain recorded in
// phase t - 1; two table buffers and two item lists alternate. The result is bit-identical to
// unpack_dxt1/dxt5/dxn/dxt5a (inc/crn_decomp.h:3944-4223), including the status the lane decoder
// reports for corrupt streams.
constexpr uint32_t kWS = 2048;                 // window stride (bits)
constexpr uint32_t kWM = 448;                  // window overlap (bits): 2 x 144 of chain overshoot + 128 of table reach
constexpr uint32_t kWX = kWS + kWM;            // positions per window
constexpr uint32_t kWWords = kWX / 32 + 4;     // staged stream words per window
constexpr uint32_t kWEmitters = 128;           // symbol-decoder threads (warps 1 .. 4)
constexpr uint32_t kWResolvers = 64;           // endpoint-index resolver threads (warps 5, 6)
constexpr uint32_t kWBuilders = 416;           // table-builder threads (warps 7 .. 19)
constexpr uint32_t kWThreads = 32 + kWEmitters + kWResolvers + kWBuilders;  // + the chain warp (warp 0)
constexpr uint32_t kWPer = (kWX + kWBuilders - 1) / kWBuilders;  // window positions per builder
constexpr uint32_t kWMaxW = 1024;              // widest row, in blocks (4096 texels)
constexpr uint32_t kWList = kWS + 4;           // chain items per phase, at most (positions increase; two past kWS)
constexpr uint32_t kWBlk = kWS + 448;          // emitted blocks per phase, at most (each costs >= 1 bit)
constexpr uint32_t kWNotDone = 0xFFFFFFFFu;
constexpr uint32_t kStaged = 512;        // reference model: its first sorted symbols in shared memory
constexpr uint32_t kStagedLong = 4096;   // other models: the symbols of their codes longer than kLutBits

// Shared-memory layout of k_crn_decode_wide (bytes), for a format reading `nm` models.
struct WideLayout {
  uint32_t lut, srt, nx, gt, words, list, rb, grow, un, bw, total;
};
__host__ __device__ constexpr uint32_t wide_align16(uint32_t v) { return (v + 15u) & ~15u; }
__host__ __device__ inline WideLayout wide_layout(uint32_t nm) {
  WideLayout L{};
  uint32_t o = 0;
  L.lut = o;   o += nm * (4u << kLutBits);       // first-level tables of the models read
  L.srt = o;   o += (nm - 1) * kStagedLong * 2u;  // long-code symbols of the models after the reference
  L.nx = o;    o += 3u * 2u * kWX * 2u;          // next0, next1, nextC (u16) for two windows
  L.gt = o;    o = wide_align16(o + 2u * kWX);   // reference group at each position, two windows
  L.words = o; o += 4u * kWWords * 4u;           // staged stream words, four windows
  L.list = o;  o += 2u * kWList * 4u;            // chain items (bit position | reference << 30), two phases
  L.rb = o;    o += 2u * kWMaxW * 2u;            // endpoint index A and B of the row above
  L.grow = o;  o = wide_align16(o + kWMaxW / 2); // the chain's reference groups of the current even row
  L.un = o;    o = wide_align16(o + 7u * kWX);   // build temporaries (code lengths at each position)
  L.bw = o;    o += 2u * 2u * kWBlk * 4u;        // decoded blocks of two item lists (decoded, being resolved)
  L.total = wide_align16(o);
  return L;
}

// Word m of a level stream (its bytes 4m .. 4m + 3, MSB first); bytes at or past `end` read as
// zero. `src` may have any alignment: the word is assembled from the aligned words around it, and
// an aligned word is only read when it holds a byte of the stream. Split in a load and a finish so
// that a caller can keep the loads in flight while it does other work.
struct RawWord {
  uint32_t lo, hi;
};
__device__ __forceinline__ RawWord stream_word_load(const uint8_t* src, uint32_t end, uint32_t m) {
  const uint32_t at = 4u * m;
  RawWord w{0u, 0u};
  if (at >= end) return w;
  const uint32_t r = (uint32_t)((uintptr_t)src & 3u);
  const uint32_t* A = reinterpret_cast<const uint32_t*>(src - r + at);
  w.lo = __ldg(A);
  if (r && at + 4u - r < end) w.hi = __ldg(A + 1);
  return w;
}
__device__ __forceinline__ uint32_t stream_word_finish(const uint8_t* src, uint32_t end, uint32_t m, RawWord raw) {
  const uint32_t at = 4u * m;
  if (at >= end) return 0u;
  const uint32_t r = (uint32_t)((uintptr_t)src & 3u);
  uint32_t w = __byte_perm(raw.lo, raw.hi, (r + 3u) | ((r + 2u) << 4) | ((r + 1u) << 8) | (r << 12));
  if (at + 4u > end) w &= 0xFFFFFFFFu << (8u * (4u - (end - at)));
  return w;
}
__device__ __forceinline__ uint32_t stream_word(const uint8_t* src, uint32_t end, uint32_t m) {
  return stream_word_finish(src, end, m, stream_word_load(src, end, m));
}

// The 32 stream bits starting at window position j (the window's staged words `w`).
__device__ __forceinline__ uint32_t window_bits(const uint32_t* w, uint32_t j) {
  return __funnelshift_l(w[(j >> 5) + 1], w[j >> 5], j & 31u);
}

// Canonical prefix decode with the first-level table `lut` and, for codes longer than kLutBits,
// the model's per-length bounds staged in shared memory: aux[0..4] = limit[12..16], aux[5..9] =
// base[12..16], aux[10] = number of symbols. Codes longer than kLutBits need no loop: the length is
// 12 plus the number of bounds at or below the bits (the bounds do not decrease with the length).
constexpr uint32_t kAuxWords = 12;
__device__ __forceinline__ uint32_t long_code_len(uint32_t v16, const uint32_t* aux) {
  uint32_t l = kLutBits + 1;
#pragma unroll
  for (int k = 0; k < kMaxCodeLen - kLutBits; k++) l += v16 >= aux[k] ? 1u : 0u;
  return l;  // kMaxCodeLen + 1: no such code
}

// Length of the code at the top of `v16` (16 bits, MSB first); an invalid code is kMaxCodeLen long,
// as in decode_sym.
__device__ __forceinline__ uint32_t code_len(uint32_t v16, const uint32_t* __restrict__ lut, const uint32_t* aux) {
  const uint32_t e = lut[v16 >> (16 - kLutBits)];
  const uint32_t l = min(long_code_len(v16, aux), (uint32_t)kMaxCodeLen);
  return e != kLutLong ? e >> 16 : l;
}

// Symbol of the code at the top of `v16` and its length in `len`. Same rules as decode_sym: an
// invalid code (or a code past the model's symbols) sets `bad`, yields symbol 0 and, when no code
// of any length matches, is kMaxCodeLen long. `st` holds the model's sorted symbols
// [aux[11], aux[11] + st_n) in shared memory; others are read from the device model.
__device__ __forceinline__ uint32_t code_sym(uint32_t v16, const uint32_t* __restrict__ lut, const uint32_t* aux,
                                             const DevModel* __restrict__ m, const uint16_t* st, uint32_t st_n,
                                             uint32_t& len, uint32_t& bad) {
  const uint32_t e = lut[v16 >> (16 - kLutBits)];
  if (e != kLutLong) {
    len = e >> 16;
    return e & 0xFFFFu;
  }
  const uint32_t l = long_code_len(v16, aux);
  if (l > (uint32_t)kMaxCodeLen) {
    bad |= 1u;
    len = kMaxCodeLen;
    return 0u;
  }
  len = l;
  const int idx = (int)aux[5 + l - (kLutBits + 1)] + (int)(v16 >> (16 - l));
  if (idx < 0 || (uint32_t)idx >= aux[10]) {
    bad |= 1u;
    return 0u;
  }
  const uint32_t k = (uint32_t)idx - aux[11];
  return k < st_n ? (uint32_t)st[k] : (uint32_t)__ldg(&m->sorted[idx]);
}

// Barriers of the table builders (named barrier 1) and of the emitters (named barrier 2); the
// other roles run on.
__device__ __forceinline__ void builder_sync() { asm volatile("bar.sync 1, %0;" ::"r"(kWBuilders) : "memory"); }
__device__ __forceinline__ void resolver_sync() { asm volatile("bar.sync 2, %0;" ::"r"(kWResolvers) : "memory"); }
__device__ __forceinline__ bool resolver_sync_or(bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.or.pred q, 2, %2, p;\n\tselp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(kWResolvers)
      : "memory");
  return r != 0u;
}

__device__ __forceinline__ uint32_t add_mod(uint32_t x, uint32_t y, uint32_t n) { return x + y >= n ? x + y - n : x + y; }

// Scan operator of the endpoint-index resolution: x -> set ? a : (x + a) mod n (b likewise).
struct IdxOp {
  uint32_t set, a, b;
};
template <bool TWO>
__device__ __forceinline__ IdxOp idx_compose(const IdxOp& f, const IdxOp& g, uint32_t nA, uint32_t nB) {
  if (g.set) return g;
  return IdxOp{f.set, add_mod(f.a, g.a, nA), TWO ? add_mod(f.b, g.b, nB) : 0u};
}

// The decoder's dynamic shared memory, named at file scope so that every pointer into it is known
// to be shared (loads and stores stay shared-window accesses after inlining).
extern __shared__ __align__(16) uint8_t wide_smem[];

// Small shared state of k_crn_decode_wide (one instance per CTA).
struct WideShared {
  uint32_t meta[2][3];  // per item list: count, first row, first item in that row
  uint32_t rmeta[2][3]; // per decoded list (for the resolvers): block count, first row, first item
  uint32_t done, carry[2], bad;
  uint32_t aux[5][kAuxWords];       // long-code bounds of the models read (slot order of the tables)
  uint32_t scan[kWResolvers / 32][3];
  uint16_t rsorted[kStaged];        // the reference model's first sorted symbols
};

template <int KIND>
__device__ __forceinline__ void wide_level(const StreamJob& J, WideShared& S, uint32_t* status) {
  constexpr bool colour = KIND == kKDxt1 || KIND == kKDxt5;
  constexpr bool two = KIND == kKDxt5 || KIND == kKDxn;
  constexpr bool five = KIND == kKDxt5;
  constexpr uint32_t nm = five ? 5u : 3u;
  uint8_t* sm = wide_smem;
  const WideLayout Ly = wide_layout(nm);
  uint16_t* srt = reinterpret_cast<uint16_t*>(sm + Ly.srt);

  const uint32_t tid = threadIdx.x;
  uint32_t* luts = reinterpret_cast<uint32_t*>(sm + Ly.lut);
  const uint32_t* lR = luts;
  const uint32_t* lDA = luts + (1u << kLutBits);
  const uint32_t* lSA = luts + (2u << kLutBits);
  const uint32_t* lDB = five ? luts + (3u << kLutBits) : lDA;
  const uint32_t* lSB = five ? luts + (4u << kLutBits) : lSA;
  // model slots of the second endpoint / selector code (the same models as the first for DXN)
  constexpr uint32_t sDB = five ? 3u : 1u, sSB = five ? 4u : 2u;
  const DevModel* mR = J.models + kMRef;
  const DevModel* mDA = J.models + (colour ? kMEp0 : kMEp1);
  const DevModel* mSA = J.models + (colour ? kMSel0 : kMSel1);
  const DevModel* mDB = J.models + kMEp1;
  const DevModel* mSB = J.models + kMSel1;
  uint16_t* nx0 = reinterpret_cast<uint16_t*>(sm + Ly.nx);
  uint16_t* nx1 = nx0 + 2 * kWX;
  uint16_t* nxC = nx1 + 2 * kWX;
  uint8_t* gt = sm + Ly.gt;
  uint32_t* words = reinterpret_cast<uint32_t*>(sm + Ly.words);
  uint32_t* list = reinterpret_cast<uint32_t*>(sm + Ly.list);
  uint16_t* rbA = reinterpret_cast<uint16_t*>(sm + Ly.rb);
  uint16_t* rbB = rbA + kWMaxW;
  uint8_t* grow = sm + Ly.grow;
  uint8_t* un = sm + Ly.un;
  uint8_t* lenR = un;            // build temporaries
  uint8_t* lenDA = un + kWX;
  uint8_t* lenSA = un + 2 * kWX;
  uint8_t* lenDB = un + 3 * kWX;
  uint8_t* lenSB = un + 4 * kWX;
  uint8_t* lenSBk = un + 5 * kWX;  // selector codes of one block (two-endpoint formats)
  uint8_t* lenEBk = un + 6 * kWX;  // endpoint codes of one block (two-endpoint formats)
  // decoded blocks of list i at bwbuf + (i & 1) * 2 * kWBlk: word 0 = reference | delta A << 2 |
  // selector A << 16, word 1 (kWBlk further) = delta B | selector B << 16
  uint32_t* bwbuf = reinterpret_cast<uint32_t*>(sm + Ly.bw);

  const uint32_t W = (J.bx + 1) & ~1u, H = (J.by + 1) & ~1u, W2 = W >> 1;
  const uint32_t rows = J.faces * H;
  const uint32_t nA = J.n_a, nB = J.n_b, nSA = J.n_sa, nSB = J.n_sb;

  {  // stage the first-level tables, long-code bounds and sorted symbols; clear the running state
    const int srcm[5] = {kMRef, colour ? kMEp0 : kMEp1, colour ? kMSel0 : kMSel1, kMEp1, kMSel1};
    for (uint32_t t = 0; t < nm; t++) {
      const uint4* src = reinterpret_cast<const uint4*>(J.models[srcm[t]].lut);
      uint4* dst = reinterpret_cast<uint4*>(luts + (t << kLutBits));
      for (uint32_t k = tid; k < (1u << kLutBits) / 4; k += blockDim.x) dst[k] = __ldg(src + k);
    }
    for (uint32_t x = tid; x < W; x += blockDim.x) rbA[x] = rbB[x] = 0;
    if (tid < nm * kAuxWords) {
      const uint32_t t = tid / kAuxWords, k = tid - t * kAuxWords;
      const DevModel* md = J.models + srcm[t];
      // aux[11]: sorted index of the first long code (offset of length 12 = base + first code)
      S.aux[t][k] = k < 5 ? __ldg(&md->limit[kLutBits + 1 + k])
                  : k < 10 ? (uint32_t)__ldg(&md->base[kLutBits + 1 + k - 5])
                  : k == 10 ? __ldg(&md->num_syms)
                  : t == 0 ? 0u
                  : (uint32_t)(__ldg(&md->base[kLutBits + 1]) + (int)(__ldg(&md->limit[kLutBits]) >> (16 - kLutBits - 1)));
    }
    if (tid == 0) {
      S.done = kWNotDone;
      S.carry[0] = S.carry[1] = 0;
      S.bad = 0;
    }
    // the stream words of window 0 (later windows are loaded one phase ahead)
    for (uint32_t m = tid; m < kWWords; m += blockDim.x) words[m] = stream_word(J.src, J.src_size, m);
  }
  __syncthreads();
  {
    const int srcm[5] = {kMRef, colour ? kMEp0 : kMEp1, colour ? kMSel0 : kMSel1, kMEp1, kMSel1};
    for (uint32_t k = tid; k < kStaged; k += blockDim.x) S.rsorted[k] = __ldg(&mR->sorted[k]);
    for (uint32_t i = tid; i < (nm - 1) * kStagedLong; i += blockDim.x) {
      const uint32_t t = 1 + i / kStagedLong, k = i % kStagedLong;
      const uint32_t idx = S.aux[t][11] + k;
      srt[i] = idx < kMaxSyms ? __ldg(&J.models[srcm[t]].sorted[idx]) : (uint16_t)0;
    }
  }
  __syncthreads();

  uint32_t c_r = 0, c_e = 0, c_j = 0;  // the chain's row, item within the row, window position
  uint32_t done_at = kWNotDone;
  const uint32_t warp = tid >> 5, lane = tid & 31u;
  const uint32_t wt = tid - (32 + kWEmitters + kWResolvers);  // builder index
  const uint32_t et = tid - 32;                               // decoder index
  const uint32_t rt = tid - (32 + kWEmitters);                // resolver index
  for (uint32_t t = 0;; t++) {
    if (tid == 0 && t >= 1 && done_at == kWNotDone) {
      // ---- the chain walks window t - 1 and records its items in list (t - 1) & 1
      const uint32_t wb = (t - 1) & 1u;
      const uint16_t* n0 = nx0 + wb * kWX;
      const uint16_t* n1 = nx1 + wb * kWX;
      const uint16_t* nC = nxC + wb * kWX;
      const uint8_t* g = gt + wb * kWX;
      uint32_t* L = list + wb * kWList;
      const uint32_t a = (t - 1) * kWS;
      S.meta[wb][1] = c_r;
      S.meta[wb][2] = c_e;
      // jp: position of the last item recorded, the loop test. Steps go in pairs with one test per
      // pair, so a loop branch never waits on a table load in flight; the only dependency of a step
      // is the table load at j. Odd-row group bytes are loaded a pair ahead.
      uint32_t n = 0, j = c_j, jp = 0, r = c_r, e = c_e;
      while (r < rows && jp < kWS) {
        if (!(r & 1u)) {
          while (e + 2 <= W2 && jp < kWS) {
            const uint32_t j1 = nC[j];
            const uint32_t g0 = g[j];
            L[n] = a + j;
            const uint32_t j2 = nC[j1];
            const uint32_t g1 = g[j1];
            L[n + 1] = a + j1;
            grow[e] = (uint8_t)g0;
            grow[e + 1] = (uint8_t)g1;
            n += 2;
            jp = j1;
            j = j2;
            e += 2;
          }
          if (e < W2 && jp < kWS) {
            const uint32_t jn = nC[j];
            grow[e] = g[j];
            L[n++] = a + j;
            jp = j;
            j = jn;
            e++;
          }
        } else if (e < W) {
          uint32_t ref0 = (grow[e >> 1] >> ((e & 1u) ? 6 : 2)) & 3u;
          while (e + 2 <= W && jp < kWS) {
            const uint32_t e1 = e + 1, e2 = min(e + 2, W - 1);
            const uint32_t gb1 = grow[e1 >> 1], gb2 = grow[e2 >> 1];
            L[n] = (a + j) | (ref0 << 30);
            const uint32_t j1 = (ref0 ? n0 : n1)[j];
            const uint32_t ref1 = (gb1 >> ((e1 & 1u) ? 6 : 2)) & 3u;
            L[n + 1] = (a + j1) | (ref1 << 30);
            const uint32_t j2 = (ref1 ? n0 : n1)[j1];
            ref0 = (gb2 >> ((e2 & 1u) ? 6 : 2)) & 3u;
            n += 2;
            jp = j1;
            j = j2;
            e += 2;
          }
          if (e < W && jp < kWS) {
            L[n++] = (a + j) | (ref0 << 30);
            jp = j;
            j = (ref0 ? n0 : n1)[j];
            e++;
          }
        }
        if (e == ((r & 1u) ? W : W2)) {
          e = 0;
          r++;
        }
      }
      S.meta[wb][0] = n;
      c_r = r;
      c_e = e;
      c_j = j - kWS;
      if (r >= rows) S.done = t;
    } else if (warp >= 1 + (kWEmitters + kWResolvers) / 32) {
      // the stream words of window t + 1, stored at the end of the build
      const uint32_t pre_m = (((t + 1) * kWS) >> 5) + wt;
      const RawWord pre = (done_at == kWNotDone && wt < kWWords) ? stream_word_load(J.src, J.src_size, pre_m)
                                                                  : RawWord{0u, 0u};
      if (done_at == kWNotDone) {
        // ---- build window t into table buffer t & 1 (its words were staged one phase ahead).
        // Each stage issues all its loads for the thread's kWPer positions before it computes and
        // stores, so the loads of one position never wait behind the stores of another.
        const uint32_t wb = t & 1u;
        const uint32_t* wd = words + (t & 3u) * kWWords;
        uint8_t* g = gt + wb * kWX;
        {
          uint32_t v[kWPer], eR[kWPer], eD[kWPer], eS[kWPer], eD2[kWPer], eS2[kWPer];
#pragma unroll
          for (uint32_t q = 0; q < kWPer; q++) v[q] = window_bits(wd, min(wt + q * kWBuilders, kWX - 1)) >> 16;
#pragma unroll
          for (uint32_t q = 0; q < kWPer; q++) {
            const uint32_t i = v[q] >> (16 - kLutBits);
            eR[q] = lR[i];
            eD[q] = lDA[i];
            eS[q] = lSA[i];
            if (five) {
              eD2[q] = lDB[i];
              eS2[q] = lSB[i];
            }
          }
#pragma unroll
          for (uint32_t q = 0; q < kWPer; q++) {
            const uint32_t j = wt + q * kWBuilders;
            if (j < kWX) {
              uint32_t sym = eR[q] & 0xFFFFu, len = eR[q] >> 16, junk = 0;
              if (eR[q] == kLutLong) sym = code_sym(v[q], lR, S.aux[0], mR, S.rsorted, kStaged, len, junk);
              g[j] = (uint8_t)sym;
              lenR[j] = (uint8_t)len;
              const uint32_t ll1 = min(long_code_len(v[q], S.aux[1]), (uint32_t)kMaxCodeLen);
              const uint32_t ll2 = min(long_code_len(v[q], S.aux[2]), (uint32_t)kMaxCodeLen);
              lenDA[j] = (uint8_t)(eD[q] != kLutLong ? eD[q] >> 16 : ll1);
              lenSA[j] = (uint8_t)(eS[q] != kLutLong ? eS[q] >> 16 : ll2);
              if (five) {
                const uint32_t ll3 = min(long_code_len(v[q], S.aux[3]), (uint32_t)kMaxCodeLen);
                const uint32_t ll4 = min(long_code_len(v[q], S.aux[4]), (uint32_t)kMaxCodeLen);
                lenDB[j] = (uint8_t)(eD2[q] != kLutLong ? eD2[q] >> 16 : ll3);
                lenSB[j] = (uint8_t)(eS2[q] != kLutLong ? eS2[q] >> 16 : ll4);
              }
            }
          }
        }
        builder_sync();
        const uint8_t* sbl = lenSA;  // length of a block's selector code(s) at each position
        const uint8_t* ebl = lenDA;  // length of a block's endpoint delta code(s)
        if (two) {
          const uint8_t* l2D = five ? lenDB : lenDA;
          const uint8_t* l2S = five ? lenSB : lenSA;
          uint32_t ls[kWPer], ld[kWPer], xs[kWPer], xd[kWPer];
#pragma unroll
          for (uint32_t q = 0; q < kWPer; q++) {
            const uint32_t j = min(wt + q * kWBuilders, kWX - 1);
            ls[q] = lenSA[j];
            ld[q] = lenDA[j];
          }
#pragma unroll
          for (uint32_t q = 0; q < kWPer; q++) {
            const uint32_t j = min(wt + q * kWBuilders, kWX - 1);
            xs[q] = l2S[min(j + ls[q], kWX - 1)];
            xd[q] = l2D[min(j + ld[q], kWX - 1)];
          }
#pragma unroll
          for (uint32_t q = 0; q < kWPer; q++) {
            const uint32_t j = wt + q * kWBuilders;
            if (j < kWX) {
              lenSBk[j] = (uint8_t)(ls[q] + xs[q]);
              lenEBk[j] = (uint8_t)(ld[q] + xd[q]);
            }
          }
          builder_sync();
          sbl = lenSBk;
          ebl = lenEBk;
        }
        uint16_t* b0 = nx0 + wb * kWX;
        uint16_t* b1 = nx1 + wb * kWX;
        {
          uint32_t sb[kWPer], qq[kWPer], s2[kWPer];
#pragma unroll
          for (uint32_t q = 0; q < kWPer; q++) {
            const uint32_t j = min(wt + q * kWBuilders, kWX - 1);
            sb[q] = sbl[j];
            qq[q] = min(j + ebl[j], kWX - 1);
          }
#pragma unroll
          for (uint32_t q = 0; q < kWPer; q++) s2[q] = sbl[qq[q]];
#pragma unroll
          for (uint32_t q = 0; q < kWPer; q++) {
            const uint32_t j = wt + q * kWBuilders;
            if (j < kWX) {
              b0[j] = (uint16_t)min(j + sb[q], kWX - 1);
              b1[j] = (uint16_t)min(qq[q] + s2[q], kWX - 1);
            }
          }
        }
        builder_sync();
        {
          uint16_t* bc = nxC + wb * kWX;
          uint32_t gg[kWPer], q1[kWPer];
#pragma unroll
          for (uint32_t q = 0; q < kWPer; q++) {
            const uint32_t j = min(wt + q * kWBuilders, kWX - 1);
            gg[q] = g[j];
            q1[q] = min(j + lenR[j], kWX - 1);
          }
#pragma unroll
          for (uint32_t q = 0; q < kWPer; q++) q1[q] = (gg[q] & 3u) ? b0[q1[q]] : b1[q1[q]];
#pragma unroll
          for (uint32_t q = 0; q < kWPer; q++) q1[q] = ((gg[q] >> 4) & 3u) ? b0[q1[q]] : b1[q1[q]];
#pragma unroll
          for (uint32_t q = 0; q < kWPer; q++) {
            const uint32_t j = wt + q * kWBuilders;
            if (j < kWX) bc[j] = (uint16_t)q1[q];
          }
        }
      }
      if (done_at == kWNotDone && wt < kWWords)
        words[((t + 1) & 3u) * kWWords + wt] = stream_word_finish(J.src, J.src_size, pre_m, pre);
    } else if (warp >= 1 && warp < 1 + kWEmitters / 32 && t >= 2 && (done_at == kWNotDone || t - 2 < done_at)) {
      // ---- the decoder warps: list t - 2 (list buffer t & 1), decoded from window t - 2's
      // staged words into block buffer (t - 2) & 1; the resolvers take it in the next phase
      const uint32_t lb = t & 1u;
      const uint32_t* L = list + lb * kWList;
      const uint32_t* wd = words + ((t - 2) & 3u) * kWWords;
      const uint32_t a2 = (t - 2) * kWS;
      const uint32_t n = S.meta[lb][0], r0 = S.meta[lb][1], e0 = S.meta[lb][2];
      // item i -> row, first block of the list's block array
      const uint32_t odd0 = r0 & 1u, be0 = odd0 ? 1u : 2u;
      const uint32_t nfirst = (odd0 ? W : W2) - e0;
      const uint32_t n1 = odd0 ? W2 : W, be1 = odd0 ? 2u : 1u;
      auto locate = [&](uint32_t i, uint32_t& r, uint32_t& blk) {
        if (i < nfirst) {
          r = r0;
          blk = i * be0;
          return;
        }
        const uint32_t ip = i - nfirst, pairs = ip / (W2 + W), rem = ip - pairs * (W2 + W);
        const uint32_t base = nfirst * be0 + pairs * 2u * W;
        if (rem < n1) {
          r = r0 + 1 + 2 * pairs;
          blk = base + rem * be1;
        } else {
          r = r0 + 2 + 2 * pairs;
          blk = base + W + (rem - n1) * be0;
        }
      };
      const uint16_t* stA = srt;
      const uint16_t* stS = srt + kStagedLong;
      const uint16_t* stDB = five ? srt + 2 * kStagedLong : stA;
      const uint16_t* stSB = five ? srt + 3 * kStagedLong : stS;
      uint32_t* bw0 = bwbuf + ((t - 2) & 1u) * 2u * kWBlk;
      uint32_t* bw1 = bw0 + kWBlk;
      uint32_t bad = 0;
      for (uint32_t i = et; i < n; i += kWEmitters) {
        const uint32_t ent = L[i];
        const uint32_t j = (ent & 0x3FFFFFFFu) - a2;
        uint32_t r, blk;
        locate(i, r, blk);
        // A bit reader in registers: acc holds the next `have` stream bits MSB first (17..64 of
        // them before each decode); a chunk pair is at most 144 bits, so at most three one-word
        // refills follow the first 64 bits. Refill k brings bits [j + 64 + 32k, + 32), which start
        // at word wi = j / 32 + 2 + k with the item's own offset sh inside it.
        uint32_t wi = j >> 5;
        const uint32_t sh = j & 31u;
        uint64_t acc = (((uint64_t)wd[wi] << 32) | wd[wi + 1]) << sh;
        if (sh) acc |= (uint64_t)(wd[wi + 2] >> (32 - sh));
        int have = 64;
        wi += 2;
        auto dec = [&](const uint32_t* lut, uint32_t slot, const DevModel* m, const uint16_t* st, uint32_t st_n) {
          if (have <= 32) {
            const uint32_t bits = sh ? (uint32_t)(((((uint64_t)wd[wi] << 32) | wd[wi + 1]) << sh) >> 32) : wd[wi];
            acc |= (uint64_t)bits << (32 - have);
            have += 32;
            wi += 1;
          }
          uint32_t len;
          const uint32_t sym = code_sym((uint32_t)(acc >> 48), lut, S.aux[slot], m, st, st_n, len, bad);
          acc <<= len;
          have -= (int)len;
          return sym;
        };
        auto block = [&](uint32_t ref, uint32_t k) {
          uint32_t dA = 0, dB = 0;
          if (!ref) {
            dA = dec(lDA, 1, mDA, stA, kStagedLong);
            if (two) dB = dec(lDB, sDB, mDB, stDB, kStagedLong);
          }
          const uint32_t sA = dec(lSA, 2, mSA, stS, kStagedLong);
          const uint32_t sB = two ? dec(lSB, sSB, mSB, stSB, kStagedLong) : 0u;
          bw0[k] = ref | (dA << 2) | (sA << 16);
          if (two) bw1[k] = dB | (sB << 16);
        };
        if (!(r & 1u)) {
          const uint32_t g = dec(lR, 0, mR, S.rsorted, kStaged) & 0xFFu;
          block(g & 3u, blk);
          block((g >> 4) & 3u, blk + 1);
        } else {
          block(ent >> 30, blk);
        }
      }
      if (bad) atomicOr(&S.bad, 1u);
      if (et == 0) {
        uint32_t total = 0;
        if (n) {
          uint32_t r, blk;
          locate(n - 1, r, blk);
          total = blk + ((r & 1u) ? 1u : 2u);
        }
        S.rmeta[(t - 2) & 1u][0] = total;
        S.rmeta[(t - 2) & 1u][1] = r0;
        S.rmeta[(t - 2) & 1u][2] = e0;
      }
    } else if (warp >= 1 + kWEmitters / 32 && t >= 3 && (done_at == kWNotDone || t - 3 < done_at)) {
      // ---- the resolver warps: the endpoint indices of list t - 3 (decoded in the previous
      // phase into block buffer (t - 3) & 1), row segment by row segment, in stream order
      const uint32_t* bw0 = bwbuf + ((t - 3) & 1u) * 2u * kWBlk;
      const uint32_t* bw1 = bw0 + kWBlk;
      const uint32_t total = S.rmeta[(t - 3) & 1u][0], r0 = S.rmeta[(t - 3) & 1u][1], e0 = S.rmeta[(t - 3) & 1u][2];
      const uint32_t odd0 = r0 & 1u;
      // The scan operator per block: a block with deltas adds them (mod the palette size), a
      // "left" reference keeps the running index, an "up" reference sets it from the row above.
      auto block_op = [&](uint32_t b, uint32_t x, bool& inexact) -> IdxOp {
        const uint32_t w0 = bw0[b], ref = w0 & 3u;
        if (ref == 0) {
          const uint32_t dA = (w0 >> 2) & 0x3FFFu, dB = two ? (bw1[b] & 0xFFFFu) : 0u;
          inexact |= dA >= nA || (two && dB >= nB);
          return IdxOp{0, dA, dB};
        }
        if (ref == 1) return IdxOp{0, 0, 0};
        return IdxOp{1, rbA[x], two ? (uint32_t)rbB[x] : 0u};
      };
      uint32_t r = r0, x = odd0 ? e0 : 2 * e0, b = 0, badi = 0;
      while (b < total) {
        const uint32_t cnt = min(W - x, total - b);
        const uint32_t f = r / H, y = r - f * H;
        const bool vis_row = y < J.by;
        const uint32_t per = (cnt + kWResolvers - 1) / kWResolvers;  // <= 16 (rows of at most 1024 blocks)
        const uint32_t k0 = min(cnt, rt * per), k1 = min(cnt, k0 + per);
        bool inexact = nA == 0 || (two && nB == 0);
        IdxOp mine{0, 0, 0};
        for (uint32_t k = k0; k < k1; k++) mine = idx_compose<two>(mine, block_op(b + k, x + k, inexact), nA, nB);
        const uint32_t cA = S.carry[0], cB = S.carry[1];
        if (resolver_sync_or(inexact)) {
          // a delta at or above its palette size: the reference's sequential rule, on one thread
          if (rt == 0) {
            uint32_t iA = cA, iB = cB;
            for (uint32_t k = 0; k < cnt; k++) {
              const uint32_t w0 = bw0[b + k], ref = w0 & 3u;
              if (ref == 0) {
                iA += (w0 >> 2) & 0x3FFFu;
                if (iA >= nA) iA -= nA;
                if (two) {
                  iB += bw1[b + k] & 0xFFFFu;
                  if (iB >= nB) iB -= nB;
                }
              } else if (ref >= 2) {
                iA = rbA[x + k];
                iB = rbB[x + k];
              }
              // the row buffer holds 16-bit indices: larger ones are corrupt in any case
              if (iA > 0xFFFFu || iB > 0xFFFFu) badi = 1;
              iA &= 0xFFFFu;
              iB &= 0xFFFFu;
              rbA[x + k] = (uint16_t)iA;
              rbB[x + k] = (uint16_t)iB;
              const uint32_t sA = w0 >> 16, sB = two ? bw1[b + k] >> 16 : 0u;
              if (iA >= nA || sA >= nSA || (two && (iB >= nB || sB >= nSB))) badi = 1;
              if (vis_row && x + k < J.bx) {
                const uint64_t at = ((uint64_t)f * J.by + y) * J.bx + x + k;
                if (two) reinterpret_cast<uint64_t*>(J.rec)[at] = (uint64_t)(iA | (sA << 16)) | ((uint64_t)(iB | (sB << 16)) << 32);
                else reinterpret_cast<uint32_t*>(J.rec)[at] = iA | (sA << 16);
              }
            }
            S.carry[0] = iA;
            S.carry[1] = iB;
          }
        } else {
          // exclusive scan of the threads' compositions: warp shuffles, then the warp totals
          const uint32_t wi = rt >> 5;
          IdxOp inc = mine;
#pragma unroll
          for (uint32_t d = 1; d < 32; d <<= 1) {
            IdxOp o;
            o.set = __shfl_up_sync(0xFFFFFFFFu, inc.set, d);
            o.a = __shfl_up_sync(0xFFFFFFFFu, inc.a, d);
            o.b = __shfl_up_sync(0xFFFFFFFFu, inc.b, d);
            if (lane >= d) inc = idx_compose<two>(o, inc, nA, nB);
          }
          if (lane == 31) {
            S.scan[wi][0] = inc.set;
            S.scan[wi][1] = inc.a;
            S.scan[wi][2] = inc.b;
          }
          IdxOp ex;
          ex.set = __shfl_up_sync(0xFFFFFFFFu, inc.set, 1);
          ex.a = __shfl_up_sync(0xFFFFFFFFu, inc.a, 1);
          ex.b = __shfl_up_sync(0xFFFFFFFFu, inc.b, 1);
          if (lane == 0) ex = IdxOp{0, 0, 0};
          resolver_sync();
          IdxOp pre_op{0, 0, 0};
#pragma unroll
          for (uint32_t w = 0; w < kWResolvers / 32; w++)
            if (w < wi) pre_op = idx_compose<two>(pre_op, IdxOp{S.scan[w][0], S.scan[w][1], S.scan[w][2]}, nA, nB);
          pre_op = idx_compose<two>(pre_op, ex, nA, nB);
          uint32_t iA = pre_op.set ? pre_op.a : add_mod(cA, pre_op.a, nA);
          uint32_t iB = two ? (pre_op.set ? pre_op.b : add_mod(cB, pre_op.b, nB)) : 0u;
          bool dummy = false;
          for (uint32_t k = k0; k < k1; k++) {
            const IdxOp o = block_op(b + k, x + k, dummy);  // reads the row above before this thread's write
            iA = o.set ? o.a : add_mod(iA, o.a, nA);
            if (two) iB = o.set ? o.b : add_mod(iB, o.b, nB);
            rbA[x + k] = (uint16_t)iA;
            if (two) rbB[x + k] = (uint16_t)iB;
            const uint32_t w0 = bw0[b + k];
            const uint32_t sA = w0 >> 16, sB = two ? bw1[b + k] >> 16 : 0u;
            if (iA >= nA || sA >= nSA || (two && (iB >= nB || sB >= nSB))) badi = 1;
            if (vis_row && x + k < J.bx) {
              const uint64_t at = ((uint64_t)f * J.by + y) * J.bx + x + k;
              if (two) reinterpret_cast<uint64_t*>(J.rec)[at] = (uint64_t)(iA | (sA << 16)) | ((uint64_t)(iB | (sB << 16)) << 32);
              else reinterpret_cast<uint32_t*>(J.rec)[at] = iA | (sA << 16);
            }
            if (k + 1 == cnt) {
              S.carry[0] = iA;
              S.carry[1] = iB;
            }
          }
        }
        resolver_sync();  // row buffer and carry are complete before the next segment reads them
        b += cnt;
        x += cnt;
        if (x == W) {
          x = 0;
          r++;
        }
      }
      if (badi) atomicOr(&S.bad, 2u);
    }
    __syncthreads();
    done_at = S.done;
    if (done_at != kWNotDone && t >= done_at + 2) break;
  }
  if (tid == 0 && S.bad) atomicMax(status, (S.bad & 1u) ? (uint32_t)kStBadCode : (uint32_t)kStBadIndex);
}

// One CTA per large level stream (`jobs`, largest first).
__global__ void __launch_bounds__(kWThreads, 1) k_crn_decode_wide(const StreamJob* __restrict__ jobs,
                                                               uint32_t* __restrict__ status) {
  __shared__ WideShared S;
  const StreamJob J = jobs[blockIdx.x];
  switch (J.kind) {
    case kKDxt1: wide_level<kKDxt1>(J, S, status); break;
    case kKDxt5: wide_level<kKDxt5>(J, S, status); break;
    case kKDxn: wide_level<kKDxn>(J, S, status); break;
    default: wide_level<kKDxt5a>(J, S, status); break;
  }
}

// Palette entry index, clamped so that records left unwritten by a stream the decoder rejected
// as corrupt can never read outside the palette (valid records are already in range).
__device__ __forceinline__ uint32_t clamp_idx(uint32_t i, uint32_t n) { return i < n ? i : 0u; }

__device__ __forceinline__ uint2 alpha_words(const DevPalettes& pal, uint32_t r) {
  const uint64_t a = (uint64_t)__ldg(pal.alpha_ep + clamp_idx(r & 0xFFFFu, pal.n_aep)) |
                     (__ldg(pal.alpha_sel + clamp_idx(r >> 16, pal.n_asel)) << 16);
  return make_uint2((uint32_t)a, (uint32_t)(a >> 32));
}

// The expansion works on tiles of TILE consecutive blocks of one face of one level; each CTA
// takes one tile from a table built on the host (no per-CTA search). A thread handles
// TILE / kExpandThreads blocks: it first loads all its index records, then gathers the palette
// words, then stores, so each thread keeps several loads in flight. With STAGE, DXT1 tiles of at
// least kStageMin blocks first copy the two colour palettes into shared memory, so the per-block
// gathers hit shared memory instead of costing a 32-byte L2 sector per 4-byte word.
// 8-byte blocks (DXT1, DXT5A), pairs of blocks: thread t handles blocks first + 2 * (k * threads +
// t) and the next one. narrow_load reads the pass's index records, narrow_emit gathers the palette
// words and stores the blocks.
template <uint32_t kPer>
__device__ __forceinline__ void narrow_load(const ExpandJob& J, uint32_t first, uint32_t nblk, uint32_t (&r)[kPer]) {
  const uint32_t* rec = reinterpret_cast<const uint32_t*>(J.rec);
  const bool rec8 = ((uintptr_t)rec & 7) == 0;  // pairs of records (b0 even) are 8-byte aligned
#pragma unroll
  for (uint32_t k = 0; k < kPer / 2; k++) {
    const uint32_t b0 = first + 2 * (k * kExpandThreads + threadIdx.x);
    if (b0 + 1 < nblk && rec8) {
      const uint2 v = __ldg(reinterpret_cast<const uint2*>(rec + b0));
      r[2 * k] = v.x;
      r[2 * k + 1] = v.y;
    } else if (b0 + 1 < nblk) {
      r[2 * k] = __ldg(rec + b0);
      r[2 * k + 1] = __ldg(rec + b0 + 1);
    } else {
      r[2 * k] = b0 < nblk ? __ldg(rec + b0) : 0u;
      r[2 * k + 1] = 0u;
    }
  }
}

template <uint32_t kPer>
__device__ __forceinline__ void narrow_emit(const ExpandJob& J, uint32_t first, uint32_t nblk, const uint32_t (&r)[kPer],
                                            const uint32_t* s_ep, const uint32_t* s_sel) {
  const uint32_t kind = J.kind, bx = J.bx;
  const DevPalettes pal = J.pal;
  const bool flat = J.flat;
  uint2 w[kPer];
#pragma unroll
  for (uint32_t k = 0; k < kPer; k++) {
    if (kind == kKDxt1) {
      const uint32_t ei = clamp_idx(r[k] & 0xFFFFu, pal.n_cep), si = clamp_idx(r[k] >> 16, pal.n_csel);
      w[k] = s_ep ? make_uint2(s_ep[ei], s_sel[si]) : make_uint2(__ldg(pal.colour_ep + ei), __ldg(pal.colour_sel + si));
    } else {
      w[k] = alpha_words(pal, r[k]);
    }
  }
#pragma unroll
  for (uint32_t k = 0; k < kPer / 2; k++) {
    const uint32_t b0 = first + 2 * (k * kExpandThreads + threadIdx.x);
    if (b0 >= nblk) break;
    if (flat && J.vec && b0 + 1 < nblk) {
      __stcs(reinterpret_cast<uint4*>(J.dst + (uint64_t)b0 * 8),
             make_uint4(w[2 * k].x, w[2 * k].y, w[2 * k + 1].x, w[2 * k + 1].y));
    } else {
      for (uint32_t q = 0; q < 2 && b0 + q < nblk; q++) {
        const uint32_t bb = b0 + q, y = bb / bx, x = bb - y * bx;
        uint32_t* d = reinterpret_cast<uint32_t*>(J.dst + (uint64_t)y * J.pitch + (uint64_t)x * 8);
        d[0] = w[2 * k + q].x;
        d[1] = w[2 * k + q].y;
      }
    }
  }
}

// 8-byte blocks over [first, end) in passes of SUB blocks, the records of each pass brought into
// shared memory by one bulk TMA copy (cp.async.bulk on an mbarrier, two buffers: the copy for
// pass i + 1 is in flight while pass i gathers and stores). A copy starts at the pass's first
// record rounded down to 16 bytes (the face's records may start mid-line; the up to three records
// before it belong to the previous face of the same buffer) and ends at its last record rounded
// down to 16 bytes; the up to three records after that are read from global memory. Waits are
// bounded: a CTA whose wait runs out reads its records from global memory from then on (same
// output) and counts the event in g_expand_stage_timeouts. Copies still in flight when the CTA is
// done are drained with a separate, much longer bound (kExpandDrainPolls) that the test hook does
// not change; a drain that runs out is counted in g_expand_drain_failures.
constexpr uint32_t kExpandWaitLimit = 1u << 22;
constexpr uint32_t kExpandDrainPolls = 1u << 26;
__device__ uint32_t g_expand_wait_polls = kExpandWaitLimit;
__device__ unsigned int g_expand_stage_timeouts;
__device__ unsigned int g_expand_drain_failures;

__device__ __forceinline__ uint32_t shared_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

template <uint32_t SUB>
__device__ __forceinline__ void narrow_tma(const ExpandJob& J, uint32_t first, uint32_t end, const uint32_t* s_ep,
                                           const uint32_t* s_sel, uint32_t* s_rec, uint64_t* bars) {
  constexpr uint32_t kPer = SUB / kExpandThreads;
  constexpr uint32_t kBuf = SUB + 4;  // words per buffer: a pass plus up to 3 leading records
  const uint32_t nblk = J.bx * J.by;
  const uint32_t* rec = reinterpret_cast<const uint32_t*>(J.rec);
  // [A, B): the 16-byte aligned byte range staged for the pass starting at f
  auto range = [&](uint32_t f, uintptr_t& A, uintptr_t& B) {
    A = reinterpret_cast<uintptr_t>(rec + f) & ~(uintptr_t)15;
    B = reinterpret_cast<uintptr_t>(rec + min(end, f + SUB)) & ~(uintptr_t)15;
    if (B < A) B = A;
  };
  auto issue = [&](uint32_t f, uint32_t buf) {
    uintptr_t A, B;
    range(f, A, B);
    const uint32_t bytes = (uint32_t)(B - A), bar = shared_u32(&bars[buf]);
    if (!bytes) return;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     shared_u32(s_rec + buf * kBuf)), "l"(A), "r"(bytes), "r"(bar)
                 : "memory");
  };
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(shared_u32(&bars[0])) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(shared_u32(&bars[1])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  uint32_t issued0 = 0, issued1 = 0, waited0 = 0, waited1 = 0;  // copies per buffer (same in every thread)
  auto staged_bytes = [&](uint32_t f) {
    uintptr_t A, B;
    range(f, A, B);
    return (uint32_t)(B - A);
  };
  if (threadIdx.x == 0) issue(first, 0);
  if (staged_bytes(first)) issued0++;
  bool live = true;
  uint32_t i = 0;
  for (uint32_t f = first; f < end; f += SUB, i++) {
    const uint32_t buf = i & 1u;
    const uint32_t nf = f + SUB;
    if (live && nf < end) {
      if (threadIdx.x == 0) issue(nf, buf ^ 1u);
      if (staged_bytes(nf)) { if (buf) issued0++; else issued1++; }
    }
    uintptr_t A, B;
    range(f, A, B);
    if (live && B > A) {
      bool done = false;
      const uint32_t bar = shared_u32(&bars[buf]), parity = (buf ? waited1 : waited0) & 1u;
      const uint32_t polls = g_expand_wait_polls;
      for (uint32_t k = 0; k < polls && !done; k++) {
        uint32_t d;
        asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
                     : "=r"(d)
                     : "r"(bar), "r"(parity)
                     : "memory");
        done = d != 0;
      }
      live = __syncthreads_and(done) != 0;
      if (live) { if (buf) waited1++; else waited0++; }
      else if (threadIdx.x == 0) atomicAdd(&g_expand_stage_timeouts, 1u);
    }
    // records of this pass: staged words for [A, B), global memory for the rest
    const uint32_t* st = s_rec + buf * kBuf;
    uint32_t r[kPer];
#pragma unroll
    for (uint32_t k = 0; k < kPer / 2; k++) {
#pragma unroll
      for (uint32_t q = 0; q < 2; q++) {
        const uint32_t b = f + 2 * (k * kExpandThreads + threadIdx.x) + q;
        const uintptr_t addr = reinterpret_cast<uintptr_t>(rec + b);
        uint32_t v = 0;
        if (b < nblk) v = (live && addr >= A && addr < B) ? st[(addr - A) >> 2] : __ldg(rec + b);
        r[2 * k + q] = v;
      }
    }
    narrow_emit<kPer>(J, f, nblk, r, s_ep, s_sel);
    __syncthreads();  // this buffer is read by all threads before it is refilled
  }
  // copies still in flight (only after a timed-out wait) land before the CTA exits (bounded)
  for (uint32_t b = 0; b < 2; b++)
    if ((b ? issued1 > waited1 : issued0 > waited0) && threadIdx.x == 0) {
      const uint32_t bar = shared_u32(&bars[b]), parity = ((b ? issued1 : issued0) - 1) & 1u;
      bool landed = false;
      for (uint32_t k = 0; k < kExpandDrainPolls && !landed; k++) {
        uint32_t d;
        asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
                     : "=r"(d)
                     : "r"(bar), "r"(parity)
                     : "memory");
        landed = d != 0;
      }
      if (!landed) atomicAdd(&g_expand_drain_failures, 1u);
    }
}

// 8-byte blocks over [first, end) in passes of SUB blocks, the next pass's records loaded before
// this pass's palette gathers and stores, so two dependent round trips overlap.
template <uint32_t SUB>
__device__ __forceinline__ void narrow_pipelined(const ExpandJob& J, uint32_t first, uint32_t end, const uint32_t* s_ep,
                                                 const uint32_t* s_sel) {
  constexpr uint32_t kPer = SUB / kExpandThreads;
  const uint32_t nblk = J.bx * J.by;
  uint32_t ra[kPer], rb[kPer];
  narrow_load<kPer>(J, first, nblk, ra);
  for (uint32_t f = first; f < end; f += SUB) {
    const bool more = f + SUB < end;
    if (more) narrow_load<kPer>(J, f + SUB, nblk, rb);
    narrow_emit<kPer>(J, f, nblk, ra, s_ep, s_sel);
    if (!more) break;
#pragma unroll
    for (uint32_t k = 0; k < kPer; k++) ra[k] = rb[k];
  }
}

template <bool WIDE, uint32_t TILE>  // WIDE: 16-byte blocks (DXT5, DXN); else 8-byte blocks (DXT1, DXT5A)
__device__ __forceinline__ void expand_tile(const ExpandJob& J, uint32_t first, const uint32_t* s_ep,
                                            const uint32_t* s_sel) {
  constexpr uint32_t kPer = TILE / kExpandThreads;  // blocks per thread and pass
  const uint32_t kind = J.kind, bx = J.bx;
  const uint32_t nblk = bx * J.by;
  const DevPalettes pal = J.pal;
  const bool flat = J.flat;  // minimal pitch: the face is one contiguous array of blocks
  if (!WIDE) {
    uint32_t r[kPer];
    narrow_load<kPer>(J, first, nblk, r);
    narrow_emit<kPer>(J, first, nblk, r, s_ep, s_sel);
    (void)kind; (void)bx; (void)pal; (void)flat;
  } else {
    constexpr uint32_t kPerW = kPer / 2;  // 16-byte blocks: half as many per thread per pass
#pragma unroll 1
    for (uint32_t pass = 0; pass < 2; pass++) {
      const uint32_t base = first + pass * kPerW * kExpandThreads;
      uint64_t r[kPerW];
      const unsigned long long* rec = reinterpret_cast<const unsigned long long*>(J.rec);
#pragma unroll
      for (uint32_t k = 0; k < kPerW; k++) {
        const uint32_t bb = base + k * kExpandThreads + threadIdx.x;
        r[k] = bb < nblk ? __ldg(rec + bb) : 0ull;
      }
      uint4 o[kPerW];
#pragma unroll
      for (uint32_t k = 0; k < kPerW; k++) {
        const uint32_t rlo = (uint32_t)r[k], rhi = (uint32_t)(r[k] >> 32);
        if (kind == kKDxt5) {
          const uint2 a = alpha_words(pal, rhi);
          o[k] = make_uint4(a.x, a.y, __ldg(pal.colour_ep + clamp_idx(rlo & 0xFFFFu, pal.n_cep)),
                            __ldg(pal.colour_sel + clamp_idx(rlo >> 16, pal.n_csel)));
        } else {
          const uint2 a = alpha_words(pal, rlo), c = alpha_words(pal, rhi);
          o[k] = make_uint4(a.x, a.y, c.x, c.y);
        }
      }
#pragma unroll
      for (uint32_t k = 0; k < kPerW; k++) {
        const uint32_t bb = base + k * kExpandThreads + threadIdx.x;
        if (bb >= nblk) break;
        const uint32_t y = flat ? 0u : bb / bx, x = flat ? bb : bb - y * bx;
        uint32_t* d = reinterpret_cast<uint32_t*>(J.dst + (uint64_t)y * J.pitch + (uint64_t)x * 16);
        if (J.vec) __stcs(reinterpret_cast<uint4*>(d), o[k]);
        else { d[0] = o[k].x; d[1] = o[k].y; d[2] = o[k].z; d[3] = o[k].w; }
      }
    }
  }
}

// Dynamic shared memory (STAGE): the staged DXT1 colour palettes, smem_words = the largest
// n_cep + n_csel of the launch's DXT1 jobs. A CTA covers TILE blocks in passes of up to
// kSubBlocks, so a large tile pays for the palette copy once.
template <uint32_t TILE, bool STAGE, bool PIPE, uint32_t SUB = kSubBlocks, bool TMA = false>
__global__ void __launch_bounds__(kExpandThreads, TMA ? 4 : 1) k_crn_expand_tiles(const ExpandJob* __restrict__ jobs,
                                                                      const uint2* __restrict__ tiles,
                                                                      uint32_t smem_words) {
  // dynamic shared memory: [TMA: 2 record buffers of SUB + 4 words, 2 mbarriers][STAGE: palettes]
  extern __shared__ __align__(16) uint32_t s_dyn[];
  constexpr uint32_t kSub = TILE < SUB ? TILE : SUB;
  constexpr uint32_t kTmaWords = TMA ? 2 * (kSub + 4) + 4 : 0;
  uint32_t* s_rec = s_dyn;
  uint64_t* s_bars = reinterpret_cast<uint64_t*>(s_dyn + (TMA ? 2 * (kSub + 4) : 0));
  uint32_t* s_pal = s_dyn + kTmaWords;
  const uint2 t = tiles[blockIdx.x];  // (job, first block)
  const ExpandJob& J = jobs[t.x];
  const uint32_t nblk = J.bx * J.by;
  const uint32_t end = min(nblk, t.y + TILE);
  if (J.kind == kKDxt1) {
    const uint32_t n_ep = J.pal.n_cep, n_sel = J.pal.n_csel;
    const bool stage = STAGE && end - t.y >= kStageMin && n_ep + n_sel <= smem_words;  // uniform per CTA
    if (stage) {
      for (uint32_t i = threadIdx.x; i < n_ep; i += kExpandThreads) s_pal[i] = __ldg(J.pal.colour_ep + i);
      for (uint32_t i = threadIdx.x; i < n_sel; i += kExpandThreads) s_pal[n_ep + i] = __ldg(J.pal.colour_sel + i);
      __syncthreads();
      if (TMA) narrow_tma<kSub>(J, t.y, end, s_pal, s_pal + n_ep, s_rec, s_bars);
      else if (PIPE) narrow_pipelined<kSub>(J, t.y, end, s_pal, s_pal + n_ep);
      else for (uint32_t f = t.y; f < end; f += kSub) expand_tile<false, kSub>(J, f, s_pal, s_pal + n_ep);
    } else {
      if (TMA) narrow_tma<kSub>(J, t.y, end, nullptr, nullptr, s_rec, s_bars);
      else if (PIPE) narrow_pipelined<kSub>(J, t.y, end, nullptr, nullptr);
      else for (uint32_t f = t.y; f < end; f += kSub) expand_tile<false, kSub>(J, f, nullptr, nullptr);
    }
  } else if (J.kind == kKDxt5a) {
    if (TMA) narrow_tma<kSub>(J, t.y, end, nullptr, nullptr, s_rec, s_bars);
    else if (PIPE) narrow_pipelined<kSub>(J, t.y, end, nullptr, nullptr);
    else for (uint32_t f = t.y; f < end; f += kSub) expand_tile<false, kSub>(J, f, nullptr, nullptr);
  } else {
    for (uint32_t f = t.y; f < end; f += kSub) expand_tile<true, kSub>(J, f, nullptr, nullptr);
  }
}

// variant v < 12: tile of 1024 << (v >> 1) blocks, palettes staged when v is odd; v = 12..15: the
// 8192- and 16384-block tiles with the next pass's records loaded ahead (staged when v is odd);
// v = 16, 17: 16384- and 32768-block tiles, pipelined, 4096-block passes (16 blocks per thread);
// v = 18..20: 16384-block tiles (palettes staged when v = 19) and 32768-block tiles whose records
// come into shared memory by double-buffered TMA copies, 2048-block passes
typedef void (*ExpandKernel)(const ExpandJob*, const uint2*, uint32_t);
const ExpandKernel kExpandKernels[kExpandVariants] = {
    k_crn_expand_tiles<1024, false, false>,  k_crn_expand_tiles<1024, true, false>,
    k_crn_expand_tiles<2048, false, false>,  k_crn_expand_tiles<2048, true, false>,
    k_crn_expand_tiles<4096, false, false>,  k_crn_expand_tiles<4096, true, false>,
    k_crn_expand_tiles<8192, false, false>,  k_crn_expand_tiles<8192, true, false>,
    k_crn_expand_tiles<16384, false, false>, k_crn_expand_tiles<16384, true, false>,
    k_crn_expand_tiles<32768, false, false>, k_crn_expand_tiles<32768, true, false>,
    k_crn_expand_tiles<8192, false, true>,   k_crn_expand_tiles<8192, true, true>,
    k_crn_expand_tiles<16384, false, true>,  k_crn_expand_tiles<16384, true, true>,
    k_crn_expand_tiles<16384, false, true, 4096>, k_crn_expand_tiles<32768, false, true, 4096>,
    k_crn_expand_tiles<16384, false, false, kTmaSub, true>, k_crn_expand_tiles<16384, true, false, kTmaSub, true>,
    k_crn_expand_tiles<32768, false, false, kTmaSub, true>};
// the tile-table index (tile of 1024 << i blocks) of each variant
constexpr int kVariantTile[kExpandVariants] = {0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 3, 3, 4, 4, 4, 5, 4, 4, 5};
// whether a variant stages the DXT1 palettes in dynamic shared memory
constexpr bool kVariantStage[kExpandVariants] = {false, true, false, true, false, true,  false, true, false, true, false,
                                                 true,  false, true, false, true, false, false, false, true, false};
// dynamic shared memory of a variant's TMA record buffers and barriers (bytes)
constexpr uint32_t kVariantTmaBytes[kExpandVariants] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
                                                        (2 * (kTmaSub + 4) + 4) * 4, (2 * (kTmaSub + 4) + 4) * 4,
                                                        (2 * (kTmaSub + 4) + 4) * 4};
// per device: the autotuner's last choice (0 until tuned); atomic, as batches on several host
// threads read and write it
std::atomic<int> g_expand_variant[64] = {};

// ------------------------------------------------------------------------------------------
// Host side.

struct UnpackContext : HostObject {
  uint32_t magic = 0x43524E47u;
  int device = -1;
  CrnFile file;
  DevBuf d_file, d_models, d_pal, d_jobs, d_records, d_status;
  DevPalettes pal{};
  uint32_t status_host[2] = {0, 0};
  // every level decoded at minimal pitch by the first unpack_level call (0: not tried yet,
  // 1: holds every level, 2: not used for this context)
  DevBuf d_level_cache;
  int level_cache_state = 0;

  uint32_t kind() const { return (uint32_t)file.kind; }
  uint32_t rec_bytes() const { return record_bytes(kind()); }
};

namespace {

bool valid_ctx(const UnpackContext* c) { return c && c->magic == 0x43524E47u; }

// Palettes in the device layout, packed back to back with 16-byte alignment. `base` is the
// device address the image will be copied to; returns the image and fills *pal.
HVec<uint8_t> palette_image(const CrnFile& F, uint8_t* base, DevPalettes* pal) {
  auto al = [](size_t v) { return (v + 15) & ~(size_t)15; };
  const size_t n_cep = F.colour_ep.size(), n_csel = F.colour_sel.size();
  const size_t n_aep = F.alpha_ep.size(), n_asel = F.alpha_sel.size() / 3;
  const size_t o_csel = al(n_cep * 4), o_asel = o_csel + al(n_csel * 4), o_aep = o_asel + al(n_asel * 8);
  const size_t total = o_aep + al(n_aep * 2) + 16;
  HVec<uint8_t> host(total, 0);
  if (n_cep) std::memcpy(host.data(), F.colour_ep.data(), n_cep * 4);
  if (n_csel) std::memcpy(host.data() + o_csel, F.colour_sel.data(), n_csel * 4);
  for (size_t i = 0; i < n_asel; i++) {
    const uint64_t v = (uint64_t)F.alpha_sel[3 * i] | ((uint64_t)F.alpha_sel[3 * i + 1] << 16) |
                       ((uint64_t)F.alpha_sel[3 * i + 2] << 32);
    std::memcpy(host.data() + o_asel + 8 * i, &v, 8);
  }
  if (n_aep) std::memcpy(host.data() + o_aep, F.alpha_ep.data(), n_aep * 2);
  pal->colour_ep = reinterpret_cast<const uint32_t*>(base);
  pal->colour_sel = reinterpret_cast<const uint32_t*>(base + o_csel);
  pal->alpha_sel = reinterpret_cast<const uint64_t*>(base + o_asel);
  pal->alpha_ep = reinterpret_cast<const uint16_t*>(base + o_aep);
  pal->n_cep = (uint32_t)n_cep;
  pal->n_csel = (uint32_t)n_csel;
  pal->n_aep = (uint32_t)n_aep;
  pal->n_asel = (uint32_t)n_asel;
  return host;
}

size_t palette_bytes(const CrnFile& F) {
  auto al = [](size_t v) { return (v + 15) & ~(size_t)15; };
  return al(F.colour_ep.size() * 4) + al(F.colour_sel.size() * 4) + al(F.alpha_sel.size() / 3 * 8) +
         al(F.alpha_ep.size() * 2) + 16;
}

HVec<DevModel> model_image(const CrnFile& F) {
  HVec<DevModel> models(kNumModels);
  F.ref_dm.to_device(models[kMRef]);
  F.ep_dm[0].to_device(models[kMEp0]);
  F.sel_dm[0].to_device(models[kMSel0]);
  F.ep_dm[1].to_device(models[kMEp1]);
  F.sel_dm[1].to_device(models[kMSel1]);
  return models;
}

int upload_context(UnpackContext* c, const uint8_t* data, uint32_t size) {
  CrnFile& F = c->file;
  cudaError_t e = cudaGetDevice(&c->device);
  if (e != cudaSuccess) return cuda_check(e, "cudaGetDevice");
  // file bytes, padded so word reads near the end stay inside the allocation
  if ((e = c->d_file.ensure(size + 64)) != cudaSuccess) return cuda_check(e, "alloc file");
  if ((e = cudaMemcpy(c->d_file.ptr, data, size, cudaMemcpyHostToDevice)) != cudaSuccess)
    return cuda_check(e, "copy file");
  HVec<DevModel> models = model_image(F);
  if ((e = c->d_models.ensure(sizeof(DevModel) * kNumModels)) != cudaSuccess) return cuda_check(e, "alloc models");
  if ((e = cudaMemcpy(c->d_models.ptr, models.data(), sizeof(DevModel) * kNumModels, cudaMemcpyHostToDevice)) !=
      cudaSuccess)
    return cuda_check(e, "copy models");
  if ((e = c->d_pal.ensure(palette_bytes(F))) != cudaSuccess) return cuda_check(e, "alloc palettes");
  HVec<uint8_t> img = palette_image(F, static_cast<uint8_t*>(c->d_pal.ptr), &c->pal);
  if ((e = cudaMemcpy(c->d_pal.ptr, img.data(), img.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
    return cuda_check(e, "copy palettes");
  if ((e = c->d_status.ensure(16)) != cudaSuccess) return cuda_check(e, "alloc status");
  return CRNGPU_OK;
}

// One level of one file to decode and expand (all pointers device memory).
struct LevelTask {
  const CrnFile* file;
  const DevModel* models;
  DevPalettes pal;
  uint32_t level;
  uint8_t* dst[6];     // face pointers
  uint32_t pitch;
  const uint8_t* src;  // compressed level stream
  uint32_t src_size;
  uint8_t* rec;        // the level's index records (faces x blocks, record_bytes each)
  uint32_t item;       // texture job this level belongs to (one warp decodes a texture job)
};

// Launch plan: jobs image [TexJob x n_item][StreamJob x n_stream][ExpandJob x n_expand],
// built on the host. Tasks with the same `item` (consecutive) form one texture job.
struct Plan {
  HVec<uint8_t> image;
  uint32_t n_item = 0, n_stream = 0, n_expand = 0, ctas = 0;
  uint32_t n_wide = 0;      // level streams for k_crn_decode_wide (one CTA each, largest first)
  uint32_t wide_smem = 0;   // its dynamic shared memory (the largest format's layout)
  size_t wide_ofs = 0;
  uint32_t rb_words = 2;    // largest row-buffer need of one texture job (words)
  uint32_t lut_words = 0;   // first-level tables staged per texture job (words)
  size_t stream_ofs = 0, expand_ofs = 0;
  size_t tile_ofs[kTileSizes] = {};
  uint32_t tile_ctas[kTileSizes] = {};
  uint32_t pal_words = 0;   // shared memory of the expansion: largest staged DXT1 palette pair
};

uint64_t level_records(const CrnFile& F, uint32_t l) {
  return (uint64_t)F.level[l].blocks_x * F.level[l].blocks_y * F.faces;
}

// Which level streams go to k_crn_decode_wide. 0 (the default): the split that minimises the
// plan's decode time (decide_wide); otherwise levels of at least this many blocks (all faces) go
// to the wide decoder. Set by crngpu_set_decode_split (tests force either decoder on every level).
std::atomic<uint32_t> g_wide_min_blocks{0};

// Decode cost model, in microseconds per block for a one-endpoint format (twice that for DXT5 and
// DXN), measured on GB300: the lane decoder's serial chain and one wide CTA's phase loop.
constexpr double kLaneUsPerBlock = 0.20, kWideUsPerBlock = 0.03;
constexpr uint32_t kWideMinBlocks = 256;  // smaller levels always go to the lane decoder

uint64_t task_blocks(const LevelTask& t) {
  const LevelInfo& li = t.file->level[t.level];
  return (uint64_t)li.blocks_x * li.blocks_y * t.file->faces;
}

bool wide_eligible(const LevelTask& t) {
  const LevelInfo& li = t.file->level[t.level];
  // list items hold a bit position below 2^30, so the stream is below 2^27 bytes
  return ((li.blocks_x + 1) & ~1u) <= kWMaxW && t.src_size < (1u << 27);
}

// Per task: true if it goes to the wide decoder. The lane decoder runs every stream side by side
// and finishes with its longest stream; the wide decoder runs `wide_slots` CTAs at once and
// finishes when its queue drains, but never before its largest level. The two run one after the
// other on the caller's stream. With the levels sorted by cost, the first k go wide for the k that
// minimises wide time + lane time of level k + 1.
HVec<bool> decide_wide(const HVec<LevelTask>& tasks, uint32_t wide_slots) {
  HVec<bool> wide(tasks.size(), false);
  const uint32_t fixed = g_wide_min_blocks.load(std::memory_order_relaxed);
  if (fixed) {
    for (size_t i = 0; i < tasks.size(); i++) wide[i] = wide_eligible(tasks[i]) && task_blocks(tasks[i]) >= fixed;
    return wide;
  }
  HVec<std::pair<double, size_t>> cost;  // lane cost, task
  double lane_rest = 0;                         // longest lane stream among the ineligible ones
  for (size_t i = 0; i < tasks.size(); i++) {
    const double w = (tasks[i].file->kind == Kind::DXT5 || tasks[i].file->kind == Kind::DXN) ? 2.0 : 1.0;
    const double c = (double)task_blocks(tasks[i]) * w;
    if (wide_eligible(tasks[i]) && task_blocks(tasks[i]) >= kWideMinBlocks) cost.push_back({c, i});
    else lane_rest = std::max(lane_rest, c * kLaneUsPerBlock);
  }
  std::stable_sort(cost.begin(), cost.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
  double best = std::max(lane_rest, cost.empty() ? 0.0 : cost[0].first * kLaneUsPerBlock), sum = 0;
  constexpr double kWideLaunchUs = 10.0;  // a second kernel launch and its fixed set-up
  size_t best_k = 0;
  for (size_t k = 1; k <= cost.size(); k++) {
    sum += cost[k - 1].first * kWideUsPerBlock;
    const double wide_t = std::max(cost[0].first * kWideUsPerBlock, sum / std::max<uint32_t>(1, wide_slots));
    const double lane_t = std::max(lane_rest, k < cost.size() ? cost[k].first * kLaneUsPerBlock : 0.0);
    if (wide_t + lane_t + kWideLaunchUs < best) {
      best = wide_t + lane_t + kWideLaunchUs;
      best_k = k;
    }
  }
  for (size_t k = 0; k < best_k; k++) wide[cost[k].second] = true;
  return wide;
}

// false if a texture job would not fit the decoder (more than 32 levels or rows too wide).
// `wide_slots`: CTAs of k_crn_decode_wide resident at once on the device (wide_slots()).
bool make_plan(const HVec<LevelTask>& tasks, Plan& p, uint32_t wide_slots) {
  HVec<TexJob> items;
  HVec<HVec<StreamJob>> item_streams;
  HVec<StreamJob> wide;
  const HVec<bool> to_wide = decide_wide(tasks, wide_slots);
  for (size_t i = 0; i < tasks.size();) {
    size_t k = i;
    while (k < tasks.size() && tasks[k].item == tasks[i].item) k++;
    const CrnFile& F = *tasks[i].file;
    const uint32_t kind = (uint32_t)F.kind;
    const bool colour = kind == kKDxt1 || kind == kKDxt5;
    TexJob T{};
    T.models = tasks[i].models;
    T.kind = kind;
    HVec<StreamJob> sj;
    uint32_t rb = 0;
    for (size_t t = i; t < k; t++) {
      const LevelInfo& li = F.level[tasks[t].level];
      StreamJob j{};
      j.src = tasks[t].src;
      j.src_size = tasks[t].src_size;
      j.models = tasks[t].models;
      j.rec = tasks[t].rec;
      j.bx = li.blocks_x;
      j.by = li.blocks_y;
      j.faces = F.faces;
      j.kind = kind;
      j.n_a = colour ? tasks[t].pal.n_cep : tasks[t].pal.n_aep;
      j.n_b = tasks[t].pal.n_aep;
      j.n_sa = colour ? tasks[t].pal.n_csel : tasks[t].pal.n_asel;
      j.n_sb = tasks[t].pal.n_asel;
      if (to_wide[t]) {
        wide.push_back(j);
        continue;
      }
      j.rb_ofs = rb;
      rb += (li.blocks_x + 1) & ~1u;
      T.work = std::max<uint64_t>(T.work, (uint64_t)li.blocks_x * li.blocks_y * F.faces * (kind == kKDxt1 || kind == kKDxt5a ? 1 : 2));
      sj.push_back(j);
    }
    i = k;
    if (sj.empty()) continue;
    if (sj.size() > 32) return false;
    T.nlev = (uint32_t)sj.size();
    // the texture's longest streams first: the decoder gives each of the first few its own warp
    std::stable_sort(sj.begin(), sj.end(),
                     [](const StreamJob& a, const StreamJob& b) { return a.bx * a.by > b.bx * b.by; });
    T.rb_words = rb;
    p.rb_words = std::max(p.rb_words, rb);
    p.lut_words = std::max(p.lut_words, models_used(kind) << kLutBits);
    items.push_back(T);
    item_streams.push_back(std::move(sj));
  }
  // the largest wide levels first, so the longest chains start first
  std::stable_sort(wide.begin(), wide.end(), [](const StreamJob& a, const StreamJob& b) {
    return (uint64_t)a.bx * a.by * a.faces * record_bytes(a.kind) > (uint64_t)b.bx * b.by * b.faces * record_bytes(b.kind);
  });
  for (const StreamJob& j : wide) p.wide_smem = std::max(p.wide_smem, wide_layout(models_used(j.kind)).total);
  // largest textures first: the persistent warps then finish at about the same time
  HVec<size_t> order(items.size());
  for (size_t i = 0; i < order.size(); i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return items[a].work > items[b].work; });
  HVec<TexJob> it_sorted;
  HVec<StreamJob> sj;
  for (size_t o : order) {
    TexJob T = items[o];
    T.first = (uint32_t)sj.size();
    it_sorted.push_back(T);
    sj.insert(sj.end(), item_streams[o].begin(), item_streams[o].end());
  }
  HVec<ExpandJob> ej;
  HVec<uint2> tiles[kTileSizes];
  for (const LevelTask& t : tasks) {
    const CrnFile& F = *t.file;
    const LevelInfo& li = F.level[t.level];
    const uint32_t kind = (uint32_t)F.kind;
    const uint32_t nblk = li.blocks_x * li.blocks_y;
    for (uint32_t f = 0; f < F.faces; f++) {
      ExpandJob j;
      j.dst = t.dst[f];
      j.rec = t.rec + (uint64_t)f * nblk * record_bytes(kind);
      j.pal = t.pal;
      j.bx = li.blocks_x;
      j.by = li.blocks_y;
      j.pitch = t.pitch;
      j.kind = kind;
      j.flat = t.pitch == li.blocks_x * F.bytes_per_block ? 1u : 0u;
      j.vec = (((uintptr_t)t.dst[f] & 15) == 0 && (j.flat || (t.pitch & 15) == 0)) ? 1u : 0u;
      for (int ts = 0; ts < kTileSizes; ts++)
        for (uint32_t b = 0; b < nblk; b += 1024u << ts) tiles[ts].push_back(make_uint2((uint32_t)ej.size(), b));
      if (kind == kKDxt1 && nblk >= kStageMin)
        p.pal_words = std::max(p.pal_words, t.pal.n_cep + t.pal.n_csel);
      ej.push_back(j);
    }
  }
  p.n_item = (uint32_t)it_sorted.size();
  p.n_stream = (uint32_t)sj.size();
  p.n_expand = (uint32_t)ej.size();
  p.n_wide = (uint32_t)wide.size();
  p.ctas = (uint32_t)tiles[0].size();
  auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
  p.stream_ofs = al(sizeof(TexJob) * it_sorted.size());
  p.expand_ofs = p.stream_ofs + al(sizeof(StreamJob) * sj.size());
  p.wide_ofs = p.expand_ofs + al(sizeof(ExpandJob) * ej.size());
  size_t end = p.wide_ofs + al(sizeof(StreamJob) * wide.size());
  for (int ts = 0; ts < kTileSizes; ts++) {
    p.tile_ofs[ts] = end;
    p.tile_ctas[ts] = (uint32_t)tiles[ts].size();
    end += al(sizeof(uint2) * tiles[ts].size());
  }
  p.image.assign(end, 0);
  std::memcpy(p.image.data(), it_sorted.data(), sizeof(TexJob) * it_sorted.size());
  std::memcpy(p.image.data() + p.stream_ofs, sj.data(), sizeof(StreamJob) * sj.size());
  std::memcpy(p.image.data() + p.expand_ofs, ej.data(), sizeof(ExpandJob) * ej.size());
  if (!wide.empty()) std::memcpy(p.image.data() + p.wide_ofs, wide.data(), sizeof(StreamJob) * wide.size());
  for (int ts = 0; ts < kTileSizes; ts++)
    std::memcpy(p.image.data() + p.tile_ofs[ts], tiles[ts].data(), sizeof(uint2) * tiles[ts].size());
  return true;
}

// Per-device set-up of the transcoder kernels (shared-memory attributes) and the figures the
// plans need: SM count, shared memory per SM, and how many wide-decoder CTAs are resident at once.
struct DecodeDevice {
  int sms = 0, smem_sm = 0;
  uint32_t wide_slots = 0;
  bool ready = false;
};

int decode_device(const DecodeDevice** out) {
  static DecodeDevice devs[64];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_check(e, "cudaGetDevice");
  if (dev < 0 || dev >= 64) { set_error("device index out of range"); return CRNGPU_E_PARAM; }
  std::lock_guard<std::mutex> lock(device_setup_mutex());
  DecodeDevice& D = devs[dev];
  if (!D.ready) {
    if ((e = cudaDeviceGetAttribute(&D.sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
      return cuda_check(e, "device attribute");
    if ((e = cudaDeviceGetAttribute(&D.smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev)) != cudaSuccess)
      return cuda_check(e, "device attribute");
    if ((e = cudaFuncSetAttribute(k_crn_decode_textures, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kDecodeSmemMax)) != cudaSuccess)
      return cuda_check(e, "decoder shared memory attribute");
    if ((e = cudaFuncSetAttribute(k_crn_decode_wide, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)wide_layout(5).total)) != cudaSuccess)
      return cuda_check(e, "wide decoder shared memory attribute");
    for (int v = 0; v < kExpandVariants; v++)
      if ((kVariantStage[v] || kVariantTmaBytes[v]) &&
          (e = cudaFuncSetAttribute(kExpandKernels[v], cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)(kVariantTmaBytes[v] + (kVariantStage[v] ? 2 * kMaxSyms * sizeof(uint32_t) : 0)))) !=
              cudaSuccess)
        return cuda_check(e, "expansion shared memory attribute");
    int per_sm = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_crn_decode_wide, kWThreads,
                                                           wide_layout(3).total)) != cudaSuccess)
      return cuda_check(e, "wide decoder occupancy");
    D.wide_slots = (uint32_t)std::max(1, per_sm) * (uint32_t)D.sms;
    D.ready = true;
  }
  *out = &D;
  return CRNGPU_OK;
}

int wide_slots(uint32_t* slots) {
  const DecodeDevice* D = nullptr;
  const int rc = decode_device(&D);
  if (rc == CRNGPU_OK) *slots = D->wide_slots;
  return rc;
}

// Persistent decoder grid: CTAs of one warp, as many as shared memory lets reside on every SM.
int decode_grid(const Plan& p, uint32_t* grid, size_t* smem) {
  const DecodeDevice* D = nullptr;
  const int rc = decode_device(&D);
  if (rc != CRNGPU_OK) return rc;
  *smem = (size_t)(p.lut_words + p.rb_words) * sizeof(uint32_t);
  // CTAs of kDecodeWarps warps: at most 2048 / (32 kDecodeWarps) per SM, fewer if shared memory binds
  const uint32_t per_sm = std::max<uint32_t>(
      1, std::min<uint32_t>(2048 / (32 * kDecodeWarps), (uint32_t)(D->smem_sm / (*smem + 1024))));
  *grid = std::max<uint32_t>(1, std::min<uint32_t>(p.n_item, per_sm * (uint32_t)D->sms));
  return CRNGPU_OK;
}

// Enqueues the counter/status clear, the decoder and the expansion for a plan whose image is
// already at d_jobs. `words` = 2 device words: [0] work counter, [1] status. Asynchronous.
int enqueue_plan(const Plan& p, const uint8_t* d_jobs, uint32_t* words, cudaStream_t s, bool decode = true,
                 int variant = -1) {
  if ((size_t)(p.lut_words + p.rb_words) * 4 > kDecodeSmemMax) {
    set_error("texture rows too wide for the decoder");
    return CRNGPU_E_PARAM;
  }
  uint32_t grid = 0;
  size_t smem = 0;
  int rc = decode_grid(p, &grid, &smem);
  if (rc != CRNGPU_OK) return rc;
  cudaError_t e;
  const TexJob* tj = reinterpret_cast<const TexJob*>(d_jobs);
  const StreamJob* sj = reinterpret_cast<const StreamJob*>(d_jobs + p.stream_ofs);
  const ExpandJob* ej = reinterpret_cast<const ExpandJob*>(d_jobs + p.expand_ofs);
  if (decode && (p.n_item || p.n_wide)) {
    if ((e = cudaMemsetAsync(words, 0, 8, s)) != cudaSuccess) return cuda_check(e, "clear work counter");
  }
  if (decode && p.n_wide) {
    const StreamJob* wj = reinterpret_cast<const StreamJob*>(d_jobs + p.wide_ofs);
    k_crn_decode_wide<<<p.n_wide, kWThreads, p.wide_smem, s>>>(wj, words + 1);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(e, "launch k_crn_decode_wide");
  }
  if (decode && p.n_item) {
    k_crn_decode_textures<<<grid, kDecodeWarps * 32, smem, s>>>(tj, p.n_item, sj, words, p.lut_words, p.rb_words,
                                                             words + 1);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(e, "launch k_crn_decode_textures");
  }
  if (p.ctas) {
    int dev = 0;
    cudaGetDevice(&dev);
    const int v = variant >= 0 ? variant : g_expand_variant[dev & 63].load(std::memory_order_relaxed);
    const int ts = kVariantTile[v];
    const uint2* tiles = reinterpret_cast<const uint2*>(d_jobs + p.tile_ofs[ts]);
    const size_t smem = kVariantTmaBytes[v] + (kVariantStage[v] ? (size_t)p.pal_words * 4 : 0);
    kExpandKernels[v]<<<p.tile_ctas[ts], kExpandThreads, smem, s>>>(ej, tiles, p.pal_words);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(e, "launch k_crn_expand_tiles");
  }
  return CRNGPU_OK;
}

int status_to_rc(uint32_t st) {
  if (!st) return CRNGPU_OK;
  set_error(st == kStBadCode ? "corrupt block stream (no such prefix code)"
                             : "corrupt block stream (palette index out of range)");
  return CRNGPU_E_CORRUPT;
}

// Decodes and expands a list of levels of one context (destinations device memory), then
// reads the status word back (synchronises `s`).
int run_levels(UnpackContext* c, HVec<LevelTask>& tasks, cudaStream_t s) {
  // one record buffer for all levels, each level's records starting on a 16-byte boundary
  uint64_t rec = 0;
  for (LevelTask& t : tasks) rec += (level_records(c->file, t.level) * c->rec_bytes() + 15) & ~(uint64_t)15;
  cudaError_t e = c->d_records.ensure(rec + 16);
  if (e != cudaSuccess) return cuda_check(e, "alloc records");
  uint64_t ofs = 0;
  for (LevelTask& t : tasks) {
    t.rec = static_cast<uint8_t*>(c->d_records.ptr) + ofs;
    ofs += (level_records(c->file, t.level) * c->rec_bytes() + 15) & ~(uint64_t)15;
  }
  Plan p;
  uint32_t slots = 0;
  int rc0 = wide_slots(&slots);
  if (rc0 != CRNGPU_OK) return rc0;
  if (!make_plan(tasks, p, slots)) { set_error("too many levels in one texture job"); return CRNGPU_E_PARAM; }
  if ((e = c->d_jobs.ensure(p.image.size() + 16)) != cudaSuccess) return cuda_check(e, "alloc jobs");
  if ((e = cudaMemcpyAsync(c->d_jobs.ptr, p.image.data(), p.image.size(), cudaMemcpyHostToDevice, s)) != cudaSuccess)
    return cuda_check(e, "copy jobs");
  uint32_t* words = static_cast<uint32_t*>(c->d_status.ptr);
  int rc = enqueue_plan(p, static_cast<const uint8_t*>(c->d_jobs.ptr), words, s);
  if (rc != CRNGPU_OK) return rc;
  // the reference reports a bad stream through its bool result; read the status word back
  if ((e = cudaMemcpyAsync(c->status_host, words, 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
    return cuda_check(e, "read status");
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_check(e, "sync");
  return status_to_rc(c->status_host[1]);
}

LevelTask context_task(UnpackContext* c, uint32_t level) {
  LevelTask t{};
  t.file = &c->file;
  t.models = static_cast<const DevModel*>(c->d_models.ptr);
  t.pal = c->pal;
  t.level = level;
  t.src = static_cast<const uint8_t*>(c->d_file.ptr) + c->file.level[level].ofs;
  t.src_size = c->file.level[level].size;
  return t;
}

uint64_t levels_bytes(const CrnFile& F, uint32_t first, uint32_t count);
void levels_tasks(UnpackContext* c, uint32_t first, uint32_t count, uint8_t* out, uint32_t item,
                  HVec<LevelTask>& tasks);

// crnd_unpack_level is called a level at a time, usually for every level of a file in turn. The
// first call on a context decodes every level in one plan into a device cache -- the levels'
// streams decode side by side, so that costs about what the largest level alone does -- and this
// call and the later ones copy their level out of it. A file with a level the decoder rejects
// (the error must belong to the level asked for), or whose levels take more than
// kLevelCacheMax bytes, is decoded a level per call instead.
constexpr uint64_t kLevelCacheMax = 64ull << 20;
constexpr int kNoLevelCache = 1;  // not a status: the caller decodes the level itself

int cached_level(UnpackContext* c, uint32_t level, void** dst_faces, uint32_t row_pitch, int mem, cudaStream_t s) {
  const CrnFile& F = c->file;
  if (c->level_cache_state == 0) {
    c->level_cache_state = 2;  // until the decode below succeeds
    const uint64_t total = levels_bytes(F, 0, F.levels);
    if (total > kLevelCacheMax) return kNoLevelCache;
    if (c->d_level_cache.ensure(total) != cudaSuccess) {
      cudaGetLastError();
      return kNoLevelCache;
    }
    HVec<LevelTask> tasks;
    levels_tasks(c, 0, F.levels, static_cast<uint8_t*>(c->d_level_cache.ptr), 0, tasks);
    const int rc = run_levels(c, tasks, s);
    if (rc == CRNGPU_E_DEVICE) return rc;
    if (rc != CRNGPU_OK) {
      clear_error();
      return kNoLevelCache;
    }
    c->level_cache_state = 1;
  }
  if (c->level_cache_state != 1) return kNoLevelCache;
  const LevelInfo& li = F.level[level];
  const uint32_t minimal = li.blocks_x * F.bytes_per_block;
  const uint64_t face_bytes = (uint64_t)minimal * li.blocks_y;
  const uint8_t* src = static_cast<const uint8_t*>(c->d_level_cache.ptr) + levels_bytes(F, 0, level);
  const cudaMemcpyKind kind = mem == CRNGPU_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  cudaError_t e;
  // row padding beyond the minimal pitch keeps the caller's bytes, as the decoder leaves it
  for (uint32_t f = 0; f < F.faces; f++)
    if ((e = cudaMemcpy2DAsync(dst_faces[f], row_pitch, src + face_bytes * f, minimal, minimal, li.blocks_y, kind, s)) !=
        cudaSuccess)
      return cuda_check(e, "copy level");
  return cuda_check(cudaStreamSynchronize(s), "sync");
}

// Shared implementation of crngpu_unpack_level / _segmented.
int unpack_one(UnpackContext* c, const uint8_t* host_src, const uint8_t* dev_src, uint32_t src_size,
               void** dst_faces, uint32_t dst_size, uint32_t row_pitch, uint32_t level, int mem, void* stream) {
  if (!valid_ctx(c) || !dst_faces || level >= c->file.levels || dst_size < 8) {
    set_error("bad context, destination or level");
    return CRNGPU_E_PARAM;
  }
  const CrnFile& F = c->file;
  const LevelInfo& li = F.level[level];
  const uint32_t minimal = li.blocks_x * F.bytes_per_block;
  if (!row_pitch) row_pitch = minimal;
  else if (row_pitch < minimal || (row_pitch & 3)) { set_error("bad row pitch"); return CRNGPU_E_PARAM; }
  const uint64_t face_bytes = (uint64_t)row_pitch * li.blocks_y;
  if (dst_size < face_bytes) { set_error("destination too small"); return CRNGPU_E_PARAM; }
  for (uint32_t f = 0; f < F.faces; f++)
    if (!dst_faces[f]) { set_error("NULL face pointer"); return CRNGPU_E_PARAM; }
  cudaStream_t s = as_stream(stream);
  cudaError_t e;
  if (F.segmented && !dev_src && !host_src) {
    set_error("segmented file: pass the level data (crngpu_unpack_level_segmented)");
    return CRNGPU_E_PARAM;
  }
  if (!dev_src && !host_src) {
    const int rc = cached_level(c, level, dst_faces, row_pitch, mem, s);
    if (rc != kNoLevelCache) return rc;
  }
  LevelTask t = context_task(c, level);
  t.pitch = row_pitch;
  if (dev_src) { t.src = dev_src; t.src_size = src_size; }
  else if (host_src) {
    DevBuf& sb = staging(2);
    if ((e = sb.ensure(src_size + 64)) != cudaSuccess) return cuda_check(e, "alloc segment");
    if ((e = cudaMemcpyAsync(sb.ptr, host_src, src_size, cudaMemcpyHostToDevice, s)) != cudaSuccess)
      return cuda_check(e, "copy segment");
    t.src = static_cast<const uint8_t*>(sb.ptr);
    t.src_size = src_size;
  }
  DevBuf* out_stage = nullptr;
  if (mem == CRNGPU_MEM_DEVICE) {
    for (uint32_t f = 0; f < F.faces; f++) t.dst[f] = static_cast<uint8_t*>(dst_faces[f]);
  } else {
    out_stage = &staging(1);
    if ((e = out_stage->ensure(face_bytes * F.faces)) != cudaSuccess) return cuda_check(e, "alloc output stage");
    for (uint32_t f = 0; f < F.faces; f++) t.dst[f] = static_cast<uint8_t*>(out_stage->ptr) + face_bytes * f;
    // rows may have pitch padding the transcoder does not write: keep the caller's bytes there
    if (row_pitch != minimal)
      for (uint32_t f = 0; f < F.faces; f++)
        if ((e = cudaMemcpyAsync(t.dst[f], dst_faces[f], face_bytes, cudaMemcpyHostToDevice, s)) != cudaSuccess)
          return cuda_check(e, "stage output");
  }
  HVec<LevelTask> tasks{t};
  int rc = run_levels(c, tasks, s);
  if (rc != CRNGPU_OK) return rc;
  if (out_stage) {
    for (uint32_t f = 0; f < F.faces; f++)
      if ((e = cudaMemcpyAsync(dst_faces[f], tasks[0].dst[f], face_bytes, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return cuda_check(e, "copy output");
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_check(e, "sync");
  }
  return CRNGPU_OK;
}

// Output bytes of levels [first, first + count) at minimal pitch.
uint64_t levels_bytes(const CrnFile& F, uint32_t first, uint32_t count) {
  uint64_t total = 0;
  for (uint32_t l = first; l < first + count; l++)
    total += (uint64_t)F.level[l].blocks_x * F.bytes_per_block * F.level[l].blocks_y * F.faces;
  return total;
}

// Level tasks writing levels [first, first + count) back to back at `out` (minimal pitch).
void levels_tasks(UnpackContext* c, uint32_t first, uint32_t count, uint8_t* out, uint32_t item,
                  HVec<LevelTask>& tasks) {
  const CrnFile& F = c->file;
  uint64_t ofs = 0;
  for (uint32_t l = first; l < first + count; l++) {
    LevelTask t = context_task(c, l);
    t.item = item;
    t.pitch = F.level[l].blocks_x * F.bytes_per_block;
    const uint64_t face_bytes = (uint64_t)t.pitch * F.level[l].blocks_y;
    for (uint32_t f = 0; f < F.faces; f++) t.dst[f] = out + ofs + f * face_bytes;
    ofs += face_bytes * F.faces;
    tasks.push_back(t);
  }
}

}  // namespace

// Test hook for the expansion's staging waits: polls per wait (drains are not affected).
int set_expand_wait_polls(uint32_t polls) {
  return cuda_check(cudaMemcpyToSymbol(g_expand_wait_polls, &polls, sizeof(polls)), "set expansion wait polls");
}

// out[0]: staging waits that ran out, out[1]: drains that ran out; reset clears both.
int expand_wait_counters(uint32_t out[2], bool reset) {
  cudaError_t e = cudaMemcpyFromSymbol(&out[0], g_expand_stage_timeouts, sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemcpyFromSymbol(&out[1], g_expand_drain_failures, sizeof(uint32_t));
  if (e == cudaSuccess && reset) {
    const uint32_t z = 0;
    e = cudaMemcpyToSymbol(g_expand_stage_timeouts, &z, sizeof(z));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_expand_drain_failures, &z, sizeof(z));
  }
  return cuda_check(e, "read expansion wait counters");
}


// A prepared batch: many levels of many contexts, decoded by one persistent launch and expanded
// by one more. The job tables and record buffer are uploaded/allocated once at creation, so a
// launch only enqueues a memset and two kernels (and can replay as a CUDA graph).
struct UnpackBatch : HostObject {
  uint32_t magic = 0x42415443u;
  int device = -1;
  Plan plan;
  DevBuf d_jobs, d_records, d_words;
  uint32_t words_host[2] = {0, 0};
  cudaGraphExec_t graph = nullptr;
  bool decoded = false;
  int variant = -1;          // expansion variant chosen by the autotuner
  float variant_ms[kExpandVariants] = {};
  uint64_t out_bytes = 0;
  ~UnpackBatch() {
    if (graph) cudaGraphExecDestroy(graph);
  }
};

}  // namespace crngpu

using namespace crngpu;

extern "C" crngpu_unpack_context crngpu_unpack_begin(const void* data, uint32_t data_size) try {
  clear_error();
  if (!data) { set_error("NULL data"); return nullptr; }
  std::unique_ptr<UnpackContext> c(new UnpackContext());
  if (!c->file.parse(static_cast<const uint8_t*>(data), data_size)) {
    set_error(c->file.error);
    return nullptr;
  }
  if (upload_context(c.get(), static_cast<const uint8_t*>(data), data_size) != CRNGPU_OK) return nullptr;
  return reinterpret_cast<crngpu_unpack_context>(c.release());
} catch (...) {
  crngpu::exception_status();
  return nullptr;
}

extern "C" int crngpu_get_info(crngpu_unpack_context ctx, uint32_t* width, uint32_t* height, uint32_t* levels,
                               uint32_t* faces, uint32_t* format, uint32_t* bytes_per_block) try {
  UnpackContext* c = reinterpret_cast<UnpackContext*>(ctx);
  if (!valid_ctx(c)) return CRNGPU_E_PARAM;
  if (width) *width = c->file.width;
  if (height) *height = c->file.height;
  if (levels) *levels = c->file.levels;
  if (faces) *faces = c->file.faces;
  if (format) *format = c->file.format;
  if (bytes_per_block) *bytes_per_block = c->file.bytes_per_block;
  return CRNGPU_OK;
} catch (...) {
  return crngpu::exception_status();
}

extern "C" int crngpu_unpack_level(crngpu_unpack_context ctx, void** dst_faces, uint32_t dst_size_in_bytes,
                                   uint32_t row_pitch_in_bytes, uint32_t level_index, int mem, void* stream) try {
  clear_error();
  return unpack_one(reinterpret_cast<UnpackContext*>(ctx), nullptr, nullptr, 0, dst_faces, dst_size_in_bytes,
                    row_pitch_in_bytes, level_index, mem, stream);
} catch (...) {
  return crngpu::exception_status();
}

extern "C" int crngpu_unpack_level_segmented(crngpu_unpack_context ctx, const void* src, uint32_t src_size_in_bytes,
                                             void** dst_faces, uint32_t dst_size_in_bytes,
                                             uint32_t row_pitch_in_bytes, uint32_t level_index, int mem,
                                             void* stream) try {
  clear_error();
  if (!src || !src_size_in_bytes) { set_error("NULL segment"); return CRNGPU_E_PARAM; }
  const uint8_t* s = static_cast<const uint8_t*>(src);
  return unpack_one(reinterpret_cast<UnpackContext*>(ctx), mem == CRNGPU_MEM_DEVICE ? nullptr : s,
                    mem == CRNGPU_MEM_DEVICE ? s : nullptr, src_size_in_bytes, dst_faces, dst_size_in_bytes,
                    row_pitch_in_bytes, level_index, mem, stream);
} catch (...) {
  return crngpu::exception_status();
}

extern "C" int64_t crngpu_unpack_levels(crngpu_unpack_context ctx, uint32_t first_level, uint32_t level_count,
                                        void* dst, uint64_t dst_size, int mem, void* stream) try {
  clear_error();
  UnpackContext* c = reinterpret_cast<UnpackContext*>(ctx);
  if (!valid_ctx(c) || !dst || !level_count || first_level + level_count > c->file.levels || c->file.segmented) {
    set_error("bad context, destination or level range (or a segmented file)");
    return CRNGPU_E_PARAM;
  }
  const uint64_t total = levels_bytes(c->file, first_level, level_count);
  if (dst_size < total) { set_error("destination too small"); return CRNGPU_E_PARAM; }
  cudaStream_t s = as_stream(stream);
  cudaError_t e;
  uint8_t* out = static_cast<uint8_t*>(dst);
  DevBuf* stage = nullptr;
  if (mem != CRNGPU_MEM_DEVICE) {
    stage = &staging(1);
    if ((e = stage->ensure(total)) != cudaSuccess) return cuda_check(e, "alloc output stage");
    out = static_cast<uint8_t*>(stage->ptr);
  }
  HVec<LevelTask> tasks;
  levels_tasks(c, first_level, level_count, out, 0, tasks);
  int rc = run_levels(c, tasks, s);
  if (rc != CRNGPU_OK) return rc;
  if (stage) {
    if ((e = cudaMemcpyAsync(dst, stage->ptr, total, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
      return cuda_check(e, "copy output");
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_check(e, "sync");
  }
  return (int64_t)total;
} catch (...) {
  return crngpu::exception_status();
}

extern "C" crngpu_unpack_batch crngpu_unpack_batch_create(const crngpu_unpack_batch_item* items, uint32_t n) try {
  clear_error();
  if (!items || !n) { set_error("empty batch"); return nullptr; }
  std::unique_ptr<UnpackBatch> b(new UnpackBatch());
  cudaError_t e = cudaGetDevice(&b->device);
  if (e != cudaSuccess) { cuda_check(e, "cudaGetDevice"); return nullptr; }
  HVec<LevelTask> tasks;
  uint64_t rec = 0;
  for (uint32_t i = 0; i < n; i++) {
    UnpackContext* c = reinterpret_cast<UnpackContext*>(items[i].ctx);
    if (!valid_ctx(c) || !items[i].dst || !items[i].level_count ||
        items[i].first_level + items[i].level_count > c->file.levels || c->device != b->device ||
        c->file.segmented) {
      set_error("batch item " + std::to_string(i) + ": bad context, destination, level range, device or a segmented file");
      return nullptr;
    }
    const uint64_t need = levels_bytes(c->file, items[i].first_level, items[i].level_count);
    if (items[i].dst_size < need) {
      set_error("batch item " + std::to_string(i) + ": destination too small");
      return nullptr;
    }
    b->out_bytes += need;
    const size_t first = tasks.size();
    levels_tasks(c, items[i].first_level, items[i].level_count, static_cast<uint8_t*>(items[i].dst), i, tasks);
    for (size_t k = first; k < tasks.size(); k++) {
      rec = (rec + 15) & ~(uint64_t)15;
      tasks[k].rec = reinterpret_cast<uint8_t*>(rec);  // offset for now; rebased below
      rec += level_records(c->file, tasks[k].level) * c->rec_bytes();
    }
  }
  if ((e = b->d_records.ensure(rec + 16)) != cudaSuccess) { cuda_check(e, "alloc records"); return nullptr; }
  for (LevelTask& t : tasks) t.rec = static_cast<uint8_t*>(b->d_records.ptr) + reinterpret_cast<uintptr_t>(t.rec);
  uint32_t slots = 0;
  if (wide_slots(&slots) != CRNGPU_OK) return nullptr;
  if (!make_plan(tasks, b->plan, slots)) { set_error("too many levels in one batch item"); return nullptr; }
  if ((e = b->d_jobs.ensure(b->plan.image.size() + 16)) != cudaSuccess) { cuda_check(e, "alloc jobs"); return nullptr; }
  if ((e = cudaMemcpy(b->d_jobs.ptr, b->plan.image.data(), b->plan.image.size(), cudaMemcpyHostToDevice)) !=
      cudaSuccess) {
    cuda_check(e, "copy jobs");
    return nullptr;
  }
  if ((e = b->d_words.ensure(16)) != cudaSuccess) { cuda_check(e, "alloc status"); return nullptr; }
  // resolve the decoder's launch shape (and its shared-memory attribute) outside any capture
  uint32_t grid = 0;
  size_t smem = 0;
  if (decode_grid(b->plan, &grid, &smem) != CRNGPU_OK) return nullptr;
  return reinterpret_cast<crngpu_unpack_batch>(b.release());
} catch (...) {
  crngpu::exception_status();
  return nullptr;
}

extern "C" int crngpu_unpack_batch_launch(crngpu_unpack_batch batch, uint32_t flags, void* stream) try {
  clear_error();
  UnpackBatch* b = reinterpret_cast<UnpackBatch*>(batch);
  if (!b || b->magic != 0x42415443u) { set_error("bad batch"); return CRNGPU_E_PARAM; }
  if (flags & ~(uint32_t)(CRNGPU_BATCH_GRAPH | CRNGPU_BATCH_EXPAND_ONLY)) { set_error("unknown flags"); return CRNGPU_E_PARAM; }
  cudaStream_t s = as_stream(stream);
  const uint8_t* jobs = static_cast<const uint8_t*>(b->d_jobs.ptr);
  uint32_t* words = static_cast<uint32_t*>(b->d_words.ptr);
  if (b->variant < 0) {
    // autotuner: decode once, then time every expansion variant on the real records (each writes
    // the same, correct output) and keep the fastest for this batch and as the device default
    int rc = enqueue_plan(b->plan, jobs, words, s, true, 0);
    if (rc != CRNGPU_OK) return rc;
    cudaEvent_t ev[2];
    cudaError_t e;
    if ((e = cudaEventCreate(&ev[0])) != cudaSuccess || (e = cudaEventCreate(&ev[1])) != cudaSuccess)
      return cuda_check(e, "events");
    float best = 3.4e38f;
    int bv = 0;
    for (int v = 0; v < kExpandVariants; v++) {
      float tot = 0.f;
      for (int rep = 0; rep < 3; rep++) {
        cudaEventRecord(ev[0], s);
        if ((rc = enqueue_plan(b->plan, jobs, words, s, false, v)) != CRNGPU_OK) break;
        cudaEventRecord(ev[1], s);
        cudaEventSynchronize(ev[1]);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev[0], ev[1]);
        if (rep) tot += ms;  // the first run of each variant warms it up
      }
      if (rc != CRNGPU_OK) break;
      b->variant_ms[v] = tot / 2;
      if (tot < best) { best = tot; bv = v; }
    }
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    if (rc != CRNGPU_OK) return rc;
    b->variant = bv;
    g_expand_variant[b->device & 63].store(bv, std::memory_order_relaxed);
    b->decoded = true;
  }
  if (flags & CRNGPU_BATCH_EXPAND_ONLY) {
    if (!b->decoded) { set_error("no decode has run on this batch"); return CRNGPU_E_PARAM; }
    return enqueue_plan(b->plan, jobs, words, s, false, b->variant);
  }
  b->decoded = true;
  if (!(flags & CRNGPU_BATCH_GRAPH)) return enqueue_plan(b->plan, jobs, words, s, true, b->variant);
  cudaError_t e;
  if (!b->graph) {
    // capture on a private stream (the legacy default stream cannot be captured), then replay
    cudaStream_t cap;
    if ((e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking)) != cudaSuccess) return cuda_check(e, "stream");
    cudaGraph_t g = nullptr;
    if ((e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) {
      cudaStreamDestroy(cap);
      return cuda_check(e, "begin capture");
    }
    int rc = enqueue_plan(b->plan, jobs, words, cap, true, b->variant);
    e = cudaStreamEndCapture(cap, &g);
    cudaStreamDestroy(cap);
    if (rc != CRNGPU_OK) { if (g) cudaGraphDestroy(g); return rc; }
    if (e != cudaSuccess) return cuda_check(e, "end capture");
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { b->graph = nullptr; return cuda_check(e, "instantiate graph"); }
  }
  if ((e = cudaGraphLaunch(b->graph, s)) != cudaSuccess) return cuda_check(e, "graph launch");
  return CRNGPU_OK;
} catch (...) {
  return crngpu::exception_status();
}

extern "C" int crngpu_unpack_batch_set_variant(crngpu_unpack_batch batch, int32_t variant) try {
  clear_error();
  UnpackBatch* b = reinterpret_cast<UnpackBatch*>(batch);
  if (!b || b->magic != 0x42415443u) { set_error("bad batch"); return CRNGPU_E_PARAM; }
  if (variant < -1 || variant >= kExpandVariants) { set_error("no such expansion variant"); return CRNGPU_E_PARAM; }
  b->variant = variant;  // -1: autotune again at the next launch
  if (b->graph) {        // a captured graph holds the old variant's launch
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  return CRNGPU_OK;
} catch (...) {
  return crngpu::exception_status();
}

extern "C" int crngpu_unpack_batch_status(crngpu_unpack_batch batch, void* stream) try {
  clear_error();
  UnpackBatch* b = reinterpret_cast<UnpackBatch*>(batch);
  if (!b || b->magic != 0x42415443u) { set_error("bad batch"); return CRNGPU_E_PARAM; }
  cudaStream_t s = as_stream(stream);
  cudaError_t e = cudaMemcpyAsync(b->words_host, b->d_words.ptr, 8, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return cuda_check(e, "read status");
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_check(e, "sync");
  return status_to_rc(b->words_host[1]);
} catch (...) {
  return crngpu::exception_status();
}

extern "C" int crngpu_unpack_batch_tuning(crngpu_unpack_batch batch, int32_t* variant, float* ms, uint32_t n) try {
  UnpackBatch* b = reinterpret_cast<UnpackBatch*>(batch);
  if (!b || b->magic != 0x42415443u) return CRNGPU_E_PARAM;
  if (variant) *variant = b->variant;
  for (uint32_t i = 0; ms && i < n && i < (uint32_t)kExpandVariants; i++) ms[i] = b->variant_ms[i];
  return kExpandVariants;
} catch (...) {
  return crngpu::exception_status();
}

extern "C" int64_t crngpu_unpack_batch_bytes(crngpu_unpack_batch batch) try {
  UnpackBatch* b = reinterpret_cast<UnpackBatch*>(batch);
  if (!b || b->magic != 0x42415443u) return CRNGPU_E_PARAM;
  return (int64_t)b->out_bytes;
} catch (...) {
  return crngpu::exception_status();
}

extern "C" int crngpu_set_decode_split(uint32_t min_blocks) try {
  clear_error();
  g_wide_min_blocks.store(min_blocks, std::memory_order_relaxed);
  return CRNGPU_OK;
} catch (...) {
  return crngpu::exception_status();
}

extern "C" int crngpu_unpack_batch_destroy(crngpu_unpack_batch batch) try {
  UnpackBatch* b = reinterpret_cast<UnpackBatch*>(batch);
  if (!b || b->magic != 0x42415443u) return CRNGPU_E_PARAM;
  b->magic = 0;
  delete b;
  return CRNGPU_OK;
} catch (...) {
  return crngpu::exception_status();
}

extern "C" int crngpu_unpack_end(crngpu_unpack_context ctx) try {
  UnpackContext* c = reinterpret_cast<UnpackContext*>(ctx);
  if (!valid_ctx(c)) return CRNGPU_E_PARAM;
  c->magic = 0;
  delete c;
  return CRNGPU_OK;
} catch (...) {
  return crngpu::exception_status();
}

extern "C" void crngpu_crn_decompress(void* src, unsigned int src_size, void* dst, unsigned int dst_size,
                                      unsigned int firstLevel, unsigned int levelCount) try {
  (void)dst_size;  // the reference wrapper does not bound-check dst either; each level is checked below
  crngpu_unpack_context ctx = crngpu_unpack_begin(src, src_size);
  if (!ctx) return;
  UnpackContext* c = reinterpret_cast<UnpackContext*>(ctx);
  uint32_t width = c->file.width >> firstLevel, height = c->file.height >> firstLevel;
  uint8_t* out = static_cast<uint8_t*>(dst);
  for (unsigned int i = firstLevel; i < firstLevel + levelCount; ++i) {
    const uint32_t bx = (width + 3) >> 2, by = (height + 3) >> 2;
    const uint32_t pitch = bx * c->file.bytes_per_block, total = pitch * by;
    void* faces[1] = {out};
    // as in the reference wrapper the output advances by the level size whether or not the
    // level unpacked (a level whose width or height shifted to 0 has size 0 and fails)
    if (c->file.faces == 1) crngpu_unpack_level(ctx, faces, total, pitch, i, CRNGPU_MEM_HOST, nullptr);
    out += total;
    width >>= 1;
    height >>= 1;
  }
  crngpu_unpack_end(ctx);
} catch (...) {
  crngpu::exception_status();
}

// ------------------------------------------------------------------------------------------
// Allocation-free transcode of one level.
//
// For callers that must not allocate GPU memory while they run: engines and streaming systems
// that reserve their whole VRAM budget up front and forbid untracked allocations afterwards, and
// real-time loops where cudaMalloc/cudaFree would block until the device is idle and stall other
// work. crngpu_unpack_level_noalloc transcodes from a .crn in host memory into the caller's
// device buffers and keeps everything else it needs -- decode tables, palettes, the level's
// compressed bytes, the per-block index records, launch descriptors, the work counter and the
// status word -- in the fixed array below, which every GPU that loads this library holds until
// the process exits. It never calls cudaMalloc, cudaFree or any allocating library routine on
// the device side; the host side only parses the file into ordinary heap memory.
//
// All calls share this one array and it keeps the contents of the last call: the work counter
// and status word are cleared on every call, and calls whose work overlaps on the GPU (other
// threads or streams) race on it, so callers serialise them.
namespace crngpu {

constexpr size_t kNoAllocScratchBytes = 16u << 20;  // 16 MiB: tables, palettes, stream, records
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

// Device address of g_noalloc_scratch, looked up once per device with that device current (in
// host code the array's name is only a host-side stand-in, not a device address). The lookup is
// made under the library's set-up mutex, so first calls from several host threads do not race.
int noalloc_scratch_ptr(unsigned char** out) {
  static unsigned char* ptrs[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_check(e, "cudaGetDevice");
  if (dev < 0 || dev >= 64) { set_error("device index out of range"); return CRNGPU_E_PARAM; }
  std::lock_guard<std::mutex> lock(device_setup_mutex());
  if (!ptrs[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_check(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    ptrs[dev] = static_cast<unsigned char*>(p);
  }
  *out = ptrs[dev];
  return CRNGPU_OK;
}

}  // namespace

}  // namespace crngpu

extern "C" int crngpu_unpack_level_noalloc(const void* crn_data, uint32_t crn_size, void** dst_faces,
                                           uint32_t dst_size_in_bytes, uint32_t row_pitch_in_bytes,
                                           uint32_t level_index, void* stream) try {
  using namespace crngpu;
  clear_error();
  if (!crn_data || !dst_faces || dst_size_in_bytes < 8) { set_error("bad arguments"); return CRNGPU_E_PARAM; }
  CrnFile F;
  if (!F.parse(static_cast<const uint8_t*>(crn_data), crn_size)) { set_error(F.error); return CRNGPU_E_CORRUPT; }
  if (level_index >= F.levels) { set_error("level out of range"); return CRNGPU_E_PARAM; }
  if (F.segmented) { set_error("segmented file: its level data is not in the buffer"); return CRNGPU_E_PARAM; }
  const LevelInfo& li = F.level[level_index];
  const uint32_t minimal = li.blocks_x * F.bytes_per_block;
  uint32_t pitch = row_pitch_in_bytes ? row_pitch_in_bytes : minimal;
  if (pitch < minimal || (pitch & 3)) { set_error("bad row pitch"); return CRNGPU_E_PARAM; }
  const uint64_t face_bytes = (uint64_t)pitch * li.blocks_y;
  if (dst_size_in_bytes < face_bytes) { set_error("destination too small"); return CRNGPU_E_PARAM; }
  for (uint32_t f = 0; f < F.faces; f++)
    if (!dst_faces[f]) { set_error("NULL face pointer"); return CRNGPU_E_PARAM; }

  // scratch layout: [counter, status][models][palettes][level stream][records][launch descriptors]
  // The descriptors go last: their size depends on the plan, which needs the record address.
  auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
  const size_t o_models = 256;
  const size_t o_pal = o_models + al(sizeof(DevModel) * kNumModels);
  const size_t o_src = o_pal + al(palette_bytes(F));
  const size_t o_rec = o_src + al((size_t)li.size + 64);
  const size_t rec_bytes = (size_t)li.blocks_x * li.blocks_y * F.faces * record_bytes((uint32_t)F.kind);
  const size_t o_jobs = o_rec + al(rec_bytes);
  if (o_jobs > kNoAllocScratchBytes) {
    set_error("level needs at least " + std::to_string(o_jobs) +
              " bytes of scratch; the allocation-free entry point has " + std::to_string(kNoAllocScratchBytes));
    return CRNGPU_E_PARAM;
  }
  unsigned char* base = nullptr;
  int rc = noalloc_scratch_ptr(&base);
  if (rc != CRNGPU_OK) return rc;
  cudaStream_t s = as_stream(stream);
  cudaError_t e;
  // host images of the tables, palettes and launch descriptors (ordinary heap, copied below)
  HVec<DevModel> models = model_image(F);
  DevPalettes pal;
  HVec<uint8_t> pal_img = palette_image(F, base + o_pal, &pal);
  LevelTask t{};
  t.file = &F;
  t.models = reinterpret_cast<const DevModel*>(base + o_models);
  t.pal = pal;
  t.level = level_index;
  for (uint32_t f = 0; f < F.faces; f++) t.dst[f] = static_cast<uint8_t*>(dst_faces[f]);
  t.pitch = pitch;
  t.src = base + o_src;
  t.src_size = li.size;
  t.rec = base + o_rec;
  t.item = 0;
  Plan p;
  uint32_t slots = 0;
  if ((rc = wide_slots(&slots)) != CRNGPU_OK) return rc;
  if (!make_plan({t}, p, slots)) { set_error("bad level"); return CRNGPU_E_PARAM; }
  const size_t need = o_jobs + al(p.image.size());
  if (need > kNoAllocScratchBytes) {
    set_error("level needs " + std::to_string(need) + " bytes of scratch; the allocation-free entry point has " +
              std::to_string(kNoAllocScratchBytes));
    return CRNGPU_E_PARAM;
  }
  struct Copy { size_t ofs; const void* src; size_t bytes; };
  const Copy copies[] = {
      {o_jobs, p.image.data(), p.image.size()},
      {o_models, models.data(), sizeof(DevModel) * kNumModels},
      {o_pal, pal_img.data(), pal_img.size()},
      {o_src, static_cast<const uint8_t*>(crn_data) + li.ofs, li.size},
  };
  for (const Copy& c : copies) {
    if (!c.bytes) continue;
    if ((e = cudaMemcpyAsync(base + c.ofs, c.src, c.bytes, cudaMemcpyHostToDevice, s)) != cudaSuccess)
      return cuda_check(e, "copy into the fixed scratch");
  }
  uint32_t* words = reinterpret_cast<uint32_t*>(base);
  if ((rc = enqueue_plan(p, base + o_jobs, words, s)) != CRNGPU_OK) return rc;
  uint32_t st[2] = {0, 0};
  if ((e = cudaMemcpyAsync(st, words, 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return cuda_check(e, "read status");
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_check(e, "sync");
  return status_to_rc(st[1]);
} catch (...) {
  return crngpu::exception_status();
}

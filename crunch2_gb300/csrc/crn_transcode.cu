// CRN -> DXTn transcoder on the GPU.
//
// Restates crnd::crn_unpacker::unpack_level and unpack_dxt1/dxt5/dxn/dxt5a
// (inc/crn_decomp.h:3537-3619, 3944-4223) as two kernels:
//   k_crn_decode  - the serial part: one warp (lane 0) per level stream Huffman-decodes the
//                   reference-group / endpoint-delta / selector symbols, resolves the
//                   left/top endpoint references and the running (mod palette size) endpoint
//                   index, and writes one index record per visible block to a scratch buffer.
//                   Streams of different levels (and textures) decode concurrently.
//   k_crn_expand  - the parallel part: every thread turns index records into finished DXT
//                   words (palette gathers from L2) and writes 16 bytes per store.
// The header, Huffman models and palettes are decoded once on the host (crn_file.cpp).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "crn_file.h"
#include "crngpu_internal.h"

namespace crngpu {

// Device status word values (written by k_crn_decode, read back by the host).
enum : uint32_t { kStOk = 0, kStBadCode = 1, kStBadIndex = 2 };

// Model slots in the device model array.
enum { kMRef = 0, kMEp0 = 1, kMSel0 = 2, kMEp1 = 3, kMSel1 = 4, kNumModels = 5 };

struct DevPalettes {
  const uint32_t* colour_ep;
  const uint32_t* colour_sel;
  const uint16_t* alpha_ep;
  const uint64_t* alpha_sel;  // 48 bits of DXT5 alpha selectors per entry
  uint32_t n_cep, n_csel, n_aep, n_asel;
};

struct DecodeJob {
  const uint8_t* src;  // level stream (device)
  uint32_t src_size;
  uint32_t bx, by, faces;
  uint64_t rec_ofs;    // first index record of this level in the scratch buffer
};

struct ExpandJob {
  uint8_t* dst;        // face 0 of the level (device)
  uint64_t face_stride;
  uint64_t rec_ofs;
  uint32_t bx, by, faces, pitch;
  uint32_t cta_begin;  // first CTA of this job in the expansion grid
  uint32_t ctas_per_row;
};

constexpr int kExpandThreads = 128;
constexpr int kMaxRowBlocks = 1024;  // 4096 px / 4, already even

// ------------------------------------------------------------------------------------------
// Bit reader: MSB-first 64-bit window; bytes past the end of the stream read as zero, as in
// symbol_codec::get_bits / decode (inc/crn_decomp.h:3162-3214). After a byte-wise head the
// stream is read as aligned 32-bit words (byte-swapped to MSB-first) with an L1 prefetch a few
// lines ahead, so the lone decoding thread rarely waits on memory.
struct Bits {
  const uint8_t* p;   // stream start
  uint32_t pos, end;  // next byte to load, stream size
  uint64_t buf;
  int n;
  __device__ __forceinline__ void init(const uint8_t* src, uint32_t size) {
    p = src; pos = 0; end = size; buf = 0; n = 0;
    // head: bytes up to the first 4-byte aligned address
    while (((uintptr_t)(p + pos) & 3) && n <= 56) {
      const uint32_t v = pos < end ? (uint32_t)__ldg(p + pos) : 0u;
      buf |= (uint64_t)v << (56 - n);
      n += 8;
      pos++;
    }
  }
  __device__ __forceinline__ void refill() {
    if (n <= 32) {
      uint32_t w;
      if (pos + 4 <= end) {
        w = __byte_perm(__ldg(reinterpret_cast<const uint32_t*>(p + pos)), 0, 0x0123);
        if ((pos & 127) == 0) asm volatile("prefetch.global.L1 [%0];" ::"l"(p + pos + 1024));
      } else if (pos < end) {
        w = __byte_perm(__ldg(reinterpret_cast<const uint32_t*>(p + pos)), 0, 0x0123);
        w &= 0xFFFFFFFFu << (8 * (4 - (end - pos)));  // zero the bytes past the end
      } else {
        w = 0;
      }
      pos += 4;
      buf |= (uint64_t)w << (32 - n);
      n += 32;
    }
  }
};

// Canonical prefix decode (symbol_codec::decode, inc/crn_decomp.h:3186-3253): 11-bit table in
// shared memory, then a walk over left-aligned per-length limits. -1: no such code.
__device__ __forceinline__ int decode_sym(Bits& b, const uint32_t* __restrict__ lut, const DevModel* __restrict__ m) {
  b.refill();
  const uint32_t v = (uint32_t)(b.buf >> 48);
  const uint32_t e = lut[v >> (16 - kLutBits)];
  uint32_t s, len;
  if (e != kLutLong) {
    s = e & 0xFFFFu;
    len = e >> 16;
  } else {
    len = kLutBits + 1;
    while (len <= (uint32_t)kMaxCodeLen && v >= __ldg(&m->limit[len])) len++;
    if (len > (uint32_t)kMaxCodeLen) return -1;
    const int idx = __ldg(&m->base[len]) + (int)(v >> (16 - len));
    if (idx < 0 || (uint32_t)idx >= m->num_syms) return -1;
    s = __ldg(&m->sorted[idx]);
  }
  b.buf <<= len;
  b.n -= (int)len;
  return (int)s;
}

// Row buffer entry (block_buffer_element, inc/crn_decomp.h:3652-3658), packed:
// bits 0-1 endpoint reference for the odd row, 2-14 endpoint index A, 15-27 endpoint index B.
__device__ __forceinline__ uint32_t rb_ref(uint32_t e) { return e & 3u; }
__device__ __forceinline__ uint32_t rb_a(uint32_t e) { return (e >> 2) & 0x1FFFu; }
__device__ __forceinline__ uint32_t rb_b(uint32_t e) { return (e >> 15) & 0x1FFFu; }

// KIND: 0 DXT1, 1 DXT5 (colour + alpha), 2 DXN (two alpha), 3 DXT5A
// Number of prefix models a format reads: ref + (colour ep, sel) + (alpha ep, sel).
template <int KIND>
__host__ __device__ constexpr int models_used() { return KIND == 1 ? 5 : 3; }

template <int KIND>
__global__ void __launch_bounds__(32) k_crn_decode(const DecodeJob* __restrict__ jobs, int njobs,
                                                    const DevModel* __restrict__ models, DevPalettes pal,
                                                    void* __restrict__ records, uint32_t* __restrict__ status) {
  __shared__ uint32_t row[kMaxRowBlocks];
  extern __shared__ uint32_t luts[];  // models_used<KIND>() x 2^kLutBits entries
  const int job_i = blockIdx.x;
  if (job_i >= njobs) return;
  // the warp copies the first-level tables this format needs into shared memory
  {
    const int slots[5] = {kMRef, KIND == 0 || KIND == 1 ? kMEp0 : kMEp1, KIND == 0 || KIND == 1 ? kMSel0 : kMSel1,
                          kMEp1, kMSel1};
    for (int t = 0; t < models_used<KIND>(); t++) {
      const uint4* src = reinterpret_cast<const uint4*>(models[slots[t]].lut);
      uint4* dst = reinterpret_cast<uint4*>(luts + t * (1 << kLutBits));
      for (int k = threadIdx.x; k < (1 << kLutBits) / 4; k += 32) dst[k] = __ldg(src + k);
    }
    __syncwarp();
  }
  if (threadIdx.x != 0) return;
  const DecodeJob job = jobs[job_i];
  const bool colour = KIND == 0 || KIND == 1;
  const int nalpha = KIND == 2 ? 2 : (KIND == 0 ? 0 : 1);
  const DevModel* m_ref = models + kMRef;
  const DevModel* m_ep0 = models + kMEp0;
  const DevModel* m_sel0 = models + kMSel0;
  const DevModel* m_ep1 = models + kMEp1;
  const DevModel* m_sel1 = models + kMSel1;
  const uint32_t* l_ref = luts;
  const uint32_t* l_ep0 = luts + (1 << kLutBits);      // colour models (DXT1, DXT5) ...
  const uint32_t* l_sel0 = luts + 2 * (1 << kLutBits);
  const uint32_t* l_ep1 = KIND == 1 ? luts + 3 * (1 << kLutBits) : l_ep0;   // ... or alpha models
  const uint32_t* l_sel1 = KIND == 1 ? luts + 4 * (1 << kLutBits) : l_sel0;
  const uint32_t W = (job.bx + 1) & ~1u, H = (job.by + 1) & ~1u;
  for (uint32_t x = 0; x < W; x++) row[x] = 0;
  Bits b;
  b.init(job.src, job.src_size);
  uint32_t cep = 0, a0 = 0, a1 = 0, group = 0;
  uint32_t* rec32 = reinterpret_cast<uint32_t*>(records) + job.rec_ofs;
  uint64_t* rec64 = reinterpret_cast<uint64_t*>(records) + job.rec_ofs;
  uint64_t out_i = 0;
  uint32_t err = kStOk;
  for (uint32_t f = 0; f < job.faces && !err; f++) {
    for (uint32_t y = 0; y < H && !err; y++) {
      const bool yvis = y < job.by;
      for (uint32_t x = 0; x < W; x++) {
        uint32_t e = row[x];
        uint32_t ref;
        if (!(y & 1)) {
          if (!(x & 1)) {
            const int g = decode_sym(b, l_ref, m_ref);
            if (g < 0) { err = kStBadCode; break; }
            group = (uint32_t)g & 0xFFu;  // reference_group is a uint8
          }
          ref = group & 3u;
          e = (e & ~3u) | ((group >> 2) & 3u);
          group >>= 4;
        } else {
          ref = rb_ref(e);
        }
        // endpoint A = colour (DXT1/DXT5) or alpha0 (DXN/DXT5A); B = alpha0 (DXT5) or alpha1 (DXN)
        if (ref == 0) {
          if (colour) {
            const int d = decode_sym(b, l_ep0, m_ep0);
            if (d < 0) { err = kStBadCode; break; }
            cep += (uint32_t)d;
            if (cep >= pal.n_cep) cep -= pal.n_cep;
            if (cep >= pal.n_cep) { err = kStBadIndex; break; }
          }
          if (nalpha >= 1) {
            const int d = decode_sym(b, l_ep1, m_ep1);
            if (d < 0) { err = kStBadCode; break; }
            a0 += (uint32_t)d;
            if (a0 >= pal.n_aep) a0 -= pal.n_aep;
            if (a0 >= pal.n_aep) { err = kStBadIndex; break; }
          }
          if (nalpha == 2) {
            const int d = decode_sym(b, l_ep1, m_ep1);
            if (d < 0) { err = kStBadCode; break; }
            a1 += (uint32_t)d;
            if (a1 >= pal.n_aep) a1 -= pal.n_aep;
            if (a1 >= pal.n_aep) { err = kStBadIndex; break; }
          }
        }
        if (ref <= 1) {
          const uint32_t A = colour ? cep : a0;
          const uint32_t B = KIND == 1 ? a0 : a1;
          e = (e & 3u) | (A << 2) | (B << 15);
        } else {
          if (colour) cep = rb_a(e); else a0 = rb_a(e);
          if (KIND == 1) a0 = rb_b(e);
          if (KIND == 2) a1 = rb_b(e);
        }
        row[x] = e;
        uint32_t cs = 0, s0 = 0, s1 = 0;
        if (colour) {
          const int s = decode_sym(b, l_sel0, m_sel0);
          if (s < 0) { err = kStBadCode; break; }
          if ((uint32_t)s >= pal.n_csel) { err = kStBadIndex; break; }
          cs = (uint32_t)s;
        }
        if (nalpha >= 1) {
          const int s = decode_sym(b, l_sel1, m_sel1);
          if (s < 0) { err = kStBadCode; break; }
          if ((uint32_t)s >= pal.n_asel) { err = kStBadIndex; break; }
          s0 = (uint32_t)s;
        }
        if (nalpha == 2) {
          const int s = decode_sym(b, l_sel1, m_sel1);
          if (s < 0) { err = kStBadCode; break; }
          if ((uint32_t)s >= pal.n_asel) { err = kStBadIndex; break; }
          s1 = (uint32_t)s;
        }
        if (yvis && x < job.bx) {
          if (KIND == 0) rec32[out_i] = cep | (cs << 16);
          else if (KIND == 3) rec32[out_i] = a0 | (s0 << 16);
          else if (KIND == 1) rec64[out_i] = (uint64_t)(cep | (cs << 16)) | ((uint64_t)(a0 | (s0 << 16)) << 32);
          else rec64[out_i] = (uint64_t)(a0 | (s0 << 16)) | ((uint64_t)(a1 | (s1 << 16)) << 32);
          out_i++;
        }
      }
    }
  }
  if (err) atomicMax(status, err);
}

// One 16-byte output chunk per thread: two 8-byte blocks (DXT1/DXT5A) or one 16-byte block.
template <int KIND>
__global__ void __launch_bounds__(kExpandThreads) k_crn_expand(const ExpandJob* __restrict__ jobs, int njobs,
                                                                DevPalettes pal, const void* __restrict__ records,
                                                                int vec_ok) {
  // find this CTA's job (jobs are few; cta_begin ascending)
  int j = 0;
  while (j + 1 < njobs && jobs[j + 1].cta_begin <= blockIdx.x) j++;
  const ExpandJob job = jobs[j];
  const uint32_t local = blockIdx.x - job.cta_begin;
  const uint32_t rowi = local / job.ctas_per_row;
  const uint32_t chunk = (local - rowi * job.ctas_per_row) * kExpandThreads + threadIdx.x;
  const uint32_t f = rowi / job.by, y = rowi - f * job.by;
  if (f >= job.faces) return;
  uint8_t* drow = job.dst + f * job.face_stride + (uint64_t)y * job.pitch;
  const uint64_t rbase = job.rec_ofs + (uint64_t)rowi * job.bx;
  if (KIND == 0 || KIND == 3) {
    const uint32_t x0 = chunk * 2;
    if (x0 >= job.bx) return;
    const uint32_t* rec = reinterpret_cast<const uint32_t*>(records) + rbase;
    auto word = [&](uint32_t r) -> uint2 {
      if (KIND == 0) return make_uint2(__ldg(pal.colour_ep + (r & 0xFFFFu)), __ldg(pal.colour_sel + (r >> 16)));
      const uint64_t a = (uint64_t)__ldg(pal.alpha_ep + (r & 0xFFFFu)) | (__ldg(pal.alpha_sel + (r >> 16)) << 16);
      return make_uint2((uint32_t)a, (uint32_t)(a >> 32));
    };
    const uint2 w0 = word(__ldg(rec + x0));
    uint32_t* d = reinterpret_cast<uint32_t*>(drow + (uint64_t)x0 * 8);
    if (x0 + 1 < job.bx) {
      const uint2 w1 = word(__ldg(rec + x0 + 1));
      if (vec_ok) {
        __stcs(reinterpret_cast<uint4*>(d), make_uint4(w0.x, w0.y, w1.x, w1.y));
      } else {
        d[0] = w0.x; d[1] = w0.y; d[2] = w1.x; d[3] = w1.y;
      }
    } else {
      d[0] = w0.x; d[1] = w0.y;
    }
  } else {
    const uint32_t x = chunk;
    if (x >= job.bx) return;
    const uint64_t r = __ldg(reinterpret_cast<const unsigned long long*>(records) + rbase + x);
    const uint32_t lo = (uint32_t)r, hi = (uint32_t)(r >> 32);
    uint4 o;
    if (KIND == 1) {
      const uint64_t a = (uint64_t)__ldg(pal.alpha_ep + (hi & 0xFFFFu)) | (__ldg(pal.alpha_sel + (hi >> 16)) << 16);
      o = make_uint4((uint32_t)a, (uint32_t)(a >> 32), __ldg(pal.colour_ep + (lo & 0xFFFFu)),
                     __ldg(pal.colour_sel + (lo >> 16)));
    } else {
      const uint64_t a = (uint64_t)__ldg(pal.alpha_ep + (lo & 0xFFFFu)) | (__ldg(pal.alpha_sel + (lo >> 16)) << 16);
      const uint64_t c = (uint64_t)__ldg(pal.alpha_ep + (hi & 0xFFFFu)) | (__ldg(pal.alpha_sel + (hi >> 16)) << 16);
      o = make_uint4((uint32_t)a, (uint32_t)(a >> 32), (uint32_t)c, (uint32_t)(c >> 32));
    }
    uint32_t* d = reinterpret_cast<uint32_t*>(drow + (uint64_t)x * 16);
    if (vec_ok) __stcs(reinterpret_cast<uint4*>(d), o);
    else { d[0] = o.x; d[1] = o.y; d[2] = o.z; d[3] = o.w; }
  }
}

// ------------------------------------------------------------------------------------------
// Host side: the unpack context.

struct UnpackContext {
  uint32_t magic = 0x43524E47u;
  int device = -1;
  CrnFile file;
  DevBuf d_file, d_models, d_pal, d_jobs, d_records, d_status;
  DevPalettes pal{};
  uint32_t status_host = 0;

  int kind_id() const { return (int)file.kind; }
  uint32_t rec_bytes() const { return (file.kind == Kind::DXT1 || file.kind == Kind::DXT5A) ? 4u : 8u; }
};

namespace {

bool valid_ctx(UnpackContext* c) { return c && c->magic == 0x43524E47u; }

int upload_context(UnpackContext* c, const uint8_t* data, uint32_t size) {
  CrnFile& F = c->file;
  cudaError_t e = cudaGetDevice(&c->device);
  if (e != cudaSuccess) return cuda_check(e, "cudaGetDevice");
  // file bytes, padded so word reads near the end stay inside the allocation
  if ((e = c->d_file.ensure(size + 64)) != cudaSuccess) return cuda_check(e, "alloc file");
  if ((e = cudaMemcpy(c->d_file.ptr, data, size, cudaMemcpyHostToDevice)) != cudaSuccess)
    return cuda_check(e, "copy file");
  std::unique_ptr<DevModel[]> models(new DevModel[kNumModels]);
  F.ref_dm.to_device(models[kMRef]);
  F.ep_dm[0].to_device(models[kMEp0]);
  F.sel_dm[0].to_device(models[kMSel0]);
  F.ep_dm[1].to_device(models[kMEp1]);
  F.sel_dm[1].to_device(models[kMSel1]);
  if ((e = c->d_models.ensure(sizeof(DevModel) * kNumModels)) != cudaSuccess) return cuda_check(e, "alloc models");
  if ((e = cudaMemcpy(c->d_models.ptr, models.get(), sizeof(DevModel) * kNumModels, cudaMemcpyHostToDevice)) !=
      cudaSuccess)
    return cuda_check(e, "copy models");
  // palettes: colour ep | colour sel | alpha sel (u64) | alpha ep, each 16-byte aligned
  auto al = [](size_t v) { return (v + 15) & ~(size_t)15; };
  const size_t n_cep = F.colour_ep.size(), n_csel = F.colour_sel.size();
  const size_t n_aep = F.alpha_ep.size(), n_asel = F.alpha_sel.size() / 3;
  const size_t o_csel = al(n_cep * 4), o_asel = o_csel + al(n_csel * 4), o_aep = o_asel + al(n_asel * 8);
  const size_t total = o_aep + al(n_aep * 2) + 16;
  std::vector<uint8_t> host(total, 0);
  if (n_cep) std::memcpy(host.data(), F.colour_ep.data(), n_cep * 4);
  if (n_csel) std::memcpy(host.data() + o_csel, F.colour_sel.data(), n_csel * 4);
  for (size_t i = 0; i < n_asel; i++) {
    const uint64_t v = (uint64_t)F.alpha_sel[3 * i] | ((uint64_t)F.alpha_sel[3 * i + 1] << 16) |
                       ((uint64_t)F.alpha_sel[3 * i + 2] << 32);
    std::memcpy(host.data() + o_asel + 8 * i, &v, 8);
  }
  if (n_aep) std::memcpy(host.data() + o_aep, F.alpha_ep.data(), n_aep * 2);
  if ((e = c->d_pal.ensure(total)) != cudaSuccess) return cuda_check(e, "alloc palettes");
  if ((e = cudaMemcpy(c->d_pal.ptr, host.data(), total, cudaMemcpyHostToDevice)) != cudaSuccess)
    return cuda_check(e, "copy palettes");
  uint8_t* base = static_cast<uint8_t*>(c->d_pal.ptr);
  c->pal.colour_ep = reinterpret_cast<const uint32_t*>(base);
  c->pal.colour_sel = reinterpret_cast<const uint32_t*>(base + o_csel);
  c->pal.alpha_sel = reinterpret_cast<const uint64_t*>(base + o_asel);
  c->pal.alpha_ep = reinterpret_cast<const uint16_t*>(base + o_aep);
  c->pal.n_cep = (uint32_t)n_cep;
  c->pal.n_csel = (uint32_t)n_csel;
  c->pal.n_aep = (uint32_t)n_aep;
  c->pal.n_asel = (uint32_t)n_asel;
  if ((e = c->d_status.ensure(16)) != cudaSuccess) return cuda_check(e, "alloc status");
  return CRNGPU_OK;
}

template <int K>
void launch_decode(const DecodeJob* jobs, int njobs, UnpackContext* c, void* rec, uint32_t* st, cudaStream_t s) {
  const size_t smem = sizeof(uint32_t) * (1 << kLutBits) * models_used<K>();  // <= 40 KB, no opt-in needed
  k_crn_decode<K><<<njobs, 32, smem, s>>>(jobs, njobs, static_cast<const DevModel*>(c->d_models.ptr), c->pal, rec, st);
}
template <int K>
void launch_expand(const ExpandJob* jobs, int njobs, uint32_t ctas, UnpackContext* c, const void* rec, int vec,
                   cudaStream_t s) {
  k_crn_expand<K><<<ctas, kExpandThreads, 0, s>>>(jobs, njobs, c->pal, rec, vec);
}

struct LevelOut {
  uint32_t level;
  uint8_t* dst[6];     // device pointer per face
  uint32_t pitch;
  const uint8_t* src;  // device pointer to the compressed level stream
  uint32_t src_size;
};

// Decodes and expands a list of levels (all destinations device memory). `records` holds
// at least sum(blocks) records; `status` is a device word (zeroed here).
int run_levels(UnpackContext* c, const std::vector<LevelOut>& outs, void* records, uint32_t* status,
               cudaStream_t s) {
  const CrnFile& F = c->file;
  std::vector<DecodeJob> dj;
  std::vector<ExpandJob> ej;
  uint64_t rec = 0;
  uint32_t ctas = 0;
  int vec_ok = 1;
  const uint32_t chunk_blocks = F.bytes_per_block == 8 ? 2 : 1;
  for (const LevelOut& o : outs) {
    const LevelInfo& li = F.level[o.level];
    dj.push_back(DecodeJob{o.src, o.src_size, li.blocks_x, li.blocks_y, F.faces, rec});
    for (uint32_t f = 0; f < F.faces; f++) {
      // faces of one level are contiguous in `records`; each face is one expansion job
      const uint32_t chunks = (li.blocks_x + chunk_blocks - 1) / chunk_blocks;
      const uint32_t per_row = (chunks + kExpandThreads - 1) / kExpandThreads;
      ExpandJob j;
      j.dst = o.dst[f];
      j.face_stride = 0;
      j.rec_ofs = rec + (uint64_t)f * li.blocks_x * li.blocks_y;
      j.bx = li.blocks_x;
      j.by = li.blocks_y;
      j.faces = 1;
      j.pitch = o.pitch;
      j.cta_begin = ctas;
      j.ctas_per_row = per_row;
      ctas += per_row * li.blocks_y;
      ej.push_back(j);
      if (((uintptr_t)o.dst[f] | o.pitch) & 15) vec_ok = 0;
    }
    rec += (uint64_t)li.blocks_x * li.blocks_y * F.faces;
  }
  const size_t jb = sizeof(DecodeJob) * dj.size(), eb = sizeof(ExpandJob) * ej.size();
  cudaError_t e = c->d_jobs.ensure(jb + eb + 16);
  if (e != cudaSuccess) return cuda_check(e, "alloc jobs");
  std::vector<uint8_t> hj(jb + eb);
  std::memcpy(hj.data(), dj.data(), jb);
  std::memcpy(hj.data() + jb, ej.data(), eb);
  if ((e = cudaMemcpyAsync(c->d_jobs.ptr, hj.data(), hj.size(), cudaMemcpyHostToDevice, s)) != cudaSuccess)
    return cuda_check(e, "copy jobs");
  if ((e = cudaMemsetAsync(status, 0, 4, s)) != cudaSuccess) return cuda_check(e, "clear status");
  const DecodeJob* djd = static_cast<const DecodeJob*>(c->d_jobs.ptr);
  const ExpandJob* ejd = reinterpret_cast<const ExpandJob*>(static_cast<uint8_t*>(c->d_jobs.ptr) + jb);
  switch (F.kind) {
    case Kind::DXT1: launch_decode<0>(djd, (int)dj.size(), c, records, status, s); break;
    case Kind::DXT5: launch_decode<1>(djd, (int)dj.size(), c, records, status, s); break;
    case Kind::DXN: launch_decode<2>(djd, (int)dj.size(), c, records, status, s); break;
    case Kind::DXT5A: launch_decode<3>(djd, (int)dj.size(), c, records, status, s); break;
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(e, "launch k_crn_decode");
  if (ctas) {
    switch (F.kind) {
      case Kind::DXT1: launch_expand<0>(ejd, (int)ej.size(), ctas, c, records, vec_ok, s); break;
      case Kind::DXT5: launch_expand<1>(ejd, (int)ej.size(), ctas, c, records, vec_ok, s); break;
      case Kind::DXN: launch_expand<2>(ejd, (int)ej.size(), ctas, c, records, vec_ok, s); break;
      case Kind::DXT5A: launch_expand<3>(ejd, (int)ej.size(), ctas, c, records, vec_ok, s); break;
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(e, "launch k_crn_expand");
  }
  // the reference reports a bad stream through its bool result; read the status word back
  if ((e = cudaMemcpyAsync(&c->status_host, status, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
    return cuda_check(e, "read status");
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_check(e, "sync");
  if (c->status_host) {
    set_error(c->status_host == kStBadCode ? "corrupt block stream (no such prefix code)"
                                           : "corrupt block stream (palette index out of range)");
    return CRNGPU_E_CORRUPT;
  }
  return CRNGPU_OK;
}

uint64_t level_records(const CrnFile& F, uint32_t l) {
  return (uint64_t)F.level[l].blocks_x * F.level[l].blocks_y * F.faces;
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
  LevelOut o;
  o.level = level;
  o.pitch = row_pitch;
  if (dev_src) { o.src = dev_src; o.src_size = src_size; }
  else if (host_src) {
    DevBuf& sb = staging(2);
    if ((e = sb.ensure(src_size + 64)) != cudaSuccess) return cuda_check(e, "alloc segment");
    if ((e = cudaMemcpyAsync(sb.ptr, host_src, src_size, cudaMemcpyHostToDevice, s)) != cudaSuccess)
      return cuda_check(e, "copy segment");
    o.src = static_cast<const uint8_t*>(sb.ptr);
    o.src_size = src_size;
  } else {
    o.src = static_cast<const uint8_t*>(c->d_file.ptr) + li.ofs;
    o.src_size = li.size;
  }
  DevBuf* out_stage = nullptr;
  if (mem == CRNGPU_MEM_DEVICE) {
    for (uint32_t f = 0; f < F.faces; f++) o.dst[f] = static_cast<uint8_t*>(dst_faces[f]);
  } else {
    out_stage = &staging(1);
    if ((e = out_stage->ensure(face_bytes * F.faces)) != cudaSuccess) return cuda_check(e, "alloc output stage");
    for (uint32_t f = 0; f < F.faces; f++) o.dst[f] = static_cast<uint8_t*>(out_stage->ptr) + face_bytes * f;
    // rows may have pitch padding the transcoder does not write: keep the caller's bytes there
    if (row_pitch != minimal)
      for (uint32_t f = 0; f < F.faces; f++)
        if ((e = cudaMemcpyAsync(o.dst[f], dst_faces[f], face_bytes, cudaMemcpyHostToDevice, s)) != cudaSuccess)
          return cuda_check(e, "stage output");
  }
  if ((e = c->d_records.ensure(level_records(F, level) * c->rec_bytes() + 16)) != cudaSuccess)
    return cuda_check(e, "alloc records");
  int rc = run_levels(c, {o}, c->d_records.ptr, static_cast<uint32_t*>(c->d_status.ptr), s);
  if (rc != CRNGPU_OK) return rc;
  if (out_stage) {
    for (uint32_t f = 0; f < F.faces; f++)
      if ((e = cudaMemcpyAsync(dst_faces[f], o.dst[f], face_bytes, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return cuda_check(e, "copy output");
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_check(e, "sync");
  }
  return CRNGPU_OK;
}

}  // namespace

}  // namespace crngpu

using namespace crngpu;

extern "C" crngpu_unpack_context crngpu_unpack_begin(const void* data, uint32_t data_size) {
  clear_error();
  std::unique_ptr<UnpackContext> c(new UnpackContext());
  if (!c->file.parse(static_cast<const uint8_t*>(data), data_size)) {
    set_error(c->file.error);
    return nullptr;
  }
  if (upload_context(c.get(), static_cast<const uint8_t*>(data), data_size) != CRNGPU_OK) return nullptr;
  return reinterpret_cast<crngpu_unpack_context>(c.release());
}

extern "C" int crngpu_get_info(crngpu_unpack_context ctx, uint32_t* width, uint32_t* height, uint32_t* levels,
                               uint32_t* faces, uint32_t* format, uint32_t* bytes_per_block) {
  UnpackContext* c = reinterpret_cast<UnpackContext*>(ctx);
  if (!valid_ctx(c)) return CRNGPU_E_PARAM;
  if (width) *width = c->file.width;
  if (height) *height = c->file.height;
  if (levels) *levels = c->file.levels;
  if (faces) *faces = c->file.faces;
  if (format) *format = c->file.format;
  if (bytes_per_block) *bytes_per_block = c->file.bytes_per_block;
  return CRNGPU_OK;
}

extern "C" int crngpu_unpack_level(crngpu_unpack_context ctx, void** dst_faces, uint32_t dst_size_in_bytes,
                                   uint32_t row_pitch_in_bytes, uint32_t level_index, int mem, void* stream) {
  clear_error();
  return unpack_one(reinterpret_cast<UnpackContext*>(ctx), nullptr, nullptr, 0, dst_faces, dst_size_in_bytes,
                    row_pitch_in_bytes, level_index, mem, stream);
}

extern "C" int crngpu_unpack_level_segmented(crngpu_unpack_context ctx, const void* src, uint32_t src_size_in_bytes,
                                             void** dst_faces, uint32_t dst_size_in_bytes,
                                             uint32_t row_pitch_in_bytes, uint32_t level_index, int mem,
                                             void* stream) {
  clear_error();
  if (!src || !src_size_in_bytes) { set_error("NULL segment"); return CRNGPU_E_PARAM; }
  const uint8_t* s = static_cast<const uint8_t*>(src);
  return unpack_one(reinterpret_cast<UnpackContext*>(ctx), mem == CRNGPU_MEM_DEVICE ? nullptr : s,
                    mem == CRNGPU_MEM_DEVICE ? s : nullptr, src_size_in_bytes, dst_faces, dst_size_in_bytes,
                    row_pitch_in_bytes, level_index, mem, stream);
}

extern "C" int64_t crngpu_unpack_levels(crngpu_unpack_context ctx, uint32_t first_level, uint32_t level_count,
                                        void* dst, uint64_t dst_size, int mem, void* stream) {
  clear_error();
  UnpackContext* c = reinterpret_cast<UnpackContext*>(ctx);
  if (!valid_ctx(c) || !dst || !level_count || first_level + level_count > c->file.levels) {
    set_error("bad context, destination or level range");
    return CRNGPU_E_PARAM;
  }
  const CrnFile& F = c->file;
  uint64_t total = 0, recs = 0;
  for (uint32_t l = first_level; l < first_level + level_count; l++) {
    total += (uint64_t)F.level[l].blocks_x * F.bytes_per_block * F.level[l].blocks_y * F.faces;
    recs += level_records(F, l);
  }
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
  std::vector<LevelOut> outs;
  uint64_t ofs = 0;
  for (uint32_t l = first_level; l < first_level + level_count; l++) {
    LevelOut o;
    o.level = l;
    o.pitch = F.level[l].blocks_x * F.bytes_per_block;
    const uint64_t face_bytes = (uint64_t)o.pitch * F.level[l].blocks_y;
    for (uint32_t f = 0; f < F.faces; f++) o.dst[f] = out + ofs + f * face_bytes;
    o.src = static_cast<const uint8_t*>(c->d_file.ptr) + F.level[l].ofs;
    o.src_size = F.level[l].size;
    ofs += face_bytes * F.faces;
    outs.push_back(o);
  }
  if ((e = c->d_records.ensure(recs * c->rec_bytes() + 16)) != cudaSuccess) return cuda_check(e, "alloc records");
  int rc = run_levels(c, outs, c->d_records.ptr, static_cast<uint32_t*>(c->d_status.ptr), s);
  if (rc != CRNGPU_OK) return rc;
  if (stage) {
    if ((e = cudaMemcpyAsync(dst, stage->ptr, total, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
      return cuda_check(e, "copy output");
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_check(e, "sync");
  }
  return (int64_t)total;
}

extern "C" int crngpu_unpack_end(crngpu_unpack_context ctx) {
  UnpackContext* c = reinterpret_cast<UnpackContext*>(ctx);
  if (!valid_ctx(c)) return CRNGPU_E_PARAM;
  c->magic = 0;
  delete c;
  return CRNGPU_OK;
}

extern "C" void crngpu_crn_decompress(void* src, unsigned int src_size, void* dst, unsigned int dst_size,
                                      unsigned int firstLevel, unsigned int levelCount) {
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
}

// ------------------------------------------------------------------------------------------
// Allocation-free transcode of one level.
//
// For callers that must not allocate GPU memory while they run: engines and streaming systems
// that reserve their whole VRAM budget up front and forbid untracked allocations afterwards, and
// real-time loops where cudaMalloc/cudaFree would block until the device is idle and stall other
// work. crngpu_unpack_level_noalloc transcodes from a .crn in host memory into the caller's
// device buffers and keeps everything else it needs -- decode tables, palettes, the level's
// compressed bytes, the per-block index records, launch descriptors and the status word -- in
// the fixed array below, which every GPU that loads this library holds until the process exits.
// It never calls cudaMalloc, cudaFree or any allocating library routine on the device side; the
// host side only parses the file into ordinary heap memory.
//
// All calls share this one array and it keeps the contents of the last call: the status word is
// cleared on every call, and calls whose work overlaps on the GPU (other threads or streams)
// race on it, so callers serialise them.
namespace crngpu {

constexpr size_t kNoAllocScratchBytes = 16u << 20;  // 16 MiB: tables, palettes, stream, records
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

// Device address of g_noalloc_scratch, looked up once per device with that device current (in
// host code the array's name is only a host-side stand-in, not a device address).
int noalloc_scratch_ptr(unsigned char** out) {
  static unsigned char* ptrs[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_check(e, "cudaGetDevice");
  if (dev < 0 || dev >= 64) { set_error("device index out of range"); return CRNGPU_E_PARAM; }
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
                                           uint32_t level_index, void* stream) {
  using namespace crngpu;
  clear_error();
  if (!crn_data || !dst_faces || dst_size_in_bytes < 8) { set_error("bad arguments"); return CRNGPU_E_PARAM; }
  CrnFile F;
  if (!F.parse(static_cast<const uint8_t*>(crn_data), crn_size)) { set_error(F.error); return CRNGPU_E_CORRUPT; }
  if (level_index >= F.levels) { set_error("level out of range"); return CRNGPU_E_PARAM; }
  const LevelInfo& li = F.level[level_index];
  const uint32_t minimal = li.blocks_x * F.bytes_per_block;
  uint32_t pitch = row_pitch_in_bytes ? row_pitch_in_bytes : minimal;
  if (pitch < minimal || (pitch & 3)) { set_error("bad row pitch"); return CRNGPU_E_PARAM; }
  const uint64_t face_bytes = (uint64_t)pitch * li.blocks_y;
  if (dst_size_in_bytes < face_bytes) { set_error("destination too small"); return CRNGPU_E_PARAM; }
  for (uint32_t f = 0; f < F.faces; f++)
    if (!dst_faces[f]) { set_error("NULL face pointer"); return CRNGPU_E_PARAM; }

  // scratch layout: [status | jobs][models][palettes][level stream][records]
  auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
  const size_t n_cep = F.colour_ep.size(), n_csel = F.colour_sel.size();
  const size_t n_aep = F.alpha_ep.size(), n_asel = F.alpha_sel.size() / 3;
  const size_t o_jobs = 256, o_models = 4096;
  const size_t o_cep = o_models + al(sizeof(DevModel) * kNumModels);
  const size_t o_csel = o_cep + al(n_cep * 4), o_asel = o_csel + al(n_csel * 4), o_aep = o_asel + al(n_asel * 8);
  const size_t o_src = o_aep + al(n_aep * 2);
  const size_t o_rec = o_src + al((size_t)li.size + 64);
  const size_t rec_bytes = (size_t)li.blocks_x * li.blocks_y * F.faces *
                           ((F.kind == Kind::DXT1 || F.kind == Kind::DXT5A) ? 4u : 8u);
  const size_t need = o_rec + al(rec_bytes);
  if (need > kNoAllocScratchBytes) {
    set_error("level needs " + std::to_string(need) + " bytes of scratch; the allocation-free entry point has " +
              std::to_string(kNoAllocScratchBytes));
    return CRNGPU_E_PARAM;
  }
  unsigned char* base = nullptr;
  int rc = noalloc_scratch_ptr(&base);
  if (rc != CRNGPU_OK) return rc;
  cudaStream_t s = as_stream(stream);
  cudaError_t e;
  // host images of the tables, palettes and launch descriptors (ordinary heap, copied below)
  std::vector<DevModel> models(kNumModels);
  F.ref_dm.to_device(models[kMRef]);
  F.ep_dm[0].to_device(models[kMEp0]);
  F.sel_dm[0].to_device(models[kMSel0]);
  F.ep_dm[1].to_device(models[kMEp1]);
  F.sel_dm[1].to_device(models[kMSel1]);
  std::vector<uint64_t> asel64(n_asel);
  for (size_t i = 0; i < n_asel; i++)
    asel64[i] = (uint64_t)F.alpha_sel[3 * i] | ((uint64_t)F.alpha_sel[3 * i + 1] << 16) |
                ((uint64_t)F.alpha_sel[3 * i + 2] << 32);
  DevPalettes pal;
  pal.colour_ep = reinterpret_cast<const uint32_t*>(base + o_cep);
  pal.colour_sel = reinterpret_cast<const uint32_t*>(base + o_csel);
  pal.alpha_sel = reinterpret_cast<const uint64_t*>(base + o_asel);
  pal.alpha_ep = reinterpret_cast<const uint16_t*>(base + o_aep);
  pal.n_cep = (uint32_t)n_cep; pal.n_csel = (uint32_t)n_csel; pal.n_aep = (uint32_t)n_aep; pal.n_asel = (uint32_t)n_asel;
  DecodeJob dj{base + o_src, li.size, li.blocks_x, li.blocks_y, F.faces, 0};
  ExpandJob ej[6];
  const uint32_t chunk_blocks = F.bytes_per_block == 8 ? 2 : 1;
  const uint32_t per_row = ((li.blocks_x + chunk_blocks - 1) / chunk_blocks + kExpandThreads - 1) / kExpandThreads;
  int vec_ok = 1;
  for (uint32_t f = 0; f < F.faces; f++) {
    ej[f].dst = static_cast<uint8_t*>(dst_faces[f]);
    ej[f].face_stride = 0;
    ej[f].rec_ofs = (uint64_t)f * li.blocks_x * li.blocks_y;
    ej[f].bx = li.blocks_x; ej[f].by = li.blocks_y; ej[f].faces = 1; ej[f].pitch = pitch;
    ej[f].cta_begin = f * per_row * li.blocks_y;
    ej[f].ctas_per_row = per_row;
    if (((uintptr_t)dst_faces[f] | pitch) & 15) vec_ok = 0;
  }
  unsigned char jobs[sizeof(DecodeJob) + 6 * sizeof(ExpandJob)];
  std::memcpy(jobs, &dj, sizeof(dj));
  std::memcpy(jobs + sizeof(dj), ej, sizeof(ExpandJob) * F.faces);
  uint32_t* status = reinterpret_cast<uint32_t*>(base);
  const DecodeJob* d_dj = reinterpret_cast<const DecodeJob*>(base + o_jobs);
  const ExpandJob* d_ej = reinterpret_cast<const ExpandJob*>(base + o_jobs + sizeof(DecodeJob));
  struct Copy { size_t ofs; const void* src; size_t bytes; };
  const Copy copies[] = {
      {o_jobs, jobs, sizeof(DecodeJob) + sizeof(ExpandJob) * F.faces},
      {o_models, models.data(), sizeof(DevModel) * kNumModels},
      {o_cep, F.colour_ep.data(), n_cep * 4},
      {o_csel, F.colour_sel.data(), n_csel * 4},
      {o_asel, asel64.data(), n_asel * 8},
      {o_aep, F.alpha_ep.data(), n_aep * 2},
      {o_src, static_cast<const uint8_t*>(crn_data) + li.ofs, li.size},
  };
  for (const Copy& c : copies) {
    if (!c.bytes) continue;
    if ((e = cudaMemcpyAsync(base + c.ofs, c.src, c.bytes, cudaMemcpyHostToDevice, s)) != cudaSuccess)
      return cuda_check(e, "copy into the fixed scratch");
  }
  if ((e = cudaMemsetAsync(status, 0, 4, s)) != cudaSuccess) return cuda_check(e, "clear status");
  const DevModel* d_models = reinterpret_cast<const DevModel*>(base + o_models);
  void* records = base + o_rec;
  const uint32_t ctas = per_row * li.blocks_y * F.faces;
  switch (F.kind) {
    case Kind::DXT1:
      k_crn_decode<0><<<1, 32, sizeof(uint32_t) * (1 << kLutBits) * models_used<0>(), s>>>(d_dj, 1, d_models, pal, records, status);
      k_crn_expand<0><<<ctas, kExpandThreads, 0, s>>>(d_ej, (int)F.faces, pal, records, vec_ok);
      break;
    case Kind::DXT5:
      k_crn_decode<1><<<1, 32, sizeof(uint32_t) * (1 << kLutBits) * models_used<1>(), s>>>(d_dj, 1, d_models, pal, records, status);
      k_crn_expand<1><<<ctas, kExpandThreads, 0, s>>>(d_ej, (int)F.faces, pal, records, vec_ok);
      break;
    case Kind::DXN:
      k_crn_decode<2><<<1, 32, sizeof(uint32_t) * (1 << kLutBits) * models_used<2>(), s>>>(d_dj, 1, d_models, pal, records, status);
      k_crn_expand<2><<<ctas, kExpandThreads, 0, s>>>(d_ej, (int)F.faces, pal, records, vec_ok);
      break;
    case Kind::DXT5A:
      k_crn_decode<3><<<1, 32, sizeof(uint32_t) * (1 << kLutBits) * models_used<3>(), s>>>(d_dj, 1, d_models, pal, records, status);
      k_crn_expand<3><<<ctas, kExpandThreads, 0, s>>>(d_ej, (int)F.faces, pal, records, vec_ok);
      break;
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(e, "launch transcode kernels");
  uint32_t st = 0;
  if ((e = cudaMemcpyAsync(&st, status, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return cuda_check(e, "read status");
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_check(e, "sync");
  if (st) {
    set_error(st == kStBadCode ? "corrupt block stream (no such prefix code)"
                               : "corrupt block stream (palette index out of range)");
    return CRNGPU_E_CORRUPT;
  }
  return CRNGPU_OK;
}

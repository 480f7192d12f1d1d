// Batched plain encode: the mip chains of many textures of any mix of sizes and formats (DXT1, the
// DXT5 family, DXN, DXT5A) encoded by one gather launch and two persistent encoder launches, one
// for colour elements and one for alpha / DXN channel elements, forked onto two streams so that
// they share the GPU, and captured into a CUDA graph. The reference encodes one image at a time
// (dxt_image::init, crnlib/crn_dxt_image.cpp:447-493, its blocks split round-robin over helper
// threads, :283-349); each block's result here is that of crngpu_compress_image on its level.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "crngpu_internal.h"

namespace crngpu {
namespace {

// up to kGatherTileBlocks consecutive blocks of one level: texel (x, y) of block (bx, by) is
// src[min(4by+y, h-1)][min(4bx+x, w-1)] (dxt_image::init_task edge clamp, crn_dxt_image.cpp:334-344)
constexpr uint32_t kGatherTileBlocks = 256;
struct GatherTile {
  const uint8_t* src;
  uint32_t w, h, blocks_x, level_block;  // first block of the tile within its level
  uint32_t first_block, count;            // first block in the gathered array, blocks in the tile
};

__global__ void __launch_bounds__(256) k_gather_tiles(const GatherTile* __restrict__ tiles, uint32_t* __restrict__ out) {
  const GatherTile t = tiles[blockIdx.x];
  for (uint32_t q = threadIdx.x; q < t.count * 16; q += blockDim.x) {
    const uint32_t lb = t.level_block + (q >> 4), tin = q & 15;
    const uint32_t by = lb / t.blocks_x, bx = lb - by * t.blocks_x;
    const uint32_t x = min(bx * 4 + (tin & 3), t.w - 1), y = min(by * 4 + (tin >> 2), t.h - 1);
    const uint8_t* p = t.src + ((size_t)y * t.w + x) * 4;
    out[((size_t)t.first_block << 4) + q] =
        (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
  }
}

int format_bpb(uint32_t fmt) {
  switch (fmt) {
    case CRNGPU_FMT_DXT1: case CRNGPU_FMT_DXT5A: return 8;
    case CRNGPU_FMT_DXT5: case CRNGPU_FMT_DXT5_CCXY: case CRNGPU_FMT_DXT5_XGXR: case CRNGPU_FMT_DXT5_XGBR:
    case CRNGPU_FMT_DXT5_AGBR: case CRNGPU_FMT_DXN_XY: case CRNGPU_FMT_DXN_YX: return 16;
    default: return 0;
  }
}

constexpr uint32_t kAlphaChunkBlocks = 8;
constexpr int kColourVariants = 4;  // colour grid: 2 (v + 1) CTAs per SM, capped at the occupancy
constexpr int kAlphaVariants = 4;   // alpha grid: 2 << v CTAs per SM, capped at the occupancy

struct EncodeBatch {
  uint32_t magic = 0x454E4342u;
  int device = 0;
  uint64_t nblocks = 0, texels = 0;
  uint32_t ntiles = 0, ncolour = 0, nalpha = 0;
  DevBuf blocks, d_tiles, d_segs, d_cchunks, d_achunks;
  DevBuf seeds;  // the colour encoder's per-block hand-off between its two kernels
  int sms = 148, colour_max = 0, alpha_max = 0;
  int colour_grid = 0, alpha_grid = 0;  // 0 until tuned
  float colour_ms[kColourVariants] = {}, alpha_ms[kAlphaVariants] = {};
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  cudaGraphExec_t graph = nullptr;
};

int enqueue(EncodeBatch* b, cudaStream_t s, int colour_grid, int alpha_grid) {
  cudaError_t e;
  if (b->ntiles) {
    k_gather_tiles<<<b->ntiles, 256, 0, s>>>(static_cast<const GatherTile*>(b->d_tiles.ptr),
                                             static_cast<uint32_t*>(b->blocks.ptr));
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(e, "launch k_gather_tiles");
  }
  const uint8_t* blk = static_cast<const uint8_t*>(b->blocks.ptr);
  const EncodeSegment* segs = static_cast<const EncodeSegment*>(b->d_segs.ptr);
  // alpha elements on the side stream, colour elements on `s`, joined before returning
  if ((e = cudaEventRecord(b->fork, s)) != cudaSuccess) return cuda_check(e, "record fork");
  if ((e = cudaStreamWaitEvent(b->side, b->fork, 0)) != cudaSuccess) return cuda_check(e, "wait fork");
  int rc = launch_dxt5a_chunks(blk, static_cast<const EncodeChunk*>(b->d_achunks.ptr), b->nalpha, segs, alpha_grid,
                               b->side);
  if (rc != CRNGPU_OK) return rc;
  if ((e = cudaEventRecord(b->join, b->side)) != cudaSuccess) return cuda_check(e, "record join");
  rc = launch_dxt1_chunks(blk, static_cast<const EncodeChunk*>(b->d_cchunks.ptr), b->ncolour, segs, b->seeds.ptr,
                          colour_grid, s);
  if (rc != CRNGPU_OK) return rc;
  if ((e = cudaStreamWaitEvent(s, b->join, 0)) != cudaSuccess) return cuda_check(e, "wait join");
  return CRNGPU_OK;
}

// Times each colour and alpha launch shape on the real work (every variant writes the same
// output) and keeps the fastest of each.
int autotune(EncodeBatch* b, cudaStream_t s) {
  cudaEvent_t ev[2];
  cudaError_t e;
  if ((e = cudaEventCreate(&ev[0])) != cudaSuccess) return cuda_check(e, "events");
  if ((e = cudaEventCreate(&ev[1])) != cudaSuccess) { cudaEventDestroy(ev[0]); return cuda_check(e, "events"); }
  const uint8_t* blk = static_cast<const uint8_t*>(b->blocks.ptr);
  const EncodeSegment* segs = static_cast<const EncodeSegment*>(b->d_segs.ptr);
  int rc = CRNGPU_OK;
  auto time_it = [&](bool colour, int grid, float& ms_out) -> int {
    float tot = 0.f;
    for (int rep = 0; rep < 2; rep++) {
      cudaEventRecord(ev[0], s);
      const int r = colour ? launch_dxt1_chunks(blk, static_cast<const EncodeChunk*>(b->d_cchunks.ptr), b->ncolour,
                                                segs, b->seeds.ptr, grid, s)
                           : launch_dxt5a_chunks(blk, static_cast<const EncodeChunk*>(b->d_achunks.ptr), b->nalpha,
                                                 segs, grid, s);
      if (r != CRNGPU_OK) return r;
      cudaEventRecord(ev[1], s);
      if ((e = cudaEventSynchronize(ev[1])) != cudaSuccess) return cuda_check(e, "tuning sync");
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ev[0], ev[1]);
      if (rep) tot += ms;  // the first run warms up
    }
    ms_out = tot;
    return CRNGPU_OK;
  };
  // gather once so the encoders read real blocks
  if (b->ntiles) {
    k_gather_tiles<<<b->ntiles, 256, 0, s>>>(static_cast<const GatherTile*>(b->d_tiles.ptr),
                                             static_cast<uint32_t*>(b->blocks.ptr));
    if ((e = cudaGetLastError()) != cudaSuccess) rc = cuda_check(e, "launch k_gather_tiles");
  }
  float best = 3.4e38f;
  for (int v = 0; v < kColourVariants && rc == CRNGPU_OK && b->ncolour; v++) {
    const int grid = std::min(b->colour_max, b->sms * 2 * (v + 1));  // 2, 4, 6, 8 CTAs per SM
    rc = time_it(true, grid, b->colour_ms[v]);
    if (rc == CRNGPU_OK && b->colour_ms[v] < best) { best = b->colour_ms[v]; b->colour_grid = grid; }
  }
  best = 3.4e38f;
  for (int v = 0; v < kAlphaVariants && rc == CRNGPU_OK && b->nalpha; v++) {
    const int grid = std::min(b->alpha_max, b->sms * (2 << v));
    rc = time_it(false, grid, b->alpha_ms[v]);
    if (rc == CRNGPU_OK && b->alpha_ms[v] < best) { best = b->alpha_ms[v]; b->alpha_grid = grid; }
  }
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  if (!b->colour_grid) b->colour_grid = b->colour_max;
  if (!b->alpha_grid) b->alpha_grid = b->alpha_max;
  return rc;
}

void destroy(EncodeBatch* b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->join) cudaEventDestroy(b->join);
  if (b->side) cudaStreamDestroy(b->side);
  b->magic = 0;
  delete b;
}

}  // namespace
}  // namespace crngpu

using namespace crngpu;

extern "C" crngpu_encode_batch crngpu_encode_batch_create(const crngpu_encode_item* items, uint32_t n, uint32_t flags) try {
  clear_error();
  if (!items || !n) { set_error("crngpu_encode_batch_create: no items"); return nullptr; }
  const bool perceptual = (flags & CRNGPU_FLAG_PERCEPTUAL) != 0;
  const bool both = (flags & CRNGPU_FLAG_USE_BOTH_BLOCK_TYPES) != 0;
  std::vector<GatherTile> tiles;
  std::vector<EncodeSegment> segs;
  std::vector<EncodeChunk> cchunks, achunks;
  uint64_t nblocks = 0, texels = 0;
  for (uint32_t i = 0; i < n; i++) {
    const crngpu_encode_item& it = items[i];
    const int bpb = format_bpb(it.format);
    if (!bpb) { set_error("crngpu_encode_batch_create: item " + std::to_string(i) + ": unsupported format"); return nullptr; }
    if (!it.rgba || !it.out || !it.width || !it.height || it.width > 16384 || it.height > 16384 || !it.levels) {
      set_error("crngpu_encode_batch_create: item " + std::to_string(i) + ": bad pointers or dimensions");
      return nullptr;
    }
    if (((uintptr_t)it.out & 7) || ((uintptr_t)it.rgba & 3)) {
      set_error("crngpu_encode_batch_create: item " + std::to_string(i) + ": out must be 8-byte, rgba 4-byte aligned");
      return nullptr;
    }
    uint32_t full = 1;
    while ((it.width >> full) || (it.height >> full)) full++;
    if (it.levels > full) {
      set_error("crngpu_encode_batch_create: item " + std::to_string(i) + ": more levels than the mip chain has");
      return nullptr;
    }
    const uint64_t first = nblocks;
    const uint8_t* src = it.rgba;
    for (uint32_t l = 0; l < it.levels; l++) {
      const uint32_t w = std::max(1u, it.width >> l), h = std::max(1u, it.height >> l);
      const uint32_t bx = (w + 3) / 4, by = (h + 3) / 4;
      const uint32_t lb = bx * by;
      for (uint32_t t = 0; t < lb; t += kGatherTileBlocks)
        tiles.push_back(GatherTile{src, w, h, bx, t, (uint32_t)(nblocks + t), std::min(kGatherTileBlocks, lb - t)});
      nblocks += lb;
      texels += (uint64_t)w * h;
      src += (size_t)w * h * 4;
    }
    if (nblocks > 0xFFFFFFFFull) { set_error("crngpu_encode_batch_create: more than 2^32 blocks"); return nullptr; }
    const uint32_t count = (uint32_t)(nblocks - first);
    auto add_seg = [&](uint8_t* out, uint32_t stride, uint32_t options, bool colour) {
      const uint32_t sid = (uint32_t)segs.size();
      segs.push_back(EncodeSegment{out, (uint32_t)first, count, stride, options});
      const uint32_t step = colour ? kColourChunkBlocks : kAlphaChunkBlocks;
      auto& list = colour ? cchunks : achunks;
      for (uint32_t b = 0; b < count; b += step)
        list.push_back(EncodeChunk{(uint32_t)first + b, std::min(step, count - b), sid});
    };
    // Uber quality: colour segments carry a dxt1_options() word, alpha segments the quality bits
    const uint32_t alpha_opts = (both ? kSegBothTypes : 0u) | (kDxtQualityUber << kSegAlphaQualityShift);
    switch (it.format) {
      case CRNGPU_FMT_DXT1:
        add_seg(it.out, 8, dxt1_options(perceptual, both, kDxtQualityUber, false, false, 128), true);
        break;
      case CRNGPU_FMT_DXT5A:
        add_seg(it.out, 8, alpha_opts | (3u << kSegCompShift), false);
        break;
      case CRNGPU_FMT_DXN_XY:
      case CRNGPU_FMT_DXN_YX: {
        const uint32_t c0 = it.format == CRNGPU_FMT_DXN_XY ? 0u : 1u;
        add_seg(it.out, 16, alpha_opts | (c0 << kSegCompShift), false);
        add_seg(it.out + 8, 16, alpha_opts | ((1u - c0) << kSegCompShift), false);
        break;
      }
      default:  // DXT5 family: alpha element, then a colour element without 3-colour blocks
        add_seg(it.out, 16, alpha_opts | (3u << kSegCompShift), false);
        add_seg(it.out + 8, 16, dxt1_options(perceptual, false, kDxtQualityUber, false, false, 128), true);
        break;
    }
  }
  EncodeBatch* b = new EncodeBatch;
  b->nblocks = nblocks;
  b->texels = texels;
  b->ntiles = (uint32_t)tiles.size();
  b->ncolour = (uint32_t)cchunks.size();
  b->nalpha = (uint32_t)achunks.size();
  cudaGetDevice(&b->device);
  cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
  b->colour_max = dxt1_chunks_max_grid();
  b->alpha_max = dxt5a_chunks_max_grid();
  cudaError_t e;
  int rc = CRNGPU_OK;
  if (b->colour_max <= 0) { set_error("crngpu_encode_batch_create: encoder shared memory attribute"); rc = CRNGPU_E_DEVICE; }
  auto upload = [&](DevBuf& d, const void* src, size_t bytes, const char* what) {
    if (rc != CRNGPU_OK || !bytes) return;
    if ((e = d.ensure(bytes)) != cudaSuccess || (e = cudaMemcpy(d.ptr, src, bytes, cudaMemcpyHostToDevice)) != cudaSuccess)
      rc = cuda_check(e, what);
  };
  if (rc == CRNGPU_OK && (e = b->blocks.ensure(nblocks * 64)) != cudaSuccess) rc = cuda_check(e, "alloc blocks");
  if (rc == CRNGPU_OK && (e = b->seeds.ensure(nblocks * kDxt1SeedBytes)) != cudaSuccess) rc = cuda_check(e, "alloc seeds");
  upload(b->d_tiles, tiles.data(), tiles.size() * sizeof(GatherTile), "upload gather tiles");
  upload(b->d_segs, segs.data(), segs.size() * sizeof(EncodeSegment), "upload segments");
  upload(b->d_cchunks, cchunks.data(), cchunks.size() * sizeof(EncodeChunk), "upload colour chunks");
  upload(b->d_achunks, achunks.data(), achunks.size() * sizeof(EncodeChunk), "upload alpha chunks");
  if (rc == CRNGPU_OK && (e = cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking)) != cudaSuccess)
    rc = cuda_check(e, "side stream");
  if (rc == CRNGPU_OK && ((e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming)) != cudaSuccess ||
                          (e = cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming)) != cudaSuccess))
    rc = cuda_check(e, "events");
  if (rc != CRNGPU_OK) { destroy(b); return nullptr; }
  return reinterpret_cast<crngpu_encode_batch>(b);
} catch (...) {
  crngpu::exception_status();
  return nullptr;
}

extern "C" int crngpu_encode_batch_launch(crngpu_encode_batch batch, uint32_t flags, void* stream) try {
  clear_error();
  EncodeBatch* b = reinterpret_cast<EncodeBatch*>(batch);
  if (!b || b->magic != 0x454E4342u) { set_error("bad batch"); return CRNGPU_E_PARAM; }
  cudaStream_t s = as_stream(stream);
  int rc;
  if (!b->colour_grid && (rc = autotune(b, s)) != CRNGPU_OK) return rc;
  if (!(flags & CRNGPU_BATCH_GRAPH)) return enqueue(b, s, b->colour_grid, b->alpha_grid);
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
    rc = enqueue(b, cap, b->colour_grid, b->alpha_grid);
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

extern "C" int crngpu_encode_batch_tuning(crngpu_encode_batch batch, int32_t* grids, float* ms, uint32_t n) try {
  clear_error();
  EncodeBatch* b = reinterpret_cast<EncodeBatch*>(batch);
  if (!b || b->magic != 0x454E4342u) { set_error("bad batch"); return CRNGPU_E_PARAM; }
  if (grids) { grids[0] = b->colour_grid; grids[1] = b->alpha_grid; }
  for (uint32_t i = 0; ms && i < n && i < (uint32_t)(kColourVariants + kAlphaVariants); i++)
    ms[i] = i < (uint32_t)kColourVariants ? b->colour_ms[i] : b->alpha_ms[i - kColourVariants];
  return kColourVariants + kAlphaVariants;
} catch (...) {
  return crngpu::exception_status();
}

extern "C" int64_t crngpu_encode_batch_size(crngpu_encode_batch batch, uint64_t* texels) try {
  clear_error();
  EncodeBatch* b = reinterpret_cast<EncodeBatch*>(batch);
  if (!b || b->magic != 0x454E4342u) { set_error("bad batch"); return CRNGPU_E_PARAM; }
  if (texels) *texels = b->texels;
  return (int64_t)b->nblocks;
} catch (...) {
  return crngpu::exception_status();
}

extern "C" int crngpu_encode_batch_destroy(crngpu_encode_batch batch) try {
  clear_error();
  EncodeBatch* b = reinterpret_cast<EncodeBatch*>(batch);
  if (!b || b->magic != 0x454E4342u) { set_error("bad batch"); return CRNGPU_E_PARAM; }
  destroy(b);
  return CRNGPU_OK;
} catch (...) {
  return crngpu::exception_status();
}

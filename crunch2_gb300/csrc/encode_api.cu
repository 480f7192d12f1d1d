// C ABI for the block encoders: batch entry points (dxt1_endpoint_optimizer::compute,
// dxt5_endpoint_optimizer::compute, crn_compress_block) and the plain image path
// (dxt_image::init, crnlib/crn_dxt_image.cpp:283-349,447-493).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "crngpu_internal.h"

namespace crngpu {

namespace {

// crngpu_block_options with their defaults (Uber, alpha threshold 128); false on a bad struct
bool read_options(const crngpu_block_options* o, uint32_t* quality, uint32_t* threshold) {
  *quality = kDxtQualityUber;
  *threshold = 128;
  if (!o) return true;
  if (o->struct_size != sizeof(crngpu_block_options) || o->dxt_quality > kDxtQualityUber ||
      o->dxt1a_alpha_threshold > 255) {
    set_error("bad crngpu_block_options");
    return false;
  }
  *quality = o->dxt_quality;
  *threshold = o->dxt1a_alpha_threshold;
  return true;
}

// Image -> 4x4 blocks with edge clamping (init_task :334-344): texel (x, y) of block (bx, by)
// is img[min(4by+y, h-1)][min(4bx+x, w-1)]. One thread per output texel.
__global__ void k_gather_blocks(const uint8_t* __restrict__ img, uint32_t w, uint32_t h, uint32_t pitch,
                                uint32_t blocks_x, uint64_t total_texels, uint32_t* __restrict__ out) {
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total_texels;
       t += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t blk = t >> 4;
    const uint32_t tin = (uint32_t)t & 15;
    const uint32_t by = (uint32_t)(blk / blocks_x), bx = (uint32_t)(blk - (uint64_t)by * blocks_x);
    const uint32_t x = min(bx * 4 + (tin & 3), w - 1), y = min(by * 4 + (tin >> 2), h - 1);
    const uint8_t* p = img + (uint64_t)y * pitch + (uint64_t)x * 4;
    out[t] = (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
  }
}

// Level -> 4x4 blocks as k_gather_blocks, each texel cooked for the target format (cook_texel).
// Several images (faces and levels) in one launch: job j covers blocks [first[j], first[j + 1]).
__global__ void k_gather_chain(const uint8_t* __restrict__ chain, const GatherImage* __restrict__ imgs, uint32_t nimg,
                               uint32_t total_blocks, uint32_t format, uint32_t* __restrict__ out) {
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (uint64_t)total_blocks * 16;
       t += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t blk = (uint32_t)(t >> 4), tin = (uint32_t)t & 15;
    uint32_t lo = 0, hi = nimg - 1;  // the image holding block blk: the last with first <= blk
    while (lo < hi) {
      const uint32_t mid = (lo + hi + 1) >> 1;
      if (imgs[mid].first <= blk) lo = mid;
      else hi = mid - 1;
    }
    const GatherImage im = imgs[lo];
    const uint32_t b = blk - im.first, by = b / im.bx, bxx = b - by * im.bx;
    const uint32_t x = min(bxx * 4 + (tin & 3), im.w - 1), y = min(by * 4 + (tin >> 2), im.h - 1);
    const uint8_t* p = chain + im.src + ((uint64_t)y * im.w + x) * 4;
    const uint32_t px = (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
    out[t] = cook_texel(format, px);
  }
}

int bytes_per_block(uint32_t fmt) {
  switch (fmt) {
    case CRNGPU_FMT_DXT1: case CRNGPU_FMT_DXT5A: return 8;
    case CRNGPU_FMT_DXT5: case CRNGPU_FMT_DXT5_CCXY: case CRNGPU_FMT_DXT5_XGXR: case CRNGPU_FMT_DXT5_XGBR:
    case CRNGPU_FMT_DXT5_AGBR: case CRNGPU_FMT_DXN_XY: case CRNGPU_FMT_DXN_YX: return 16;
    default: return 0;
  }
}

// Launches the element encoders of one format on device buffers (dxt_image element layout,
// crnlib/crn_dxt_image.cpp:150-200: DXT5 = alpha block then colour block, DXN = X then Y) with
// the optimizer parameters set_block_pixels derives from the pack parameters (:1436-1522): the
// DXT5 colour element never uses 3-colour blocks, transparency or the black trial. d_err
// (optional) receives the DXT1 errors; the black trial needs them, so it uses the per-thread
// staging buffer when d_err is NULL.
int encode_device(const uint8_t* d_in, uint32_t n, uint32_t fmt, uint32_t flags, uint32_t quality, uint32_t threshold,
                  uint8_t* d_out, uint64_t* d_err, cudaStream_t s) {
  const bool perceptual = (flags & CRNGPU_FLAG_PERCEPTUAL) != 0;
  const bool both = (flags & CRNGPU_FLAG_USE_BOTH_BLOCK_TYPES) != 0;
  const bool gray = (flags & CRNGPU_FLAG_GRAYSCALE) != 0;
  switch (fmt) {
    case CRNGPU_FMT_DXT1: {
      const uint32_t opts =
          dxt1_options(perceptual, both, quality, gray, (flags & CRNGPU_FLAG_DXT1A) != 0, threshold);
      // try_alpha_as_black_optimization runs when 3-colour blocks are allowed (crn_dxt1.cpp:2239)
      const bool black = both && (flags & CRNGPU_FLAG_TRANSPARENT_BLACK);
      if (black && !d_err) {
        DevBuf& be = staging(3);
        cudaError_t e = be.ensure((size_t)n * 8);
        if (e != cudaSuccess) return cuda_check(e, "alloc error stage");
        d_err = static_cast<uint64_t*>(be.ptr);
      }
      int rc = launch_dxt1(d_in, n, opts, d_out, 8, d_err, s);
      if (rc == CRNGPU_OK && black) rc = launch_dxt1_black_trial(d_in, n, opts, d_out, 8, d_err, s);
      return rc;
    }
    case CRNGPU_FMT_DXT5A: return launch_dxt5a(d_in, n, 3, both, quality, d_out, 8, s);
    case CRNGPU_FMT_DXN_XY:
    case CRNGPU_FMT_DXN_YX: {
      const int c0 = fmt == CRNGPU_FMT_DXN_XY ? 0 : 1;
      int rc = launch_dxt5a(d_in, n, c0, both, quality, d_out, 16, s);
      if (rc == CRNGPU_OK) rc = launch_dxt5a(d_in, n, 1 - c0, both, quality, d_out + 8, 16, s);
      return rc;
    }
    default: {  // DXT5 family: alpha element, then a colour element that may not use 3-colour blocks
      int rc = launch_dxt5a(d_in, n, 3, both, quality, d_out, 16, s);
      if (rc == CRNGPU_OK)
        rc = launch_dxt1(d_in, n, dxt1_options(perceptual, false, quality, gray, false, threshold), d_out + 8, 16,
                         nullptr, s);
      return rc;
    }
  }
}

// Runs `fn(d_in, d_out, d_err)` with host or device buffers; host buffers are staged.
template <typename F>
int with_buffers(const uint8_t* in, size_t in_bytes, uint8_t* out, size_t out_bytes, uint64_t* err, size_t err_bytes,
                 int mem, cudaStream_t s, F fn) {
  if (mem == CRNGPU_MEM_DEVICE) {
    if (((uintptr_t)in & 15) || ((uintptr_t)out & 7) || ((uintptr_t)err & 7)) {
      set_error("device buffers must be 16-byte (input) / 8-byte (output) aligned");
      return CRNGPU_E_PARAM;
    }
    return fn(in, out, err);
  }
  cudaError_t e;
  DevBuf& bi = staging(0);
  DevBuf& bo = staging(1);
  DevBuf& be = staging(3);
  if ((e = bi.ensure(in_bytes)) != cudaSuccess) return cuda_check(e, "alloc input stage");
  if ((e = bo.ensure(out_bytes)) != cudaSuccess) return cuda_check(e, "alloc output stage");
  if (err && (e = be.ensure(err_bytes)) != cudaSuccess) return cuda_check(e, "alloc error stage");
  if ((e = cudaMemcpyAsync(bi.ptr, in, in_bytes, cudaMemcpyHostToDevice, s)) != cudaSuccess)
    return cuda_check(e, "copy input");
  int rc = fn(static_cast<const uint8_t*>(bi.ptr), static_cast<uint8_t*>(bo.ptr),
              err ? static_cast<uint64_t*>(be.ptr) : nullptr);
  if (rc != CRNGPU_OK) return rc;
  if ((e = cudaMemcpyAsync(out, bo.ptr, out_bytes, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
    return cuda_check(e, "copy output");
  if (err && (e = cudaMemcpyAsync(err, be.ptr, err_bytes, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
    return cuda_check(e, "copy errors");
  return cuda_check(cudaStreamSynchronize(s), "sync");
}

}  // namespace

int launch_gather_chain(const uint8_t* d_chain, const GatherImage* d_imgs, uint32_t nimg, uint32_t blocks,
                        uint32_t format, uint32_t* d_out, cudaStream_t s) {
  if (!nimg || !blocks) return CRNGPU_OK;
  const uint64_t texels = (uint64_t)blocks * 16;
  const uint32_t grid = (uint32_t)std::min<uint64_t>((texels + 255) / 256, 65535);
  k_gather_chain<<<grid, 256, 0, s>>>(d_chain, d_imgs, nimg, blocks, format, d_out);
  return cuda_check(cudaGetLastError(), "launch k_gather_chain");
}

int64_t dds_plain_chain(const uint8_t* rgba_levels, uint32_t width, uint32_t height, uint32_t levels, uint32_t faces,
                        uint32_t format, uint32_t flags, uint32_t quality, uint32_t threshold, void* out,
                        uint64_t out_capacity) {
  const int bpb = bytes_per_block(format);
  if (!bpb) { set_error("unsupported format"); return CRNGPU_E_UNSUPPORTED; }
  if (!rgba_levels || !width || !height || width > 4096 || height > 4096 || !levels || levels > 16 ||
      (faces != 1 && faces != 6)) {
    set_error("dds_plain_chain: bad dimensions, level or face count");
    return CRNGPU_E_PARAM;
  }
  uint32_t full = 1;
  while ((width >> full) || (height >> full)) full++;
  if (levels > full) { set_error("dds_plain_chain: more levels than the mip chain has"); return CRNGPU_E_PARAM; }
  // the images in DDS order (face after face, level after level), which is also the input order
  std::vector<GatherImage> imgs;
  uint64_t src = 0;
  uint32_t blocks = 0;
  for (uint32_t f = 0; f < faces; f++)
    for (uint32_t l = 0; l < levels; l++) {
      const uint32_t w = std::max(1u, width >> l), h = std::max(1u, height >> l);
      const uint32_t bx = (w + 3) / 4, by = (h + 3) / 4;
      imgs.push_back(GatherImage{src, w, h, bx, blocks});
      src += (uint64_t)w * h * 4;
      blocks += bx * by;
    }
  const uint64_t need = (uint64_t)blocks * bpb;
  if (!out || out_capacity < need) return (int64_t)need;
  cudaStream_t s = nullptr;
  cudaError_t e;
  DevBuf& chain = staging(4);
  DevBuf& table = staging(5);
  DevBuf& gathered = staging(6);
  DevBuf& encoded = staging(7);
  if ((e = chain.ensure(src)) != cudaSuccess || (e = table.ensure(sizeof(GatherImage) * imgs.size())) != cudaSuccess ||
      (e = gathered.ensure((size_t)blocks * 64)) != cudaSuccess || (e = encoded.ensure(need)) != cudaSuccess)
    return cuda_check(e, "alloc chain buffers");
  if ((e = cudaMemcpyAsync(chain.ptr, rgba_levels, src, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
      (e = cudaMemcpyAsync(table.ptr, imgs.data(), sizeof(GatherImage) * imgs.size(), cudaMemcpyHostToDevice, s)) !=
          cudaSuccess)
    return cuda_check(e, "upload chain");
  int rc = launch_gather_chain(static_cast<const uint8_t*>(chain.ptr), static_cast<const GatherImage*>(table.ptr),
                               (uint32_t)imgs.size(), blocks, format, static_cast<uint32_t*>(gathered.ptr), s);
  if (rc != CRNGPU_OK) return rc;
  rc = encode_device(static_cast<const uint8_t*>(gathered.ptr), blocks, format, flags, quality, threshold,
                         static_cast<uint8_t*>(encoded.ptr), nullptr, s);
  if (rc != CRNGPU_OK) return rc;
  if ((e = cudaMemcpyAsync(out, encoded.ptr, need, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return cuda_check(e, "copy result");
  return (int64_t)need;
}

}  // namespace crngpu

using namespace crngpu;

extern "C" int crngpu_dxt1_optimize_batch(const uint8_t* rgba_blocks, uint32_t n, const crngpu_dxt1_params* params,
                                          uint8_t* out_blocks, uint64_t* out_error, int mem, void* stream) try {
  clear_error();
  const bool legacy = params && params->struct_size == 16;  // the four-field layout: Uber, no extras
  if (!params || (!legacy && params->struct_size != sizeof(crngpu_dxt1_params)) ||
      (n && (!rgba_blocks || !out_blocks))) {
    set_error("bad arguments");
    return CRNGPU_E_PARAM;
  }
  const uint32_t quality = legacy ? kDxtQualityUber : params->dxt_quality;
  const uint32_t threshold = legacy ? 128u : params->dxt1a_alpha_threshold;
  if (quality > kDxtQualityUber || threshold > 255) { set_error("bad quality or alpha threshold"); return CRNGPU_E_PARAM; }
  const bool gray = !legacy && params->grayscale_sampling, dxt1a = !legacy && params->dxt1a;
  const bool black = !legacy && params->use_transparent_indices_for_black && params->use_alpha_blocks;
  const uint32_t opts = dxt1_options(params->perceptual != 0, params->use_alpha_blocks != 0, quality, gray, dxt1a,
                                     threshold);
  if (!n) return CRNGPU_OK;
  cudaStream_t s = as_stream(stream);
  return with_buffers(rgba_blocks, (size_t)n * 64, out_blocks, (size_t)n * 8, out_error, (size_t)n * 8, mem, s,
                      [&](const uint8_t* in, uint8_t* out, uint64_t* err) {
                        uint64_t* e = err;
                        if (black && !e) {
                          DevBuf& be = staging(3);
                          cudaError_t ce = be.ensure((size_t)n * 8);
                          if (ce != cudaSuccess) return cuda_check(ce, "alloc error stage");
                          e = static_cast<uint64_t*>(be.ptr);
                        }
                        int rc = launch_dxt1(in, n, opts, out, 8, e, s);
                        if (rc == CRNGPU_OK && black) rc = launch_dxt1_black_trial(in, n, opts, out, 8, e, s);
                        return rc;
                      });
} catch (...) {
  return crngpu::exception_status();
}

extern "C" int crngpu_dxt5a_optimize_batch(const uint8_t* rgba_blocks, uint32_t n, uint32_t comp_index,
                                           int32_t use_both_block_types, uint8_t* out_blocks, int mem, void* stream) try {
  clear_error();
  if (comp_index > 3 || (n && (!rgba_blocks || !out_blocks))) { set_error("bad arguments"); return CRNGPU_E_PARAM; }
  if (!n) return CRNGPU_OK;
  cudaStream_t s = as_stream(stream);
  return with_buffers(rgba_blocks, (size_t)n * 64, out_blocks, (size_t)n * 8, nullptr, 0, mem, s,
                      [&](const uint8_t* in, uint8_t* out, uint64_t*) {
                        return launch_dxt5a(in, n, (int)comp_index, use_both_block_types != 0, kDxtQualityUber, out, 8,
                                           s);
                      });
} catch (...) {
  return crngpu::exception_status();
}

extern "C" int crngpu_compress_blocks(const uint8_t* rgba_blocks, uint32_t n, uint32_t format, uint32_t flags,
                                      uint8_t* out_blocks, int mem, void* stream) try {
  return crngpu_compress_blocks_ex(rgba_blocks, n, format, flags, nullptr, out_blocks, mem, stream);
} catch (...) {
  return crngpu::exception_status();
}

extern "C" int crngpu_compress_blocks_ex(const uint8_t* rgba_blocks, uint32_t n, uint32_t format, uint32_t flags,
                                         const crngpu_block_options* options, uint8_t* out_blocks, int mem,
                                         void* stream) try {
  clear_error();
  uint32_t quality, threshold;
  if (!read_options(options, &quality, &threshold)) return CRNGPU_E_PARAM;
  const int bpb = bytes_per_block(format);
  if (!bpb) { set_error("unsupported format"); return CRNGPU_E_UNSUPPORTED; }
  if (n && (!rgba_blocks || !out_blocks)) { set_error("bad arguments"); return CRNGPU_E_PARAM; }
  if (!n) return bpb;
  cudaStream_t s = as_stream(stream);
  const int rc = with_buffers(rgba_blocks, (size_t)n * 64, out_blocks, (size_t)n * bpb, nullptr, 0, mem, s,
                              [&](const uint8_t* in, uint8_t* out, uint64_t*) {
                                return encode_device(in, n, format, flags, quality, threshold, out, nullptr, s);
                              });
  return rc == CRNGPU_OK ? bpb : rc;
} catch (...) {
  return crngpu::exception_status();
}

extern "C" int64_t crngpu_compress_image(const uint8_t* rgba, uint32_t width, uint32_t height, uint32_t pitch_bytes,
                                         uint32_t format, uint32_t flags, uint8_t* out, uint64_t out_size, int mem,
                                         void* stream) try {
  return crngpu_compress_image_ex(rgba, width, height, pitch_bytes, format, flags, nullptr, out, out_size, mem,
                                  stream);
} catch (...) {
  return crngpu::exception_status();
}

extern "C" int64_t crngpu_compress_image_ex(const uint8_t* rgba, uint32_t width, uint32_t height,
                                            uint32_t pitch_bytes, uint32_t format, uint32_t flags,
                                            const crngpu_block_options* options, uint8_t* out, uint64_t out_size,
                                            int mem, void* stream) try {
  clear_error();
  uint32_t quality, threshold;
  if (!read_options(options, &quality, &threshold)) return CRNGPU_E_PARAM;
  const int bpb = bytes_per_block(format);
  if (!bpb) { set_error("unsupported format"); return CRNGPU_E_UNSUPPORTED; }
  if (!rgba || !out || !width || !height) { set_error("bad arguments"); return CRNGPU_E_PARAM; }
  if (!pitch_bytes) pitch_bytes = width * 4;
  if (pitch_bytes < width * 4) { set_error("bad pitch"); return CRNGPU_E_PARAM; }
  const uint32_t bx = (width + 3) / 4, by = (height + 3) / 4;
  const uint64_t n = (uint64_t)bx * by;
  const uint64_t need = n * (uint64_t)bpb;
  if (out_size < need || n > 0xFFFFFFFFull) { set_error("output too small"); return CRNGPU_E_PARAM; }
  cudaStream_t s = as_stream(stream);
  cudaError_t e;
  const size_t img_bytes = (size_t)pitch_bytes * (height - 1) + (size_t)width * 4;
  DevBuf& blocks = staging(2);
  if ((e = blocks.ensure(n * 64)) != cudaSuccess) return cuda_check(e, "alloc blocks");
  const uint8_t* d_img = rgba;
  if (mem != CRNGPU_MEM_DEVICE) {
    DevBuf& bi = staging(0);
    if ((e = bi.ensure(img_bytes)) != cudaSuccess) return cuda_check(e, "alloc image stage");
    if ((e = cudaMemcpyAsync(bi.ptr, rgba, img_bytes, cudaMemcpyHostToDevice, s)) != cudaSuccess)
      return cuda_check(e, "copy image");
    d_img = static_cast<const uint8_t*>(bi.ptr);
  }
  const uint64_t texels = n * 16;
  const uint32_t grid = (uint32_t)((texels + 255) / 256 < 65535 * 8 ? (texels + 255) / 256 : 65535 * 8);
  k_gather_blocks<<<grid, 256, 0, s>>>(d_img, width, height, pitch_bytes, bx, texels, static_cast<uint32_t*>(blocks.ptr));
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(e, "launch k_gather_blocks");
  uint8_t* d_out = out;
  DevBuf* so = nullptr;
  if (mem != CRNGPU_MEM_DEVICE) {
    so = &staging(1);
    if ((e = so->ensure(need)) != cudaSuccess) return cuda_check(e, "alloc output stage");
    d_out = static_cast<uint8_t*>(so->ptr);
  } else if ((uintptr_t)out & 7) {
    set_error("device output must be 8-byte aligned");
    return CRNGPU_E_PARAM;
  }
  int rc = encode_device(static_cast<const uint8_t*>(blocks.ptr), (uint32_t)n, format, flags, quality, threshold, d_out,
                         nullptr, s);
  if (rc != CRNGPU_OK) return rc;
  if (so) {
    if ((e = cudaMemcpyAsync(out, so->ptr, need, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
      return cuda_check(e, "copy output");
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_check(e, "sync");
  }
  return (int64_t)need;
} catch (...) {
  return crngpu::exception_status();
}

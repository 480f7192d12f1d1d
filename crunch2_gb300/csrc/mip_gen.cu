// Mip generation on the GPU: crnlib's mipmapped_texture::generate_mipmaps
// (crnlib/crn_mipmapped_texture.cpp:2140-2215) with its resampler, image_utils::
// resample_multithreaded (crnlib/crn_image_utils.cpp:662-874) over threaded_resampler
// (crnlib/crn_threaded_resampler.cpp:66-357). Every level is resampled from the level-0 image:
//
//   k_mip_linearize   level 0 RGBA8 -> float4 (the sRGB-to-linear table for R, G, B when gamma
//                     filtering, v / 255 otherwise and for alpha);
//   k_mip_resample_x  per source row and destination column: the weighted sum of the column's
//                     contributors (one float4 per texel, contributor order);
//   k_mip_resample_y  per destination texel: the weighted sum over its row contributors, clamped to
//                     [0, 1], then back to 8 bits (255 v + 0.5 truncated, or the 8192-entry
//                     linear-to-sRGB table).
//
// The contributor lists (Resampler::make_clist, crnlib/crn_resampler.cpp:119-412: filter support
// stretched by the scale factor and the filter scale, weights normalised, the rounding residue
// added to the largest weight, clamp or wrap addressing) and the two gamma tables are built on the
// host with the reference's float expressions; the kernels add in the reference's order with
// round-to-nearest multiplies and adds (no contraction), so every level matches the reference.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <tuple>
#include <vector>

#include "crngpu_internal.h"

namespace crngpu {
namespace mip {
namespace {

// ---- the mip filters of crn_mip_filter (crnlib/crn_resample_filters.cpp), published kernels:
// box, tent (triangle), Lanczos (sinc windowed by sinc, 4 lobes), Mitchell-Netravali (B = C = 1/3),
// Kaiser-windowed sinc (40 dB attenuation, half-width 3)
constexpr double kPi = 3.14159265358979323846;

float f_box(float t) { return (t >= -0.5f && t < 0.5f) ? 1.0f : 0.0f; }

float f_tent(float t) {
  if (t < 0.0f) t = -t;
  return t < 1.0f ? 1.0f - t : 0.0f;
}

double sinc(double x) {
  x = x * kPi;
  if (x < 0.01f && x > -0.01f) return 1.0f + x * x * (-1.0f / 6.0f + x * x * 1.0f / 120.0f);
  return std::sin(x) / x;
}

float clean(double t) {
  const float eps = .0000125f;
  if (std::fabs(t) < eps) return 0.0f;
  return (float)t;
}

float f_lanczos4(float t) {
  if (t < 0.0f) t = -t;
  return t < 4.0f ? clean(sinc(t) * sinc(t / 4.0f)) : 0.0f;
}

float mitchell(float t, const float B, const float C) {
  const float tt = t * t;
  if (t < 0.0f) t = -t;
  if (t < 1.0f) {
    t = (((12.0f - 9.0f * B - 6.0f * C) * (t * tt)) + ((-18.0f + 12.0f * B + 6.0f * C) * tt) + (6.0f - 2.0f * B));
    return t / 6.0f;
  }
  if (t < 2.0f) {
    t = (((-1.0f * B - 6.0f * C) * (t * tt)) + ((6.0f * B + 30.0f * C) * tt) + ((-12.0f * B - 48.0f * C) * t) +
         (8.0f * B + 24.0f * C));
    return t / 6.0f;
  }
  return 0.0f;
}
float f_mitchell(float t) { return mitchell(t, 1.0f / 3.0f, 1.0f / 3.0f); }

// modified Bessel function of the first kind, order 0, by its power series
double bessel0(double x) {
  const double eps_ratio = 1E-16;
  const double xh = 0.5 * x;
  double sum = 1.0, pw = 1.0, ds = 1.0;
  int k = 0;
  while (ds > sum * eps_ratio) {
    ++k;
    pw = pw * (xh / k);
    ds = pw * pw;
    sum = sum + ds;
  }
  return sum;
}

double kaiser(double alpha, double half_width, double x) {
  const double ratio = x / half_width;
  return bessel0(alpha * std::sqrt(1 - ratio * ratio)) / bessel0(alpha);
}

float f_kaiser(float t) {
  if (t < 0.0f) t = -t;
  if (t < 3) {
    const float att = 40.0f;
    const float alpha = (float)(std::exp(std::log((double)0.58417 * (att - 20.96)) * 0.4) + 0.07886 * (att - 20.96));
    return (float)clean(sinc(t) * kaiser(alpha, 3, t));
  }
  return 0.0f;
}

struct Filter {
  float (*fn)(float);
  float support;
};
const Filter kFilters[5] = {{f_box, 0.5f}, {f_tent, 1.0f}, {f_lanczos4, 4.0f}, {f_mitchell, 2.0f}, {f_kaiser, 3.0f}};

// Contributors of every destination sample along one axis: list i is [first[i], first[i] + n[i])
// of (pixel, weight).
struct Contribs {
  std::vector<uint32_t> first, n, pixel;
  std::vector<float> weight;
};

int wrap_or_clamp(int j, int src, bool wrap) {
  if (j < 0) return wrap ? (((-j) % src) ? src - ((-j) % src) : 0) : 0;
  if (j >= src) return wrap ? j % src : src - 1;
  return j;
}

// Resampler::make_clist (crnlib/crn_resampler.cpp:119-412) with a zero source offset
bool make_contribs(int src, int dst, const Filter& F, float filter_scale, bool wrap, Contribs& c) {
  const float oo_filter_scale = 1.0f / filter_scale;
  const float nudge = 0.5f;
  const float xscale = dst / (float)src;
  const bool down = xscale < 1.0f;
  const float half_width = down ? (F.support / xscale) * filter_scale : F.support * filter_scale;
  c.first.assign(dst, 0);
  c.n.assign(dst, 0);
  c.pixel.clear();
  c.weight.clear();
  for (int i = 0; i < dst; i++) {
    float center = ((float)i + nudge) / xscale;
    center -= nudge;
    const int left = (int)(float)std::floor(center - half_width);
    const int right = (int)(float)std::ceil(center + half_width);
    auto arg = [&](int j) { return down ? (center - (float)j) * xscale * oo_filter_scale : (center - (float)j) * oo_filter_scale; };
    float total = 0;
    for (int j = left; j <= right; j++) total += F.fn(arg(j));
    const float norm = (float)(1.0f / total);
    total = 0;
    int max_k = -1;
    float max_w = -1e+20f;
    c.first[i] = (uint32_t)c.pixel.size();
    for (int j = left; j <= right; j++) {
      const float w = F.fn(arg(j)) * norm;
      if (w == 0.0f) continue;
      const int k = (int)(c.pixel.size() - c.first[i]);
      c.pixel.push_back((uint32_t)wrap_or_clamp(j, src, wrap));
      c.weight.push_back(w);
      total += w;
      if (w > max_w) { max_w = w; max_k = k; }
    }
    c.n[i] = (uint32_t)(c.pixel.size() - c.first[i]);
    if (max_k < 0 || !c.n[i]) return false;
    if (total != 1.0f) c.weight[c.first[i] + max_k] += 1.0f - total;
  }
  return true;
}

// ---- kernels

__global__ void k_mip_linearize(const uint8_t* __restrict__ src, uint64_t texels, const float* __restrict__ to_linear,
                                int srgb, float4* __restrict__ dst) {
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < texels; t += (uint64_t)gridDim.x * blockDim.x) {
    const uchar4 p = reinterpret_cast<const uchar4*>(src)[t];
    const float inv = 1.0f / 255.0f;
    float4 v;
    v.x = srgb ? to_linear[p.x] : __fmul_rn((float)p.x, inv);
    v.y = srgb ? to_linear[p.y] : __fmul_rn((float)p.y, inv);
    v.z = srgb ? to_linear[p.z] : __fmul_rn((float)p.z, inv);
    v.w = __fmul_rn((float)p.w, inv);
    dst[t] = v;
  }
}

// one thread per (source row, destination column)
__global__ void k_mip_resample_x(const float4* __restrict__ src, uint32_t src_w, uint32_t src_h, uint32_t dst_w,
                                 const uint32_t* __restrict__ first, const uint32_t* __restrict__ n,
                                 const uint32_t* __restrict__ pixel, const float* __restrict__ weight,
                                 float4* __restrict__ tmp) {
  const uint64_t total = (uint64_t)src_h * dst_w;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t y = (uint32_t)(t / dst_w), x = (uint32_t)(t - (uint64_t)y * dst_w);
    const float4* row = src + (size_t)y * src_w;
    float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
    const uint32_t k0 = first[x], k1 = k0 + n[x];
    for (uint32_t k = k0; k < k1; k++) {
      const float4 p = row[pixel[k]];
      const float w = weight[k];
      s.x = __fadd_rn(s.x, __fmul_rn(p.x, w));
      s.y = __fadd_rn(s.y, __fmul_rn(p.y, w));
      s.z = __fadd_rn(s.z, __fmul_rn(p.z, w));
      s.w = __fadd_rn(s.w, __fmul_rn(p.w, w));
    }
    tmp[t] = s;
  }
}

__device__ __forceinline__ uint8_t to_u8_linear(float v) {
  int c = (int)__fadd_rn(__fmul_rn(255.0f, v), .5f);
  return (uint8_t)(c < 0 ? 0 : c > 255 ? 255 : c);
}

// one thread per destination texel
__global__ void k_mip_resample_y(const float4* __restrict__ tmp, uint32_t dst_w, uint32_t dst_h,
                                 const uint32_t* __restrict__ first, const uint32_t* __restrict__ n,
                                 const uint32_t* __restrict__ pixel, const float* __restrict__ weight,
                                 const uint8_t* __restrict__ to_srgb, int srgb, int alpha, uchar4* __restrict__ out) {
  const uint64_t total = (uint64_t)dst_h * dst_w;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t y = (uint32_t)(t / dst_w), x = (uint32_t)(t - (uint64_t)y * dst_w);
    const uint32_t k0 = first[y], cnt = n[y];
    float4 v;
    if (cnt == 1) {
      v = tmp[(size_t)pixel[k0] * dst_w + x];
    } else {
      const float4 p = tmp[(size_t)pixel[k0] * dst_w + x];
      const float w = weight[k0];
      v = make_float4(__fmul_rn(p.x, w), __fmul_rn(p.y, w), __fmul_rn(p.z, w), __fmul_rn(p.w, w));
      for (uint32_t k = k0 + 1; k < k0 + cnt; k++) {
        const float4 q = tmp[(size_t)pixel[k] * dst_w + x];
        const float wk = weight[k];
        v.x = __fadd_rn(v.x, __fmul_rn(q.x, wk));
        v.y = __fadd_rn(v.y, __fmul_rn(q.y, wk));
        v.z = __fadd_rn(v.z, __fmul_rn(q.z, wk));
        v.w = __fadd_rn(v.w, __fmul_rn(q.w, wk));
      }
    }
    v.x = fminf(fmaxf(v.x, 0.0f), 1.0f);
    v.y = fminf(fmaxf(v.y, 0.0f), 1.0f);
    v.z = fminf(fmaxf(v.z, 0.0f), 1.0f);
    v.w = fminf(fmaxf(v.w, 0.0f), 1.0f);
    uchar4 o;
    if (srgb) {
      auto g = [&](float c) {
        int j = (int)__fadd_rn(__fmul_rn(8192.0f, c), .5f);
        j = j < 0 ? 0 : j > 8191 ? 8191 : j;
        return to_srgb[j];
      };
      o.x = g(v.x); o.y = g(v.y); o.z = g(v.z);
    } else {
      o.x = to_u8_linear(v.x); o.y = to_u8_linear(v.y); o.z = to_u8_linear(v.z);
    }
    o.w = alpha ? to_u8_linear(v.w) : (uint8_t)255;
    out[t] = o;
  }
}

// Contributor lists and gamma tables depend only on their parameters: computed once per process.
const Contribs* cached_contribs(int src, int dst, uint32_t filter, float filter_scale, bool wrap) {
  static std::mutex mu;
  static std::map<std::tuple<int, int, uint32_t, float, bool>, std::unique_ptr<Contribs>> cache;
  std::lock_guard<std::mutex> lock(mu);
  auto key = std::make_tuple(src, dst, filter, filter_scale, wrap);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second.get();
  std::unique_ptr<Contribs> c(new Contribs);
  if (!make_contribs(src, dst, kFilters[filter], filter_scale, wrap, *c)) return nullptr;
  return (cache[key] = std::move(c)).get();
}

struct GammaTables {
  float to_linear[256];
  uint8_t to_srgb[8192];
  GammaTables() {
    // resample_multithreaded's tables with the source gamma generate_mipmaps leaves at 2.2
    const float gamma = 2.2f;
    for (int i = 0; i < 256; ++i) to_linear[i] = (float)std::pow(i * 1.0f / 255.0f, gamma);
    const float inv_size = 1.0f / 8192, inv_gamma = 1.0f / gamma;
    for (int i = 0; i < 8192; ++i) {
      const int k = (int)(255.0f * std::pow(i * inv_size, inv_gamma) + .5f);
      to_srgb[i] = (uint8_t)(k < 0 ? 0 : k > 255 ? 255 : k);
    }
  }
};

unsigned grid_for(uint64_t work) {
  const uint64_t g = (work + 255) / 256;
  return (unsigned)(g < 65535ull * 16 ? (g ? g : 1) : 65535ull * 16);
}

}  // namespace
}  // namespace mip
}  // namespace crngpu

using namespace crngpu;
using namespace crngpu::mip;

extern "C" int64_t crngpu_generate_mipmaps(const uint8_t* rgba, uint32_t width, uint32_t height, uint32_t levels,
                                           uint32_t filter, float filter_scale, uint32_t flags, uint8_t* out,
                                           uint64_t out_size, int mem, void* stream) try {
  clear_error();
  if (!rgba || !out || !width || !height || width > 16384 || height > 16384 || filter > 4 || !(filter_scale > 0.0f)) {
    set_error("crngpu_generate_mipmaps: bad arguments");
    return CRNGPU_E_PARAM;
  }
  uint32_t full = 1;
  while ((width >> full) || (height >> full)) full++;
  if (!levels) levels = full;
  if (levels > full) { set_error("crngpu_generate_mipmaps: more levels than the mip chain has"); return CRNGPU_E_PARAM; }
  uint64_t need = 0;
  for (uint32_t l = 0; l < levels; l++) need += (uint64_t)std::max(1u, width >> l) * std::max(1u, height >> l) * 4;
  if (out_size < need) { set_error("crngpu_generate_mipmaps: output too small"); return CRNGPU_E_PARAM; }
  const bool srgb = (flags & CRNGPU_MIP_SRGB) != 0, wrap = (flags & CRNGPU_MIP_WRAP) != 0,
             alpha = (flags & CRNGPU_MIP_ALPHA) != 0;
  cudaStream_t s = as_stream(stream);
  static const GammaTables gt;
  const float* to_linear = gt.to_linear;
  const uint8_t* to_srgb = gt.to_srgb;
  // contributor lists of every level, both axes, in one upload
  struct Axis { uint32_t ofs_first, ofs_pix, count; };
  std::vector<uint32_t> firsts, ns, pixels;
  std::vector<float> weights;
  std::vector<Axis> ax(2 * levels);
  for (uint32_t l = 1; l < levels; l++)
    for (int a = 0; a < 2; a++) {
      const int src = a ? (int)height : (int)width;
      const int dst = std::max(1, src >> l);
      const Contribs* cp = cached_contribs(src, dst, filter, filter_scale, wrap);
      if (!cp) {
        set_error("crngpu_generate_mipmaps: filter has no contributors");
        return CRNGPU_E_PARAM;
      }
      const Contribs& c = *cp;
      Axis& A = ax[2 * l + a];
      A.ofs_first = (uint32_t)firsts.size();
      A.ofs_pix = (uint32_t)pixels.size();
      A.count = (uint32_t)dst;
      for (uint32_t f : c.first) firsts.push_back(f);
      for (uint32_t k : c.n) ns.push_back(k);
      pixels.insert(pixels.end(), c.pixel.begin(), c.pixel.end());
      weights.insert(weights.end(), c.weight.begin(), c.weight.end());
    }
  const uint64_t texels0 = (uint64_t)width * height;
  cudaError_t e;
  DevBuf& tables = staging(4);
  DevBuf& work = staging(5);
  const size_t tab_bytes = 256 * 4 + 8192 + (firsts.size() + ns.size() + pixels.size()) * 4 + weights.size() * 4 + 64;
  const size_t max_tmp = (size_t)std::max(1u, width >> 1) * height;  // largest x-pass image (level 1)
  if ((e = tables.ensure(tab_bytes)) != cudaSuccess) return cuda_check(e, "alloc mip tables");
  if ((e = work.ensure((texels0 + max_tmp) * sizeof(float4) + texels0 * 4)) != cudaSuccess)
    return cuda_check(e, "alloc mip work");
  std::vector<uint8_t> host(tab_bytes, 0);
  size_t o = 0;
  auto put = [&](const void* p, size_t bytes) { std::memcpy(host.data() + o, p, bytes); o += (bytes + 15) & ~(size_t)15; };
  const size_t o_lin = o; put(to_linear, sizeof(gt.to_linear));
  const size_t o_srgb = o; put(to_srgb, sizeof(gt.to_srgb));
  const size_t o_first = o; put(firsts.data(), firsts.size() * 4);
  const size_t o_n = o; put(ns.data(), ns.size() * 4);
  const size_t o_pix = o; put(pixels.data(), pixels.size() * 4);
  const size_t o_w = o; put(weights.data(), weights.size() * 4);
  if ((e = cudaMemcpyAsync(tables.ptr, host.data(), o, cudaMemcpyHostToDevice, s)) != cudaSuccess)
    return cuda_check(e, "upload mip tables");
  uint8_t* tb = static_cast<uint8_t*>(tables.ptr);
  float4* base = static_cast<float4*>(work.ptr);
  float4* tmp = base + texels0;
  uint8_t* d_in = reinterpret_cast<uint8_t*>(tmp + max_tmp);
  uint8_t* d_out = out;
  // host buffers are staged through device memory
  DevBuf* so = nullptr;
  if (mem != CRNGPU_MEM_DEVICE) {
    if ((e = cudaMemcpyAsync(d_in, rgba, texels0 * 4, cudaMemcpyHostToDevice, s)) != cudaSuccess)
      return cuda_check(e, "copy level 0");
    so = &staging(6);
    if ((e = so->ensure(need)) != cudaSuccess) return cuda_check(e, "alloc mip output");
    d_out = static_cast<uint8_t*>(so->ptr);
  } else {
    if (((uintptr_t)rgba & 3) || ((uintptr_t)out & 3)) { set_error("device buffers must be 4-byte aligned"); return CRNGPU_E_PARAM; }
    d_in = const_cast<uint8_t*>(rgba);
  }
  // level 0 as given
  if ((e = cudaMemcpyAsync(d_out, d_in, texels0 * 4, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
    return cuda_check(e, "copy level 0 out");
  if (levels > 1) {
    k_mip_linearize<<<grid_for(texels0), 256, 0, s>>>(d_in, texels0, reinterpret_cast<const float*>(tb + o_lin),
                                                        srgb ? 1 : 0, base);
    uint64_t ofs = texels0 * 4;
    for (uint32_t l = 1; l < levels; l++) {
      const uint32_t dw = std::max(1u, width >> l), dh = std::max(1u, height >> l);
      const Axis& X = ax[2 * l], &Y = ax[2 * l + 1];
      const uint32_t* fi = reinterpret_cast<const uint32_t*>(tb + o_first);
      const uint32_t* nn = reinterpret_cast<const uint32_t*>(tb + o_n);
      const uint32_t* px = reinterpret_cast<const uint32_t*>(tb + o_pix);
      const float* wt = reinterpret_cast<const float*>(tb + o_w);
      // contributor offsets are local to each axis list: rebase the pixel / weight pointers
      k_mip_resample_x<<<grid_for((uint64_t)height * dw), 256, 0, s>>>(base, width, height, dw, fi + X.ofs_first,
                                                                        nn + X.ofs_first, px + X.ofs_pix,
                                                                        wt + X.ofs_pix, tmp);
      k_mip_resample_y<<<grid_for((uint64_t)dh * dw), 256, 0, s>>>(tmp, dw, dh, fi + Y.ofs_first, nn + Y.ofs_first,
                                                                    px + Y.ofs_pix, wt + Y.ofs_pix, tb + o_srgb,
                                                                    srgb ? 1 : 0, alpha ? 1 : 0,
                                                                    reinterpret_cast<uchar4*>(d_out + ofs));
      ofs += (uint64_t)dw * dh * 4;
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(e, "launch mip kernels");
  }
  if (so) {
    if ((e = cudaMemcpyAsync(out, so->ptr, need, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
      return cuda_check(e, "copy mips");
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_check(e, "sync");
  }
  return (int64_t)need;
} catch (...) {
  return crngpu::exception_status();
}

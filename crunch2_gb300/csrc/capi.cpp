// Library-wide pieces of the C ABI: version, last-error text, device buffers.
#include <cuda_runtime.h>

#include <cstdlib>
#include <mutex>
#include <new>
#include <string>

#include "crngpu_internal.h"
#include "host_alloc.h"

namespace crngpu {

namespace {
thread_local std::string g_last_error;
}

std::mutex& device_setup_mutex() {
  static std::mutex mu;
  return mu;
}

void set_error(const std::string& msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }

int exception_status() noexcept {
  int rc = CRNGPU_E_DEVICE;
  const char* msg = "internal error";
  try {
    throw;
  } catch (const std::bad_alloc&) {
    rc = CRNGPU_E_NOMEM;
    msg = "out of host memory";
  } catch (...) {
  }
  try {
    g_last_error = msg;
  } catch (...) {
  }
  return rc;
}
const char* last_error_cstr() { return g_last_error.c_str(); }

int cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return CRNGPU_OK;
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return CRNGPU_E_DEVICE;
}

cudaError_t DevBuf::ensure(size_t bytes) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (ptr && cap >= bytes && dev == device) return cudaSuccess;
  release();
  size_t want = bytes < 256 ? 256 : bytes;
  want = (want + want / 4 + 255) & ~(size_t)255;  // grow with headroom, 256-byte multiple
  e = cudaMalloc(&ptr, want);
  if (e != cudaSuccess) {
    ptr = nullptr;
    cap = 0;
    return e;
  }
  cap = want;
  device = dev;
  return cudaSuccess;
}

void DevBuf::release() {
  if (ptr) {
    int cur = -1;
    cudaGetDevice(&cur);
    if (device >= 0 && device != cur) cudaSetDevice(device);
    cudaFree(ptr);
    if (device >= 0 && device != cur && cur >= 0) cudaSetDevice(cur);
  }
  ptr = nullptr;
  cap = 0;
  device = -1;
}

// Host allocation hooks of the transcoder's state (host_alloc.h). Each allocation carries a
// 16-byte header with the hooks that made it, so it is always freed by the same allocator.
namespace {
struct HostHooks {
  HostReallocFn realloc_fn = nullptr;
  HostMsizeFn msize_fn = nullptr;
  void* user = nullptr;
};
std::mutex g_host_mu;
HostHooks g_host;
struct alignas(16) AllocHeader {
  HostReallocFn fn;
  void* user;
};
}  // namespace

// Staging buffers for host-memory calls; one set per host thread so concurrent callers on
// different threads never share them.
DevBuf& staging(int slot) {
  thread_local DevBuf bufs[8];
  return bufs[slot & 7];
}

void set_host_hooks(HostReallocFn realloc_fn, HostMsizeFn msize_fn, void* user) {
  std::lock_guard<std::mutex> lock(g_host_mu);
  g_host = (realloc_fn && msize_fn) ? HostHooks{realloc_fn, msize_fn, user} : HostHooks{};
}

void* host_alloc(size_t bytes) {
  HostHooks h;
  {
    std::lock_guard<std::mutex> lock(g_host_mu);
    h = g_host;
  }
  const size_t total = bytes + sizeof(AllocHeader);
  void* p = nullptr;
  if (h.realloc_fn) {
    size_t actual = 0;
    p = h.realloc_fn(nullptr, total, &actual, true, h.user);
  } else {
    p = std::malloc(total);
  }
  if (!p) return nullptr;
  AllocHeader* hd = static_cast<AllocHeader*>(p);
  hd->fn = h.realloc_fn;
  hd->user = h.user;
  return hd + 1;
}

void host_free(void* q) {
  if (!q) return;
  AllocHeader* hd = static_cast<AllocHeader*>(q) - 1;
  if (hd->fn) hd->fn(hd, 0, nullptr, true, hd->user);
  else std::free(hd);
}

}  // namespace crngpu

namespace crngpu {
int set_work_counter(bool on, cudaStream_t s);
int read_work_counter(uint64_t* value, cudaStream_t s);
int set_stage_wait_polls(uint32_t polls);
int stage_wait_counters(uint32_t out[2], bool reset);
int set_expand_wait_polls(uint32_t polls);
int expand_wait_counters(uint32_t out[2], bool reset);
int set_mma_wait_polls(uint32_t polls);
int mma_wait_counter(uint32_t* out, bool reset);
}

extern "C" int crngpu_force_wait_timeouts(int on) {
  crngpu::clear_error();
  const uint32_t stage = on ? 0u : (1u << 22), mma = on ? 0u : (1u << 24);
  int rc = crngpu::set_stage_wait_polls(stage);
  if (rc == CRNGPU_OK) rc = crngpu::set_expand_wait_polls(stage);
  if (rc == CRNGPU_OK) rc = crngpu::set_mma_wait_polls(mma);
  return rc;
}

extern "C" int crngpu_wait_counters(crngpu_wait_stats* out, int reset) {
  crngpu::clear_error();
  if (!out) { crngpu::set_error("NULL output"); return CRNGPU_E_PARAM; }
  uint32_t st[2] = {0, 0}, ex[2] = {0, 0}, mma = 0;
  int rc = crngpu::stage_wait_counters(st, reset != 0);
  if (rc == CRNGPU_OK) rc = crngpu::expand_wait_counters(ex, reset != 0);
  if (rc == CRNGPU_OK) rc = crngpu::mma_wait_counter(&mma, reset != 0);
  if (rc != CRNGPU_OK) return rc;
  out->encode_stage_timeouts = st[0];
  out->encode_drain_failures = st[1];
  out->expand_stage_timeouts = ex[0];
  out->expand_drain_failures = ex[1];
  out->mma_wait_timeouts = mma;
  return CRNGPU_OK;
}

extern "C" int crngpu_profile_counters(int enable, uint64_t* dxt1_evaluations, void* stream) {
  crngpu::clear_error();
  cudaStream_t s = crngpu::as_stream(stream);
  if (dxt1_evaluations) {
    const int rc = crngpu::read_work_counter(dxt1_evaluations, s);
    if (rc != CRNGPU_OK) return rc;
  }
  return crngpu::set_work_counter(enable != 0, s);
}

extern "C" const char* crngpu_version(void) { return "crngpu 0.1 (sm_103a)"; }
extern "C" const char* crngpu_last_error(void) { return crngpu::last_error_cstr(); }

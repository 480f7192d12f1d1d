// Host memory of the transcoder's state (contexts, parsed files, palettes, launch plans, batches)
// goes through the allocation hooks a caller installs with crnd_set_memory_callbacks, as the
// reference's crnd allocates all of its state through them (crnd_malloc / crnd_realloc / crnd_free,
// inc/crn_decomp.h:2436-2535). Without hooks it is malloc / free. Every allocation remembers the
// hooks that made it, so memory is always returned to the allocator it came from even if the
// hooks change in between.
#pragma once
#include <cstddef>
#include <new>
#include <utility>
#include <vector>

namespace crngpu {

using HostReallocFn = void* (*)(void* p, size_t size, size_t* actual_size, bool movable, void* user);
using HostMsizeFn = size_t (*)(void* p, void* user);

// Installs (or, with a NULL function, removes) the hooks for later allocations.
void set_host_hooks(HostReallocFn realloc_fn, HostMsizeFn msize_fn, void* user);
void* host_alloc(size_t bytes);  // NULL on failure
void host_free(void* p);

template <class T>
struct HostAlloc {
  using value_type = T;
  HostAlloc() = default;
  template <class U>
  HostAlloc(const HostAlloc<U>&) {}
  T* allocate(size_t n) {
    void* p = host_alloc(n * sizeof(T));
    if (!p) throw std::bad_alloc();
    return static_cast<T*>(p);
  }
  void deallocate(T* p, size_t) { host_free(p); }
  template <class U>
  bool operator==(const HostAlloc<U>&) const { return true; }
  template <class U>
  bool operator!=(const HostAlloc<U>&) const { return false; }
};

template <class T>
using HVec = std::vector<T, HostAlloc<T>>;

// Base for objects allocated with new / delete through the hooks.
struct HostObject {
  static void* operator new(size_t n) {
    void* p = host_alloc(n);
    if (!p) throw std::bad_alloc();
    return p;
  }
  static void* operator new(size_t n, const std::nothrow_t&) noexcept { return host_alloc(n); }
  static void operator delete(void* p) { host_free(p); }
  static void operator delete(void* p, const std::nothrow_t&) noexcept { host_free(p); }
};

}  // namespace crngpu

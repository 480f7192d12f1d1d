// Internal helpers shared by the crngpu translation units (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/crngpu.h"

namespace crngpu {

// Thread-local last-error text behind crngpu_last_error().
void set_error(const std::string& msg);
void clear_error();
const char* last_error_cstr();

// Records `what` + the CUDA error string and returns CRNGPU_E_DEVICE when e != cudaSuccess.
int cuda_check(cudaError_t e, const char* what);

// A device buffer owned by the library; grows on demand, never shrinks.
struct DevBuf {
  void* ptr = nullptr;
  size_t cap = 0;
  int device = -1;
  cudaError_t ensure(size_t bytes);
  void release();
  ~DevBuf() { release(); }
};

// Per-device scratch for host-memory calls (input/output staging).
DevBuf& staging(int slot);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

}  // namespace crngpu

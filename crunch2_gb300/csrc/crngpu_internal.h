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

// Per-thread scratch for host-memory calls (input/output staging), slots 0..7: 0-3 the encoders,
// 4-6 mip generation.
DevBuf& staging(int slot);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Batched block encoding (many textures, mixed formats). A segment is one element of one texture
// over its gathered blocks [first_block, first_block + count): the colour half of DXT1/DXT5, the
// alpha of DXT5/DXT5A or one DXN channel; block b's 8 bytes go to out + (b - first_block) * stride.
struct EncodeSegment {
  uint8_t* out;
  uint32_t first_block, count, stride, options;
};
constexpr uint32_t kSegPerceptual = 1u, kSegThreeColour = 2u, kSegBothTypes = 4u, kSegCompShift = 8u;
// a run of consecutive blocks of one segment, the unit a warp takes
struct EncodeChunk {
  uint32_t first, count, segment;
};
constexpr uint32_t kColourChunkBlocks = 8;  // blocks per DXT1 chunk (the encoder's blocks per warp)
int dxt1_chunks_max_grid();
int dxt5a_chunks_max_grid();
int launch_dxt1_chunks(const uint8_t* d_blocks, const EncodeChunk* d_chunks, uint32_t nchunks,
                       const EncodeSegment* d_segs, int grid, cudaStream_t s);
int launch_dxt5a_chunks(const uint8_t* d_blocks, const EncodeChunk* d_chunks, uint32_t nchunks,
                        const EncodeSegment* d_segs, int grid, cudaStream_t s);

}  // namespace crngpu

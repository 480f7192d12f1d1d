// Learned DXT1 endpoint proposal: a 48 -> 256 (GELU) -> 256 (GELU) -> 8 MLP trained and run on
// the 5th-generation tensor cores (tcgen05.mma, BF16 operands from shared memory, FP32
// accumulators in tensor memory). This part has no counterpart in the reference; it replaces
// the initial guess and most of the refinement of dxt1_endpoint_optimizer (crnlib/crn_dxt1.cpp)
// for blocks where it is good enough, and the exact optimizer stays the fallback and the arbiter of that error.
//
// Inputs: 16 texels x RGB scaled to [0, 1]. Outputs: y[0..5] = low/high endpoint (r/31, g/63,
// b/31) of the plain optimizer's 4-colour solution, y[6] = log2(1 + block error)/16, the
// network's prediction of the error the plain optimizer reaches (the fallback bound); y[7] unused.
//
// Inference (crngpu_mlp_forward, the learned encode) runs as one fused persistent kernel,
// k_mlp_infer: weights resident in shared memory, activations kept on the SM.
// Training GEMMs go through k_gemm_tc: C[M x N] = sum_k A(m, k) B(n, k), a 128 x BN tile per CTA,
// K staged 64 at a time into shared memory in the no-swizzle K-major core-matrix layout
// (8 x 8 BF16 core matrices, 128 bytes each), four K=16 MMAs per stage issued by one thread,
// completion through tcgen05.commit on an mbarrier (bounded wait), epilogue from TMEM with
// tcgen05.ld. Operands are fp32, bf16 or raw RGBA8 blocks with arbitrary strides, so the
// transposed products of the backward pass need no separate transpose kernels.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>

#include "crngpu_internal.h"

namespace crngpu {



namespace mlp {

constexpr int kIn = 48, kHid = 256, kOut = 8, kOutPad = 16;
constexpr int BM = 128, BK = 64;
constexpr int kTmemCols = 128;
constexpr uint32_t kWaitLimit = 1u << 24;  // bounded mbarrier polls (~ tens of ms), then error

enum OpKind : int { OP_F32 = 0, OP_BF16 = 1, OP_PIXELS = 2 };
// epilogues
enum Epi : int {
  EPI_STORE = 0,       // C = acc (+ bias)
  EPI_BIAS_GELU = 1,   // Cpre = acc + bias (fp32), Cb = bf16(gelu(Cpre))
  EPI_GELU_GRAD = 2,   // Cb = bf16(acc * gelu'(pre)), C (fp32) = same value
};

struct Operand {
  const void* p;
  int kind;
  long long s_row, s_k;  // element (row, k) at p[row * s_row + k * s_k]; OP_PIXELS: see load_op
  int pix_sample_is_row; // OP_PIXELS: 1 -> row = sample, k = feature; 0 -> row = feature, k = sample
};

struct GemmArgs {
  Operand a, b;
  int M, N, K;
  int epi;
  float* C;              // fp32 out (row-major, ldc)
  __nv_bfloat16* Cb;     // bf16 out (row-major, ldc)
  const float* pre;      // EPI_GELU_GRAD: pre-activation (row-major, ldc)
  const float* bias;     // per column
  int ldc;
  uint32_t* err;         // set to 1 if an mbarrier wait timed out
  int kslice;            // split K: CTA z covers K columns [z * kslice, (z + 1) * kslice) (0: all of K)
  float* part;           // split K: CTA z writes its raw partial tile to part + z * M * N (row-major, N)
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (r, k) of a tile with `kt` K-columns in the no-swizzle K-major layout
__device__ __forceinline__ uint32_t kmaj_off(int r, int k, int kt) {
  return (uint32_t)((r >> 3) * ((kt >> 3) * 128) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// tcgen05 shared-memory matrix descriptor: start, leading (K) and stride (8-row) byte offsets,
// descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr & 0x3FFFF) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

__device__ __forceinline__ float gelu(float x) {
  const float c = 0.7978845608f;  // sqrt(2/pi), tanh form
  return 0.5f * x * (1.f + tanhf(c * (x + 0.044715f * x * x * x)));
}
__device__ __forceinline__ float gelu_grad(float x) {
  const float c = 0.7978845608f;
  const float t = tanhf(c * (x + 0.044715f * x * x * x));
  return 0.5f * (1.f + t) + 0.5f * x * (1.f - t * t) * c * (1.f + 3.f * 0.044715f * x * x);
}

__device__ __forceinline__ float load_op(const Operand& o, int row, int k, int rows, int ks) {
  if (row >= rows || k >= ks) return 0.f;
  switch (o.kind) {
    // read-only inputs of the product: non-coherent loads, which the compiler may also move ahead of
    // the shared-memory stores of the staging loop
    case OP_F32: return __ldg(reinterpret_cast<const float*>(o.p) + row * o.s_row + k * o.s_k);
    case OP_BF16: return __bfloat162float(__ldg(reinterpret_cast<const __nv_bfloat16*>(o.p) + row * o.s_row + k * o.s_k));
    default: {
      const int s = o.pix_sample_is_row ? row : k, f = o.pix_sample_is_row ? k : row;
      const uint8_t* px = reinterpret_cast<const uint8_t*>(o.p);
      return (float)__ldg(px + (long long)s * 64 + (f / 3) * 4 + f % 3) * (1.0f / 255.0f);
    }
  }
}

// Polls of a first wait on a tcgen05.commit (a test hook can lower it to force the timeout path);
// after a timeout the in-flight MMAs are drained with kDrainPolls, which the hook does not change,
// so TMEM and shared memory are never released under a running MMA. Timeouts are counted.
constexpr uint32_t kDrainPolls = 1u << 26;
__device__ uint32_t g_mma_wait_polls = kWaitLimit;
__device__ unsigned int g_mma_wait_timeouts;

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint32_t polls) {
  uint32_t done = 0;
  for (uint32_t it = 0; it < polls && !done; it++) {
    asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
                 : "=r"(done)
                 : "r"(bar), "r"(parity));
  }
  return done != 0;
}

// C tile (blockIdx.x: 128 rows of M, blockIdx.y: BN columns of N) = A x B^T over all of K, or --
// split K, for products whose M x N has few tiles but whose K is the batch -- over the slice of K
// of blockIdx.z, written raw to g.part for k_splitk_sum.
template <int BN>
__global__ void __launch_bounds__(128) k_gemm_tc(GemmArgs g) {
  __shared__ __align__(1024) unsigned char sa[BM * BK * 2];
  __shared__ __align__(1024) unsigned char sb[BN * BK * 2];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "n"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)));
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base;
  const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
  uint32_t phase = 0;
  bool ok = true;
  const int kbeg = g.kslice ? (int)blockIdx.z * g.kslice : 0;
  const int kend = g.kslice ? min(g.K, kbeg + g.kslice) : g.K;
  const int nk = (kend - kbeg + BK - 1) / BK;
  for (int kc = 0; kc < nk; kc++) {
    const int k0 = kbeg + kc * BK;
    // stage A (BM x BK) and B (BN x BK); the faster-varying index follows the operand's
    // contiguous dimension so global reads coalesce. Eight elements per thread at a time: their
    // loads are all in flight before the first conversion and store.
    auto stage = [&](const Operand& o, int rows_tile, int row0, int rows, unsigned char* dst) {
      if (o.kind == OP_BF16 && o.s_k == 1 && (o.s_row & 7) == 0 && ((uintptr_t)o.p & 15) == 0) {
        // BF16 rows with K contiguous: 8 consecutive K of a row are one 16-byte segment of the
        // K-major core-matrix layout, copied with one load and one store
        const __nv_bfloat16* src = reinterpret_cast<const __nv_bfloat16*>(o.p);
#pragma unroll 4
        for (int e = tid; e < rows_tile * (BK / 8); e += 128) {
          const int r = e / (BK / 8), kg = e - r * (BK / 8);
          const int row = row0 + r, k = k0 + kg * 8;
          uint4 v = make_uint4(0u, 0u, 0u, 0u);
          if (row < rows && k + 8 <= g.K) {
            v = __ldg(reinterpret_cast<const uint4*>(src + (long long)row * o.s_row + k));
          } else if (row < rows) {
            __nv_bfloat16 h[8];
#pragma unroll
            for (int u = 0; u < 8; u++) h[u] = k + u < g.K ? src[(long long)row * o.s_row + k + u] : __float2bfloat16(0.f);
            v = *reinterpret_cast<const uint4*>(h);
          }
          *reinterpret_cast<uint4*>(dst + kmaj_off(r, kg * 8, BK)) = v;
        }
        return;
      }
      const bool rmaj = o.kind != OP_PIXELS && o.s_row == 1;
      for (int e0 = tid; e0 < rows_tile * BK; e0 += 128 * 8) {
        float v[8];
        int rr[8], kk[8];
#pragma unroll
        for (int u = 0; u < 8; u++) {
          const int e = e0 + u * 128;
          if (rmaj) { rr[u] = e % rows_tile; kk[u] = e / rows_tile; } else { kk[u] = e % BK; rr[u] = e / BK; }
          v[u] = e < rows_tile * BK ? load_op(o, row0 + rr[u], k0 + kk[u], rows, g.K) : 0.f;
        }
#pragma unroll
        for (int u = 0; u < 8; u++)
          if (e0 + u * 128 < rows_tile * BK)
            *reinterpret_cast<__nv_bfloat16*>(dst + kmaj_off(rr[u], kk[u], BK)) = __float2bfloat16(v[u]);
      }
    };
    stage(g.a, BM, m0, g.M, sa);
    stage(g.b, BN, n0, g.N, sb);
    asm volatile("fence.proxy.async.shared::cta;");  // generic-proxy smem writes -> tensor core reads
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
      for (int ks = 0; ks < BK / 16; ks++) {
        const uint64_t ad = make_desc(smem_u32(sa) + ks * 256, 128, (BK / 8) * 128);
        const uint64_t bd = make_desc(smem_u32(sb) + ks * 256, 128, (BK / 8) * 128);
        const uint32_t acc = (kc > 0 || ks > 0) ? 1u : 0u;
        asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                     "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
                     "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(&mbar)));
    }
    // the MMAs read shared memory asynchronously: wait before restaging it
    const bool done = mbar_wait(smem_u32(&mbar), phase, g_mma_wait_polls);
    asm volatile("tcgen05.fence::after_thread_sync;");
    ok = __syncthreads_and(done) != 0;  // uniform across the CTA
    if (!ok) {
      // drain the in-flight MMAs (long bound) before TMEM is released
      if (tid == 0) atomicAdd(&g_mma_wait_timeouts, 1u);
      mbar_wait(smem_u32(&mbar), phase, kDrainPolls);
      asm volatile("tcgen05.fence::after_thread_sync;");
      break;
    }
    phase ^= 1;
  }
  if (!ok) {
    if (tid == 0) atomicExch(g.err, 1u);
  } else {
    // epilogue: warp w owns rows 32w..32w+31 of the tile, 16 columns per tcgen05.ld
    const int row = m0 + warp * 32 + lane;
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 16) {
      uint32_t r[16];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;");
      if (row < g.M) {
#pragma unroll
        for (int j = 0; j < 16; j++) {
          const int col = n0 + c0 + j;
          if (col >= g.N) continue;
          float v = __uint_as_float(r[j]);
          if (g.part) {
            g.part[((long long)blockIdx.z * g.M + row) * g.N + col] = v;
            continue;
          }
          const long long o = (long long)row * g.ldc + col;
          if (g.epi == EPI_STORE) {
            if (g.bias) v += g.bias[col];
            if (g.C) g.C[o] = v;
            if (g.Cb) g.Cb[o] = __float2bfloat16(v);
          } else if (g.epi == EPI_BIAS_GELU) {
            v += g.bias[col];
            g.C[o] = v;
            g.Cb[o] = __float2bfloat16(gelu(v));
          } else {
            v *= gelu_grad(g.pre[o]);
            if (g.C) g.C[o] = v;
            g.Cb[o] = __float2bfloat16(v);
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(kTmemCols));
}

// Split K: C[row, col] (+ bias) = the sum of the slices' partial tiles, in slice order.
__global__ void k_splitk_sum(const float* __restrict__ part, int slices, int M, int N, float* __restrict__ C, int ldc,
                             const float* __restrict__ bias) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M * N) return;
  const int row = i / N, col = i - row * N;
  float v = 0.f;
  for (int z = 0; z < slices; z++) v += part[(long long)z * M * N + i];
  if (bias) v += bias[col];
  C[(long long)row * ldc + col] = v;
}

// ------------------------------------------------------------------------------------------
// Fused inference: the whole 48 -> 256 -> 256 -> 16 forward pass of 128 blocks per tile in one
// persistent CTA per SM. All weights stay in shared memory in the K-major core-matrix layout
// (W2 128 KB, W1 24 KB, W3 8 KB); the activations of a tile never leave the SM: input features
// and hidden layers go through one 64 KB shared-memory tile (features alias its first 12 KB),
// accumulators through 256 TMEM columns reused by all three layers. Same arithmetic as the
// training forward (bf16 operands, fp32 accumulation, bias + tanh-GELU in fp32, bf16 hidden).
constexpr int kInferThreads = 256;
constexpr uint32_t kSmW2 = 0, kSmW1 = kSmW2 + kHid * kHid * 2, kSmW3 = kSmW1 + kHid * kIn * 2,
                   kSmH = kSmW3 + kOutPad * kHid * 2, kSmB1 = kSmH + BM * kHid * 2, kSmB2 = kSmB1 + kHid * 4,
                   kSmB3 = kSmB2 + kHid * 4, kSmBar = kSmB3 + kOutPad * 4, kSmTmem = kSmBar + 8,
                   kInferSmem = kSmTmem + 8;
static_assert(kInferSmem <= 232448, "fused forward exceeds the 227 KB shared-memory limit");

// byte offset of the 16-byte row segment (row r, K-group kg) in a K-major tile with kt K-columns
__device__ __forceinline__ uint32_t kseg(int r, int kg, int kt) {
  return (uint32_t)((r >> 3) * ((kt >> 3) * 128) + kg * 128 + (r & 7) * 16);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc) {
  asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
               "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
               "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;");
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);  // .x = a (low half), .y = b
  return *reinterpret_cast<const uint32_t*>(&h);
}

// hidden-layer epilogue: TMEM accumulators of this thread's row, columns [c_lo, c_lo + 128),
// + bias, GELU, bf16 into the K-major hidden tile
__device__ __forceinline__ void hidden_epilogue(uint32_t tmem, int quarter, int row, int c_lo, const float* bias,
                                                unsigned char* sH) {
#pragma unroll 1
  for (int c0 = c_lo; c0 < c_lo + 128; c0 += 16) {
    uint32_t r[16];
    tmem_ld16(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c0, r);
    uint32_t w[8];
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const float a = gelu(__uint_as_float(r[2 * j]) + bias[c0 + 2 * j]);
      const float b = gelu(__uint_as_float(r[2 * j + 1]) + bias[c0 + 2 * j + 1]);
      w[j] = pack_bf16(a, b);
    }
    *reinterpret_cast<uint4*>(sH + kseg(row, c0 >> 3, kHid)) = make_uint4(w[0], w[1], w[2], w[3]);
    *reinterpret_cast<uint4*>(sH + kseg(row, (c0 >> 3) + 1, kHid)) = make_uint4(w[4], w[5], w[6], w[7]);
  }
}

// Waits for the tcgen05.commit of this phase; false (uniform across the CTA) on timeout, after a
// second bounded wait so the tensor core is done with shared memory and TMEM before the caller exits.
__device__ __forceinline__ bool tile_wait(uint32_t bar, uint32_t phase) {
  const bool done = mbar_wait(bar, phase, g_mma_wait_polls);
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (__syncthreads_and(done)) return true;
  if (threadIdx.x == 0) atomicAdd(&g_mma_wait_timeouts, 1u);
  mbar_wait(bar, phase, kDrainPolls);
  asm volatile("tcgen05.fence::after_thread_sync;");
  return false;
}

__global__ void __launch_bounds__(kInferThreads, 1)
    k_mlp_infer(const uint8_t* __restrict__ blocks, int n, const __nv_bfloat16* __restrict__ W1,
                const __nv_bfloat16* __restrict__ W2, const __nv_bfloat16* __restrict__ W3,
                const float* __restrict__ b1, const float* __restrict__ b2, const float* __restrict__ b3,
                float* __restrict__ y, uint32_t* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* sW1 = sm + kSmW1;
  unsigned char* sW2 = sm + kSmW2;
  unsigned char* sW3 = sm + kSmW3;
  unsigned char* sH = sm + kSmH;  // features (first 12 KB) / hidden layer of the current tile
  float* sB1 = reinterpret_cast<float*>(sm + kSmB1);
  float* sB2 = reinterpret_cast<float*>(sm + kSmB2);
  float* sB3 = reinterpret_cast<float*>(sm + kSmB3);
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + kSmBar);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + kSmTmem);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  // weights (row-major bf16 [rows x K]) -> K-major core matrices, 16 bytes at a time
  for (int e = tid; e < kHid * (kHid / 8); e += kInferThreads) {
    const int r = e >> 5, kg = e & 31;
    *reinterpret_cast<uint4*>(sW2 + kseg(r, kg, kHid)) = __ldg(reinterpret_cast<const uint4*>(W2 + r * kHid + kg * 8));
  }
  for (int e = tid; e < kHid * (kIn / 8); e += kInferThreads) {
    const int r = e / (kIn / 8), kg = e % (kIn / 8);
    *reinterpret_cast<uint4*>(sW1 + kseg(r, kg, kIn)) = __ldg(reinterpret_cast<const uint4*>(W1 + r * kIn + kg * 8));
  }
  for (int e = tid; e < kOutPad * (kHid / 8); e += kInferThreads) {
    const int r = e >> 5, kg = e & 31;
    *reinterpret_cast<uint4*>(sW3 + kseg(r, kg, kHid)) = __ldg(reinterpret_cast<const uint4*>(W3 + r * kHid + kg * 8));
  }
  for (int e = tid; e < kHid; e += kInferThreads) { sB1[e] = b1[e]; sB2[e] = b2[e]; }
  if (tid < kOutPad) sB3[tid] = b3[tid];
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(smem_u32(tmem_slot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)));
  asm volatile("fence.proxy.async.shared::cta;");
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;
  const uint32_t bar = smem_u32(mbar);
  const uint32_t id256 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kHid >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
  const uint32_t id16 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kOutPad >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
  const uint32_t aH = smem_u32(sH), aW1 = smem_u32(sW1), aW2 = smem_u32(sW2), aW3 = smem_u32(sW3);
  const int quarter = warp & 3, half = warp >> 2;
  const int erow = quarter * 32 + lane;  // the tile row whose accumulators this thread reads
  uint32_t phase = 0;
  bool ok = true;
  const int ntiles = (n + BM - 1) / BM;
#pragma unroll 1
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long row0 = (long long)tile * BM;
    {  // features: thread (row, half) converts texels 8*half .. 8*half+7 (24 features, 3 K-groups)
      const int r = tid & (BM - 1), hf = tid >> 7;
      uint4 v0 = make_uint4(0, 0, 0, 0), v1 = v0;
      if (row0 + r < n) {
        const uint4* src = reinterpret_cast<const uint4*>(blocks + (row0 + r) * 64 + hf * 32);
        v0 = __ldg(src);
        v1 = __ldg(src + 1);
      }
      const uint32_t px[8] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w};
      float f[24];
#pragma unroll
      for (int t = 0; t < 8; t++)
#pragma unroll
        for (int c = 0; c < 3; c++) f[t * 3 + c] = (float)((px[t] >> (8 * c)) & 255u) * (1.0f / 255.0f);
#pragma unroll
      for (int g = 0; g < 3; g++)
        *reinterpret_cast<uint4*>(sH + kseg(r, hf * 3 + g, kIn)) =
            make_uint4(pack_bf16(f[g * 8], f[g * 8 + 1]), pack_bf16(f[g * 8 + 2], f[g * 8 + 3]),
                       pack_bf16(f[g * 8 + 4], f[g * 8 + 5]), pack_bf16(f[g * 8 + 6], f[g * 8 + 7]));
    }
    asm volatile("fence.proxy.async.shared::cta;");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (tid == 0) {  // layer 1: [128 x 48] x [48 x 256]
      asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
      for (int ks = 0; ks < kIn / 16; ks++)
        mma_bf16(tmem, make_desc(aH + ks * 256, 128, (kIn / 8) * 128), make_desc(aW1 + ks * 256, 128, (kIn / 8) * 128),
                 id256, ks > 0);
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar));
    }
    if (!(ok = tile_wait(bar, phase))) break;
    phase ^= 1;
    hidden_epilogue(tmem, quarter, erow, half * 128, sB1, sH);
    asm volatile("fence.proxy.async.shared::cta;");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (tid == 0) {  // layer 2: [128 x 256] x [256 x 256]
      asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
      for (int ks = 0; ks < kHid / 16; ks++)
        mma_bf16(tmem, make_desc(aH + ks * 256, 128, (kHid / 8) * 128), make_desc(aW2 + ks * 256, 128, (kHid / 8) * 128),
                 id256, ks > 0);
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar));
    }
    if (!(ok = tile_wait(bar, phase))) break;
    phase ^= 1;
    hidden_epilogue(tmem, quarter, erow, half * 128, sB2, sH);
    asm volatile("fence.proxy.async.shared::cta;");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (tid == 0) {  // layer 3: [128 x 256] x [256 x 16]
      asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
      for (int ks = 0; ks < kHid / 16; ks++)
        mma_bf16(tmem, make_desc(aH + ks * 256, 128, (kHid / 8) * 128), make_desc(aW3 + ks * 256, 128, (kHid / 8) * 128),
                 id16, ks > 0);
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar));
    }
    if (!(ok = tile_wait(bar, phase))) break;
    phase ^= 1;
    if (half == 0) {
      uint32_t r[16];
      tmem_ld16(tmem + ((uint32_t)(quarter * 32) << 16), r);
      if (row0 + erow < n) {
        float4* dst = reinterpret_cast<float4*>(y + (row0 + erow) * kOutPad);
#pragma unroll
        for (int q = 0; q < 4; q++)
          dst[q] = make_float4(__uint_as_float(r[4 * q]) + sB3[4 * q], __uint_as_float(r[4 * q + 1]) + sB3[4 * q + 1],
                               __uint_as_float(r[4 * q + 2]) + sB3[4 * q + 2],
                               __uint_as_float(r[4 * q + 3]) + sB3[4 * q + 3]);
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();  // TMEM columns and the feature tile are reused by the next tile
  }
  if (!ok && tid == 0) atomicExch(err, 1u);
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem));
}

// ------------------------------------------------------------------------------------------
// elementwise / reduction kernels

// Loss gradient dY and loss partial sums. Outputs 0..5 (endpoints): squared error, dY = 2 (y - t) / B.
// Output 6 (the error bound): squared error when tau <= 0; otherwise the quantile (pinball) loss
// bw * max(tau (t - y), (1 - tau) (y - t)), whose minimiser is the tau-quantile of the plain
// optimizer's error given the block, i.e. an upper bound that holds for a fraction tau of blocks.
__global__ void k_loss_grad(const float* __restrict__ y, const float* __restrict__ t, int B, float* __restrict__ dy,
                            float* __restrict__ loss, float tau, float bw) {
  float acc = 0.f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B * kOutPad; i += gridDim.x * blockDim.x) {
    const int s = i / kOutPad, c = i % kOutPad;
    float g = 0.f;
    if (c < 7) {
      const float d = y[(long long)s * kOutPad + c] - t[(long long)s * kOut + c];
      if (c == 6 && tau > 0.f) {
        acc += bw * (d > 0.f ? (1.f - tau) * d : -tau * d);
        g = bw * (d > 0.f ? (1.f - tau) : -tau) / (float)B;
      } else {
        acc += d * d;
        g = 2.f * d / (float)B;
      }
    }
    dy[i] = g;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xFFFFFFFFu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc / (float)B);
}

// column sums of a row-major [rows x cols] fp32 matrix -> out[cols]
__global__ void k_colsum(const float* __restrict__ x, int rows, int cols, float* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  float s = 0.f;
  for (int r = 0; r < rows; r++) s += x[(long long)r * cols + c];
  out[c] = s;
}

// AdamW on fp32 master weights; refreshes the bf16 copy. mask: parameters that stay zero.
__global__ void k_adamw(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                        __nv_bfloat16* __restrict__ wb, int n, float lr, float b1, float b2, float eps, float wd,
                        float bc1, float bc2, int rows_live, int row_len) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (i / row_len >= rows_live) { w[i] = 0.f; if (wb) wb[i] = __float2bfloat16(0.f); continue; }
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    float wi = w[i] * (1.f - lr * wd);
    wi -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16(wi);
  }
}

// Training targets from the plain optimizer's blocks: endpoints of the 4-colour solution in
// [0, 1] units, and log2(1 + error) / 16.
__global__ void k_make_targets(const uint8_t* __restrict__ blocks8, const uint64_t* __restrict__ err, int n,
                               float* __restrict__ t) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint8_t* b = blocks8 + (long long)i * 8;
    uint32_t lo = b[0] | (b[1] << 8), hi = b[2] | (b[3] << 8);
    if (lo <= hi) { const uint32_t x = lo; lo = hi; hi = x; }  // 3-colour blocks: order as 4-colour
    float* o = t + (long long)i * kOut;
    o[0] = (float)(lo >> 11) / 31.f; o[1] = (float)((lo >> 5) & 63) / 63.f; o[2] = (float)(lo & 31) / 31.f;
    o[3] = (float)(hi >> 11) / 31.f; o[4] = (float)((hi >> 5) & 63) / 63.f; o[5] = (float)(hi & 31) / 31.f;
    o[6] = log2f(1.f + (float)err[i]) / 16.f;
    o[7] = 0.f;
  }
}

// Learned encode, per block: quantise the predicted endpoints, choose selectors, refit the
// endpoints by least squares from those selectors (refine_solution level 0,
// crnlib/crn_dxt1.cpp:525-600), polish with a short greedy search of +-1 steps on the six
// endpoint components, check the 3-colour block on the same endpoints, and keep the block unless
// its error is above `threshold` x the network's predicted bound; those blocks are queued for the
// exact optimizer.
__device__ __forceinline__ int q565(float v, int hi) {
  int x = __float2int_rn(v * (float)hi);
  return x < 0 ? 0 : (x > hi ? hi : x);
}
__device__ __forceinline__ void expand565(uint32_t c, int* o) {
  const int r = c >> 11, g = (c >> 5) & 63, b = c & 31;
  o[0] = (r << 3) | (r >> 2); o[1] = (g << 2) | (g >> 4); o[2] = (b << 3) | (b >> 2);
}
// error of the 4-colour (three = false) or 3-colour palette of (lo, hi); selectors in 2-bit slots
__device__ uint32_t block_error(const uint32_t* px, uint32_t lo, uint32_t hi, bool perceptual, bool three,
                                uint32_t* sel_out) {
  int c[4][3];
  expand565(lo, c[0]);
  expand565(hi, c[1]);
  for (int k = 0; k < 3; k++) {
    if (three) {
      c[2][k] = (c[0][k] + c[1][k]) >> 1;
    } else {
      c[2][k] = (c[0][k] * 2 + c[1][k]) / 3;
      c[3][k] = (c[1][k] * 2 + c[0][k]) / 3;
    }
  }
  const int nk = three ? 3 : 4;
  const int wr = perceptual ? 8 : 1, wg = perceptual ? 25 : 1;
  uint32_t err = 0, sel = 0;
#pragma unroll 4
  for (int p = 0; p < 16; p++) {
    const int r = px[p] & 255, g = (px[p] >> 8) & 255, b = (px[p] >> 16) & 255;
    uint32_t best = 0xFFFFFFFFu;
    int bi = 0;
    for (int k = 0; k < nk; k++) {
      const int dr = r - c[k][0], dg = g - c[k][1], db = b - c[k][2];
      const uint32_t d = (uint32_t)(wr * dr * dr + wg * dg * dg + db * db);
      if (d < best) { best = d; bi = k; }
    }
    err += best;
    sel |= (uint32_t)bi << (2 * p);
  }
  *sel_out = sel;
  return err;
}

// y holds the proposals of blocks base .. base + n - 1; indices written to `fallback` are batch-wide
__global__ void k_learned_refit(const uint8_t* __restrict__ blocks, const float* __restrict__ y, uint32_t base, int n,
                                int perceptual, uint8_t* __restrict__ out, uint32_t* __restrict__ fallback,
                                uint32_t* __restrict__ nfall, float threshold) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const long long i = (long long)base + j;
    uint32_t px[16];
    const uint4* p4 = reinterpret_cast<const uint4*>(blocks + i * 64);
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const uint4 v = __ldg(p4 + q);
      px[4 * q] = v.x; px[4 * q + 1] = v.y; px[4 * q + 2] = v.z; px[4 * q + 3] = v.w;
    }
    const bool perc = perceptual != 0;
    const float* yi = y + (long long)j * kOutPad;
    int e[6] = {q565(yi[0], 31), q565(yi[1], 63), q565(yi[2], 31), q565(yi[3], 31), q565(yi[4], 63), q565(yi[5], 31)};
    auto pk = [](const int* v) { return (uint32_t)((v[0] << 11) | (v[1] << 5) | v[2]); };
    uint32_t sel;
    uint32_t err = block_error(px, pk(e), pk(e + 3), perc, false, &sel);
    // least-squares refit from the selectors (points at 1, 0, 2/3, 1/3 of the low endpoint)
    {
      float aa = 0.f, ab = 0.f, bb = 0.f, ax[3] = {0, 0, 0}, bx[3] = {0, 0, 0};
      const float wlow[4] = {1.f, 0.f, 2.f / 3.f, 1.f / 3.f};
      for (int p = 0; p < 16; p++) {
        const float a = wlow[(sel >> (2 * p)) & 3], b = 1.f - a;
        aa += a * a; ab += a * b; bb += b * b;
        const float x[3] = {(float)(px[p] & 255), (float)((px[p] >> 8) & 255), (float)((px[p] >> 16) & 255)};
        for (int k = 0; k < 3; k++) { ax[k] += a * x[k]; bx[k] += b * x[k]; }
      }
      const float det = aa * bb - ab * ab;
      if (fabsf(det) > 1e-6f) {
        const float inv = 1.f / det;
        const int lim[3] = {31, 63, 31};
        int f[6];
        for (int k = 0; k < 3; k++) {
          f[k] = q565((ax[k] * bb - bx[k] * ab) * inv / 255.f, lim[k]);
          f[3 + k] = q565((bx[k] * aa - ax[k] * ab) * inv / 255.f, lim[k]);
        }
        uint32_t nsel;
        const uint32_t nerr = block_error(px, pk(f), pk(f + 3), perc, false, &nsel);
        if (nerr < err) { err = nerr; sel = nsel; for (int k = 0; k < 6; k++) e[k] = f[k]; }
      }
    }
    // greedy polish: up to three rounds of the best single +-1 move over the six components
#pragma unroll 1
    for (int round = 0; round < 3; round++) {
      int best_k = -1, best_d = 0;
      uint32_t best_err = err, best_sel = sel;
#pragma unroll 1
      for (int k = 0; k < 6; k++) {
        const int lim = (k % 3) == 1 ? 63 : 31;
        for (int d = -1; d <= 1; d += 2) {
          const int v = e[k] + d;
          if (v < 0 || v > lim) continue;
          int f[6] = {e[0], e[1], e[2], e[3], e[4], e[5]};
          f[k] = v;
          uint32_t nsel;
          const uint32_t nerr = block_error(px, pk(f), pk(f + 3), perc, false, &nsel);
          if (nerr < best_err) { best_err = nerr; best_sel = nsel; best_k = k; best_d = d; }
        }
      }
      if (best_k < 0) break;
      e[best_k] += best_d;
      err = best_err;
      sel = best_sel;
    }
    uint32_t lo = pk(e), hi = pk(e + 3);
    // 4-colour blocks need low > high (swap and remap selectors 0<->1, 2<->3); equal endpoints
    // are nudged apart as the reference does (crnlib/crn_dxt1.cpp:1563-1583)
    if (lo < hi) {
      const uint32_t t = lo; lo = hi; hi = t;
      sel ^= 0x55555555u;
    } else if (lo == hi) {
      if ((lo & 31) != 31) lo++; else hi--;
      err = block_error(px, lo, hi, perc, false, &sel);
    }
    // the 3-colour block on the same endpoints (low <= high, mid-point palette)
    {
      uint32_t sel3;
      const uint32_t err3 = block_error(px, hi, lo, perc, true, &sel3);
      if (err3 < err) { err = err3; sel = sel3; const uint32_t t = lo; lo = hi; hi = t; }
    }
    const float bound = exp2f(yi[6] * 16.f) - 1.f;
    *reinterpret_cast<uint2*>(out + i * 8) = make_uint2(lo | (hi << 16), sel);
    if (!(threshold > 0.f) || (float)err > threshold * fmaxf(bound, 1.f)) {  // threshold <= 0: all exact
      const uint32_t at = atomicAdd(nfall, 1u);
      fallback[at] = (uint32_t)i;
    }
  }
}

__global__ void k_gather_idx(const uint8_t* __restrict__ blocks, const uint32_t* __restrict__ idx,
                             const uint32_t* __restrict__ count, uint8_t* __restrict__ out) {
  const uint32_t n = *count;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n * 4; t += gridDim.x * blockDim.x) {
    const uint32_t i = t >> 2, q = t & 3;
    reinterpret_cast<uint4*>(out)[t] = reinterpret_cast<const uint4*>(blocks + (long long)idx[i] * 64)[q];
  }
}
__global__ void k_scatter_idx(const uint8_t* __restrict__ enc, const uint32_t* __restrict__ idx,
                              const uint32_t* __restrict__ count, uint8_t* __restrict__ out) {
  const uint32_t n = *count;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    *reinterpret_cast<uint2*>(out + (long long)idx[i] * 8) = reinterpret_cast<const uint2*>(enc)[i];
}

// ------------------------------------------------------------------------------------------
// Host side

struct Param {
  int rows, cols, rows_live;
  DevBuf w, g, m, v, wb;  // fp32 master, grad, Adam moments, bf16 copy (weights only)
  size_t n() const { return (size_t)rows * cols; }
};

struct Net {
  uint32_t magic = 0x4D4C5030u;
  int device = -1;
  Param W1, b1, W2, b2, W3, b3;
  int step = 0;
  float bound_tau = 0.f, bound_weight = 1.f;  // loss of the error-bound output (see k_loss_grad)
  // activations / scratch sized for the largest batch seen
  int cap = 0;
  DevBuf pre1, h1, pre2, h2, y, dy, dpre2, dpre1, dh_b, dh_b1, targets, loss, errflag;
  DevBuf splitk;  // partial tiles of the split-K weight-gradient products
  // learned encode scratch
  DevBuf fb_idx, fb_count, fb_in, fb_out, chunk_y;
  std::vector<Param*> params() { return {&W1, &b1, &W2, &b2, &W3, &b3}; }
};

int alloc_param(Param& p, int rows, int cols, int rows_live, bool bf16) {
  p.rows = rows; p.cols = cols; p.rows_live = rows_live;
  cudaError_t e;
  if ((e = p.w.ensure(p.n() * 4)) != cudaSuccess) return cuda_check(e, "alloc weights");
  if ((e = p.g.ensure(p.n() * 4)) != cudaSuccess) return cuda_check(e, "alloc grads");
  if ((e = p.m.ensure(p.n() * 4)) != cudaSuccess) return cuda_check(e, "alloc adam m");
  if ((e = p.v.ensure(p.n() * 4)) != cudaSuccess) return cuda_check(e, "alloc adam v");
  cudaMemset(p.m.ptr, 0, p.n() * 4);
  cudaMemset(p.v.ptr, 0, p.n() * 4);
  cudaMemset(p.g.ptr, 0, p.n() * 4);
  if (bf16 && (e = p.wb.ensure(p.n() * 2)) != cudaSuccess) return cuda_check(e, "alloc bf16 weights");
  return CRNGPU_OK;
}

int upload(Param& p, const std::vector<float>& host) {
  cudaError_t e = cudaMemcpy(p.w.ptr, host.data(), p.n() * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_check(e, "upload weights");
  if (p.wb.ptr) {
    std::vector<__nv_bfloat16> hb(p.n());
    for (size_t i = 0; i < p.n(); i++) hb[i] = __float2bfloat16(host[i]);
    if ((e = cudaMemcpy(p.wb.ptr, hb.data(), p.n() * 2, cudaMemcpyHostToDevice)) != cudaSuccess)
      return cuda_check(e, "upload bf16 weights");
  }
  return CRNGPU_OK;
}

int ensure_batch(Net& net, int B) {
  if (B <= net.cap) return CRNGPU_OK;
  cudaError_t e;
  const size_t hid = (size_t)B * kHid;
  DevBuf* f32[] = {&net.pre1, &net.pre2, &net.dpre2, &net.dpre1};
  for (DevBuf* b : f32)
    if ((e = b->ensure(hid * 4)) != cudaSuccess) return cuda_check(e, "alloc activations");
  DevBuf* b16[] = {&net.h1, &net.h2, &net.dh_b, &net.dh_b1};
  for (DevBuf* b : b16)
    if ((e = b->ensure(hid * 2)) != cudaSuccess) return cuda_check(e, "alloc activations");
  if ((e = net.y.ensure((size_t)B * kOutPad * 4)) != cudaSuccess) return cuda_check(e, "alloc outputs");
  if ((e = net.dy.ensure((size_t)B * kOutPad * 4)) != cudaSuccess) return cuda_check(e, "alloc output grads");
  if ((e = net.targets.ensure((size_t)B * kOut * 4)) != cudaSuccess) return cuda_check(e, "alloc targets");
  if ((e = net.loss.ensure(16)) != cudaSuccess) return cuda_check(e, "alloc loss");
  if ((e = net.errflag.ensure(16)) != cudaSuccess) return cuda_check(e, "alloc flag");
  net.cap = B;
  return CRNGPU_OK;
}

Operand op_f32(const float* p, long long s_row, long long s_k) { return Operand{p, OP_F32, s_row, s_k, 0}; }
Operand op_bf16(const __nv_bfloat16* p, long long s_row, long long s_k) { return Operand{p, OP_BF16, s_row, s_k, 0}; }
Operand op_pixels(const uint8_t* p, bool sample_is_row) { return Operand{p, OP_PIXELS, 0, 0, sample_is_row ? 1 : 0}; }

// Each CTA allocates kTmemCols of the SM's 512 tensor-memory columns; an unused dynamic
// shared-memory reservation brings every CTA to about 57 KB so at most 4 CTAs share an SM and
// the allocations never wait on each other.
int gemm(GemmArgs g, cudaStream_t s, DevBuf* split_scratch = nullptr) {
  static bool attr_done[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  {
    std::lock_guard<std::mutex> lock(device_setup_mutex());
    if (dev >= 0 && dev < 64 && !attr_done[dev]) {  // > 48 KB per CTA in total needs the opt-in
      cudaError_t e = cudaFuncSetAttribute(k_gemm_tc<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, 40 << 10);
      if (e == cudaSuccess) e = cudaFuncSetAttribute(k_gemm_tc<48>, cudaFuncAttributeMaxDynamicSharedMemorySize, 36 << 10);
      if (e == cudaSuccess) e = cudaFuncSetAttribute(k_gemm_tc<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, 24 << 10);
      if (e != cudaSuccess) return cuda_check(e, "set k_gemm_tc shared memory");
      attr_done[dev] = true;
    }
  }
  const unsigned gx = (g.M + BM - 1) / BM;
  const unsigned bn = g.N <= 16 ? 16u : g.N <= 48 ? 48u : 128u;
  const unsigned gy = (g.N + bn - 1) / bn;
  // Products with few output tiles and a long K (the weight gradients: K is the batch) split K so
  // that about 128 CTAs share the work; the slices are summed by k_splitk_sum in a fixed order.
  unsigned gz = 1;
  g.kslice = 0;
  g.part = nullptr;
  if (split_scratch && g.epi == EPI_STORE && g.C && !g.Cb && gx * gy < 32 && g.K >= 4 * BK) {
    gz = std::min<unsigned>(128 / (gx * gy), (unsigned)((g.K + BK - 1) / BK));
    const int slice = ((g.K + (int)gz - 1) / (int)gz + BK - 1) / BK * BK;
    gz = (unsigned)((g.K + slice - 1) / slice);
    cudaError_t e = split_scratch->ensure((size_t)gz * g.M * g.N * sizeof(float));
    if (e != cudaSuccess) return cuda_check(e, "alloc split-K scratch");
    g.kslice = slice;
    g.part = static_cast<float*>(split_scratch->ptr);
  }
  const dim3 grid(gx, gy, gz);
  if (bn == 16) k_gemm_tc<16><<<grid, 128, 40 << 10, s>>>(g);
  else if (bn == 48) k_gemm_tc<48><<<grid, 128, 36 << 10, s>>>(g);
  else k_gemm_tc<128><<<grid, 128, 24 << 10, s>>>(g);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_check(e, "launch k_gemm_tc");
  if (g.part) {
    k_splitk_sum<<<(g.M * g.N + 255) / 256, 256, 0, s>>>(g.part, (int)gz, g.M, g.N, g.C, g.ldc, g.bias);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_check(e, "launch k_splitk_sum");
  }
  return CRNGPU_OK;
}

GemmArgs args(Operand a, Operand b, int M, int N, int K, int epi, float* C, __nv_bfloat16* Cb, const float* pre,
              const float* bias, int ldc, Net& net) {
  GemmArgs g;
  g.a = a; g.b = b; g.M = M; g.N = N; g.K = K; g.epi = epi; g.C = C; g.Cb = Cb; g.pre = pre; g.bias = bias; g.ldc = ldc;
  g.err = static_cast<uint32_t*>(net.errflag.ptr);
  g.kslice = 0;
  g.part = nullptr;
  return g;
}

// forward over B samples whose pixels are `blocks` (device); y -> net.y [B x 16]
int forward(Net& net, const uint8_t* blocks, int B, cudaStream_t s) {
  int rc;
  float* pre1 = static_cast<float*>(net.pre1.ptr);
  float* pre2 = static_cast<float*>(net.pre2.ptr);
  __nv_bfloat16* h1 = static_cast<__nv_bfloat16*>(net.h1.ptr);
  __nv_bfloat16* h2 = static_cast<__nv_bfloat16*>(net.h2.ptr);
  // L1: pre1 = X W1^T + b1, h1 = gelu(pre1)
  if ((rc = gemm(args(op_pixels(blocks, true), op_bf16(static_cast<__nv_bfloat16*>(net.W1.wb.ptr), kIn, 1), B, kHid,
                      kIn, EPI_BIAS_GELU, pre1, h1, nullptr, static_cast<float*>(net.b1.w.ptr), kHid, net),
                 s)) != CRNGPU_OK)
    return rc;
  if ((rc = gemm(args(op_bf16(h1, kHid, 1), op_bf16(static_cast<__nv_bfloat16*>(net.W2.wb.ptr), kHid, 1), B, kHid,
                      kHid, EPI_BIAS_GELU, pre2, h2, nullptr, static_cast<float*>(net.b2.w.ptr), kHid, net),
                 s)) != CRNGPU_OK)
    return rc;
  return gemm(args(op_bf16(h2, kHid, 1), op_bf16(static_cast<__nv_bfloat16*>(net.W3.wb.ptr), kHid, 1), B, kOutPad, kHid,
                   EPI_STORE, static_cast<float*>(net.y.ptr), nullptr, nullptr, static_cast<float*>(net.b3.w.ptr),
                   kOutPad, net),
              s);
}

// inference over n blocks (device) -> y [n x 16] with the fused kernel, one persistent CTA per SM
int infer(Net& net, const uint8_t* blocks, uint32_t n, float* y, cudaStream_t s) {
  static bool attr_done[64] = {};
  static int sms[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_check(e, "cudaGetDevice");
  if (dev < 0 || dev >= 64) { set_error("device index out of range"); return CRNGPU_E_DEVICE; }
  {
    std::lock_guard<std::mutex> lock(device_setup_mutex());
    if (!attr_done[dev]) {
      e = cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInferSmem);
      if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess) return cuda_check(e, "set up k_mlp_infer");
      attr_done[dev] = true;
    }
  }
  if ((e = net.errflag.ensure(16)) != cudaSuccess) return cuda_check(e, "alloc flag");
  if (!n) return CRNGPU_OK;
  const uint32_t tiles = (n + BM - 1) / BM;
  const uint32_t grid = tiles < (uint32_t)sms[dev] ? tiles : (uint32_t)sms[dev];
  k_mlp_infer<<<grid, kInferThreads, kInferSmem, s>>>(
      blocks, (int)n, static_cast<__nv_bfloat16*>(net.W1.wb.ptr), static_cast<__nv_bfloat16*>(net.W2.wb.ptr),
      static_cast<__nv_bfloat16*>(net.W3.wb.ptr), static_cast<float*>(net.b1.w.ptr), static_cast<float*>(net.b2.w.ptr),
      static_cast<float*>(net.b3.w.ptr), y, static_cast<uint32_t*>(net.errflag.ptr));
  return cuda_check(cudaGetLastError(), "launch k_mlp_infer");
}

// gradients of the mean squared error for targets in net.targets; loss -> net.loss
int backward(Net& net, const uint8_t* blocks, int B, cudaStream_t s) {
  int rc;
  float* dy = static_cast<float*>(net.dy.ptr);
  float* dpre2 = static_cast<float*>(net.dpre2.ptr);
  float* dpre1 = static_cast<float*>(net.dpre1.ptr);
  __nv_bfloat16* dhb = static_cast<__nv_bfloat16*>(net.dh_b.ptr);    // bf16 dpre2
  __nv_bfloat16* dhb1 = static_cast<__nv_bfloat16*>(net.dh_b1.ptr);  // bf16 dpre1 (own buffer: dhb is read meanwhile)
  cudaMemsetAsync(net.loss.ptr, 0, 4, s);
  k_loss_grad<<<256, 256, 0, s>>>(static_cast<float*>(net.y.ptr), static_cast<float*>(net.targets.ptr), B, dy,
                                  static_cast<float*>(net.loss.ptr), net.bound_tau, net.bound_weight);
  // dW3 [16 x 256] = dY^T H2 ; db3 = colsum(dY)
  if ((rc = gemm(args(op_f32(dy, 1, kOutPad), op_bf16(static_cast<__nv_bfloat16*>(net.h2.ptr), 1, kHid), kOutPad, kHid,
                      B, EPI_STORE, static_cast<float*>(net.W3.g.ptr), nullptr, nullptr, nullptr, kHid, net),
                 s, &net.splitk)) != CRNGPU_OK)
    return rc;
  k_colsum<<<1, kOutPad, 0, s>>>(dy, B, kOutPad, static_cast<float*>(net.b3.g.ptr));
  // dpre2 = (dY W3) * gelu'(pre2)
  if ((rc = gemm(args(op_f32(dy, kOutPad, 1), op_f32(static_cast<float*>(net.W3.w.ptr), 1, kHid), B, kHid, kOutPad,
                      EPI_GELU_GRAD, dpre2, dhb, static_cast<float*>(net.pre2.ptr), nullptr, kHid, net),
                 s)) != CRNGPU_OK)
    return rc;
  // dW2 [256 x 256] = dpre2^T H1 ; db2
  if ((rc = gemm(args(op_bf16(dhb, 1, kHid), op_bf16(static_cast<__nv_bfloat16*>(net.h1.ptr), 1, kHid), kHid, kHid, B,
                      EPI_STORE, static_cast<float*>(net.W2.g.ptr), nullptr, nullptr, nullptr, kHid, net),
                 s, &net.splitk)) != CRNGPU_OK)
    return rc;
  k_colsum<<<(kHid + 127) / 128, 128, 0, s>>>(dpre2, B, kHid, static_cast<float*>(net.b2.g.ptr));
  // dpre1 = (dpre2 W2) * gelu'(pre1)
  if ((rc = gemm(args(op_bf16(dhb, kHid, 1), op_f32(static_cast<float*>(net.W2.w.ptr), 1, kHid), B, kHid, kHid,
                      EPI_GELU_GRAD, dpre1, dhb1, static_cast<float*>(net.pre1.ptr), nullptr, kHid, net),
                 s)) != CRNGPU_OK)
    return rc;
  // dW1 [256 x 48] = dpre1^T X ; db1
  if ((rc = gemm(args(op_bf16(dhb1, 1, kHid), op_pixels(blocks, false), kHid, kIn, B, EPI_STORE,
                      static_cast<float*>(net.W1.g.ptr), nullptr, nullptr, nullptr, kIn, net),
                 s, &net.splitk)) != CRNGPU_OK)
    return rc;
  k_colsum<<<(kHid + 127) / 128, 128, 0, s>>>(dpre1, B, kHid, static_cast<float*>(net.b1.g.ptr));
  return cuda_check(cudaGetLastError(), "backward kernels");
}

int check_flag(Net& net, cudaStream_t s) {
  uint32_t f = 0;
  cudaError_t e = cudaMemcpyAsync(&f, net.errflag.ptr, 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_check(e, "read mma status");
  if (f) { set_error("tensor-core wait timed out"); return CRNGPU_E_DEVICE; }
  return CRNGPU_OK;
}

}  // namespace mlp
// Test hook for the tcgen05 commit waits: polls per first wait (drains are not affected).
int set_mma_wait_polls(uint32_t polls) {
  return cuda_check(cudaMemcpyToSymbol(mlp::g_mma_wait_polls, &polls, sizeof(polls)), "set mma wait polls");
}

// Number of first waits that ran out since the last reset.
int mma_wait_counter(uint32_t* out, bool reset) {
  cudaError_t e = cudaMemcpyFromSymbol(out, mlp::g_mma_wait_timeouts, sizeof(uint32_t));
  if (e == cudaSuccess && reset) {
    const uint32_t z = 0;
    e = cudaMemcpyToSymbol(mlp::g_mma_wait_timeouts, &z, sizeof(z));
  }
  return cuda_check(e, "read mma wait counter");
}

}  // namespace crngpu

using namespace crngpu;
using namespace crngpu::mlp;

extern "C" void* crngpu_mlp_create(uint64_t seed) try {
  clear_error();
  Net* net = new Net();
  cudaGetDevice(&net->device);
  std::mt19937_64 rng(seed);
  auto init = [&](Param& p, int rows, int cols, int rows_live, bool is_bias, int fan_in) {
    if (alloc_param(p, rows, cols, rows_live, !is_bias) != CRNGPU_OK) return false;
    std::vector<float> h(p.n(), 0.f);
    if (!is_bias) {
      const float bound = std::sqrt(6.0f / (float)fan_in) * 0.5f;
      std::uniform_real_distribution<float> u(-bound, bound);
      for (int r = 0; r < rows_live; r++)
        for (int c = 0; c < cols; c++) h[(size_t)r * cols + c] = u(rng);
    }
    return upload(p, h) == CRNGPU_OK;
  };
  if (!init(net->W1, kHid, kIn, kHid, false, kIn) || !init(net->b1, 1, kHid, 1, true, 1) ||
      !init(net->W2, kHid, kHid, kHid, false, kHid) || !init(net->b2, 1, kHid, 1, true, 1) ||
      !init(net->W3, kOutPad, kHid, 7, false, kHid) || !init(net->b3, 1, kOutPad, 1, true, 1)) {
    delete net;
    return nullptr;
  }
  cudaDeviceSynchronize();
  return net;
} catch (...) {
  crngpu::exception_status();
  return nullptr;
}

extern "C" int crngpu_mlp_destroy(void* h) try {
  Net* net = static_cast<Net*>(h);
  if (!net || net->magic != 0x4D4C5030u) return CRNGPU_E_PARAM;
  net->magic = 0;
  delete net;
  return CRNGPU_OK;
} catch (...) {
  return crngpu::exception_status();
}

// Parameter access for checkpoints and gradient checks. which: 0 W1, 1 b1, 2 W2, 3 b2, 4 W3, 5 b3;
// what: 0 weights, 1 gradients. count = number of floats in the buffer.
extern "C" int crngpu_mlp_param(void* h, int which, int what, float* host, uint32_t count, int write) try {
  Net* net = static_cast<Net*>(h);
  if (!net || net->magic != 0x4D4C5030u || which < 0 || which > 5 || !host) return CRNGPU_E_PARAM;
  Param* p = net->params()[which];
  if (count != p->n()) { set_error("size mismatch"); return CRNGPU_E_PARAM; }
  void* dev = what ? p->g.ptr : p->w.ptr;
  if (write) {
    std::vector<float> v(host, host + count);
    if (what == 0) return upload(*p, v);
    return cuda_check(cudaMemcpy(dev, host, count * 4, cudaMemcpyHostToDevice), "write param");
  }
  return cuda_check(cudaMemcpy(host, dev, count * 4, cudaMemcpyDeviceToHost), "read param");
} catch (...) {
  return crngpu::exception_status();
}

// Loss of the error-bound output: tau <= 0 squared error (weight ignored); 0 < tau < 1 the
// tau-quantile (pinball) loss scaled by `weight`.
extern "C" int crngpu_mlp_set_bound_loss(void* h, float tau, float weight) try {
  Net* net = static_cast<Net*>(h);
  if (!net || net->magic != 0x4D4C5030u || !(tau < 1.f) || !(weight > 0.f)) return CRNGPU_E_PARAM;
  net->bound_tau = tau > 0.f ? tau : 0.f;
  net->bound_weight = weight;
  return CRNGPU_OK;
} catch (...) {
  return crngpu::exception_status();
}

// Forward pass over n blocks (device RGBA8, n x 64) -> y (device, n x 16 fp32).
extern "C" int crngpu_mlp_forward(void* h, const uint8_t* d_blocks, uint32_t n, float* d_y, void* stream) try {
  clear_error();
  Net* net = static_cast<Net*>(h);
  if (!net || net->magic != 0x4D4C5030u || !d_blocks || !d_y) return CRNGPU_E_PARAM;
  if (n > (1u << 28)) { set_error("crngpu_mlp_forward: at most 2^28 blocks per call"); return CRNGPU_E_PARAM; }
  cudaStream_t s = as_stream(stream);
  cudaError_t e = net->errflag.ensure(16);
  if (e != cudaSuccess) return cuda_check(e, "alloc flag");
  cudaMemsetAsync(net->errflag.ptr, 0, 4, s);
  int rc = infer(*net, d_blocks, n, d_y, s);
  if (rc != CRNGPU_OK) return rc;
  return check_flag(*net, s);
} catch (...) {
  return crngpu::exception_status();
}

// Gradients of the loss for n blocks and targets (device, n x 8 fp32) into the gradient buffers;
// *loss (host) receives the loss. Does not update the weights.
extern "C" int crngpu_mlp_gradients(void* h, const uint8_t* d_blocks, const float* d_targets, uint32_t n, float* loss,
                                    void* stream) try {
  clear_error();
  Net* net = static_cast<Net*>(h);
  if (!net || net->magic != 0x4D4C5030u || !d_blocks || !d_targets || !n) return CRNGPU_E_PARAM;
  cudaStream_t s = as_stream(stream);
  int rc = ensure_batch(*net, (int)n);
  if (rc != CRNGPU_OK) return rc;
  cudaMemsetAsync(net->errflag.ptr, 0, 4, s);
  cudaMemcpyAsync(net->targets.ptr, d_targets, (size_t)n * kOut * 4, cudaMemcpyDeviceToDevice, s);
  if ((rc = forward(*net, d_blocks, (int)n, s)) != CRNGPU_OK) return rc;
  if ((rc = backward(*net, d_blocks, (int)n, s)) != CRNGPU_OK) return rc;
  if (loss) cudaMemcpyAsync(loss, net->loss.ptr, 4, cudaMemcpyDeviceToHost, s);
  return check_flag(*net, s);
} catch (...) {
  return crngpu::exception_status();
}

// One AdamW step (betas 0.9/0.999, eps 1e-8) on a batch: forward, backward, update.
extern "C" int crngpu_mlp_train_step(void* h, const uint8_t* d_blocks, const float* d_targets, uint32_t n, float lr,
                                     float weight_decay, float* loss, void* stream) try {
  int rc = crngpu_mlp_gradients(h, d_blocks, d_targets, n, loss, stream);
  if (rc != CRNGPU_OK) return rc;
  Net* net = static_cast<Net*>(h);
  cudaStream_t s = as_stream(stream);
  net->step++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float bc1 = 1.f - std::pow(b1, (float)net->step), bc2 = 1.f - std::pow(b2, (float)net->step);
  for (Param* p : net->params()) {
    const bool is_bias = p->rows == 1;
    k_adamw<<<64, 256, 0, s>>>(static_cast<float*>(p->w.ptr), static_cast<float*>(p->g.ptr),
                               static_cast<float*>(p->m.ptr), static_cast<float*>(p->v.ptr),
                               static_cast<__nv_bfloat16*>(p->wb.ptr), (int)p->n(), lr, b1, b2, 1e-8f,
                               is_bias ? 0.f : weight_decay, bc1, bc2, is_bias ? 1 : p->rows_live, p->cols);
  }
  return cuda_check(cudaGetLastError(), "launch k_adamw");
} catch (...) {
  return crngpu::exception_status();
}

// Training targets from plain-optimizer output (device): blocks8 (n x 8) + errors (n) -> n x 8.
extern "C" int crngpu_mlp_make_targets(const uint8_t* d_blocks8, const uint64_t* d_err, uint32_t n, float* d_targets,
                                       void* stream) try {
  if (!d_blocks8 || !d_err || !d_targets) return CRNGPU_E_PARAM;
  k_make_targets<<<(n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096, 256, 0, as_stream(stream)>>>(d_blocks8, d_err,
                                                                                                  (int)n, d_targets);
  return cuda_check(cudaGetLastError(), "launch k_make_targets");
} catch (...) {
  return crngpu::exception_status();
}

// Learned DXT1 encode of n blocks (device RGBA8 in, device dxt1 out): MLP proposal, one
// selector refit, and the exact optimizer for blocks whose error exceeds threshold x the
// predicted bound. *fallbacks (host, optional) receives how many blocks fell back.
extern "C" int crngpu_dxt1_learned_ex(void* h, const uint8_t* d_blocks, uint32_t n, int perceptual, float threshold,
                                      uint32_t fallback_quality, uint8_t* d_out, uint32_t* fallbacks, void* stream) try {
  clear_error();
  Net* net = static_cast<Net*>(h);
  if (!net || net->magic != 0x4D4C5030u || !d_blocks || !d_out) return CRNGPU_E_PARAM;
  if (fallback_quality > kDxtQualityUber) { set_error("crngpu_dxt1_learned: bad fallback quality"); return CRNGPU_E_PARAM; }
  if (!n) return CRNGPU_OK;
  if (n > (1u << 28)) { set_error("crngpu_dxt1_learned: at most 2^28 blocks per call"); return CRNGPU_E_PARAM; }
  cudaStream_t s = as_stream(stream);
  const uint32_t chunk = 1u << 20;
  int rc;
  cudaError_t e;
  if ((e = net->errflag.ensure(16)) != cudaSuccess) return cuda_check(e, "alloc flag");
  if ((e = net->chunk_y.ensure((size_t)(n < chunk ? n : chunk) * kOutPad * 4)) != cudaSuccess)
    return cuda_check(e, "alloc proposals");
  if ((e = net->fb_idx.ensure((size_t)n * 4)) != cudaSuccess) return cuda_check(e, "alloc fallback list");
  if ((e = net->fb_count.ensure(16)) != cudaSuccess) return cuda_check(e, "alloc fallback count");
  uint32_t* idx = static_cast<uint32_t*>(net->fb_idx.ptr);
  uint32_t* cnt_d = static_cast<uint32_t*>(net->fb_count.ptr);
  cudaMemsetAsync(cnt_d, 0, 4, s);
  cudaMemsetAsync(net->errflag.ptr, 0, 4, s);
  if (fallbacks) *fallbacks = 0;
  // proposals for every block (chunked to bound the activation buffers); blocks above the bound
  // are appended to one list of indices into the whole batch
  for (uint32_t c0 = 0; c0 < n; c0 += chunk) {
    const uint32_t cn = n - c0 < chunk ? n - c0 : chunk;
    if ((rc = infer(*net, d_blocks + (size_t)c0 * 64, cn, static_cast<float*>(net->chunk_y.ptr), s)) != CRNGPU_OK)
      return rc;
    k_learned_refit<<<(cn + 127) / 128, 128, 0, s>>>(d_blocks, static_cast<float*>(net->chunk_y.ptr), c0, (int)cn,
                                                      perceptual, d_out, idx, cnt_d, threshold);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(e, "launch k_learned_refit");
  }
  // blocks above the bound: the exact optimizer on a compacted copy, scattered back. The count
  // stays on the device: the gather, both encoder kernels and the scatter read it there, so the
  // call never waits for the host between the proposals and the fallback.
  if ((e = net->fb_in.ensure((size_t)n * 64)) != cudaSuccess) return cuda_check(e, "alloc fallback blocks");
  if ((e = net->fb_out.ensure((size_t)n * 8)) != cudaSuccess) return cuda_check(e, "alloc fallback out");
  const uint32_t sweep = (uint32_t)std::min<uint64_t>(((uint64_t)n * 4 + 255) / 256, 8192);
  k_gather_idx<<<sweep, 256, 0, s>>>(d_blocks, idx, cnt_d, static_cast<uint8_t*>(net->fb_in.ptr));
  if ((rc = launch_dxt1_count(static_cast<uint8_t*>(net->fb_in.ptr), n, cnt_d,
                              dxt1_options(perceptual != 0, true, fallback_quality, false, false, 128),
                              static_cast<uint8_t*>(net->fb_out.ptr), 8, s)) != CRNGPU_OK)
    return rc;
  k_scatter_idx<<<(sweep + 3) / 4, 256, 0, s>>>(static_cast<uint8_t*>(net->fb_out.ptr), idx, cnt_d, d_out);
  uint32_t cnt = 0;
  if (fallbacks && (e = cudaMemcpyAsync(&cnt, cnt_d, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
    return cuda_check(e, "read fallback count");
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(e, "learned encode kernels");
  rc = check_flag(*net, s);  // synchronises the stream
  if (rc != CRNGPU_OK) return rc;
  if (fallbacks) {
    if (cnt > n) { set_error("crngpu_dxt1_learned: fallback count out of range"); return CRNGPU_E_DEVICE; }
    *fallbacks = cnt;
  }
  return CRNGPU_OK;
} catch (...) {
  return crngpu::exception_status();
}

extern "C" int crngpu_dxt1_learned(void* h, const uint8_t* d_blocks, uint32_t n, int perceptual, float threshold,
                                   uint8_t* d_out, uint32_t* fallbacks, void* stream) try {
  return crngpu_dxt1_learned_ex(h, d_blocks, n, perceptual, threshold, kDxtQualityUber, d_out, fallbacks, stream);
} catch (...) {
  return crngpu::exception_status();
}

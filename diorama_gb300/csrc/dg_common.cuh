// Shared by every translation unit of libdiorama_gb300: the data layouts of the
// reference's GPU structs, the context/buffer objects behind the C ABI, error
// plumbing, and the device math the forward and backward passes share.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <cstring>
#include <deque>
#include <string>
#include <vector>

#include "../../include/diorama_gb300.h"

namespace dg {

// ---------------------------------------------------------------- layouts
// struct Gaussian (src/shaders/common.wgsl:11-17, src/gaussians.ts:38-46): position
// xyz, opacity, scale xyz, pad, rotation (w,x,y,z), color rgb, pad.
constexpr uint32_t FLOATS_PER_GAUSSIAN = 16;
// struct Splat2D (src/shaders/common.wgsl:20-26): mean xy, depth, radius, conic
// (a,b,c), pad, color rgb, opacity. The reference leaves the pad unwritten; this
// build's preprocess stores the splat's blend cutoff there (blend_cutoff, 0 when
// culled), so the blend kernels read it instead of taking a log per tile.
constexpr uint32_t SPLAT_CUTOFF_SLOT = 7;
constexpr uint32_t FLOATS_PER_SPLAT = 12;
// Spherical-harmonic coefficients 1..15, rgb each, coefficient-major (src/gaussians.ts:34-36).
constexpr uint32_t SH_REST_FLOATS = 45;
// Adam moment slots per Gaussian, one vec2 each (src/trainer.ts:17).
constexpr uint32_t MOMENT_SLOTS = FLOATS_PER_GAUSSIAN + SH_REST_FLOATS;
// The trainer keeps a set's moments in two planes (the same 61 vec2 slots per
// Gaussian as the reference, MOMENT_SLOTS * 8 bytes per Gaussian in all): first
// the 16 parameter slots of every Gaussian (128-byte records), then the 45 SH
// slots of every Gaussian. A run of consecutive Gaussians then has its SH
// moments in one contiguous run indexed like its SH coefficients (g * 45 + k),
// and its parameter moments in 16-byte-aligned records, so Adam streams both with
// 16-byte accesses and no per-slot index arithmetic. The reference interleaves
// the 61 slots per Gaussian (488-byte records, 16-byte aligned only for every
// other Gaussian); the checkpoint files keep that per-Gaussian order.
__host__ __device__ __forceinline__ size_t param_moment_at(uint32_t g, uint32_t k) {
  return (size_t)g * FLOATS_PER_GAUSSIAN + k;
}
__host__ __device__ __forceinline__ size_t sh_moment_at(uint32_t count, uint32_t g, uint32_t k) {
  return (size_t)count * FLOATS_PER_GAUSSIAN + (size_t)g * SH_REST_FLOATS + k;
}
// Gradients per splat from the blend's backward (src/shaders/rasterizeBackward.wgsl:124-126).
constexpr uint32_t SPLAT_GRADS = 9;
constexpr uint32_t TILE = 16;
// At most 2^16 tiles, as the sort looks at 16 bits of the tile index (src/tileRasterizer.ts:10).
constexpr uint32_t TILE_INDEX_BITS = 16;

// The Camera uniform (src/shaders/common.wgsl:4-8): 144 bytes.
struct Camera {
  float view[16];  // column-major
  float proj[16];
  float viewport[2];
  float pad[2];
};
static_assert(sizeof(Camera) == 144, "Camera is 144 bytes like the reference's uniform");

// Bits of the device error word that bounded waits set instead of hanging.
constexpr uint32_t DEVICE_ERROR_SCAN_WAIT = 1u << 0;
constexpr uint32_t DEVICE_ERROR_SORT_WAIT = 1u << 1;
constexpr uint32_t DEVICE_ERROR_COPY_WAIT = 1u << 2;  // a bulk copy's mbarrier
constexpr uint32_t DEVICE_ERROR_MMA_WAIT = 1u << 3;   // a tensor-core product's mbarrier
// Iteration cap of every spin on another block's status (about a second at worst).
constexpr uint32_t SPIN_LIMIT = 1u << 22;

// ---------------------------------------------------------------- errors
void set_error(const std::string& message);
dg_status fail(dg_status code, const std::string& message);
dg_status cuda_fail(cudaError_t err, const char* what);

#define DG_CUDA(call)                                             \
  do {                                                            \
    cudaError_t dg_err_ = (call);                                 \
    if (dg_err_ != cudaSuccess) return ::dg::cuda_fail(dg_err_, #call); \
  } while (0)

#define DG_TRY(call)                         \
  do {                                       \
    dg_status dg_st_ = (call);               \
    if (dg_st_ != DG_OK) return dg_st_;      \
  } while (0)

#define DG_REQUIRE(cond, msg)                                 \
  do {                                                        \
    if (!(cond)) return ::dg::fail(DG_ERROR_INVALID_ARGUMENT, msg); \
  } while (0)

inline uint32_t ceil_div(uint64_t a, uint64_t b) { return (uint32_t)((a + b - 1) / b); }

}  // namespace dg

// ---------------------------------------------------------------- objects

// A device allocation standing in for a GPUBuffer. Owned buffers are freed by
// dg_buffer_destroy; wrapped ones only forget the pointer.
struct dg_buffer {
  dg_context* ctx;
  void* ptr;
  uint64_t bytes;
  bool owned;
};

// The "device" and its "queue": one CUDA device and one stream, in order.
struct dg_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  uint32_t* device_error = nullptr;  // set by bounded waits
  int sm_count = 0;
  // Pinned staging ring for queue.writeBuffer: each write is copied here at call
  // time, so the caller's memory is free on return, as with WebGPU.
  char* staging = nullptr;
  size_t staging_bytes = 0;
  size_t staging_head = 0;
  struct Pending {
    size_t begin, end;
    cudaEvent_t done;
  };
  std::deque<Pending> pending;
  std::vector<cudaEvent_t> free_events;
  bool capturing = false;
  // Kernels launched through this context (graph replays add their kernel count).
  uint64_t launches = 0;
  // Per-kernel timing (dg_context_set_kernel_timing): an event pair around every
  // launch made outside graph capture, summed per kernel name on request.
  bool timing = false;
  struct Timed {
    const char* name;
    cudaEvent_t start, end;
  };
  std::vector<Timed> timed;
  std::vector<cudaEvent_t> timing_pool;
  cudaEvent_t pending_start = nullptr;
};

namespace dg {
// Kernel launch bookkeeping: counts the launch and, when kernel timing is on and
// no graph is being captured, brackets it with an event pair.
void timing_begin(dg_context* ctx);
void timing_end(dg_context* ctx, const char* name);
}  // namespace dg

// DG_LAUNCH(ctx, "name", kernel<<<grid, block, smem, stream>>>(args...));
#define DG_LAUNCH(ctx, name, ...)               \
  do {                                          \
    ::dg::timing_begin(ctx);                    \
    __VA_ARGS__;                                \
    (ctx)->launches++;                          \
    ::dg::timing_end(ctx, name);                \
    DG_CUDA(cudaGetLastError());                \
  } while (0)

namespace dg {
// Enqueue a host→device copy with writeBuffer semantics (the source is
// snapshotted now). Not allowed while a graph is being captured.
dg_status write_async(dg_context* ctx, void* dst, const void* src, size_t bytes);
dg_status alloc_buffer(dg_context* ctx, uint64_t bytes, dg_buffer** out);
void free_buffer(dg_buffer* b);
inline void* ptr_of(dg_buffer* b) { return b ? b->ptr : nullptr; }
template <typename T>
inline T* typed(dg_buffer* b) {
  return reinterpret_cast<T*>(b ? b->ptr : nullptr);
}
}  // namespace dg

// ---------------------------------------------------------------- device math
namespace dg {

// e^x by Cody-Waite reduction x = n ln2 + r (|r| <= ln2/2), e^r from its Taylor
// series to degree 7 by Horner's rule, and scaling by 2^n through the exponent
// bits, for -87 <= x <= 88 (the blend calls it only on powers between a splat's
// cutoff, above ln(1/255) - 1e-3, and 0). The blend's forward and backward both
// use it, so their alpha tests agree exactly; its error is about one ulp.
__host__ __device__ __forceinline__ float exp_blend_core(float x) {
  float n = rintf(x * 1.44269504088896341f);
  float r = fmaf(n, -0.693145751953125f, x);
  r = fmaf(n, -1.428606820309417232e-6f, r);
  float p = 1.98412698412698413e-4f;
  p = fmaf(p, r, 1.38888888888888889e-3f);
  p = fmaf(p, r, 8.33333333333333333e-3f);
  p = fmaf(p, r, 4.16666666666666667e-2f);
  p = fmaf(p, r, 1.66666666666666667e-1f);
  p = fmaf(p, r, 0.5f);
  p = fmaf(p, r, 1.0f);
  p = fmaf(p, r, 1.0f);
  int32_t e = (int32_t)n + 127;
#ifdef __CUDA_ARCH__
  float scale = __int_as_float(e << 23);
#else
  float scale;
  uint32_t bits = (uint32_t)e << 23;
  std::memcpy(&scale, &bits, 4);
#endif
  return p * scale;
}

// exp_blend_core over the whole float range: 0 below -87, infinity above 88.
__host__ __device__ __forceinline__ float exp_blend(float x) {
  if (x < -87.0f) return 0.0f;
  if (x > 88.0f) return INFINITY;
  return exp_blend_core(x);
}

__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }

#ifdef __CUDACC__  // device code below; host-only translation units skip it
// Two float32 values in one 64-bit register, for Blackwell's packed FP32
// instructions: each lane of add/mul/fma .rn.f32x2 rounds exactly as the scalar
// add/mul/fma .rn.f32 does (subnormals kept), so two independent sums advance in
// one instruction per step with the same results. Unlike the scalar forms, a
// packed multiply whose result feeds a packed add may be contracted by the
// assembler into one fused multiply-add: write f2_fma where a product is added.
struct F2 {
  unsigned long long v;
};
__device__ __forceinline__ F2 f2(float lo, float hi) {
  F2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ F2 f2_load(const float2* p) { return F2{*reinterpret_cast<const unsigned long long*>(p)}; }
__device__ __forceinline__ void f2_store(float2* p, F2 a) { *reinterpret_cast<unsigned long long*>(p) = a.v; }
__device__ __forceinline__ F2 f2_mul(F2 a, F2 b) {
  F2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
  F2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ F2 f2_fma(F2 a, F2 b, F2 c) {
  F2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
  return r;
}
__device__ __forceinline__ float f2_lo(F2 a) {
  float lo;
  asm("{\n\t.reg .b32 hi;\n\tmov.b64 {%0, hi}, %1;\n\t}" : "=f"(lo) : "l"(a.v));
  return lo;
}
__device__ __forceinline__ float f2_hi(F2 a) {
  float hi;
  asm("{\n\t.reg .b32 lo;\n\tmov.b64 {lo, %0}, %1;\n\t}" : "=f"(hi) : "l"(a.v));
  return hi;
}

// ---- mbarriers in shared memory (bulk copies and tensor-core commits complete on them).
__device__ __forceinline__ uint32_t smem_address(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t arrivals) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_address(bar)), "r"(arrivals) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(done)
      : "r"(smem_address(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
// L2 eviction priorities. A kernel that streams far more data than L2 holds but
// reads a small part of it twice marks the stream evict-first and the part it
// will read again evict-last, so the stream does not push that part out first.
__device__ __forceinline__ uint64_t l2_policy_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;\n" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t l2_policy_evict_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;\n" : "=l"(p));
  return p;
}

// Waits for phase `parity` of the barrier to complete, at most SPIN_LIMIT polls
// (each try_wait may itself suspend the thread for a while). Returns false if it
// gave up.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  for (uint32_t spin = 0; spin < SPIN_LIMIT; spin++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// exp_blend_core of two values at once: the polynomial's fused multiply-adds run
// as packed pairs, each lane the same fmaf as exp_blend_core's, so both results
// are exp_blend_core's bit for bit.
__device__ __forceinline__ void exp_blend_core2(float x0, float x1, float& e0, float& e1) {
  const float n0 = rintf(x0 * 1.44269504088896341f), n1 = rintf(x1 * 1.44269504088896341f);
  const F2 n = f2(n0, n1);
  F2 r = f2_fma(n, f2(-0.693145751953125f, -0.693145751953125f), f2(x0, x1));
  r = f2_fma(n, f2(-1.428606820309417232e-6f, -1.428606820309417232e-6f), r);
  F2 p = f2(1.98412698412698413e-4f, 1.98412698412698413e-4f);
  p = f2_fma(p, r, f2(1.38888888888888889e-3f, 1.38888888888888889e-3f));
  p = f2_fma(p, r, f2(8.33333333333333333e-3f, 8.33333333333333333e-3f));
  p = f2_fma(p, r, f2(4.16666666666666667e-2f, 4.16666666666666667e-2f));
  p = f2_fma(p, r, f2(1.66666666666666667e-1f, 1.66666666666666667e-1f));
  p = f2_fma(p, r, f2(0.5f, 0.5f));
  p = f2_fma(p, r, f2(1.0f, 1.0f));
  p = f2_fma(p, r, f2(1.0f, 1.0f));
  e0 = f2_lo(p) * __int_as_float(((int32_t)n0 + 127) << 23);
  e1 = f2_hi(p) * __int_as_float(((int32_t)n1 + 127) << 23);
}
#endif  // __CUDACC__

constexpr float SH_C0 = 0.28209479177387814f;
constexpr float SH_C1 = 0.4886025119029199f;

}  // namespace dg

// Device code of the renderer's forward and backward passes. This header is
// compiled into dg_render.cu with --fmad=false, so every product is rounded
// before it is added exactly as written; fused multiply-adds appear only where
// fmaf is spelled out. The CPU oracle (oracle/oracle.c) evaluates the same
// expressions in the same order, so forward splats and images agree bit for bit.
#pragma once
#include "dg_common.cuh"

namespace dg {

// The projection shared by preprocess and its backward: the view-space center
// and the 2D covariance (src/shaders/preprocess.wgsl:27-57). Matrices are held
// as columns m[col][row]; every sum runs from index 0 upwards.
struct Projection {
  float t[3], depth;
  float r[3][3], q[4], qlen;
  float m[3][3], cov3d[3][3];
  float focal[2], limit[2], tx, ty;
  float jw[3][2];
  float w[3][3];
  float a, b, c, det;
};

// The view-space z of a Gaussian's center, computed exactly as project() does.
__device__ __forceinline__ float view_z(const Camera& cam, const float* g) {
  float z = cam.view[0 * 4 + 2] * g[0];
  z = z + cam.view[1 * 4 + 2] * g[1];
  z = z + cam.view[2 * 4 + 2] * g[2];
  z = z + cam.view[3 * 4 + 2] * 1.0f;
  return z;
}

__device__ __forceinline__ void rotation_matrix(const float raw[4], float r[3][3], float q[4], float& len_out) {
  float dot = raw[0] * raw[0];
  dot = dot + raw[1] * raw[1];
  dot = dot + raw[2] * raw[2];
  dot = dot + raw[3] * raw[3];
  float len = sqrtf(dot);
  float qw = raw[0] / len, qx = raw[1] / len, qy = raw[2] / len, qz = raw[3] / len;
  r[0][0] = 1.0f - 2.0f * (qy * qy + qz * qz);
  r[0][1] = 2.0f * (qx * qy + qw * qz);
  r[0][2] = 2.0f * (qx * qz - qw * qy);
  r[1][0] = 2.0f * (qx * qy - qw * qz);
  r[1][1] = 1.0f - 2.0f * (qx * qx + qz * qz);
  r[1][2] = 2.0f * (qy * qz + qw * qx);
  r[2][0] = 2.0f * (qx * qz + qw * qy);
  r[2][1] = 2.0f * (qy * qz - qw * qx);
  r[2][2] = 1.0f - 2.0f * (qx * qx + qy * qy);
  q[0] = qw;
  q[1] = qx;
  q[2] = qy;
  q[3] = qz;
  len_out = len;
}

__device__ __forceinline__ void project(const Camera& cam, const float* g, Projection& p) {
  for (int row = 0; row < 3; row++) {
    float v = cam.view[0 * 4 + row] * g[0];
    v = v + cam.view[1 * 4 + row] * g[1];
    v = v + cam.view[2 * 4 + row] * g[2];
    v = v + cam.view[3 * 4 + row] * 1.0f;
    p.t[row] = v;
  }
  p.depth = -p.t[2];
  rotation_matrix(g + 8, p.r, p.q, p.qlen);
#pragma unroll
  for (int col = 0; col < 3; col++)
#pragma unroll
    for (int row = 0; row < 3; row++) p.m[col][row] = p.r[col][row] * g[4 + col];
#pragma unroll
  for (int col = 0; col < 3; col++)
#pragma unroll
    for (int row = 0; row < 3; row++) {
      float v = p.m[0][row] * p.m[0][col];
      v = v + p.m[1][row] * p.m[1][col];
      v = v + p.m[2][row] * p.m[2][col];
      p.cov3d[col][row] = v;
    }
  p.focal[0] = cam.proj[0] * cam.viewport[0] * 0.5f;
  p.focal[1] = cam.proj[5] * cam.viewport[1] * 0.5f;
  p.limit[0] = 1.3f * cam.viewport[0] * 0.5f / p.focal[0];
  p.limit[1] = 1.3f * cam.viewport[1] * 0.5f / p.focal[1];
  const float depth = p.depth;
  p.tx = clampf(p.t[0] / depth, -p.limit[0], p.limit[0]) * depth;
  p.ty = clampf(p.t[1] / depth, -p.limit[1], p.limit[1]) * depth;
  float j[3][2];
  j[0][0] = p.focal[0] / depth;
  j[0][1] = 0.0f;
  j[1][0] = 0.0f;
  j[1][1] = -p.focal[1] / depth;
  j[2][0] = p.focal[0] * p.tx / (depth * depth);
  j[2][1] = -p.focal[1] * p.ty / (depth * depth);
#pragma unroll
  for (int col = 0; col < 3; col++)
#pragma unroll
    for (int row = 0; row < 3; row++) p.w[col][row] = cam.view[col * 4 + row];
#pragma unroll
  for (int col = 0; col < 3; col++)
#pragma unroll
    for (int row = 0; row < 2; row++) {
      float v = j[0][row] * p.w[col][0];
      v = v + j[1][row] * p.w[col][1];
      v = v + j[2][row] * p.w[col][2];
      p.jw[col][row] = v;
    }
  float t1[3][2];
#pragma unroll
  for (int col = 0; col < 3; col++)
#pragma unroll
    for (int row = 0; row < 2; row++) {
      float v = p.jw[0][row] * p.cov3d[col][0];
      v = v + p.jw[1][row] * p.cov3d[col][1];
      v = v + p.jw[2][row] * p.cov3d[col][2];
      t1[col][row] = v;
    }
  float cov[2][2];
#pragma unroll
  for (int col = 0; col < 2; col++)
#pragma unroll
    for (int row = 0; row < 2; row++) {
      float v = t1[0][row] * p.jw[0][col];
      v = v + t1[1][row] * p.jw[1][col];
      v = v + t1[2][row] * p.jw[2][col];
      cov[col][row] = v;
    }
  p.a = cov[0][0] + 0.3f;
  p.b = cov[0][1];
  p.c = cov[1][1] + 0.3f;
  p.det = p.a * p.c - p.b * p.b;
}

__device__ __forceinline__ void camera_position(const Camera& cam, float out[3]) {
#pragma unroll
  for (int col = 0; col < 3; col++) {
    float v = cam.view[col * 4 + 0] * cam.view[12];
    v = v + cam.view[col * 4 + 1] * cam.view[13];
    v = v + cam.view[col * 4 + 2] * cam.view[14];
    out[col] = -v;
  }
}

__device__ __forceinline__ float normalize3(const float v[3], float out[3]) {
  float dot = v[0] * v[0];
  dot = dot + v[1] * v[1];
  dot = dot + v[2] * v[2];
  float len = sqrtf(dot);
  out[0] = v[0] / len;
  out[1] = v[1] / len;
  out[2] = v[2] / len;
  return len;
}

// src/shaders/gaussianMath.wgsl:30-44
__device__ __forceinline__ void sh_basis(const float d[3], float b[15]) {
  const float C2[5] = {1.0925484305920792f, -1.0925484305920792f, 0.31539156525252005f, -1.0925484305920792f,
                       0.5462742152789498f};
  const float C3[7] = {-0.5900435899266435f, 2.890611442640554f, -0.4570457994644658f, 0.3731763325901154f,
                       -0.4570457994644658f, 1.445305721320277f, -0.5900435899266435f};
  float x = d[0], y = d[1], z = d[2];
  float xx = x * x, yy = y * y, zz = z * z;
  b[0] = -SH_C1 * y;
  b[1] = SH_C1 * z;
  b[2] = -SH_C1 * x;
  b[3] = C2[0] * x * y;
  b[4] = C2[1] * y * z;
  b[5] = C2[2] * (2.0f * zz - xx - yy);
  b[6] = C2[3] * x * z;
  b[7] = C2[4] * (xx - yy);
  b[8] = C3[0] * y * (3.0f * xx - yy);
  b[9] = C3[1] * x * y * z;
  b[10] = C3[2] * y * (4.0f * zz - xx - yy);
  b[11] = C3[3] * z * (2.0f * zz - 3.0f * xx - 3.0f * yy);
  b[12] = C3[4] * x * (4.0f * zz - xx - yy);
  b[13] = C3[5] * z * (xx - yy);
  b[14] = C3[6] * x * (xx - 3.0f * yy);
}

// src/shaders/gaussianMath.wgsl:47-71, as g[k][axis].
__device__ __forceinline__ void sh_basis_gradient(const float d[3], float g[15][3]) {
  const float C2[5] = {1.0925484305920792f, -1.0925484305920792f, 0.31539156525252005f, -1.0925484305920792f,
                       0.5462742152789498f};
  const float C3[7] = {-0.5900435899266435f, 2.890611442640554f, -0.4570457994644658f, 0.3731763325901154f,
                       -0.4570457994644658f, 1.445305721320277f, -0.5900435899266435f};
  float x = d[0], y = d[1], z = d[2];
  float xx = x * x, yy = y * y, zz = z * z;
  g[0][0] = 0.0f; g[0][1] = -SH_C1; g[0][2] = 0.0f;
  g[1][0] = 0.0f; g[1][1] = 0.0f; g[1][2] = SH_C1;
  g[2][0] = -SH_C1; g[2][1] = 0.0f; g[2][2] = 0.0f;
  g[3][0] = C2[0] * y; g[3][1] = C2[0] * x; g[3][2] = C2[0] * 0.0f;
  g[4][0] = C2[1] * 0.0f; g[4][1] = C2[1] * z; g[4][2] = C2[1] * y;
  g[5][0] = C2[2] * (-2.0f * x); g[5][1] = C2[2] * (-2.0f * y); g[5][2] = C2[2] * (4.0f * z);
  g[6][0] = C2[3] * z; g[6][1] = C2[3] * 0.0f; g[6][2] = C2[3] * x;
  g[7][0] = C2[4] * (2.0f * x); g[7][1] = C2[4] * (-2.0f * y); g[7][2] = C2[4] * 0.0f;
  g[8][0] = C3[0] * (6.0f * x * y); g[8][1] = C3[0] * (3.0f * xx - 3.0f * yy); g[8][2] = C3[0] * 0.0f;
  g[9][0] = C3[1] * (y * z); g[9][1] = C3[1] * (x * z); g[9][2] = C3[1] * (x * y);
  g[10][0] = C3[2] * (-2.0f * x * y); g[10][1] = C3[2] * (4.0f * zz - xx - 3.0f * yy); g[10][2] = C3[2] * (8.0f * y * z);
  g[11][0] = C3[3] * (-6.0f * x * z); g[11][1] = C3[3] * (-6.0f * y * z);
  g[11][2] = C3[3] * (6.0f * zz - 3.0f * xx - 3.0f * yy);
  g[12][0] = C3[4] * (4.0f * zz - 3.0f * xx - yy); g[12][1] = C3[4] * (-2.0f * x * y); g[12][2] = C3[4] * (8.0f * x * z);
  g[13][0] = C3[5] * (2.0f * x * z); g[13][1] = C3[5] * (-2.0f * y * z); g[13][2] = C3[5] * (xx - yy);
  g[14][0] = C3[6] * (3.0f * xx - 3.0f * yy); g[14][1] = C3[6] * (-6.0f * x * y); g[14][2] = C3[6] * 0.0f;
}

// ------------------------------------------------------------------ blending
// The exponent of a splat at a pixel, `power = -0.5 (a dx^2 + c dy^2) - b dx dy`
// (src/shaders/rasterize.wgsl:68), from A = -0.5 a and C = -0.5 c (exact
// scalings), evaluated as dx (A dx - b dy) + (C dy) dy: three products and two
// fused multiply-adds instead of five products and three sums (WGSL leaves
// contraction to the implementation; the oracle evaluates this same sequence).
// Written with round-to-nearest intrinsics, which the compiler neither fuses
// further nor splits, so the forward and backward passes compute identical powers
// whatever their --fmad setting.
__device__ __forceinline__ float blend_power(float A, float b, float C, float dx, float dy) {
  const float t = __fmaf_rn(A, dx, -__fmul_rn(b, dy));
  return __fmaf_rn(t, dx, __fmul_rn(__fmul_rn(C, dy), dy));
}

// A power below which alpha = opacity * exp(power) is certainly under 1/255, so
// the exp can be skipped with the same outcome: ln(1 / (255 opacity)), lowered by
// 1e-3 to cover the float error of exp_blend and of the product (~1e-7 relative).
__device__ __forceinline__ float blend_cutoff(float opacity) {
  return logf(1.0f / (255.0f * opacity)) - 1e-3f;
}

// Whether a splat can reach any pixel center of the rectangle
// [dxl, dxh] x [dyl, dyh] (offsets pixel - mean): the maximum of the concave
// quadratic q = A dx^2 - b dx dy + C dy^2 over the rectangle, compared with the
// cutoff. The maximum is at the mean if the rectangle holds it, else on an edge,
// where each 1D maximum is clamped to the edge. The margin covers the rounding
// of both this maximum and the per-pixel power (a few ulps of the terms' sizes),
// so a splat this rejects would have been skipped at every pixel anyway. The
// quadratics are fused multiply-adds (one rounding each, inside that margin).
__device__ __forceinline__ bool rect_reachable(float A, float b, float C, float kx, float ky, float cut, float dxl,
                                               float dxh, float dyl, float dyh) {
  if (dxl <= 0.0f && dxh >= 0.0f && dyl <= 0.0f && dyh >= 0.0f) return 0.0f >= cut;
  // (A dx - b dy) dx + C dy dy
  auto q = [&](float dx, float dy) {
    return __fmaf_rn(__fmaf_rn(A, dx, -__fmul_rn(b, dy)), dx, __fmul_rn(__fmul_rn(C, dy), dy));
  };
  const float y1 = fminf(fmaxf(ky * dxl, dyl), dyh), y2 = fminf(fmaxf(ky * dxh, dyl), dyh);
  const float x1 = fminf(fmaxf(kx * dyl, dxl), dxh), x2 = fminf(fmaxf(kx * dyh, dxl), dxh);
  const float qmax = fmaxf(fmaxf(q(dxl, y1), q(dxh, y2)), fmaxf(q(x1, dyl), q(x2, dyh)));
  const float mx = fmaxf(fabsf(dxl), fabsf(dxh)), my = fmaxf(fabsf(dyl), fabsf(dyh));
  const float terms = __fmaf_rn(__fmaf_rn(fabsf(A), mx, fabsf(b) * my), mx, fabsf(C) * my * my);
  return __fmaf_rn(1e-6f, terms, qmax) + 1e-6f >= cut;
}

// CTA sizes of the blend kernels. The forward's 4 warps blend a block of a long
// tile list together (3 computing alphas, 1 blending; 96 and 160 threads measured
// slower: 331 and 363 us against 323 at 1.1M Gaussians); otherwise every warp
// takes items of its own.
#ifndef DG_FWD_THREADS
#define DG_FWD_THREADS 128
#endif
constexpr uint32_t FWD_THREADS = DG_FWD_THREADS;  // 96 or 128 (measured 324 and 288 us at 1.1M)
constexpr uint32_t FWD_WARPS = FWD_THREADS / 32;
constexpr uint32_t PRODUCERS = FWD_WARPS - 1;  // cooperative blending: warps computing alphas for warp 0
constexpr uint32_t BWD_THREADS = 128;
constexpr uint32_t BWD_WARPS = BWD_THREADS / 32;
// The backward pass walks a tile's list in chunks of CHUNK entries, each starting
// from the state the forward pass saved at the chunk's end (a checkpoint per
// CHUNK entries). A multiple of the 32-entry window.
constexpr uint32_t CHUNK = 512;
// Tiles with more entries than this are blended by a whole CTA in the forward pass.
#ifndef DG_COOP_MIN
#define DG_COOP_MIN 128
#endif
constexpr uint32_t COOP_MIN = DG_COOP_MIN;
// The frame's work plan (dg_render.cu, plan_kernel): a header of PLAN_HEADER
// words (cooperative tiles, tiles, backward chunks, spare), the tiles in the
// order the forward pass takes them, then the backward's (tile, chunk) pairs.
constexpr uint32_t PLAN_HEADER = 4;

// A warp's own window of up to 32 list entries, staged in its slice of shared
// memory: only the splats that can reach the warp's 8x4 pixel block, in list
// order. `raw` receives the splat records of the next window by cp.async while
// the current one blends.
struct WarpStage {
  float4 mean[32];   // mean x, y, opacity, 0
  float4 quad[32];   // A = -0.5 a, b, C = -0.5 c, cutoff
  float4 color[32];  // rgb, opacity
  uint32_t pos[32];  // position in the tile's list
  uint32_t index[32];
  float4 raw[32][3];  // lane l: the 48-byte record of its entry of the window in flight
  uint32_t live_count;  // cooperative blending: entries queued for warp 0
};

// A pixel's state at the start of chunk boundary k of a tile (after every entry
// before position k * CHUNK): transmittance and the colour blended so far. One
// slot of 8 blocks x 32 pixels per CHUNK entries of the pair list; boundary k of
// the tile whose list starts at run_x has slot (run_x + k * CHUNK) / CHUNK, which
// no other boundary of any tile shares.
__device__ __forceinline__ size_t checkpoint_at(uint32_t run_x, uint32_t k, uint32_t block, uint32_t lane) {
  const size_t slot = (run_x + k * CHUNK) / CHUNK;
  return (slot * 8u + block) * 32u + lane;
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// ---- Bulk copies (the Tensor Memory Accelerator's untiled form) completed on an
// mbarrier in shared memory.
// One arrival that also announces `bytes` of copies the barrier waits for.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_address(bar)), "r"(bytes)
               : "memory");
}
// Copies `bytes` (a multiple of 16; both addresses 16-byte aligned) from global
// src to shared dst; the barrier's transaction count drops as they land.
__device__ __forceinline__ void bulk_copy_to_shared(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
          smem_address(dst)),
      "l"(src), "r"(bytes), "r"(smem_address(bar))
      : "memory");
}
// The same with an L2 eviction policy for the lines it reads (l2_policy_*).
__device__ __forceinline__ void bulk_copy_to_shared(void* dst, const void* src, uint32_t bytes, uint64_t* bar,
                                                    uint64_t policy) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;\n" ::"r"(
          smem_address(dst)),
      "l"(src), "r"(bytes), "r"(smem_address(bar)), "l"(policy)
      : "memory");
}

// ---- Loads and stores with an L2 eviction policy (l2_policy_*, dg_common.cuh).
__device__ __forceinline__ float4 ld_hinted(const void* p, uint64_t policy) {
  float4 v;
  asm volatile("ld.global.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;\n"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "l"(p), "l"(policy)
               : "memory");
  return v;
}
__device__ __forceinline__ void st_hinted(void* p, float4 v, uint64_t policy) {
  asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;\n" ::"l"(p), "f"(v.x), "f"(v.y), "f"(v.z),
               "f"(v.w), "l"(policy)
               : "memory");
}

// Starts copying n floats from global src to shared dst, spread over the CTA's
// threads: every 16-byte chunk is issued at once (cp.async), instead of each
// thread waiting for one load before issuing the next. The caller waits
// (cp_async_wait_all) and synchronizes the CTA before reading dst.
__device__ __forceinline__ void stage_floats_async(float* dst, const float* __restrict__ src, uint32_t n) {
  if (((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15) == 0) {
    const uint32_t vecs = n / 4;
    for (uint32_t k = threadIdx.x; k < vecs; k += blockDim.x) cp_async16(dst + 4 * k, src + 4 * k);
    for (uint32_t k = vecs * 4 + threadIdx.x; k < n; k += blockDim.x) dst[k] = src[k];
  } else {
    for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) dst[k] = src[k];
  }
}

// Starts copying the splat record of this lane's entry of a window into `raw`.
__device__ __forceinline__ void stage_issue(WarpStage& st, const float* __restrict__ splats, uint32_t index,
                                            bool valid) {
  if (valid) {
    const uint32_t lane = threadIdx.x & 31u;
    const float4* s = reinterpret_cast<const float4*>(splats + (size_t)index * FLOATS_PER_SPLAT);
    cp_async16(&st.raw[lane][0], s);
    cp_async16(&st.raw[lane][1], s + 1);
    cp_async16(&st.raw[lane][2], s + 2);
  }
}

__device__ __forceinline__ uint4 tile_rect(float mx, float my, float radius, uint2 tiles);

// The 16x16 tile a blend item's block lies in, for blend tiles of several 16x16
// tiles: the block keeps only the entries of that tile's own list (the splats
// whose tile rectangle holds it). Unused (member == false) for 16x16 blend tiles.
struct TileMember {
  bool member;
  uint32_t tx, ty;
  uint2 tiles;
};

// Waits for the window [lo, min(lo + 32, hi)) issued by stage_issue (lane l holds
// entry lo + l, splat `index`) and keeps, in list order, the splats that can reach
// the warp's block, whose pixel centers span [x0, x0 + 7] x [y0, y0 + 3] (and,
// with a TileMember, belong to its 16x16 tile's list). Returns how many were
// kept. All 32 lanes must call it. Every value read from `raw` is consumed before
// this returns, so the caller may issue the next window at once. cut_in_record:
// the splats carry their blend cutoff in slot SPLAT_CUTOFF_SLOT (this build's
// preprocess wrote them), else it is computed here.
__device__ __forceinline__ uint32_t stage_commit(WarpStage& st, uint32_t run_x, uint32_t lo, uint32_t hi,
                                                 uint32_t index, float x0, float y0, bool cut_in_record,
                                                 const TileMember& tm = TileMember{false, 0u, 0u, {0u, 0u}}) {
  cp_async_wait_all();
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t k = lo + lane;
  bool keep = false;
  float2 mean = make_float2(0.f, 0.f);
  float4 quad = make_float4(0.f, 0.f, 0.f, 0.f), color = quad;
  if (k < hi) {
    const float4 s0 = st.raw[lane][0], s1 = st.raw[lane][1];
    color = st.raw[lane][2];
    mean = make_float2(s0.x, s0.y);
    const float A = -0.5f * s1.x, b = s1.y, C = -0.5f * s1.z;
    const float cut = cut_in_record ? s1.w : blend_cutoff(color.w);
    quad = make_float4(A, b, C, cut);
    keep = cut < 0.0f && rect_reachable(A, b, C, __fdividef(b, 2.0f * A), __fdividef(b, 2.0f * C), cut,
                                        x0 - mean.x, x0 + 7.0f - mean.x, y0 - mean.y, y0 + 3.0f - mean.y);
    if (tm.member && keep) {
      const uint4 rect = tile_rect(mean.x, mean.y, s0.w, tm.tiles);
      keep = tm.tx >= rect.x && tm.tx < rect.z && tm.ty >= rect.y && tm.ty < rect.w;
    }
  }
  const uint32_t kept = __ballot_sync(0xffffffffu, keep);
  if (keep) {
    const uint32_t at = __popc(kept & ((1u << lane) - 1u));
    st.mean[at] = make_float4(mean.x, mean.y, color.w, 0.0f);
    st.quad[at] = quad;
    st.color[at] = color;
    st.pos[at] = k - run_x;
    st.index[at] = index;
  }
  __syncwarp();
  return __popc(kept);
}


// Like stage_commit for a window whose entries the block blended are known:
// lane l keeps entry lo + l when bit l of `blended` is set (lanes past hi must
// have it clear), with no rectangle test.
__device__ __forceinline__ uint32_t stage_commit_blended(WarpStage& st, uint32_t run_x, uint32_t lo, uint32_t index,
                                                         uint32_t blended, bool cut_in_record) {
  cp_async_wait_all();
  const uint32_t lane = threadIdx.x & 31u;
  const bool keep = (blended >> lane) & 1u;
  if (keep) {
    const uint32_t at = __popc(blended & ((1u << lane) - 1u));
    const float4 s0 = st.raw[lane][0], s1 = st.raw[lane][1], color = st.raw[lane][2];
    st.mean[at] = make_float4(s0.x, s0.y, color.w, 0.0f);
    st.quad[at] = make_float4(-0.5f * s1.x, s1.y, -0.5f * s1.z, cut_in_record ? s1.w : blend_cutoff(color.w));
    st.color[at] = color;
    st.pos[at] = lo + lane - run_x;
    st.index[at] = index;
  }
  __syncwarp();
  return __popc(blended);
}

// tile_count / tile_rect (src/shaders/common.wgsl:31-42).
__device__ __forceinline__ uint2 tile_grid(const Camera& cam) {
  return make_uint2(((uint32_t)cam.viewport[0] + TILE - 1u) / TILE, ((uint32_t)cam.viewport[1] + TILE - 1u) / TILE);
}

__device__ __forceinline__ uint4 tile_rect(float mx, float my, float radius, uint2 tiles) {
  float lox = clampf(floorf((mx - radius) / 16.0f), 0.0f, (float)tiles.x);
  float loy = clampf(floorf((my - radius) / 16.0f), 0.0f, (float)tiles.y);
  float hix = clampf(floorf((mx + radius) / 16.0f) + 1.0f, 0.0f, (float)tiles.x);
  float hiy = clampf(floorf((my + radius) / 16.0f) + 1.0f, 0.0f, (float)tiles.y);
  return make_uint4((uint32_t)lox, (uint32_t)loy, (uint32_t)hix, (uint32_t)hiy);
}

// Blend tiles: a batch of views may blend and sort in tiles of 2^twl x 2^thl
// 16x16 tiles (32x16, 32x32 pixels). A splat is listed once for each blend tile
// its 16x16-tile rectangle touches, so there are fewer pairs than 16x16 ones, and
// each 8x4 block keeps only the entries of its own 16x16 tile's list
// (TileMember): every pixel blends exactly the splats, in exactly the order, of
// the 16x16 tiling. Coverage itself stays 16x16: a splat's square of half-size
// ceil(3 sigma) does not bound where its alpha reaches 1/255 (opacity above
// 0.36 reaches it past 3 sigma), so tiles cut smaller than 16x16 would drop
// contributions the reference blends.
__host__ __device__ __forceinline__ uint32_t blend_tiles_along(uint32_t tiles, uint32_t log2) {
  return (tiles + (1u << log2) - 1u) >> log2;
}

// The blend tiles that a 16x16-tile rectangle touches (empty stays empty).
__device__ __forceinline__ uint4 blend_rect(uint4 rect, uint32_t twl, uint32_t thl) {
  if (rect.z <= rect.x || rect.w <= rect.y) return make_uint4(0u, 0u, 0u, 0u);
  return make_uint4(rect.x >> twl, rect.y >> thl, blend_tiles_along(rect.z, twl), blend_tiles_along(rect.w, thl));
}

}  // namespace dg

// The renderer's backward passes: the blend's (src/shaders/rasterizeBackward.wgsl)
// and the preprocess's (src/shaders/preprocessBackward.wgsl).
//
// Compiled with the default --fmad=true: gradients only need to agree to rounding
// (their tile sums meet through float atomics anyway). The arithmetic that decides
// which splats a pixel blended (blend_power, exp_blend_core, the alpha product and its
// thresholds) is written with non-fusing intrinsics or explicit fmaf, so it makes
// exactly the forward pass's decisions.
#include "dg_adam.cuh"
#include "dg_render.cuh"
#include "dg_render_kernels.cuh"

namespace dg {
namespace {

__device__ __forceinline__ void load_camera(Camera& dst, const Camera* src) {
  const float* s = reinterpret_cast<const float*>(src);
  float* d = reinterpret_cast<float*>(&dst);
  for (int k = threadIdx.x; k < 36; k += blockDim.x) d[k] = s[k];
}

// One halving step of a reduce-scatter over the warp: a lane holding M partial
// sums keeps the lower or the upper half of them (by bit D of its lane index) and
// adds its partner's copy of that half. With M == 1 both lanes keep the sum.
template <int M, int D>
__device__ __forceinline__ void reduce_half(float* v, uint32_t lane) {
  if constexpr (M == 1) {
    v[0] = v[0] + __shfl_xor_sync(0xffffffffu, v[0], D);
  } else {
    constexpr int H = (M + 1) / 2;
    const bool upper = lane & D;
#pragma unroll
    for (int k = 0; k < H; k++) {
      const float lo = v[k], hi = H + k < M ? v[H + k] : 0.0f;
      const float got = __shfl_xor_sync(0xffffffffu, upper ? lo : hi, D);
      v[k] = (upper ? hi : lo) + got;
    }
  }
}

// Sums N <= 32 values over the warp's 32 lanes with about N shuffles (N = 18:
// 20 shuffles in 5 dependent steps, against 5 N in 5 N steps for N separate
// butterflies). Afterwards lane l holds the total of value reduce_slot<N>(l), or
// a copy or padding where that is -1. Clobbers v.
template <int N>
__device__ __forceinline__ float warp_reduce_scatter(float (&v)[N], uint32_t lane) {
  static_assert(N <= 32, "one value per lane at most");
  constexpr int M2 = (N + 1) / 2, M3 = (M2 + 1) / 2, M4 = (M3 + 1) / 2, M5 = (M4 + 1) / 2;
  static_assert(M5 == 1 || (M5 == 2 && N > 16), "the last step leaves one value per lane");
  reduce_half<N, 16>(v, lane);
  reduce_half<M2, 8>(v, lane);
  reduce_half<M3, 4>(v, lane);
  reduce_half<M4, 2>(v, lane);
  reduce_half<M5, 1>(v, lane);
  return v[0];
}

// Which of the N values lane `lane` holds after warp_reduce_scatter<N>: the index
// ranges each step keeps, followed for this lane's bits; -1 for padding or for the
// upper lane of a pair that holds the same sum.
template <int N>
__device__ __forceinline__ int reduce_slot(uint32_t lane) {
  int base = 0, real = N, m = N;
#pragma unroll
  for (int d = 16; d >= 1; d >>= 1) {
    if (m == 1) {
      if (lane & d) real = 0;
      continue;
    }
    const int h = (m + 1) / 2;
    if (lane & d) {
      base += h;
      real = real > h ? real - h : 0;
    } else {
      real = real < h ? real : h;
    }
    m = h;
  }
  return real > 0 ? base : -1;
}

// The exponent, Gaussian and alpha of a splat at this lane's pixel, and whether
// the forward pass blended it there (the same decisions, made with the same
// non-fusing arithmetic).
struct BlendTerm {
  float dx, dy, G, alpha;
  bool blended;
};

// The terms of two entries at once (their exps as one packed pair).
__device__ __forceinline__ void blend_terms(const WarpStage& st, uint32_t e0, uint32_t e1, bool eligible0,
                                            bool eligible1, float cx, float cy, BlendTerm& t0, BlendTerm& t1) {
  const float4 m0 = st.mean[e0], m1 = st.mean[e1];  // .z: opacity
  const float4 q0 = st.quad[e0], q1 = st.quad[e1];
  t0.dx = cx - m0.x;
  t0.dy = cy - m0.y;
  t1.dx = cx - m1.x;
  t1.dy = cy - m1.y;
  const float power0 = blend_power(q0.x, q0.y, q0.z, t0.dx, t0.dy);
  const float power1 = blend_power(q1.x, q1.y, q1.z, t1.dx, t1.dy);
  const bool need0 = eligible0 && power0 >= q0.w && power0 <= 0.0f;
  const bool need1 = eligible1 && power1 >= q1.w && power1 <= 0.0f;
  exp_blend_core2(need0 ? power0 : 0.0f, need1 ? power1 : 0.0f, t0.G, t1.G);
  t0.alpha = fminf(0.99f, __fmul_rn(m0.z, t0.G));
  t1.alpha = fminf(0.99f, __fmul_rn(m1.z, t1.G));
  t0.blended = need0 && t0.alpha >= 1.0f / 255.0f;
  t1.blended = need1 && t1.alpha >= 1.0f / 255.0f;
}

// A pixel's state on its back-to-front walk: the transmittance in front of the
// current splat, the colour composited behind it and the last splat passed.
struct PixelBackward {
  float T, pgx, pgy, pgz, tf_bg;  // tf_bg: the final T times (background . pixel gradient)
  float bhx, bhy, bhz;  // colour of everything behind
  float na, ncx, ncy, ncz;

  // Starts the walk at a point where the transmittance is T0 and the colour
  // composited behind, relative to T0, is `behind`.
  __device__ __forceinline__ void begin(float final_T, float T0, float3 behind, float gx, float gy, float gz,
                                        float4 bg) {
    T = T0;
    pgx = gx;
    pgy = gy;
    pgz = gz;
    tf_bg = final_T * (bg.x * gx + bg.y * gy + bg.z * gz);
    bhx = behind.x;
    bhy = behind.y;
    bhz = behind.z;
    na = ncx = ncy = ncz = 0.0f;
  }

  // Steps in front of a splat this pixel blended and writes its 9 gradient shares.
  __device__ __forceinline__ void shares(const BlendTerm& t, float4 q, float4 c, float* w) {
    const float alpha = t.alpha, G = t.G, dx = t.dx, dy = t.dy;
    // 1 / (1 - alpha), used twice; the approximate reciprocal (~1 ulp) is plenty:
    // a chunk's chain of divisions is at most CHUNK entries long.
    float inv;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(inv) : "f"(1.0f - alpha));
    T = T * inv;
    // The colour behind, na nc + (1 - na) bh, as bh + na (nc - bh).
    bhx = fmaf(na, ncx - bhx, bhx);
    bhy = fmaf(na, ncy - bhy, bhy);
    bhz = fmaf(na, ncz - bhz, bhz);
    na = alpha;
    ncx = c.x;
    ncy = c.y;
    ncz = c.z;
    const float dotv = (c.x - bhx) * pgx + (c.y - bhy) * pgy + (c.z - bhz) * pgz;
    const float alpha_grad = T * dotv - inv * tf_bg;
    const float power_grad = alpha_grad * c.w * G;
    // The conic is (a, b, c) = (-2A, b, -2C): the power's gradient is
    // -(a dx + b dy, b dx + c dy) for the mean and (-dx^2 / 2, -dx dy, -dy^2 / 2)
    // for the conic, here as multiples of (power_grad dx, power_grad dy).
    const float pdx = power_grad * dx, pdy = power_grad * dy;
    w[0] = -2.0f * q.x * pdx + q.y * pdy;
    w[1] = q.y * pdx - 2.0f * q.z * pdy;
    w[2] = -0.5f * pdx * dx;
    w[3] = -pdx * dy;
    w[4] = -0.5f * pdy * dy;
    w[5] = alpha_grad * G;
    const float wt = alpha * T;
    w[6] = wt * pgx;
    w[7] = wt * pgy;
    w[8] = wt * pgz;
  }
};

// The start of the back-to-front window that ends at `end`: max(floor, end - 32).
__device__ __forceinline__ uint32_t window_start(uint32_t end, uint32_t floor) {
  return end - floor > 32u ? end - 32u : floor;
}

// The blend mask words of `block` covering a chunk's positions [lo, hi) (at most
// CHUNK / 32 + 1 words): lane l holds word (lo / 32) + l, or 0 past them.
__device__ __forceinline__ uint32_t chunk_mask_words(const uint32_t* __restrict__ mask, uint32_t lo, uint32_t hi,
                                                     uint32_t block, uint32_t lane) {
  static_assert(CHUNK / 32 + 1 <= 32, "a chunk's mask words fit in the warp's lanes");
  const uint32_t w = (lo >> 5) + lane;
  return w <= ((hi - 1u) >> 5) ? mask[(size_t)w * 8u + block] : 0u;
}

// The blend mask bits of window [lo, hi) (none when it is empty) from the chunk's
// words in the lanes (chunk_mask_words from position base). All lanes must call it.
__device__ __forceinline__ uint32_t window_blended(uint32_t words, uint32_t base, uint32_t lo, uint32_t hi) {
  const uint32_t at = (lo >> 5) - (base >> 5), shift = lo & 31u;
  const uint32_t a = __shfl_sync(0xffffffffu, words, at & 31u), b = __shfl_sync(0xffffffffu, words, (at + 1u) & 31u);
  if (hi <= lo) return 0u;
  const uint32_t bits = shift ? (a >> shift) | (b << (32u - shift)) : a;
  return hi - lo >= 32u ? bits : bits & ((1u << (hi - lo)) - 1u);
}

// src/shaders/rasterizeBackward.wgsl:50-163. The work is split into independent
// items, one per (tile, CHUNK-entry chunk of its list, 8x4 pixel block), taken by
// persistent warps from a counter in the plan's order, so no warp waits for
// another and a long list is spread over many warps. For an item, the warp walks
// its chunk back to front from the largest `last` among its pixels, keeping in its
// own slice of shared memory, 32 entries at a time, only the splats some pixel of
// its block blended in the forward pass (the forward's blend mask; the records of
// the next window are copied in meanwhile). Each pixel
// starts from its state behind the chunk: the transmittance the forward pass saved
// at the chunk's end, and the colour behind it, (final colour - colour saved) /
// that transmittance; behind its last splat (the whole list for most tiles) these
// are the final transmittance and nothing. Splats are then taken two at a time:
// their alphas are computed together, then each pixel recovers the transmittance
// in front of each splat by dividing by (1 - alpha), in list order. The 18
// gradient shares of the pair are summed over the warp's 32 pixels in one
// reduce-scatter and added to the splats' global gradients, one atomic add per
// nonzero total.
__global__ void __launch_bounds__(BWD_THREADS, 6) rasterize_backward_kernel(
    const Camera* __restrict__ camera, const float4* __restrict__ raster_params, const float* __restrict__ splats,
    const uint32_t* __restrict__ pair_splats, const uint2* __restrict__ ranges, const uint32_t* __restrict__ plan,
    const uint2* __restrict__ chunks, const float4* __restrict__ pixel_color, const uint32_t* __restrict__ pixel_last,
    const float4* __restrict__ checkpoints, const uint32_t* __restrict__ blend_mask,
    const float4* __restrict__ pixel_grads, float* __restrict__ splat_grads, uint32_t* __restrict__ work_counter,
    bool cut_in_record) {
  __shared__ WarpStage stages[BWD_WARPS];
  const uint32_t lane = threadIdx.x & 31u;
  WarpStage& st = stages[threadIdx.x >> 5];
  const float vpx = camera->viewport[0], vpy = camera->viewport[1];
  const uint32_t tiles_x = ((uint32_t)vpx + TILE - 1u) / TILE;
  const uint32_t items = plan[2] * 8u;
  const float4 bg = raster_params[0];
  const int my_slot = reduce_slot<2 * SPLAT_GRADS>(lane);
  // Value my_slot belongs to the pair's first (further back) splat when below 9.
  const uint32_t my_entry = my_slot >= (int)SPLAT_GRADS ? 1u : 0u;
  const uint32_t my_grad = my_slot >= 0 ? (uint32_t)my_slot - my_entry * SPLAT_GRADS : 0u;
  while (true) {
    uint32_t item = 0;
    if (lane == 0) item = atomicAdd(work_counter, 1u);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= items) break;
    const uint2 chunk = chunks[item >> 3];
    const uint32_t tile = chunk.x, block = item & 7u;
    const uint32_t bx = (tile % tiles_x) * TILE + (block & 1u) * 8u, by = (tile / tiles_x) * TILE + (block >> 1) * 4u;
    const uint32_t px = bx + (lane & 7u), py = by + (lane >> 3);
    const bool inside = (float)px < vpx && (float)py < vpy;
    const float cx = (float)px + 0.5f, cy = (float)py + 0.5f;
    const uint2 run = ranges[tile];
    const uint32_t chunk_lo = run.x + chunk.y * CHUNK, chunk_hi = min(chunk_lo + CHUNK, run.y);
    const uint32_t boundary = (chunk.y + 1u) * CHUNK;  // the chunk's end, relative to run.x
    float4 color = make_float4(0.f, 0.f, 0.f, 0.f), pg = color;
    uint32_t last = 0;
    if (inside) {
      const uint32_t p = py * (uint32_t)vpx + px;
      color = pixel_color[p];
      last = pixel_last[p];
      pg = pixel_grads[p];
    }
    // Splats at or past the warp's largest `last` contribute nothing to it.
    const uint32_t end_all = min(chunk_hi, run.x + __reduce_max_sync(0xffffffffu, last));
    if (end_all <= chunk_lo) continue;
    float T0 = color.w;
    float3 behind = make_float3(0.f, 0.f, 0.f);
    if (last > boundary) {  // the pixel blends splats behind this chunk
      const float4 ck = checkpoints[checkpoint_at(run.x, chunk.y + 1u, block, lane)];
      const float inv = 1.0f / ck.x;
      T0 = ck.x;
      behind = make_float3((color.x - color.w * bg.x - ck.y) * inv, (color.y - color.w * bg.y - ck.z) * inv,
                           (color.z - color.w * bg.z - ck.w) * inv);
    }
    PixelBackward px_state;
    px_state.begin(color.w, T0, behind, pg.x, pg.y, pg.z, bg);
    // Windows run back to front: [lo, end) with lo = max(chunk_lo, end - 32). Only
    // the entries some pixel of the block blended (the forward pass's mask) are
    // staged. This lane's entry of the window in flight and of the next one.
    const uint32_t words = chunk_mask_words(blend_mask, chunk_lo, end_all, block, lane);
    uint32_t end = end_all;
    uint32_t lo = window_start(end, chunk_lo);
    uint32_t bits = window_blended(words, chunk_lo, lo, end);
    uint32_t index = (bits >> lane) & 1u ? pair_splats[lo + lane] : 0u;
    stage_issue(st, splats, index, (bits >> lane) & 1u);
    uint32_t next_lo = window_start(lo, chunk_lo);
    uint32_t next_bits = window_blended(words, chunk_lo, next_lo, lo);
    uint32_t next_index = (next_bits >> lane) & 1u ? pair_splats[next_lo + lane] : 0u;
    while (end > chunk_lo) {
      const uint32_t staged = stage_commit_blended(st, run.x, lo, index, bits, cut_in_record);
      {
        stage_issue(st, splats, next_index, (next_bits >> lane) & 1u);
        end = lo;
        lo = next_lo;
        bits = next_bits;
        index = next_index;
        next_lo = window_start(lo, chunk_lo);
        next_bits = window_blended(words, chunk_lo, next_lo, lo);
        next_index = (next_bits >> lane) & 1u ? pair_splats[next_lo + lane] : 0u;
      }
      for (uint32_t slot = staged; slot > 0;) {
        // Entries j0 (further back, taken first) and j1 = j0 - 1 when there is one.
        const uint32_t j0 = slot - 1, j1 = slot >= 2 ? slot - 2 : j0;
        const bool pair = slot >= 2;
        slot = pair ? slot - 2 : 0;
        BlendTerm t0, t1;
        blend_terms(st, j0, j1, inside && st.pos[j0] < last, pair && inside && st.pos[j1] < last, cx, cy, t0, t1);
        if (!__any_sync(0xffffffffu, t0.blended || t1.blended)) continue;
        float v[2 * SPLAT_GRADS];
#pragma unroll
        for (int q = 0; q < 2 * (int)SPLAT_GRADS; q++) v[q] = 0.0f;
        // Back to front: j0, then j1.
        if (t0.blended) px_state.shares(t0, st.quad[j0], st.color[j0], v);
        if (t1.blended) px_state.shares(t1, st.quad[j1], st.color[j1], v + SPLAT_GRADS);
        const float total = warp_reduce_scatter(v, lane);
        if (my_slot >= 0 && total != 0.0f && (my_entry == 0 || pair))
          atomicAdd(&splat_grads[(size_t)st.index[my_entry ? j1 : j0] * SPLAT_GRADS + my_grad], total);
      }
      __syncwarp();
    }
    cp_async_wait_all();
  }
}

#ifndef DG_PBWD_THREADS
#define DG_PBWD_THREADS 128
#endif
constexpr uint32_t PBWD_THREADS = DG_PBWD_THREADS;  // a multiple of 32

// Copies n floats between global and shared memory, 16 bytes at a time where both
// ends allow it; all threads of the CTA take part.
__device__ __forceinline__ void copy_floats(float* __restrict__ dst, const float* __restrict__ src, uint32_t n) {
  if (((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15) == 0) {
    const uint32_t vecs = n / 4;
    for (uint32_t k = threadIdx.x; k < vecs; k += blockDim.x)
      reinterpret_cast<float4*>(dst)[k] = reinterpret_cast<const float4*>(src)[k];
    for (uint32_t k = vecs * 4 + threadIdx.x; k < n; k += blockDim.x) dst[k] = src[k];
  } else {
    for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) dst[k] = src[k];
  }
}

// src/shaders/preprocessBackward.wgsl:28-181 for one Gaussian: the 16-float
// Gaussian gradient (slots 7 and 15 zero) to out, and the 45 SH gradients over
// its 45 SH coefficients in shv (shared memory).
// gaussian: the Gaussian's 16 activated floats (16-byte aligned); radius: its
// splat's radius (0 when it was not drawn); grads: its 9 splat gradients. shv
// holds its SH coefficients and receives their gradients.
__device__ __forceinline__ void preprocess_backward_one(const Camera& cam, const float* __restrict__ gaussian,
                                                        float* shv, uint32_t basis_count, float radius,
                                                        const float* __restrict__ grads, float (&out)[16]) {
#pragma unroll
  for (int k = 0; k < 16; k++) out[k] = 0.0f;
  if (radius == 0.0f) {
    for (uint32_t k = 0; k < SH_REST_FLOATS; k++) shv[k] = 0.0f;
    return;
  }
  float grad[9];
#pragma unroll
  for (int k = 0; k < 9; k++) grad[k] = grads[k];
  float g[16];
  {
    const float4* gp = reinterpret_cast<const float4*>(gaussian);
#pragma unroll
    for (int k = 0; k < 4; k++) {
      float4 q = gp[k];
      g[4 * k] = q.x; g[4 * k + 1] = q.y; g[4 * k + 2] = q.z; g[4 * k + 3] = q.w;
    }
  }
  Projection p;
  project(cam, g, p);
  const float depth = p.depth;
  const float ratio0 = p.t[0] / depth, ratio1 = p.t[1] / depth;
  const float free0 = fabsf(ratio0) > p.limit[0] ? 0.0f : 1.0f;
  const float free1 = fabsf(ratio1) > p.limit[1] ? 0.0f : 1.0f;
  const float depth2 = depth * depth, depth3 = depth2 * depth;
  const float a = p.a, b = p.b, c = p.c, det = p.det;
  // 1. conic -> 2D covariance
  const float det2 = det * det;
  const float a_grad = (-c * c * grad[2] + b * c * grad[3] - b * b * grad[4]) / det2;
  const float b_grad = (2.0f * b * c * grad[2] - (det + 2.0f * b * b) * grad[3] + 2.0f * a * b * grad[4]) / det2;
  const float c_grad = (-b * b * grad[2] + a * b * grad[3] - a * a * grad[4]) / det2;
  const float G2[2][2] = {{a_grad, 0.5f * b_grad}, {0.5f * b_grad, c_grad}};
  // 2. Σ' = T Σ Tᵀ with T = J W
  float Gjw[3][2];
#pragma unroll
  for (int col = 0; col < 3; col++)
#pragma unroll
    for (int row = 0; row < 2; row++) {
      float v = G2[0][row] * p.jw[col][0];
      v = v + G2[1][row] * p.jw[col][1];
      Gjw[col][row] = v;
    }
  float cov3d_grad[3][3];
#pragma unroll
  for (int col = 0; col < 3; col++)
#pragma unroll
    for (int row = 0; row < 3; row++) {
      float v = p.jw[row][0] * Gjw[col][0];
      v = v + p.jw[row][1] * Gjw[col][1];
      cov3d_grad[col][row] = v;
    }
  float t3[3][2];
#pragma unroll
  for (int col = 0; col < 3; col++)
#pragma unroll
    for (int row = 0; row < 2; row++) {
      float v = (2.0f * Gjw[0][row]) * p.cov3d[col][0];
      v = v + (2.0f * Gjw[1][row]) * p.cov3d[col][1];
      v = v + (2.0f * Gjw[2][row]) * p.cov3d[col][2];
      t3[col][row] = v;
    }
  float jg[3][2];
#pragma unroll
  for (int col = 0; col < 3; col++)
#pragma unroll
    for (int row = 0; row < 2; row++) {
      float v = t3[0][row] * p.w[0][col];
      v = v + t3[1][row] * p.w[1][col];
      v = v + t3[2][row] * p.w[2][col];
      jg[col][row] = v;
    }
  // 3. J moves with t
  float tg[3];
  tg[0] = jg[2][0] * free0 * p.focal[0] / depth2;
  tg[1] = jg[2][1] * free1 * -p.focal[1] / depth2;
  tg[2] = 0.0f;
  const float depth_grad = jg[0][0] * (-p.focal[0] / depth2) + jg[1][1] * (p.focal[1] / depth2) +
                           jg[2][0] * (-(1.0f + free0) * p.focal[0] * p.tx / depth3) +
                           jg[2][1] * ((1.0f + free1) * p.focal[1] * p.ty / depth3);
  tg[2] = tg[2] - depth_grad;
  // 4. the 2D center
  float clip[4];
#pragma unroll
  for (int row = 0; row < 4; row++) {
    float v = cam.proj[0 * 4 + row] * p.t[0];
    v = v + cam.proj[1 * 4 + row] * p.t[1];
    v = v + cam.proj[2 * 4 + row] * p.t[2];
    v = v + cam.proj[3 * 4 + row] * 1.0f;
    clip[row] = v;
  }
  const float ng0 = grad[0] * 0.5f * cam.viewport[0], ng1 = grad[1] * -0.5f * cam.viewport[1];
  float ndc_dot = ng0 * clip[0];
  ndc_dot = ndc_dot + ng1 * clip[1];
  const float clip_grad[4] = {ng0 / clip[3], ng1 / clip[3], 0.0f, -ndc_dot / (clip[3] * clip[3])};
#pragma unroll
  for (int col = 0; col < 3; col++) {
    float v = cam.proj[col * 4 + 0] * clip_grad[0];
    v = v + cam.proj[col * 4 + 1] * clip_grad[1];
    v = v + cam.proj[col * 4 + 2] * clip_grad[2];
    v = v + cam.proj[col * 4 + 3] * clip_grad[3];
    tg[col] = tg[col] + v;
  }
  // 5. colour
  float campos[3], off[3], dir[3], basis[15];
  camera_position(cam, campos);
  off[0] = g[0] - campos[0];
  off[1] = g[1] - campos[1];
  off[2] = g[2] - campos[2];
  const float dist = normalize3(off, dir);
  sh_basis(dir, basis);
  const float* coef = shv;
  float raw_color[3] = {g[12], g[13], g[14]};
  // These SH loops stay rolled: unrolled (basis and bgrad in registers) the
  // fused backward + Adam kernel takes 112 registers, 4 CTAs per SM instead of
  // 5, and runs slower (435 vs 408 us at 1.1M Gaussians).
  for (uint32_t k = 0; k < basis_count; k++)
#pragma unroll
    for (int ch = 0; ch < 3; ch++) raw_color[ch] = raw_color[ch] + basis[k] * coef[k * 3 + ch];
  float raw_grad[3];
#pragma unroll
  for (int ch = 0; ch < 3; ch++) raw_grad[ch] = raw_color[ch] < 0.0f ? 0.0f : grad[6 + ch];
  float dgrad[3] = {0.0f, 0.0f, 0.0f};
  {
    float bgrad[15][3];
    sh_basis_gradient(dir, bgrad);
    // Each coefficient is read before its slot of shv takes the gradient.
    for (uint32_t k = 0; k < SH_REST_FLOATS / 3; k++) {
      if (k < basis_count) {
        float d = coef[k * 3] * raw_grad[0];
        d = d + coef[k * 3 + 1] * raw_grad[1];
        d = d + coef[k * 3 + 2] * raw_grad[2];
#pragma unroll
        for (int ch = 0; ch < 3; ch++) shv[k * 3 + ch] = basis[k] * raw_grad[ch];
#pragma unroll
        for (int ax = 0; ax < 3; ax++) dgrad[ax] = dgrad[ax] + bgrad[k][ax] * d;
      } else {
#pragma unroll
        for (int ch = 0; ch < 3; ch++) shv[k * 3 + ch] = 0.0f;
      }
    }
  }
  float dd = dir[0] * dgrad[0];
  dd = dd + dir[1] * dgrad[1];
  dd = dd + dir[2] * dgrad[2];
  // 6. position
#pragma unroll
  for (int col = 0; col < 3; col++) {
    float v = p.w[col][0] * tg[0];
    v = v + p.w[col][1] * tg[1];
    v = v + p.w[col][2] * tg[2];
    out[col] = v + (dgrad[col] - dir[col] * dd) / dist;
  }
  // 7. scale and rotation
  float mg[3][3];
#pragma unroll
  for (int col = 0; col < 3; col++)
#pragma unroll
    for (int row = 0; row < 3; row++) {
      float v = 2.0f * cov3d_grad[0][row] * p.m[col][0];
      v = v + 2.0f * cov3d_grad[1][row] * p.m[col][1];
      v = v + 2.0f * cov3d_grad[2][row] * p.m[col][2];
      mg[col][row] = v;
    }
#pragma unroll
  for (int k = 0; k < 3; k++) {
    float v = mg[k][0] * p.r[k][0];
    v = v + mg[k][1] * p.r[k][1];
    v = v + mg[k][2] * p.r[k][2];
    out[4 + k] = v;
  }
  float rg[3][3];
#pragma unroll
  for (int col = 0; col < 3; col++)
#pragma unroll
    for (int row = 0; row < 3; row++) rg[col][row] = mg[col][row] * g[4 + col];
  const float qw = p.q[0], qx = p.q[1], qy = p.q[2], qz = p.q[3];
  const float g00 = rg[0][0], g01 = rg[1][0], g02 = rg[2][0];
  const float g10 = rg[0][1], g11 = rg[1][1], g12 = rg[2][1];
  const float g20 = rg[0][2], g21 = rg[1][2], g22 = rg[2][2];
  float qg[4];
  qg[0] = 2.0f * (-qz * g01 + qy * g02 + qz * g10 - qx * g12 - qy * g20 + qx * g21);
  qg[1] = 2.0f * (qy * g01 + qz * g02 + qy * g10 - 2.0f * qx * g11 - qw * g12 + qz * g20 + qw * g21 - 2.0f * qx * g22);
  qg[2] = 2.0f * (-2.0f * qy * g00 + qx * g01 + qw * g02 + qx * g10 + qz * g12 - qw * g20 + qz * g21 - 2.0f * qy * g22);
  qg[3] = 2.0f * (-2.0f * qz * g00 - qw * g01 + qx * g02 + qw * g10 - 2.0f * qz * g11 + qy * g12 + qx * g20 + qy * g21);
  float qd = p.q[0] * qg[0];
  qd = qd + p.q[1] * qg[1];
  qd = qd + p.q[2] * qg[2];
  qd = qd + p.q[3] * qg[3];
  out[3] = grad[5];
#pragma unroll
  for (int k = 0; k < 4; k++) out[8 + k] = (qg[k] - p.q[k] * qd) / p.qlen;
  out[12] = raw_grad[0];
  out[13] = raw_grad[1];
  out[14] = raw_grad[2];
}

__device__ __forceinline__ void store16(float* __restrict__ dst, const float (&v)[16]) {
#pragma unroll
  for (int k = 0; k < 4; k++)
    reinterpret_cast<float4*>(dst)[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
}

// One thread per Gaussian. The CTA's SH coefficients are staged in shared memory
// and its SH gradients written back from there, both as contiguous copies (a
// thread's own 45 floats would otherwise be 180 bytes apart from its neighbour's).
__global__ void __launch_bounds__(PBWD_THREADS) preprocess_backward_kernel(
    const Camera* __restrict__ camera, const float* __restrict__ gaussians, const float* __restrict__ sh,
    uint32_t count, const uint32_t* __restrict__ scene_params, const float* __restrict__ splats,
    const float* __restrict__ splat_grads, float* __restrict__ gaussian_grads, float* __restrict__ sh_grads) {
  __shared__ Camera s_cam;
  __shared__ __align__(16) float s_sh[PBWD_THREADS * SH_REST_FLOATS];
  load_camera(s_cam, camera);
  const uint32_t block_start = blockIdx.x * PBWD_THREADS;
  const uint32_t here = min(PBWD_THREADS, count - block_start);
  stage_floats_async(s_sh, sh + (size_t)block_start * SH_REST_FLOATS, here * SH_REST_FLOATS);
  cp_async_wait_all();
  __syncthreads();
  const uint32_t degree = scene_params[0];
  const uint32_t basis_count = (degree + 1u) * (degree + 1u) - 1u;
  const uint32_t i = block_start + threadIdx.x;
  if (i < count) {
    float out[16];
    preprocess_backward_one(s_cam, gaussians + (size_t)i * FLOATS_PER_GAUSSIAN, s_sh + threadIdx.x * SH_REST_FLOATS,
                            basis_count, splats[(size_t)i * FLOATS_PER_SPLAT + 3],
                            splat_grads + (size_t)i * SPLAT_GRADS, out);
    store16(gaussian_grads + (size_t)i * FLOATS_PER_GAUSSIAN, out);
  }
  __syncthreads();
  copy_floats(sh_grads + (size_t)block_start * SH_REST_FLOATS, s_sh, here * SH_REST_FLOATS);
}

// The fused kernel's tuning: the 16-byte groups of slots (four slots each) a
// thread loads before stepping them in the Adam passes.
#ifndef DG_ADAM_SH_QUADS
#define DG_ADAM_SH_QUADS 3
#endif
#ifndef DG_ADAM_P_QUADS
#define DG_ADAM_P_QUADS 4
#endif
// A minimum of resident CTAs per SM caps the registers (without one ptxas
// settles at 96 a thread, 5 CTAs of 128 per SM; an explicit minimum of 1 lets it
// take 141).
#ifdef DG_PBWD_MIN_BLOCKS
#define DG_PBWD_BOUNDS __launch_bounds__(PBWD_THREADS, DG_PBWD_MIN_BLOCKS)
#else
#define DG_PBWD_BOUNDS __launch_bounds__(PBWD_THREADS)
#endif

__device__ __forceinline__ float4 f4_load(const float* p) { return *reinterpret_cast<const float4*>(p); }

// The training step's preprocess backward with Adam applied at once
// (src/shaders/preprocessBackward.wgsl:28-181, then src/shaders/adam.wgsl:80-107).
// A CTA takes 128 consecutive Gaussians:
// 1. one bulk copy (TMA) brings their SH coefficients, a contiguous 23 KB, into
//    shared memory, completed on an mbarrier;
// 2. each thread computes one Gaussian's gradients into shared memory (the SH
//    coefficients staged there turn into their gradients; the 16 parameter
//    gradients go to a row of pitch 17) and adds its densification statistics
//    (src/shaders/adam.wgsl:126-134);
// 3. Adam steps the CTA's SH slots: their coefficients, SH moments (the second
//    plane of the moment buffer) and gradients share one index, so each thread
//    takes 16-byte groups of four slots;
// 4. Adam steps the raw parameter slots a quarter record (four slots) at a time:
//    raw values, parameter moments (the first plane) and activated values move
//    as 16-byte groups. Slots 7 and 15 (pads: a densified Gaussian's kind and
//    step) keep their raw value and moments; their activated value is 0, as the
//    reference leaves it (src/shaders/adam.wgsl:60-71 does not write them).
// The 244 bytes of gradients per Gaussian never go to memory and back;
// gaussian_grads and sh_grads (may be NULL) also receive them. The host checks
// that every buffer starts 16-byte aligned. A copy that does not complete within
// the wait limit sets DEVICE_ERROR_COPY_WAIT and the CTA returns.
__global__ void DG_PBWD_BOUNDS preprocess_backward_adam_kernel(
    const Camera* __restrict__ camera, float* __restrict__ gaussians, float* __restrict__ sh, uint32_t count,
    const uint32_t* __restrict__ scene_params, const float* __restrict__ radii, const float* __restrict__ splat_grads,
    const AdamParams* __restrict__ adam, float* __restrict__ params, float2* __restrict__ moments,
    float4* __restrict__ stats, float2* __restrict__ aux, float* __restrict__ gaussian_grads,
    float* __restrict__ sh_grads, uint32_t* __restrict__ error) {
  constexpr uint32_t GP = FLOATS_PER_GAUSSIAN + 1;  // a row pitch prime to 32
  __shared__ Camera s_cam;
  __shared__ __align__(16) float s_sh[PBWD_THREADS * SH_REST_FLOATS];  // coefficients, then their gradients
  __shared__ float s_pg[PBWD_THREADS * GP];                            // parameter gradients
  __shared__ AdamParams s_ap;
  __shared__ __align__(8) uint64_t s_bar;
  const uint32_t block_start = blockIdx.x * PBWD_THREADS;
  const uint32_t here = min(PBWD_THREADS, count - block_start);
  const uint32_t sh_total = here * SH_REST_FLOATS;
  float* sh_block = sh + (size_t)block_start * SH_REST_FLOATS;
  const uint32_t quads = sh_total / 4;  // the 16-byte groups (all of a full CTA's 5,760 floats)
  if (threadIdx.x == 0) {
    mbar_init(&s_bar, 1);
    mbar_arrive_expect_tx(&s_bar, quads * 16);
    // Kept in L2 for the Adam pass, which reads the coefficients again.
    bulk_copy_to_shared(s_sh, sh_block, quads * 16, &s_bar, l2_policy_evict_last());
    s_ap = *adam;
  }
  __syncthreads();  // the barrier is initialized before anyone waits on it
  load_camera(s_cam, camera);
  for (uint32_t e = quads * 4 + threadIdx.x; e < sh_total; e += PBWD_THREADS) s_sh[e] = sh_block[e];
  const bool copied = mbar_wait_bounded(&s_bar, 0);
  if (__syncthreads_or(!copied)) {
    if (threadIdx.x == 0) atomicOr(error, DEVICE_ERROR_COPY_WAIT);
    mbar_wait_bounded(&s_bar, 0);  // the copy may still be writing this CTA's shared memory
    return;
  }
  const uint32_t degree = scene_params[0];
  const uint32_t basis_count = (degree + 1u) * (degree + 1u) - 1u;
  const uint32_t i = block_start + threadIdx.x;
  if (i < count) {
    float out[16];
    const float radius = radii[i];
    const float* grads = splat_grads + (size_t)i * SPLAT_GRADS;
    preprocess_backward_one(s_cam, gaussians + (size_t)i * FLOATS_PER_GAUSSIAN, s_sh + threadIdx.x * SH_REST_FLOATS,
                            basis_count, radius, grads, out);
#pragma unroll
    for (int k = 0; k < 16; k++) s_pg[threadIdx.x * GP + k] = out[k];
    if (gaussian_grads) store16(gaussian_grads + (size_t)i * FLOATS_PER_GAUSSIAN, out);
    accumulate_stats_values(s_ap.viewport, radius, grads[0], grads[1], stats, aux, i);
  }
  __syncthreads();
  if (sh_grads) copy_floats(sh_grads + (size_t)block_start * SH_REST_FLOATS, s_sh, sh_total);
  const AdamParams& ap = s_ap;
  const float inv_bc1 = ap.inv_bias_correction1, inv_sqrt_bc2 = ap.inv_sqrt_bias_correction2;
  // The streams below are read and written once: evict them first, so the
  // coefficients staged with evict-last stay in L2 until step 3 reads them again.
  const uint64_t stream = l2_policy_evict_first();

  // 3. The SH slots, four at a time; a thread loads a batch of groups before
  // stepping them, so that enough reads are in flight.
  {
    constexpr uint32_t B = DG_ADAM_SH_QUADS;
    float4* m_block = reinterpret_cast<float4*>(moments + sh_moment_at(count, block_start, 0));
    const float lr = ap.sh_lr;
    for (uint32_t base = threadIdx.x; base < quads; base += PBWD_THREADS * B) {
      float4 v[B], m0[B], m1[B];
#pragma unroll
      for (uint32_t u = 0; u < B; u++) {
        const uint32_t q = base + u * PBWD_THREADS;
        if (q < quads) {
          v[u] = ld_hinted(sh_block + 4 * q, stream);
          m0[u] = ld_hinted(m_block + 2 * q, stream);
          m1[u] = ld_hinted(m_block + 2 * q + 1, stream);
        }
      }
#pragma unroll
      for (uint32_t u = 0; u < B; u++) {
        const uint32_t q = base + u * PBWD_THREADS;
        if (q < quads) {
          const float4 g = f4_load(s_sh + 4 * q);
          float2 a = make_float2(m0[u].x, m0[u].y), b = make_float2(m0[u].z, m0[u].w);
          float2 c = make_float2(m1[u].x, m1[u].y), d = make_float2(m1[u].z, m1[u].w);
          float4 out;
          out.x = adam_step_fast(v[u].x, g.x, a, lr, inv_bc1, inv_sqrt_bc2);
          out.y = adam_step_fast(v[u].y, g.y, b, lr, inv_bc1, inv_sqrt_bc2);
          out.z = adam_step_fast(v[u].z, g.z, c, lr, inv_bc1, inv_sqrt_bc2);
          out.w = adam_step_fast(v[u].w, g.w, d, lr, inv_bc1, inv_sqrt_bc2);
          st_hinted(sh_block + 4 * q, out, stream);
          st_hinted(m_block + 2 * q, make_float4(a.x, a.y, b.x, b.y), stream);
          st_hinted(m_block + 2 * q + 1, make_float4(c.x, c.y, d.x, d.y), stream);
        }
      }
    }
    // The last floats of a partial CTA, one slot at a time.
    float2* m_slots = moments + sh_moment_at(count, block_start, 0);
    for (uint32_t e = quads * 4 + threadIdx.x; e < sh_total; e += PBWD_THREADS) {
      float2 m = m_slots[e];
      sh_block[e] = adam_step_fast(sh_block[e], s_sh[e], m, lr, inv_bc1, inv_sqrt_bc2);
      m_slots[e] = m;
    }
  }

  // 4. The raw parameter slots, a quarter record at a time (PBWD_THREADS is a
  // multiple of 4, so a thread always takes the same quarter of its records).
  {
    constexpr uint32_t B = DG_ADAM_P_QUADS;
    float* p_block = params + (size_t)block_start * FLOATS_PER_GAUSSIAN;
    float* a_block = gaussians + (size_t)block_start * FLOATS_PER_GAUSSIAN;
    float4* m_block = reinterpret_cast<float4*>(moments + param_moment_at(block_start, 0));
    const uint32_t p_quads = here * 4;
    const uint32_t k0 = 4 * (threadIdx.x & 3u);
    for (uint32_t base = threadIdx.x; base < p_quads; base += PBWD_THREADS * B) {
      float4 x[B], m0[B], m1[B];
#pragma unroll
      for (uint32_t u = 0; u < B; u++) {
        const uint32_t q = base + u * PBWD_THREADS;
        if (q < p_quads) {
          x[u] = ld_hinted(p_block + 4 * q, stream);
          m0[u] = ld_hinted(m_block + 2 * q, stream);
          m1[u] = ld_hinted(m_block + 2 * q + 1, stream);
        }
      }
#pragma unroll
      for (uint32_t u = 0; u < B; u++) {
        const uint32_t q = base + u * PBWD_THREADS;
        if (q < p_quads) {
          const float* grad = s_pg + (q >> 2) * GP + k0;
          float xs[4] = {x[u].x, x[u].y, x[u].z, x[u].w};
          float2 ms[4] = {make_float2(m0[u].x, m0[u].y), make_float2(m0[u].z, m0[u].w),
                          make_float2(m1[u].x, m1[u].y), make_float2(m1[u].z, m1[u].w)};
          float act[4];
#pragma unroll
          for (uint32_t j = 0; j < 4; j++) {
            const uint32_t k = k0 + j;
            if (j == 3 && (k == 7 || k == 15)) {
              act[j] = 0.0f;  // a pad: raw value and moments stay as they are
            } else {
              xs[j] = adam_param_slot(ap, k, xs[j], grad[j], ms[j], act[j]);
            }
          }
          st_hinted(p_block + 4 * q, make_float4(xs[0], xs[1], xs[2], xs[3]), stream);
          st_hinted(m_block + 2 * q, make_float4(ms[0].x, ms[0].y, ms[1].x, ms[1].y), stream);
          st_hinted(m_block + 2 * q + 1, make_float4(ms[2].x, ms[2].y, ms[3].x, ms[3].y), stream);
          st_hinted(a_block + 4 * q, make_float4(act[0], act[1], act[2], act[3]), stream);
        }
      }
    }
  }
}


}  // namespace

dg_status launch_rasterize_backward(dg_tile_rasterizer* tr, dg_buffer* pixel_grads, dg_buffer* splat_grads) {
  dg_context* ctx = tr->ctx;
  uint32_t* counter = typed<uint32_t>(tr->work) + 2;
  DG_CUDA(cudaMemsetAsync(counter, 0, sizeof(uint32_t), ctx->stream));
  DG_LAUNCH(ctx, "rasterize_backward",
            rasterize_backward_kernel<<<blend_grid(ctx, (const void*)rasterize_backward_kernel, BWD_THREADS,
                                                    tr->tiles_x * tr->tiles_y * 8u),
                                        BWD_THREADS, 0, ctx->stream>>>(
                typed<const Camera>(tr->camera), typed<float4>(tr->raster_params), typed<float>(tr->splats),
                typed<uint32_t>(tr->values), typed<uint2>(tr->ranges), typed<uint32_t>(tr->work_plan),
                typed<uint2>(tr->chunks), typed<float4>(tr->pixel_color), typed<uint32_t>(tr->pixel_last),
                typed<float4>(tr->checkpoints), typed<uint32_t>(tr->blend_mask), typed<float4>(pixel_grads),
                typed<float>(splat_grads), counter, tr->splat_cutoffs));
  return DG_OK;
}

dg_status launch_preprocess_backward_adam(dg_renderer* r, const AdamParams* adam, float* params, float2* moments,
                                         float4* stats, float2* aux, bool keep_gradients) {
  // Every stream of the kernel moves 16-byte groups from the start of each buffer.
  const void* starts[] = {params, moments, ptr_of(r->gaussians), ptr_of(r->sh)};
  for (const void* p : starts)
    DG_REQUIRE((reinterpret_cast<uintptr_t>(p) & 15) == 0, "the training buffers must start 16-byte aligned");
  DG_LAUNCH(r->ctx, "preprocess_backward_adam",
            preprocess_backward_adam_kernel<<<ceil_div(r->count, PBWD_THREADS), PBWD_THREADS, 0, r->ctx->stream>>>(
                typed<const Camera>(r->camera), typed<float>(r->gaussians), typed<float>(r->sh), r->count,
                typed<uint32_t>(r->scene_params), typed<float>(r->radii), typed<float>(r->grad_splats), adam, params,
                moments, stats, aux, keep_gradients ? typed<float>(r->grad_gaussians) : nullptr,
                keep_gradients ? typed<float>(r->grad_sh) : nullptr, r->ctx->device_error));
  return DG_OK;
}

dg_status launch_preprocess_backward(dg_renderer* r) {
  DG_LAUNCH(r->ctx, "preprocess_backward",
            preprocess_backward_kernel<<<ceil_div(r->count, PBWD_THREADS), PBWD_THREADS, 0, r->ctx->stream>>>(
                typed<const Camera>(r->camera), typed<float>(r->gaussians), typed<float>(r->sh), r->count,
                typed<uint32_t>(r->scene_params), typed<float>(r->splats), typed<float>(r->grad_splats),
                typed<float>(r->grad_gaussians), typed<float>(r->grad_sh)));
  return DG_OK;
}

}  // namespace dg

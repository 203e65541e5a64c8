// The renderer: preprocess (src/shaders/preprocess.wgsl), the tile stage
// (src/shaders/tiles.wgsl), the forward blend (src/shaders/rasterize.wgsl) and
// both backward passes (src/shaders/rasterizeBackward.wgsl,
// src/shaders/preprocessBackward.wgsl), behind the TileRasterizer and
// GaussianRenderer objects of src/tileRasterizer.ts and src/gaussianRenderer.ts.
//
// Compiled with --fmad=false (see dg_render_kernels.cuh).
#include "dg_render.cuh"
#include "dg_render_kernels.cuh"

#include <algorithm>

namespace dg {
namespace {

#ifndef DG_PRE_THREADS
#define DG_PRE_THREADS 128
#endif
constexpr int PRE_THREADS = DG_PRE_THREADS;  // 64 and 96 measured slower (84.8, 88.8 us against 75.8 at 1.1M)
constexpr int DUP_THREADS = 256;
constexpr int RANGE_THREADS = 256;

__device__ __forceinline__ void load_camera(Camera& dst, const Camera* src) {
  const float* s = reinterpret_cast<const float*>(src);
  float* d = reinterpret_cast<float*>(&dst);
  for (int k = threadIdx.x; k < 36; k += blockDim.x) d[k] = s[k];
}

// ------------------------------------------------------------------ preprocess
// src/shaders/preprocess.wgsl:21-88 for one Gaussian g (16 activated floats)
// seen by camera cam, its SH coefficients at shv: writes the 48-byte splat to out
// (zeros when culled) and returns the tiles it touches
// (src/shaders/tiles.wgsl:24-35; blend tiles of 2^twl x 2^thl tiles for a batch
// of views) and its depth's bits (0 when culled).
struct Projected {
  uint32_t tiles, depth_bits;
  float radius;  // 0 when culled
};

__device__ __forceinline__ Projected preprocess_one(const Camera& cam, const float (&g)[16], const float* shv,
                                                    uint32_t basis_count, float4* __restrict__ out,
                                                    uint32_t twl = 0, uint32_t thl = 0) {
  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
  auto culled = [&]() {
    out[0] = zero;
    out[1] = zero;
    out[2] = zero;
    return Projected{0u, 0u, 0.0f};
  };
  if (-view_z(cam, g) <= 0.2f) return culled();
  Projection p;
  project(cam, g, p);
  if (p.det <= 0.0f) return culled();
  const float mid = 0.5f * (p.a + p.c);
  const float lambda = mid + sqrtf(fmaxf(0.1f, mid * mid - p.det));
  const float radius = ceilf(3.0f * sqrtf(lambda));
  float clip[4];
#pragma unroll
  for (int row = 0; row < 4; row++) {
    float v = cam.proj[0 * 4 + row] * p.t[0];
    v = v + cam.proj[1 * 4 + row] * p.t[1];
    v = v + cam.proj[2 * 4 + row] * p.t[2];
    v = v + cam.proj[3 * 4 + row] * 1.0f;
    clip[row] = v;
  }
  const float vpx = cam.viewport[0], vpy = cam.viewport[1];
  const float mx = (clip[0] / clip[3] * 0.5f + 0.5f) * vpx;
  const float my = (clip[1] / clip[3] * -0.5f + 0.5f) * vpy;
  if (mx + radius < 0.0f || my + radius < 0.0f || mx - radius > vpx || my - radius > vpy) return culled();
  float color[3] = {g[12], g[13], g[14]};
  if (basis_count > 0) {
    float campos[3], off[3], dir[3], basis[15];
    camera_position(cam, campos);
    off[0] = g[0] - campos[0];
    off[1] = g[1] - campos[1];
    off[2] = g[2] - campos[2];
    normalize3(off, dir);
    sh_basis(dir, basis);
    // Unrolled over all 15 terms (the ones past basis_count skipped), so the
    // basis stays in registers; the sums run in the same order as a loop to
    // basis_count.
#pragma unroll
    for (uint32_t k = 0; k < 15; k++) {
      if (k < basis_count) {
        color[0] = color[0] + basis[k] * shv[k * 3 + 0];
        color[1] = color[1] + basis[k] * shv[k * 3 + 1];
        color[2] = color[2] + basis[k] * shv[k * 3 + 2];
      }
    }
  }
  out[0] = make_float4(mx, my, p.depth, radius);
  out[1] = make_float4(p.c / p.det, -p.b / p.det, p.a / p.det, blend_cutoff(g[3]));
  out[2] = make_float4(fmaxf(color[0], 0.0f), fmaxf(color[1], 0.0f), fmaxf(color[2], 0.0f), g[3]);
  const uint4 rect = blend_rect(tile_rect(mx, my, radius, tile_grid(cam)), twl, thl);
  return Projected{(rect.z - rect.x) * (rect.w - rect.y), __float_as_uint(p.depth), radius};
}

// Stages the SH coefficients of Gaussians [first, first + n) into shared memory
// with coalesced loads (45 floats per Gaussian; the odd stride makes the
// per-thread reads conflict-free). All threads of the CTA take part.
__device__ __forceinline__ void stage_sh(float* s_sh, const float* __restrict__ sh, uint32_t first, uint32_t n) {
  stage_floats_async(s_sh, sh + (size_t)first * SH_REST_FLOATS, n * SH_REST_FLOATS);
  cp_async_wait_all();
}

__device__ __forceinline__ void load_gaussian(const float* __restrict__ gaussians, uint32_t i, float (&g)[16]) {
  const float4* gp = reinterpret_cast<const float4*>(gaussians + (size_t)i * FLOATS_PER_GAUSSIAN);
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const float4 q = gp[k];
    g[4 * k] = q.x;
    g[4 * k + 1] = q.y;
    g[4 * k + 2] = q.z;
    g[4 * k + 3] = q.w;
  }
}

// One thread per Gaussian, one view. When tile_counts is given, the tiles each
// splat touches are written too (src/shaders/tiles.wgsl:24-35, fused); when
// depth_keys is given, the depth's bits (0 when culled) and the splat's index,
// the input of the depth sort; when radii is given, each splat's radius densely
// (the training step's fused backward reads it there, not from the 48-byte
// splat records).
//
// Persistent CTAs over blocks of PRE_THREADS Gaussians: while a CTA projects one
// block, the next block's SH coefficients are already copying into the other
// half of s_sh (cp.async) and its Gaussian records loading into registers, so
// the loads of one block wait behind the arithmetic of the previous one instead
// of in front of it.
__global__ void __launch_bounds__(PRE_THREADS) preprocess_kernel(const Camera* __restrict__ camera,
                                                                 const float* __restrict__ gaussians,
                                                                 const float* __restrict__ sh, uint32_t count,
                                                                 const uint32_t* __restrict__ scene_params,
                                                                 float* __restrict__ splats,
                                                                 uint32_t* __restrict__ tile_counts,
                                                                 uint32_t* __restrict__ depth_keys,
                                                                 uint32_t* __restrict__ depth_order,
                                                                 float* __restrict__ radii) {
  __shared__ Camera s_cam;
  __shared__ __align__(16) float s_sh[2][PRE_THREADS * SH_REST_FLOATS];
  load_camera(s_cam, camera);
  const uint32_t degree = scene_params[0];
  const uint32_t basis_count = (degree + 1u) * (degree + 1u) - 1u;
  const uint32_t blocks = (count + PRE_THREADS - 1) / PRE_THREADS;
  const uint32_t mine = blockIdx.x < blocks ? (blocks - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  auto first_of = [&](uint32_t step) { return (blockIdx.x + step * gridDim.x) * PRE_THREADS; };
  // Starts block `step`'s SH copy; threads past the end load the last record.
  auto fetch = [&](uint32_t step, float (&g)[16]) {
    const uint32_t first = first_of(step);
    if (basis_count > 0)
      stage_floats_async(s_sh[step & 1], sh + (size_t)first * SH_REST_FLOATS,
                         min((uint32_t)PRE_THREADS, count - first) * SH_REST_FLOATS);
    load_gaussian(gaussians, min(first + threadIdx.x, count - 1u), g);
  };
  float g[16];
  if (mine > 0) fetch(0, g);
  for (uint32_t step = 0; step < mine; step++) {
    cp_async_wait_all();
    __syncthreads();  // this block's SH is in; every thread is done with the block before last
    float next[16];
    if (step + 1 < mine) fetch(step + 1, next);
    const uint32_t i = first_of(step) + threadIdx.x;
    if (i < count) {
      const Projected pr = preprocess_one(s_cam, g, s_sh[step & 1] + threadIdx.x * SH_REST_FLOATS, basis_count,
                                          reinterpret_cast<float4*>(splats + (size_t)i * FLOATS_PER_SPLAT));
      if (tile_counts) tile_counts[i] = pr.tiles;
      if (depth_keys) depth_keys[i] = pr.depth_bits;
      if (depth_order) depth_order[i] = i;
      if (radii) radii[i] = pr.radius;
    }
    if (step + 1 < mine) {
#pragma unroll
      for (int k = 0; k < 16; k++) g[k] = next[k];
    }
  }
}

// CTAs of preprocess_kernel that fit on the device at once (its grid).
uint32_t preprocess_grid(const dg_context* ctx, uint32_t count) {
  // Queried once per process (a function-local static initializes thread-safely).
  static const int per_sm = [] {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, preprocess_kernel, PRE_THREADS, 0) != cudaSuccess) n = 1;
    return std::max(1, n);
  }();
  const uint32_t blocks = std::max(1u, ceil_div(count, PRE_THREADS));
  return std::min(blocks, (uint32_t)per_sm * (uint32_t)ctx->sm_count);
}

// The same for a batch of views sharing one viewport: each CTA stages its
// Gaussians and their SH coefficients once and projects them into every view.
// Splat (view v, Gaussian i) is number v * count + i; its depth-sort key puts
// the view above the depth's bits, so one sort orders every view by depth.
__global__ void __launch_bounds__(PRE_THREADS) preprocess_views_kernel(
    const Camera* __restrict__ cameras, uint32_t views, const float* __restrict__ gaussians,
    const float* __restrict__ sh, uint32_t count, const uint32_t* __restrict__ scene_params,
    float* __restrict__ splats, uint32_t* __restrict__ tile_counts, uint2* __restrict__ depth_keys,
    uint32_t* __restrict__ depth_order, uint32_t twl, uint32_t thl) {
  __shared__ float s_sh[PRE_THREADS * SH_REST_FLOATS];
  const uint32_t degree = scene_params[0];
  const uint32_t basis_count = (degree + 1u) * (degree + 1u) - 1u;
  const uint32_t block_start = blockIdx.x * PRE_THREADS;
  if (basis_count > 0) stage_sh(s_sh, sh, block_start, min((uint32_t)PRE_THREADS, count - block_start));
  __syncthreads();
  const uint32_t i = block_start + threadIdx.x;
  if (i >= count) return;
  float g[16];
  load_gaussian(gaussians, i, g);
  for (uint32_t v = 0; v < views; v++) {
    const size_t at = (size_t)v * count + i;
    const Projected pr = preprocess_one(cameras[v], g, s_sh + threadIdx.x * SH_REST_FLOATS, basis_count,
                                        reinterpret_cast<float4*>(splats + at * FLOATS_PER_SPLAT), twl, thl);
    tile_counts[at] = pr.tiles;
    depth_keys[at] = make_uint2(pr.depth_bits, v);
    depth_order[at] = (uint32_t)at;
  }
}

// The depth-first tile sort (the renderer's path). The reference sorts 64-bit
// (tile, depth) keys (src/shaders/tiles.wgsl:37-60, src/radixSort.ts:101-104).
// Here the splats are first sorted by depth alone (stable, so equal depths keep
// index order), their pairs are then emitted in that order, and a stable sort on
// the 16-bit tile index finishes the job. Within a tile the pairs end up by depth
// with ties by splat index: exactly the reference's order, from sorting N 32-bit
// keys plus K 16-bit ones instead of K 48-bit ones.

// Enough CTAs of `threads` to keep every SM busy in a grid-stride loop over n
// items (at most one CTA per `threads` items).
inline uint32_t stride_grid(const dg_context* ctx, uint64_t n, uint32_t threads) {
  return std::max(1u, std::min(ceil_div(n, threads), (uint32_t)ctx->sm_count * 8u));
}

// duplicate_kernel's warp-cooperative emission over splats in depth order: the
// pairs of 32 consecutive sorted splats are one contiguous run of slots. Keys are
// the tile index alone (u32), values the splat index. For a batch of views
// (splat v * per_view + i is Gaussian i in view v), the key of a tile of view v
// is v << view_shift | its tile index within the view; the tiles are blend tiles
// of 2^twl x 2^thl 16x16 tiles (1 x 1 outside batches of views).
__global__ void __launch_bounds__(DUP_THREADS) duplicate_sorted_kernel(const Camera* __restrict__ camera,
                                                                       const float* __restrict__ splats,
                                                                       const uint32_t* __restrict__ order,
                                                                       const uint32_t* __restrict__ offsets,
                                                                       uint32_t count, uint32_t per_view,
                                                                       uint32_t view_shift, uint32_t capacity,
                                                                       uint32_t* __restrict__ keys,
                                                                       uint32_t* __restrict__ values, uint32_t twl,
                                                                       uint32_t thl) {
  __shared__ uint32_t s_excl[DUP_THREADS];
  __shared__ uint32_t s_w[DUP_THREADS];       // the splat's tile rectangle's width
  __shared__ float s_inv[DUP_THREADS];        // 1 / width
  __shared__ uint32_t s_index[DUP_THREADS];
  __shared__ uint32_t s_corner[DUP_THREADS];  // the key of its rectangle's first tile
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t j = blockIdx.x * DUP_THREADS + threadIdx.x;
  const uint32_t first = blockIdx.x * DUP_THREADS + warp * 32;
  if (first >= count) return;  // warp-uniform
  const Camera& cam = *camera;
  const uint2 tiles16 = tile_grid(cam);
  const uint2 tiles = make_uint2(blend_tiles_along(tiles16.x, twl), blend_tiles_along(tiles16.y, thl));
  uint32_t n = 0, index = 0;
  uint4 rect = make_uint4(0, 0, 0, 0);
  if (j < count) {
    index = order[j];
    const float4 s = reinterpret_cast<const float4*>(splats + (size_t)index * FLOATS_PER_SPLAT)[0];
    if (s.w != 0.0f) {
      rect = blend_rect(tile_rect(s.x, s.y, s.w, tiles16), twl, thl);
      n = (rect.z - rect.x) * (rect.w - rect.y);
    }
  }
  uint32_t incl = n;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t v = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += v;
  }
  const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
  const uint32_t slot0 = offsets[first];
  uint32_t* excl = s_excl + warp * 32;
  excl[lane] = incl - n;
  const uint32_t view = per_view >= count ? 0u : index / per_view;  // one view: no division
  const uint32_t rw = rect.z - rect.x;
  s_w[threadIdx.x] = rw;
  s_inv[threadIdx.x] = rw ? 1.0f / (float)rw : 0.0f;
  s_index[threadIdx.x] = index;
  s_corner[threadIdx.x] = (view << view_shift) + rect.y * tiles.x + rect.x;
  __syncwarp();
  for (uint32_t k = lane; k < total; k += 32) {
    int lo = 0;
#pragma unroll
    for (int step = 16; step > 0; step >>= 1)
      if (excl[lo + step] <= k) lo += step;
    const int src = warp * 32 + lo;
    // The pair's row and column in the splat's rectangle: local / w and local % w
    // by a float reciprocal, whose quotient (local < 2^22) is off by at most one,
    // then corrected from the remainder; exact.
    const uint32_t local = k - excl[lo];
    const int32_t w = (int32_t)s_w[src];
    int32_t q = (int32_t)((float)local * s_inv[src]);
    int32_t r = (int32_t)local - q * w;
    if (r < 0) {
      q -= 1;
      r += w;
    } else if (r >= w) {
      q += 1;
      r -= w;
    }
    const uint32_t slot = slot0 + k;
    if (slot < capacity) {
      keys[slot] = s_corner[src] + (uint32_t)q * tiles.x + (uint32_t)r;
      values[slot] = s_index[src];
    }
  }
}

// The reference's sorted 64-bit keys (tile << 32 | depth bits), rebuilt from the
// depth-first path's tile keys and splats, for inspection.
__global__ void materialize_keys_kernel(const uint32_t* __restrict__ tile_keys, const uint32_t* __restrict__ values,
                                        const float* __restrict__ splats, const uint32_t* __restrict__ pair_total,
                                        uint32_t capacity, uint64_t* __restrict__ out) {
  const uint32_t n = min(pair_total[0], capacity);
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t depth_bits = __float_as_uint(splats[(size_t)values[k] * FLOATS_PER_SPLAT + 2]);
  out[k] = ((uint64_t)tile_keys[k] << 32) | depth_bits;
}

// src/shaders/tiles.wgsl:24-35 (for splats the renderer did not preprocess).
__global__ void count_tiles_kernel(const Camera* __restrict__ camera, const float* __restrict__ splats, uint32_t count,
                                   uint32_t* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const Camera& cam = *camera;
  const float4 s = reinterpret_cast<const float4*>(splats + (size_t)i * FLOATS_PER_SPLAT)[0];
  uint32_t touched = 0;
  if (s.w > 0.0f) {
    uint4 rect = tile_rect(s.x, s.y, s.w, tile_grid(cam));
    touched = (rect.z - rect.x) * (rect.w - rect.y);
  }
  out[i] = touched;
}

// src/shaders/tiles.wgsl:37-60. Each warp writes the pairs of its 32 splats
// together: those occupy one contiguous run of slots (the scan put them there),
// so every lane writes the next slot of the run and the stores coalesce. A pair
// is (key = tile << 32 | depth bits, value = splat index), dropped past capacity.
__global__ void __launch_bounds__(DUP_THREADS) duplicate_kernel(const Camera* __restrict__ camera,
                                                                const float* __restrict__ splats,
                                                                const uint32_t* __restrict__ offsets, uint32_t count,
                                                                uint32_t capacity, uint64_t* __restrict__ keys,
                                                                uint32_t* __restrict__ values) {
  __shared__ uint32_t s_excl[DUP_THREADS];
  __shared__ uint32_t s_x0[DUP_THREADS];
  __shared__ uint32_t s_y0[DUP_THREADS];
  __shared__ uint32_t s_w[DUP_THREADS];
  __shared__ uint32_t s_depth[DUP_THREADS];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t i = blockIdx.x * DUP_THREADS + threadIdx.x;
  const uint32_t first = blockIdx.x * DUP_THREADS + warp * 32;
  if (first >= count) return;  // warp-uniform
  const Camera& cam = *camera;
  const uint2 tiles = tile_grid(cam);
  uint32_t n = 0;
  uint4 rect = make_uint4(0, 0, 0, 0);
  uint32_t depth_bits = 0;
  if (i < count) {
    const float4 s = reinterpret_cast<const float4*>(splats + (size_t)i * FLOATS_PER_SPLAT)[0];
    if (s.w != 0.0f) {
      rect = tile_rect(s.x, s.y, s.w, tiles);
      n = (rect.z - rect.x) * (rect.w - rect.y);
      depth_bits = __float_as_uint(s.z);
    }
  }
  uint32_t incl = n;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    uint32_t v = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += v;
  }
  const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
  const uint32_t slot0 = offsets[first];
  uint32_t* excl = s_excl + warp * 32;
  excl[lane] = incl - n;
  s_x0[threadIdx.x] = rect.x;
  s_y0[threadIdx.x] = rect.y;
  s_w[threadIdx.x] = rect.z - rect.x;
  s_depth[threadIdx.x] = depth_bits;
  __syncwarp();
  for (uint32_t k = lane; k < total; k += 32) {
    // The last lane whose run starts at or before k owns pair k.
    int lo = 0;
#pragma unroll
    for (int step = 16; step > 0; step >>= 1)
      if (excl[lo + step] <= k) lo += step;
    const int src = warp * 32 + lo;
    const uint32_t local = k - excl[lo];
    const uint32_t w = s_w[src];
    const uint32_t y = s_y0[src] + local / w;
    const uint32_t x = s_x0[src] + local % w;
    const uint32_t slot = slot0 + k;
    if (slot < capacity) {
      keys[slot] = ((uint64_t)(y * tiles.x + x) << 32) | s_depth[src];
      values[slot] = first + lo;
    }
  }
}

// src/shaders/tiles.wgsl:65-84. The tile index is word STRIDE - 1 of each key:
// the high word of the reference's 64-bit keys, or the whole u32 key of the
// depth-first path.
template <int STRIDE>
__global__ void __launch_bounds__(RANGE_THREADS) find_ranges_kernel(const uint32_t* __restrict__ key_words,
                                                                    const uint32_t* __restrict__ pair_total,
                                                                    uint32_t capacity, uint32_t tiles,
                                                                    uint32_t view_shift, uint32_t tiles_per_view,
                                                                    uint2* __restrict__ ranges) {
  const uint32_t n = min(pair_total[0], capacity);
  // A key's tile: view * tiles_per_view + local tile for a batch of views keyed
  // view << view_shift | local tile; the key itself when view_shift is 0 and
  // tiles_per_view 1.
  const uint32_t local_mask = (1u << view_shift) - 1u;
  auto tile_of = [&](uint32_t key) { return (key >> view_shift) * tiles_per_view + (key & local_mask); };
  // Pair i with key `key` after pair i - 1 with key `prev_key` (none for i = 0).
  auto edge = [&](uint32_t i, uint32_t key, uint32_t prev_key) {
    const uint32_t tile = tile_of(key), prev = i ? tile_of(prev_key) : ~0u;
    if (tile >= tiles) return;  // only possible after a sort whose bounded wait gave up
    if (tile != prev) {
      if (i > 0 && prev < tiles) ranges[prev].y = i;
      ranges[tile].x = i;
    }
    if (i == n - 1) ranges[tile].y = n;
  };
  // A grid-stride loop over a few CTAs per SM (one thread per pair would spend
  // more on launching tens of thousands of tiny CTAs than on the pairs); u32 keys
  // come four at a time.
  const uint32_t stride = gridDim.x * RANGE_THREADS, first = blockIdx.x * RANGE_THREADS + threadIdx.x;
  if constexpr (STRIDE == 1) {
    const uint32_t quads = n / 4;
    for (uint32_t q = first; q < quads; q += stride) {
      const uint4 k = reinterpret_cast<const uint4*>(key_words)[q];
      const uint32_t i = 4 * q;
      edge(i, k.x, i ? key_words[i - 1] : 0u);
      edge(i + 1, k.y, k.x);
      edge(i + 2, k.z, k.y);
      edge(i + 3, k.w, k.z);
    }
    for (uint32_t i = 4 * quads + first; i < n; i += stride) edge(i, key_words[i], i ? key_words[i - 1] : 0u);
  } else {
    for (uint32_t i = first; i < n; i += stride)
      edge(i, key_words[STRIDE * (size_t)i + (STRIDE - 1)],
           i ? key_words[STRIDE * (size_t)(i - 1) + (STRIDE - 1)] : 0u);
  }
}

__device__ __forceinline__ unsigned char to_unorm8(float v) {
  return (unsigned char)__float2uint_rn(clampf(v, 0.0f, 1.0f) * 255.0f);
}

// ------------------------------------------------------------------ work plan
// Orders the frame's blend work; one CTA. The forward pass takes tiles with more
// than coop_min entries first, longest first by powers of two, then the rest; the
// backward pass (when chunks is given) takes the (tile, chunk) pairs of tiles
// with several chunks first. Order within a group follows atomics and does not
// change any result.
constexpr uint32_t PLAN_THREADS = 1024;

__global__ void __launch_bounds__(PLAN_THREADS) plan_kernel(const uint2* __restrict__ ranges, uint32_t tiles,
                                                            uint32_t coop_min, uint32_t* __restrict__ plan,
                                                            uint2* __restrict__ chunks) {
  __shared__ uint32_t s_bucket[32];  // cooperative tiles by floor(log2(length)); then write cursors
  __shared__ uint32_t s_light, s_multi, s_single;
  const uint32_t tid = threadIdx.x;
  if (tid < 32) s_bucket[tid] = 0;
  if (tid == 0) s_multi = 0;
  __syncthreads();
  for (uint32_t t = tid; t < tiles; t += PLAN_THREADS) {
    const uint2 r = ranges[t];
    const uint32_t len = r.y - r.x;
    if (len > coop_min) atomicAdd(&s_bucket[31 - __clz(len)], 1u);
    const uint32_t nb = (len + CHUNK - 1) / CHUNK;
    if (nb > 1) atomicAdd(&s_multi, nb);
  }
  __syncthreads();
  if (tid == 0) {
    uint32_t at = 0;
    for (int k = 31; k >= 0; k--) {
      const uint32_t c = s_bucket[k];
      s_bucket[k] = at;
      at += c;
    }
    plan[0] = at;
    plan[1] = tiles;
    s_light = at;
    s_single = s_multi;
    s_multi = 0;
  }
  __syncthreads();
  uint32_t* order = plan + PLAN_HEADER;
  for (uint32_t t = tid; t < tiles; t += PLAN_THREADS) {
    const uint2 r = ranges[t];
    const uint32_t len = r.y - r.x;
    order[len > coop_min ? atomicAdd(&s_bucket[31 - __clz(len)], 1u) : atomicAdd(&s_light, 1u)] = t;
    if (!chunks) continue;
    const uint32_t nb = (len + CHUNK - 1) / CHUNK;
    if (nb > 1) {
      const uint32_t at = atomicAdd(&s_multi, nb);
      for (uint32_t k = 0; k < nb; k++) chunks[at + k] = make_uint2(t, k);
    } else if (nb == 1) {
      chunks[atomicAdd(&s_single, 1u)] = make_uint2(t, 0u);
    }
  }
  __syncthreads();
  if (tid == 0) {
    plan[2] = s_single;
    plan[3] = 0;
  }
}

// Writes the checkpoints of boundaries [k_from, k_to) of a tile with one pixel state.
__device__ __forceinline__ void save_checkpoints(float4* __restrict__ checkpoints, uint32_t run_x, uint32_t k_from,
                                                 uint32_t k_to, uint32_t block, uint32_t lane, float T, float r,
                                                 float g, float b) {
  if (!checkpoints) return;
  for (uint32_t k = k_from; k < k_to; k++) checkpoints[checkpoint_at(run_x, k, block, lane)] = make_float4(T, r, g, b);
}

// One pixel's front-to-back blend (src/shaders/rasterize.wgsl:62-92), the lane's
// pixel of a warp's 8x4 block.
struct PixelBlend {
  float cx, cy;
  float T, r, g, b;
  uint32_t last;
  bool done;

  // The alphas of up to 4 staged entries e[0..n) of `st` at this pixel, 0 where
  // the pixel does not blend the splat (alpha under 1/255; a power under the
  // splat's cutoff skips the exp with the same outcome). Computed together:
  // independent work the SM can overlap. Returns false, with all alphas 0, when
  // no lane reaches any of the 4 cutoffs.
  __device__ __forceinline__ bool alphas4(const WarpStage& st, const uint32_t (&e)[4], uint32_t n, bool active,
                                          float (&alpha)[4]) const {
    float power[4], opacity[4];
    bool need[4], any = false;
#pragma unroll
    for (uint32_t u = 0; u < 4; u++) {
      const float4 m = st.mean[e[u]];
      const float4 q = st.quad[e[u]];
      power[u] = blend_power(q.x, q.y, q.z, cx - m.x, cy - m.y);
      opacity[u] = m.z;
      need[u] = active && u < n && power[u] >= q.w && power[u] <= 0.0f;
      any |= need[u];
    }
    if (!__any_sync(0xffffffffu, any)) {
#pragma unroll
      for (uint32_t u = 0; u < 4; u++) alpha[u] = 0.0f;
      return false;
    }
    float G[4];
    exp_blend_core2(need[0] ? power[0] : 0.0f, need[1] ? power[1] : 0.0f, G[0], G[1]);
    exp_blend_core2(need[2] ? power[2] : 0.0f, need[3] ? power[3] : 0.0f, G[2], G[3]);
#pragma unroll
    for (uint32_t u = 0; u < 4; u++) {
      const float a = fminf(0.99f, opacity[u] * G[u]);
      alpha[u] = need[u] && a >= 1.0f / 255.0f ? a : 0.0f;
    }
    return true;
  }

  // Blends one splat of alpha `alpha` (0: not blended here) and colour c whose
  // 1-based list position is pos1; stops before the splat that would take the
  // transmittance below 1e-4 (src/shaders/rasterize.wgsl:62-92). Without
  // branches: a splat the pixel does not take adds c * 0 (colours are
  // non-negative, so the sums do not change) and keeps T and last. While the pixel
  // runs T >= 1e-4, so alpha 0 (remaining = T) never stops it.
  __device__ __forceinline__ void blend(float alpha, float4 c, uint32_t pos1) {
    const float remaining = T * (1.0f - alpha);
    done = done || remaining < 0.0001f;
    const bool take = !done && alpha != 0.0f;
    // color += c alpha T (src/shaders/rasterize.wgsl:88) as c (alpha T) + color,
    // one fused multiply-add per channel (the oracle's same sequence).
    const float w = take ? __fmul_rn(alpha, T) : 0.0f;
    r = __fmaf_rn(c.x, w, r);
    g = __fmaf_rn(c.y, w, g);
    b = __fmaf_rn(c.z, w, b);
    T = take ? remaining : T;
    last = take ? pos1 : last;
  }

  // Applies up to 4 staged entries e[0..n) of `st` in list order. Sets bit
  // (position - base) of `blended` for each entry with a nonzero alpha at some
  // pixel of the warp that had not stopped: every entry a pixel blends, and at
  // most a last one it stopped at.
  __device__ __forceinline__ void apply4(const WarpStage& st, const uint32_t (&e)[4], uint32_t n, uint32_t base,
                                         uint32_t& blended) {
    float alpha[4];
    if (!alphas4(st, e, n, !done, alpha)) return;
    const uint32_t mine = (alpha[0] != 0.0f ? 1u : 0u) | (alpha[1] != 0.0f ? 2u : 0u) |
                          (alpha[2] != 0.0f ? 4u : 0u) | (alpha[3] != 0.0f ? 8u : 0u);
    const uint32_t any = __reduce_or_sync(0xffffffffu, mine);
#pragma unroll
    for (uint32_t u = 0; u < 4; u++) {
      if ((any >> u) & 1u) {  // the same on every lane
        const uint32_t pos = st.pos[e[u]];
        blended |= 1u << (pos - base);
        blend(alpha[u], st.color[e[u]], pos + 1);
      }
    }
  }
};

// The blend mask: bit p % 32 of word (p / 32) * 8 + block is set when some pixel
// of 8x4 block `block` of the tile holding pair p blended that pair's splat. The
// forward pass sets the bits, the backward pass walks only those entries. Both
// helpers take the 32 bits of positions [p0, p0 + 32) of the pair list.
__device__ __forceinline__ void publish_blended(uint32_t* __restrict__ mask, uint32_t p0, uint32_t block,
                                                uint32_t bits) {
  if (bits == 0 || !mask) return;
  const uint32_t w = p0 >> 5, shift = p0 & 31u;
  const uint32_t lo = bits << shift, hi = shift ? bits >> (32u - shift) : 0u;
  if (lo) atomicOr(&mask[(size_t)w * 8u + block], lo);
  if (hi) atomicOr(&mask[(size_t)(w + 1) * 8u + block], hi);
}

// The geometry of a blend item: tile `tile` (of the view tile / tiles_per_view
// when several views are blended together), 8x4 block `block`, this lane's pixel.
// A blend tile of 2^twl x 2^thl 16x16 tiles has 8 blocks per 16x16 tile, those
// of its 16x16 tile k numbered 8k to 8k + 7 (k row-major within the blend tile).
struct BlendItem {
  uint32_t px, py;
  size_t pixel;  // index in the views' stacked pixel buffers
  bool inside;
  float x0, y0;  // the block's first pixel center
  uint2 run;
  uint32_t tx, ty;  // the block's 16x16 tile
  __device__ __forceinline__ BlendItem(uint32_t tile, uint32_t block, uint32_t lane, uint32_t tiles_x,
                                       uint32_t tiles_per_view, float vpx, float vpy, const uint2* __restrict__ ranges,
                                       uint32_t twl = 0, uint32_t thl = 0) {
    const uint32_t view = tile / tiles_per_view, local = tile - view * tiles_per_view;
    const uint32_t blend_x = blend_tiles_along(tiles_x, twl), sub = block >> 3;
    tx = ((local % blend_x) << twl) + (sub & ((1u << twl) - 1u));
    ty = ((local / blend_x) << thl) + (sub >> twl);
    const uint32_t bx = tx * TILE + (block & 1u) * 8u, by = ty * TILE + ((block >> 1) & 3u) * 4u;
    px = bx + (lane & 7u);
    py = by + (lane >> 3);
    inside = (float)px < vpx && (float)py < vpy;
    const uint32_t width = (uint32_t)vpx, height = (uint32_t)vpy;
    pixel = (size_t)view * width * height + (size_t)py * width + px;
    x0 = (float)bx + 0.5f;
    y0 = (float)by + 0.5f;
    run = ranges[tile];
  }
};

__device__ __forceinline__ void write_pixel(const BlendItem& it, const PixelBlend& pb, float4 bg,
                                            uchar4* __restrict__ target, float4* __restrict__ pixel_color,
                                            uint32_t* __restrict__ pixel_last) {
  if (!it.inside) return;
  const float fr = pb.r + pb.T * bg.x, fg = pb.g + pb.T * bg.y, fb = pb.b + pb.T * bg.z;
  pixel_color[it.pixel] = make_float4(fr, fg, fb, pb.T);
  pixel_last[it.pixel] = pb.last;
  if (target) target[it.pixel] = make_uchar4(to_unorm8(fr), to_unorm8(fg), to_unorm8(fb), 255);
}

// src/shaders/rasterize.wgsl:32-100. The work is split into items, one per (tile,
// 8x4 pixel block): 8 per 16x16 tile, taken from counters by persistent CTAs and
// warps in the plan's order. With blend tiles of 2^TWL x 2^THL 16x16 tiles (a
// batch of views only: no checkpoints or blend mask), each block keeps only its
// own 16x16 tile's entries of the blend tile's list. Whatever the split, each pixel blends the tile's list
// front to back exactly as the plain loop over every entry does, so results are
// bit-identical to it; the split only decides who does the work:
//
// - Tiles with more entries than the plan's threshold (COOP_MIN unless tuned)
//   come first, each block blended by a whole CTA. Three of its warps take
//   consecutive 32-entry windows, keep the splats that can reach the block and
//   compute their alphas at the block's pixels, queueing those some pixel blends;
//   warp 0 applies the queues in list order one round behind, so the alphas of the
//   next 96 entries are computed while it blends. The costly part of each splat
//   (power, exp, alpha) is spread over the CTA; only the short transmittance update
//   stays serial, and it overlaps the rest.
// - Every warp then takes the other blocks on its own, walking the list 32
//   entries at a time.
//
// In both, a window's splat records are copied into shared memory while the
// previous one blends, a splat rejected for the block has alpha below 1/255 at
// all of its pixels, and a power under the splat's cutoff skips the exp: none of
// these changes a result. The pixel state at each CHUNK boundary of the list is
// saved for the backward pass, and which entries each block blended.
template <uint32_t TWL, uint32_t THL>
__global__ void __launch_bounds__(FWD_THREADS) rasterize_kernel(
    const Camera* __restrict__ camera, const float4* __restrict__ raster_params, const float* __restrict__ splats,
    const uint32_t* __restrict__ pair_splats, const uint2* __restrict__ ranges, const uint32_t* __restrict__ plan,
    uint32_t tiles_per_view, uchar4* __restrict__ target, float4* __restrict__ pixel_color,
    uint32_t* __restrict__ pixel_last, float4* __restrict__ checkpoints, uint32_t* __restrict__ blend_mask,
    uint32_t* __restrict__ counters, bool cut_in_record) {
  __shared__ WarpStage stages[FWD_WARPS];
  // Cooperative blending, double-buffered by round: each producer's queued entries
  // (alpha per pixel; colour with the 1-based list position's bits in w) and their count.
  __shared__ float s_alpha[2][PRODUCERS][32][32];
  __shared__ float4 s_qcolor[2][PRODUCERS][32];
  __shared__ uint32_t s_qlive[2][PRODUCERS];
  __shared__ uint32_t s_item, s_stop, s_done;  // s_done: warp 0's pixels that have stopped
  constexpr uint32_t BLOCK_SHIFT = 3u + TWL + THL, BLOCK_MASK = (1u << BLOCK_SHIFT) - 1u;
  constexpr bool MEMBER = TWL + THL > 0;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  WarpStage& st = stages[warp];
  const float vpx = camera->viewport[0], vpy = camera->viewport[1];
  const uint32_t tiles_x = ((uint32_t)vpx + TILE - 1u) / TILE;
  const uint2 tiles16 = make_uint2(tiles_x, ((uint32_t)vpy + TILE - 1u) / TILE);
  const float4 bg = raster_params[0];
  const uint32_t cooperative = plan[0], tiles = plan[1];
  const uint32_t* order = plan + PLAN_HEADER;

  // Cooperative items: one block of a long tile per CTA. Warps 1..PRODUCERS take
  // consecutive 32-entry windows of round r (window pw of the round is producer
  // pw's), keep the splats that can reach the block, compute their alphas at the
  // 32 pixels and queue the entries some pixel blends into buffer r % 2; warp 0
  // meanwhile applies round r - 1's queues, window by window in list order. One
  // barrier per round hands the buffers over.
  constexpr uint32_t STRIDE = 32u * PRODUCERS;  // entries per round
  while (true) {
    __syncthreads();  // everyone has read the previous s_item
    if (threadIdx.x == 0) {
      s_item = atomicAdd(&counters[0], 1u);
      s_done = 0;
      s_stop = 0;
    }
    __syncthreads();
    const uint32_t item = s_item;
    if (item >= cooperative << BLOCK_SHIFT) break;
    const uint32_t block = item & BLOCK_MASK;
    const BlendItem it(order[item >> BLOCK_SHIFT], block, lane, tiles_x, tiles_per_view, vpx, vpy, ranges, TWL, THL);
    const TileMember tm{MEMBER, it.tx, it.ty, tiles16};
    const uint2 run = it.run;
    PixelBlend pb{(float)it.px + 0.5f, (float)it.py + 0.5f, 1.0f, 0.0f, 0.0f, 0.0f, 0u, !it.inside};
    uint32_t next_k = 1;  // the next checkpoint boundary (warp 0)
    const uint32_t pw = warp - 1u;  // producer index (warps >= 1)
    // This producer lane's entry of the window in flight and of the one after it.
    uint32_t index = 0, next_index = 0;
    if (warp > 0) {
      const uint32_t k = run.x + 32u * pw + lane;
      if (k < run.y) index = pair_splats[k];
      stage_issue(st, splats, index, k < run.y);
      if (k + STRIDE < run.y) next_index = pair_splats[k + STRIDE];
    }
    const uint32_t rounds = (run.y - run.x + STRIDE - 1u) / STRIDE;
    for (uint32_t r = 0; r <= rounds; r++) {
      const uint32_t buf = r & 1u;
      if (warp > 0) {
        const uint32_t start = run.x + r * STRIDE + 32u * pw;
        if (r < rounds && start < run.y) {
          const uint32_t staged = stage_commit(st, run.x, start, run.y, index, it.x0, it.y0, cut_in_record, tm);
          {
            const uint32_t k = start + STRIDE + lane;
            stage_issue(st, splats, next_index, k < run.y);
            index = next_index;
            next_index = k + STRIDE < run.y ? pair_splats[k + STRIDE] : 0u;
          }
          // Pixels warp 0 has stopped take no part (it publishes the mask after
          // each window it applies; the mask only grows, so a stale copy only
          // keeps an entry that a fresh one would drop).
          uint32_t live = 0, blended = 0;
          for (uint32_t j = 0; j < staged; j += 4) {
            const uint32_t e[4] = {j, min(j + 1, staged - 1), min(j + 2, staged - 1), min(j + 3, staged - 1)};
            const uint32_t done_mask = *reinterpret_cast<volatile uint32_t*>(&s_done);
            const bool active = it.inside && !((done_mask >> lane) & 1u);
            float alpha[4];
            if (!pb.alphas4(st, e, staged - j, active, alpha)) continue;
            // Entry u is queued when some pixel's alpha is nonzero (then u < the
            // entries left, and e[u] = j + u). Lane u < 4 queues entry u's colour and
            // position and its blend-mask bit; every lane its alphas.
            const uint32_t mine = (alpha[0] != 0.0f ? 1u : 0u) | (alpha[1] != 0.0f ? 2u : 0u) |
                                  (alpha[2] != 0.0f ? 4u : 0u) | (alpha[3] != 0.0f ? 8u : 0u);
            const uint32_t any = __reduce_or_sync(0xffffffffu, mine);
            uint32_t bit = 0;
            if (lane < 4 && ((any >> lane) & 1u)) {
              const uint32_t slot = live + __popc(any & ((1u << lane) - 1u));
              const float4 c = st.color[j + lane];
              const uint32_t pos = st.pos[j + lane];
              s_qcolor[buf][pw][slot] = make_float4(c.x, c.y, c.z, __uint_as_float(pos + 1));
              bit = 1u << (pos - (start - run.x));
            }
            blended |= __reduce_or_sync(0xffffffffu, bit);
#pragma unroll
            for (uint32_t u = 0; u < 4; u++)
              if ((any >> u) & 1u) s_alpha[buf][pw][live++][lane] = alpha[u];
          }
          if (lane == 0) {
            s_qlive[buf][pw] = live;
            publish_blended(blend_mask, start, block, blended);
          }
        } else if (lane == 0) {
          s_qlive[buf][pw] = 0;
        }
      } else if (r > 0) {
        // Warp 0: round r - 1, in list order.
        const uint32_t prev = buf ^ 1u;
        for (uint32_t w = 0; w < PRODUCERS; w++) {
          const uint32_t ws = run.x + (r - 1u) * STRIDE + 32u * w;
          if (ws >= run.y) break;
          if (ws - run.x == next_k * CHUNK) {
            save_checkpoints(checkpoints, run.x, next_k, next_k + 1, block, lane, pb.T, pb.r, pb.g, pb.b);
            next_k++;
          }
          const uint32_t n = s_qlive[prev][w];
#pragma unroll 4
          for (uint32_t m = 0; m < n; m++) {
            const float4 q = s_qcolor[prev][w][m];
            pb.blend(s_alpha[prev][w][m][lane], q, __float_as_uint(q.w));
          }
          const uint32_t done = __ballot_sync(0xffffffffu, pb.done);
          if (lane == 0) *reinterpret_cast<volatile uint32_t*>(&s_done) = done;
        }
        if (lane == 0) s_stop = s_done == 0xffffffffu;
      }
      __syncthreads();
      if (s_stop) break;
    }
    cp_async_wait_all();
    if (warp == 0) {
      save_checkpoints(checkpoints, run.x, next_k, (run.y - run.x + CHUNK - 1) / CHUNK, block, lane, pb.T, pb.r, pb.g,
                       pb.b);
      write_pixel(it, pb, bg, target, pixel_color, pixel_last);
    }
  }

  // Independent items: one block per warp.
  while (true) {
    uint32_t item = 0;
    if (lane == 0) item = atomicAdd(&counters[1], 1u);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= (tiles - cooperative) << BLOCK_SHIFT) break;
    const uint32_t block = item & BLOCK_MASK;
    const BlendItem it(order[cooperative + (item >> BLOCK_SHIFT)], block, lane, tiles_x, tiles_per_view, vpx, vpy,
                       ranges, TWL, THL);
    const TileMember tm{MEMBER, it.tx, it.ty, tiles16};
    const uint2 run = it.run;
    PixelBlend pb{(float)it.px + 0.5f, (float)it.py + 0.5f, 1.0f, 0.0f, 0.0f, 0.0f, 0u, !it.inside};
    uint32_t next_k = 1;
    uint32_t index = 0, next_index = 0;
    {
      const uint32_t k = run.x + lane;
      if (k < run.y) index = pair_splats[k];
      stage_issue(st, splats, index, k < run.y);
      if (k + 32u < run.y) next_index = pair_splats[k + 32u];
    }
    for (uint32_t start = run.x; start < run.y; start += 32) {
      if (__all_sync(0xffffffffu, pb.done)) break;
      if (start - run.x == next_k * CHUNK) {
        save_checkpoints(checkpoints, run.x, next_k, next_k + 1, block, lane, pb.T, pb.r, pb.g, pb.b);
        next_k++;
      }
      const uint32_t staged = stage_commit(st, run.x, start, run.y, index, it.x0, it.y0, cut_in_record, tm);
      {
        const uint32_t k = start + 32u + lane;
        stage_issue(st, splats, next_index, k < run.y);
        index = next_index;
        next_index = k + 32u < run.y ? pair_splats[k + 32u] : 0u;
      }
      uint32_t blended = 0;
      for (uint32_t j = 0; j < staged; j += 4) {
        if (__all_sync(0xffffffffu, pb.done)) break;
        const uint32_t e[4] = {j, min(j + 1, staged - 1), min(j + 2, staged - 1), min(j + 3, staged - 1)};
        pb.apply4(st, e, staged - j, start - run.x, blended);
      }
      if (lane == 0) publish_blended(blend_mask, start, block, blended);
      __syncwarp();
    }
    cp_async_wait_all();  // a window may still be in flight after an early stop
    save_checkpoints(checkpoints, run.x, next_k, (run.y - run.x + CHUNK - 1) / CHUNK, block, lane, pb.T, pb.r, pb.g,
                     pb.b);
    write_pixel(it, pb, bg, target, pixel_color, pixel_last);
  }
}

// The empty-scene render pass: clear the target to the background (src/gaussianRenderer.ts:178-184).
__global__ void clear_target_kernel(uchar4* __restrict__ target, uint32_t pixels, float r, float g, float b) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < pixels) target[i] = make_uchar4(to_unorm8(r), to_unorm8(g), to_unorm8(b), 255);
}

}  // namespace

// ------------------------------------------------------------ TileRasterizer

static dg_status ensure_plan(dg_tile_rasterizer* tr);

static dg_status make_pairs(dg_tile_rasterizer* tr, uint32_t capacity) {
  dg_context* ctx = tr->ctx;
  free_buffer(tr->keys);
  free_buffer(tr->values);
  free_buffer(tr->keys_alt);
  free_buffer(tr->values_alt);
  free_buffer(tr->sort_scratch);
  tr->keys = tr->values = tr->keys_alt = tr->values_alt = tr->sort_scratch = nullptr;
  tr->plan = sort_plan(capacity, TILE_INDEX_BITS);
  tr->tile_plan = sort_plan_low_bits(capacity, TILE_INDEX_BITS);
  tr->pair_capacity = capacity;
  DG_TRY(alloc_buffer(ctx, (size_t)capacity * 8, &tr->keys));
  DG_TRY(alloc_buffer(ctx, (size_t)capacity * 4, &tr->values));
  DG_TRY(alloc_buffer(ctx, (size_t)capacity * 8, &tr->keys_alt));
  DG_TRY(alloc_buffer(ctx, (size_t)capacity * 4, &tr->values_alt));
  DG_TRY(alloc_buffer(ctx, std::max(sort_scratch_bytes(tr->plan), sort_scratch_bytes(tr->tile_plan)),
                      &tr->sort_scratch));
  return ensure_plan(tr);
}


dg_status rasterizer_create(dg_context* ctx, dg_buffer* camera, dg_buffer* splats, uint32_t count,
                            uint32_t initial_pair_capacity, bool depth_first, bool own_splats,
                            dg_tile_rasterizer** out) {
  auto* tr = new dg_tile_rasterizer();
  tr->splat_cutoffs = own_splats;
  tr->ctx = ctx;
  tr->camera = camera;
  tr->splats = splats;
  tr->count = count;
  dg_status st = alloc_buffer(ctx, (size_t)std::max(count, 1u) * 4, &tr->tile_offsets);
  if (st == DG_OK) st = alloc_buffer(ctx, 4, &tr->scan_total);
  if (st == DG_OK) st = alloc_buffer(ctx, scan_scratch_bytes(std::max(count, 1u)), &tr->scan_scratch);
  if (st == DG_OK) st = alloc_buffer(ctx, 16, &tr->raster_params);
  if (st == DG_OK) st = alloc_buffer(ctx, 16, &tr->work);
  if (st == DG_OK && cudaMallocHost(&tr->pinned_totals, 4 * dg_tile_rasterizer::READBACKS) != cudaSuccess)
    st = fail(DG_ERROR_OUT_OF_MEMORY, "pinned");
  for (uint32_t k = 0; k < dg_tile_rasterizer::READBACKS && st == DG_OK; k++)
    if (cudaEventCreateWithFlags(&tr->readback_events[k], cudaEventDisableTiming) != cudaSuccess)
      st = fail(DG_ERROR_CUDA, "event");
  uint32_t capacity = initial_pair_capacity ? initial_pair_capacity : std::max(1u << 16, count * 8u);
  if (st == DG_OK) st = make_pairs(tr, capacity);
  tr->depth_first = depth_first;
  tr->coop_min = COOP_MIN;
  if (st == DG_OK && depth_first) {
    const size_t n = std::max(count, 1u);
    tr->depth_plan = sort_plan_low_bits(std::max(count, 1u), 32);
    st = alloc_buffer(ctx, n * 4, &tr->depth_keys);
    if (st == DG_OK) st = alloc_buffer(ctx, n * 4, &tr->depth_values);
    if (st == DG_OK) st = alloc_buffer(ctx, n * 4, &tr->depth_keys_alt);
    if (st == DG_OK) st = alloc_buffer(ctx, n * 4, &tr->depth_values_alt);
    if (st == DG_OK) st = alloc_buffer(ctx, sort_scratch_bytes(tr->depth_plan), &tr->depth_scratch);
    if (st == DG_OK) st = alloc_buffer(ctx, n * 4, &tr->counts_sorted);
  }
  if (st != DG_OK) {
    dg_tile_rasterizer_destroy(tr);
    return st;
  }
  *out = tr;
  return DG_OK;
}

dg_status rasterizer_prepare(dg_tile_rasterizer* tr, const float viewport[2], const float background[3]) {
  const uint32_t tiles_x = ceil_div((uint32_t)viewport[0], TILE), tiles_y = ceil_div((uint32_t)viewport[1], TILE);
  if ((uint64_t)tiles_x * tiles_y > (1u << TILE_INDEX_BITS))
    return fail(DG_ERROR_INVALID_ARGUMENT, "A " + std::to_string((int)viewport[0]) + "x" +
                                               std::to_string((int)viewport[1]) +
                                               " viewport has more tiles than the sort can tell apart.");
  tr->tiles_x = tiles_x;
  tr->tiles_y = tiles_y;
  tr->viewport[0] = viewport[0];
  tr->viewport[1] = viewport[1];
  const uint32_t tiles = tiles_x * tiles_y;
  // The depth-first path's tile keys are tile indices below `tiles`: its last
  // pass sorts 4 bits when they cover the rest (up to 4096 tiles).
  uint32_t tile_bits = 1;
  while (tile_bits < 32 && (1u << tile_bits) < tiles) tile_bits++;
  sort_plan_key_bits(tr->tile_plan, tile_bits);
  if (!tr->ranges || tr->ranges_tiles < tiles) {
    free_buffer(tr->ranges);
    tr->ranges = nullptr;
    DG_TRY(alloc_buffer(tr->ctx, (size_t)std::max(tiles, 1u) * 8, &tr->ranges));
    tr->ranges_tiles = tiles;
    DG_TRY(ensure_plan(tr));
  }
  const uint32_t pixels = (uint32_t)viewport[0] * (uint32_t)viewport[1];
  if (!tr->pixel_color || tr->pixel_count < pixels) {
    free_buffer(tr->pixel_color);
    free_buffer(tr->pixel_last);
    tr->pixel_color = tr->pixel_last = nullptr;
    DG_TRY(alloc_buffer(tr->ctx, (size_t)std::max(pixels, 1u) * 16, &tr->pixel_color));
    DG_TRY(alloc_buffer(tr->ctx, (size_t)std::max(pixels, 1u) * 4, &tr->pixel_last));
    tr->pixel_count = pixels;
  }
  const float params[4] = {background[0], background[1], background[2], 1.0f};
  return write_async(tr->ctx, tr->raster_params->ptr, params, sizeof(params));
}

dg_status rasterizer_launch(dg_tile_rasterizer* tr, dg_buffer* target, bool counts_ready) {
  dg_context* ctx = tr->ctx;
  cudaStream_t st = ctx->stream;
  const uint32_t count = tr->count;
  const auto* cam = typed<const Camera>(tr->camera);
  DG_CUDA(cudaMemsetAsync(tr->ranges->ptr, 0, (size_t)tr->tiles_x * tr->tiles_y * 8, st));
  if (tr->depth_first && counts_ready) {
    // tile_offsets holds each splat's tile count; depth_keys/depth_values its depth
    // bits and index (both written by the renderer's preprocess).
    uint32_t* order = typed<uint32_t>(tr->depth_values);
    if (count > 0) {
      DG_TRY(sort_launch(ctx, tr->depth_plan, tr->depth_keys->ptr, order, tr->depth_keys_alt->ptr,
                         typed<uint32_t>(tr->depth_values_alt), nullptr, tr->depth_scratch->ptr));
    }
    // The splats' tile counts in depth order, scanned: the scan gathers them
    // through the sort's permutation as it loads them.
    DG_TRY(scan_launch(ctx, typed<uint32_t>(tr->counts_sorted), count, nullptr, typed<uint32_t>(tr->scan_total),
                       tr->scan_scratch->ptr, count > 0 ? order : nullptr, typed<uint32_t>(tr->tile_offsets)));
    if (count > 0) {
      DG_LAUNCH(ctx, "duplicate",
                duplicate_sorted_kernel<<<ceil_div(count, DUP_THREADS), DUP_THREADS, 0, st>>>(
                    cam, typed<float>(tr->splats), order, typed<uint32_t>(tr->counts_sorted), count, count, 0u,
                    tr->pair_capacity, typed<uint32_t>(tr->keys), typed<uint32_t>(tr->values), 0u, 0u));
    }
    DG_TRY(sort_launch(ctx, tr->tile_plan, tr->keys->ptr, typed<uint32_t>(tr->values), tr->keys_alt->ptr,
                       typed<uint32_t>(tr->values_alt), typed<uint32_t>(tr->scan_total), tr->sort_scratch->ptr));
    DG_LAUNCH(ctx, "find_ranges",
              find_ranges_kernel<1><<<stride_grid(ctx, tr->pair_capacity, RANGE_THREADS), RANGE_THREADS, 0,
                                      st>>>(typed<uint32_t>(tr->keys), typed<uint32_t>(tr->scan_total),
                                            tr->pair_capacity, tr->tiles_x * tr->tiles_y, 0u, 1u, typed<uint2>(tr->ranges)));
    tr->keys_are_tiles = true;
    return launch_rasterize(tr, target);
  }
  tr->keys_are_tiles = false;
  if (count > 0) {
    if (!counts_ready) {
      DG_LAUNCH(ctx, "count_tiles",
                count_tiles_kernel<<<ceil_div(count, 256), 256, 0, st>>>(cam, typed<float>(tr->splats), count,
                                                                        typed<uint32_t>(tr->tile_offsets)));
    }
  }
  DG_TRY(scan_launch(ctx, typed<uint32_t>(tr->tile_offsets), count, nullptr, typed<uint32_t>(tr->scan_total),
                     tr->scan_scratch->ptr));
  if (count > 0) {
    DG_LAUNCH(ctx, "duplicate",
              duplicate_kernel<<<ceil_div(count, DUP_THREADS), DUP_THREADS, 0, st>>>(
                  cam, typed<float>(tr->splats), typed<uint32_t>(tr->tile_offsets), count, tr->pair_capacity,
                  typed<uint64_t>(tr->keys), typed<uint32_t>(tr->values)));
  }
  DG_TRY(sort_launch(ctx, tr->plan, tr->keys->ptr, typed<uint32_t>(tr->values), tr->keys_alt->ptr,
                     typed<uint32_t>(tr->values_alt), typed<uint32_t>(tr->scan_total), tr->sort_scratch->ptr));
  DG_LAUNCH(ctx, "find_ranges",
            find_ranges_kernel<2><<<stride_grid(ctx, tr->pair_capacity, RANGE_THREADS), RANGE_THREADS, 0,
                                    st>>>(typed<uint32_t>(tr->keys), typed<uint32_t>(tr->scan_total),
                                          tr->pair_capacity, tr->tiles_x * tr->tiles_y, 0u, 1u,
                                          typed<uint2>(tr->ranges)));
  return launch_rasterize(tr, target);
}

dg_status launch_rasterize(dg_tile_rasterizer* tr, dg_buffer* target) {
  dg_context* ctx = tr->ctx;
  DG_CUDA(cudaMemsetAsync(tr->blend_mask->ptr, 0, tr->blend_mask->bytes, ctx->stream));
  BlendForward f{};
  f.camera = typed<const Camera>(tr->camera);
  f.raster_params = typed<float4>(tr->raster_params);
  f.splats = typed<float>(tr->splats);
  f.pair_splats = typed<uint32_t>(tr->values);
  f.ranges = typed<uint2>(tr->ranges);
  f.tiles = f.tiles_per_view = tr->tiles_x * tr->tiles_y;
  f.coop_min = tr->coop_min;
  f.plan = typed<uint32_t>(tr->work_plan);
  f.chunks = typed<uint2>(tr->chunks);
  f.target = target ? typed<uchar4>(target) : nullptr;
  f.pixel_color = typed<float4>(tr->pixel_color);
  f.pixel_last = typed<uint32_t>(tr->pixel_last);
  f.checkpoints = typed<float4>(tr->checkpoints);
  f.blend_mask = typed<uint32_t>(tr->blend_mask);
  f.counters = typed<uint32_t>(tr->work);
  f.splat_cutoffs = tr->splat_cutoffs;
  return blend_forward(ctx, f);
}

template <uint32_t TWL, uint32_t THL>
static dg_status launch_rasterize_kernel(dg_context* ctx, const BlendForward& f) {
  const auto kernel = rasterize_kernel<TWL, THL>;
  const uint32_t items = f.tiles << (3u + TWL + THL);
  DG_LAUNCH(ctx, "rasterize",
            kernel<<<blend_grid(ctx, (const void*)kernel, FWD_THREADS, items), FWD_THREADS, 0, ctx->stream>>>(
                f.camera, f.raster_params, f.splats, f.pair_splats, f.ranges, f.plan, f.tiles_per_view, f.target,
                f.pixel_color, f.pixel_last, f.checkpoints, f.blend_mask, f.counters, f.splat_cutoffs));
  return DG_OK;
}

dg_status blend_forward(dg_context* ctx, const BlendForward& f) {
  const BlendShape sh = f.shape;
  DG_REQUIRE(sh.twl <= MAX_BLEND_TILE_LOG2 && sh.thl <= MAX_BLEND_TILE_LOG2, "blend tiles of at most 2 x 2 tiles");
  DG_REQUIRE(sh.twl + sh.thl == 0 || (!f.checkpoints && !f.blend_mask && !f.chunks),
             "blend tiles larger than 16x16 have no backward pass");
  DG_CUDA(cudaMemsetAsync(f.counters, 0, 16, ctx->stream));
  DG_LAUNCH(ctx, "plan",
            plan_kernel<<<1, PLAN_THREADS, 0, ctx->stream>>>(f.ranges, f.tiles, f.coop_min, f.plan, f.chunks));
  if (sh.twl == 0 && sh.thl == 0) return launch_rasterize_kernel<0, 0>(ctx, f);
  if (sh.twl == 1 && sh.thl == 0) return launch_rasterize_kernel<1, 0>(ctx, f);
  if (sh.twl == 0 && sh.thl == 1) return launch_rasterize_kernel<0, 1>(ctx, f);
  return launch_rasterize_kernel<1, 1>(ctx, f);
}

uint32_t blend_grid(dg_context* ctx, const void* kernel, uint32_t threads, uint32_t items) {
  // As many CTAs as can be resident at once; each keeps taking items, so a CTA
  // that could not start until another finished would find none.
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, (int)threads, 0) != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    per_sm = 1;
  }
  return std::max(1u, std::min(ceil_div(items, threads / 32u), (uint32_t)(ctx->sm_count * per_sm)));
}

dg_status views_preprocess_launch(dg_context* ctx, const Camera* cameras, uint32_t views, const float* gaussians,
                                  const float* sh, uint32_t count, const uint32_t* scene_params, float* splats,
                                  uint32_t* tile_counts, uint2* depth_keys, uint32_t* order, BlendShape shape) {
  DG_LAUNCH(ctx, "preprocess",
            preprocess_views_kernel<<<ceil_div(count, PRE_THREADS), PRE_THREADS, 0, ctx->stream>>>(
                cameras, views, gaussians, sh, count, scene_params, splats, tile_counts, depth_keys, order,
                shape.twl, shape.thl));
  return DG_OK;
}


dg_status duplicate_sorted_launch(dg_context* ctx, const Camera* camera, const float* splats, const uint32_t* order,
                                  const uint32_t* offsets, uint32_t count, uint32_t per_view, uint32_t view_shift,
                                  uint32_t capacity, uint32_t* keys, uint32_t* values, BlendShape shape) {
  DG_LAUNCH(ctx, "duplicate",
            duplicate_sorted_kernel<<<ceil_div(count, DUP_THREADS), DUP_THREADS, 0, ctx->stream>>>(
                camera, splats, order, offsets, count, per_view, view_shift, capacity, keys, values, shape.twl,
                shape.thl));
  return DG_OK;
}

dg_status find_view_ranges_launch(dg_context* ctx, const uint32_t* tile_keys, const uint32_t* pair_total,
                                  uint32_t capacity, uint32_t view_shift, uint32_t tiles_per_view, uint32_t tiles,
                                  uint2* ranges) {
  DG_LAUNCH(ctx, "find_ranges",
            find_ranges_kernel<1><<<stride_grid(ctx, capacity, RANGE_THREADS), RANGE_THREADS, 0, ctx->stream>>>(
                tile_keys, pair_total, capacity, tiles, view_shift, tiles_per_view, ranges));
  return DG_OK;
}

// The work plan, the backward's chunk list and the checkpoints, sized for the
// allocated tiles and pair capacity.
static dg_status ensure_plan(dg_tile_rasterizer* tr) {
  const size_t tiles = std::max(tr->ranges_tiles, 1u);
  const size_t slots = (size_t)tr->pair_capacity / CHUNK + 1;
  struct Need {
    dg_buffer** buf;
    size_t bytes;
  } needs[] = {{&tr->work_plan, (PLAN_HEADER + tiles) * 4},
               {&tr->chunks, (tiles + slots) * 8},
               {&tr->checkpoints, slots * 8 * 32 * 16},
               {&tr->blend_mask, ((size_t)tr->pair_capacity / 32 + 2) * 8 * 4}};
  for (const Need& n : needs) {
    if (*n.buf && (*n.buf)->bytes >= n.bytes) continue;
    free_buffer(*n.buf);
    *n.buf = nullptr;
    DG_TRY(alloc_buffer(tr->ctx, n.bytes, n.buf));
  }
  return DG_OK;
}

// The sorted keys in the reference's 64-bit form, rebuilt if the last frame took
// the depth-first path.
dg_buffer* rasterizer_sorted_keys(dg_tile_rasterizer* tr) {
  if (!tr->keys_are_tiles) return tr->keys;
  if (!tr->keys64 || tr->keys64->bytes < (uint64_t)tr->pair_capacity * 8) {
    free_buffer(tr->keys64);
    tr->keys64 = nullptr;
    if (alloc_buffer(tr->ctx, (size_t)tr->pair_capacity * 8, &tr->keys64) != DG_OK) return nullptr;
  }
  materialize_keys_kernel<<<std::max(1u, ceil_div(tr->pair_capacity, 256)), 256, 0, tr->ctx->stream>>>(
      typed<uint32_t>(tr->keys), typed<uint32_t>(tr->values), typed<float>(tr->splats), typed<uint32_t>(tr->scan_total),
      tr->pair_capacity, typed<uint64_t>(tr->keys64));
  tr->ctx->launches++;
  return tr->keys64;
}

// Consumes the queued readbacks whose copies are done (all of them with `wait`),
// oldest first, growing the pair buffers when a frame needed more pairs than
// they hold: the reference's afterSubmit (src/tileRasterizer.ts:229-244), whose
// promise resolves for every frame.
static dg_status consume_readbacks(dg_tile_rasterizer* tr, bool wait) {
  constexpr uint32_t R = dg_tile_rasterizer::READBACKS;
  while (tr->readback_tail != tr->readback_head) {
    cudaEvent_t e = tr->readback_events[tr->readback_tail % R];
    if (!wait && cudaEventQuery(e) == cudaErrorNotReady) break;
    DG_CUDA(cudaEventSynchronize(e));
    tr->last_pair_count = tr->pinned_totals[tr->readback_tail % R];
    tr->readback_tail++;
    DG_TRY(rasterizer_reserve_pairs(tr, tr->last_pair_count));
  }
  return DG_OK;
}

dg_status rasterizer_reserve_pairs(dg_tile_rasterizer* tr, uint64_t pairs) {
  if (pairs <= tr->pair_capacity) return DG_OK;
  const double want = std::ceil(std::log2((double)pairs * 1.25));
  DG_REQUIRE(want < 30, "the frame needs more pairs than the sort can hold");
  return make_pairs(tr, 1u << (uint32_t)want);
}

dg_status rasterizer_queue_readback(dg_tile_rasterizer* tr) {
  constexpr uint32_t R = dg_tile_rasterizer::READBACKS;
  if (tr->readback_head - tr->readback_tail == R) {  // full: the oldest first
    DG_CUDA(cudaEventSynchronize(tr->readback_events[tr->readback_tail % R]));
    DG_TRY(consume_readbacks(tr, false));
  }
  const uint32_t slot = tr->readback_head % R;
  DG_CUDA(cudaMemcpyAsync(tr->pinned_totals + slot, tr->scan_total->ptr, 4, cudaMemcpyDeviceToHost, tr->ctx->stream));
  DG_CUDA(cudaEventRecord(tr->readback_events[slot], tr->ctx->stream));
  tr->readback_head++;
  return DG_OK;
}

dg_status rasterizer_launch_backward(dg_tile_rasterizer* tr, dg_buffer* pixel_grads, dg_buffer* splat_grads) {
  dg_context* ctx = tr->ctx;
  DG_CUDA(cudaMemsetAsync(splat_grads->ptr, 0, (size_t)tr->count * SPLAT_GRADS * 4, ctx->stream));
  return launch_rasterize_backward(tr, pixel_grads, splat_grads);
}

// ------------------------------------------------------------ GaussianRenderer

static void destroy_scene(dg_renderer* r) {
  free_buffer(r->gaussians);
  free_buffer(r->splats);
  free_buffer(r->sh);
  free_buffer(r->scene_params);
  free_buffer(r->grad_splats);
  free_buffer(r->grad_gaussians);
  free_buffer(r->grad_sh);
  free_buffer(r->radii);
  if (r->rasterizer) dg_tile_rasterizer_destroy(r->rasterizer);
  r->gaussians = r->splats = r->sh = r->scene_params = r->radii = nullptr;
  r->grad_splats = r->grad_gaussians = r->grad_sh = nullptr;
  r->rasterizer = nullptr;
  r->has_scene = false;
  r->count = 0;
}

static dg_status create_scene(dg_renderer* r, uint32_t count, dg_buffer* gaussians, dg_buffer* sh, uint32_t degree,
                              uint32_t pair_capacity) {
  r->has_scene = true;
  r->count = count;
  r->gaussians = gaussians;
  r->sh = sh;
  DG_TRY(alloc_buffer(r->ctx, 16, &r->scene_params));
  const uint32_t params[4] = {degree, 0, 0, 0};
  DG_TRY(write_async(r->ctx, r->scene_params->ptr, params, sizeof(params)));
  DG_TRY(alloc_buffer(r->ctx, (size_t)count * FLOATS_PER_SPLAT * 4, &r->splats));
  DG_TRY(alloc_buffer(r->ctx, (size_t)std::max(count, 1u) * 4, &r->radii));
  DG_TRY(rasterizer_create(r->ctx, r->camera, r->splats, count, pair_capacity, true, true, &r->rasterizer));
  return DG_OK;
}

dg_status renderer_write_camera(dg_renderer* r, const dg_camera* camera) {
  Camera c{};
  std::memcpy(c.view, camera->view, 64);
  std::memcpy(c.proj, camera->proj, 64);
  c.viewport[0] = camera->viewport[0];
  c.viewport[1] = camera->viewport[1];
  r->last_viewport[0] = camera->viewport[0];
  r->last_viewport[1] = camera->viewport[1];
  return write_async(r->ctx, r->camera->ptr, &c, sizeof(c));
}

dg_status renderer_prepare(dg_renderer* r, const dg_camera* camera, const float background[3]) {
  DG_TRY(renderer_write_camera(r, camera));
  if (!r->has_scene) return DG_OK;
  return rasterizer_prepare(r->rasterizer, camera->viewport, background);
}

dg_status renderer_launch_forward(dg_renderer* r, dg_buffer* target) {
  dg_context* ctx = r->ctx;
  if (r->count > 0) {
    DG_LAUNCH(ctx, "preprocess",
              preprocess_kernel<<<preprocess_grid(ctx, r->count), PRE_THREADS, 0, ctx->stream>>>(
                  typed<const Camera>(r->camera), typed<float>(r->gaussians), typed<float>(r->sh), r->count,
                  typed<uint32_t>(r->scene_params), typed<float>(r->splats),
                  typed<uint32_t>(r->rasterizer->tile_offsets), typed<uint32_t>(r->rasterizer->depth_keys),
                  typed<uint32_t>(r->rasterizer->depth_values), typed<float>(r->radii)));
  }
  return rasterizer_launch(r->rasterizer, target, true);
}

dg_status renderer_ensure_gradients(dg_renderer* r) {
  if (r->grad_splats) return DG_OK;
  DG_TRY(alloc_buffer(r->ctx, (size_t)r->count * SPLAT_GRADS * 4, &r->grad_splats));
  DG_TRY(alloc_buffer(r->ctx, (size_t)r->count * FLOATS_PER_GAUSSIAN * 4, &r->grad_gaussians));
  DG_TRY(alloc_buffer(r->ctx, (size_t)r->count * SH_REST_FLOATS * 4, &r->grad_sh));
  return DG_OK;
}

dg_status renderer_launch_backward(dg_renderer* r, dg_buffer* pixel_grads, bool write_gaussian_grads) {
  DG_TRY(rasterizer_launch_backward(r->rasterizer, pixel_grads, r->grad_splats));
  if (!write_gaussian_grads || r->count == 0) return DG_OK;
  return launch_preprocess_backward(r);
}

const Camera* renderer_camera(dg_renderer* r) { return typed<const Camera>(r->camera); }

}  // namespace dg

using namespace dg;

extern "C" {

dg_status dg_tile_rasterizer_create(dg_context* ctx, dg_buffer* camera, dg_buffer* splats, uint32_t count,
                                    uint32_t initial_pair_capacity, dg_tile_rasterizer** out) {
  DG_REQUIRE(ctx && camera && splats && out, "NULL argument");
  DG_REQUIRE(camera->bytes >= sizeof(Camera), "camera buffer is smaller than the 144-byte Camera uniform");
  DG_REQUIRE(splats->bytes >= (uint64_t)count * FLOATS_PER_SPLAT * 4, "splat buffer too small for count");
  return rasterizer_create(ctx, camera, splats, count, initial_pair_capacity, false, false, out);
}

dg_status dg_tile_rasterizer_encode(dg_tile_rasterizer* tr, dg_buffer* target, const float viewport[2],
                                    const float background[3]) {
  DG_REQUIRE(tr && viewport && background, "NULL argument");
  if (target)
    DG_REQUIRE(target->bytes >= (uint64_t)(uint32_t)viewport[0] * (uint32_t)viewport[1] * 4,
               "target is smaller than the viewport");
  DG_TRY(rasterizer_prepare(tr, viewport, background));
  DG_TRY(rasterizer_launch(tr, target, false));
  return rasterizer_queue_readback(tr);
}

dg_status dg_tile_rasterizer_encode_backward(dg_tile_rasterizer* tr, const float viewport[2], dg_buffer* pixel_grads,
                                             dg_buffer* splat_grads) {
  DG_REQUIRE(tr && viewport && pixel_grads && splat_grads, "NULL argument");
  if (!tr->pixel_color || !tr->ranges) return fail(DG_ERROR_STATE, "Encode a frame before its backward pass.");
  DG_REQUIRE(splat_grads->bytes >= (uint64_t)tr->count * SPLAT_GRADS * 4, "splat gradient buffer too small");
  DG_REQUIRE(pixel_grads->bytes >= (uint64_t)tr->pixel_count * 16, "pixel gradient buffer too small");
  return rasterizer_launch_backward(tr, pixel_grads, splat_grads);
}

dg_status dg_tile_rasterizer_after_submit(dg_tile_rasterizer* tr, int32_t wait) {
  DG_REQUIRE(tr, "NULL argument");
  return consume_readbacks(tr, wait != 0);
}

uint32_t dg_tile_rasterizer_last_pair_count(const dg_tile_rasterizer* tr) { return tr ? tr->last_pair_count : 0; }
uint32_t dg_tile_rasterizer_pair_capacity(const dg_tile_rasterizer* tr) { return tr ? tr->pair_capacity : 0; }
dg_buffer* dg_tile_rasterizer_pair_splats(dg_tile_rasterizer* tr) { return tr ? tr->values : nullptr; }
dg_buffer* dg_tile_rasterizer_ranges(dg_tile_rasterizer* tr) { return tr ? tr->ranges : nullptr; }
dg_buffer* dg_tile_rasterizer_pair_keys(dg_tile_rasterizer* tr) { return tr ? rasterizer_sorted_keys(tr) : nullptr; }
dg_buffer* dg_tile_rasterizer_pixel_color(dg_tile_rasterizer* tr) { return tr ? tr->pixel_color : nullptr; }
dg_buffer* dg_tile_rasterizer_pixel_last(dg_tile_rasterizer* tr) { return tr ? tr->pixel_last : nullptr; }
dg_buffer* dg_tile_rasterizer_tile_offsets(dg_tile_rasterizer* tr) { return tr ? tr->tile_offsets : nullptr; }
dg_buffer* dg_tile_rasterizer_pair_total(dg_tile_rasterizer* tr) { return tr ? tr->scan_total : nullptr; }

dg_status dg_tile_rasterizer_destroy(dg_tile_rasterizer* tr) {
  if (!tr) return DG_OK;
  for (dg_buffer* b : {tr->tile_offsets, tr->scan_total, tr->scan_scratch, tr->raster_params, tr->keys, tr->values,
                       tr->keys_alt, tr->values_alt, tr->sort_scratch, tr->ranges, tr->pixel_color, tr->pixel_last,
                       tr->depth_keys, tr->depth_values, tr->depth_keys_alt, tr->depth_values_alt, tr->depth_scratch,
                       tr->counts_sorted, tr->keys64, tr->work, tr->work_plan, tr->chunks, tr->checkpoints,
                       tr->blend_mask})
    free_buffer(b);
  for (cudaEvent_t e : tr->readback_events)
    if (e) {
      cudaEventSynchronize(e);
      cudaEventDestroy(e);
    }
  if (tr->pinned_totals) cudaFreeHost(tr->pinned_totals);
  delete tr;
  return DG_OK;
}

dg_status dg_renderer_create(dg_context* ctx, uint32_t initial_pair_capacity, dg_renderer** out) {
  DG_REQUIRE(ctx && out, "NULL argument");
  auto* r = new dg_renderer();
  r->ctx = ctx;
  r->initial_pair_capacity = initial_pair_capacity;
  r->view_coop_min = COOP_MIN;
  r->view_shape = BlendShape{0u, 0u};
  r->view_graph = true;
  dg_status st = alloc_buffer(ctx, sizeof(Camera), &r->camera);
  if (st != DG_OK) {
    delete r;
    return st;
  }
  *out = r;
  return DG_OK;
}

dg_status dg_renderer_set_gaussians(dg_renderer* r, const float* data, uint32_t count, const float* sh_rest,
                                    uint64_t sh_floats, uint32_t degree) {
  DG_REQUIRE(r, "NULL argument");
  if (count == 0) {
    destroy_scene(r);
    return DG_OK;
  }
  DG_REQUIRE(data, "NULL Gaussian data");
  if (sh_rest && sh_floats != (uint64_t)count * SH_REST_FLOATS)
    return fail(DG_ERROR_INVALID_ARGUMENT, "Expected " + std::to_string((uint64_t)count * SH_REST_FLOATS) +
                                               " spherical-harmonic floats, got " + std::to_string(sh_floats) + ".");
  DG_REQUIRE(degree <= 3, "SH degree is at most 3");
  dg_buffer *g = nullptr, *s = nullptr;
  DG_TRY(alloc_buffer(r->ctx, (size_t)count * FLOATS_PER_GAUSSIAN * 4, &g));
  DG_TRY(write_async(r->ctx, g->ptr, data, (size_t)count * FLOATS_PER_GAUSSIAN * 4));
  // Without SH the buffer is still sized for count Gaussians, so training can
  // raise the degree later; its coefficients are zero.
  DG_TRY(alloc_buffer(r->ctx, (size_t)count * SH_REST_FLOATS * 4, &s));
  if (sh_rest) DG_TRY(write_async(r->ctx, s->ptr, sh_rest, (size_t)count * SH_REST_FLOATS * 4));
  destroy_scene(r);
  return create_scene(r, count, g, s, sh_rest ? degree : 0, r->initial_pair_capacity);
}

dg_status dg_renderer_adopt_gaussians(dg_renderer* r, uint32_t count, dg_buffer* gaussians, dg_buffer* sh,
                                      uint32_t degree) {
  DG_REQUIRE(r && gaussians && sh, "NULL argument");
  DG_REQUIRE(gaussians->bytes >= (uint64_t)count * FLOATS_PER_GAUSSIAN * 4, "Gaussian buffer too small");
  DG_REQUIRE(sh->bytes >= (uint64_t)count * SH_REST_FLOATS * 4, "SH buffer too small");
  uint32_t capacity = r->rasterizer ? r->rasterizer->pair_capacity : r->initial_pair_capacity;
  destroy_scene(r);
  return create_scene(r, count, gaussians, sh, degree, capacity);
}

dg_status dg_renderer_set_sh_degree(dg_renderer* r, uint32_t degree) {
  DG_REQUIRE(r, "NULL argument");
  DG_REQUIRE(degree <= 3, "SH degree is at most 3");
  if (!r->has_scene) return DG_OK;
  const uint32_t params[4] = {degree, 0, 0, 0};
  return write_async(r->ctx, r->scene_params->ptr, params, sizeof(params));
}

dg_status dg_renderer_encode(dg_renderer* r, dg_buffer* target, const dg_camera* camera, const float background[3]) {
  DG_REQUIRE(r && camera && background, "NULL argument");
  const uint32_t pixels = (uint32_t)camera->viewport[0] * (uint32_t)camera->viewport[1];
  if (target) DG_REQUIRE(target->bytes >= (uint64_t)pixels * 4, "target is smaller than the viewport");
  DG_TRY(renderer_prepare(r, camera, background));
  if (!r->has_scene) {
    if (target && pixels) {
      DG_LAUNCH(r->ctx, "clear_target",
                clear_target_kernel<<<ceil_div(pixels, 256), 256, 0, r->ctx->stream>>>(
                    typed<uchar4>(target), pixels, background[0], background[1], background[2]));
    }
    return DG_OK;
  }
  DG_TRY(renderer_launch_forward(r, target));
  return rasterizer_queue_readback(r->rasterizer);
}

dg_status dg_renderer_encode_draw(dg_renderer* r, dg_buffer* target, dg_buffer* splats, uint32_t count,
                                  const float viewport[2], const float background[3]) {
  DG_REQUIRE(r && splats && viewport && background, "NULL argument");
  dg_camera cam{};
  for (int k = 0; k < 16; k++) cam.view[k] = cam.proj[k] = (k % 5 == 0) ? 1.0f : 0.0f;
  cam.viewport[0] = viewport[0];
  cam.viewport[1] = viewport[1];
  DG_TRY(renderer_write_camera(r, &cam));
  if (r->draw_rasterizer) dg_tile_rasterizer_destroy(r->draw_rasterizer);
  r->draw_rasterizer = nullptr;
  DG_TRY(dg_tile_rasterizer_create(r->ctx, r->camera, splats, count, r->initial_pair_capacity, &r->draw_rasterizer));
  return dg_tile_rasterizer_encode(r->draw_rasterizer, target, viewport, background);
}

dg_status dg_renderer_encode_backward(dg_renderer* r, dg_buffer* pixel_grads) {
  DG_REQUIRE(r && pixel_grads, "NULL argument");
  if (!r->has_scene) return DG_OK;
  if (!r->rasterizer->pixel_color || !r->rasterizer->ranges)
    return fail(DG_ERROR_STATE, "Encode a frame before its backward pass.");
  DG_REQUIRE(pixel_grads->bytes >= (uint64_t)r->rasterizer->pixel_count * 16, "pixel gradient buffer too small");
  DG_TRY(renderer_ensure_gradients(r));
  return renderer_launch_backward(r, pixel_grads, true);
}

dg_status dg_renderer_after_submit(dg_renderer* r, int32_t wait) {
  DG_REQUIRE(r, "NULL argument");
  if (!r->rasterizer) return DG_OK;
  return dg_tile_rasterizer_after_submit(r->rasterizer, wait);
}

uint32_t dg_renderer_count(const dg_renderer* r) { return r ? r->count : 0; }
dg_buffer* dg_renderer_splat_buffer(dg_renderer* r) { return r ? r->splats : nullptr; }
dg_buffer* dg_renderer_gaussian_buffer(dg_renderer* r) { return r ? r->gaussians : nullptr; }
dg_buffer* dg_renderer_sh_buffer(dg_renderer* r) { return r ? r->sh : nullptr; }
dg_buffer* dg_renderer_pixel_buffer(dg_renderer* r) {
  return r && r->rasterizer ? r->rasterizer->pixel_color : nullptr;
}
dg_buffer* dg_renderer_pixel_last_buffer(dg_renderer* r) {
  return r && r->rasterizer ? r->rasterizer->pixel_last : nullptr;
}
dg_buffer* dg_renderer_gradient_gaussians(dg_renderer* r) { return r ? r->grad_gaussians : nullptr; }
dg_buffer* dg_renderer_gradient_sh(dg_renderer* r) { return r ? r->grad_sh : nullptr; }
dg_buffer* dg_renderer_gradient_splats(dg_renderer* r) { return r ? r->grad_splats : nullptr; }
dg_tile_rasterizer* dg_renderer_tiles(dg_renderer* r) { return r ? r->rasterizer : nullptr; }
dg_tile_rasterizer* dg_renderer_draw_tiles(dg_renderer* r) { return r ? r->draw_rasterizer : nullptr; }

dg_status dg_renderer_destroy(dg_renderer* r) {
  if (!r) return DG_OK;
  destroy_scene(r);
  if (r->draw_rasterizer) dg_tile_rasterizer_destroy(r->draw_rasterizer);
  view_batch_destroy(r->views);
  free_buffer(r->camera);
  delete r;
  return DG_OK;
}

}  // extern "C"

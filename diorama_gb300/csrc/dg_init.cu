// Training's starting Gaussians from a point cloud (src/loadDataset.ts:93-149):
// for each point the mean squared distance to its 3 nearest other points, then
// one Gaussian per point sized by it.
//
// The reference finds the neighbours by brute force (src/shaders/nearestNeighbors.wgsl:13-44),
// N² distances. Here the points are sorted along a Morton (Z-order) curve of 21
// bits per axis, which makes every cell of the implicit octree over the points a
// contiguous run of the sorted array. Each point then
//   1. takes the third-smallest squared distance R² among its 2·WINDOW neighbours
//      in curve order: its three nearest points lie within R;
//   2. picks the finest octree level whose cells are at least R (plus a rounding
//      margin) wide, so that every point within R lies in its own cell at that
//      level or one of the 26 around it;
//   3. scans those cells (a galloping binary search finds each one's run), skipping
//      a cell once its nearest face is farther than the best third distance so far.
// The search is exact: it finds the same three smallest squared distances, each
// computed as the reference computes it (d = q - p, then d.x² + d.y² + d.z²
// rounded in that order; this file is compiled without contraction), so every
// result is the brute force's bit for bit. The visiting order does not matter:
// the three smallest values of a set do not depend on the order they are met in.
//
// The octree spans the points' bounds trimmed to the mean ± 3 standard deviations
// per axis (so that a few far outliers do not coarsen it); points outside are
// clamped onto its border. Quantizing is monotone and non-expansive in each
// coordinate, so the cell arguments above hold for clamped points too. Points
// with a non-finite coordinate are no point's neighbours (their distances are
// infinite or NaN, never below the starting 3.4e38) and get the reference's
// result for a point without neighbours.
#include <cmath>
#include <cstring>

#include "dg_common.cuh"
#include "dg_scan.cuh"

namespace dg {
namespace {

constexpr uint32_t KNN_THREADS = 256;
constexpr uint32_t BITS = 21;         // per axis: 63-bit Morton codes
constexpr int32_t WINDOW = 8;         // curve neighbours on each side for the first bound
constexpr float FAR = 3.4e38f;        // nearestNeighbors.wgsl:19, the starting "distance"

struct Octree {
  float lo[3];
  float scale;  // finest cells per unit length
  float h0;     // finest cell width
  float slack;  // margin for rounding in the quantizing and in the cell faces
};

// Order-preserving u32 image of a float, for atomicMin/atomicMax.
__device__ __forceinline__ uint32_t ordered(float f) {
  const uint32_t b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

inline float unordered(uint32_t o) {
  const uint32_t b = (o & 0x80000000u) ? (o & 0x7fffffffu) : ~o;
  float f;
  std::memcpy(&f, &b, 4);
  return f;
}

struct Moments {
  uint32_t lo[3], hi[3];  // ordered images
  double sum[3], sum2[3];
  uint32_t finite;        // points with three finite coordinates
};

__device__ __forceinline__ bool finite3(float4 p) { return isfinite(p.x) && isfinite(p.y) && isfinite(p.z); }

__global__ void __launch_bounds__(KNN_THREADS) bounds_kernel(const float4* __restrict__ points, uint32_t n,
                                                             Moments* __restrict__ out) {
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  double sum[3] = {0, 0, 0}, sum2[3] = {0, 0, 0};
  uint32_t finite = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 p = points[i];
    if (!finite3(p)) continue;
    const float c[3] = {p.x, p.y, p.z};
    finite++;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      lo[k] = fminf(lo[k], c[k]);
      hi[k] = fmaxf(hi[k], c[k]);
      sum[k] += c[k];
      sum2[k] += (double)c[k] * c[k];
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    finite += __shfl_xor_sync(0xffffffffu, finite, off);
#pragma unroll
    for (int k = 0; k < 3; k++) {
      lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], off));
      hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], off));
      sum[k] += __shfl_xor_sync(0xffffffffu, sum[k], off);
      sum2[k] += __shfl_xor_sync(0xffffffffu, sum2[k], off);
    }
  }
  if ((threadIdx.x & 31) == 0 && finite) {
    atomicAdd(&out->finite, finite);
#pragma unroll
    for (int k = 0; k < 3; k++) {
      atomicMin(&out->lo[k], ordered(lo[k]));
      atomicMax(&out->hi[k], ordered(hi[k]));
      atomicAdd(&out->sum[k], sum[k]);
      atomicAdd(&out->sum2[k], sum2[k]);
    }
  }
}

// Finest-level cell coordinate of a position, clamped into the octree (NaN
// coordinates land at 0).
__device__ __forceinline__ void quantize(const Octree& o, float x, float y, float z, uint32_t q[3]) {
  const float p[3] = {x, y, z};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const float t = floorf((p[k] - o.lo[k]) * o.scale);
    q[k] = (uint32_t)fminf(fmaxf(t, 0.0f), (float)((1u << BITS) - 1u));
  }
}

// The bits of v (up to 21) spread to every third bit.
__device__ __forceinline__ uint64_t spread3(uint32_t v) {
  uint64_t x = v & 0x1fffffu;
  x = (x | x << 32) & 0x1f00000000ffffull;
  x = (x | x << 16) & 0x1f0000ff0000ffull;
  x = (x | x << 8) & 0x100f00f00f00f00full;
  x = (x | x << 4) & 0x10c30c30c30c30c3ull;
  x = (x | x << 2) & 0x1249249249249249ull;
  return x;
}

__device__ __forceinline__ uint64_t morton(uint32_t x, uint32_t y, uint32_t z) {
  return spread3(x) | spread3(y) << 1 | spread3(z) << 2;
}

// Each point's Morton code (the sort key, as (low, high) words) and index.
__global__ void morton_kernel(const float4* __restrict__ points, uint32_t n, Octree o, uint2* __restrict__ keys,
                              uint32_t* __restrict__ values) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p = points[i];
  uint32_t q[3];
  quantize(o, p.x, p.y, p.z, q);
  const uint64_t code = morton(q[0], q[1], q[2]);
  keys[i] = make_uint2((uint32_t)code, (uint32_t)(code >> 32));
  values[i] = i;
}

// The points in curve order, each carrying its original index in w.
__global__ void gather_points_kernel(const float4* __restrict__ points, uint32_t n, const uint32_t* __restrict__ order,
                                     float4* __restrict__ sorted) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const uint32_t i = order[s];
  const float4 p = points[i];
  sorted[s] = make_float4(p.x, p.y, p.z, __uint_as_float(i));
}

struct Best {
  float x = FAR, y = FAR, z = FAR;  // the three smallest squared distances, smallest first

  // nearestNeighbors.wgsl:26-41
  __device__ __forceinline__ void offer(float d2) {
    if (d2 < z) {
      if (d2 < y) {
        z = y;
        if (d2 < x) {
          y = x;
          x = d2;
        } else {
          y = d2;
        }
      } else {
        z = d2;
      }
    }
  }
};

__device__ __forceinline__ float distance2(float4 q, float px, float py, float pz) {
  const float dx = q.x - px, dy = q.y - py, dz = q.z - pz;
  return dx * dx + dy * dy + dz * dz;
}

__device__ __forceinline__ uint64_t key_at(const uint2* __restrict__ keys, int32_t i) {
  const uint2 k = keys[i];
  return (uint64_t)k.y << 32 | k.x;
}

// The first index whose key is >= target, searched outwards from `from`
// (galloping, then binary): a few steps for a cell near the point's own.
__device__ int32_t lower_bound_from(const uint2* __restrict__ keys, int32_t n, int32_t from, uint64_t target) {
  int32_t lo, hi;  // keys[lo] < target <= keys[hi], with lo = -1 or hi = n at the ends
  if (key_at(keys, from) < target) {
    lo = from;
    int32_t step = 1;
    hi = from + 1;
    while (hi < n && key_at(keys, hi) < target) {
      lo = hi;
      step <<= 1;
      hi = from + step < n ? from + step : n;
    }
  } else {
    hi = from;
    int32_t step = 1;
    lo = from - 1;
    while (lo >= 0 && key_at(keys, lo) >= target) {
      hi = lo;
      step <<= 1;
      lo = from - step >= 0 ? from - step : -1;
    }
  }
  while (hi - lo > 1) {
    const int32_t mid = lo + ((hi - lo) >> 1);
    if (key_at(keys, mid) < target) lo = mid;
    else hi = mid;
  }
  return hi;
}

// The first index in [lo, hi) whose key is >= target (hi if none).
__device__ __forceinline__ int32_t lower_bound_in(const uint2* __restrict__ keys, int32_t lo, int32_t hi,
                                                  uint64_t target) {
  while (lo < hi) {
    const int32_t mid = lo + ((hi - lo) >> 1);
    if (key_at(keys, mid) < target) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// A lower bound on the squared distance from p to any point of cell c at
// `level`, less the rounding margin per axis. The border cells' outer faces are
// open: the points clamped onto the border lie beyond them.
__device__ __forceinline__ float cell_gap2(const Octree& o, const float p[3], const uint32_t c[3], uint32_t level) {
  const float h = ldexpf(o.h0, (int)level);
  const uint32_t last = (1u << (BITS - level)) - 1u;
  float g2 = 0.0f;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    float g = 0.0f;
    if (c[k] > 0) g = fmaxf(g, (o.lo[k] + (float)c[k] * h) - p[k]);
    if (c[k] < last) g = fmaxf(g, p[k] - (o.lo[k] + (float)(c[k] + 1) * h));
    g = fmaxf(g - o.slack, 0.0f);
    g2 += g * g;
  }
  return g2;
}

// A cell being searched: its coordinates at `level`, its run of the sorted
// points, and the next of its 8 children to try.
struct Frame {
  uint32_t c[3];
  int32_t begin, end;
  uint32_t level, next;
};

constexpr int32_t LEAF = 32;  // cells with at most this many points are scanned whole

// One thread per point, in curve order (a warp's points are neighbours and
// search the same cells). A cell of more than LEAF points is searched through its
// children, nearest first (the child on the point's side of each axis, then those
// differing in one axis, two, three), each skipped once its box is farther than
// the best third distance so far: a point beside a dense region visits only the
// part of it that can hold a nearer point.
__global__ void __launch_bounds__(KNN_THREADS) knn_query_kernel(const float4* __restrict__ sorted,
                                                                const uint2* __restrict__ keys, uint32_t n, Octree o,
                                                                float* __restrict__ distance2_out) {
  const int32_t s = (int32_t)(blockIdx.x * blockDim.x + threadIdx.x);
  if (s >= (int32_t)n) return;
  const float4 me = sorted[s];
  const uint32_t self = __float_as_uint(me.w);
  if (!finite3(me)) {
    distance2_out[self] = (FAR + FAR + FAR) / 3.0f;  // no neighbours: nearestNeighbors.wgsl:43
    return;
  }
  const int32_t count = (int32_t)n;
  // 1. A first bound from the curve neighbours.
  Best window;
  for (int32_t j = max(s - WINDOW, 0); j <= min(s + WINDOW, count - 1); j++)
    if (j != s) window.offer(distance2(sorted[j], me.x, me.y, me.z));
  // Every point with a computed squared distance <= window.z is within `reach`
  // (the factor covers the rounding of the computed distances).
  const float reach = sqrtf(window.z) * 1.000001f + o.slack;
  // 2. The finest level whose cells are at least `reach` wide (the root if none):
  // every point within `reach` is in the point's cell or one of the 26 around it.
  uint32_t level = 0;
  while (level < BITS && ldexpf(o.h0, (int)level) < reach) level++;
  uint32_t q[3];
  quantize(o, me.x, me.y, me.z, q);
  const int32_t cells = 1 << (BITS - level);
  const int32_t c[3] = {(int32_t)(q[0] >> level), (int32_t)(q[1] >> level), (int32_t)(q[2] >> level)};
  const float p[3] = {me.x, me.y, me.z};
  // 3. The point's own cell, then the 26 around it, each searched down to leaves.
  Best best;
  Frame stack[BITS + 1];
  for (int32_t cell = 0; cell < 27 && best.z != 0.0f; cell++) {
    const int32_t t = cell == 0 ? 13 : (cell <= 13 ? cell - 1 : cell);  // 13 is the centre
    const int32_t cc[3] = {c[0] + t % 3 - 1, c[1] + (t / 3) % 3 - 1, c[2] + t / 9 - 1};
    if (cc[0] < 0 || cc[1] < 0 || cc[2] < 0 || cc[0] >= cells || cc[1] >= cells || cc[2] >= cells) continue;
    const uint32_t uc[3] = {(uint32_t)cc[0], (uint32_t)cc[1], (uint32_t)cc[2]};
    if (cell_gap2(o, p, uc, level) > fminf(window.z, best.z) * 1.000002f) continue;
    const uint64_t prefix = morton(uc[0], uc[1], uc[2]);
    const int32_t begin = lower_bound_from(keys, count, s, prefix << (3 * level));
    const int32_t end = lower_bound_from(keys, count, s, (prefix + 1) << (3 * level));
    if (begin == end) continue;
    int32_t top = 0;
    stack[0] = Frame{{uc[0], uc[1], uc[2]}, begin, end, level, 0};
    while (top >= 0 && best.z != 0.0f) {  // a zero third distance cannot improve
      Frame& f = stack[top];
      if (f.next == 0 && (f.end - f.begin <= LEAF || f.level == 0)) {
        for (int32_t j = f.begin; j < f.end; j++)
          if (j != s) best.offer(distance2(sorted[j], me.x, me.y, me.z));
        top--;
        continue;
      }
      if (f.next == 8) {
        top--;
        continue;
      }
      // Nearest child first: per axis, the half on the point's side.
      const uint32_t cl = f.level - 1;
      uint32_t near = 0;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        const uint32_t pk = q[k] >> f.level;
        const uint32_t side = pk == f.c[k] ? (q[k] >> cl) & 1u : (pk > f.c[k] ? 1u : 0u);
        near |= side << k;
      }
      // Nibble i of `order` is the i-th child's offset from the nearest (XOR):
      // 0, then 1, 2, 4 (one axis apart), 3, 5, 6 (two), 7 (the far corner).
      constexpr uint32_t order = 0x76534210u;
      const uint32_t k = ((order >> (4 * f.next)) & 0xfu) ^ near;
      f.next++;
      const uint32_t ch[3] = {2 * f.c[0] + (k & 1u), 2 * f.c[1] + ((k >> 1) & 1u), 2 * f.c[2] + (k >> 2)};
      if (cell_gap2(o, p, ch, cl) > fminf(window.z, best.z) * 1.000002f) continue;
      const uint64_t cp = morton(ch[0], ch[1], ch[2]);
      const int32_t cb = lower_bound_in(keys, f.begin, f.end, cp << (3 * cl));
      const int32_t ce = lower_bound_in(keys, cb, f.end, (cp + 1) << (3 * cl));
      if (cb == ce) continue;
      stack[++top] = Frame{{ch[0], ch[1], ch[2]}, cb, ce, cl, 0};
    }
  }
  distance2_out[self] = (best.x + best.y + best.z) / 3.0f;  // nearestNeighbors.wgsl:43
}

__global__ void pad_points_kernel(const float* __restrict__ positions, uint32_t n, float4* __restrict__ points) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  points[i] = make_float4(positions[3 * i], positions[3 * i + 1], positions[3 * i + 2], 0.0f);
}

// src/loadDataset.ts:99-121 for point i: the host arithmetic is float64 there, so
// it is float64 here, rounded to float32 on the store as a Float32Array store rounds.
__global__ void initial_gaussians_kernel(const float4* __restrict__ points, const uint8_t* __restrict__ colors,
                                         const float* __restrict__ distance2, uint32_t n, float opacity_logit,
                                         float* __restrict__ params) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p = points[i];
  const double log_scale = 0.5 * log(fmax((double)distance2[i], 1e-7));
  float out[16];
  const float pos[3] = {p.x, p.y, p.z};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    out[k] = pos[k];
    out[4 + k] = (float)log_scale;
    out[12 + k] = (float)(((double)colors[3 * i + k] / 255.0 - 0.5) / 0.28209479177387814);
  }
  out[3] = opacity_logit;
  out[7] = 0.0f;
  out[8] = 1.0f;  // the quaternion (1, 0, 0, 0)
  out[9] = out[10] = out[11] = 0.0f;
  out[15] = 0.0f;
  float4* dst = reinterpret_cast<float4*>(params + (size_t)i * FLOATS_PER_GAUSSIAN);
#pragma unroll
  for (int q = 0; q < 4; q++) dst[q] = make_float4(out[4 * q], out[4 * q + 1], out[4 * q + 2], out[4 * q + 3]);
}

// A stream-ordered allocation freed when it goes out of scope (after the work
// already enqueued on the stream).
struct Scratch {
  cudaStream_t stream;
  void* ptr = nullptr;
  explicit Scratch(cudaStream_t s) : stream(s) {}
  ~Scratch() {
    if (ptr) cudaFreeAsync(ptr, stream);
  }
  template <typename T>
  T* at(size_t offset) const {
    return reinterpret_cast<T*>(static_cast<char*>(ptr) + offset);
  }
};

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// The octree for these bounds and moments.
Octree choose_octree(const Moments& m) {
  Octree o{};
  const double count = m.finite ? (double)m.finite : 1.0;
  double extent = 0.0, maxabs = 0.0;
  for (int k = 0; k < 3; k++) {
    double lo = unordered(m.lo[k]), hi = unordered(m.hi[k]);
    if (!(lo <= hi)) lo = hi = 0.0;  // no finite points
    const double mean = m.sum[k] / count;
    const double sd = std::sqrt(std::max(0.0, m.sum2[k] / count - mean * mean));
    lo = std::max(lo, mean - 3.0 * sd);
    hi = std::min(hi, mean + 3.0 * sd);
    if (!(lo <= hi)) lo = hi = mean;
    o.lo[k] = (float)lo;
    extent = std::max(extent, hi - lo);
    maxabs = std::max(maxabs, std::max(std::fabs(lo), std::fabs(hi)));
  }
  if (!(extent > 0.0) || !std::isfinite(extent)) extent = 1.0;
  const double cells = (double)(1u << BITS);
  o.scale = (float)(cells / extent);
  o.h0 = (float)(extent / cells);
  // Quantizing rounds (p - lo) and the product with scale, and the faces
  // lo + c·h round too: a few finest cells plus a few ulps of the coordinates.
  o.slack = (float)(4.0 * extent / cells + 8.0 * maxabs * 1.2e-7);
  return o;
}

// Mean neighbour distances of n points (float4, xyz + padding) into distance2.
// Blocks on one readback of the bounds.
dg_status neighbor_distance2(dg_context* ctx, const float4* points, uint32_t n, float* distance2) {
  if (n == 0) return DG_OK;
  cudaStream_t st = ctx->stream;
  Moments m{};
  {
    Scratch moments(st);
    DG_CUDA(cudaMallocAsync(&moments.ptr, sizeof(Moments), st));
    Moments init{};
    for (int k = 0; k < 3; k++) init.lo[k] = 0xffffffffu;
    DG_TRY(write_async(ctx, moments.ptr, &init, sizeof init));
    const uint32_t blocks = std::min(ceil_div(n, KNN_THREADS), (uint32_t)ctx->sm_count * 4u);
    DG_LAUNCH(ctx, "knn_bounds", bounds_kernel<<<blocks, KNN_THREADS, 0, st>>>(points, n, moments.at<Moments>(0)));
    DG_CUDA(cudaMemcpyAsync(&m, moments.ptr, sizeof m, cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
  }
  const Octree o = choose_octree(m);
  // 63-bit keys: all 32 low-word bits and 31 high-word bits, 8 even passes.
  const SortPlan plan = sort_plan_digits(n, 2, 3 * BITS - 32);
  const size_t off_values = align256((size_t)n * 8);
  const size_t off_keys_alt = align256(off_values + (size_t)n * 4);
  const size_t off_values_alt = align256(off_keys_alt + (size_t)n * 8);
  const size_t off_sort = align256(off_values_alt + (size_t)n * 4);
  const size_t off_sorted = align256(off_sort + sort_scratch_bytes(plan));
  Scratch scratch(st);
  DG_CUDA(cudaMallocAsync(&scratch.ptr, off_sorted + (size_t)n * 16, st));
  uint2* keys = scratch.at<uint2>(0);
  uint32_t* values = scratch.at<uint32_t>(off_values);
  float4* sorted = scratch.at<float4>(off_sorted);
  const uint32_t grid = ceil_div(n, KNN_THREADS);
  DG_LAUNCH(ctx, "knn_morton", morton_kernel<<<grid, KNN_THREADS, 0, st>>>(points, n, o, keys, values));
  DG_TRY(sort_launch(ctx, plan, keys, values, scratch.at<void>(off_keys_alt), scratch.at<uint32_t>(off_values_alt),
                     nullptr, scratch.at<void>(off_sort)));
  DG_LAUNCH(ctx, "knn_gather", gather_points_kernel<<<grid, KNN_THREADS, 0, st>>>(points, n, values, sorted));
  DG_LAUNCH(ctx, "knn_query", knn_query_kernel<<<grid, KNN_THREADS, 0, st>>>(sorted, keys, n, o, distance2));
  return DG_OK;
}

}  // namespace
}  // namespace dg

using namespace dg;

dg_status dg_mean_neighbor_distance2_buffers(dg_context* ctx, dg_buffer* points, uint32_t count,
                                             dg_buffer* distance2) {
  DG_REQUIRE(ctx && points && distance2, "NULL argument");
  DG_REQUIRE((uint64_t)count * 16 <= points->bytes, "points buffer smaller than count × 16 bytes");
  DG_REQUIRE((uint64_t)count * 4 <= distance2->bytes, "distance2 buffer smaller than count × 4 bytes");
  return neighbor_distance2(ctx, typed<float4>(points), count, typed<float>(distance2));
}

dg_status dg_mean_neighbor_distance2(dg_context* ctx, const float* positions, uint32_t count, float* distance2) {
  DG_REQUIRE(ctx && (count == 0 || (positions && distance2)), "NULL argument");
  if (count == 0) return DG_OK;
  cudaStream_t st = ctx->stream;
  // positions (12 B per point), points (16 B, 16-byte aligned), distance2 (4 B)
  const size_t off_points = align256((size_t)count * 12);
  const size_t off_out = off_points + (size_t)count * 16;
  Scratch dev(st);
  DG_CUDA(cudaMallocAsync(&dev.ptr, off_out + (size_t)count * 4, st));
  float4* points = dev.at<float4>(off_points);
  float* out = dev.at<float>(off_out);
  DG_CUDA(cudaMemcpyAsync(dev.ptr, positions, (size_t)count * 12, cudaMemcpyHostToDevice, st));
  DG_LAUNCH(ctx, "knn_pad_points",
            pad_points_kernel<<<ceil_div(count, KNN_THREADS), KNN_THREADS, 0, st>>>(dev.at<float>(0), count, points));
  DG_TRY(neighbor_distance2(ctx, points, count, out));
  DG_CUDA(cudaMemcpyAsync(distance2, out, (size_t)count * 4, cudaMemcpyDeviceToHost, st));
  DG_CUDA(cudaStreamSynchronize(st));
  return DG_OK;
}

dg_status dg_initial_gaussians(dg_context* ctx, const float* positions, const uint8_t* colors, uint32_t count,
                               float* params, float* sh) {
  DG_REQUIRE(ctx && (count == 0 || (positions && colors && params && sh)), "NULL argument");
  if (count == 0) return DG_OK;
  cudaStream_t st = ctx->stream;
  // positions (12 B), points (16 B), distance2 (4 B), params (64 B), colors (3 B)
  const size_t off_points = align256((size_t)count * 12);
  const size_t off_dist = off_points + (size_t)count * 16;
  const size_t off_params = align256(off_dist + (size_t)count * 4);
  const size_t off_colors = off_params + (size_t)count * 64;
  Scratch dev(st);
  DG_CUDA(cudaMallocAsync(&dev.ptr, off_colors + (size_t)count * 3, st));
  float4* points = dev.at<float4>(off_points);
  float* dist = dev.at<float>(off_dist);
  float* dparams = dev.at<float>(off_params);
  uint8_t* dcolors = dev.at<uint8_t>(off_colors);
  DG_CUDA(cudaMemcpyAsync(dev.ptr, positions, (size_t)count * 12, cudaMemcpyHostToDevice, st));
  DG_CUDA(cudaMemcpyAsync(dcolors, colors, (size_t)count * 3, cudaMemcpyHostToDevice, st));
  const uint32_t grid = ceil_div(count, KNN_THREADS);
  DG_LAUNCH(ctx, "knn_pad_points", pad_points_kernel<<<grid, KNN_THREADS, 0, st>>>(dev.at<float>(0), count, points));
  DG_TRY(neighbor_distance2(ctx, points, count, dist));
  // Math.log(0.1 / 0.9) (src/loadDataset.ts:102), rounded to float32.
  const float opacity_logit = (float)std::log(0.1 / 0.9);
  DG_LAUNCH(ctx, "initial_gaussians", initial_gaussians_kernel<<<grid, KNN_THREADS, 0, st>>>(
                                          points, dcolors, dist, count, opacity_logit, dparams));
  DG_CUDA(cudaMemcpyAsync(params, dparams, (size_t)count * 64, cudaMemcpyDeviceToHost, st));
  DG_CUDA(cudaStreamSynchronize(st));
  std::memset(sh, 0, (size_t)count * SH_REST_FLOATS * 4);  // new Float32Array: zeros
  return DG_OK;
}

// PrefixSum (src/prefixSum.ts:10-103, src/shaders/prefixSum.wgsl:31-91): an
// exclusive scan of u32 values in place, whose length can come from a device
// buffer, writing the grand total to `total[0]`.
//
// The reference runs a 512-value Blelloch scan per workgroup, recursively, with
// 2·levels + 1 dispatches. Here it is ONE launch: a single-pass scan with
// decoupled look-back (Merrill & Garland 2016). Each CTA takes the next tile of
// 4096 values by an atomic ticket (so the tiles before it are already running),
// scans it with warp shuffles, publishes its aggregate, and looks back over its
// predecessors' published values a warp at a time. Every wait is bounded: after
// SPIN_LIMIT polls it sets DEVICE_ERROR_SCAN_WAIT and stops waiting.
#include "dg_common.cuh"
#include "dg_scan.cuh"

#include <cuda/atomic>
#include <string>

namespace dg {

namespace {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;
constexpr uint32_t SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;  // 4096
constexpr uint64_t FLAG_AGGREGATE = 1ull << 62;
constexpr uint64_t FLAG_PREFIX = 2ull << 62;
constexpr uint64_t FLAG_MASK = 3ull << 62;

__device__ __forceinline__ uint64_t load_status(uint64_t* p) {
  cuda::atomic_ref<uint64_t, cuda::thread_scope_device> ref(*p);
  return ref.load(cuda::memory_order_relaxed);
}
__device__ __forceinline__ void store_status(uint64_t* p, uint64_t v) {
  cuda::atomic_ref<uint64_t, cuda::thread_scope_device> ref(*p);
  ref.store(v, cuda::memory_order_relaxed);
}

__device__ __forceinline__ uint32_t warp_inclusive(uint32_t v, int lane) {
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    uint32_t n = __shfl_up_sync(0xffffffffu, v, d);
    if (lane >= d) v += n;
  }
  return v;
}

// With `gather`, value j is source[gather[j]] and data only receives the scan.
__global__ void __launch_bounds__(SCAN_THREADS) scan_kernel(uint32_t* __restrict__ data, uint32_t capacity,
                                                          const uint32_t* __restrict__ count_ptr,
                                                          uint32_t* __restrict__ total, uint64_t* __restrict__ status,
                                                          uint32_t* __restrict__ ticket, uint32_t* __restrict__ error,
                                                          const uint32_t* __restrict__ gather,
                                                          const uint32_t* __restrict__ source) {
  __shared__ uint32_t s_tile;
  __shared__ uint32_t s_warp[SCAN_THREADS / 32];
  __shared__ uint32_t s_prefix;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  uint32_t n = count_ptr ? min(*count_ptr, capacity) : capacity;
  uint32_t tiles = max(1u, (n + SCAN_TILE - 1) / SCAN_TILE);
  // The grid covers the capacity; CTAs past this call's tiles leave at once, and
  // the first `tiles` CTAs take the tickets 0..tiles-1, in arrival order.
  if (blockIdx.x >= tiles) return;
  if (tid == 0) s_tile = atomicAdd(ticket, 1u);
  __syncthreads();
  const uint32_t tile = s_tile;
  if (tile >= tiles) return;

  // Each thread owns SCAN_ITEMS consecutive values.
  const uint64_t base = (uint64_t)tile * SCAN_TILE + (uint64_t)tid * SCAN_ITEMS;
  uint32_t v[SCAN_ITEMS];
  const uint32_t* in = gather ? gather : data;
  const bool full = base + SCAN_ITEMS <= n &&
                    ((reinterpret_cast<uintptr_t>(data) | reinterpret_cast<uintptr_t>(in)) & 15) == 0;
  if (full) {
    const uint4* p = reinterpret_cast<const uint4*>(in + base);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS / 4; k++) {
      uint4 q = p[k];
      v[4 * k] = q.x; v[4 * k + 1] = q.y; v[4 * k + 2] = q.z; v[4 * k + 3] = q.w;
    }
  } else {
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) v[k] = base + k < n ? in[base + k] : 0u;
  }
  if (gather) {  // the 16 gathers of a thread go out together
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) v[k] = base + k < n ? source[v[k]] : 0u;
  }
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) sum += v[k];
  uint32_t incl = warp_inclusive(sum, lane);
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < SCAN_THREADS / 32 ? s_warp[lane] : 0u;
    uint32_t wi = warp_inclusive(w, lane);
    if (lane < SCAN_THREADS / 32) s_warp[lane] = wi - w;  // exclusive per warp
    uint32_t aggregate = __shfl_sync(0xffffffffu, wi, 31);
    // Publish and look back.
    uint32_t exclusive = 0;
    if (tile == 0) {
      if (lane == 0) store_status(&status[0], FLAG_PREFIX | aggregate);
    } else {
      if (lane == 0) store_status(&status[tile], FLAG_AGGREGATE | aggregate);
      int64_t look = (int64_t)tile - 1;
      uint32_t spins = 0;
      while (true) {
        int64_t idx = look - lane;
        uint64_t s = idx >= 0 ? load_status(&status[idx]) : (FLAG_PREFIX | 0ull);
        while (!__all_sync(0xffffffffu, (s & FLAG_MASK) != 0)) {
          if (++spins > SPIN_LIMIT) {
            if (lane == 0) atomicOr(error, DEVICE_ERROR_SCAN_WAIT);
            s = FLAG_PREFIX;  // give up: the values are wrong, but nothing hangs
            break;
          }
          if ((s & FLAG_MASK) == 0) s = load_status(&status[idx]);
        }
        if ((s & FLAG_MASK) == 0) s = FLAG_PREFIX;
        uint32_t prefix_lanes = __ballot_sync(0xffffffffu, (s & FLAG_MASK) == FLAG_PREFIX);
        uint32_t value = (uint32_t)(s & 0xffffffffull);
        if (prefix_lanes) {
          int first = __ffs(prefix_lanes) - 1;  // the nearest predecessor with a full prefix
          uint32_t part = lane <= first ? value : 0u;
#pragma unroll
          for (int d = 16; d > 0; d >>= 1) part += __shfl_xor_sync(0xffffffffu, part, d);
          exclusive += part;
          break;
        }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) value += __shfl_xor_sync(0xffffffffu, value, d);
        exclusive += value;
        look -= 32;
      }
      if (lane == 0) store_status(&status[tile], FLAG_PREFIX | (uint64_t)(uint32_t)(exclusive + aggregate));
    }
    if (lane == 0) {
      s_prefix = exclusive;
      if (tile == tiles - 1) *total = exclusive + aggregate;
    }
  }
  __syncthreads();
  uint32_t running = s_prefix + s_warp[warp] + incl - sum;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    uint32_t x = v[k];
    v[k] = running;
    running += x;
  }
  if (full) {
    uint4* p = reinterpret_cast<uint4*>(data + base);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS / 4; k++) p[k] = make_uint4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
  } else {
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++)
      if (base + k < n) data[base + k] = v[k];
  }
}

__device__ __forceinline__ uint4 ld_u4_hinted(const uint4* p, uint64_t policy) {
  uint4 v;
  asm volatile("ld.global.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;\n"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(p), "l"(policy)
               : "memory");
  return v;
}
__device__ __forceinline__ void st_u4_hinted(uint4* p, uint4 v, uint64_t policy) {
  asm volatile("st.global.L2::cache_hint.v4.u32 [%0], {%1, %2, %3, %4}, %5;\n" ::"l"(p), "r"(v.x), "r"(v.y), "r"(v.z),
               "r"(v.w), "l"(policy)
               : "memory");
}

// Loads a thread's SCAN_ITEMS consecutive values of tile `tile` (zeros past n),
// with L2 eviction policy `policy` (l2_policy_*). `full`: all of them are in
// range and 16-byte aligned.
__device__ __forceinline__ void load_items(const uint32_t* __restrict__ data, uint32_t n, uint32_t tile,
                                           uint32_t (&v)[SCAN_ITEMS], bool& full, uint64_t& base, uint64_t policy) {
  base = (uint64_t)tile * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
  full = base + SCAN_ITEMS <= n && (reinterpret_cast<uintptr_t>(data) & 15) == 0;
  if (full) {
    const uint4* p = reinterpret_cast<const uint4*>(data + base);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS / 4; k++) {
      const uint4 q = ld_u4_hinted(p + k, policy);
      v[4 * k] = q.x; v[4 * k + 1] = q.y; v[4 * k + 2] = q.z; v[4 * k + 3] = q.w;
    }
  } else {
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) v[k] = base + k < n ? data[base + k] : 0u;
  }
}

// Large scans without a gather: reduce, then re-scan each tile from its prefix, the
// sum of the tile sums before it, which each CTA adds up itself from L2 (up to
// FOLD_MAX_TILES tiles; past that a single-pass scan of the tile sums runs in
// between). A second read of the values, but no look-back: in one wave of
// single-pass CTAs, a tile early in the wave waits on a chain of look-backs about
// as long as its place in the wave (at 12M values the single-pass scan ran at
// ~0.3 of the copy rate). The reduce reads the values with an L2 evict-last
// policy (48 MB at 12M values, well inside L2), so the re-scan reads them from
// L2, with evict-first loads and stores as their last use.
__global__ void __launch_bounds__(SCAN_THREADS) scan_reduce_kernel(const uint32_t* __restrict__ data, uint32_t capacity,
                                                                   const uint32_t* __restrict__ count,
                                                                   uint32_t* __restrict__ tile_sums) {
  __shared__ uint32_t s_warp[SCAN_THREADS / 32];
  const uint32_t n = count ? min(*count, capacity) : capacity;
  uint32_t v[SCAN_ITEMS];
  bool full;
  uint64_t base;
  load_items(data, n, blockIdx.x, v, full, base, l2_policy_evict_last());
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) sum += v[k];
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, d);
  if ((threadIdx.x & 31) == 0) s_warp[threadIdx.x >> 5] = sum;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
#pragma unroll
    for (int w = 0; w < SCAN_THREADS / 32; w++) t += s_warp[w];
    tile_sums[blockIdx.x] = t;
  }
}

// fold: tile_sums holds each tile's sum, and each CTA adds up those before its
// own; the last tile's CTA writes the grand total. Otherwise tile_sums holds the
// scanned tile sums (each tile's exclusive prefix) and `total` is not touched.
__global__ void __launch_bounds__(SCAN_THREADS) scan_tiles_kernel(uint32_t* __restrict__ data, uint32_t capacity,
                                                                  const uint32_t* __restrict__ count,
                                                                  const uint32_t* __restrict__ tile_sums, bool fold,
                                                                  uint32_t* __restrict__ total) {
  __shared__ uint32_t s_warp[SCAN_THREADS / 32];
  __shared__ uint32_t s_part[SCAN_THREADS / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t n = count ? min(*count, capacity) : capacity;
  const uint32_t tiles = (uint32_t)(((uint64_t)n + SCAN_TILE - 1) / SCAN_TILE);  // tiles holding values
  if (blockIdx.x >= tiles) {  // the whole CTA
    if (fold && n == 0 && blockIdx.x == 0 && tid == 0) *total = 0;
    return;
  }
  // The tile sums before this tile (L2 reads, issued with the tile's own loads).
  uint32_t part = 0;
  if (fold)
    for (uint32_t j = tid; j < blockIdx.x; j += SCAN_THREADS) part += tile_sums[j];
  const uint64_t last_use = l2_policy_evict_first();
  uint32_t v[SCAN_ITEMS];
  bool full;
  uint64_t base;
  load_items(data, n, blockIdx.x, v, full, base, last_use);
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) sum += v[k];
  const uint32_t incl = warp_inclusive(sum, lane);
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) part += __shfl_xor_sync(0xffffffffu, part, d);
  if (lane == 31) s_warp[warp] = incl;
  if (lane == 0) s_part[warp] = part;
  __syncthreads();
  uint32_t before = 0;
  if (fold) {
#pragma unroll
    for (int w = 0; w < SCAN_THREADS / 32; w++) before += s_part[w];
  } else {
    before = tile_sums[blockIdx.x];
  }
#pragma unroll
  for (int w = 0; w < SCAN_THREADS / 32; w++) before += w < warp ? s_warp[w] : 0u;
  uint32_t running = before + incl - sum;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    const uint32_t x = v[k];
    v[k] = running;
    running += x;
  }
  if (fold && blockIdx.x == tiles - 1 && tid == SCAN_THREADS - 1) *total = running;
  if (full) {
    uint4* p = reinterpret_cast<uint4*>(data + base);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS / 4; k++)
      st_u4_hinted(p + k, make_uint4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]), last_use);
  } else {
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++)
      if (base + k < n) data[base + k] = v[k];
  }
}

// From this many values (and without a gather) the two-level scan runs: at 1.1M
// values the single pass is faster (16 us against 21), at 12M the two-level one
// (37 us against 49).
constexpr uint32_t TWO_LEVEL_MIN = 1u << 21;
// Up to this many tiles (16.7M values) each re-scanning CTA adds up the tile sums
// before it itself (at most 16 L2 reads a thread).
constexpr uint32_t FOLD_MAX_TILES = 4096;

size_t single_pass_scratch_bytes(uint32_t capacity) {
  uint32_t tiles = std::max(1u, ceil_div(capacity, SCAN_TILE));
  return 256 + (size_t)tiles * sizeof(uint64_t);
}

}  // namespace

size_t scan_scratch_bytes(uint32_t capacity) {
  const size_t single = single_pass_scratch_bytes(capacity);
  if (capacity < TWO_LEVEL_MIN) return single;
  // Two-level: the tile sums, then the single-pass scan's scratch for scanning them.
  const uint32_t tiles = std::max(1u, ceil_div(capacity, SCAN_TILE));
  const size_t sums = ((size_t)tiles * 4 + 255) & ~(size_t)255;
  return std::max(single, sums + single_pass_scratch_bytes(tiles));
}

dg_status scan_launch(dg_context* ctx, uint32_t* data, uint32_t capacity, const uint32_t* count, uint32_t* total,
                      void* scratch, const uint32_t* gather, const uint32_t* source) {
  uint32_t tiles = std::max(1u, ceil_div(capacity, SCAN_TILE));
  if (!gather && capacity >= TWO_LEVEL_MIN) {
    auto* sums = static_cast<uint32_t*>(scratch);
    void* inner = static_cast<char*>(scratch) + (((size_t)tiles * 4 + 255) & ~(size_t)255);
    DG_LAUNCH(ctx, "scan_reduce",
              scan_reduce_kernel<<<tiles, SCAN_THREADS, 0, ctx->stream>>>(data, capacity, count, sums));
    const bool fold = tiles <= FOLD_MAX_TILES;
    if (!fold) DG_TRY(scan_launch(ctx, sums, tiles, nullptr, total, inner));  // tiles < TWO_LEVEL_MIN: single pass
    DG_LAUNCH(ctx, "scan",
              scan_tiles_kernel<<<tiles, SCAN_THREADS, 0, ctx->stream>>>(data, capacity, count, sums, fold, total));
    return DG_OK;
  }
  auto* ticket = static_cast<uint32_t*>(scratch);
  auto* status = reinterpret_cast<uint64_t*>(static_cast<char*>(scratch) + 256);
  DG_CUDA(cudaMemsetAsync(scratch, 0, single_pass_scratch_bytes(capacity), ctx->stream));
  DG_LAUNCH(ctx, "scan",
            scan_kernel<<<tiles, SCAN_THREADS, 0, ctx->stream>>>(data, capacity, count, total, status, ticket,
                                                                 ctx->device_error, gather, source));
  return DG_OK;
}

// ---------------------------------------------------------------------------
// The scan for callers that cannot allocate device memory.
//
// Some callers must not call cudaMalloc or any allocating routine: code that runs
// under a memory budget fixed up front, code that cannot tolerate the implicit
// synchronization an allocation may cause, or hosts that own every allocation
// themselves. For them, dg_prefix_sum_no_alloc keeps the scan's look-back state
// (a ticket, an error word and one status word per 4096-value tile) in the
// file-scope array below instead of a buffer it allocates. The array is sized for
// NO_ALLOC_MAX_VALUES values and, like any __device__ variable, is held by every
// GPU that loads the library until the process exits.
constexpr uint32_t NO_ALLOC_MAX_VALUES = 1u << 24;
constexpr uint32_t NO_ALLOC_MAX_TILES = NO_ALLOC_MAX_VALUES / SCAN_TILE;     // 4096
constexpr size_t NO_ALLOC_BYTES = 256 + (size_t)NO_ALLOC_MAX_TILES * 8;      // ~32.25 KB
static __device__ __align__(256) unsigned char g_no_alloc_scratch[NO_ALLOC_BYTES];

// Host code must not use g_no_alloc_scratch's name as an address: on the host it
// is only a stand-in for the symbol. Each call looks up the device address on
// the current device, which must be the stream's. The lookup is cheap once the
// library's module is loaded on that device (the first call there loads it);
// a fresh lookup on every call stays right after cudaDeviceReset or under another
// context, where a cached address would point at freed memory.
constexpr uint32_t NO_ALLOC_ERROR_OFFSET = 4;  // the give-up word, after the ticket

static dg_status no_alloc_scratch_address(cudaStream_t stream, void** out) {
  int device = -1, stream_device = -1;
  DG_CUDA(cudaGetDevice(&device));
  DG_CUDA(cudaStreamGetDevice(stream, &stream_device));
  DG_REQUIRE(stream_device == device, "the stream belongs to another device than the current one");
  void* ptr = nullptr;
  cudaError_t err = cudaGetSymbolAddress(&ptr, g_no_alloc_scratch);
  if (err != cudaSuccess) return cuda_fail(err, "cudaGetSymbolAddress(no-alloc scan scratch)");
  *out = ptr;
  return DG_OK;
}

}  // namespace dg

using namespace dg;

extern "C" dg_status dg_prefix_sum_no_alloc(void* stream, uint32_t* data, uint32_t count, uint32_t* total) {
  DG_REQUIRE(data && total, "NULL argument");
  if (count > NO_ALLOC_MAX_VALUES)
    return fail(DG_ERROR_INVALID_ARGUMENT, "dg_prefix_sum_no_alloc scans at most " +
                                               std::to_string(NO_ALLOC_MAX_VALUES) + " values; got " +
                                               std::to_string(count));
  auto s = static_cast<cudaStream_t>(stream);
  void* scratch = nullptr;
  DG_TRY(no_alloc_scratch_address(s, &scratch));
  const uint32_t tiles = std::max(1u, ceil_div(count, SCAN_TILE));
  auto* ticket = static_cast<uint32_t*>(scratch);
  auto* error = reinterpret_cast<uint32_t*>(static_cast<char*>(scratch) + NO_ALLOC_ERROR_OFFSET);
  auto* status = reinterpret_cast<uint64_t*>(static_cast<char*>(scratch) + 256);
  // The previous call left its ticket and status words behind: clear what this
  // call's tiles will read. The give-up word is left alone: it keeps any earlier
  // give-up until dg_prefix_sum_no_alloc_check reads and clears it.
  DG_CUDA(cudaMemsetAsync(ticket, 0, sizeof(uint32_t), s));
  DG_CUDA(cudaMemsetAsync(status, 0, (size_t)tiles * sizeof(uint64_t), s));
  scan_kernel<<<tiles, SCAN_THREADS, 0, s>>>(data, count, nullptr, total, status, ticket, error, nullptr,
                                                          nullptr);
  DG_CUDA(cudaGetLastError());
  return DG_OK;
}

// Waits for the stream, then reads and clears the give-up word that the scan's
// bounded look-back sets instead of hanging.
extern "C" dg_status dg_prefix_sum_no_alloc_check(void* stream, uint32_t* bits) {
  auto s = static_cast<cudaStream_t>(stream);
  void* scratch = nullptr;
  DG_TRY(no_alloc_scratch_address(s, &scratch));
  auto* error = reinterpret_cast<uint32_t*>(static_cast<char*>(scratch) + NO_ALLOC_ERROR_OFFSET);
  uint32_t value = 0;
  DG_CUDA(cudaMemcpyAsync(&value, error, sizeof(value), cudaMemcpyDeviceToHost, s));
  DG_CUDA(cudaStreamSynchronize(s));
  if (bits) *bits = value;
  if (value) {
    DG_CUDA(cudaMemsetAsync(error, 0, sizeof(uint32_t), s));
    DG_CUDA(cudaStreamSynchronize(s));
    return fail(DG_ERROR_DEVICE_WAIT,
                "a look-back of dg_prefix_sum_no_alloc gave up waiting; the results since the last check are wrong "
                "(error bits " + std::to_string(value) + ")");
  }
  return DG_OK;
}

// Test hook: ORs bits into the give-up word, as a timed-out look-back would, so
// that the reporting path can be tested without making a GPU wait run out.
extern "C" dg_status dg_prefix_sum_no_alloc_inject_error(void* stream, uint32_t bits) {
  auto s = static_cast<cudaStream_t>(stream);
  void* scratch = nullptr;
  DG_TRY(no_alloc_scratch_address(s, &scratch));
  auto* error = reinterpret_cast<uint32_t*>(static_cast<char*>(scratch) + NO_ALLOC_ERROR_OFFSET);
  uint32_t value = 0;
  DG_CUDA(cudaMemcpyAsync(&value, error, sizeof(value), cudaMemcpyDeviceToHost, s));
  DG_CUDA(cudaStreamSynchronize(s));
  value |= bits;
  DG_CUDA(cudaMemcpyAsync(error, &value, sizeof(value), cudaMemcpyHostToDevice, s));
  DG_CUDA(cudaStreamSynchronize(s));
  return DG_OK;
}

struct dg_prefix_sum {
  dg_context* ctx;
  dg_buffer* data;
  dg_buffer* count;  // borrowed, may be NULL
  uint32_t capacity;
  dg_buffer* total;
  dg_buffer* scratch;
};

extern "C" {

dg_status dg_prefix_sum_create(dg_context* ctx, dg_buffer* data, uint32_t capacity, dg_buffer* count,
                               dg_prefix_sum** out) {
  DG_REQUIRE(ctx && data && out, "NULL argument");
  DG_REQUIRE((uint64_t)capacity * 4 <= data->bytes, "capacity exceeds the data buffer");
  DG_REQUIRE(!count || count->bytes >= 4, "count buffer too small");
  auto* s = new dg_prefix_sum{ctx, data, count, capacity, nullptr, nullptr};
  dg_status st = alloc_buffer(ctx, 4, &s->total);
  if (st == DG_OK) st = alloc_buffer(ctx, scan_scratch_bytes(capacity), &s->scratch);
  if (st != DG_OK) {
    dg_prefix_sum_destroy(s);
    return st;
  }
  *out = s;
  return DG_OK;
}

dg_status dg_prefix_sum_encode(dg_prefix_sum* s) {
  DG_REQUIRE(s, "NULL argument");
  return scan_launch(s->ctx, typed<uint32_t>(s->data), s->capacity, s->count ? typed<uint32_t>(s->count) : nullptr,
                     typed<uint32_t>(s->total), s->scratch->ptr);
}

dg_buffer* dg_prefix_sum_total(dg_prefix_sum* s) { return s ? s->total : nullptr; }

dg_status dg_prefix_sum_destroy(dg_prefix_sum* s) {
  if (!s) return DG_OK;
  free_buffer(s->total);
  free_buffer(s->scratch);
  delete s;
  return DG_OK;
}

}  // extern "C"

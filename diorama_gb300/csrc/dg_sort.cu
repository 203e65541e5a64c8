// RadixSort (src/radixSort.ts:27-142, src/shaders/radixSort.wgsl:45-120): a
// stable LSD radix sort of u32 keys, or u64 keys stored as (low, high) of which
// the high word contributes `high_bits` bits, each key carrying a u32 value.
//
// The pass plan is the reference's: 8-bit digits, four passes over the low word,
// then 2·ceil(high_bits/16) over the high word, ping-ponging so the result lands
// back in keys/values. Any stable LSD sort over the same digits yields the same
// permutation, so the result is bit-identical to the reference's.
//
// The reference runs count_digits, a multi-level scan and scatter per pass (three
// or more dispatches and four barriers per 256-key chunk). Here it is onesweep
// (Adinets & Merrill 2022): one upfront kernel reads every key once and builds
// the digit histograms of all passes, then each pass is ONE kernel. A CTA takes
// the next tile of 3840 keys by ticket, ranks each key within its warp with
// ballots (stable: warp-striped loads are ranked round by round), publishes its
// per-digit counts, looks back over earlier tiles' counts (bounded waits), and
// scatters through shared memory so each digit's run is written contiguously.
#include "dg_common.cuh"
#include "dg_scan.cuh"

#include <cuda/atomic>

namespace dg {

namespace {

constexpr int SORT_THREADS = 256;
constexpr int SORT_WARPS = SORT_THREADS / 32;
#ifndef DG_SORT_ITEMS
#define DG_SORT_ITEMS 15
#endif
#ifndef DG_SORT_MIN_BLOCKS
#define DG_SORT_MIN_BLOCKS 3  // resident CTAs per SM the pass kernel's registers allow
#endif
// Keys per thread: 15 at 3 CTAs per SM measured fastest (per in-step pass 29.0 us,
// 26M keys 1,319 us) against 8 and 11 (36.0, 30.8 us: smaller tiles, longer
// look-backs) and 19 and 23 at 2 CTAs per SM (31.5, 30.7 us).
constexpr int SORT_ITEMS = DG_SORT_ITEMS;
constexpr uint32_t WARP_ITEMS = 32 * SORT_ITEMS;             // 480
constexpr uint32_t SORT_TILE = SORT_THREADS * SORT_ITEMS;    // 3840
constexpr uint32_t RADIX = 256;
constexpr uint32_t FLAG_AGGREGATE = 1u << 30;
constexpr uint32_t FLAG_PREFIX = 2u << 30;
constexpr uint32_t FLAG_MASK = 3u << 30;
constexpr uint32_t VALUE_MASK = (1u << 30) - 1;
constexpr int HIST_THREADS = 256;
constexpr int MAX_PASSES = 8;
#ifndef DG_SORT_LOOK_WIDTH
#define DG_SORT_LOOK_WIDTH 4
#endif
constexpr int LOOK_WIDTH = DG_SORT_LOOK_WIDTH;  // predecessors read per look-back step (4-32 measured: 4-8 best)

template <int KW>
struct KeyOf;
template <>
struct KeyOf<1> {
  using type = uint32_t;
};
template <>
struct KeyOf<2> {
  using type = uint64_t;
};

__device__ __forceinline__ uint32_t load_status(uint32_t* p) {
  cuda::atomic_ref<uint32_t, cuda::thread_scope_device> ref(*p);
  return ref.load(cuda::memory_order_relaxed);
}
__device__ __forceinline__ void store_status(uint32_t* p, uint32_t v) {
  cuda::atomic_ref<uint32_t, cuda::thread_scope_device> ref(*p);
  ref.store(v, cuda::memory_order_relaxed);
}

struct PassShifts {
  uint32_t shift[MAX_PASSES];
};

// Digit histograms of every pass from one read of the keys. Each thread takes
// HIST_ITEMS consecutive keys and counts runs of equal digits in a register,
// adding a run to the CTA's shared histogram when the digit changes: a splat's
// pairs sit next to each other with the same depth and nearby tiles, so runs are
// common, and the lanes of a warp rarely land on one bin in the same instant.
constexpr uint32_t HIST_ITEMS = 8;
#ifndef DG_HIST_ROUNDS
// HIST_ITEMS-key rounds per thread the grid is sized for (at most 8 CTAs per SM):
// 1, 2 and 4 measured 16.7, 16.0 and 17.0 us per in-step histogram.
#define DG_HIST_ROUNDS 2
#endif

template <int KW>
__global__ void __launch_bounds__(HIST_THREADS) sort_histogram_kernel(const typename KeyOf<KW>::type* __restrict__ keys,
                                                                      uint32_t capacity, const uint32_t* __restrict__ count,
                                                                      uint32_t passes, PassShifts shifts,
                                                                      uint32_t* __restrict__ hist) {
  using K = typename KeyOf<KW>::type;
  __shared__ uint32_t s_hist[MAX_PASSES][RADIX];
  for (uint32_t i = threadIdx.x; i < passes * RADIX; i += HIST_THREADS) s_hist[i / RADIX][i % RADIX] = 0;
  __syncthreads();
  const uint32_t n = count ? min(*count, capacity) : capacity;
  const uint64_t stride = (uint64_t)gridDim.x * HIST_THREADS * HIST_ITEMS;
  for (uint64_t base = ((uint64_t)blockIdx.x * HIST_THREADS + threadIdx.x) * HIST_ITEMS; base < n; base += stride) {
    K k[HIST_ITEMS];
    const uint64_t left = (uint64_t)n - base;
    const uint32_t m = left < HIST_ITEMS ? (uint32_t)left : HIST_ITEMS;
    if (m == HIST_ITEMS && (reinterpret_cast<uintptr_t>(keys + base) & 15) == 0) {
      // 16-byte loads (base is a multiple of 8 keys: 32 or 64 bytes in).
      const uint4* src = reinterpret_cast<const uint4*>(keys + base);
#pragma unroll
      for (uint32_t q = 0; q < HIST_ITEMS * sizeof(K) / 16; q++)
        reinterpret_cast<uint4*>(k)[q] = src[q];
    } else {
#pragma unroll
      for (uint32_t j = 0; j < HIST_ITEMS; j++) k[j] = j < m ? keys[base + j] : K(0);
    }
    for (uint32_t p = 0; p < passes; p++) {
      uint32_t run_digit = (uint32_t)((uint64_t)k[0] >> shifts.shift[p]) & 0xffu, run = 1;
#pragma unroll
      for (uint32_t j = 1; j < HIST_ITEMS; j++) {
        if (j >= m) break;
        const uint32_t d = (uint32_t)((uint64_t)k[j] >> shifts.shift[p]) & 0xffu;
        if (d == run_digit) {
          run++;
        } else {
          atomicAdd(&s_hist[p][run_digit], run);
          run_digit = d;
          run = 1;
        }
      }
      atomicAdd(&s_hist[p][run_digit], run);
    }
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < passes * RADIX; i += HIST_THREADS) {
    uint32_t c = s_hist[i / RADIX][i % RADIX];
    if (c) atomicAdd(&hist[i], c);
  }
}

// Exclusive scan of one value per thread over the CTA's 256 threads.
__device__ __forceinline__ uint32_t block_exclusive_256(uint32_t v, uint32_t* s_tmp) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    uint32_t n = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += n;
  }
  if (lane == 31) s_tmp[warp] = incl;
  __syncthreads();
  uint32_t before = 0;
#pragma unroll
  for (int w = 0; w < SORT_WARPS; w++) before += w < warp ? s_tmp[w] : 0u;
  __syncthreads();
  return before + incl - v;
}

// One pass over digits of DBITS bits (8, or 4 for a last pass whose key bits
// above it are all zero): fewer ballots per key, and with 16 digits the per-tile
// prefix work and look-back run on 16 threads instead of 256.
template <int KW, int DBITS>
__global__ void __launch_bounds__(SORT_THREADS, DG_SORT_MIN_BLOCKS)
    sort_pass_kernel(const typename KeyOf<KW>::type* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
                     typename KeyOf<KW>::type* __restrict__ keys_out, uint32_t* __restrict__ vals_out,
                     uint32_t capacity, const uint32_t* __restrict__ count, uint32_t shift,
                     const uint32_t* __restrict__ pass_hist, uint32_t* __restrict__ status,
                     uint32_t* __restrict__ ticket, uint32_t* __restrict__ error) {
  using K = typename KeyOf<KW>::type;
  extern __shared__ __align__(16) unsigned char smem[];
  K* s_keys = reinterpret_cast<K*>(smem);
  uint32_t* s_vals = reinterpret_cast<uint32_t*>(s_keys + SORT_TILE);
  uint32_t* s_whist = s_vals + SORT_TILE;          // [warp][digit]
  uint32_t* s_block_start = s_whist + SORT_WARPS * RADIX;
  uint32_t* s_base = s_block_start + RADIX;
  uint32_t* s_tmp = s_base + RADIX;
  __shared__ uint32_t s_tile;

  constexpr uint32_t DIGITS = 1u << DBITS, DMASK = DIGITS - 1u;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t n = count ? min(*count, capacity) : capacity;
  const uint32_t tiles = (n + SORT_TILE - 1) / SORT_TILE;
  // The grid covers the capacity; CTAs past the tiles of this call's keys leave at
  // once. The first `tiles` CTAs take the tickets 0..tiles-1, in arrival order.
  if (blockIdx.x >= tiles) return;
  if (tid == 0) s_tile = atomicAdd(ticket, 1u);
  for (int i = tid; i < SORT_WARPS * RADIX; i += SORT_THREADS) s_whist[i] = 0;
  __syncthreads();
  const uint32_t tile = s_tile;
  if (tile >= tiles) return;

  // Load, warp-striped: warp w owns keys [w*480, w*480+480) of the tile, round j
  // reads 32 consecutive ones, so order within the tile is (warp, round, lane).
  const uint32_t base = tile * SORT_TILE + warp * WARP_ITEMS + lane;
  K key[SORT_ITEMS];
  uint32_t val[SORT_ITEMS];
  uint32_t rank[SORT_ITEMS];
#pragma unroll
  for (int j = 0; j < SORT_ITEMS; j++) {
    uint32_t idx = base + j * 32;
    bool valid = idx < n;
    key[j] = valid ? keys_in[idx] : K(0);
    val[j] = valid ? vals_in[idx] : 0u;
  }
  const uint32_t lt_mask = (1u << lane) - 1u;
  uint32_t* my_hist = s_whist + warp * DIGITS;
#pragma unroll
  for (int j = 0; j < SORT_ITEMS; j++) {
    bool valid = base + j * 32 < n;
    uint32_t d = (uint32_t)(key[j] >> shift) & DMASK;
    uint32_t peers = __ballot_sync(0xffffffffu, valid);
#pragma unroll
    for (int b = 0; b < DBITS; b++) {
      uint32_t bit = (d >> b) & 1u;
      uint32_t vote = __ballot_sync(0xffffffffu, bit);
      peers &= bit ? vote : ~vote;
    }
    int leader = valid ? __ffs(peers) - 1 : lane;
    uint32_t old = 0;
    if (valid && lane == leader) {
      old = my_hist[d];
      my_hist[d] = old + __popc(peers);
    }
    old = __shfl_sync(0xffffffffu, old, leader);
    rank[j] = old + __popc(peers & lt_mask);
    __syncwarp();
  }
  __syncthreads();

  // Per digit (thread = digit, threads past the digits idle): offsets of each
  // warp's run, and the tile's count.
  const uint32_t d = tid;
  const bool digit = d < DIGITS;
  uint32_t running = 0;
  if (digit) {
#pragma unroll
    for (int w = 0; w < SORT_WARPS; w++) {
      uint32_t c = s_whist[w * DIGITS + d];
      s_whist[w * DIGITS + d] = running;
      running += c;
    }
    store_status(&status[tile * RADIX + d], (tile == 0 ? FLAG_PREFIX : FLAG_AGGREGATE) | running);
  }
  const uint32_t tile_count = running;
  const uint32_t block_start = block_exclusive_256(tile_count, s_tmp);
  const uint32_t global_start = block_exclusive_256(digit ? pass_hist[d] : 0u, s_tmp);
  if (digit) s_block_start[d] = block_start;

  // Decoupled look-back over earlier tiles, for this thread's digit: the states
  // of LOOK_WIDTH predecessors are read together (one round trip instead of
  // LOOK_WIDTH), then taken in order back to the first inclusive prefix.
  uint32_t prefix = 0;
  if (digit && tile > 0) {
    int32_t look = (int32_t)tile - 1;
    uint32_t spins = 0;
    bool found = false;
    while (look >= 0 && !found) {
      uint32_t st[LOOK_WIDTH];
#pragma unroll
      for (int k = 0; k < LOOK_WIDTH; k++)
        st[k] = look - k >= 0 ? load_status(&status[(look - k) * RADIX + d]) : FLAG_PREFIX;
#pragma unroll
      for (int k = 0; k < LOOK_WIDTH; k++) {
        if (found || look - k < 0) break;
        uint32_t s = st[k];
        while ((s & FLAG_MASK) == 0) {
          if (++spins > SPIN_LIMIT) {
            atomicOr(error, DEVICE_ERROR_SORT_WAIT);
            s = FLAG_PREFIX;  // give up: the order is wrong, but nothing hangs
            break;
          }
          s = load_status(&status[(look - k) * RADIX + d]);
        }
        prefix += s & VALUE_MASK;
        found = (s & FLAG_MASK) == FLAG_PREFIX;
      }
      look -= LOOK_WIDTH;
    }
    store_status(&status[tile * RADIX + d], FLAG_PREFIX | ((prefix + tile_count) & VALUE_MASK));
  }
  if (digit) s_base[d] = global_start + prefix - block_start;
  __syncthreads();

  // Place each key at its rank within the tile, grouped by digit.
#pragma unroll
  for (int j = 0; j < SORT_ITEMS; j++) {
    if (base + j * 32 < n) {
      uint32_t dj = (uint32_t)(key[j] >> shift) & DMASK;
      uint32_t pos = s_block_start[dj] + s_whist[warp * DIGITS + dj] + rank[j];
      s_keys[pos] = key[j];
      s_vals[pos] = val[j];
    }
  }
  __syncthreads();
  const uint32_t here = min(SORT_TILE, n - tile * SORT_TILE);
  for (uint32_t k = tid; k < here; k += SORT_THREADS) {
    K kk = s_keys[k];
    uint32_t dk = (uint32_t)(kk >> shift) & DMASK;
    uint32_t out = s_base[dk] + k;
    // Only a look-back that gave up (error bit already set) can place a key
    // outside the output; drop it rather than write out of bounds.
    if (out >= n) continue;
    keys_out[out] = kk;
    vals_out[out] = s_vals[k];
  }
}

template <int KW>
size_t pass_smem_bytes() {
  return SORT_TILE * (sizeof(typename KeyOf<KW>::type) + 4) + (SORT_WARPS * RADIX + 2 * RADIX + 32) * 4;
}

struct ScratchLayout {
  size_t tickets, hist, status, total;
  uint32_t max_tiles;
};

ScratchLayout layout_of(const SortPlan& plan) {
  ScratchLayout l;
  l.max_tiles = std::max(1u, ceil_div(plan.capacity, SORT_TILE));
  l.tickets = 0;
  l.hist = 256;
  l.status = l.hist + (size_t)plan.passes * RADIX * 4;
  l.total = l.status + (size_t)plan.passes * l.max_tiles * RADIX * 4;
  return l;
}

template <int KW>
dg_status launch_typed(dg_context* ctx, const SortPlan& plan, void* keys, uint32_t* values, void* keys_alt,
                       uint32_t* values_alt, const uint32_t* count, void* scratch) {
  using K = typename KeyOf<KW>::type;
  ScratchLayout l = layout_of(plan);
  char* s = static_cast<char*>(scratch);
  auto* tickets = reinterpret_cast<uint32_t*>(s + l.tickets);
  auto* hist = reinterpret_cast<uint32_t*>(s + l.hist);
  auto* status = reinterpret_cast<uint32_t*>(s + l.status);
  DG_CUDA(cudaMemsetAsync(scratch, 0, l.total, ctx->stream));
  PassShifts shifts{};
  for (uint32_t p = 0; p < plan.passes; p++) shifts.shift[p] = plan.shift[p];
  uint32_t hist_blocks =
      std::min<uint32_t>(ceil_div(plan.capacity, HIST_THREADS * HIST_ITEMS * DG_HIST_ROUNDS), (uint32_t)ctx->sm_count * 8);
  hist_blocks = std::max(1u, hist_blocks);
  DG_LAUNCH(ctx, "sort_histogram",
            sort_histogram_kernel<KW><<<hist_blocks, HIST_THREADS, 0, ctx->stream>>>(
                static_cast<const K*>(keys), plan.capacity, count, plan.passes, shifts, hist));
  size_t smem = pass_smem_bytes<KW>();
  K* in_k = static_cast<K*>(keys);
  uint32_t* in_v = values;
  K* out_k = static_cast<K*>(keys_alt);
  uint32_t* out_v = values_alt;
  for (uint32_t p = 0; p < plan.passes; p++) {
    const auto kernel = plan.narrow_last && p + 1 == plan.passes ? sort_pass_kernel<KW, 4> : sort_pass_kernel<KW, 8>;
    DG_LAUNCH(ctx, "sort_pass",
              kernel<<<l.max_tiles, SORT_THREADS, smem, ctx->stream>>>(
                  in_k, in_v, out_k, out_v, plan.capacity, count, shifts.shift[p], hist + p * RADIX,
                  status + (size_t)p * l.max_tiles * RADIX, tickets + p, ctx->device_error));
    std::swap(in_k, out_k);
    std::swap(in_v, out_v);
  }
  return DG_OK;
}

}  // namespace

dg_status sort_init() {
  // The pass kernels use more than the default 48 KB of dynamic shared memory.
  DG_CUDA(cudaFuncSetAttribute(sort_pass_kernel<1, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)pass_smem_bytes<1>()));
  DG_CUDA(cudaFuncSetAttribute(sort_pass_kernel<1, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)pass_smem_bytes<1>()));
  DG_CUDA(cudaFuncSetAttribute(sort_pass_kernel<2, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)pass_smem_bytes<2>()));
  DG_CUDA(cudaFuncSetAttribute(sort_pass_kernel<2, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)pass_smem_bytes<2>()));
  return DG_OK;
}

SortPlan sort_plan(uint32_t capacity, uint32_t high_bits) {
  SortPlan p{};
  p.capacity = capacity;
  p.key_words = high_bits > 0 ? 2 : 1;
  p.high_bits = high_bits;
  p.passes = 4 + 2 * ((high_bits + 15) / 16);
  for (uint32_t k = 0; k < p.passes; k++) p.shift[k] = k < 4 ? k * 8 : 32 + (k - 4) * 8;
  return p;
}

SortPlan sort_plan_low_bits(uint32_t capacity, uint32_t bits) {
  SortPlan p{};
  p.capacity = capacity;
  p.key_words = 1;
  p.high_bits = 0;
  p.passes = 2 * ((bits + 15) / 16);
  for (uint32_t k = 0; k < p.passes; k++) p.shift[k] = k * 8;
  return p;
}

SortPlan sort_plan_digits(uint32_t capacity, uint32_t key_words, uint32_t bits) {
  SortPlan p{};
  p.capacity = capacity;
  p.key_words = key_words;
  p.high_bits = key_words == 2 ? bits : 0;
  p.passes = key_words == 2 ? 4 + (bits + 7) / 8 : std::max(1u, (bits + 7) / 8);
  for (uint32_t k = 0; k < p.passes; k++) p.shift[k] = k * 8;
  sort_plan_key_bits(p, key_words == 2 ? 32 + bits : bits);
  return p;
}

void sort_plan_key_bits(SortPlan& p, uint32_t bits) {
  // The last pass's digit: bits [shift, shift + 8) of the key; only `bits` vary.
  const uint32_t last = p.shift[p.passes - 1];
  p.narrow_last = bits <= last + 4;
}

size_t sort_scratch_bytes(const SortPlan& plan) { return layout_of(plan).total; }

dg_status sort_launch(dg_context* ctx, const SortPlan& plan, void* keys, uint32_t* values, void* keys_alt,
                      uint32_t* values_alt, const uint32_t* count, void* scratch) {
  if (plan.key_words == 2)
    return launch_typed<2>(ctx, plan, keys, values, keys_alt, values_alt, count, scratch);
  return launch_typed<1>(ctx, plan, keys, values, keys_alt, values_alt, count, scratch);
}

}  // namespace dg

using namespace dg;

struct dg_radix_sort {
  dg_context* ctx;
  SortPlan plan;
  dg_buffer* keys;
  dg_buffer* values;
  dg_buffer* keys_alt;
  dg_buffer* values_alt;
  dg_buffer* scratch;
  dg_buffer* count;  // borrowed, may be NULL
};

extern "C" {

dg_status dg_radix_sort_create(dg_context* ctx, uint32_t capacity, uint32_t high_bits, dg_buffer* count,
                               dg_radix_sort** out) {
  DG_REQUIRE(ctx && out, "NULL argument");
  DG_REQUIRE(high_bits <= 32, "high_bits is at most 32");
  DG_REQUIRE(capacity < (1u << 30), "capacity must be below 2^30 keys");
  DG_REQUIRE(!count || count->bytes >= 4, "count buffer too small");
  auto* s = new dg_radix_sort{ctx, sort_plan(capacity, high_bits), nullptr, nullptr, nullptr, nullptr, nullptr, count};
  size_t kb = (size_t)capacity * (high_bits > 0 ? 8 : 4);
  dg_status st = alloc_buffer(ctx, kb, &s->keys);
  if (st == DG_OK) st = alloc_buffer(ctx, (size_t)capacity * 4, &s->values);
  if (st == DG_OK) st = alloc_buffer(ctx, kb, &s->keys_alt);
  if (st == DG_OK) st = alloc_buffer(ctx, (size_t)capacity * 4, &s->values_alt);
  if (st == DG_OK) st = alloc_buffer(ctx, sort_scratch_bytes(s->plan), &s->scratch);
  if (st != DG_OK) {
    dg_radix_sort_destroy(s);
    return st;
  }
  *out = s;
  return DG_OK;
}

dg_buffer* dg_radix_sort_keys(dg_radix_sort* s) { return s ? s->keys : nullptr; }
dg_buffer* dg_radix_sort_values(dg_radix_sort* s) { return s ? s->values : nullptr; }
uint32_t dg_radix_sort_capacity(const dg_radix_sort* s) { return s ? s->plan.capacity : 0; }

dg_status dg_radix_sort_encode(dg_radix_sort* s) {
  DG_REQUIRE(s, "NULL argument");
  return sort_launch(s->ctx, s->plan, s->keys->ptr, typed<uint32_t>(s->values), s->keys_alt->ptr,
                     typed<uint32_t>(s->values_alt), s->count ? typed<uint32_t>(s->count) : nullptr, s->scratch->ptr);
}

dg_status dg_radix_sort_destroy(dg_radix_sort* s) {
  if (!s) return DG_OK;
  free_buffer(s->keys);
  free_buffer(s->values);
  free_buffer(s->keys_alt);
  free_buffer(s->values_alt);
  free_buffer(s->scratch);
  delete s;
  return DG_OK;
}

}  // extern "C"

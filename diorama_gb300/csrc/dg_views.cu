// Batched rendering of many views of one scene: every stage of the frame runs
// once over all the views of a batch (one preprocess launch projecting each
// Gaussian into every view, one depth sort over (view, depth) keys, one tile
// sort over the views' stacked tile numbers, one blend over all their tiles),
// and a batch whose pair count is known is replayed as one CUDA graph. Each view
// gets exactly the pairs, order and blend of a single-view render, so its image
// is bit-identical to GaussianRenderer.encode's. The views per batch, the
// blend's cooperative threshold and the blend tiles (16x16, 32x16, 16x32 or
// 32x32 pixels; dg_render_kernels.cuh, blend_rect) come from a small autotuner
// (dg_renderer_tune_views) or are set by the caller.
#include "dg_render.cuh"
#include "dg_render_kernels.cuh"  // plan layout and blend constants (no kernels here)

#include <algorithm>
#include <cstring>
#include <vector>

namespace dg {
namespace {

// Bits needed to number n things (at least 1).
uint32_t bits_for(uint32_t n) {
  uint32_t b = 1;
  while (b < 32 && (1ull << b) < n) b++;
  return b;
}

// Where a batch's pair keys hold the view: above the whole 8-bit digits that
// number a view's tiles, so the tile sort's passes never read it. A batch holds
// fewer than 2^24 tiles, so the view always fits above them.
uint32_t view_shift_for(uint32_t tiles_per_view) { return (bits_for(tiles_per_view) + 7) / 8 * 8; }

dg_status ensure(dg_context* ctx, dg_buffer** buf, size_t bytes) {
  if (*buf && (*buf)->bytes >= bytes) return DG_OK;
  free_buffer(*buf);
  *buf = nullptr;
  return alloc_buffer(ctx, std::max<size_t>(bytes, 16), buf);
}

}  // namespace
}  // namespace dg

using namespace dg;

// The buffers of one batch of views (grown on demand, reused across calls).
struct dg_view_batch {
  dg_context* ctx = nullptr;
  uint32_t views = 0, count = 0, tiles_per_view = 0, pixels = 0;
  BlendShape shape{0u, 0u};
  uint32_t pair_capacity = 0;
  dg_buffer *cameras = nullptr, *raster_params = nullptr, *splats = nullptr, *tile_counts = nullptr;
  dg_buffer *depth_keys = nullptr, *depth_keys_alt = nullptr, *order = nullptr, *order_alt = nullptr;
  dg_buffer *depth_scratch = nullptr, *counts_sorted = nullptr, *scan_scratch = nullptr, *scan_total = nullptr;
  dg_buffer *keys = nullptr, *keys_alt = nullptr, *values = nullptr, *values_alt = nullptr, *sort_scratch = nullptr;
  dg_buffer *ranges = nullptr, *plan = nullptr, *pixel_color = nullptr, *pixel_last = nullptr, *work = nullptr;
  uint32_t* pinned_total = nullptr;
  // The captured batch (valid while its key matches).
  cudaGraphExec_t graph = nullptr;
  struct Key {
    uint32_t views, count, capacity, coop_min;
    BlendShape shape;
    const void *gaussians, *targets, *keys;
    bool operator==(const Key& o) const {
      return views == o.views && count == o.count && capacity == o.capacity && coop_min == o.coop_min &&
             shape == o.shape && gaussians == o.gaussians && targets == o.targets && keys == o.keys;
    }
  } key{};
  uint32_t last_total = 0;
};

namespace dg {

void view_batch_destroy(dg_view_batch* b) {
  if (!b) return;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  for (dg_buffer* x : {b->cameras, b->raster_params, b->splats, b->tile_counts, b->depth_keys, b->depth_keys_alt,
                       b->order, b->order_alt, b->depth_scratch, b->counts_sorted, b->scan_scratch, b->scan_total,
                       b->keys, b->keys_alt, b->values, b->values_alt, b->sort_scratch, b->ranges, b->plan,
                       b->pixel_color, b->pixel_last, b->work})
    free_buffer(x);
  if (b->pinned_total) cudaFreeHost(b->pinned_total);
  delete b;
}

namespace {

dg_status grow_pairs(dg_view_batch* b, uint32_t capacity) {
  dg_context* ctx = b->ctx;
  const SortPlan tile_plan = sort_plan_digits(capacity, 1, bits_for(b->tiles_per_view));
  DG_TRY(ensure(ctx, &b->keys, (size_t)capacity * 4));
  DG_TRY(ensure(ctx, &b->keys_alt, (size_t)capacity * 4));
  DG_TRY(ensure(ctx, &b->values, (size_t)capacity * 4));
  DG_TRY(ensure(ctx, &b->values_alt, (size_t)capacity * 4));
  DG_TRY(ensure(ctx, &b->sort_scratch, sort_scratch_bytes(tile_plan)));
  b->pair_capacity = capacity;
  return DG_OK;
}

// Sizes the batch for `views` views of `count` Gaussians at `pixels` pixels in
// tiles_per_view blend tiles each.
dg_status prepare(dg_view_batch* b, uint32_t views, uint32_t count, uint32_t tiles_per_view, uint32_t pixels) {
  dg_context* ctx = b->ctx;
  const size_t n = (size_t)views * count;
  if (n >= (1ull << 31)) return fail(DG_ERROR_INVALID_ARGUMENT, "too many view x Gaussian pairs in one batch");
  if ((uint64_t)views * tiles_per_view >= (1ull << 24))
    return fail(DG_ERROR_INVALID_ARGUMENT, "too many tiles in one batch of views");
  const bool reshaped = views != b->views || count != b->count || tiles_per_view != b->tiles_per_view;
  b->views = views;
  b->count = count;
  b->tiles_per_view = tiles_per_view;
  b->pixels = pixels;
  const SortPlan depth_plan = sort_plan_digits((uint32_t)n, 2, bits_for(views));
  DG_TRY(ensure(ctx, &b->cameras, (size_t)views * sizeof(Camera)));
  DG_TRY(ensure(ctx, &b->raster_params, 16));
  DG_TRY(ensure(ctx, &b->splats, n * FLOATS_PER_SPLAT * 4));
  DG_TRY(ensure(ctx, &b->tile_counts, n * 4));
  DG_TRY(ensure(ctx, &b->depth_keys, n * 8));
  DG_TRY(ensure(ctx, &b->depth_keys_alt, n * 8));
  DG_TRY(ensure(ctx, &b->order, n * 4));
  DG_TRY(ensure(ctx, &b->order_alt, n * 4));
  DG_TRY(ensure(ctx, &b->depth_scratch, sort_scratch_bytes(depth_plan)));
  DG_TRY(ensure(ctx, &b->counts_sorted, n * 4));
  DG_TRY(ensure(ctx, &b->scan_scratch, scan_scratch_bytes((uint32_t)n)));
  DG_TRY(ensure(ctx, &b->scan_total, 16));
  DG_TRY(ensure(ctx, &b->ranges, (size_t)views * tiles_per_view * 8));
  DG_TRY(ensure(ctx, &b->plan, (PLAN_HEADER + (size_t)views * tiles_per_view) * 4));
  DG_TRY(ensure(ctx, &b->pixel_color, (size_t)views * pixels * 16));
  DG_TRY(ensure(ctx, &b->pixel_last, (size_t)views * pixels * 4));
  DG_TRY(ensure(ctx, &b->work, 16));
  if (!b->pinned_total && cudaMallocHost(&b->pinned_total, 4) != cudaSuccess)
    return fail(DG_ERROR_OUT_OF_MEMORY, "pinned");
  if (reshaped || b->pair_capacity == 0) {
    // A first guess: the previous batch's pairs per view, else 4 per Gaussian.
    const uint64_t guess = b->last_total ? (uint64_t)b->last_total * 9 / 8 : (uint64_t)n * 4;
    DG_TRY(grow_pairs(b, (uint32_t)std::min<uint64_t>(std::max<uint64_t>(guess, 1u << 16), 0xF0000000u)));
  }
  return DG_OK;
}

// The launches of one batch, in order (capturable: no host synchronization).
dg_status launch_batch(dg_renderer* r, dg_view_batch* b, uchar4* targets, uint32_t coop_min) {
  dg_context* ctx = r->ctx;
  const uint32_t n = b->views * b->count;
  const uint32_t tiles = b->views * b->tiles_per_view;
  DG_TRY(views_preprocess_launch(ctx, typed<Camera>(b->cameras), b->views, typed<float>(r->gaussians),
                                 typed<float>(r->sh), b->count, typed<uint32_t>(r->scene_params),
                                 typed<float>(b->splats), typed<uint32_t>(b->tile_counts), typed<uint2>(b->depth_keys),
                                 typed<uint32_t>(b->order), b->shape));
  // (view, depth) keys: 4 passes over the depth bits and one per 8 bits of view.
  const SortPlan depth_plan = sort_plan_digits(n, 2, bits_for(b->views));
  DG_TRY(sort_launch(ctx, depth_plan, b->depth_keys->ptr, typed<uint32_t>(b->order), b->depth_keys_alt->ptr,
                     typed<uint32_t>(b->order_alt), nullptr, b->depth_scratch->ptr));
  uint32_t* order = depth_plan.passes & 1 ? typed<uint32_t>(b->order_alt) : typed<uint32_t>(b->order);
  DG_TRY(scan_launch(ctx, typed<uint32_t>(b->counts_sorted), n, nullptr, typed<uint32_t>(b->scan_total),
                     b->scan_scratch->ptr, order, typed<uint32_t>(b->tile_counts)));
  // Pairs in depth order, view-major, keyed view << shift | local tile: a stable
  // sort on the local tile's bits alone leaves every (view, tile) run contiguous
  // and in depth order, an 8-bit pass fewer than sorting global tile numbers.
  const uint32_t shift = view_shift_for(b->tiles_per_view);
  DG_TRY(duplicate_sorted_launch(ctx, typed<Camera>(b->cameras), typed<float>(b->splats), order,
                                 typed<uint32_t>(b->counts_sorted), n, b->count, shift, b->pair_capacity,
                                 typed<uint32_t>(b->keys), typed<uint32_t>(b->values), b->shape));
  const SortPlan tile_plan = sort_plan_digits(b->pair_capacity, 1, bits_for(b->tiles_per_view));
  DG_TRY(sort_launch(ctx, tile_plan, b->keys->ptr, typed<uint32_t>(b->values), b->keys_alt->ptr,
                     typed<uint32_t>(b->values_alt), typed<uint32_t>(b->scan_total), b->sort_scratch->ptr));
  const bool odd = tile_plan.passes & 1;
  const uint32_t* tile_keys = typed<uint32_t>(odd ? b->keys_alt : b->keys);
  const uint32_t* pair_splats = typed<uint32_t>(odd ? b->values_alt : b->values);
  DG_CUDA(cudaMemsetAsync(b->ranges->ptr, 0, (size_t)tiles * 8, ctx->stream));
  DG_TRY(find_view_ranges_launch(ctx, tile_keys, typed<uint32_t>(b->scan_total), b->pair_capacity, shift,
                                 b->tiles_per_view, tiles, typed<uint2>(b->ranges)));
  BlendForward f{};
  f.camera = typed<Camera>(b->cameras);
  f.raster_params = typed<float4>(b->raster_params);
  f.splats = typed<float>(b->splats);
  f.pair_splats = pair_splats;
  f.ranges = typed<uint2>(b->ranges);
  f.tiles = tiles;
  f.tiles_per_view = b->tiles_per_view;
  f.coop_min = coop_min;
  f.plan = typed<uint32_t>(b->plan);
  f.target = targets;
  f.pixel_color = typed<float4>(b->pixel_color);
  f.pixel_last = typed<uint32_t>(b->pixel_last);
  f.counters = typed<uint32_t>(b->work);
  f.shape = b->shape;
  f.splat_cutoffs = true;  // preprocess_views_kernel's splats
  DG_TRY(blend_forward(ctx, f));
  DG_CUDA(cudaMemcpyAsync(b->pinned_total, b->scan_total->ptr, 4, cudaMemcpyDeviceToHost, ctx->stream));
  return DG_OK;
}

// Renders one batch (views[0..count)), replaying its graph when the key matches
// and growing the pair buffers (then rendering again) when the pairs overflowed.
dg_status render_batch(dg_renderer* r, dg_view_batch* b, const dg_camera* cams, uint32_t count, const float bg[3],
                       uchar4* targets, uint32_t coop_min, BlendShape shape, bool use_graph) {
  dg_context* ctx = r->ctx;
  const uint32_t w = (uint32_t)cams[0].viewport[0], h = (uint32_t)cams[0].viewport[1];
  const uint32_t tiles_per_view =
      blend_tiles_along(ceil_div(w, TILE), shape.twl) * blend_tiles_along(ceil_div(h, TILE), shape.thl);
  DG_TRY(prepare(b, count, r->count, tiles_per_view, w * h));
  b->shape = shape;
  std::vector<Camera> cameras(count);
  for (uint32_t k = 0; k < count; k++) {
    Camera& c = cameras[k];
    c = Camera{};
    std::memcpy(c.view, cams[k].view, 64);
    std::memcpy(c.proj, cams[k].proj, 64);
    c.viewport[0] = cams[k].viewport[0];
    c.viewport[1] = cams[k].viewport[1];
  }
  DG_TRY(write_async(ctx, b->cameras->ptr, cameras.data(), count * sizeof(Camera)));
  const float params[4] = {bg[0], bg[1], bg[2], 1.0f};
  DG_TRY(write_async(ctx, b->raster_params->ptr, params, sizeof(params)));
  for (int attempt = 0; attempt < 2; attempt++) {
    const dg_view_batch::Key key{count, r->count, b->pair_capacity, coop_min, shape, r->gaussians->ptr, targets,
                                 b->keys->ptr};
    if (use_graph) {
      if (!b->graph || !(key == b->key)) {
        if (b->graph) cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
        cudaGraph_t graph;
        DG_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        ctx->capturing = true;
        const dg_status st = launch_batch(r, b, targets, coop_min);
        ctx->capturing = false;
        const cudaError_t end = cudaStreamEndCapture(ctx->stream, &graph);
        if (st != DG_OK) {
          if (end == cudaSuccess) cudaGraphDestroy(graph);
          return st;
        }
        DG_CUDA(end);
        const cudaError_t inst = cudaGraphInstantiate(&b->graph, graph, 0);
        cudaGraphDestroy(graph);
        DG_CUDA(inst);
        b->key = key;
      }
      DG_CUDA(cudaGraphLaunch(b->graph, ctx->stream));
    } else {
      DG_TRY(launch_batch(r, b, targets, coop_min));
    }
    DG_CUDA(cudaStreamSynchronize(ctx->stream));
    const uint32_t total = *b->pinned_total;
    b->last_total = total;
    if (total <= b->pair_capacity) return DG_OK;
    DG_TRY(grow_pairs(b, (uint32_t)std::min<uint64_t>((uint64_t)total * 9 / 8 + 1024, 0xF0000000u)));
  }
  return fail(DG_ERROR_STATE, "the batch's pair count kept growing");
}

dg_view_batch* batch_of(dg_renderer* r) {
  if (!r->views) {
    r->views = new dg_view_batch();
    r->views->ctx = r->ctx;
  }
  return r->views;
}

dg_status check_views(dg_renderer* r, const dg_camera* cams, uint32_t count) {
  DG_REQUIRE(r && cams, "NULL argument");
  DG_REQUIRE(count > 0, "no views");
  DG_REQUIRE(r->has_scene && r->count > 0, "no Gaussians to render");
  for (uint32_t k = 1; k < count; k++)
    if (cams[k].viewport[0] != cams[0].viewport[0] || cams[k].viewport[1] != cams[0].viewport[1])
      return fail(DG_ERROR_INVALID_ARGUMENT, "All views of a batch must be the same size.");
  const uint32_t tiles = ceil_div((uint32_t)cams[0].viewport[0], TILE) * ceil_div((uint32_t)cams[0].viewport[1], TILE);
  DG_REQUIRE(tiles <= (1u << TILE_INDEX_BITS), "A view has more tiles than the sort can tell apart.");
  return DG_OK;
}

}  // namespace

dg_status views_render(dg_renderer* r, const dg_camera* cams, uint32_t count, const float bg[3], uchar4* targets,
                       float4* pixel_colors, uint32_t batch, uint32_t coop_min, BlendShape shape) {
  DG_TRY(check_views(r, cams, count));
  dg_context* ctx = r->ctx;
  dg_view_batch* b = batch_of(r);
  batch = std::max(1u, std::min(batch ? batch : count, count));
  const size_t pixels = (size_t)cams[0].viewport[0] * (uint32_t)cams[0].viewport[1];
  for (uint32_t first = 0; first < count; first += batch) {
    const uint32_t n = std::min(batch, count - first);
    DG_TRY(render_batch(r, b, cams + first, n, bg, targets ? targets + first * pixels : nullptr, coop_min, shape,
                        r->view_graph));
    if (pixel_colors)
      DG_CUDA(cudaMemcpyAsync(pixel_colors + first * pixels, b->pixel_color->ptr, n * pixels * 16,
                              cudaMemcpyDeviceToDevice, ctx->stream));
  }
  return DG_OK;
}

}  // namespace dg

// ------------------------------------------------------------------ C ABI

dg_status dg_renderer_render_views(dg_renderer* r, const dg_camera* cameras, uint32_t count, const float background[3],
                                   dg_buffer* targets, dg_buffer* pixel_colors) {
  DG_REQUIRE(r && cameras && background, "NULL argument");
  DG_TRY(check_views(r, cameras, count));
  const size_t pixels = (size_t)cameras[0].viewport[0] * (uint32_t)cameras[0].viewport[1];
  DG_REQUIRE(!targets || targets->bytes >= pixels * count * 4, "targets hold fewer than count rgba8 images");
  DG_REQUIRE(!pixel_colors || pixel_colors->bytes >= pixels * count * 16,
             "pixel_colors hold fewer than count vec4 images");
  return views_render(r, cameras, count, background, targets ? typed<uchar4>(targets) : nullptr,
                      pixel_colors ? typed<float4>(pixel_colors) : nullptr, r->view_batch, r->view_coop_min,
                      r->view_shape);
}

dg_status dg_renderer_set_view_batching(dg_renderer* r, uint32_t batch, uint32_t coop_min, int32_t graph) {
  DG_REQUIRE(r, "NULL argument");
  r->view_batch = batch;
  r->view_coop_min = coop_min ? coop_min : COOP_MIN;
  r->view_graph = graph != 0;
  return DG_OK;
}

dg_status dg_renderer_view_batching(const dg_renderer* r, uint32_t* batch, uint32_t* coop_min) {
  DG_REQUIRE(r && batch && coop_min, "NULL argument");
  *batch = r->view_batch;
  *coop_min = r->view_coop_min;
  return DG_OK;
}

dg_status dg_renderer_set_view_tile(dg_renderer* r, uint32_t width, uint32_t height) {
  DG_REQUIRE(r, "NULL argument");
  if ((width != 16 && width != 32) || (height != 16 && height != 32))
    return fail(DG_ERROR_INVALID_ARGUMENT, "blend tiles are 16 or 32 pixels wide and 16 or 32 high");
  r->view_shape = BlendShape{width == 32 ? 1u : 0u, height == 32 ? 1u : 0u};
  return DG_OK;
}

dg_status dg_renderer_view_tile(const dg_renderer* r, uint32_t* width, uint32_t* height) {
  DG_REQUIRE(r && width && height, "NULL argument");
  *width = TILE << r->view_shape.twl;
  *height = TILE << r->view_shape.thl;
  return DG_OK;
}

// The autotuner: times every candidate (views per batch) x (cooperative
// threshold) on the given views with 16x16 blend tiles, then the 32x16, 16x32
// and 32x32 blend tiles at the fastest of those, each after a warm-up render,
// and keeps the fastest for later dg_renderer_render_views calls. seconds[k]
// (optional, room for 32) gets the time of candidate k in the order tried.
dg_status dg_renderer_tune_views(dg_renderer* r, const dg_camera* cameras, uint32_t count, const float background[3],
                                 dg_buffer* targets, uint32_t* best_batch, uint32_t* best_coop_min, double* seconds,
                                 uint32_t* tried) {
  DG_REQUIRE(r && cameras && background && best_batch && best_coop_min, "NULL argument");
  DG_TRY(check_views(r, cameras, count));
  dg_context* ctx = r->ctx;
  const size_t pixels = (size_t)cameras[0].viewport[0] * (uint32_t)cameras[0].viewport[1];
  DG_REQUIRE(!targets || targets->bytes >= pixels * count * 4, "targets hold fewer than count rgba8 images");
  uchar4* out = targets ? typed<uchar4>(targets) : nullptr;
  std::vector<uint32_t> batches;
  for (uint32_t b : {1u, 4u, 8u, 16u, 32u, count})
    if (b <= count && std::find(batches.begin(), batches.end(), b) == batches.end()) batches.push_back(b);
  const uint32_t thresholds[] = {128u, 512u, 1024u, 2048u};
  cudaEvent_t start, stop;
  DG_CUDA(cudaEventCreate(&start));
  DG_CUDA(cudaEventCreate(&stop));
  double best = 1e30;
  BlendShape best_shape{0u, 0u};
  uint32_t k = 0;
  // One candidate: a warm-up render (sizes, graphs), then the timed one.
  auto time_candidate = [&](uint32_t b, uint32_t t, BlendShape shape) -> dg_status {
    DG_TRY(views_render(r, cameras, count, background, out, nullptr, b, t, shape));
    DG_CUDA(cudaEventRecord(start, ctx->stream));
    DG_TRY(views_render(r, cameras, count, background, out, nullptr, b, t, shape));
    DG_CUDA(cudaEventRecord(stop, ctx->stream));
    DG_CUDA(cudaEventSynchronize(stop));
    float ms = 0.0f;
    DG_CUDA(cudaEventElapsedTime(&ms, start, stop));
    if (seconds && k < 32) seconds[k] = ms * 1e-3;
    k++;
    if (ms * 1e-3 < best) {
      best = ms * 1e-3;
      *best_batch = b;
      *best_coop_min = t;
      best_shape = shape;
    }
    return DG_OK;
  };
  dg_status st = DG_OK;
  for (uint32_t b : batches) {
    for (uint32_t t : thresholds) {
      st = time_candidate(b, t, BlendShape{0u, 0u});
      if (st != DG_OK) break;
    }
    if (st != DG_OK) break;
  }
  if (st == DG_OK) {
    const uint32_t b = *best_batch, t = *best_coop_min;
    for (BlendShape shape : {BlendShape{1u, 0u}, BlendShape{0u, 1u}, BlendShape{1u, 1u}}) {
      st = time_candidate(b, t, shape);
      if (st != DG_OK) break;
    }
  }
  cudaEventDestroy(start);
  cudaEventDestroy(stop);
  if (tried) *tried = k;
  if (st != DG_OK) return st;
  r->view_batch = *best_batch;
  r->view_coop_min = *best_coop_min;
  r->view_shape = best_shape;
  return DG_OK;
}

// The last batch's per-pixel results (views x pixels), for inspection.
dg_buffer* dg_renderer_views_pixel_last(dg_renderer* r) { return r && r->views ? r->views->pixel_last : nullptr; }

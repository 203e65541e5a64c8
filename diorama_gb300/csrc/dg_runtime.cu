// Context, buffers and errors: the GPUDevice / GPUQueue / GPUBuffer layer of the
// reference (src/gpu.ts:8-46, src/readback.ts) on one CUDA device and stream.
#include "dg_common.cuh"
#include "dg_scan.cuh"

#include <cuda_profiler_api.h>

#include <algorithm>
#include <cstdio>

namespace dg {

static thread_local std::string g_last_error;

void set_error(const std::string& message) { g_last_error = message; }

dg_status fail(dg_status code, const std::string& message) {
  g_last_error = message;
  return code;
}

dg_status cuda_fail(cudaError_t err, const char* what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorName(err) + " (" + cudaGetErrorString(err) + ")";
  return err == cudaErrorMemoryAllocation ? DG_ERROR_OUT_OF_MEMORY : DG_ERROR_CUDA;
}

static constexpr size_t STAGING_BYTES = 64u << 20;
static constexpr size_t STAGING_LIMIT = 1u << 20;  // larger writes copy straight from the caller

dg_status write_async(dg_context* ctx, void* dst, const void* src, size_t bytes) {
  if (bytes == 0) return DG_OK;
  if (ctx->capturing) return fail(DG_ERROR_STATE, "buffer writes are not allowed while a step graph is being captured");
  if (bytes > STAGING_LIMIT) {
    // Pageable source: cudaMemcpyAsync stages it before returning, so the caller
    // may reuse its memory at once.
    DG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    return DG_OK;
  }
  size_t aligned = (bytes + 255) & ~size_t(255);
  if (ctx->staging_head + aligned > ctx->staging_bytes) ctx->staging_head = 0;
  size_t begin = ctx->staging_head, end = begin + aligned;
  // Entries are retired in order; wait for any that still read this range.
  while (true) {
    bool clash = false;
    for (auto& p : ctx->pending)
      if (p.begin < end && begin < p.end) clash = true;
    if (!clash) break;
    // The ring is first in, first out: retire the oldest copy and look again.
    auto oldest = ctx->pending.front();
    DG_CUDA(cudaEventSynchronize(oldest.done));
    ctx->free_events.push_back(oldest.done);
    ctx->pending.pop_front();
  }
  std::memcpy(ctx->staging + begin, src, bytes);
  DG_CUDA(cudaMemcpyAsync(dst, ctx->staging + begin, bytes, cudaMemcpyHostToDevice, ctx->stream));
  cudaEvent_t ev;
  if (!ctx->free_events.empty()) {
    ev = ctx->free_events.back();
    ctx->free_events.pop_back();
  } else {
    DG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  }
  DG_CUDA(cudaEventRecord(ev, ctx->stream));
  ctx->pending.push_back({begin, end, ev});
  ctx->staging_head = end;
  // Keep the queue short: retire whatever is already done.
  while (!ctx->pending.empty() && cudaEventQuery(ctx->pending.front().done) == cudaSuccess) {
    ctx->free_events.push_back(ctx->pending.front().done);
    ctx->pending.pop_front();
  }
  return DG_OK;
}

dg_status alloc_buffer(dg_context* ctx, uint64_t bytes, dg_buffer** out) {
  void* ptr = nullptr;
  if (bytes > 0) {
    DG_CUDA(cudaMallocAsync(&ptr, bytes, ctx->stream));
    cudaError_t err = cudaMemsetAsync(ptr, 0, bytes, ctx->stream);
    if (err != cudaSuccess) {
      cudaFreeAsync(ptr, ctx->stream);
      return cuda_fail(err, "cudaMemsetAsync");
    }
  }
  *out = new dg_buffer{ctx, ptr, bytes, true};
  return DG_OK;
}

static cudaEvent_t timing_event(dg_context* ctx) {
  if (!ctx->timing_pool.empty()) {
    cudaEvent_t e = ctx->timing_pool.back();
    ctx->timing_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

void timing_begin(dg_context* ctx) {
  if (!ctx->timing || ctx->capturing) return;
  ctx->pending_start = timing_event(ctx);
  cudaEventRecord(ctx->pending_start, ctx->stream);
}

void timing_end(dg_context* ctx, const char* name) {
  if (!ctx->timing || ctx->capturing || !ctx->pending_start) return;
  cudaEvent_t end = timing_event(ctx);
  cudaEventRecord(end, ctx->stream);
  ctx->timed.push_back({name, ctx->pending_start, end});
  ctx->pending_start = nullptr;
}

void free_buffer(dg_buffer* b) {
  if (!b) return;
  // Stream-ordered free: the GPU keeps the memory until work already enqueued is
  // done, as WebGPU keeps a destroyed buffer alive for submitted work.
  if (b->owned && b->ptr) cudaFreeAsync(b->ptr, b->ctx->stream);
  delete b;
}

}  // namespace dg

using namespace dg;

extern "C" {

const char* dg_last_error(void) { return g_last_error.c_str(); }

int32_t dg_abi_version(void) { return 1; }

dg_status dg_context_create(int32_t device, dg_context** out) {
  DG_REQUIRE(out, "out is NULL");
  *out = nullptr;
  int count = 0;
  DG_CUDA(cudaGetDeviceCount(&count));
  DG_REQUIRE(device >= 0 && device < count, "no such CUDA device");
  DG_CUDA(cudaSetDevice(device));
  auto* ctx = new dg_context();
  ctx->device = device;
  cudaError_t err = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (err != cudaSuccess) {
    delete ctx;
    return cuda_fail(err, "cudaStreamCreate");
  }
  cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
  err = cudaMalloc(&ctx->device_error, sizeof(uint32_t));
  if (err == cudaSuccess) err = cudaMemset(ctx->device_error, 0, sizeof(uint32_t));
  if (err == cudaSuccess) err = cudaMallocHost(&ctx->staging, STAGING_BYTES);
  if (err != cudaSuccess) {
    dg_context_destroy(ctx);
    return cuda_fail(err, "context allocation");
  }
  ctx->staging_bytes = STAGING_BYTES;
  if (dg_status st = sort_init(); st != DG_OK) {
    dg_context_destroy(ctx);
    return st;
  }
  // Keep freed pool memory for reuse across densifications instead of returning it.
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t threshold = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
  }
  *out = ctx;
  return DG_OK;
}

dg_status dg_context_destroy(dg_context* ctx) {
  if (!ctx) return DG_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (auto& p : ctx->pending) cudaEventDestroy(p.done);
  for (auto e : ctx->free_events) cudaEventDestroy(e);
  for (auto& t : ctx->timed) {
    cudaEventDestroy(t.start);
    cudaEventDestroy(t.end);
  }
  for (auto e : ctx->timing_pool) cudaEventDestroy(e);
  if (ctx->staging) cudaFreeHost(ctx->staging);
  if (ctx->device_error) cudaFree(ctx->device_error);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return DG_OK;
}

dg_status dg_context_synchronize(dg_context* ctx) {
  DG_REQUIRE(ctx, "ctx is NULL");
  DG_CUDA(cudaStreamSynchronize(ctx->stream));
  return DG_OK;
}

dg_status dg_context_check(dg_context* ctx, uint32_t* bits) {
  DG_REQUIRE(ctx, "ctx is NULL");
  uint32_t value = 0;
  DG_CUDA(cudaMemcpyAsync(&value, ctx->device_error, 4, cudaMemcpyDeviceToHost, ctx->stream));
  DG_CUDA(cudaStreamSynchronize(ctx->stream));
  if (bits) *bits = value;
  if (value) {
    DG_CUDA(cudaMemsetAsync(ctx->device_error, 0, 4, ctx->stream));
    return fail(DG_ERROR_DEVICE_WAIT, "a bounded wait on the GPU gave up (error bits " + std::to_string(value) + ")");
  }
  return DG_OK;
}

dg_status dg_context_launch_count(dg_context* ctx, uint64_t* out) {
  DG_REQUIRE(ctx && out, "NULL argument");
  *out = ctx->launches;
  return DG_OK;
}

dg_status dg_context_profile(dg_context* ctx, int32_t enabled) {
  DG_REQUIRE(ctx, "NULL argument");
  DG_CUDA(cudaStreamSynchronize(ctx->stream));
  DG_CUDA(enabled ? cudaProfilerStart() : cudaProfilerStop());
  return DG_OK;
}

dg_status dg_context_set_kernel_timing(dg_context* ctx, int32_t enabled) {
  DG_REQUIRE(ctx, "NULL argument");
  ctx->timing = enabled != 0;
  return DG_OK;
}

dg_status dg_context_kernel_timing_report(dg_context* ctx, char* text, uint64_t capacity) {
  DG_REQUIRE(ctx && text && capacity > 0, "NULL argument");
  DG_CUDA(cudaStreamSynchronize(ctx->stream));
  struct Total {
    std::string name;
    uint64_t launches = 0;
    double ms = 0;
  };
  std::vector<Total> totals;
  for (auto& t : ctx->timed) {
    float ms = 0;
    cudaEventElapsedTime(&ms, t.start, t.end);
    auto it = std::find_if(totals.begin(), totals.end(), [&](const Total& x) { return x.name == t.name; });
    if (it == totals.end()) {
      totals.push_back({t.name, 0, 0});
      it = totals.end() - 1;
    }
    it->launches++;
    it->ms += ms;
    ctx->timing_pool.push_back(t.start);
    ctx->timing_pool.push_back(t.end);
  }
  ctx->timed.clear();
  std::string out;
  for (auto& t : totals) out += t.name + " " + std::to_string(t.launches) + " " + std::to_string(t.ms) + "\n";
  std::snprintf(text, capacity, "%s", out.c_str());
  return DG_OK;
}

struct dg_event {
  dg_context* ctx;
  cudaEvent_t event;
};

dg_status dg_event_create(dg_context* ctx, dg_event** out) {
  DG_REQUIRE(ctx && out, "NULL argument");
  auto* e = new dg_event{ctx, nullptr};
  cudaError_t err = cudaEventCreate(&e->event);
  if (err != cudaSuccess) {
    delete e;
    return cuda_fail(err, "cudaEventCreate");
  }
  *out = e;
  return DG_OK;
}

dg_status dg_event_record(dg_event* e) {
  DG_REQUIRE(e, "NULL argument");
  DG_CUDA(cudaEventRecord(e->event, e->ctx->stream));
  return DG_OK;
}

dg_status dg_event_elapsed(dg_event* start, dg_event* end, float* ms) {
  DG_REQUIRE(start && end && ms, "NULL argument");
  DG_CUDA(cudaEventSynchronize(end->event));
  DG_CUDA(cudaEventElapsedTime(ms, start->event, end->event));
  return DG_OK;
}

dg_status dg_event_destroy(dg_event* e) {
  if (!e) return DG_OK;
  cudaEventDestroy(e->event);
  delete e;
  return DG_OK;
}

dg_status dg_host_alloc(uint64_t bytes, void** out) {
  DG_REQUIRE(out, "NULL argument");
  DG_CUDA(cudaMallocHost(out, bytes));
  return DG_OK;
}

dg_status dg_host_free(void* ptr) {
  if (ptr) DG_CUDA(cudaFreeHost(ptr));
  return DG_OK;
}

dg_status dg_buffer_write_pinned(dg_buffer* b, uint64_t offset, const void* src, uint64_t bytes) {
  DG_REQUIRE(b && (src || bytes == 0), "NULL argument");
  DG_REQUIRE(offset + bytes <= b->bytes, "write past the end of the buffer");
  if (bytes)
    DG_CUDA(cudaMemcpyAsync(static_cast<char*>(b->ptr) + offset, src, bytes, cudaMemcpyHostToDevice, b->ctx->stream));
  return DG_OK;
}

dg_status dg_buffer_create(dg_context* ctx, uint64_t bytes, dg_buffer** out) {
  DG_REQUIRE(ctx && out, "NULL argument");
  return alloc_buffer(ctx, bytes, out);
}

dg_status dg_buffer_wrap(dg_context* ctx, void* device_ptr, uint64_t bytes, dg_buffer** out) {
  DG_REQUIRE(ctx && out, "NULL argument");
  *out = new dg_buffer{ctx, device_ptr, bytes, false};
  return DG_OK;
}

dg_status dg_buffer_destroy(dg_buffer* buffer) {
  free_buffer(buffer);
  return DG_OK;
}

uint64_t dg_buffer_size(const dg_buffer* buffer) { return buffer ? buffer->bytes : 0; }

void* dg_buffer_device_pointer(const dg_buffer* buffer) { return buffer ? buffer->ptr : nullptr; }

dg_status dg_buffer_write(dg_buffer* b, uint64_t offset, const void* src, uint64_t bytes) {
  DG_REQUIRE(b && (src || bytes == 0), "NULL argument");
  DG_REQUIRE(offset + bytes <= b->bytes, "write past the end of the buffer");
  return write_async(b->ctx, static_cast<char*>(b->ptr) + offset, src, bytes);
}

dg_status dg_buffer_read(dg_buffer* b, uint64_t offset, void* dst, uint64_t bytes) {
  DG_REQUIRE(b && (dst || bytes == 0), "NULL argument");
  DG_REQUIRE(offset + bytes <= b->bytes, "read past the end of the buffer");
  if (bytes) DG_CUDA(cudaMemcpyAsync(dst, static_cast<char*>(b->ptr) + offset, bytes, cudaMemcpyDeviceToHost, b->ctx->stream));
  DG_CUDA(cudaStreamSynchronize(b->ctx->stream));
  return DG_OK;
}

dg_status dg_buffer_clear(dg_buffer* b, uint64_t offset, uint64_t bytes) {
  DG_REQUIRE(b, "NULL argument");
  DG_REQUIRE(offset + bytes <= b->bytes, "clear past the end of the buffer");
  if (bytes) DG_CUDA(cudaMemsetAsync(static_cast<char*>(b->ptr) + offset, 0, bytes, b->ctx->stream));
  return DG_OK;
}

dg_status dg_buffer_copy(dg_buffer* src, uint64_t src_offset, dg_buffer* dst, uint64_t dst_offset, uint64_t bytes) {
  DG_REQUIRE(src && dst, "NULL argument");
  DG_REQUIRE(src_offset + bytes <= src->bytes && dst_offset + bytes <= dst->bytes, "copy past the end of a buffer");
  if (bytes)
    DG_CUDA(cudaMemcpyAsync(static_cast<char*>(dst->ptr) + dst_offset, static_cast<char*>(src->ptr) + src_offset, bytes,
                            cudaMemcpyDeviceToDevice, src->ctx->stream));
  return DG_OK;
}

}  // extern "C"

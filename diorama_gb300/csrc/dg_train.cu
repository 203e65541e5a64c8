// Training: Adam with activation (src/shaders/adam.wgsl), densification as
// stream compaction (src/shaders/densify.wgsl), and the Trainer loop of
// src/trainer.ts, with each optimize() step optionally replayed as one captured
// CUDA graph.
#include "dg_adam.cuh"
#include "dg_common.cuh"
#include "dg_loss.cuh"
#include "dg_mlp.cuh"
#include "dg_ply.h"
#include "dg_render.cuh"
#include "dg_scan.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <unordered_map>

namespace dg {
namespace {

constexpr uint32_t RESET_SLOT = 3;          // opacity's Adam slot
constexpr float RESET_LOGIT = -4.59511985013459f;  // logit(0.01), src/shaders/adam.wgsl:112
constexpr float SPLIT_SHRINK = 1.6f;
constexpr float LOG_SPLIT_SHRINK = 0.470003629245735553f;  // ln 1.6

// DensifyParams (src/shaders/densify.wgsl:149-161)
struct DensifyParams {
  float grad_threshold, clone_max_size, min_opacity, max_size;
  uint32_t seed;
};

__device__ __forceinline__ float sigmoidf_(float x) { return 1.0f / (1.0f + expf(-x)); }

// The activated value of raw slot k (src/shaders/adam.wgsl:60-71); slots 7 and 15 are not written.
__device__ __forceinline__ float activated(uint32_t k, float raw) {
  if (k >= 4 && k <= 6) return expf(raw);
  if (k == 3) return sigmoidf_(raw);
  if (k >= 12 && k <= 14) return 0.5f + SH_C0 * raw;
  return raw;
}


// src/shaders/adam.wgsl:112-121
__global__ void reset_opacity_kernel(float* __restrict__ params, float2* __restrict__ moments,
                                     float* __restrict__ gaussians, uint32_t count) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const size_t at = (size_t)i * FLOATS_PER_GAUSSIAN + 3;
  const float v = fminf(params[at], RESET_LOGIT);
  params[at] = v;
  moments[param_moment_at(i, RESET_SLOT)] = make_float2(0.f, 0.f);
  gaussians[at] = sigmoidf_(v);
}

// src/shaders/adam.wgsl:126-134 on a step without Adam (a densification step);
// on the others the backward pass with Adam accumulates them.
__global__ void stats_kernel(const AdamParams* __restrict__ ap, const float* __restrict__ splats,
                             const float* __restrict__ splat_grads, float4* __restrict__ stats,
                             float2* __restrict__ aux, uint32_t count) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  accumulate_stats_one(ap->viewport, splats, splat_grads, stats, aux, i);
}

// What happens to a Gaussian (src/shaders/densify.wgsl:72-85): 0 drop, 1 keep,
// 2 clone, 3 split. p0, p1: the first 32 bytes of its record (slots 3-6: opacity
// logit, log-scales); s: its statistics. A candidate the learned proposal
// declined (vetoed) is kept as it is, subject to the same pruning.
__device__ __forceinline__ uint32_t densify_decide(const DensifyParams& dp, float4 p0, float4 p1, float4 s,
                                                   bool vetoed) {
  const float grad = s.y > 0.0f ? s.x / s.y : 0.0f;
  const float size = expf(fmaxf(p1.x, fmaxf(p1.y, p1.z)));
  const float opacity = sigmoidf_(p0.w);
  auto removed = [&](float o, float sz) { return o < dp.min_opacity || (dp.max_size > 0.0f && sz > dp.max_size); };
  if (grad >= dp.grad_threshold && !vetoed) {
    if (size <= dp.clone_max_size) return removed(opacity, size) ? 0u : 2u;
    return removed(opacity, size / SPLIT_SHRINK) ? 0u : 3u;
  }
  return removed(opacity, size) ? 0u : 1u;
}

__device__ __forceinline__ uint32_t densify_action(const DensifyParams& dp, const float* __restrict__ params,
                                                   const float4* __restrict__ stats, uint32_t i,
                                                   const uint8_t* __restrict__ veto = nullptr) {
  const float4* record = reinterpret_cast<const float4*>(params + (size_t)i * FLOATS_PER_GAUSSIAN);
  return densify_decide(dp, record[0], record[1], stats[i], veto && veto[i]);
}

// src/shaders/densify.wgsl:96-107. Grid-stride over the resident CTAs: the tallies
// go to four global counters once per CTA, not once per 256 Gaussians. (Four
// Gaussians a thread with their loads issued together measured slower: 26.3
// against 23.8 us at 1.1M.)
__global__ void __launch_bounds__(256) densify_count_kernel(DensifyParams dp, const float* __restrict__ params,
                                                            const float4* __restrict__ stats,
                                                            const uint8_t* __restrict__ veto, uint32_t count,
                                                            uint32_t* __restrict__ outputs,
                                                            uint8_t* __restrict__ actions,
                                                            uint32_t* __restrict__ counters) {
  __shared__ uint32_t local[4];
  if (threadIdx.x < 4) local[threadIdx.x] = 0;
  __syncthreads();
  uint32_t mine[4] = {0, 0, 0, 0};
  for (uint32_t base = blockIdx.x * 256; base < count; base += gridDim.x * 256) {
    const uint32_t i = base + threadIdx.x;
    uint32_t a = 4;  // none
    if (i < count) {
      a = densify_action(dp, params, stats, i, veto);
      outputs[i] = a == 0 ? 0u : (a >= 2 ? 2u : 1u);
      actions[i] = (uint8_t)a;  // for the copy kernel, decided once
    }
#pragma unroll
    for (uint32_t v = 0; v < 4; v++) mine[v] += __popc(__ballot_sync(0xffffffffu, a == v));
  }
  // One shared-memory atomic per warp and action, one global one per CTA and action.
  if ((threadIdx.x & 31u) == 0)
#pragma unroll
    for (uint32_t v = 0; v < 4; v++)
      if (mine[v]) atomicAdd(&local[v], mine[v]);
  __syncthreads();
  if (threadIdx.x < 4 && local[threadIdx.x]) atomicAdd(&counters[threadIdx.x], local[threadIdx.x]);
}

__device__ __forceinline__ uint32_t pcg(uint32_t v) {
  const uint32_t state = v * 747796405u + 2891336453u;
  const uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
  return (word >> 22u) ^ word;
}

__device__ __forceinline__ float unit_of(uint32_t h) { return ((float)(h >> 8u) + 0.5f) / 16777216.0f; }

// Moment slot k (0-60) of Gaussian g in a set of n, in the two planes of
// param_moment_at / sh_moment_at.
__device__ __forceinline__ size_t moment_slot(uint32_t n, uint32_t g, uint32_t k) {
  return k < FLOATS_PER_GAUSSIAN ? param_moment_at(g, k) : sh_moment_at(n, g, k - FLOATS_PER_GAUSSIAN);
}

// What one lane reads of one Gaussian: the moments and values of its two slots
// (lane and lane + 32), and on lane 0 the identity and the steps seen.
struct SlotPair {
  float2 m[2];
  float v[2];
  uint32_t id;
  float seen;
};

__device__ __forceinline__ void densify_load(const float* __restrict__ params, const float* __restrict__ sh,
                                             const float2* __restrict__ moments, const uint32_t* __restrict__ ids,
                                             const float2* __restrict__ aux, uint32_t count, uint32_t i,
                                             uint32_t lane, SlotPair& s) {
#pragma unroll
  for (uint32_t h = 0; h < 2; h++) {
    const uint32_t k = lane + 32u * h;
    if (k < MOMENT_SLOTS) {
      s.m[h] = moments[moment_slot(count, i, k)];
      s.v[h] = k < FLOATS_PER_GAUSSIAN ? params[(size_t)i * FLOATS_PER_GAUSSIAN + k]
                                       : sh[(size_t)i * SH_REST_FLOATS + (k - FLOATS_PER_GAUSSIAN)];
    }
  }
  if (lane == 0) {
    s.id = ids[i];
    s.seen = aux[i].y;
  }
}

// Split children's positions: center + R (scale ⊙ n), n ~ N(0, I) from PCG and
// Box-Muller, for Gaussian i (raw record p) whose children are outputs o and o + 1.
__device__ __forceinline__ void place_split(const DensifyParams& dp, const float* __restrict__ p, uint32_t i,
                                            uint32_t o, float* __restrict__ new_params,
                                            float* __restrict__ new_gaussians) {
  // rotation_matrix (src/shaders/gaussianMath.wgsl:13-25)
  float dot = p[8] * p[8];
  dot = dot + p[9] * p[9];
  dot = dot + p[10] * p[10];
  dot = dot + p[11] * p[11];
  const float len = sqrtf(dot);
  const float qw = p[8] / len, qx = p[9] / len, qy = p[10] / len, qz = p[11] / len;
  float r[3][3];
  r[0][0] = 1.0f - 2.0f * (qy * qy + qz * qz);
  r[0][1] = 2.0f * (qx * qy + qw * qz);
  r[0][2] = 2.0f * (qx * qz - qw * qy);
  r[1][0] = 2.0f * (qx * qy - qw * qz);
  r[1][1] = 1.0f - 2.0f * (qx * qx + qz * qz);
  r[1][2] = 2.0f * (qy * qz + qw * qx);
  r[2][0] = 2.0f * (qx * qz + qw * qy);
  r[2][1] = 2.0f * (qy * qz - qw * qx);
  r[2][2] = 1.0f - 2.0f * (qx * qx + qy * qy);
  for (uint32_t c = 0; c < 2; c++) {
    const uint32_t h1 = pcg(dp.seed ^ pcg(2u * i + c));
    const uint32_t h2 = pcg(h1), h3 = pcg(h2), h4 = pcg(h3);
    const float tau = 6.283185307179586f;
    const float r1 = sqrtf(-2.0f * logf(unit_of(h1)));
    const float r2 = sqrtf(-2.0f * logf(unit_of(h3)));
    const float n0 = r1 * cosf(tau * unit_of(h2)), n1 = r1 * sinf(tau * unit_of(h2)), n2 = r2 * cosf(tau * unit_of(h4));
    const float sv[3] = {expf(p[4]) * n0, expf(p[5]) * n1, expf(p[6]) * n2};
    float* out = new_params + (size_t)(o + c) * FLOATS_PER_GAUSSIAN;
    float* act = new_gaussians + (size_t)(o + c) * FLOATS_PER_GAUSSIAN;
#pragma unroll
    for (int row = 0; row < 3; row++) {
      float v = r[0][row] * sv[0];
      v = v + r[1][row] * sv[1];
      v = v + r[2][row] * sv[2];
      out[row] = p[row] + v;
      act[row] = out[row];  // positions activate to themselves
    }
  }
}

// Writes the outputs of Gaussian i, whose action is a (1 keep, 2 clone, 3 split)
// and whose first output is o (src/shaders/densify.wgsl:148-180): a kept Gaussian
// and a clone's original keep their moments, identity and steps seen; new ones
// get zero moments, identity first_id + their output index and zero statistics;
// a clone's copy and split children are stamped with their kind and the step
// (slots 7 and 15), split children shrink by 1.6 (their positions are left to
// place_split). The activated values follow (src/shaders/adam.wgsl:74-77).
__device__ __forceinline__ void densify_store(const DensifyParams& dp, uint32_t first_id, uint32_t new_count,
                                              uint32_t a, uint32_t o, uint32_t lane, const SlotPair& s,
                                              float* __restrict__ new_params, float* __restrict__ new_sh,
                                              float2* __restrict__ new_moments, uint32_t* __restrict__ new_ids,
                                              float2* __restrict__ new_aux, float* __restrict__ new_gaussians) {
  const uint32_t copies = a == 1 ? 1u : 2u;
  const float2 zero = make_float2(0.f, 0.f);
  for (uint32_t c = 0; c < copies; c++) {
    const uint32_t dst = o + c;
    const bool keep = (a == 1 || a == 2) && c == 0;
    if (lane == 0) {
      new_ids[dst] = keep ? s.id : first_id + dst;
      new_aux[dst] = make_float2(0.0f, keep ? s.seen : 0.0f);
    }
#pragma unroll
    for (uint32_t h = 0; h < 2; h++) {
      const uint32_t k = lane + 32u * h;
      if (k >= MOMENT_SLOTS) continue;
      new_moments[moment_slot(new_count, dst, k)] = keep ? s.m[h] : zero;
      if (k < FLOATS_PER_GAUSSIAN) {
        float v = s.v[h];
        if (a == 2 && c == 1) {
          if (k == 7) v = 1.0f;
          if (k == 15) v = (float)dp.seed;
        }
        if (a == 3) {
          if (k < 3) continue;  // place_split's
          if (k >= 4 && k <= 6) v = s.v[h] - LOG_SPLIT_SHRINK;
          if (k == 7) v = 2.0f;
          if (k == 15) v = (float)dp.seed;
        }
        new_params[(size_t)dst * FLOATS_PER_GAUSSIAN + k] = v;
        if (k != 7 && k != 15) new_gaussians[(size_t)dst * FLOATS_PER_GAUSSIAN + k] = activated(k, v);
      } else {
        new_sh[(size_t)dst * SH_REST_FLOATS + (k - FLOATS_PER_GAUSSIAN)] = s.v[h];
      }
    }
  }
}

// src/shaders/densify.wgsl:148-180, split in two for coalescing. Each warp takes
// 32 consecutive Gaussians at a time: lane l reads the action and output offset
// of Gaussian l in one coalesced pass, then the warp copies the live ones two at
// a time, a moment slot per lane (lanes l and l + 32 of the 61; each slot's
// moment, raw value or SH coefficient is a contiguous run across the lanes), with
// both Gaussians' reads issued before their writes; split children's positions
// come last.
__global__ void __launch_bounds__(256) densify_copy_kernel(DensifyParams dp, const float* __restrict__ params,
                                                           const uint8_t* __restrict__ actions,
                                                           const float* __restrict__ sh,
                                                           const float2* __restrict__ moments,
                                                           const uint32_t* __restrict__ ids,
                                                           const float2* __restrict__ aux,
                                                           const uint32_t* __restrict__ outputs, uint32_t count,
                                                           uint32_t new_count, uint32_t first_id,
                                                           float* __restrict__ new_params,
                                                           float* __restrict__ new_sh,
                                                           float2* __restrict__ new_moments,
                                                           uint32_t* __restrict__ new_ids,
                                                           float2* __restrict__ new_aux,
                                                           float* __restrict__ new_gaussians) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, warps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t first = warp * 32u; first < count; first += warps * 32u) {
    const uint32_t mine = first + lane;
    const uint32_t my_action = mine < count ? actions[mine] : 0u;
    const uint32_t my_output = my_action ? outputs[mine] : 0u;
    uint32_t live = __ballot_sync(0xffffffffu, my_action != 0);
    while (live) {
      const uint32_t j0 = __ffs(live) - 1;
      live &= live - 1;
      const bool two = live != 0;  // the same on every lane
      const uint32_t j1 = two ? __ffs(live) - 1 : j0;
      if (two) live &= live - 1;
      const uint32_t a0 = __shfl_sync(0xffffffffu, my_action, j0), o0 = __shfl_sync(0xffffffffu, my_output, j0);
      const uint32_t a1 = __shfl_sync(0xffffffffu, my_action, j1), o1 = __shfl_sync(0xffffffffu, my_output, j1);
      SlotPair s0, s1;
      densify_load(params, sh, moments, ids, aux, count, first + j0, lane, s0);
      if (two) densify_load(params, sh, moments, ids, aux, count, first + j1, lane, s1);
      densify_store(dp, first_id, new_count, a0, o0, lane, s0, new_params, new_sh, new_moments, new_ids, new_aux,
                    new_gaussians);
      if (two)
        densify_store(dp, first_id, new_count, a1, o1, lane, s1, new_params, new_sh, new_moments, new_ids, new_aux,
                      new_gaussians);
    }
  }
  // Then the split children's positions, a thread per Gaussian (no other thread
  // writes those three values).
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
    if (actions[i] == 3) place_split(dp, params + (size_t)i * FLOATS_PER_GAUSSIAN, i, outputs[i], new_params,
                                     new_gaussians);
}

// The learned densification's inputs (see DG_MLP_FEATURES in the header),
// for every Gaussian.
struct FeatureParams {
  float centroid[3];
  float inv_extent, inv_threshold, inv_interval;
  float iteration;
};

__global__ void densify_features_kernel(FeatureParams fp, const float* __restrict__ params,
                                        const float4* __restrict__ stats, const float2* __restrict__ aux,
                                        uint32_t count, float* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float* p = params + (size_t)i * FLOATS_PER_GAUSSIAN;
  const float4 s = stats[i];
  const float2 a = aux[i];
  const float n = fmaxf(s.y, 1.0f);
  const float mean = s.y > 0.0f ? s.x / s.y : 0.0f;
  const float var = s.y > 0.0f ? fmaxf(a.x / n - mean * mean, 0.0f) : 0.0f;
  const float dx = p[0] - fp.centroid[0], dy = p[1] - fp.centroid[1], dz = p[2] - fp.centroid[2];
  const float r = 0.5f + SH_C0 * p[12], g = 0.5f + SH_C0 * p[13], b = 0.5f + SH_C0 * p[14];
  float* f = out + (size_t)i * 12;
  f[0] = mean * fp.inv_threshold;
  f[1] = s.y * fp.inv_interval;
  f[2] = log1pf(s.z);
  f[3] = p[4];
  f[4] = p[5];
  f[5] = p[6];
  f[6] = sigmoidf_(p[3]);
  f[7] = sqrtf(dx * dx + dy * dy + dz * dz) * fp.inv_extent;
  f[8] = 0.299f * r + 0.587f * g + 0.114f * b;
  f[9] = (fp.iteration - p[15]) * 1e-3f;
  f[10] = a.y * 1e-3f;
  f[11] = sqrtf(var) * fp.inv_threshold;
}

// The learned decision: a plain-rule candidate the model is confident about
// (max(p, 1 - p) >= min_confidence) is vetoed when p < 0.5. tallies: scored,
// confident, vetoed.
__global__ void densify_veto_kernel(DensifyParams dp, const float* __restrict__ params,
                                    const float4* __restrict__ stats, const float* __restrict__ survive,
                                    float min_confidence, uint32_t count, uint8_t* __restrict__ veto,
                                    unsigned long long* __restrict__ tallies) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  uint8_t v = 0;
  if (densify_action(dp, params, stats, i) >= 2) {
    const float p = survive[i];
    atomicAdd(&tallies[0], 1ull);
    if (fmaxf(p, 1.0f - p) >= min_confidence) {
      atomicAdd(&tallies[1], 1ull);
      if (p < 0.5f) {
        v = 1;
        atomicAdd(&tallies[2], 1ull);
      }
    }
  }
  veto[i] = v;
}

// The densify log: each clone/split candidate's features and the identities of
// its new children (a clone's copy; both halves of a split), and the identities
// of the Gaussians dropped. Slots come from atomics; order does not matter.
__global__ void densify_log_kernel(DensifyParams dp, const float* __restrict__ params,
                                   const float4* __restrict__ stats, const uint8_t* __restrict__ veto,
                                   const float* __restrict__ features, const uint32_t* __restrict__ ids,
                                   const uint32_t* __restrict__ outputs, uint32_t count, uint32_t first_id,
                                   float* __restrict__ log, uint32_t* __restrict__ dropped,
                                   uint32_t* __restrict__ cursors) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const uint32_t a = densify_action(dp, params, stats, i, veto);
  if (a == 0) {
    dropped[atomicAdd(&cursors[1], 1u)] = ids[i];
    return;
  }
  if (a < 2) return;
  const uint32_t slot = atomicAdd(&cursors[0], 1u);
  float* row = log + (size_t)slot * 14;
  for (int k = 0; k < 12; k++) row[k] = features[(size_t)i * 12 + k];
  const uint32_t o = outputs[i];
  const uint32_t c0 = a == 2 ? first_id + o + 1 : first_id + o, c1 = a == 2 ? 0xffffffffu : first_id + o + 1;
  row[12] = __uint_as_float(c0);
  row[13] = __uint_as_float(c1);
}

__global__ void iota_kernel(uint32_t* __restrict__ out, uint32_t count) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) out[i] = i;
}

}  // namespace
}  // namespace dg

using namespace dg;

// Trainer (src/trainer.ts:103-446).
struct dg_trainer {
  dg_context* ctx;
  dg_training_settings settings;
  struct View {
    dg_camera camera;
    dg_buffer* image;
  };
  std::vector<View> views;
  uint32_t iteration = 0, sh_degree = 0, adam_steps = 0, count = 0;
  dg_renderer* renderer = nullptr;
  dg_training_loss* loss = nullptr;
  dg_buffer* target = nullptr;  // the "training render" rgba8 texture
  dg_buffer* params = nullptr;
  dg_buffer* moments = nullptr;
  dg_buffer* stats = nullptr;
  dg_buffer* adam_params = nullptr;
  uint32_t random_state = 1;  // mulberry32(1), src/trainer.ts:121
  std::vector<uint32_t> queue;
  bool due_densify = false, due_reset = false;
  std::vector<dg_densification> densifications;
  // The captured optimize() step.
  bool graph_enabled = false;
  bool keep_gradients = false;  // store the Gaussian gradients Adam consumes in registers
  // Loss values requested and not yet taken: [loss_tail, loss_head) of a ring of
  // pinned slots, each with the event its copy completes.
  static constexpr uint32_t LOSS_RING = 16;
  double* loss_ring = nullptr;
  cudaEvent_t loss_events[LOSS_RING] = {};
  uint32_t loss_head = 0, loss_tail = 0;
  // Photos from pinned host memory (set_host_photos): each step's photo is copied
  // into one of two device slots on an upload stream, the next step's while the
  // current one runs. slot_free[s]: the last step reading slot s is done;
  // slot_ready[s]: its upload is done.
  std::vector<const void*> host_photos;
  dg_buffer* photo_slots[2] = {nullptr, nullptr};
  cudaStream_t upload_stream = nullptr;
  cudaEvent_t slot_free[2] = {}, slot_ready[2] = {};
  int64_t prefetch_view = -1;  // the view already uploading into prefetch_slot
  uint32_t prefetch_slot = 0, slot_used = 1;
  cudaGraphExec_t graph_exec = nullptr;
  uint64_t graph_launches = 0;
  struct Key {
    uint32_t count, capacity;
    void *gaussians, *pairs, *pixel_grads;
    bool operator==(const Key& o) const {
      return count == o.count && capacity == o.capacity && gaussians == o.gaussians && pairs == o.pairs &&
             pixel_grads == o.pixel_grads;
    }
  } graph_key{};
  // Learned densification. Every Gaussian has an identity (children get fresh
  // ones) and aux statistics (float2: squared gradient norms since the last
  // densification, steps seen over its life).
  dg_buffer* ids = nullptr;
  dg_buffer* aux = nullptr;
  uint32_t next_id = 0;
  float centroid[3] = {0.0f, 0.0f, 0.0f};  // of the training cameras
  dg_densify_mlp* mlp = nullptr;
  float mlp_confidence = 0.6f;
  uint64_t mlp_tallies[3] = {0, 0, 0};  // scored, confident, vetoed
  // The densify log: samples wait until their horizon; a child dropped before it
  // counts against its sample.
  bool log_enabled = false;
  uint32_t log_horizon = 1000;
  struct Pending {
    float features[12];
    uint32_t children[2];
    uint32_t due, alive;
    bool resolved;
  };
  std::vector<Pending> pending;
  std::unordered_map<uint32_t, uint32_t> tracked;  // child identity -> pending index
  std::vector<float> done_features;
  std::vector<uint8_t> done_labels;
};

namespace dg {

static double mulberry32_next(uint32_t& state) {
  state = state + 0x6d2b79f5u;
  uint32_t t = state;
  t = (t ^ (t >> 15)) * (t | 1u);
  t ^= t + (t ^ (t >> 7)) * (t | 61u);
  return (double)(t ^ (t >> 14)) / 4294967296.0;
}

// Every view once, in a random order, then reshuffle (src/trainer.ts:395-404).
static uint32_t next_view(dg_trainer* t) {
  if (t->queue.empty()) {
    t->queue.resize(t->views.size());
    for (uint32_t k = 0; k < t->views.size(); k++) t->queue[k] = k;
    for (int64_t i = (int64_t)t->queue.size() - 1; i > 0; i--) {
      int64_t j = (int64_t)std::floor(mulberry32_next(t->random_state) * (double)(i + 1));
      std::swap(t->queue[i], t->queue[j]);
    }
  }
  uint32_t v = t->queue.back();
  t->queue.pop_back();
  return v;
}

// The view the next optimize() renders, without taking it (a new round is
// shuffled first if needed, exactly as next_view would).
static uint32_t peek_view(dg_trainer* t) {
  if (t->queue.empty()) t->queue.push_back(next_view(t));
  return t->queue.back();
}

// Copies view `view`'s host photo into slot `slot` on the upload stream, once
// the last step that read the slot is done.
static dg_status upload_photo(dg_trainer* t, uint32_t slot, uint32_t view) {
  const uint64_t bytes = t->photo_slots[slot]->bytes;
  DG_CUDA(cudaStreamWaitEvent(t->upload_stream, t->slot_free[slot], 0));
  DG_CUDA(cudaMemcpyAsync(t->photo_slots[slot]->ptr, t->host_photos[view], bytes, cudaMemcpyHostToDevice,
                          t->upload_stream));
  DG_CUDA(cudaEventRecord(t->slot_ready[slot], t->upload_stream));
  t->prefetch_view = view;
  t->prefetch_slot = slot;
  return DG_OK;
}

static dg_status launch_stats(dg_trainer* t) {
  dg_renderer* r = t->renderer;
  DG_LAUNCH(t->ctx, "stats",
            stats_kernel<<<ceil_div(t->count, 256), 256, 0, t->ctx->stream>>>(
                typed<AdamParams>(t->adam_params), typed<float>(r->splats), typed<float>(r->grad_splats),
                typed<float4>(t->stats), typed<float2>(t->aux), t->count));
  return DG_OK;
}

// The kernels of one optimize() step, in order. Everything the host decides per
// step (camera, photo, SH degree, learning rates) is in device uniforms written
// before this runs, so the same launches can be captured once and replayed.
static dg_status launch_step(dg_trainer* t, bool with_adam) {
  dg_renderer* r = t->renderer;
  DG_TRY(renderer_launch_forward(r, t->target));
  DG_TRY(loss_launch(t->loss, r->rasterizer->pixel_color));
  // The splat gradients; each Gaussian's own gradients come from the preprocess
  // backward pass, which on an Adam step applies Adam to them at once and adds up
  // the densification statistics (on a densification step nothing uses them
  // unless they are kept).
  DG_TRY(renderer_launch_backward(r, t->loss->pixel_grads, !with_adam && t->keep_gradients));
  if (with_adam)
    DG_TRY(launch_preprocess_backward_adam(r, typed<AdamParams>(t->adam_params), typed<float>(t->params),
                                           typed<float2>(t->moments), typed<float4>(t->stats),
                                           typed<float2>(t->aux), t->keep_gradients));
  else
    DG_TRY(launch_stats(t));
  return DG_OK;
}

static void drop_graph(dg_trainer* t) {
  if (t->graph_exec) cudaGraphExecDestroy(t->graph_exec);
  t->graph_exec = nullptr;
}

static dg_status run_graph_step(dg_trainer* t) {
  dg_renderer* r = t->renderer;
  dg_trainer::Key key{t->count, r->rasterizer->pair_capacity, r->gaussians->ptr, r->rasterizer->keys->ptr,
                      t->loss->pixel_grads->ptr};
  if (!t->graph_exec || !(key == t->graph_key)) {
    drop_graph(t);
    cudaGraph_t graph;
    const uint64_t before = t->ctx->launches;
    DG_CUDA(cudaStreamBeginCapture(t->ctx->stream, cudaStreamCaptureModeThreadLocal));
    t->ctx->capturing = true;
    dg_status st = launch_step(t, true);
    t->ctx->capturing = false;
    cudaError_t end = cudaStreamEndCapture(t->ctx->stream, &graph);
    if (st != DG_OK) {
      if (end == cudaSuccess) cudaGraphDestroy(graph);
      return st;
    }
    DG_CUDA(end);
    cudaError_t inst = cudaGraphInstantiate(&t->graph_exec, graph, 0);
    cudaGraphDestroy(graph);
    DG_CUDA(inst);
    t->graph_key = key;
    t->graph_launches = t->ctx->launches - before;
    t->ctx->launches = before;
  }
  DG_CUDA(cudaGraphLaunch(t->graph_exec, t->ctx->stream));
  t->ctx->launches += t->graph_launches;
  return DG_OK;
}

static dg_status storage(dg_trainer* t, size_t bytes, dg_buffer** out) { return alloc_buffer(t->ctx, bytes, out); }

// Labels the pending samples whose horizon has come (1: a child is still alive)
// and drops resolved entries once they are most of the list.
static void resolve_samples(dg_trainer* t) {
  uint32_t resolved = 0;
  for (auto& p : t->pending) {
    if (!p.resolved && p.due <= t->iteration) {
      p.resolved = true;
      t->done_features.insert(t->done_features.end(), p.features, p.features + 12);
      t->done_labels.push_back(p.alive > 0 ? 1 : 0);
      for (uint32_t c : p.children)
        if (c != 0xffffffffu) t->tracked.erase(c);
    }
    resolved += p.resolved;
  }
  if (resolved > 1024 && 2 * resolved > t->pending.size()) {
    std::vector<dg_trainer::Pending> keep;
    for (auto& p : t->pending)
      if (!p.resolved) keep.push_back(p);
    t->pending.swap(keep);
    t->tracked.clear();
    for (uint32_t k = 0; k < t->pending.size(); k++)
      for (uint32_t c : t->pending[k].children)
        if (c != 0xffffffffu) t->tracked[c] = k;
  }
}

// The camera center of a column-major world-to-camera matrix: -R^T t.
static void camera_center(const float* view, float* out) {
  for (int j = 0; j < 3; j++) out[j] = -(view[j * 4 + 0] * view[12] + view[j * 4 + 1] * view[13] + view[j * 4 + 2] * view[14]);
}

}  // namespace dg

// A grid-stride kernel's grid of 256-thread CTAs over `units` items: at most one
// wave of the CTAs that fit on the GPU at once (a second, partial wave would
// leave most SMs idle while it finishes).
template <typename Kernel>
static uint32_t resident_grid(const dg_context* ctx, Kernel kernel, uint32_t units) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, 0) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  return std::max(1u, std::min(ceil_div(units, 256u), (uint32_t)(ctx->sm_count * per_sm)));
}

extern "C" {

void dg_training_settings_default(dg_training_settings* s, double extent) {
  if (!s) return;
  s->extent = extent;
  s->position_lr_steps = 30000;
  s->position_lr[0] = 0.00016;
  s->position_lr[1] = 0.0000016;
  s->opacity_lr = 0.025;
  s->scale_lr = 0.005;
  s->rotation_lr = 0.001;
  s->color_lr = 0.0025;
  s->sh_lr = 0.0025 / 20;
  s->sh_degree_interval = 1000;
  s->densify_from = 500;
  s->densify_until = 15000;
  s->densify_interval = 100;
  s->densify_grad_threshold = 0.0002;
  s->percent_dense = 0.01;
  s->min_opacity = 0.005;
  s->opacity_reset_interval = 3000;
  s->background[0] = s->background[1] = s->background[2] = 0.0f;
}

dg_status dg_trainer_create(dg_context* ctx, const float* params, const float* sh, uint32_t count,
                            const dg_training_view* views, uint32_t view_count, const dg_training_settings* settings,
                            dg_trainer** out) {
  DG_REQUIRE(ctx && params && sh && views && settings && out, "NULL argument");
  DG_REQUIRE(view_count > 0, "no training views");
  DG_REQUIRE(count > 0, "no Gaussians");
  DG_REQUIRE(count < (1u << 26), "at most 2^26 Gaussians (Adam indexes slots with 32 bits)");
  const float w = views[0].camera.viewport[0], h = views[0].camera.viewport[1];
  for (uint32_t k = 0; k < view_count; k++)
    if (views[k].camera.viewport[0] != w || views[k].camera.viewport[1] != h)
      return fail(DG_ERROR_INVALID_ARGUMENT, "All training views must be the same size.");
  for (uint32_t k = 0; k < view_count; k++)
    DG_REQUIRE(views[k].image && views[k].image->bytes >= (uint64_t)w * h * 4, "a view's image is too small");
  auto* t = new dg_trainer();
  t->ctx = ctx;
  t->settings = *settings;
  for (uint32_t k = 0; k < view_count; k++) t->views.push_back({views[k].camera, views[k].image});
  t->count = count;
  // Activate on the host once, as the reference does (src/trainer.ts:138-140).
  std::vector<float> act((size_t)count * FLOATS_PER_GAUSSIAN, 0.0f);
  for (size_t at = 0; at < act.size(); at += FLOATS_PER_GAUSSIAN) {
    for (int k = 0; k < 3; k++) {
      act[at + k] = params[at + k];
      act[at + 4 + k] = (float)std::exp((double)params[at + 4 + k]);
      act[at + 12 + k] = (float)(0.5 + 0.28209479177387814 * (double)params[at + 12 + k]);
    }
    act[at + 3] = (float)(1.0 / (1.0 + std::exp(-(double)params[at + 3])));
    for (int k = 8; k < 12; k++) act[at + k] = params[at + k];
  }
  dg_status st = dg_renderer_create(ctx, 0, &t->renderer);
  if (st == DG_OK) st = dg_renderer_set_gaussians(t->renderer, act.data(), count, sh, (uint64_t)count * SH_REST_FLOATS, 0);
  if (st == DG_OK) st = dg_training_loss_create(ctx, (uint32_t)w, (uint32_t)h, &t->loss);
  if (st == DG_OK) st = storage(t, (size_t)w * h * 4, &t->target);
  if (st == DG_OK) st = storage(t, (size_t)count * FLOATS_PER_GAUSSIAN * 4, &t->params);
  if (st == DG_OK) st = write_async(ctx, t->params->ptr, params, (size_t)count * FLOATS_PER_GAUSSIAN * 4);
  if (st == DG_OK) st = storage(t, (size_t)count * MOMENT_SLOTS * 8, &t->moments);
  if (st == DG_OK) st = storage(t, (size_t)count * 16, &t->stats);
  if (st == DG_OK) st = storage(t, sizeof(AdamParams), &t->adam_params);
  if (st == DG_OK) st = storage(t, (size_t)count * 4, &t->ids);
  if (st == DG_OK) st = storage(t, (size_t)count * 8, &t->aux);
  if (st == DG_OK) {
    iota_kernel<<<ceil_div(count, 256), 256, 0, ctx->stream>>>(typed<uint32_t>(t->ids), count);
    ctx->launches++;
    t->next_id = count;
    for (uint32_t k = 0; k < view_count; k++) {
      float c[3];
      camera_center(views[k].camera.view, c);
      for (int j = 0; j < 3; j++) t->centroid[j] += c[j] / view_count;
    }
  }
  if (st == DG_OK) st = renderer_ensure_gradients(t->renderer);
  if (st != DG_OK) {
    dg_trainer_destroy(t);
    return st;
  }
  *out = t;
  return DG_OK;
}

dg_status dg_trainer_optimize(dg_trainer* t) {
  DG_REQUIRE(t, "NULL argument");
  const dg_training_settings& s = t->settings;
  const uint32_t it = ++t->iteration;
  dg_renderer* r = t->renderer;
  if (it % s.sh_degree_interval == 0 && t->sh_degree < 3) DG_TRY(dg_renderer_set_sh_degree(r, ++t->sh_degree));
  const bool densifying = it < s.densify_until;
  const bool densify_now = densifying && it > s.densify_from && it % s.densify_interval == 0;
  const uint32_t view_index = next_view(t);
  const dg_trainer::View& view = t->views[view_index];
  // Uniforms of this step: camera, background, photo, learning rates.
  DG_TRY(renderer_prepare(r, &view.camera, s.background));
  const void* photo = view.image->ptr;
  const bool from_host = !t->host_photos.empty();
  uint32_t slot = 0;
  if (from_host) {
    if (t->prefetch_view == (int64_t)view_index) {
      slot = t->prefetch_slot;
    } else {
      slot = t->slot_used ^ 1u;
      DG_TRY(upload_photo(t, slot, view_index));
    }
    t->prefetch_view = -1;
    DG_CUDA(cudaStreamWaitEvent(t->ctx->stream, t->slot_ready[slot], 0));
    photo = t->photo_slots[slot]->ptr;
  }
  DG_TRY(write_async(t->ctx, t->loss->target_slot->ptr, &photo, sizeof(photo)));
  if (!densify_now) t->adam_steps++;
  const double progress = std::min(1.0, it / s.position_lr_steps);
  const double position_lr =
      std::exp(std::log(s.position_lr[0]) * (1 - progress) + std::log(s.position_lr[1]) * progress) * s.extent;
  AdamParams ap{};
  ap.bias_correction1 = (float)(1 - std::pow(0.9, t->adam_steps));
  ap.bias_correction2 = (float)(1 - std::pow(0.999, t->adam_steps));
  ap.inv_bias_correction1 = (float)(1.0 / (double)ap.bias_correction1);
  ap.inv_sqrt_bias_correction2 = (float)(1.0 / std::sqrt((double)ap.bias_correction2));
  ap.position_lr = (float)position_lr;
  ap.opacity_lr = (float)s.opacity_lr;
  ap.scale_lr = (float)s.scale_lr;
  ap.rotation_lr = (float)s.rotation_lr;
  ap.color_lr = (float)s.color_lr;
  ap.sh_lr = (float)s.sh_lr;
  ap.viewport[0] = view.camera.viewport[0];
  ap.viewport[1] = view.camera.viewport[1];
  DG_TRY(write_async(t->ctx, t->adam_params->ptr, &ap, sizeof(ap)));
  if (t->graph_enabled && !densify_now) {
    DG_TRY(run_graph_step(t));
  } else {
    DG_TRY(launch_step(t, !densify_now));
  }
  // The frame's pair count, for afterSubmit (src/tileRasterizer.ts:187-191): queued
  // after the step (outside any captured graph), consumed once it has arrived; a
  // frame that needed more pairs than the buffers hold grows them for the next.
  dg_tile_rasterizer* tr = r->rasterizer;
  DG_TRY(rasterizer_queue_readback(tr));
  DG_TRY(dg_tile_rasterizer_after_submit(tr, 0));
  t->due_densify = densify_now;
  t->due_reset = densifying && it % s.opacity_reset_interval == 0;
  if (from_host) {
    // This step's reads of the slot are enqueued; the next step's photo goes
    // into the other slot while this one runs.
    DG_CUDA(cudaEventRecord(t->slot_free[slot], t->ctx->stream));
    t->slot_used = slot;
    DG_TRY(upload_photo(t, slot ^ 1u, peek_view(t)));
  }
  return DG_OK;
}

dg_status dg_trainer_maintain(dg_trainer* t) {
  DG_REQUIRE(t, "NULL argument");
  const bool densify = t->due_densify, reset = t->due_reset;
  t->due_densify = t->due_reset = false;
  if (densify) DG_TRY(dg_trainer_densify(t, t->iteration > t->settings.opacity_reset_interval));
  if (reset) DG_TRY(dg_trainer_reset_opacity(t));
  return DG_OK;
}

dg_status dg_trainer_step(dg_trainer* t) {
  DG_TRY(dg_trainer_optimize(t));
  return dg_trainer_maintain(t);
}

dg_status dg_trainer_densify(dg_trainer* t, int32_t prune_large) {
  DG_REQUIRE(t, "NULL argument");
  dg_context* ctx = t->ctx;
  const dg_training_settings& s = t->settings;
  const uint32_t count = t->count;
  DensifyParams dp;
  dp.grad_threshold = (float)s.densify_grad_threshold;
  dp.clone_max_size = (float)(s.percent_dense * s.extent);
  dp.min_opacity = (float)s.min_opacity;
  dp.max_size = prune_large ? (float)(0.1 * s.extent) : 0.0f;
  dp.seed = t->iteration;
  std::vector<dg_buffer*> temps;
  auto temp = [&](size_t bytes, dg_buffer** out) {
    const dg_status st = alloc_buffer(ctx, std::max<size_t>(bytes, 16), out);
    if (st == DG_OK) temps.push_back(*out);
    return st;
  };
  auto release = [&]() {
    for (dg_buffer* b : temps) free_buffer(b);
    temps.clear();
  };
  dg_status st = DG_OK;
  dg_buffer *outputs = nullptr, *counters = nullptr, *scratch = nullptr;
  dg_buffer *features = nullptr, *survive = nullptr, *veto = nullptr, *tallies = nullptr;
  if (st == DG_OK) st = temp((size_t)count * 4 + 4, &outputs);  // + the scan total
  dg_buffer* actions = nullptr;
  if (st == DG_OK) st = temp(count, &actions);
  if (st == DG_OK) st = temp(16, &counters);
  if (st == DG_OK) st = temp(scan_scratch_bytes(count), &scratch);
  // The learned proposal's inputs, and its decision on the plain rule's candidates.
  if (st == DG_OK && (t->log_enabled || t->mlp)) {
    st = temp((size_t)count * 12 * 4, &features);
    if (st == DG_OK) {
      FeatureParams fp;
      for (int j = 0; j < 3; j++) fp.centroid[j] = t->centroid[j];
      fp.inv_extent = (float)(1.0 / s.extent);
      fp.inv_threshold = (float)(1.0 / s.densify_grad_threshold);
      fp.inv_interval = 1.0f / (float)std::max(1u, s.densify_interval);
      fp.iteration = (float)t->iteration;
      DG_LAUNCH(ctx, "densify_features",
                densify_features_kernel<<<ceil_div(count, 256), 256, 0, ctx->stream>>>(
                    fp, typed<float>(t->params), typed<float4>(t->stats), typed<float2>(t->aux), count,
                    typed<float>(features)));
    }
  }
  if (st == DG_OK && t->mlp) {
    st = temp((size_t)count * 4, &survive);
    if (st == DG_OK) st = temp(count, &veto);
    if (st == DG_OK) st = temp(24, &tallies);
    if (st == DG_OK) st = mlp_predict_launch(t->mlp, typed<float>(features), count, typed<float>(survive));
    if (st == DG_OK) {
      DG_LAUNCH(ctx, "densify_veto",
                densify_veto_kernel<<<ceil_div(count, 256), 256, 0, ctx->stream>>>(
                    dp, typed<float>(t->params), typed<float4>(t->stats), typed<float>(survive), t->mlp_confidence,
                    count, typed<uint8_t>(veto), typed<unsigned long long>(tallies)));
    }
  }
  if (st != DG_OK) {
    release();
    return st;
  }
  const uint8_t* veto_ptr = veto ? typed<uint8_t>(veto) : nullptr;
  DG_LAUNCH(ctx, "densify_count",
            densify_count_kernel<<<resident_grid(ctx, densify_count_kernel, count), 256, 0, ctx->stream>>>(
                dp, typed<float>(t->params), typed<float4>(t->stats), veto_ptr, count, typed<uint32_t>(outputs),
                typed<uint8_t>(actions), typed<uint32_t>(counters)));
  uint32_t* total_ptr = typed<uint32_t>(outputs) + count;
  st = scan_launch(ctx, typed<uint32_t>(outputs), count, nullptr, total_ptr, scratch->ptr);
  uint32_t readback[5];
  unsigned long long tally[3] = {0, 0, 0};
  if (st == DG_OK) {
    DG_CUDA(cudaMemcpyAsync(readback, total_ptr, 4, cudaMemcpyDeviceToHost, ctx->stream));
    DG_CUDA(cudaMemcpyAsync(readback + 1, counters->ptr, 16, cudaMemcpyDeviceToHost, ctx->stream));
    if (tallies) DG_CUDA(cudaMemcpyAsync(tally, tallies->ptr, 24, cudaMemcpyDeviceToHost, ctx->stream));
    DG_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  if (st != DG_OK) {
    release();
    return st;
  }
  const uint32_t new_count = readback[0];
  if (new_count == 0) {
    release();
    return fail(DG_ERROR_STATE, "Densification removed every Gaussian.");
  }
  if (new_count >= (1u << 26)) {
    release();
    return fail(DG_ERROR_STATE, "Densification would exceed 2^26 Gaussians (Adam indexes slots with 32 bits).");
  }
  for (int k = 0; k < 3; k++) t->mlp_tallies[k] += tally[k];
  t->densifications.push_back(
      {t->iteration, count, new_count, readback[2], readback[3], readback[4], readback[1]});
  const uint32_t first_id = t->next_id;
  // The log: candidates' features and new children, and the identities dropped.
  const uint32_t candidates = readback[3] + readback[4], dropped_count = readback[1];
  std::vector<float> log_rows;
  std::vector<uint32_t> dropped_ids;
  if (t->log_enabled) {
    dg_buffer *log = nullptr, *dropped = nullptr, *cursors = nullptr;
    st = temp((size_t)candidates * 14 * 4, &log);
    if (st == DG_OK) st = temp((size_t)dropped_count * 4, &dropped);
    if (st == DG_OK) st = temp(8, &cursors);
    if (st == DG_OK) {
      DG_LAUNCH(ctx, "densify_log",
                densify_log_kernel<<<ceil_div(count, 256), 256, 0, ctx->stream>>>(
                    dp, typed<float>(t->params), typed<float4>(t->stats), veto_ptr, typed<float>(features),
                    typed<uint32_t>(t->ids), typed<uint32_t>(outputs), count, first_id, typed<float>(log),
                    typed<uint32_t>(dropped), typed<uint32_t>(cursors)));
      log_rows.resize((size_t)candidates * 14);
      dropped_ids.resize(dropped_count);
      if (candidates)
        DG_CUDA(cudaMemcpyAsync(log_rows.data(), log->ptr, log_rows.size() * 4, cudaMemcpyDeviceToHost, ctx->stream));
      if (dropped_count)
        DG_CUDA(cudaMemcpyAsync(dropped_ids.data(), dropped->ptr, dropped_count * 4, cudaMemcpyDeviceToHost,
                                ctx->stream));
    }
  }
  dg_buffer *params = nullptr, *sh = nullptr, *moments = nullptr, *stats = nullptr, *gaussians = nullptr;
  dg_buffer *ids = nullptr, *aux = nullptr;
  if (st == DG_OK) st = storage(t, (size_t)new_count * FLOATS_PER_GAUSSIAN * 4, &params);
  if (st == DG_OK) st = storage(t, (size_t)new_count * SH_REST_FLOATS * 4, &sh);
  if (st == DG_OK) st = storage(t, (size_t)new_count * MOMENT_SLOTS * 8, &moments);
  if (st == DG_OK) st = storage(t, (size_t)new_count * 16, &stats);
  if (st == DG_OK) st = storage(t, (size_t)new_count * FLOATS_PER_GAUSSIAN * 4, &gaussians);
  if (st == DG_OK) st = storage(t, (size_t)new_count * 4, &ids);
  if (st == DG_OK) st = storage(t, (size_t)new_count * 8, &aux);
  if (st != DG_OK) {
    for (dg_buffer* b : {params, sh, moments, stats, gaussians, ids, aux}) free_buffer(b);
    release();
    return st;
  }
  dg_renderer* r = t->renderer;
  DG_LAUNCH(ctx, "densify_copy",
            densify_copy_kernel<<<resident_grid(ctx, densify_copy_kernel, count), 256, 0, ctx->stream>>>(
                dp, typed<float>(t->params), typed<uint8_t>(actions), typed<float>(r->sh),
                typed<float2>(t->moments), typed<uint32_t>(t->ids), typed<float2>(t->aux), typed<uint32_t>(outputs),
                count, new_count, first_id, typed<float>(params), typed<float>(sh), typed<float2>(moments),
                typed<uint32_t>(ids), typed<float2>(aux), typed<float>(gaussians)));
  // The last frame's pair count (every queued readback has arrived: the counts
  // above were read back), scaled to the new count with 10% to spare, sizes the
  // new set's pair buffers, so the frames after a densification do not overflow
  // them while their own readbacks are in flight (the reference grows them a
  // frame or two later, after such a frame, src/tileRasterizer.ts:229-244).
  st = dg_tile_rasterizer_after_submit(r->rasterizer, 1);
  const double last_pairs = r->rasterizer ? (double)r->rasterizer->last_pair_count : 0.0;
  // Hand the new set to the renderer; the old buffers go once the work above is done.
  drop_graph(t);
  if (st == DG_OK) st = dg_renderer_adopt_gaussians(r, new_count, gaussians, sh, t->sh_degree);
  if (st == DG_OK) st = rasterizer_reserve_pairs(r->rasterizer, (uint64_t)(last_pairs * new_count / count * 1.1));
  if (st == DG_OK) st = renderer_ensure_gradients(r);
  if (t->log_enabled && st == DG_OK) {
    DG_CUDA(cudaStreamSynchronize(ctx->stream));
    // Drops first (they happened before the new children existed), then the new samples.
    for (uint32_t id : dropped_ids) {
      auto it = t->tracked.find(id);
      if (it == t->tracked.end()) continue;
      dg_trainer::Pending& p = t->pending[it->second];
      if (p.alive > 0) p.alive--;
      t->tracked.erase(it);
    }
    for (uint32_t k = 0; k < candidates; k++) {
      const float* row = log_rows.data() + (size_t)k * 14;
      dg_trainer::Pending p{};
      std::memcpy(p.features, row, 12 * 4);
      std::memcpy(p.children, row + 12, 8);
      p.due = t->iteration + t->log_horizon;
      p.alive = p.children[1] == 0xffffffffu ? 1u : 2u;
      p.resolved = false;
      for (uint32_t c : p.children)
        if (c != 0xffffffffu) t->tracked[c] = (uint32_t)t->pending.size();
      t->pending.push_back(p);
    }
  }
  resolve_samples(t);
  for (dg_buffer* b : {t->params, t->moments, t->stats, t->ids, t->aux}) free_buffer(b);
  release();
  t->params = params;
  t->moments = moments;
  t->stats = stats;
  t->ids = ids;
  t->aux = aux;
  t->count = new_count;
  t->next_id = first_id + new_count;
  return st;
}

dg_status dg_trainer_set_keep_gradients(dg_trainer* t, int32_t enabled) {
  DG_REQUIRE(t, "NULL argument");
  t->keep_gradients = enabled != 0;
  drop_graph(t);
  return DG_OK;
}

dg_status dg_trainer_set_densify_log(dg_trainer* t, int32_t enabled, uint32_t horizon) {
  DG_REQUIRE(t, "NULL argument");
  t->log_enabled = enabled != 0;
  t->log_horizon = horizon ? horizon : 1000;
  return DG_OK;
}

dg_status dg_trainer_take_densify_samples(dg_trainer* t, float* features, uint8_t* labels, uint32_t capacity,
                                          uint32_t* count, uint32_t* pending) {
  DG_REQUIRE(t && count, "NULL argument");
  resolve_samples(t);
  const uint32_t have = (uint32_t)t->done_labels.size();
  uint32_t waiting = 0;
  for (const auto& p : t->pending) waiting += !p.resolved;
  if (pending) *pending = waiting;
  if (!features) {
    *count = have;
    return DG_OK;
  }
  DG_REQUIRE(labels, "NULL argument");
  const uint32_t n = std::min(capacity, have);
  std::memcpy(features, t->done_features.data(), (size_t)n * 12 * 4);
  std::memcpy(labels, t->done_labels.data(), n);
  t->done_features.erase(t->done_features.begin(), t->done_features.begin() + (size_t)n * 12);
  t->done_labels.erase(t->done_labels.begin(), t->done_labels.begin() + n);
  *count = n;
  return DG_OK;
}

dg_status dg_trainer_set_densify_mlp(dg_trainer* t, dg_densify_mlp* mlp, float min_confidence) {
  DG_REQUIRE(t, "NULL argument");
  DG_REQUIRE(min_confidence >= 0.5f && min_confidence <= 1.0f, "min_confidence must be in [0.5, 1]");
  t->mlp = mlp;
  t->mlp_confidence = min_confidence;
  return DG_OK;
}

dg_status dg_trainer_densify_mlp_stats(const dg_trainer* t, uint64_t* scored, uint64_t* confident, uint64_t* vetoed) {
  DG_REQUIRE(t && scored && confident && vetoed, "NULL argument");
  *scored = t->mlp_tallies[0];
  *confident = t->mlp_tallies[1];
  *vetoed = t->mlp_tallies[2];
  return DG_OK;
}

dg_status dg_trainer_reset_opacity(dg_trainer* t) {
  DG_REQUIRE(t, "NULL argument");
  DG_LAUNCH(t->ctx, "reset_opacity",
            reset_opacity_kernel<<<ceil_div(t->count, 256), 256, 0, t->ctx->stream>>>(
                typed<float>(t->params), typed<float2>(t->moments), typed<float>(t->renderer->gaussians),
                t->count));
  return DG_OK;
}

dg_status dg_trainer_export_raw(dg_trainer* t, float* params, float* sh) {
  DG_REQUIRE(t && params && sh, "NULL argument");
  DG_CUDA(cudaMemcpyAsync(params, t->params->ptr, (size_t)t->count * FLOATS_PER_GAUSSIAN * 4, cudaMemcpyDeviceToHost,
                          t->ctx->stream));
  DG_CUDA(cudaMemcpyAsync(sh, t->renderer->sh->ptr, (size_t)t->count * SH_REST_FLOATS * 4, cudaMemcpyDeviceToHost,
                          t->ctx->stream));
  DG_CUDA(cudaStreamSynchronize(t->ctx->stream));
  return DG_OK;
}

dg_status dg_trainer_last_loss(dg_trainer* t, double* out) {
  DG_REQUIRE(t && out, "NULL argument");
  return dg_training_loss_read(t->loss, out);
}

dg_status dg_trainer_evaluate(dg_trainer* t, const dg_training_view* views, uint32_t view_count, int32_t with_ssim,
                              double* psnr, double* ssim) {
  DG_REQUIRE(t && views && psnr && ssim, "NULL argument");
  DG_REQUIRE(view_count > 0, "no views");
  dg_context* ctx = t->ctx;
  for (uint32_t k = 1; k < view_count; k++)
    DG_REQUIRE(views[k].camera.viewport[0] == views[0].camera.viewport[0] &&
                   views[k].camera.viewport[1] == views[0].camera.viewport[1],
               "All evaluated views must be the same size.");
  const uint32_t w = (uint32_t)views[0].camera.viewport[0], h = (uint32_t)views[0].camera.viewport[1];
  const size_t pixels = (size_t)w * h;
  for (uint32_t k = 0; k < view_count; k++)
    DG_REQUIRE(views[k].image && views[k].image->bytes >= pixels * 4, "a view's image is too small");
  dg_buffer *sums = nullptr, *slot = nullptr, *rendered = nullptr;
  DG_TRY(alloc_buffer(ctx, view_count * 16, &sums));
  DG_TRY(alloc_buffer(ctx, 8 * view_count, &slot));
  DG_TRY(alloc_buffer(ctx, pixels * 16 * view_count, &rendered));
  std::vector<const void*> photos(view_count);
  std::vector<dg_camera> cameras(view_count);
  for (uint32_t k = 0; k < view_count; k++) {
    photos[k] = views[k].image->ptr;
    cameras[k] = views[k].camera;
  }
  DG_TRY(write_async(ctx, slot->ptr, photos.data(), 8 * view_count));
  // Every view rendered in batches (dg_views.cu), then scored on the GPU.
  dg_renderer* r = t->renderer;
  DG_TRY(views_render(r, cameras.data(), view_count, t->settings.background, nullptr, typed<float4>(rendered),
                      r->view_batch, r->view_coop_min, r->view_shape));
  for (uint32_t k = 0; k < view_count; k++) {
    dg_buffer view_rendered{ctx, static_cast<char*>(rendered->ptr) + pixels * 16 * k, pixels * 16, false};
    dg_buffer view_slot{ctx, static_cast<char*>(slot->ptr) + 8 * k, 8, false};
    DG_TRY(metrics_launch(ctx, &view_rendered, &view_slot, w, h, typed<double>(sums) + 2 * k));
  }
  std::vector<double> host(2 * view_count);
  DG_CUDA(cudaMemcpyAsync(host.data(), sums->ptr, 16 * view_count, cudaMemcpyDeviceToHost, ctx->stream));
  DG_CUDA(cudaStreamSynchronize(ctx->stream));
  double psnr_total = 0, ssim_total = 0;
  for (uint32_t k = 0; k < view_count; k++) {
    const double pixels = (double)(uint32_t)views[k].camera.viewport[0] * (uint32_t)views[k].camera.viewport[1];
    psnr_total += 10.0 * std::log10(1.0 / (host[2 * k + 1] / (3.0 * pixels)));
    ssim_total += host[2 * k] / (3.0 * pixels);
  }
  free_buffer(sums);
  free_buffer(slot);
  free_buffer(rendered);
  *psnr = psnr_total / view_count;
  *ssim = with_ssim ? ssim_total / view_count : NAN;
  return DG_OK;
}

dg_status dg_trainer_next_view(dg_trainer* t, uint32_t* index) {
  DG_REQUIRE(t && index, "NULL argument");
  if (t->queue.empty()) {
    // Refill exactly as next_view() would; it then takes the same view.
    uint32_t v = next_view(t);
    t->queue.push_back(v);
  }
  *index = t->queue.back();
  return DG_OK;
}

dg_status dg_trainer_loss_value(dg_trainer* t, double* out) {
  DG_REQUIRE(t && out, "NULL argument");
  DG_TRY(loss_sum_launch(t->loss));
  DG_CUDA(cudaMemcpyAsync(out, typed<double>(t->loss->sum_scratch) + t->loss->sum_blocks, 8, cudaMemcpyDeviceToHost,
                          t->ctx->stream));
  DG_CUDA(cudaStreamSynchronize(t->ctx->stream));
  return DG_OK;
}

dg_status dg_trainer_set_host_photos(dg_trainer* t, const void* const* photos, uint32_t count) {
  DG_REQUIRE(t, "NULL argument");
  if (t->upload_stream) DG_CUDA(cudaStreamSynchronize(t->upload_stream));
  t->host_photos.clear();
  t->prefetch_view = -1;
  if (!photos) return DG_OK;
  DG_REQUIRE(count == t->views.size(), "one host photo per training view");
  for (uint32_t k = 0; k < count; k++) DG_REQUIRE(photos[k], "NULL host photo");
  const uint64_t bytes = (uint64_t)t->views[0].camera.viewport[0] * (uint64_t)t->views[0].camera.viewport[1] * 4;
  if (!t->upload_stream) {
    DG_CUDA(cudaStreamCreateWithFlags(&t->upload_stream, cudaStreamNonBlocking));
    for (int k = 0; k < 2; k++) {
      DG_CUDA(cudaEventCreateWithFlags(&t->slot_free[k], cudaEventDisableTiming));
      DG_CUDA(cudaEventCreateWithFlags(&t->slot_ready[k], cudaEventDisableTiming));
      DG_TRY(storage(t, bytes, &t->photo_slots[k]));
    }
  }
  // Nothing has read the slots yet: free as of now.
  for (int k = 0; k < 2; k++) DG_CUDA(cudaEventRecord(t->slot_free[k], t->ctx->stream));
  t->host_photos.assign(photos, photos + count);
  return DG_OK;
}

dg_status dg_trainer_request_loss(dg_trainer* t) {
  DG_REQUIRE(t, "NULL argument");
  DG_REQUIRE(t->loss_head - t->loss_tail < dg_trainer::LOSS_RING,
             "too many loss values requested and not taken (take some first)");
  if (!t->loss_ring) {
    DG_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&t->loss_ring), dg_trainer::LOSS_RING * sizeof(double),
                          cudaHostAllocDefault));
    for (cudaEvent_t& e : t->loss_events) DG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  const uint32_t slot = t->loss_head % dg_trainer::LOSS_RING;
  DG_TRY(loss_sum_launch(t->loss));
  DG_CUDA(cudaMemcpyAsync(&t->loss_ring[slot], typed<double>(t->loss->sum_scratch) + t->loss->sum_blocks, 8,
                          cudaMemcpyDeviceToHost, t->ctx->stream));
  DG_CUDA(cudaEventRecord(t->loss_events[slot], t->ctx->stream));
  t->loss_head++;
  return DG_OK;
}

dg_status dg_trainer_take_loss(dg_trainer* t, int32_t wait, double* out, int32_t* ready) {
  DG_REQUIRE(t && out && ready, "NULL argument");
  DG_REQUIRE(t->loss_tail < t->loss_head, "no loss value requested");
  const uint32_t slot = t->loss_tail % dg_trainer::LOSS_RING;
  if (wait) {
    DG_CUDA(cudaEventSynchronize(t->loss_events[slot]));
  } else {
    const cudaError_t q = cudaEventQuery(t->loss_events[slot]);
    if (q == cudaErrorNotReady) {
      *ready = 0;
      return DG_OK;
    }
    DG_CUDA(q);
  }
  *out = t->loss_ring[slot];
  *ready = 1;
  t->loss_tail++;
  return DG_OK;
}

uint32_t dg_trainer_iteration(const dg_trainer* t) { return t ? t->iteration : 0; }
dg_status dg_trainer_set_iteration(dg_trainer* t, uint32_t iteration) {
  DG_REQUIRE(t, "NULL argument");
  t->iteration = iteration;
  return DG_OK;
}
uint32_t dg_trainer_sh_degree(const dg_trainer* t) { return t ? t->sh_degree : 0; }
uint32_t dg_trainer_adam_steps(const dg_trainer* t) { return t ? t->adam_steps : 0; }
uint32_t dg_trainer_count(const dg_trainer* t) { return t ? t->count : 0; }
dg_renderer* dg_trainer_renderer(dg_trainer* t) { return t ? t->renderer : nullptr; }
dg_buffer* dg_trainer_params(dg_trainer* t) { return t ? t->params : nullptr; }
dg_buffer* dg_trainer_moments(dg_trainer* t) { return t ? t->moments : nullptr; }
dg_buffer* dg_trainer_stats(dg_trainer* t) { return t ? t->stats : nullptr; }
uint32_t dg_trainer_densification_count(const dg_trainer* t) { return t ? (uint32_t)t->densifications.size() : 0; }
dg_status dg_trainer_densification(const dg_trainer* t, uint32_t index, dg_densification* out) {
  DG_REQUIRE(t && out, "NULL argument");
  DG_REQUIRE(index < t->densifications.size(), "no such densification");
  *out = t->densifications[index];
  return DG_OK;
}

dg_status dg_trainer_set_graph(dg_trainer* t, int32_t enabled) {
  DG_REQUIRE(t, "NULL argument");
  t->graph_enabled = enabled != 0;
  if (!t->graph_enabled) drop_graph(t);
  return DG_OK;
}

dg_status dg_trainer_destroy(dg_trainer* t) {
  if (!t) return DG_OK;
  if (t->ctx) cudaStreamSynchronize(t->ctx->stream);
  drop_graph(t);
  dg_renderer_destroy(t->renderer);
  dg_training_loss_destroy(t->loss);
  for (dg_buffer* b : {t->target, t->params, t->moments, t->stats, t->adam_params, t->ids, t->aux}) free_buffer(b);
  if (t->loss_ring) {
    for (cudaEvent_t e : t->loss_events)
      if (e) cudaEventDestroy(e);
    cudaFreeHost(t->loss_ring);
  }
  if (t->upload_stream) {
    cudaStreamSynchronize(t->upload_stream);
    cudaStreamDestroy(t->upload_stream);
    for (int k = 0; k < 2; k++) {
      cudaEventDestroy(t->slot_free[k]);
      cudaEventDestroy(t->slot_ready[k]);
      free_buffer(t->photo_slots[k]);
    }
  }
  delete t;
  return DG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- checkpoints
// No reference counterpart: the reference saves trained Gaussians
// (src/plyWriter.ts) but cannot resume training. A checkpoint is a .ply whose
// vertex element holds writeGaussianPly's 62 properties first, so that the
// reference's reader (src/plyLoader.ts) and other 3DGS viewers open it as a
// scene, followed by the rest of each Gaussian's training state as further float
// properties: the raw parameters' pad floats 7 and 15 (densification stamps),
// Adam's 61 moment pairs, the densification statistics and the learned
// densification's statistics. Further elements hold the identities, the
// trainer's counters, the rest of the current round of views and the
// densification history. Resuming from it continues the run exactly where it
// stopped (up to the float-atomic order of the backward pass).

namespace dg {
namespace {

constexpr const char* CHECKPOINT_COMMENT = "diorama_gb300 training checkpoint 1";
const char* const TRAINER_FIELDS[] = {"iteration", "sh_degree",   "adam_steps", "random_state",
                                      "next_id",   "view_count", "due_densify", "due_reset"};
const char* const DENSIFICATION_FIELDS[] = {"step", "before", "after", "kept", "cloned", "split", "removed"};
const char* const STAT_NAMES[] = {"densify_grad_sum", "densify_grad_count", "densify_max_radius", "densify_stat_3",
                                  "densify_grad_sq_sum", "densify_steps_seen"};

std::vector<PlyElement> checkpoint_elements(uint32_t count, uint32_t queue, uint32_t history) {
  PlyElement vertex{"vertex", count, gaussian_vertex_properties()};
  vertex.properties.push_back(PlyProperty{"pad_7", PlyType::Float});
  vertex.properties.push_back(PlyProperty{"pad_15", PlyType::Float});
  for (uint32_t k = 0; k < MOMENT_SLOTS; k++) {
    vertex.properties.push_back(PlyProperty{"adam_m_" + std::to_string(k), PlyType::Float});
    vertex.properties.push_back(PlyProperty{"adam_v_" + std::to_string(k), PlyType::Float});
  }
  for (const char* n : STAT_NAMES) vertex.properties.push_back(PlyProperty{n, PlyType::Float});
  PlyElement ids{"gaussian_id", count, {PlyProperty{"id", PlyType::Uint}}};
  PlyElement trainer{"trainer", 1, {}};
  for (const char* n : TRAINER_FIELDS) trainer.properties.push_back(PlyProperty{n, PlyType::Uint});
  PlyElement order{"view_queue", queue, {PlyProperty{"view", PlyType::Uint}}};
  PlyElement history_e{"densification", history, {}};
  for (const char* n : DENSIFICATION_FIELDS) history_e.properties.push_back(PlyProperty{n, PlyType::Uint});
  return {vertex, ids, trainer, order, history_e};
}

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) fclose(f);
  }
};

}  // namespace
}  // namespace dg

dg_status dg_trainer_save_checkpoint(dg_trainer* t, const char* path) {
  DG_REQUIRE(t && path, "NULL argument");
  const uint32_t n = t->count;
  std::vector<float> params((size_t)n * FLOATS_PER_GAUSSIAN), sh((size_t)n * SH_REST_FLOATS),
      moments((size_t)n * MOMENT_SLOTS * 2), stats((size_t)n * 4), aux((size_t)n * 2);
  std::vector<uint32_t> ids(n);
  cudaStream_t st = t->ctx->stream;
  DG_CUDA(cudaMemcpyAsync(params.data(), t->params->ptr, params.size() * 4, cudaMemcpyDeviceToHost, st));
  DG_CUDA(cudaMemcpyAsync(sh.data(), t->renderer->sh->ptr, sh.size() * 4, cudaMemcpyDeviceToHost, st));
  DG_CUDA(cudaMemcpyAsync(moments.data(), t->moments->ptr, moments.size() * 4, cudaMemcpyDeviceToHost, st));
  DG_CUDA(cudaMemcpyAsync(stats.data(), t->stats->ptr, stats.size() * 4, cudaMemcpyDeviceToHost, st));
  DG_CUDA(cudaMemcpyAsync(aux.data(), t->aux->ptr, aux.size() * 4, cudaMemcpyDeviceToHost, st));
  DG_CUDA(cudaMemcpyAsync(ids.data(), t->ids->ptr, ids.size() * 4, cudaMemcpyDeviceToHost, st));
  DG_CUDA(cudaStreamSynchronize(st));
  const auto elements = checkpoint_elements(n, (uint32_t)t->queue.size(), (uint32_t)t->densifications.size());
  const std::string header = ply_header_text(elements, {CHECKPOINT_COMMENT});
  File file;
  file.f = fopen(path, "wb");
  if (!file.f) return fail(DG_ERROR_INVALID_ARGUMENT, std::string("cannot open ") + path + " for writing");
  bool ok = fwrite(header.data(), 1, header.size(), file.f) == header.size();
  const size_t stride = elements[0].properties.size();
  std::vector<float> rows;
  const size_t batch = 4096;
  for (size_t first = 0; ok && first < n; first += batch) {
    const size_t here = std::min(batch, (size_t)n - first);
    rows.assign(here * stride, 0.0f);
    for (size_t r = 0; r < here; r++) {
      const size_t i = first + r;
      float* row = rows.data() + r * stride;
      gaussian_row(params.data() + i * FLOATS_PER_GAUSSIAN, sh.data() + i * SH_REST_FLOATS, row);
      size_t at = 62;
      row[at++] = params[i * FLOATS_PER_GAUSSIAN + 7];
      row[at++] = params[i * FLOATS_PER_GAUSSIAN + 15];
      // The moments in the reference's per-Gaussian order: 16 parameter slots, then 45 SH slots.
      std::memcpy(row + at, moments.data() + param_moment_at((uint32_t)i, 0) * 2, FLOATS_PER_GAUSSIAN * 8);
      std::memcpy(row + at + FLOATS_PER_GAUSSIAN * 2, moments.data() + sh_moment_at(n, (uint32_t)i, 0) * 2,
                  SH_REST_FLOATS * 8);
      at += MOMENT_SLOTS * 2;
      std::memcpy(row + at, stats.data() + i * 4, 16);
      std::memcpy(row + at + 4, aux.data() + i * 2, 8);
    }
    ok = fwrite(rows.data(), 4, rows.size(), file.f) == rows.size();
  }
  const uint32_t counters[] = {t->iteration, t->sh_degree, t->adam_steps, t->random_state, t->next_id,
                               (uint32_t)t->views.size(), t->due_densify ? 1u : 0u, t->due_reset ? 1u : 0u};
  ok = ok && fwrite(ids.data(), 4, n, file.f) == n;
  ok = ok && fwrite(counters, 4, 8, file.f) == 8;
  ok = ok && fwrite(t->queue.data(), 4, t->queue.size(), file.f) == t->queue.size();
  for (const auto& d : t->densifications) {
    const uint32_t row[] = {d.step, d.before, d.after, d.kept, d.cloned, d.split, d.removed};
    ok = ok && fwrite(row, 4, 7, file.f) == 7;
  }
  if (!ok) return fail(DG_ERROR_INVALID_ARGUMENT, std::string("writing ") + path + " failed");
  return DG_OK;
}

dg_status dg_trainer_resume(dg_context* ctx, const char* path, const dg_training_view* views, uint32_t view_count,
                            const dg_training_settings* settings, dg_trainer** out) {
  DG_REQUIRE(ctx && path && out, "NULL argument");
  std::vector<uint8_t> bytes;
  {
    File file;
    file.f = fopen(path, "rb");
    if (!file.f) return fail(DG_ERROR_INVALID_ARGUMENT, std::string("cannot open ") + path);
    fseek(file.f, 0, SEEK_END);
    const long size = ftell(file.f);
    fseek(file.f, 0, SEEK_SET);
    if (size < 0) return fail(DG_ERROR_INVALID_ARGUMENT, std::string("cannot read ") + path);
    bytes.resize((size_t)size);
    if (fread(bytes.data(), 1, bytes.size(), file.f) != bytes.size())
      return fail(DG_ERROR_INVALID_ARGUMENT, std::string("cannot read ") + path);
  }
  PlyHeader h;
  DG_TRY(ply_parse_header(bytes.data(), bytes.size(), &h));
  bool tagged = false;
  for (const auto& c : h.comments) tagged = tagged || c == CHECKPOINT_COMMENT;
  DG_REQUIRE(tagged, "not a training checkpoint (a plain .ply has no training state to resume)");
  const char* names[] = {"vertex", "gaussian_id", "trainer", "view_queue", "densification"};
  DG_REQUIRE(h.elements.size() >= 5, "a training checkpoint has 5 elements");
  std::vector<uint64_t> offset(5);
  uint64_t at = h.body;
  for (int e = 0; e < 5; e++) {
    DG_REQUIRE(h.elements[e].name == names[e] && !h.elements[e].opaque, "unexpected element in the checkpoint");
    offset[e] = at;
    at += h.elements[e].count * h.elements[e].row_bytes();
  }
  DG_REQUIRE(at <= bytes.size(), "The .ply file is shorter than its header says.");
  const PlyElement& v = h.elements[0];
  const uint32_t n = (uint32_t)v.count;
  DG_REQUIRE(h.elements[1].count == n && h.elements[2].count == 1, "inconsistent checkpoint element counts");
  // Each element's properties are located by name (all 4-byte floats or uints).
  auto column = [&](const PlyElement& e, const std::string& name, int* out_col) -> dg_status {
    const int k = e.find(name);
    if (k < 0 || e.properties[k].type == PlyType::Uchar)
      return fail(DG_ERROR_INVALID_ARGUMENT, "the checkpoint has no \"" + name + "\" property");
    *out_col = k;
    return DG_OK;
  };
  auto word = [&](int e, uint64_t row, int col) {
    uint32_t w;
    std::memcpy(&w, bytes.data() + offset[e] + row * h.elements[e].row_bytes() + (uint64_t)col * 4, 4);
    return w;
  };
  auto real = [&](int e, uint64_t row, int col) {
    const uint32_t w = word(e, row, col);
    float f;
    std::memcpy(&f, &w, 4);
    return f;
  };
  // Raw parameter k from its vertex property (src/plyWriter.ts:8-12 names them).
  const char* param_names[FLOATS_PER_GAUSSIAN] = {"x",     "y",     "z",     "opacity", "scale_0", "scale_1",
                                                  "scale_2", "pad_7", "rot_0", "rot_1",   "rot_2",   "rot_3",
                                                  "f_dc_0", "f_dc_1", "f_dc_2", "pad_15"};
  int pc[FLOATS_PER_GAUSSIAN], rc[SH_REST_FLOATS], mc[MOMENT_SLOTS * 2], sc[6], idc, uc[8], qc, dc[7];
  for (uint32_t k = 0; k < FLOATS_PER_GAUSSIAN; k++) DG_TRY(column(v, param_names[k], &pc[k]));
  for (uint32_t k = 0; k < SH_REST_FLOATS; k++) DG_TRY(column(v, "f_rest_" + std::to_string(k), &rc[k]));
  for (uint32_t k = 0; k < MOMENT_SLOTS; k++) {
    DG_TRY(column(v, "adam_m_" + std::to_string(k), &mc[2 * k]));
    DG_TRY(column(v, "adam_v_" + std::to_string(k), &mc[2 * k + 1]));
  }
  for (int k = 0; k < 6; k++) DG_TRY(column(v, STAT_NAMES[k], &sc[k]));
  DG_TRY(column(h.elements[1], "id", &idc));
  for (int k = 0; k < 8; k++) DG_TRY(column(h.elements[2], TRAINER_FIELDS[k], &uc[k]));
  DG_TRY(column(h.elements[3], "view", &qc));
  for (int k = 0; k < 7; k++) DG_TRY(column(h.elements[4], DENSIFICATION_FIELDS[k], &dc[k]));
  DG_REQUIRE(word(2, 0, uc[5]) == view_count, "the checkpoint was trained on a different number of views");

  constexpr uint32_t per_channel = SH_REST_FLOATS / 3;
  std::vector<float> params((size_t)n * FLOATS_PER_GAUSSIAN), sh((size_t)n * SH_REST_FLOATS),
      moments((size_t)n * MOMENT_SLOTS * 2), stats((size_t)n * 4), aux((size_t)n * 2);
  std::vector<uint32_t> ids(n);
  for (uint64_t i = 0; i < n; i++) {
    for (uint32_t k = 0; k < FLOATS_PER_GAUSSIAN; k++) params[i * FLOATS_PER_GAUSSIAN + k] = real(0, i, pc[k]);
    for (uint32_t c = 0; c < per_channel; c++)
      for (uint32_t channel = 0; channel < 3; channel++)
        sh[i * SH_REST_FLOATS + c * 3 + channel] = real(0, i, rc[channel * per_channel + c]);
    for (uint32_t k = 0; k < MOMENT_SLOTS; k++) {  // the file's per-Gaussian order into the two planes
      const size_t at = k < FLOATS_PER_GAUSSIAN ? param_moment_at((uint32_t)i, k)
                                                : sh_moment_at(n, (uint32_t)i, k - FLOATS_PER_GAUSSIAN);
      moments[at * 2] = real(0, i, mc[2 * k]);
      moments[at * 2 + 1] = real(0, i, mc[2 * k + 1]);
    }
    for (int k = 0; k < 4; k++) stats[i * 4 + k] = real(0, i, sc[k]);
    for (int k = 0; k < 2; k++) aux[i * 2 + k] = real(0, i, sc[4 + k]);
    ids[i] = word(1, i, idc);
  }
  dg_trainer* t = nullptr;
  DG_TRY(dg_trainer_create(ctx, params.data(), sh.data(), n, views, view_count, settings, &t));
  dg_status st = write_async(ctx, t->moments->ptr, moments.data(), moments.size() * 4);
  if (st == DG_OK) st = write_async(ctx, t->stats->ptr, stats.data(), stats.size() * 4);
  if (st == DG_OK) st = write_async(ctx, t->aux->ptr, aux.data(), aux.size() * 4);
  if (st == DG_OK) st = write_async(ctx, t->ids->ptr, ids.data(), ids.size() * 4);
  t->iteration = word(2, 0, uc[0]);
  const uint32_t degree = word(2, 0, uc[1]);
  t->adam_steps = word(2, 0, uc[2]);
  t->random_state = word(2, 0, uc[3]);
  t->next_id = word(2, 0, uc[4]);
  t->due_densify = word(2, 0, uc[6]) != 0;
  t->due_reset = word(2, 0, uc[7]) != 0;
  for (uint64_t k = 0; k < h.elements[3].count; k++) {
    const uint32_t view = word(3, k, qc);
    if (view >= view_count && st == DG_OK) st = fail(DG_ERROR_INVALID_ARGUMENT, "a queued view is out of range");
    t->queue.push_back(view);
  }
  for (uint64_t k = 0; k < h.elements[4].count; k++) {
    uint32_t f[7];
    for (int j = 0; j < 7; j++) f[j] = word(4, k, dc[j]);
    t->densifications.push_back(dg_densification{f[0], f[1], f[2], f[3], f[4], f[5], f[6]});
  }
  if (st == DG_OK && degree > 3) st = fail(DG_ERROR_INVALID_ARGUMENT, "SH degree above 3 in the checkpoint");
  if (st == DG_OK && degree > 0) st = dg_renderer_set_sh_degree(t->renderer, degree);
  if (st == DG_OK) t->sh_degree = degree;
  if (st == DG_OK) st = cudaStreamSynchronize(ctx->stream) == cudaSuccess ? DG_OK : fail(DG_ERROR_CUDA, "resume upload");
  if (st != DG_OK) {
    dg_trainer_destroy(t);
    return st;
  }
  *out = t;
  return DG_OK;
}

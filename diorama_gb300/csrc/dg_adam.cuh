// Adam's per-slot arithmetic (src/shaders/adam.wgsl:52-106) and the
// densification statistics (src/shaders/adam.wgsl:126-134), used by the backward
// pass that applies Adam as soon as it has a Gaussian's gradients
// (dg_render_bwd.cu) and by the trainer's own kernels (dg_train.cu).
#pragma once
#include "dg_common.cuh"

namespace dg {

// AdamParams (src/shaders/adam.wgsl:9-22)
struct AdamParams {
  float bias_correction1, bias_correction2;
  float position_lr, opacity_lr, scale_lr, rotation_lr, color_lr, sh_lr;
  float viewport[2];
  // Reciprocals of the bias corrections (and of the second's square root), from the host.
  float inv_bias_correction1, inv_sqrt_bias_correction2;
};

__device__ __forceinline__ float sqrt_approx(float x) {
  float r;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// One Adam step (beta 0.9 / 0.999, eps 1e-15) with the host's reciprocals of the
// bias corrections and approximate square root and division: within a few ulps
// of value - lr (m / bc1) / (sqrt(v / bc2) + eps).
__device__ __forceinline__ float adam_step_fast(float value, float grad, float2& m, float lr, float inv_bc1,
                                                float inv_sqrt_bc2) {
  m.x = 0.9f * m.x + 0.1f * grad;
  m.y = 0.999f * m.y + 0.001f * grad * grad;
  return value - __fdividef(lr * (m.x * inv_bc1), sqrt_approx(m.y) * inv_sqrt_bc2 + 1e-15f);
}

// Raw slot k (0-15, not 7 or 15) of a Gaussian: its gradient g0 with respect to
// the activated value goes through the activation's chain rule, Adam steps the
// raw value x, and the new activated value is returned in `activated`
// (src/shaders/adam.wgsl:60-106). Without branches: the slots of a Gaussian
// share a warp, and each would otherwise take its own path; one expf serves the
// sigmoid (k = 3) and the exponential (k = 4-6), with the values of the per-slot
// formulas bit for bit.
__device__ __forceinline__ float adam_param_slot(const AdamParams& ap, uint32_t k, float x, float g0, float2& m,
                                                 float& activated) {
  const bool opacity = k == 3, scale = k >= 4 && k <= 6, color = k >= 12;
  const float ex = expf(opacity ? -x : x);
  const float sig = 1.0f / (1.0f + ex);
  const float grad = opacity ? g0 * sig * (1.0f - sig) : scale ? g0 * ex : color ? g0 * SH_C0 : g0;
  const float lr = k < 3 ? ap.position_lr
                 : opacity ? ap.opacity_lr
                 : scale ? ap.scale_lr
                 : color ? ap.color_lr
                         : ap.rotation_lr;
  const float next = adam_step_fast(x, grad, m, lr, ap.inv_bias_correction1, ap.inv_sqrt_bias_correction2);
  const float ey = expf(opacity ? -next : next);
  activated = opacity ? 1.0f / (1.0f + ey) : scale ? ey : color ? 0.5f + SH_C0 * next : next;
  return next;
}

// src/shaders/adam.wgsl:126-134 for Gaussian i: if it was drawn (radius > 0), the
// length of its screen-space mean gradient in pixels, a count and the largest
// radius go into stats; aux (the learned densification's extra statistics) gets
// the squared length and the count of steps seen over the Gaussian's life.
// The same from the values: the splat's radius and its mean's two gradients.
__device__ __forceinline__ void accumulate_stats_values(const float* __restrict__ viewport, float radius,
                                                        float mean_grad_x, float mean_grad_y,
                                                        float4* __restrict__ stats, float2* __restrict__ aux,
                                                        uint32_t i) {
  if (radius == 0.0f) return;
  const float gx = mean_grad_x * viewport[0] * 0.5f;
  const float gy = mean_grad_y * viewport[1] * 0.5f;
  const float len = sqrtf(gx * gx + gy * gy);
  const float4 s = stats[i];
  stats[i] = make_float4(s.x + len, s.y + 1.0f, fmaxf(s.z, radius), 0.0f);
  const float2 a = aux[i];
  aux[i] = make_float2(a.x + len * len, a.y + 1.0f);
}

__device__ __forceinline__ void accumulate_stats_one(const float* __restrict__ viewport,
                                                     const float* __restrict__ splats,
                                                     const float* __restrict__ splat_grads, float4* __restrict__ stats,
                                                     float2* __restrict__ aux, uint32_t i) {
  accumulate_stats_values(viewport, splats[(size_t)i * FLOATS_PER_SPLAT + 3], splat_grads[(size_t)i * SPLAT_GRADS],
                          splat_grads[(size_t)i * SPLAT_GRADS + 1], stats, aux, i);
}

}  // namespace dg

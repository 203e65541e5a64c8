// Internal entry point of the learned densification's model (dg_mlp.cu).
#pragma once
#include "dg_common.cuh"

namespace dg {
// survive[i] = P(candidate i's children survive) for features [n][12], on the context's stream.
dg_status mlp_predict_launch(dg_densify_mlp* m, const float* features, uint32_t n, float* survive);
}  // namespace dg

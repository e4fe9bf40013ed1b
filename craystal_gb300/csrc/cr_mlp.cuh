// cr_mlp.cuh -- device-side interface of the radiance-cache network
// (cr_mlp.cu), used by the cached integrator (cr_cache.cu).
#pragma once

#include "cr_internal.cuh"

namespace cr {

struct MlpState;

constexpr int kMlpInputs = 7;  // position (3, in [0,1]), direction (3, in [0,1]), roughness

int mlpCreate(const cr_mlp_config* cfg, MlpState** out);
void mlpDestroy(MlpState* s);
// outputs n x 3 (RGB), clamped at 0 when clampNonNeg
int mlpInferDevice(MlpState* s, const float* in, uint64_t n, float* out, bool clampNonNeg, cudaStream_t st);
// adds dW of the mean relative L2 loss of n samples; loss sum in mlpLossPtr
int mlpGradDevice(MlpState* s, const float* in, const float* target, uint64_t n, cudaStream_t st);
// one Adam step on the accumulated gradient plus dW of n samples; clears it
int mlpTrainStepDevice(MlpState* s, const float* in, const float* target, uint64_t n, cudaStream_t st);
float* mlpLossPtr(MlpState* s);
// reports a tensor-core wait of the inference that ran out (synchronises)
int mlpCheck(MlpState* s);

}  // namespace cr

struct cr_mlp {
    cr::MlpState* s;
};

// Activations of the warm-start network: ReLU and the exact GELU,
// gelu(x) = x Phi(x) = x/2 (1 + erf(x / sqrt 2)), with its derivative
// gelu'(x) = Phi(x) + x phi(x), phi(x) = exp(-x^2/2) / sqrt(2 pi).
#pragma once
#include <cuda_bf16.h>

#define LBM_NN_ACT_RELU 0
#define LBM_NN_ACT_GELU 1

__device__ __forceinline__ float nn_gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }

__device__ __forceinline__ float nn_gelu_grad(float x) {
    return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

// Derivative of the activation at a stored value: ReLU takes the activation
// output (or the pre-activation; both are > 0 at the same places), GELU the
// pre-activation.
__device__ __forceinline__ float nn_act_grad(int act, float stored) {
    return act == LBM_NN_ACT_GELU ? nn_gelu_grad(stored) : (stored > 0.f ? 1.f : 0.f);
}

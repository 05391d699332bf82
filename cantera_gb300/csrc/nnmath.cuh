// nnmath.cuh - activation functions of the surrogate network, shared by its GEMM kernels.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace gbchem {

// GELU, tanh form: 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3)))
__device__ __forceinline__ float gelu(float x) {
    const float u = 0.7978845608028654f * fmaf(0.044715f * x, x * x, x);
    return 0.5f * x * (1.0f + tanhf(u));
}
__device__ __forceinline__ float geluGrad(float x) {
    const float u = 0.7978845608028654f * fmaf(0.044715f * x, x * x, x);
    const float t = tanhf(u);
    return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * 0.7978845608028654f * fmaf(0.134145f, x * x, 1.0f);
}

}  // namespace gbchem

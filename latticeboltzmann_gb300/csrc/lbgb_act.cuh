// The surrogate's activation (GELU, tanh form) and its derivative, shared by
// the element-wise kernels and the fused GEMM epilogue, so that both give
// the same values.
#pragma once

namespace lbgb {

constexpr float SQ2PI = 0.7978845608028654f;

// tanh by the hardware approximation (one MUFU instruction, relative error
// ~2^-11): the activations it feeds are rounded to BF16 (2^-8) anyway
__device__ __forceinline__ float tanh_hw(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float gelu_f(float x) {
    return 0.5f * x * (1.f + tanh_hw(SQ2PI * (x + 0.044715f * x * x * x)));
}
__device__ __forceinline__ float gelu_df(float x) {
    const float t = tanh_hw(SQ2PI * (x + 0.044715f * x * x * x));
    return 0.5f * (1.f + t) + 0.5f * x * (1.f - t * t) * SQ2PI * (1.f + 3.f * 0.044715f * x * x);
}

}  // namespace lbgb

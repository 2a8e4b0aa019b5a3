// The warm-start network's activation: GELU in its tanh form,
//   gelu(z) = z/2 (1 + tanh(c (z + a z^3))),  c = sqrt(2/pi), a = 0.044715,
// with tanh from the SFU (tanh.approx.f32, relative error about 2^-11, below
// the BF16 rounding of the stored activations).  Training and both inference
// kernels use these two functions, so the network is evaluated as trained.
#pragma once

namespace sp {
namespace act {

constexpr float kC = 0.7978845608028654f;  // sqrt(2/pi)
constexpr float kA = 0.044715f;

__device__ __forceinline__ float tanh_sfu(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// c (z + a z^3) = z (c + c a z^2); z/2 (1 + t) = fma(z/2, t, z/2): five FP32
// operations and one SFU tanh
__device__ __forceinline__ float gelu(float z) {
    const float t = tanh_sfu(z * fmaf(kC * kA, z * z, kC));
    const float h = 0.5f * z;
    return fmaf(h, t, h);
}

__device__ __forceinline__ float gelu_grad(float z) {
    const float t = tanh_sfu(kC * fmaf(kA * z, z * z, z));
    return 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * kC * fmaf(3.0f * kA, z * z, 1.0f);
}

}  // namespace act
}  // namespace sp

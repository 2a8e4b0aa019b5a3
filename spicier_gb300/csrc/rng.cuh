// Stateless hash RNG of the Monte Carlo sweeps, on device and host.
//
// Integer part identical to crates/spicier-batched-sweep/src/rng.rs:39-95
// (SplitMix64 finaliser, index mixing, top-53-bit scaling), so uniform draws
// are bit-exact on every platform.  The Gaussian (rng.rs:120-131) needs ln
// and cos; those come from cr_math.cuh, which returns the correctly rounded
// result, so a draw equals the reference's whenever the host libm rounds
// correctly too.
#pragma once
#include <stdint.h>

#include "cr_math.cuh"

#ifndef SP_HD
#define SP_HD __host__ __device__ __forceinline__
#endif

namespace sp {

SP_HD uint64_t splitmix64(uint64_t x) {
    x += 0x9e3779b97f4a7c15ULL;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
    return x ^ (x >> 31);
}

SP_HD uint64_t combine_indices(uint64_t seed, uint32_t sweep, uint32_t param) {
    return seed ^ ((uint64_t)sweep * 0x517cc1b727220a95ULL) ^
           ((uint64_t)param * 0x5851f42d4c957f2dULL);
}

// (h >> 11) * 2^-53: exact (53-bit integer times a power of two), built from
// the integer directly (no FP64 instruction).
SP_HD double rng_uniform(uint64_t seed, uint32_t sweep, uint32_t param) {
    uint64_t h = splitmix64(combine_indices(seed, sweep, param));
    return cr::u53_to_double(h >> 11);
}

SP_HD float rng_uniform_f32(uint64_t seed, uint32_t sweep, uint32_t param) {
    uint64_t h = splitmix64(combine_indices(seed, sweep, param));
    return (float)(h >> 40) * 5.9604644775390625e-08f;
}

// Box-Muller on parameter slots 2p and 2p+1 with u1 clamped to 1e-10.
// 2*pi is the double 6.283185307179586 (2.0 * std::f64::consts::PI, exact),
// and the product with u2 is rounded once, as in the reference.
SP_HD double rng_gaussian(uint64_t seed, uint32_t sweep, uint32_t param, unsigned* hard) {
    double u1 = rng_uniform(seed, sweep, param * 2u);
    double u2 = rng_uniform(seed, sweep, param * 2u + 1u);
    // max(u1, 1e-10) on the bit patterns (both non-negative)
    u1 = cr::dbits(u1) > 0x3DDB7CDFD9D7BDBBULL ? u1 : 1e-10;
    const double l = cr_log(u1, hard);  // < 0, normal
    // -2 l exactly: flip the sign and raise the exponent by one
    const double m2l = cr::bdouble((cr::dbits(l) ^ (1ULL << 63)) + (1ULL << 52));
#if defined(__CUDA_ARCH__)
    // the two products and the square root on the FP64 pipe (IEEE round to
    // nearest, never contracted), which the integer-bound ln and cos leave idle
    const double c = cr_cos(__dmul_rn(6.283185307179586, u2), hard);
    return __dmul_rn(__dsqrt_rn(m2l), c);
#else
    const double c = cr_cos(6.283185307179586 * u2, hard);
    return sqrt(m2l) * c;
#endif
}

// FP32 variant (rng.rs:138-145): the reference's f32 ln/cos are not pinned
// (host libm), so this uses the device's single-precision functions.
SP_HD float rng_gaussian_f32(uint64_t seed, uint32_t sweep, uint32_t param) {
    float u1 = rng_uniform_f32(seed, sweep, param * 2u);
    float u2 = rng_uniform_f32(seed, sweep, param * 2u + 1u);
    u1 = u1 > 1e-7f ? u1 : 1e-7f;
    return sqrtf(-2.0f * logf(u1)) * cosf(2.0f * 3.14159265f * u2);
}

}  // namespace sp

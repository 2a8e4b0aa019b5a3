// FP64 <-> FP32 conversions on the integer pipe, round to nearest even, for
// every input (zeros, subnormals, overflow, Inf, NaN): GB300's FP64 pipe
// issues the hardware conversions at the FP64 rate.  Branch-free, so the
// compiler does not if-convert a hardware fallback into every call.
#pragma once
#include <stdint.h>

namespace sp {

__device__ __forceinline__ float f64_to_f32_int(double x) {
    const uint64_t b = (uint64_t)__double_as_longlong(x);
    const unsigned int sign = (unsigned int)(b >> 32) & 0x80000000u;
    const int ex = (int)((b >> 52) & 0x7ff);
    const uint64_t m = (b & ((1ULL << 52) - 1)) | (ex ? (1ULL << 52) : 0ULL);
    const int e = ex - 1023 + 127;
    int sh = e >= 1 ? 29 : 30 - e;
    sh = sh > 63 ? 63 : sh;
    const uint64_t q = m >> sh, rem = m & ((1ULL << sh) - 1), half = 1ULL << (sh - 1);
    unsigned int f = (unsigned int)q + (unsigned int)(rem > half || (rem == half && (q & 1)));
    f = e >= 1 ? f + ((unsigned int)(e - 1) << 23) : f;
    f = (e >= 255 || f >= 0x7f800000u) ? 0x7f800000u : f;
    f = ex == 0x7ff ? (0x7f800000u | (unsigned int)(m >> 29) | ((b & ((1ULL << 52) - 1)) ? 0x400000u : 0u)) : f;
    return __uint_as_float(sign | f);
}

__device__ __forceinline__ double f32_to_f64_int(float x) {
    const unsigned int f = __float_as_uint(x);
    const uint64_t sign = (uint64_t)(f & 0x80000000u) << 32;
    const unsigned int e = (f >> 23) & 0xff, m = f & 0x7fffffu;
    const int lz = __clz(m) - 8;
    const uint64_t sub = m ? ((uint64_t)(1023 - 126 - lz) << 52) | ((uint64_t)((m << lz) & 0x7fffffu) << 29) : 0ULL;
    const uint64_t nrm = ((uint64_t)(e - 127 + 1023) << 52) | ((uint64_t)m << 29);
    const uint64_t inf = (0x7ffULL << 52) | ((uint64_t)m << 29) | (m ? (1ULL << 51) : 0ULL);  // NaN quietened
    return __longlong_as_double((long long)(sign | (e == 0 ? sub : (e == 255 ? inf : nrm))));
}

}  // namespace sp

// Correctly rounded ln, exp and cos for the hash-RNG draws (Box-Muller,
// log-uniform), evaluated in 128-bit integer fixed point.
//
// The reference draws z = sqrt(-2 ln u1) cos(2 pi u2) with the host libm
// (crates/spicier-batched-sweep/src/rng.rs:120-131), whose ln and cos are not
// correctly rounded; two libms (or glibc and CUDA) disagree in the last bit of
// a few percent of draws.  These functions return the correctly rounded
// result instead, so device and host give the same bits, and they agree with
// any libm wherever that libm rounds correctly.
//
// Why integers: GB300 issues FP64 at about 1/60 of its FP32/INT32 rate, so a
// double-double evaluation would be several times slower than this one, which
// runs on the integer pipe (64-bit limbs, 64x64->128 products).
//
// Formats: ln works in Q8.120 (value = integer * 2^-120), cos in Q3.125.
// Every evaluation carries an absolute error bound err (in units of the last
// bit).  The conversion to double rounds to nearest-even and adds one to
// *hard whenever the exact value, known only to +-err units, could lie on the
// other side of a rounding midpoint.  A result is correctly rounded whenever
// *hard is left unchanged.  The domains cover the Box-Muller arguments with
// room to spare: ln takes x in [2^-360, 2^360), cos takes |t| < 8; any other
// input (zero, negative, NaN, Inf, out of range) returns NaN and counts as
// hard.
//
// ln x  = e ln 2 + (-ln c_i) + ln(1 + r),  x = m 2^e, m in [1, 2),
//         c_i ~ 1/m from the top 8 mantissa bits, r = m c_i - 1 in [0, 2^-8)
//         exact; ln(1+r) by its Taylor series (15 terms, Horner, the inner
//         8 levels in Q0.64).  Within 2^-16 of 1 the series runs in
//         d = |x - 1| instead, relative to d (ln_near1).
// cos t = +-cos a or +-sin a,  a = |t - k pi/2| <= pi/4,  a = j/512 + d,
//         cos/sin(j/512) from the table, cos/sin(d) by Taylor series in d^2
//         (five terms each, the innermost in 64 bits), products without their
//         low partial product (error bound 512 units of 2^-125).
#pragma once
#include <math.h>
#include <cmath>
#include <stdint.h>
#include <string.h>

#include "cr_tables.h"

#ifndef SP_HD
#if defined(__CUDACC__)
#define SP_HD __host__ __device__ __forceinline__
#else
#define SP_HD inline
#endif
#endif

namespace sp {
namespace cr {

typedef unsigned __int128 u128;

struct LnRow {
    uint64_t c, th, tl, pad;
};
struct CosRow {
    uint64_t ch, cl, sh, sl;
};
struct W2 {
    uint64_t hi, lo;
};

struct ExpRow {
    uint64_t hi, lo;
};

#if defined(__CUDACC__)
__device__ const LnRow kLnRowsDev[256] = SP_CR_LN_ROWS;
__device__ const CosRow kCosRowsDev[404] = SP_CR_COS_ROWS;
__device__ const ExpRow kExpRowsDev[181] = SP_CR_EXP_ROWS;
#endif
static const LnRow kLnRowsHost[256] = SP_CR_LN_ROWS;
static const CosRow kCosRowsHost[404] = SP_CR_COS_ROWS;
static const ExpRow kExpRowsHost[181] = SP_CR_EXP_ROWS;

SP_HD ExpRow exp_row(int i) {
#if defined(__CUDA_ARCH__)
    const ulonglong2 a = __ldg(reinterpret_cast<const ulonglong2*>(&kExpRowsDev[i]));
    return ExpRow{a.x, a.y};
#else
    return kExpRowsHost[i];
#endif
}

SP_HD LnRow ln_row(int i) {
#if defined(__CUDA_ARCH__)
    const ulonglong2* p = reinterpret_cast<const ulonglong2*>(&kLnRowsDev[i]);
    const ulonglong2 a = __ldg(p), b = __ldg(p + 1);
    return LnRow{a.x, a.y, b.x, b.y};
#else
    return kLnRowsHost[i];
#endif
}

SP_HD CosRow cos_row(int j) {
#if defined(__CUDA_ARCH__)
    const ulonglong2* p = reinterpret_cast<const ulonglong2*>(&kCosRowsDev[j]);
    const ulonglong2 a = __ldg(p), b = __ldg(p + 1);
    return CosRow{a.x, a.y, b.x, b.y};
#else
    return kCosRowsHost[j];
#endif
}

SP_HD u128 mk(uint64_t hi, uint64_t lo) { return ((u128)hi << 64) | lo; }
SP_HD u128 mk(W2 w) { return mk(w.hi, w.lo); }
SP_HD uint64_t hi64(u128 v) { return (uint64_t)(v >> 64); }
SP_HD uint64_t lo64(u128 v) { return (uint64_t)v; }

SP_HD int clz64(uint64_t v) {
#if defined(__CUDA_ARCH__)
    return __clzll((long long)v);
#else
    return v ? __builtin_clzll(v) : 64;
#endif
}

SP_HD int bitlen(u128 v) {
    const uint64_t h = hi64(v);
    return h ? 128 - clz64(h) : 64 - clz64(lo64(v));
}

SP_HD uint64_t dbits(double x) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    memcpy(&b, &x, 8);
    return b;
#endif
}

SP_HD double bdouble(uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double x;
    memcpy(&x, &b, 8);
    return x;
#endif
}

// -x as a sign-bit flip on the integer pipe (the IEEE negation, NaN included)
SP_HD double dneg(double x) { return bdouble(dbits(x) ^ (1ULL << 63)); }
SP_HD double dneg_if(bool c, double x) { return bdouble(dbits(x) ^ ((uint64_t)c << 63)); }

// (a * b) >> F for unsigned fixed-point a, b (F in 65..127); the 256-bit
// product is formed exactly and truncated, so the error is below one unit.
template <int F>
SP_HD u128 mulq(u128 a, u128 b) {
    const uint64_t a0 = lo64(a), a1 = hi64(a), b0 = lo64(b), b1 = hi64(b);
    const u128 p00 = (u128)a0 * b0, p01 = (u128)a0 * b1, p10 = (u128)a1 * b0, p11 = (u128)a1 * b1;
    const u128 mid = (u128)hi64(p00) + lo64(p01) + lo64(p10);
    const u128 top = p11 + hi64(p01) + hi64(p10) + hi64(mid);
    constexpr int s = F - 64;
    return (top << (64 - s)) | (lo64(mid) >> s);
}

// (a * b) >> F without the low partial product a_lo b_lo: three 64x64
// products instead of four, at most 2^(128-F) + 1 units below the exact value.
template <int F>
SP_HD u128 mulq3(u128 a, u128 b) {
    const uint64_t a0 = lo64(a), a1 = hi64(a), b0 = lo64(b), b1 = hi64(b);
    const u128 p01 = (u128)a0 * b1, p10 = (u128)a1 * b0, p11 = (u128)a1 * b1;
    const u128 mid = (u128)lo64(p01) + lo64(p10);
    const u128 top = p11 + hi64(p01) + hi64(p10) + hi64(mid);
    constexpr int s = F - 64;
    return (top << (64 - s)) | (lo64(mid) >> s);
}

// (r0 * h) >> 68: r = r0 2^-68 times a Q8.120 value, below one unit of error.
SP_HD u128 mul_r68(uint64_t r0, u128 h) {
    const u128 p0 = (u128)r0 * lo64(h), p1 = (u128)r0 * hi64(h);
    return (p1 + hi64(p0)) >> 4;
}

// v 2^-F rounded to nearest-even as a positive double (v needs at least 54
// significant bits, which every caller guarantees), with gradual underflow
// (subnormal results round at 2^-1074) and overflow to +Inf; counts an
// undecided rounding in *hard.
SP_HD double round_fixed(u128 v, int F, uint64_t err, unsigned* hard) {
    const int n = bitlen(v);
    const int ex = n - 1 - F;                     // exponent of the leading bit
    if (ex > 1023) return bdouble(0x7FF0000000000000ULL);
    const bool sub = ex < -1022;
    const int w = sub ? F - 1074 : n - 53;         // discarded low bits (1..127)
    if (w >= 128) return 0.0;                      // below half the smallest subnormal
    const uint64_t m = (uint64_t)(v >> w);
    const u128 rem = v & (((u128)1 << w) - 1);
    const u128 half = (u128)1 << (w - 1);
    const u128 dist = rem > half ? rem - half : half - rem;
    if (hard && dist <= err) ++*hard;
    const uint64_t up = (rem > half || (rem == half && (m & 1))) ? 1 : 0;
    if (sub) return bdouble(m + up);               // a carry into bit 52 gives the smallest normal
    return bdouble(((uint64_t)(ex + 1023) << 52) + (m - (1ULL << 52)) + up);  // a carry may give +Inf
}

// round_fixed for the 64-bit fast paths, whose v has at least 54 significant
// bits and whose result is a normal double: v normalised by one shift (its
// leading bit at 127), so that the 53 kept bits, the midpoint and the rest
// sit at fixed positions, and err scaled by the same shift.  The same result
// and the same count in *undecided as round_fixed, with one variable-width
// shift of v where round_fixed needs three.
SP_HD double round_fixed_fast(u128 v, int F, uint64_t err, unsigned* undecided) {
    const uint64_t h0 = hi64(v);
    const int lz = h0 ? clz64(h0) : 64 + clz64(lo64(v));
    const u128 u = v << lz;                      // leading bit at 127
    const uint64_t m = hi64(u) >> 11;            // the 53 kept bits
    const u128 rem = u & (((u128)1 << 75) - 1);  // the rest; the midpoint is 2^74
    const u128 half = (u128)1 << 74;
    const u128 dist = rem >= half ? rem - half : half - rem;
    if (dist <= ((u128)err << lz)) ++*undecided;
    const uint64_t up = (rem > half || (rem == half && (m & 1))) ? 1 : 0;
    return bdouble(((uint64_t)(127 - lz - F + 1023) << 52) + (m - (1ULL << 52)) + up);  // a carry may raise the exponent
}

// ln x for x within 2^-16 of 1, relative to d = |x - 1| = D 2^-e exactly
// (e = 53 below 1, 52 above): ln(1 +- d) = +-d B with B = 1 -+ d/2 + d^2/3
// -+ ... (8 terms), so the result keeps about 2^-118 relative accuracy however
// close x is to 1, where the general path's absolute accuracy would not decide
// the rounding of ln(1 - k 2^-53).  Integer operations only.
SP_HD double ln_near1(uint64_t xb, unsigned* hard) {
    const bool below = xb < 0x3FF0000000000000ULL;
    const uint64_t frac = xb & ((1ULL << 52) - 1);
    const uint64_t D = below ? (1ULL << 52) - frac : frac;  // < 2^37
    const int e = below ? 53 : 52;
    const u128 d = (u128)D << (120 - e);                    // Q8.120, exact
    const W2 inv128[6] = SP_CR_LN_INV128;                    // 1/2 .. 1/7
    u128 g = (u128)1 << 117;                                 // 1/8
    const u128 one = (u128)1 << 120;
    if (below) {
#pragma unroll
        for (int j = 5; j >= 0; --j) g = mk(inv128[j]) + mulq<120>(d, g);
        g = one + mulq<120>(d, g);
    } else {
#pragma unroll
        for (int j = 5; j >= 0; --j) g = mk(inv128[j]) - mulq<120>(d, g);
        g = one - mulq<120>(d, g);
    }
    // |ln x| = Dn B 2^-(e+z+120) with Dn = D 2^z normalised to 53 bits: the
    // product Dn B (< 2^174) shifted right by 48 keeps 124+ significant bits
    const int z = clz64(D) - 11;
    const uint64_t Dn = D << z;
    const u128 p0 = (u128)Dn * lo64(g), p1 = (u128)Dn * hi64(g);
    const u128 v = (p1 << 16) + (p0 >> 48);
    const double r = round_fixed(v, e + z + 72, 80, hard);
    return dneg_if(below, r);
}

// IEEE-exact (round to nearest even) multiply, divide and square root of
// finite positive-normal doubles whose results are normal, by integer
// operations: GB300's FP64 pipe issues at a small fraction of the integer
// rate, and the results are the IEEE ones bit for bit (a correctly rounded
// result is unique).  Callers check the domain.

// a b for normal a, b (either sign) with a normal product.
SP_HD double mul_rn(double a, double b) {
    const uint64_t ba = dbits(a), bb = dbits(b);
    const uint64_t ma = (ba & ((1ULL << 52) - 1)) | (1ULL << 52), mb = (bb & ((1ULL << 52) - 1)) | (1ULL << 52);
    const int ea = (int)((ba >> 52) & 0x7ff), eb = (int)((bb >> 52) & 0x7ff);
    const u128 p = (u128)ma * mb;  // [2^104, 2^106)
    const int top = (int)(p >> 105);  // 1 when the product has 106 bits
    const int sh = 52 + top;
    uint64_t q = (uint64_t)(p >> sh);
    const uint64_t rem = (uint64_t)p & ((1ULL << sh) - 1), half = 1ULL << (sh - 1);
    q += (rem > half || (rem == half && (q & 1))) ? 1 : 0;  // q = 2^53 carries into the exponent below
    const uint64_t e = (uint64_t)(ea + eb - 1023 + top);
    return bdouble(((ba ^ bb) & (1ULL << 63)) | ((e << 52) + (q - (1ULL << 52))));
}

// a / b for positive normal a, b with a normal quotient.
SP_HD double div_pos(double a, double b) {
    const uint64_t ba = dbits(a), bb = dbits(b);
    const uint64_t ma = (ba & ((1ULL << 52) - 1)) | (1ULL << 52), mb = (bb & ((1ULL << 52) - 1)) | (1ULL << 52);
    int e = (int)(ba >> 52) - (int)(bb >> 52) + 1023;
    // quotient mantissa q = floor(ma 2^s / mb) has 53 bits with s = 52 or 53
    const int s = ma >= mb ? 52 : 53;
    e -= s - 52;
    // reciprocal 2^63 / (mb 2^-52) ~ R in (2^62, 2^63]: FP32 estimate, one
    // 32-bit Newton step, one 64-bit step
#if defined(__CUDA_ARCH__)
    const float rf = __frcp_rn((float)(uint32_t)(mb >> 29));  // mb 2^-29 in [2^23, 2^24)
#else
    const float rf = 1.0f / (float)(uint32_t)(mb >> 29);
#endif
    uint32_t r32 = (uint32_t)(rf * 0x1p54f);  // 2^31 / (mb 2^-52), in (2^30, 2^31]
    {
        const uint32_t m32 = (uint32_t)(mb >> 21);                        // mb 2^-21 in [2^31, 2^32)
        const uint64_t e32 = (uint64_t)m32 * r32;                         // ~2^62
        const uint32_t c32 = (uint32_t)(((1ULL << 63) - e32) >> 31) ;     // (2 - e) 2^31 ~ 2^32
        r32 = (uint32_t)(((uint64_t)r32 * c32) >> 32) << 1;               // refined, ~2^31
    }
    uint64_t R = (uint64_t)r32 << 32;  // ~2^63 / (mb 2^-52)
    {
        const u128 mr = (u128)mb * R;                                     // ~2^115
        const uint64_t corr = (uint64_t)((((u128)1 << 116) - mr) >> 52);  // (2 - mb R 2^-115) 2^63
        R = (uint64_t)(((u128)R * corr) >> 63);
    }
    const uint64_t a54 = ma << (s - 52);  // num = a54 2^52
    uint64_t q = (uint64_t)(((u128)a54 * R) >> 63);  // ~ num / mb, within a few units
    // exact remainder of num = q mb + rem, then at most two corrections each way
    const u128 num = (u128)a54 << 52;
    __int128 rem = (__int128)(num - (u128)q * mb);
    for (int it = 0; it < 2 && rem < 0; ++it) {
        --q;
        rem += mb;
    }
    for (int it = 0; it < 2 && rem >= (__int128)mb; ++it) {
        ++q;
        rem -= mb;
    }
    const uint64_t r = (uint64_t)rem;
    q += (2 * r > mb || (2 * r == mb && (q & 1))) ? 1 : 0;
    return bdouble(((uint64_t)e << 52) + (q - (1ULL << 52)));
}

// sqrt(x) for positive normal x.
SP_HD double sqrt_pos(double x) {
    const uint64_t b = dbits(x);
    int E = (int)(b >> 52) - 1023;
    uint64_t M = (b & ((1ULL << 52) - 1)) | (1ULL << 52);
    if (E & 1) {
        M <<= 1;
        E -= 1;
    }
    // r = floor(sqrt(M 2^52)), M 2^52 in [2^104, 2^106): r in [2^52, 2^53)
    const uint64_t U = M << 10;  // u = M 2^-52 in [1, 4), as u 2^62
    const float uf = (float)(uint32_t)(M >> 30) * 0x1p-22f;
#if defined(__CUDA_ARCH__)
    const float gf = rsqrtf(uf);
#else
    const float gf = 1.0f / std::sqrt(uf);
#endif
    // g = 1/sqrt(u): one 32-bit Newton step (g 2^31), one 64-bit step (g 2^63)
    uint32_t g32 = (uint32_t)(gf * 0x1p31f);
    {
        const uint32_t u32 = (uint32_t)(U >> 32);                        // u 2^30
        const uint32_t a = (uint32_t)(((uint64_t)g32 * g32) >> 32);      // g^2 2^30
        const uint32_t bb = (uint32_t)(((uint64_t)u32 * a) >> 32);       // u g^2 2^28
        const uint32_t t = (3u << 28) - bb;                              // (3 - u g^2) 2^28
        g32 = (uint32_t)(((uint64_t)g32 * t) >> 29);                     // g (3 - u g^2)/2 2^31
    }
    uint64_t G = (uint64_t)g32 << 32;
    {
        const uint64_t A = (uint64_t)(((u128)G * G) >> 64);  // g^2 2^62
        const uint64_t B = (uint64_t)(((u128)U * A) >> 64);  // u g^2 2^60
        const uint64_t T = (3ULL << 60) - B;                  // (3 - u g^2) 2^60
        G = (uint64_t)(((u128)G * T) >> 64) << 3;             // 2^63
    }
    uint64_t r = (uint64_t)(((u128)U * G) >> 64) >> 9;  // sqrt(u) 2^52, within a few units
    const u128 N = (u128)M << 52;
    __int128 rem = (__int128)(N - (u128)r * r);  // N - r^2
    for (int it = 0; it < 2 && rem < 0; ++it) {
        --r;
        rem += 2 * (__int128)r + 1;
    }
    for (int it = 0; it < 2 && rem > 2 * (__int128)r; ++it) {
        rem -= 2 * (__int128)r + 1;
        ++r;
    }
    r += rem > (__int128)r ? 1 : 0;  // round to nearest (no ties: N is an integer)
    return bdouble(((uint64_t)(E / 2 + 1023) << 52) + (r - (1ULL << 52)));
}

}  // namespace cr

// IEEE multiply / divide / square root that run on the integer pipe on the
// device for operands and results in the normal range, and in hardware
// otherwise (a call the compiler does not speculate); plain operators on the
// host.  Bit-identical to the operators everywhere.
#if defined(__CUDA_ARCH__)
__device__ __noinline__ static double hw_mul(double a, double b) { return a * b; }
__device__ __noinline__ static double hw_div(double a, double b) { return a / b; }
__device__ __noinline__ static double hw_sqrt(double a) { return sqrt(a); }
#endif

SP_HD double ieee_mul(double a, double b) {
#if defined(__CUDA_ARCH__)
    if (cr::dbits(b) == 0x3FF0000000000000ULL) return a;  // a * 1 = a for every non-signalling a
    const int ea = (int)((cr::dbits(a) >> 52) & 0x7ff), eb = (int)((cr::dbits(b) >> 52) & 0x7ff);
    const int e = ea + eb - 1023;
    if (ea != 0 && eb != 0 && ea != 0x7ff && eb != 0x7ff && e >= 2 && e <= 2045) return cr::mul_rn(a, b);
    return hw_mul(a, b);
#else
    return a * b;
#endif
}

SP_HD double ieee_div(double a, double b) {
#if defined(__CUDA_ARCH__)
    const uint64_t ba = cr::dbits(a), bb = cr::dbits(b);
    const int ea = (int)(ba >> 52), eb = (int)(bb >> 52);  // sign bit included: negative operands fail below
    const int e = ea - eb + 1023;
    if (ea > 0 && ea < 0x7ff && eb > 0 && eb < 0x7ff && e >= 2 && e <= 2045) return cr::div_pos(a, b);
    return hw_div(a, b);
#else
    return a / b;
#endif
}

SP_HD double ieee_sqrt(double a) {
#if defined(__CUDA_ARCH__)
    const int ea = (int)(cr::dbits(a) >> 52);  // sign bit included
    if (ea > 0 && ea < 0x7ff) return cr::sqrt_pos(a);
    return hw_sqrt(a);
#else
    return sqrt(a);
#endif
}

namespace cr {

// D 2^-53 as a double for an integer D < 2^53 (exact), by integer operations.
SP_HD double u53_to_double(uint64_t m) {
    if (m == 0) return 0.0;
    const int p = 63 - clz64(m);
    return bdouble(((uint64_t)(1023 + p - 53) << 52) | ((m << (52 - p)) & ((1ULL << 52) - 1)));
}

SP_HD double out_of_domain(unsigned* hard) {
    if (hard) ++*hard;
    return bdouble(0x7ff8000000000000ULL);
}

}  // namespace cr

namespace cr {

SP_HD uint64_t mulhi64(uint64_t a, uint64_t b) { return (uint64_t)(((u128)a * b) >> 64); }

// Fast path of ln for x = m 2^e outside (1 - 2^-16, 1 + 2^-16): the same
// reduction as the full path, ln(1 + r) = r - r^2 P(r) with P in 64-bit
// Horner (r^2 P < 2^-15.6, so its 64-bit relative accuracy is about 2^-77
// absolute), summed with the 128-bit table value and e ln 2.  Returns false
// when the error bound (2^44 units of 2^-120) does not decide the rounding.
SP_HD bool ln_fast(int e, uint64_t frac, double* out) {
    const LnRow row = ln_row((int)(frac >> 44));
    const uint64_t r0 = ((1ULL << 52) | frac) * row.c;  // r 2^68, exact
    const uint64_t r64 = r0 >> 4;                       // r 2^64
    const uint64_t cf[8] = SP_CR_LN_FAST;               // 1/2 .. 1/9
    uint64_t h = cf[7];
#pragma unroll
    for (int j = 6; j >= 0; --j) h = cf[j] - mulhi64(r64, h);  // P(r) 2^64
    const uint64_t R2 = (uint64_t)(((u128)r0 * r0) >> 58);     // r^2 2^78
    const uint64_t q = mulhi64(R2, h);                           // r^2 P 2^78
    const u128 lnm = mk(row.th, row.tl) + ((u128)r0 << 52) - ((u128)q << 42);
    const W2 ln2w = {SP_CR_LN2};
    const uint64_t ae = (uint64_t)(e < 0 ? -e : e);
    const u128 eln2 = mk(ln2w) * ae;
    const uint64_t err = (1ULL << 44) + 8 + ae;
    unsigned undecided = 0;
    const double r = e >= 0 ? round_fixed_fast(eln2 + lnm, 120, err, &undecided)
                            : dneg(round_fixed_fast(eln2 - lnm, 120, err, &undecided));
    *out = r;
    return undecided == 0;
}

// Fast path of cos: the full path's reduction a = |t - k pi/2| = j/512 + d,
// then 1 - cos d = w Pc(w) and sin d = d - d w Ps(w) in 64-bit Horner, the
// products with the table's cos/sin(j/512) in 64 bits except y d, formed
// from the 128-bit table value and d to a few units of 2^-125.  Error bound
// 2^47 units of 2^-125; returns false when that does not decide the rounding.
SP_HD bool cos_fast(u128 a, int k, bool neg, double* out) {
    const int j = (int)(a >> 116);  // floor(512 a)
    if (j > 403) return false;
    const u128 d = a - ((u128)j << 116);                   // d 2^125, d < 2^-9
    const uint64_t dh = (uint64_t)(d >> 52);               // d 2^73 (truncated)
    const uint64_t dl = (uint64_t)d & ((1ULL << 52) - 1);  // the rest, units of 2^-125
    const uint64_t W = mulhi64(dh, dh);                    // w = d^2, 2^82
    const uint64_t w64 = W >> 18;                          // w 2^64
    const uint64_t cc[4] = SP_CR_COS_FAST, sc[4] = SP_CR_SIN_FAST;
    uint64_t pc = cc[2] - mulhi64(w64, cc[3]);
    pc = cc[1] - mulhi64(w64, pc);
    pc = cc[0] - mulhi64(w64, pc);  // Pc 2^64
    uint64_t ps = sc[2] - mulhi64(w64, sc[3]);
    ps = sc[1] - mulhi64(w64, ps);
    ps = sc[0] - mulhi64(w64, ps);  // Ps 2^64
    const uint64_t CM = mulhi64(W, pc);               // 1 - cos d, 2^82
    const uint64_t SDC = mulhi64(mulhi64(dh, W), ps);  // d w Ps, 2^91
    const CosRow row = cos_row(j);
    const int q = k & 3;
    const bool odd = (q & 1) != 0;
    // cos a = C - C (1 - cos d) - S sin d;  sin a = S - S (1 - cos d) + C sin d
    const u128 X = odd ? mk(row.sh, row.sl) : mk(row.ch, row.cl);  // 2^125
    const u128 Y = odd ? mk(row.ch, row.cl) : mk(row.sh, row.sl);
    const uint64_t X63 = (uint64_t)(X >> 62), Y63 = (uint64_t)(Y >> 62);  // 2^63
    const u128 yd = (((u128)hi64(Y) * dh + hi64((u128)lo64(Y) * dh)) >> 9) + (((u128)Y63 * dl) >> 63);  // y d
    const u128 xcm = (u128)mulhi64(X63, CM) << 44;    // x (1 - cos d)
    const u128 ysdc = (u128)mulhi64(Y63, SDC) << 35;  // y d w Ps
    const u128 v = odd ? (X + yd) - (xcm + ysdc) : (X + ysdc) - (xcm + yd);
    unsigned undecided = 0;
    const double r = round_fixed_fast(v, 125, 1ULL << 47, &undecided);
    const bool negative = (q == 2) || (q == 1 && !neg) || (q == 3 && neg);
    *out = dneg_if(negative, r);
    return undecided == 0;
}

}  // namespace cr

// Correctly rounded natural logarithm (see the header comment for the domain):
// the 64-bit fast path (fast = true), and the 128-bit evaluation wherever it
// cannot decide the rounding (or always, fast = false).
SP_HD double cr_log_impl(double x, unsigned* hard, bool fast) {
    using namespace cr;
    const uint64_t b = dbits(x);
    const int bexp = (int)(b >> 52);  // sign bit included: negative x lands above 2047
    if (bexp < 1023 - 360 || bexp > 1023 + 359) return out_of_domain(hard);
    // x in (1 - 2^-16, 1 + 2^-16): positive doubles order like their bit patterns
    if (b > 0x3FEFFFE000000000ULL && b < 0x3FF0001000000000ULL) return b == 0x3FF0000000000000ULL ? 0.0 : ln_near1(b, hard);
    const int e = bexp - 1023;
    if (fast) {
        double r;
        if (ln_fast(e, b & ((1ULL << 52) - 1), &r)) return r;
    }
    const uint64_t frac = b & ((1ULL << 52) - 1);
    const LnRow row = ln_row((int)(frac >> 44));
    const uint64_t r0 = ((1ULL << 52) | frac) * row.c;  // m c_i 2^68 - 2^68, exact (< 2^61)
    // Horner for ln(1+r) = r (1 - r (1/2 - r (1/3 - ... r/15)))
    const uint64_t r64 = r0 >> 4;
    const uint64_t inv64[8] = SP_CR_LN_INV64;  // 1/8 .. 1/15, Q0.64
    uint64_t h = inv64[7];
#pragma unroll
    for (int j = 6; j >= 0; --j) h = inv64[j] - (uint64_t)(((u128)r64 * h) >> 64);
    const W2 inv128[6] = SP_CR_LN_INV128;  // 1/2 .. 1/7, Q8.120
    u128 H = (u128)h << 56;
#pragma unroll
    for (int j = 5; j >= 0; --j) H = mk(inv128[j]) - mul_r68(r0, H);
    const u128 l1 = ((u128)r0 << 52) - mul_r68(r0, mul_r68(r0, H));
    const u128 lnm = mk(row.th, row.tl) + l1;  // ln m, in [0, ln 2)
    const W2 ln2w = {SP_CR_LN2};
    const uint64_t ae = (uint64_t)(e < 0 ? -e : e);
    const u128 eln2 = mk(ln2w) * ae;
    const uint64_t err = 8 + ((ae + 1) >> 1);
    if (e >= 0) return round_fixed(eln2 + lnm, 120, err, hard);
    return dneg(round_fixed(eln2 - lnm, 120, err, hard));
}

SP_HD double cr_log(double x, unsigned* hard) { return cr_log_impl(x, hard, true); }

// Correctly rounded exponential (subnormal results and overflow to +Inf
// included); |x| < 2^-54 returns 1, x < -746 returns 0, x > 710 +Inf, NaN
// returns NaN (counted as hard).
//   exp x = 2^k exp(j/256) exp(d),  x - k ln 2 = j/256 + d,  d in [0, 2^-8),
// with x - k ln 2 formed exactly in Q12.116 (up to ln 2's rounding, carried
// in the error bound) and exp(d) - 1 by its 12-term Taylor series.
SP_HD double cr_exp(double x, unsigned* hard) {
    using namespace cr;
    typedef __int128 s128;
    const uint64_t b = dbits(x);
    const int bexp = (int)((b >> 52) & 0x7ff);
    if (bexp < 1023 - 54) return 1.0;  // exp(x) within 2^-54 of 1 rounds to 1
    if (x != x) return out_of_domain(hard);
    if (x < -746.0) return 0.0;
    if (x > 710.0) return bdouble(0x7FF0000000000000ULL);
    const u128 X = (u128)((1ULL << 52) | (b & ((1ULL << 52) - 1))) << (bexp - 1075 + 116);  // |x|, Q12.116
    const int k = (int)floor(x * 1.4426950408889634 + 0.5);
    const W2 ln2w = {SP_CR_EXP_LN2};
    const uint64_t ak = (uint64_t)(k < 0 ? -k : k);
    const u128 kl = mk(ln2w) * ak;
    const s128 r = ((b >> 63) ? -(s128)X : (s128)X) - (k < 0 ? -(s128)kl : (s128)kl);
    const int j = (int)(r >> 108);                            // floor(256 r)
    const u128 d = (u128)(r - ((s128)j << 108)) << 10;         // Q2.126, [0, 2^-8)
    const W2 coef[11] = SP_CR_EXP_COEF;                         // 1/2! .. 1/12!
    u128 acc = mk(coef[10]);
#pragma unroll
    for (int i = 9; i >= 0; --i) acc = mk(coef[i]) + mulq3<126>(d, acc);
    const u128 em1 = mulq3<126>(d, ((u128)1 << 126) + mulq3<126>(d, acc));  // exp(d) - 1
    const ExpRow row = exp_row(j + 90);
    const u128 t = mk(row.hi, row.lo);
    const u128 v = t + mulq3<126>(t, em1);
    return round_fixed(v, 126 - k, 128 + 768 * ak, hard);  // 13 three-product multiplies: <= 5 units each
}

// log1p for a > -1 from the correctly rounded ln (Goldberg's correction):
// u = 1 + a rounded, then ln(u) a / (u - 1).  Accurate to about an ulp, not
// correctly rounded, but built only from cr_log and IEEE operations without
// contraction, so host and device give the same bits.
SP_HD double pm_log1p(double a, unsigned* hard) {
    const double u = 1.0 + a;
    if (u == 1.0) return a;
    return cr_log(u, hard) * (a / (u - 1.0));
}

// Correctly rounded cosine (see the header comment for the domain): the
// 64-bit fast path (fast = true), else the 128-bit evaluation.
SP_HD double cr_cos_impl(double t, unsigned* hard, bool fast) {
    using namespace cr;
    const uint64_t b = dbits(t) & ~(1ULL << 63);  // cos is even
    const int bexp = (int)(b >> 52);
    if (bexp >= 1023 + 3) return out_of_domain(hard);  // |t| >= 8, Inf, NaN
    // |t| < 2^-27: 1 - t^2/2 lies above the midpoint 1 - 2^-54, so cos rounds to 1
    if (bexp < 1023 - 27) return 1.0;
    const u128 T = (u128)((1ULL << 52) | (b & ((1ULL << 52) - 1))) << (bexp - 1075 + 125);
    // k = the multiple of pi/2 nearest to t (t < 8: k <= 5), by comparisons
    const W2 pio2w = {SP_CR_PIO2};
    const u128 pio2 = mk(pio2w);
    int k = 0;
#pragma unroll
    for (int m = 0; m < 5; ++m) k += (T >= pio2 * (uint64_t)m + (pio2 >> 1)) ? 1 : 0;
    const u128 kp = pio2 * (uint64_t)k;
    const bool neg = T < kp;
    const u128 a = neg ? kp - T : T - kp;
    if (fast) {
        double r;
        if (cos_fast(a, k, neg, &r)) return r;
    }
    int j = (int)(a >> 116);  // floor(512 a)
    uint64_t err = 512;
    if (j > 403) {  // cannot happen for |t - k pi/2| <= pi/4 + 2^-40
        j = 403;
        err = ~0ULL;
    }
    const u128 d = a - ((u128)j << 116);                    // [0, 2^-9)
    const u128 w = mulq3<125>(d, d);                        // < 2^-18
    const uint64_t w64 = (uint64_t)(w >> 61);               // w in Q0.64
    const W2 cc[3] = SP_CR_COS_COEF;                        // 1/2!, 1/4!, 1/6!
    const W2 sc[3] = SP_CR_SIN_COEF;                        // 1/3!, 1/5!, 1/7!
    const uint64_t ct[2] = SP_CR_COS_TAIL, st[2] = SP_CR_SIN_TAIL;  // 1/8!, 1/10! and 1/9!, 1/11! (Q0.64)
    // Horner in w: the innermost level in 64 bits (its error is scaled by w^4 <= 2^-72)
    const uint64_t c4 = ct[0] - (uint64_t)(((u128)w64 * ct[1]) >> 64);
    const uint64_t s4 = st[0] - (uint64_t)(((u128)w64 * st[1]) >> 64);
    u128 accc = mk(cc[2]) - mulq3<125>(w, (u128)c4 << 61);
    u128 accs = mk(sc[2]) - mulq3<125>(w, (u128)s4 << 61);
    accc = mk(cc[1]) - mulq3<125>(w, accc);
    accs = mk(sc[1]) - mulq3<125>(w, accs);
    accc = mk(cc[0]) - mulq3<125>(w, accc);
    accs = mk(sc[0]) - mulq3<125>(w, accs);
    const u128 cm = mulq3<125>(w, accc);                      // 1 - cos d
    const u128 sd = d - mulq3<125>(d, mulq3<125>(w, accs));   // sin d
    const CosRow row = cos_row(j);
    const u128 c0 = mk(row.ch, row.cl), s0 = mk(row.sh, row.sl);
    const int q = k & 3;
    u128 v;
    if ((q & 1) == 0)
        v = c0 - mulq3<125>(c0, cm) - mulq3<125>(s0, sd);  // cos a
    else
        v = s0 - mulq3<125>(s0, cm) + mulq3<125>(c0, sd);  // sin a
    // cos t = cos a, -sign(z) sin a, -cos a, sign(z) sin a for q = 0..3
    const bool negative = (q == 2) || (q == 1 && !neg) || (q == 3 && neg);
    const double r = round_fixed(v, 125, err, hard);
    return dneg_if(negative, r);
}

SP_HD double cr_cos(double t, unsigned* hard) { return cr_cos_impl(t, hard, true); }

}  // namespace sp

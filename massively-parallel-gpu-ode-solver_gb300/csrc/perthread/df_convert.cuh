// Conversions between FP64 and double-float built from integer operations,
// and the FP64-accurate step-size factor of the precision split.
//
// On GB300 a hardware float<->double conversion (cvt.f64.f32 / cvt.f32.f64)
// issues to the FP64 pipe and costs as much as an FP64 fused multiply-add
// (measured: ~5e11 per second per GPU each, against ~3e13 FP32 FMAs), while
// the same conversion assembled from shifts, masks and adds runs on the
// integer pipe roughly 17x faster. The precision-split solver converts its
// FP64 state to double-float stage inputs and its double-float stage sums back
// to FP64 every step, so it uses these:
//
//   widen(f)    float -> double, exact (IEEE single embeds in double); float
//               subnormals become signed zeros (they only occur as the low
//               part of values near 1e-31 and below);
//   to_double   double-float -> double: widen(hi) + widen(lo) in one FP64
//               add (the nearest double to the pair);
//   split(x)    double -> double-float: the leading 24 significant bits of x
//               are hi, the next 24 bits lo (both truncated, so hi + lo is
//               within 2^-47 |x| of x), renormalised so that |lo| <= ulp(hi)/2;
//               values whose low part would leave float's normal range
//               (|x| < 2^-74 or |x| >= 2^128), zeros, infinities and NaNs
//               take the exact conversion of dfloat(double) instead;
//   in_float_range(x)  x is zero, not finite (infinities and NaNs are the
//               non-finite status's business) or its magnitude lies in float's
//               normal range [2^-126, 2^128), where a double-float keeps its
//               ~48 bits.
//
// The functions compile for the host as well (bit patterns through memcpy),
// so the CPU tests check them against exact references.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#include "dfloat.cuh"

namespace mpgos {
namespace df {

MPGOS_DF_HD uint32_t float_bits(float f)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}

MPGOS_DF_HD float float_from_bits(uint32_t u)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}

MPGOS_DF_HD uint32_t double_hi(double x)
{
#if defined(__CUDA_ARCH__)
    return static_cast<uint32_t>(__double2hiint(x));
#else
    uint64_t u;
    memcpy(&u, &x, 8);
    return static_cast<uint32_t>(u >> 32);
#endif
}

MPGOS_DF_HD uint32_t double_lo(double x)
{
#if defined(__CUDA_ARCH__)
    return static_cast<uint32_t>(__double2loint(x));
#else
    uint64_t u;
    memcpy(&u, &x, 8);
    return static_cast<uint32_t>(u);
#endif
}

MPGOS_DF_HD double double_from_words(uint32_t hi, uint32_t lo)
{
#if defined(__CUDA_ARCH__)
    return __hiloint2double(static_cast<int>(hi), static_cast<int>(lo));
#else
    const uint64_t u = (static_cast<uint64_t>(hi) << 32) | lo;
    double x;
    memcpy(&x, &u, 8);
    return x;
#endif
}

MPGOS_DF_HD int leading_zeros(uint32_t v)  // v != 0
{
#if defined(__CUDA_ARCH__)
    return __clz(static_cast<int>(v));
#else
    return __builtin_clz(v);
#endif
}

// float -> double by moving the exponent and mantissa fields
MPGOS_DF_HD double widen(float f)
{
    const uint32_t b   = float_bits(f);
    const uint32_t mag = b & 0x7fffffffu;
    uint32_t hi = (b & 0x80000000u) | ((mag >> 3) + (896u << 20));   // exponent bias 127 -> 1023
    uint32_t lo = b << 29;
    if (mag < 0x00800000u) {            // zero or subnormal
        hi = b & 0x80000000u;
        lo = 0u;
    } else if (mag >= 0x7f800000u) {    // infinity or NaN (payload kept)
        hi |= 0x7ff00000u;
    }
    return double_from_words(hi, lo);
}

MPGOS_DF_HD double to_double(dfloat v) { return widen(v.hi) + widen(v.lo); }

MPGOS_DF_HD bool in_float_range(double x)
{
    const uint32_t h = double_hi(x);
    const uint32_t e = (h >> 20) & 0x7ffu;
    const bool zero  = ((h & 0x7fffffffu) | double_lo(x)) == 0u;
    return zero || e == 0x7ffu || (e >= 897u && e <= 1150u);
}

// the exact conversion, out of line so that the rare slow path of split is a
// branch rather than FP64 conversions predicated into every call
#if defined(__CUDACC__)
static __host__ __device__ __noinline__
#else
static inline
#endif
dfloat split_exact(double x)
{
    return dfloat(x);
}

MPGOS_DF_HD dfloat split(double x)
{
    const uint32_t H = double_hi(x), L = double_lo(x);
    const uint32_t e = (H >> 20) & 0x7ffu;
    if (e < 949u || e > 1150u) return split_exact(x);   // outside the fast path's range (also 0, inf, NaN)
    const uint32_t s = H & 0x80000000u;
    // hi: sign, exponent rebased to float, the top 23 stored mantissa bits
    // (20 from the high word, 3 from the low word)
    const uint32_t m = (H & 0x7fffffffu) - (896u << 20);
    const uint32_t hib = s | (m << 3) | (L >> 29);
    // lo: the remaining 29 bits as an integer r, scaled by the double's ulp
    // 2^(e - 1075); its leading one moves to bit 23 and the exponent follows
    const uint32_t r = L & 0x1fffffffu;
    uint32_t lob = s;
    if (r != 0u) {
        const int n = leading_zeros(r);                   // 3 .. 31
        const uint32_t mant = (r << n) >> 8;              // leading one at bit 23
        lob = s | (((e - 918u - static_cast<uint32_t>(n)) << 23) + mant);
    }
    return quick_two_sum(float_from_bits(hib), float_from_bits(lob));
}

MPGOS_DF_HD double d_fma(double a, double b, double c)
{
#if defined(__CUDA_ARCH__)
    return __fma_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}

// ---- the step-size factor of the precision split ----------------------------

// log2 of a non-negative double to ~2e-6: the exponent from the bit pattern,
// the top 20 mantissa bits through the float log2. Zero and subnormals give
// -inf; infinities and NaNs a value above 1024.
MPGOS_DF_HD float log2_estimate(double x)
{
    const uint32_t h = double_hi(x);
    const int e      = static_cast<int>((h >> 20) & 0x7ffu);
    const float m    = float_from_bits(0x3f800000u | ((h & 0x000fffffu) << 3));   // [1, 2)
#if defined(__CUDA_ARCH__)
    const float lm = __log2f(m);
#else
    const float lm = std::log2(m);
#endif
    return e == 0 ? -INFINITY : static_cast<float>(e - 1023) + lm;
}

// 1/a to float precision for a positive normal double a: a float reciprocal
// of the mantissa, the exponent negated on the integer pipe.
MPGOS_DF_HD double reciprocal_estimate(double a)
{
    const uint32_t h = double_hi(a);
    const int e      = static_cast<int>((h >> 20) & 0x7ffu);
    const float m    = float_from_bits(0x3f800000u | ((h & 0x000fffffu) << 3));   // [1, 2)
    const double r   = widen(f_rcp(m));                                            // (0.5, 1]
    // multiply by 2^(1023 - e): add to r's exponent field
    const uint32_t rh = double_hi(r) + (static_cast<uint32_t>(1023 - e) << 20);
    return double_from_words(rh, double_lo(r));
}

// R^(1/n), R = tol / err (positive, finite), n = 5 (fifth) or 4, to a few
// ulp of FP64 from an FP32 estimate y0 (relative error ~1e-6, so |w| ~ 5e-6
// and the neglected w^3 term stays below 1e-17):
// with w = tol / (y0^n err) - 1, R^(1/n) = y0 (1 + w)^(1/n)
//   = y0 (1 + w/n - (n-1) w^2 / (2 n^2) + O(w^3));
// the quotient uses one Newton step on the float reciprocal (error ~1e-14 of
// 1/a, so ~1e-14 |w| in w), tol - a is exact (Sterbenz) near the root.
MPGOS_DF_HD double root_refine(float y0, double tol, double err, bool fifth)
{
    const double y  = widen(y0);
    const double y2 = y * y;
    const double y4 = y2 * y2;
    const double yn = fifth ? y4 * y : y4;
    const double a  = yn * err;
    const double r0 = reciprocal_estimate(a);
    const double r  = d_fma(r0, d_fma(-a, r0, 1.0), r0);
    const double w  = (tol - a) * r;
    const double c1 = fifth ? 0.2 : 0.25;
    const double c2 = fifth ? -0.08 : -0.09375;
    return d_fma(y, w * d_fma(w, c2, c1), y);
}

// FP32 estimate of R^(1/n) from log2 R (clamped to float's range)
MPGOS_DF_HD float root_estimate(float log2_ratio, bool fifth)
{
    const float l = std::fmin(std::fmax(log2_ratio * (fifth ? 0.2f : 0.25f), -120.0f), 120.0f);
#if defined(__CUDA_ARCH__)
    return exp2f(l);
#else
    return std::exp2(l);
#endif
}

}  // namespace df
}  // namespace mpgos

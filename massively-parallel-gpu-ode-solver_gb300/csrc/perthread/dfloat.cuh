// Double-float arithmetic on the FP32 pipe.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2,
// about 48 significant bits (relative precision ~4e-15) and the exponent
// range of float. On GB300 the FP32 pipe issues ~64x more operations per
// clock than the FP64 pipe, and a double-float add or multiply costs 7-11
// FP32 operations, so stage arithmetic that needs more than float but not
// the full 53 bits of double runs several times faster here than in FP64.
//
// Algorithms (all published, restated here):
//   two_sum         Knuth, TAOCP vol. 2, 4.2.2 (error-free sum, 6 flops)
//   quick_two_sum   Dekker 1971 (error-free sum for |a| >= |b|, 3 flops)
//   two_prod        error-free product with a fused multiply-add
//   add             "sloppy" double-float add of Hida, Li & Bailey (QD
//                   library, 2001): error <= ~2^-46 (|a| + |b|)
//   mul             double-float multiply with FMA (same source)
//   fma, dot2       a*b + c and a*b + c*d: the exact leading products summed
//                   by two_sum, all low-order terms folded into one tail
//                   (the same error class as add)
//   prod_sum        sums of products accumulated as (two_sum of the leading
//                   floats, one float of tails), normalised once at the end
//   div             two long-division correction steps on a float quotient
//   sqrt            Karp & Markstein 1997 (Newton corrections from rsqrt)
// sin, cos and sincospi run on the FP32 pipe too (Cody-Waite reduction and
// Taylor series, below); exp, log and pow evaluate in FP64 through CUDA's
// double functions and round back (one FP64 evaluation per call).
//
// Hook code templated on its precision (the reference's
// `template <class Precision> __device__ void PerThread_OdeFunction(...)`)
// instantiates unchanged with Precision = mpgos::df::dfloat: literals and
// double parameters convert implicitly, the math functions are found by
// argument-dependent lookup.
#pragma once

#include <cmath>

#if defined(__CUDACC__)
#include <cuda_runtime.h>
#define MPGOS_DF_HD __host__ __device__ __forceinline__
#else
#define MPGOS_DF_HD inline
#endif

namespace mpgos {
namespace df {

// Correctly rounded float operations that the compiler may not fuse or
// reorder: the CUDA intrinsics on the device; on the host (used by the CPU
// tests of this header, built with -ffp-contract=off) plain IEEE arithmetic.
MPGOS_DF_HD float f_add(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
MPGOS_DF_HD float f_sub(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
MPGOS_DF_HD float f_mul(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
MPGOS_DF_HD float f_fma(float a, float b, float c)
{
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}
MPGOS_DF_HD float f_rint(float a)
{
#if defined(__CUDA_ARCH__)
    return rintf(a);
#else
    return std::nearbyint(a);
#endif
}
MPGOS_DF_HD float f_rcp(float a)
{
#if defined(__CUDA_ARCH__)
    return __frcp_rn(a);
#else
    return 1.0f / a;
#endif
}

struct dfloat {
    float hi, lo;

    dfloat() = default;
    MPGOS_DF_HD constexpr dfloat(float h, float l) : hi(h), lo(l) {}
    MPGOS_DF_HD dfloat(double d) : hi(static_cast<float>(d)), lo(0.0f)
    {
        lo = static_cast<float>(d - static_cast<double>(hi));
    }
    MPGOS_DF_HD constexpr dfloat(float f) : hi(f), lo(0.0f) {}
    MPGOS_DF_HD constexpr dfloat(int i) : hi(static_cast<float>(i)), lo(0.0f) {}
    MPGOS_DF_HD explicit operator double() const
    {
        return static_cast<double>(hi) + static_cast<double>(lo);
    }
    MPGOS_DF_HD explicit operator float() const { return hi; }
};

// ---- error-free transformations ----------------------------------------------
MPGOS_DF_HD dfloat two_sum(float a, float b)
{
    const float s  = f_add(a, b);
    const float bb = f_sub(s, a);
    const float e  = f_add(f_sub(a, f_sub(s, bb)), f_sub(b, bb));
    return dfloat(s, e);
}

MPGOS_DF_HD dfloat quick_two_sum(float a, float b)
{
    const float s = f_add(a, b);
    return dfloat(s, f_sub(b, f_sub(s, a)));
}

MPGOS_DF_HD dfloat two_prod(float a, float b)
{
    const float p = f_mul(a, b);
    return dfloat(p, f_fma(a, b, -p));
}

// ---- arithmetic ------------------------------------------------------------------
MPGOS_DF_HD dfloat operator+(dfloat a, dfloat b)
{
    dfloat s = two_sum(a.hi, b.hi);
    const float e = f_add(s.lo, f_add(a.lo, b.lo));
    return quick_two_sum(s.hi, e);
}

MPGOS_DF_HD dfloat operator-(dfloat a) { return dfloat(-a.hi, -a.lo); }

MPGOS_DF_HD dfloat operator-(dfloat a, dfloat b) { return a + (-b); }

MPGOS_DF_HD dfloat operator*(dfloat a, dfloat b)
{
    dfloat p = two_prod(a.hi, b.hi);
    float e = f_fma(a.hi, b.lo, p.lo);
    e = f_fma(a.lo, b.hi, e);
    return quick_two_sum(p.hi, e);
}

// a * b + c with one renormalisation (the sloppy add of the exact leading
// product and c, the product's and c's low parts folded into the tail):
// 15 FP32 operations instead of 18 for a multiply then an add.
MPGOS_DF_HD dfloat fma(dfloat a, dfloat b, dfloat c)
{
    const dfloat p = two_prod(a.hi, b.hi);
    const dfloat s = two_sum(p.hi, c.hi);
    float e = f_add(p.lo, c.lo);
    e = f_fma(a.hi, b.lo, e);
    e = f_fma(a.lo, b.hi, e);
    e = f_add(e, s.lo);
    return quick_two_sum(s.hi, e);
}

// a * b + c * d the same way (19 operations instead of 25).
MPGOS_DF_HD dfloat dot2(dfloat a, dfloat b, dfloat c, dfloat d)
{
    const dfloat p = two_prod(a.hi, b.hi);
    const dfloat q = two_prod(c.hi, d.hi);
    const dfloat s = two_sum(p.hi, q.hi);
    float e = f_add(p.lo, q.lo);
    e = f_fma(a.hi, b.lo, e);
    e = f_fma(a.lo, b.hi, e);
    e = f_fma(c.hi, d.lo, e);
    e = f_fma(c.lo, d.hi, e);
    e = f_add(e, s.lo);
    return quick_two_sum(s.hi, e);
}

// Sum of double-float products kept unnormalised between terms: the leading
// floats are summed by two_sum, every rounding error and cross product goes
// into the trailing float, normalised once when the sum is used
// (prod_sum_start: 4 FP32 operations, prod_sum_add: 12 per further term
// instead of 15 for a fused multiply-add with renormalisation).
struct prod_sum {
    float h, l;
};

MPGOS_DF_HD prod_sum prod_sum_start(dfloat a, dfloat b)
{
    const dfloat p = two_prod(a.hi, b.hi);
    return prod_sum{p.hi, f_fma(a.hi, b.lo, f_fma(a.lo, b.hi, p.lo))};
}

MPGOS_DF_HD void prod_sum_add(prod_sum& s, dfloat a, dfloat b)
{
    const dfloat p = two_prod(a.hi, b.hi);
    const dfloat t = two_sum(s.h, p.hi);
    s.h = t.hi;
    s.l = f_add(s.l, f_add(t.lo, f_fma(a.hi, b.lo, f_fma(a.lo, b.hi, p.lo))));
}

MPGOS_DF_HD dfloat prod_sum_value(prod_sum s) { return quick_two_sum(s.h, s.l); }

// c + a * s for an unnormalised product sum s (15 operations, the same as
// fma(a, value(s), c) without normalising s first).
MPGOS_DF_HD dfloat prod_sum_axpy(dfloat a, prod_sum s, dfloat c)
{
    const dfloat p = two_prod(a.hi, s.h);
    float e = f_fma(a.hi, s.l, f_fma(a.lo, s.h, p.lo));
    const dfloat t = two_sum(p.hi, c.hi);
    e = f_add(e, f_add(c.lo, t.lo));
    return quick_two_sum(t.hi, e);
}

// a * f for a float f (one product term fewer)
MPGOS_DF_HD dfloat mul_f(dfloat a, float f)
{
    dfloat p = two_prod(a.hi, f);
    return quick_two_sum(p.hi, f_fma(a.lo, f, p.lo));
}

MPGOS_DF_HD dfloat operator/(dfloat a, dfloat b)
{
    const float r  = f_rcp(b.hi);
    const float q1 = f_mul(a.hi, r);
    dfloat q = quick_two_sum(q1, f_mul((a - b * dfloat(q1)).hi, r));
    return q + dfloat(f_mul((a - b * q).hi, r));
}

MPGOS_DF_HD dfloat& operator+=(dfloat& a, dfloat b) { return a = a + b; }
MPGOS_DF_HD dfloat& operator-=(dfloat& a, dfloat b) { return a = a - b; }
MPGOS_DF_HD dfloat& operator*=(dfloat& a, dfloat b) { return a = a * b; }
MPGOS_DF_HD dfloat& operator/=(dfloat& a, dfloat b) { return a = a / b; }

// ---- comparisons (hi decides unless equal) ---------------------------------------
MPGOS_DF_HD bool operator<(dfloat a, dfloat b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
MPGOS_DF_HD bool operator>(dfloat a, dfloat b) { return b < a; }
MPGOS_DF_HD bool operator<=(dfloat a, dfloat b) { return !(b < a) && a.hi == a.hi && b.hi == b.hi; }
MPGOS_DF_HD bool operator>=(dfloat a, dfloat b) { return b <= a; }
MPGOS_DF_HD bool operator==(dfloat a, dfloat b) { return a.hi == b.hi && a.lo == b.lo; }
MPGOS_DF_HD bool operator!=(dfloat a, dfloat b) { return !(a == b); }

// ---- functions ---------------------------------------------------------------------
MPGOS_DF_HD dfloat abs(dfloat a) { return (a.hi < 0.0f) ? -a : a; }
MPGOS_DF_HD dfloat fabs(dfloat a) { return abs(a); }
MPGOS_DF_HD dfloat fmin(dfloat a, dfloat b) { return (b < a) ? b : a; }
MPGOS_DF_HD dfloat fmax(dfloat a, dfloat b) { return (a < b) ? b : a; }
MPGOS_DF_HD bool isfinite(dfloat a) { return std::isfinite(a.hi); }
MPGOS_DF_HD bool isnan(dfloat a) { return std::isnan(a.hi); }

MPGOS_DF_HD dfloat sqrt(dfloat a)
{
    if (!(a.hi > 0.0f)) return dfloat(std::sqrt(a.hi), 0.0f);
    const float x = 1.0f / std::sqrt(a.hi);
    const float y = f_mul(a.hi, x);
    const dfloat yy = two_prod(y, y);
    const dfloat s = quick_two_sum(y, f_mul((a - yy).hi, f_mul(x, 0.5f)));
    return s + dfloat(f_mul((a - s * s).hi, f_mul(x, 0.5f)));
}

// ---- sine and cosine on the FP32 pipe --------------------------------------------
// Cody & Waite (1980) reduction x = k pi/2 + r with pi/2 split into three
// floats (each k * P_i exact as a double-float; |k| < 2^22), then the Taylor
// series of sin and cos on |r| <= pi/4: terms through r^9 / r^8 in
// double-float by Horner's rule, the tail (r^11.. r^17 / r^10.. r^16, below
// 2e-8 in size) in float. Error: a few 1e-16 plus the double-float rounding of
// the reduction, ~|x| 2^-48 (the precision the argument itself carries).
namespace detail {
constexpr float PIO2_1 = 0x1.921fb6p+0f;
constexpr float PIO2_2 = -0x1.777a5cp-25f;
constexpr float PIO2_3 = -0x1.ee59dap-50f;

MPGOS_DF_HD dfloat reduce_pio2(dfloat x, int& quadrant)
{
    const float k = f_rint(f_mul(x.hi, 0.63661977236758134f));
    dfloat r = x - two_prod(k, PIO2_1);
    r = r - two_prod(k, PIO2_2);
    r = r - two_prod(k, PIO2_3);
    quadrant = static_cast<int>(k) & 3;
    return r;
}

// sin(r) for |r| <= pi/4
MPGOS_DF_HD dfloat sin_kernel(dfloat r)
{
    const dfloat z = r * r;
    const float zf = z.hi;
    float tail = 1.0f / 6402373705728000.0f;                 // 1/17!
    tail = f_fma(zf, tail, -1.0f / 1307674368000.0f);        // -1/15!
    tail = f_fma(zf, tail, 1.0f / 6227020800.0f);            // 1/13!
    tail = f_fma(zf, tail, -1.0f / 39916800.0f);             // -1/11!
    dfloat p = dfloat(0x1.71de3ap-19f, 0x1.55b1ccp-45f) + mul_f(z, tail);   // 1/9!
    p = dfloat(-0x1.a01a02p-13f, 0x1.7f97fap-39f) + z * p;                // -1/7!
    p = dfloat(0x1.111112p-7f, -0x1.dddddep-32f) + z * p;                  // 1/5!
    p = dfloat(-0x1.555556p-3f, 0x1.555556p-28f) + z * p;                  // -1/3!
    return r + (r * z) * p;
}

// cos(r) for |r| <= pi/4
MPGOS_DF_HD dfloat cos_kernel(dfloat r)
{
    const dfloat z = r * r;
    const float zf = z.hi;
    float tail = 1.0f / 20922789888000.0f;                   // 1/16!
    tail = f_fma(zf, tail, -1.0f / 87178291200.0f);          // -1/14!
    tail = f_fma(zf, tail, 1.0f / 479001600.0f);             // 1/12!
    tail = f_fma(zf, tail, -1.0f / 3628800.0f);              // -1/10!
    dfloat p = dfloat(0x1.a01a02p-16f, -0x1.7f97fap-42f) + mul_f(z, tail);  // 1/8!
    p = dfloat(-0x1.6c16c2p-10f, 0x1.27d27ep-35f) + z * p;                // -1/6!
    p = dfloat(0x1.555556p-5f, -0x1.555556p-30f) + z * p;                  // 1/4!
    p = dfloat(-0.5f, 0.0f) + z * p;
    return dfloat(1.0f) + z * p;
}
}  // namespace detail

MPGOS_DF_HD dfloat sin(dfloat a)
{
    int q;
    const dfloat r = detail::reduce_pio2(a, q);
    switch (q) {
        case 0: return detail::sin_kernel(r);
        case 1: return detail::cos_kernel(r);
        case 2: return -detail::sin_kernel(r);
        default: return -detail::cos_kernel(r);
    }
}

MPGOS_DF_HD dfloat cos(dfloat a)
{
    int q;
    const dfloat r = detail::reduce_pio2(a, q);
    switch (q) {
        case 0: return detail::cos_kernel(r);
        case 1: return -detail::sin_kernel(r);
        case 2: return -detail::cos_kernel(r);
        default: return detail::sin_kernel(r);
    }
}
MPGOS_DF_HD dfloat exp(dfloat a) { return dfloat(std::exp(static_cast<double>(a))); }
MPGOS_DF_HD dfloat log(dfloat a) { return dfloat(std::log(static_cast<double>(a))); }
MPGOS_DF_HD dfloat pow(dfloat a, dfloat b)
{
    return dfloat(std::pow(static_cast<double>(a), static_cast<double>(b)));
}
MPGOS_DF_HD dfloat pow(dfloat a, double b) { return dfloat(std::pow(static_cast<double>(a), b)); }
MPGOS_DF_HD dfloat pow(dfloat a, int n)
{
    return dfloat(std::pow(static_cast<double>(a), static_cast<double>(n)));
}
// sin and cos of one argument with one reduction
MPGOS_DF_HD void sincos(dfloat a, dfloat* s, dfloat* c)
{
    int q;
    const dfloat r = detail::reduce_pio2(a, q);
    const dfloat sk = detail::sin_kernel(r), ck = detail::cos_kernel(r);
    switch (q) {
        case 0: *s = sk; *c = ck; break;
        case 1: *s = ck; *c = -sk; break;
        case 2: *s = -sk; *c = -ck; break;
        default: *s = -ck; *c = sk; break;
    }
}

// sin(pi a) and cos(pi a) with pi a formed in double-float
MPGOS_DF_HD void sincospi(dfloat a, dfloat* s, dfloat* c)
{
    const dfloat x = a * dfloat(0x1.921fb6p+1f, -0x1.777a5cp-24f);   // pi
    *s = sin(x);
    *c = cos(x);
}

}  // namespace df
}  // namespace mpgos

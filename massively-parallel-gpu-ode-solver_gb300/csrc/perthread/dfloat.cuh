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
//   div             two long-division correction steps on a float quotient
//   sqrt            Karp & Markstein 1997 (Newton corrections from rsqrt)
// Transcendental functions (cos, sin, exp, log, pow, sincospi) evaluate in
// FP64 through CUDA's double functions and round back: hooks call them once
// per right-hand side, so they cost little next to the stage arithmetic.
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

MPGOS_DF_HD dfloat cos(dfloat a) { return dfloat(std::cos(static_cast<double>(a))); }
MPGOS_DF_HD dfloat sin(dfloat a) { return dfloat(std::sin(static_cast<double>(a))); }
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
#if defined(__CUDACC__)
MPGOS_DF_HD void sincospi(dfloat a, dfloat* s, dfloat* c)
{
    double sd, cd;
    ::sincospi(static_cast<double>(a), &sd, &cd);
    *s = dfloat(sd);
    *c = dfloat(cd);
}
#endif

}  // namespace df
}  // namespace mpgos

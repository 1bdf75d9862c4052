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
// sin, cos, sincospi, exp, log and pow run on the FP32 pipe too (Cody-Waite
// reductions, a table of sin / cos at multiples of pi/128 (Tang 1991), Taylor
// series, one Newton step for log; below); only arguments outside their
// ranges fall back to CUDA's FP64 functions.
//
// Hook code templated on its precision (the reference's
// `template <class Precision> __device__ void PerThread_OdeFunction(...)`)
// instantiates unchanged with Precision = mpgos::df::dfloat: literals and
// double parameters convert implicitly, the math functions are found by
// argument-dependent lookup.
#pragma once

#include <cmath>

#include "dfloat_trig_table.h"

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
MPGOS_DF_HD float f_nan()
{
#if defined(__CUDA_ARCH__)
    return __int_as_float(0x7fffffff);
#else
    return std::nanf("");
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
        // beyond the float range hi is infinite and carries the value alone
        if (!std::isinf(hi)) lo = static_cast<float>(d - static_cast<double>(hi));
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

// a + b with the error bounded relative to the result rather than to the
// operands (both parts summed by two_sum; 20 operations; the "IEEE" add of
// the same source), for sums that cancel
MPGOS_DF_HD dfloat add_accurate(dfloat a, dfloat b)
{
    dfloat s = two_sum(a.hi, b.hi);
    const dfloat t = two_sum(a.lo, b.lo);
    s = quick_two_sum(s.hi, f_add(s.lo, t.hi));
    return quick_two_sum(s.hi, f_add(s.lo, t.lo));
}

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

// ---- table-driven sine and cosine (Tang 1991) ------------------------------------
// x = k pi/128 + r: k the nearest integer to x 128/pi, r by Cody & Waite with
// pi/128 in three floats (the pi/2 split above scaled by 2^-6, each product
// k P_i exact by two_prod; |r| <= 0.58 pi/128 for |x| < 2^14). With k = 64 q + j
// the table gives sin and cos of the angle a = q pi/2 + j pi/128 (entries of
// three floats, rotated by the quadrant q); with z = r^2
//   h = 1 - cos r = z/2 - z^2/24 + z^3/720,   s = sin r = r - r z (1/6 - z/120)
// (the next terms are below 1e-19 at |r| <= 0.58 pi/128), and
//   cos x = C - (C h + S s),   sin x = S - (S h - C s)
// so that the table value enters exactly and only the small correction
// (|.| < 0.015) carries the rounding of the polynomials and products.
// About 100 FP32 operations for either function against ~150 for the series
// on |r| <= pi/4, and half the dependent chain.
namespace detail {
constexpr float INV_PIO128 = 0x1.45f306p+5f;   // 128/pi
constexpr float PIO128_1 = PIO2_1 * 0x1p-6f;   // pi/128 = (PIO2_1 + PIO2_2 + PIO2_3) 2^-6
constexpr float PIO128_2 = PIO2_2 * 0x1p-6f;
constexpr float PIO128_3 = PIO2_3 * 0x1p-6f;
constexpr float SIXTH_HI = 0x1.555556p-3f;     // 1/6 = SIXTH_HI + SIXTH_LO
constexpr float SIXTH_LO = -0x1.555556p-28f;
// |x| below: the table path (a plugin may define MPGOS_DF_TRIG_SERIES to take
// the series path for every argument)
#ifdef MPGOS_DF_TRIG_SERIES
constexpr float TRIG_TABLE_LIMIT = 0.0f;
constexpr float TRIGPI_TABLE_LIMIT = 0.0f;
#else
constexpr float TRIG_TABLE_LIMIT = 0x1p+14f;
constexpr float TRIGPI_TABLE_LIMIT = 0x1p+16f;
#endif
// A plugin whose sin / cos / sincos arguments stay below TRIG_TABLE_LIMIT in
// magnitude, and its sincospi arguments below TRIGPI_TABLE_LIMIT, may define
// MPGOS_DF_TRIG_BOUNDED: every call then runs the table path alone, without
// the branch to the wide-range path, and an argument outside the bound (or
// not finite) gives NaN, which the solver reports as a non-finite step.
// Without the branch the compiler can interleave a call with the independent
// work around it (the state arithmetic of a right-hand side, the forcing terms
// of the other stages; sin and cos of one argument share their reduction).
#if defined(MPGOS_DF_TRIG_BOUNDED) && defined(MPGOS_DF_TRIG_SERIES)
#error "MPGOS_DF_TRIG_BOUNDED and MPGOS_DF_TRIG_SERIES exclude each other"
#endif
#ifdef MPGOS_DF_TRIG_BOUNDED
constexpr bool TRIG_BOUNDED = true;
#else
constexpr bool TRIG_BOUNDED = false;
#endif

#if defined(__CUDACC__)
static __device__ const float4 TRIG_MAIN_DEV[64] = {MPGOS_DF_TRIG_TABLE_MAIN};
static __device__ const float2 TRIG_TAIL_DEV[64] = {MPGOS_DF_TRIG_TABLE_TAIL};
#endif
static const float TRIG_MAIN_HOST[64][4] = {MPGOS_DF_TRIG_TABLE_MAIN};
static const float TRIG_TAIL_HOST[64][2] = {MPGOS_DF_TRIG_TABLE_TAIL};

// x - k pi/128 for |x| < 2^14, k the nearest integer to x 128/pi
MPGOS_DF_HD dfloat reduce_pio128(dfloat x, int& k)
{
    const float kf = f_rint(f_mul(x.hi, INV_PIO128));
    const dfloat p1 = two_prod(kf, PIO128_1);
    const dfloat p2 = two_prod(kf, PIO128_2);
    const dfloat a = two_sum(x.hi, -p1.hi);                       // exact (Sterbenz)
    const dfloat u = two_sum(a.hi, f_add(f_sub(x.lo, p1.lo), a.lo));   // the only rounding at ~2^-24 |x|
    const dfloat b = two_sum(u.hi, -p2.hi);
    float e = f_sub(u.lo, p2.lo);                                  // the rest at ~2^-24 |r|
    e = f_fma(-kf, PIO128_3, e);
    e = f_add(e, b.lo);
    k = static_cast<int>(kf);
    return two_sum(b.hi, e);
}

// A + A2 - w for a table value A + A2 (A2 the third float) and a small w:
// the accurate add (both parts by two_sum), A2 joining the last tail, so the
// result carries one rounding of its own low float
MPGOS_DF_HD dfloat table_minus(dfloat A, float A2, dfloat w)
{
    const dfloat t = two_sum(A.hi, -w.hi);
    const dfloat u = two_sum(A.lo, -w.lo);
    const dfloat v = quick_two_sum(t.hi, f_add(t.lo, u.hi));
    return quick_two_sum(v.hi, f_add(v.lo, f_add(u.lo, A2)));
}

// sin and cos of k pi/128 + r, |r| <= 0.6 pi/128
MPGOS_DF_HD void sincos_table(dfloat r, int k, dfloat* s_out, dfloat* c_out)
{
    const int j = k & 63, q = (k >> 6) & 3;
#if defined(__CUDA_ARCH__)
    const float4 m = __ldg(&TRIG_MAIN_DEV[j]);
    const float2 t = __ldg(&TRIG_TAIL_DEV[j]);
    const dfloat S(m.x, m.y), C(m.z, m.w);
    const float S2 = t.x, C2 = t.y;
#else
    const dfloat S(TRIG_MAIN_HOST[j][0], TRIG_MAIN_HOST[j][1]), C(TRIG_MAIN_HOST[j][2], TRIG_MAIN_HOST[j][3]);
    const float S2 = TRIG_TAIL_HOST[j][0], C2 = TRIG_TAIL_HOST[j][1];
#endif
    // rotate by the quadrant without branches: (sin a, cos a) of a = q pi/2 + j pi/128
    const bool odd = (q & 1) != 0, sneg = (q & 2) != 0, cneg = ((q + 1) & 2) != 0;
    dfloat Sa = odd ? C : S, Ca = odd ? S : C;
    float Sa2 = odd ? C2 : S2, Ca2 = odd ? S2 : C2;
    Sa = sneg ? -Sa : Sa;
    Sa2 = sneg ? -Sa2 : Sa2;
    Ca = cneg ? -Ca : Ca;
    Ca2 = cneg ? -Ca2 : Ca2;
    // z = r^2 (unnormalised pair), h = 1 - cos r, s = sin r
    const dfloat zz = two_prod(r.hi, r.hi);
    const float zh = zz.hi, zl = f_fma(f_add(r.hi, r.hi), r.lo, zz.lo);
    const float g = f_mul(f_mul(zh, zh), f_fma(zh, -1.0f / 720.0f, 1.0f / 24.0f));
    const dfloat h(f_mul(0.5f, zh), f_fma(0.5f, zl, -g));
    const dfloat rz = two_prod(r.hi, zh);                                  // r z
    const float rzl = f_fma(r.hi, zl, f_fma(r.lo, zh, rz.lo));
    const dfloat m6 = two_prod(rz.hi, SIXTH_HI);                           // r z (1/6 - z/120)
    const float m6l = f_fma(rz.hi, f_fma(zh, -1.0f / 120.0f, SIXTH_LO), f_fma(rzl, SIXTH_HI, m6.lo));
    const dfloat s0 = quick_two_sum(r.hi, -m6.hi);
    const dfloat s(s0.hi, f_add(s0.lo, f_sub(r.lo, m6l)));
    *c_out = table_minus(Ca, Ca2, dot2(Ca, h, Sa, s));
    *s_out = table_minus(Sa, Sa2, dot2(Sa, h, -Ca, s));
}

// sin(pi a), cos(pi a) for |a| < TRIGPI_TABLE_LIMIT: a = k/128 + f, k the
// nearest integer to 128 a, f exact
MPGOS_DF_HD void sincospi_table(dfloat a, dfloat* s, dfloat* c)
{
    const float k = f_rint(f_mul(a.hi, 128.0f));
    const dfloat f = two_sum(f_sub(a.hi, f_mul(k, 0x1p-7f)), a.lo);
    const dfloat r = f * dfloat(0x1.921fb6p+1f, -0x1.777a5cp-24f);   // pi
    sincos_table(r, static_cast<int>(k), s, c);
}

// MPGOS_DF_TRIG_BOUNDED forms: the table path on the argument, on zero in its
// place when it is outside the bound, and NaN selected for such arguments
MPGOS_DF_HD void sincos_bounded(dfloat a, dfloat* s, dfloat* c)
{
    const bool in = std::fabs(a.hi) < TRIG_TABLE_LIMIT;
    int k;
    const dfloat r = reduce_pio128(in ? a : dfloat(0.0f), k);
    dfloat ts, tc;
    sincos_table(r, k, &ts, &tc);
    const dfloat nan(f_nan(), f_nan());
    *s = in ? ts : nan;
    *c = in ? tc : nan;
}
MPGOS_DF_HD void sincospi_bounded(dfloat a, dfloat* s, dfloat* c)
{
    const bool in = std::fabs(a.hi) < TRIGPI_TABLE_LIMIT;
    dfloat ts, tc;
    sincospi_table(in ? a : dfloat(0.0f), &ts, &tc);
    const dfloat nan(f_nan(), f_nan());
    *s = in ? ts : nan;
    *c = in ? tc : nan;
}
}  // namespace detail

MPGOS_DF_HD dfloat sin(dfloat a)
{
    if constexpr (detail::TRIG_BOUNDED) {
        dfloat s, c;
        detail::sincos_bounded(a, &s, &c);
        return s;
    }
    if (std::fabs(a.hi) < detail::TRIG_TABLE_LIMIT) {
        int k;
        const dfloat r = detail::reduce_pio128(a, k);
        dfloat s, c;
        detail::sincos_table(r, k, &s, &c);
        return s;
    }
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
    if constexpr (detail::TRIG_BOUNDED) {
        dfloat s, c;
        detail::sincos_bounded(a, &s, &c);
        return c;
    }
    if (std::fabs(a.hi) < detail::TRIG_TABLE_LIMIT) {
        int k;
        const dfloat r = detail::reduce_pio128(a, k);
        dfloat s, c;
        detail::sincos_table(r, k, &s, &c);
        return c;
    }
    int q;
    const dfloat r = detail::reduce_pio2(a, q);
    switch (q) {
        case 0: return detail::cos_kernel(r);
        case 1: return -detail::sin_kernel(r);
        case 2: return -detail::cos_kernel(r);
        default: return detail::sin_kernel(r);
    }
}
// ---- exp, log and pow on the FP32 pipe ------------------------------------------
// exp: Cody & Waite reduction x = k ln2 + r (k the nearest integer to x/ln2,
// ln2 split into three floats so that every k * L_i is an exact double-float),
// r scaled by 2^-2 (|r/4| <= ln2/8), expm1 of the scaled value by its Taylor
// series (through r^5 in double-float by Horner's rule, the tail r^6..r^11
// in float, below 6e-10 of the result), squared back twice through
// (1 + e)^2 - 1 = e (e + 2), then 1 + e scaled by 2^k exactly.
// log: a = 2^E m with m in [sqrt(1/2), sqrt(2)); log m = 2 atanh(s) with
// s = (m - 1)/(m + 1), |s| <= 0.172, by its series s (2 + 2 z/3 + 2 z^2/5 ...)
// in z = s^2 (through z^5 in double-float, z^6..z^10 in float), so log m
// keeps double-float precision relative to itself; log a = E ln2 + log m.
// pow(a, b) = exp(b log a) for a > 0, with the integer part of b E taken out
// exactly: b log a = n ln2 + ((b E - n) ln2 + b log m), n the nearest integer
// to b log2 a and b E - n formed from the exact products b.hi E and b.lo E,
// so the reduced argument carries no rounding of the size of b E.
// Arguments these do not cover (|x| > 80 for exp, a <= 0, non-finite or
// subnormal a for log and pow) go through the FP64 functions.
namespace detail {
constexpr float LN2_1 = 0x1.62e430p-1f;
constexpr float LN2_2 = -0x1.05c610p-29f;
constexpr float LN2_3 = -0x1.950d88p-54f;
constexpr float INV_LN2 = 0x1.715476p+0f;

MPGOS_DF_HD float pow2i(int k)  // 2^k for -126 <= k <= 127
{
#if defined(__CUDA_ARCH__)
    return __int_as_float((k + 127) << 23);
#else
    return std::ldexp(1.0f, k);
#endif
}

// exp(x) - 1 for |x| <= ln2/8
MPGOS_DF_HD dfloat expm1_kernel(dfloat x)
{
    const float xf = x.hi;
    float tail = 1.0f / 39916800.0f;                    // 1/11!
    tail = f_fma(xf, tail, 1.0f / 3628800.0f);          // 1/10!
    tail = f_fma(xf, tail, 1.0f / 362880.0f);           // 1/9!
    tail = f_fma(xf, tail, 1.0f / 40320.0f);            // 1/8!
    tail = f_fma(xf, tail, 1.0f / 5040.0f);             // 1/7!
    tail = f_fma(xf, tail, 1.0f / 720.0f);              // 1/6!
    dfloat p = fma(x, dfloat(tail), dfloat(0x1.111112p-7f, -0x1.dddddep-32f));   // 1/5!
    p = fma(x, p, dfloat(0x1.555556p-5f, -0x1.555556p-30f));                      // 1/4!
    p = fma(x, p, dfloat(0x1.555556p-3f, -0x1.555556p-28f));                      // 1/3!
    p = fma(x, p, dfloat(0.5f));
    p = fma(x, p, dfloat(1.0f));
    return x * p;
}

// exp(r) 2^k for |r| <= ln2/2 + a little and an integer k in [-126, 127]
MPGOS_DF_HD dfloat exp_scaled(dfloat r, int k)
{
    dfloat e = expm1_kernel(dfloat(f_mul(r.hi, 0.25f), f_mul(r.lo, 0.25f)));
#pragma unroll
    for (int i = 0; i < 2; i++) {
        const dfloat t = two_sum(e.hi, 2.0f);
        e = e * quick_two_sum(t.hi, f_add(t.lo, e.lo));       // e (e + 2)
    }
    const dfloat s = quick_two_sum(1.0f, e.hi);                    // |e| < 1/2
    const dfloat v = quick_two_sum(s.hi, f_add(s.lo, e.lo));
    const float scale = pow2i(k);
    return dfloat(f_mul(v.hi, scale), f_mul(v.lo, scale));
}

// x - k ln2 for an integer-valued float k (|k| < 2^8)
MPGOS_DF_HD dfloat minus_k_ln2(dfloat x, float k)
{
    dfloat r = x - two_prod(k, LN2_1);
    r = r - two_prod(k, LN2_2);
    return r - two_prod(k, LN2_3);
}

// exp(x) for |x.hi| <= 80
MPGOS_DF_HD dfloat exp_reduced(dfloat x)
{
    const float k = f_rint(f_mul(x.hi, INV_LN2));
    return exp_scaled(minus_k_ln2(x, k), static_cast<int>(k));
}

// a = 2^E m, m in [sqrt(1/2), sqrt(2)), for a normal positive a.hi
MPGOS_DF_HD dfloat split_exponent(dfloat a, int& E)
{
#if defined(__CUDA_ARCH__)
    E = ((__float_as_int(a.hi) >> 23) & 0xff) - 127;
#else
    E = std::ilogb(a.hi);
#endif
    float f = pow2i(-E);
    if (f_mul(a.hi, f) > 1.41421356f) {
        E += 1;
        f = f_mul(f, 0.5f);
    }
    return dfloat(f_mul(a.hi, f), f_mul(a.lo, f));   // exact
}

// a / b with three quotient digits (the "accurate" division of the same
// source as the add; error ~2^-49 relative against ~2^-46 for operator/)
MPGOS_DF_HD dfloat div_accurate(dfloat a, dfloat b)
{
    const float rb = f_rcp(b.hi);
    const float q1 = f_mul(a.hi, rb);
    dfloat r = a - mul_f(b, q1);
    const float q2 = f_mul(r.hi, rb);
    r = r - mul_f(b, q2);
    const float q3 = f_mul(r.hi, rb);
    const dfloat q = quick_two_sum(q1, q2);
    return q + dfloat(q3);
}

// log m for m in [sqrt(1/2), sqrt(2)]
MPGOS_DF_HD dfloat log_reduced(dfloat m)
{
    const dfloat num = two_sum(f_sub(m.hi, 1.0f), m.lo);   // m - 1 (m.hi - 1 exact)
    const dfloat s = div_accurate(num, m + dfloat(1.0f));
    const dfloat z = s * s;
    const float zf = z.hi;
    float tail = 1.0f / 21.0f;
    tail = f_fma(zf, tail, 1.0f / 19.0f);
    tail = f_fma(zf, tail, 1.0f / 17.0f);
    tail = f_fma(zf, tail, 1.0f / 15.0f);
    tail = f_fma(zf, tail, 1.0f / 13.0f);
    dfloat p = fma(z, dfloat(tail), dfloat(0x1.745d18p-4f, -0x1.745d18p-29f));   // 1/11
    p = fma(z, p, dfloat(0x1.c71c72p-4f, -0x1.c71c72p-31f));                      // 1/9
    p = fma(z, p, dfloat(0x1.24924ap-3f, -0x1.b6db6ep-28f));                      // 1/7
    p = fma(z, p, dfloat(0x1.99999ap-3f, -0x1.99999ap-29f));                      // 1/5
    p = fma(z, p, dfloat(0x1.555556p-2f, -0x1.555556p-27f));                      // 1/3
    p = fma(z, p, dfloat(1.0f));
    const dfloat t = s * p;
    return dfloat(f_mul(t.hi, 2.0f), f_mul(t.lo, 2.0f));
}
}  // namespace detail

MPGOS_DF_HD dfloat exp(dfloat a)
{
    if (!(std::fabs(a.hi) <= 80.0f)) return dfloat(std::exp(static_cast<double>(a)));
    return detail::exp_reduced(a);
}

MPGOS_DF_HD dfloat log(dfloat a)
{
    if (!(a.hi >= 0x1p-126f && a.hi <= 0x1.fffffep+127f)) return dfloat(std::log(static_cast<double>(a)));
    int E;
    const dfloat m = detail::split_exponent(a, E);
    const dfloat l = detail::log_reduced(m);
    return detail::minus_k_ln2(l, -static_cast<float>(E));
}

MPGOS_DF_HD dfloat pow(dfloat a, dfloat b)
{
    if (!(a.hi >= 0x1p-126f && a.hi <= 0x1.fffffep+127f && std::fabs(b.hi) <= 0x1p+16f))
        return dfloat(std::pow(static_cast<double>(a), static_cast<double>(b)));
    int E;
    const dfloat m = detail::split_exponent(a, E);
    const dfloat bl = b * detail::log_reduced(m);          // b log m
    const float ef = static_cast<float>(E);
    const dfloat p = two_prod(b.hi, ef), q = two_prod(b.lo, ef);   // b E = p + q exactly
    const float n = f_rint(f_add(p.hi, f_mul(bl.hi, detail::INV_LN2)));   // ~ b log2 a
    if (!(std::fabs(n) <= 115.0f)) return dfloat(std::pow(static_cast<double>(a), static_cast<double>(b)));
    const dfloat g = add_accurate(add_accurate(two_sum(p.hi, -n), dfloat(p.lo)), q);   // b E - n
    const dfloat r = add_accurate(g * dfloat(detail::LN2_1, detail::LN2_2), bl);      // (b E - n) ln2 + b log m
    return detail::exp_scaled(r, static_cast<int>(n));
}
MPGOS_DF_HD dfloat pow(dfloat a, double b) { return pow(a, dfloat(b)); }
// integer powers by repeated squaring (|n| <= 64), others as above
MPGOS_DF_HD dfloat pow(dfloat a, int n)
{
    if (n < -64 || n > 64) return pow(a, dfloat(static_cast<float>(n)));
    unsigned m = static_cast<unsigned>(n < 0 ? -n : n);
    dfloat r(1.0f), base = a;
    while (m != 0) {
        if (m & 1u) r = r * base;
        m >>= 1;
        if (m != 0) base = base * base;
    }
    return n < 0 ? dfloat(1.0f) / r : r;
}
namespace detail {
// sin(r + q pi/2) and cos(r + q pi/2) from both kernels of r, selected without
// branches (lanes of a warp in different quadrants do not diverge)
MPGOS_DF_HD void sincos_quadrant(dfloat r, int q, dfloat* s, dfloat* c)
{
    const dfloat sk = sin_kernel(r), ck = cos_kernel(r);
    const bool odd = (q & 1) != 0;
    const dfloat ss = odd ? ck : sk, cc = odd ? sk : ck;
    *s = (q & 2) != 0 ? -ss : ss;
    *c = ((q + 1) & 2) != 0 ? -cc : cc;
}
}  // namespace detail

// sin and cos of one argument with one reduction
MPGOS_DF_HD void sincos(dfloat a, dfloat* s, dfloat* c)
{
    if constexpr (detail::TRIG_BOUNDED) {
        detail::sincos_bounded(a, s, c);
        return;
    }
    if (std::fabs(a.hi) < detail::TRIG_TABLE_LIMIT) {
        int k;
        const dfloat r = detail::reduce_pio128(a, k);
        detail::sincos_table(r, k, s, c);
        return;
    }
    int q;
    const dfloat r = detail::reduce_pio2(a, q);
    detail::sincos_quadrant(r, q, s, c);
}

// sin(pi a) and cos(pi a): a = k/128 + f with k the nearest integer to 128 a
// and |f| <= 1/256, f exact (a.hi - k/128 is exact by Sterbenz's lemma, the
// low part joins by two_sum), then the table path on pi f (|a| < 2^16; up to
// 2^22 the same with k/2 and both series kernels); no rounding grows with |a|.
MPGOS_DF_HD void sincospi(dfloat a, dfloat* s, dfloat* c)
{
    if constexpr (detail::TRIG_BOUNDED) {
        detail::sincospi_bounded(a, s, c);
        return;
    }
    if (std::fabs(a.hi) < detail::TRIGPI_TABLE_LIMIT) {
        detail::sincospi_table(a, s, c);
        return;
    }
    if (!(std::fabs(a.hi) < 0x1p+22f)) {   // beyond, a is an integer or half-integer multiple
        sincos(a * dfloat(0x1.921fb6p+1f, -0x1.777a5cp-24f), s, c);
        return;
    }
    const float k = f_rint(f_mul(a.hi, 2.0f));
    const dfloat f = two_sum(f_sub(a.hi, f_mul(k, 0.5f)), a.lo);
    const dfloat r = f * dfloat(0x1.921fb6p+1f, -0x1.777a5cp-24f);   // pi
    detail::sincos_quadrant(r, static_cast<int>(k) & 3, s, c);
}

}  // namespace df
}  // namespace mpgos

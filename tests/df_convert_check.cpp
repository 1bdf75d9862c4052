// CPU check of the integer-pipe conversions and the step-factor refinement of
// the precision-split solver (csrc/perthread/df_convert.cuh), compiled for the
// host by tests/test_dfloat_cpu.py. Prints one line per check: name, value
// (a count of failures or a maximum error, as stated per line).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>

#include "df_convert.cuh"

using mpgos::df::dfloat;

static long double val(dfloat a) { return (long double)a.hi + (long double)a.lo; }

static bool normalised(dfloat a)
{
    if (a.hi == 0.0f) return a.lo == 0.0f;
    const float up = std::nextafter(std::fabs(a.hi), INFINITY) - std::fabs(a.hi);
    return std::fabs(a.lo) <= 0.5f * up;
}

int main()
{
    std::mt19937_64 rng(20261204);
    std::uniform_real_distribution<double> u01(0.0, 1.0);

    // widen: bit-exact against the hardware conversion for normal floats,
    // infinities, zeros; subnormals to signed zero; NaN stays NaN
    long widen_bad = 0;
    for (int i = 0; i < 2000000; i++) {
        uint32_t b = static_cast<uint32_t>(rng());
        float f;
        std::memcpy(&f, &b, 4);
        const double w = mpgos::df::widen(f);
        if (std::isnan(f)) {
            widen_bad += !std::isnan(w);
        } else if (std::fpclassify(f) == FP_SUBNORMAL) {
            widen_bad += !(w == 0.0 && std::signbit(w) == std::signbit(f));
        } else {
            const double ref = static_cast<double>(f);
            widen_bad += std::memcmp(&w, &ref, 8) != 0;
        }
    }
    for (float f : {0.0f, -0.0f, INFINITY, -INFINITY, 1.0f, -1.0f, 0x1p-126f, 0x1.fffffep127f}) {
        const double w = mpgos::df::widen(f), ref = static_cast<double>(f);
        widen_bad += std::memcmp(&w, &ref, 8) != 0;
    }
    std::printf("widen_mismatches %ld\n", widen_bad);

    // split: |hi + lo - x| <= 2^-47 |x| (two truncations then renormalised),
    // normalised pairs, exactness for values a double-float holds exactly,
    // the exact fallback outside the fast path's range
    long split_bad = 0, split_norm = 0;
    long double split_err = 0;
    for (int i = 0; i < 2000000; i++) {
        const double mag = std::ldexp(1.0 + u01(rng), static_cast<int>(u01(rng) * 250.0) - 120);
        const double x = (rng() & 1) ? -mag : mag;
        const dfloat d = mpgos::df::split(x);
        if (!(std::fabs(x) >= 0x1p-74 && std::fabs(x) < 0x1p128)) continue;   // the fast path's range
        const long double e = std::fabs(val(d) - (long double)x) / std::fabs((long double)x);
        if (e > split_err) split_err = e;
        if (!normalised(d)) split_norm++;
        if (!(e <= 0x1p-47)) split_bad++;
    }
    for (double x : {0.0, -0.0, 1.0, -2.5, 10.0, 1e-30, 3e38, 1e300, -1e-300, 0x1p-74, 0x1p-75}) {
        const dfloat d = mpgos::df::split(x), r = dfloat(x);
        const bool in_fast = std::fabs(x) >= 0x1p-74 && std::fabs(x) < 0x1p128;
        if (!in_fast) split_bad += !(d.hi == r.hi && d.lo == r.lo);   // exact fallback
        if (x == 1.0 || x == -2.5 || x == 10.0) split_bad += !(d.hi == (float)x && d.lo == 0.0f);
    }
    std::printf("split_max_rel_err %.3Le\n", split_err);
    std::printf("split_bound_violations %ld\n", split_bad);
    std::printf("split_unnormalised %ld\n", split_norm);

    // to_double: the nearest double to hi + lo
    long td_bad = 0;
    for (int i = 0; i < 1000000; i++) {
        // lo stays a normal float (widen maps float subnormals to zero)
        const double x = std::ldexp(u01(rng) - 0.5, static_cast<int>(u01(rng) * 170.0) - 70);
        const dfloat d(x);
        const double t = mpgos::df::to_double(d), ref = static_cast<double>(d.hi) + static_cast<double>(d.lo);
        td_bad += std::memcmp(&t, &ref, 8) != 0;
    }
    std::printf("to_double_mismatches %ld\n", td_bad);

    // in_float_range: zero, non-finite and float's normal range in; the rest out
    long range_bad = 0;
    for (double x : {0.0, -0.0, 1.0, 0x1p-126, 0x1.fffffffffffffp127, (double)INFINITY, (double)NAN})
        range_bad += !mpgos::df::in_float_range(x);
    for (double x : {0x1p128, -0x1p128, 0x1.fffffffffffffp-127, 1e-300, 1e300})
        range_bad += mpgos::df::in_float_range(x);
    std::printf("range_mismatches %ld\n", range_bad);

    // step factor: R^(1/5) and R^(1/4) against long double, R = tol / err over
    // twelve decades, tol and err over wide magnitudes; error in ulp of the result
    long double root_ulp = 0;
    for (int i = 0; i < 1000000; i++) {
        const bool fifth = (i & 1) == 0;
        const double n = fifth ? 5.0 : 4.0;
        const double err = std::ldexp(1.0 + u01(rng), -static_cast<int>(u01(rng) * 60.0));
        const double R = std::pow(10.0, -6.0 + 12.0 * u01(rng));
        const double tol = err * R;
        const long double exact = std::pow((long double)tol / (long double)err, 1.0L / (long double)n);
        const float l2 = mpgos::df::log2_estimate(tol) - mpgos::df::log2_estimate(err);
        const float y0 = mpgos::df::root_estimate(l2, fifth);
        const double y = mpgos::df::root_refine(y0, tol, err, fifth);
        const long double ulp = std::ldexp(1.0L, std::ilogb(static_cast<double>(exact)) - 52);
        const long double e = std::fabs((long double)y - exact) / ulp;
        if (e > root_ulp) root_ulp = e;
    }
    std::printf("root_max_ulp %.3Lf\n", root_ulp);
    return 0;
}

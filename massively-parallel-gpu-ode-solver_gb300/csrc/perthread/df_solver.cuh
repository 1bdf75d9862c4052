// Per-thread RKCK45 solver in double-float arithmetic (DF_STAGE mode).
//
// Every per-instance quantity of one launch (state, stages, time, step,
// error, tolerances, event values) is a double-float (dfloat.cuh: ~48
// significant bits) evaluated on the FP32 pipe; FP64 is touched only to load
// the instance, to round back on write-back and for transcendental functions
// inside user hooks. The algorithm is the reference's loop
// (SingleSystem_PerThread_Solver.cuh:117-435) with the Cash-Karp stepper
// instantiated for dfloat, the reference's event handling and dense output,
// and this controller:
//   accept  iff err_i < max(rtol_i * max(|xn_i|, |x_i|), atol_i) for all i,
//           compared exactly in double-float;
//   factor  0.9 * (min_i tol_i / err_i)^(1/5) (1/4 after a rejection),
//           formed as 0.9 * exp2(min_i (log2 tol_i - log2 err_i) / 5) in FP32
//           from the leading floats (relative error ~1e-7, like FAST_CONTROL),
//           clamped to [shrink, grow]; the new step is dt * factor in
//           double-float, clamped to [min_dt, max_dt].
// The last step of the time domain ends exactly on its upper bound.
//
// Precision: the stage sums and the right-hand side carry ~4e-15 relative
// rounding per operation instead of 1.1e-16; against a local error of order
// the tolerance (1e-10 in the headline configuration) this moves the end
// states of non-chaotic instances by ~1e-13 relative and the embedded error
// estimate by ~1e-6 relative, both far inside the 1e-9 parity bar. The
// exponent range is float's (|values| within ~1e-38..3e38); systems whose
// states or parameters leave it must not use this mode; an instance that
// starts from such a value gets MPGOS_INSTANCE_RANGE.
#pragma once

#include "df_convert.cuh"

// The solver steps (begin, attempt, end) take the instance by reference from
// one call site each. Left out of line, the whole instance lives in local
// memory: the compiler does that for the Keller-Miksis kernels with the
// right-hand side inlined six times (448-592 bytes of stack per thread), not
// for the out-of-line twins that the autotuner picks for that system, nor for
// small systems. Forcing the steps inline removes it but multiplies the
// optimiser's time (a Keller-Miksis kernel set 57 s -> 356 s, the drop-in
// tutorial's translation unit 95 s -> over 20 min), so it is opt-in: define
// MPGOS_FORCE_INLINE_STEPS.
#ifndef MPGOS_STEP_INLINE
#if defined(MPGOS_FORCE_INLINE_STEPS)
#define MPGOS_STEP_INLINE __forceinline__
#else
#define MPGOS_STEP_INLINE
#endif
#endif

namespace mpgos {
namespace pt {

using df::dfloat;

struct DfOptions {
    dfloat initial_dt, max_dt, min_dt, min_dt_guard, dense_min_dt;
    double initial_dt64;
    float grow, shrink;
    int ndo, dense_freq;
    long long max_attempts;
};

template <class S>
struct DfInstance {
    static constexpr int SD = S::SD;
    long long i;
    dfloat td[2];
    dfloat x[SD];
    dfloat cp[AtLeastOne<S::NCP>::value];
    dfloat acc[AtLeastOne<S::NA>::value];
    int acci[AtLeastOne<S::NIA>::value];
    dfloat ga[AtLeastOne<S::NE>::value];
    dfloat t, dt, new_dt, dense_next;
    double td64[2];  // the FP64 time domain as loaded (written back unless a hook changed it)
    double t64;      // RK4: the time in FP64 (the reference's fixed-step time grid, step for step)
    int didx, skipped, terminate, udt, status, nacc, nrej;
    long long attempts;
};

// FP64 value of a double-float that started as the FP64 value `orig`: `orig`
// itself while unchanged (a double-float keeps 48 of its 53 bits, so the round
// trip alone would move it), else the double-float's value.
__device__ __forceinline__ double df_to_double(dfloat v, double orig)
{
    return (v == dfloat(orig)) ? orig : static_cast<double>(v);
}

template <class S>
struct DfStaged {
    dfloat* sp;
    int* spi;
    const dfloat* rtol;
    const dfloat* atol;
    const dfloat* etol;
    const int* edir;
};

// Controller of DF_STAGE (see the file comment).
// The system's right-hand side in double-float: inlined, or (OUTLINE, the
// MODE_OUTLINE_RHS kernels) one out-of-line function whose code is in the
// kernel once instead of once per stage. Large right-hand sides (the
// Keller-Miksis system's pow, sin, cos and divisions in double-float)
// inlined six times per step overflow the instruction cache, and the warps
// then wait on instruction fetch more than on anything else; a call costs a
// few instructions and the arrays it passes by address.
template <int SD, class P>
__device__ __noinline__ void df_rhs_outlined(int tid, int nt, P* F, P* X, P T, P* cp, P* sp, int* spi, P* acc,
                                             int* acci)
{
    PerThread_OdeFunction(tid, nt, F, X, T, cp, sp, spi, acc, acci);
}

template <int SD, bool OUTLINE, class P>
__device__ __forceinline__ void df_rhs(int tid, int nt, P* F, P* X, P T, P* cp, P* sp, int* spi, P* acc, int* acci)
{
    if constexpr (OUTLINE) df_rhs_outlined<SD, P>(tid, nt, F, X, T, cp, sp, spi, acc, acci);
    else PerThread_OdeFunction(tid, nt, F, X, T, cp, sp, spi, acc, acci);
}

// Cash-Karp 4(5) step in double-float: the scheme of step_rkck45
// (SingleSystem_PerThread_ExplicitRungeKutta_Steppers.cuh:121-289, same
// coefficients and stage order). Each stage sum sum_j a_j k_j is accumulated
// unnormalised (df::prod_sum: 12 FP32 operations per term after the first)
// and applied as X = x + dt * sum in one renormalising step. The embedded
// error estimate dt |sum_j e_j k_j| + 1e-18 is accumulated the same way and
// delivered in FP32: it cancels down to ~tol of terms of size |k| dt, so its
// double-float rounding is already ~1e-6 of it at tol 1e-10 and the FP32
// rounding of the result (6e-8) adds nothing the controller could see.
template <int SD, bool OUTLINE>
__device__ __forceinline__ void step_rkck45_df(int tid, int nt, dfloat t, dfloat dt, dfloat* x, dfloat* xn,
                                               float* err, int& finite, dfloat* cp, dfloat* sp, int* spi,
                                               dfloat* acc, int* acci)
{
    using df::fma;
    using df::prod_sum;
    using df::prod_sum_add;
    using df::prod_sum_axpy;
    using df::prod_sum_start;
    dfloat X[SD];
    dfloat k1[SD], k2[SD], k3[SD], k4[SD], k5[SD], k6[SD];

    df_rhs<SD, OUTLINE>(tid, nt, k1, x, t, cp, sp, spi, acc, acci);

#pragma unroll
    for (int i = 0; i < SD; i++) X[i] = prod_sum_axpy(dt, prod_sum_start(dfloat(1.0 / 5.0), k1[i]), x[i]);
    df_rhs<SD, OUTLINE>(tid, nt, k2, X, fma(dt, dfloat(1.0 / 5.0), t), cp, sp, spi, acc, acci);

#pragma unroll
    for (int i = 0; i < SD; i++) {
        prod_sum s = prod_sum_start(dfloat(3.0 / 40.0), k1[i]);
        prod_sum_add(s, dfloat(9.0 / 40.0), k2[i]);
        X[i] = prod_sum_axpy(dt, s, x[i]);
    }
    df_rhs<SD, OUTLINE>(tid, nt, k3, X, fma(dt, dfloat(3.0 / 10.0), t), cp, sp, spi, acc, acci);

#pragma unroll
    for (int i = 0; i < SD; i++) {
        prod_sum s = prod_sum_start(dfloat(3.0 / 10.0), k1[i]);
        prod_sum_add(s, dfloat(-9.0 / 10.0), k2[i]);
        prod_sum_add(s, dfloat(6.0 / 5.0), k3[i]);
        X[i] = prod_sum_axpy(dt, s, x[i]);
    }
    df_rhs<SD, OUTLINE>(tid, nt, k4, X, fma(dt, dfloat(3.0 / 5.0), t), cp, sp, spi, acc, acci);

#pragma unroll
    for (int i = 0; i < SD; i++) {
        prod_sum s = prod_sum_start(dfloat(-11.0 / 54.0), k1[i]);
        prod_sum_add(s, dfloat(5.0 / 2.0), k2[i]);
        prod_sum_add(s, dfloat(-70.0 / 27.0), k3[i]);
        prod_sum_add(s, dfloat(35.0 / 27.0), k4[i]);
        X[i] = prod_sum_axpy(dt, s, x[i]);
    }
    df_rhs<SD, OUTLINE>(tid, nt, k5, X, t + dt, cp, sp, spi, acc, acci);

#pragma unroll
    for (int i = 0; i < SD; i++) {
        prod_sum s = prod_sum_start(dfloat(1631.0 / 55296.0), k1[i]);
        prod_sum_add(s, dfloat(175.0 / 512.0), k2[i]);
        prod_sum_add(s, dfloat(575.0 / 13824.0), k3[i]);
        prod_sum_add(s, dfloat(44275.0 / 110592.0), k4[i]);
        prod_sum_add(s, dfloat(253.0 / 4096.0), k5[i]);
        X[i] = prod_sum_axpy(dt, s, x[i]);
    }
    df_rhs<SD, OUTLINE>(tid, nt, k6, X, fma(dt, dfloat(7.0 / 8.0), t), cp, sp, spi, acc, acci);

#pragma unroll
    for (int i = 0; i < SD; i++) {
        prod_sum s = prod_sum_start(dfloat(37.0 / 378.0), k1[i]);
        prod_sum_add(s, dfloat(250.0 / 621.0), k3[i]);
        prod_sum_add(s, dfloat(125.0 / 594.0), k4[i]);
        prod_sum_add(s, dfloat(512.0 / 1771.0), k6[i]);
        xn[i] = prod_sum_axpy(dt, s, x[i]);
        prod_sum e = prod_sum_start(dfloat(37.0 / 378.0 - 2825.0 / 27648.0), k1[i]);
        prod_sum_add(e, dfloat(250.0 / 621.0 - 18575.0 / 48384.0), k3[i]);
        prod_sum_add(e, dfloat(125.0 / 594.0 - 13525.0 / 55296.0), k4[i]);
        prod_sum_add(e, dfloat(0.0 - 277.0 / 14336.0), k5[i]);
        prod_sum_add(e, dfloat(512.0 / 1771.0 - 1.0 / 4.0), k6[i]);
        err[i] = fmaf(dt.hi, fabsf(e.h + e.l), 1e-18f);
        // finiteness on the exponent bits (integer pipe; no conversion to double)
        if ((__float_as_uint(xn[i].hi) & 0x7f800000u) == 0x7f800000u ||
            (__float_as_uint(err[i]) & 0x7f800000u) == 0x7f800000u)
            finite = 0;
    }
}

// Step-size control of the double-float solver
// (SingleSystem_PerThread_ExplicitRungeKutta_ErrorControllers.cuh:23-85 in
// structure): tolerance max(rtol max(|xn|, |x|), atol) and the accept test in
// FP32 on the leading floats (their rounding, ~6e-8, is far below the error
// estimate's own), factor 0.9 (tol/err)^(1/5 or 1/4) through FP32 log2/exp2.
// Classic RK4 step in double-float (SingleSystem_PerThread_ExplicitRungeKutta_Steppers.cuh:6-117:
// x + dt (k1 + 2 k2 + 2 k3 + k4) / 6), stage sums as unnormalised product sums.
template <int SD, bool OUTLINE>
__device__ __forceinline__ void step_rk4_df(int tid, int nt, dfloat t, dfloat dt, dfloat* x, dfloat* xn, int& finite,
                                            dfloat* cp, dfloat* sp, int* spi, dfloat* acc, int* acci)
{
    using df::prod_sum;
    using df::prod_sum_add;
    using df::prod_sum_axpy;
    using df::prod_sum_start;
    dfloat X[SD], k1[SD], k2[SD], k3[SD], k4[SD];
    const dfloat half(0.5);
    const dfloat th = df::fma(dt, half, t);
    df_rhs<SD, OUTLINE>(tid, nt, k1, x, t, cp, sp, spi, acc, acci);
#pragma unroll
    for (int i = 0; i < SD; i++) X[i] = prod_sum_axpy(dt, prod_sum_start(half, k1[i]), x[i]);
    df_rhs<SD, OUTLINE>(tid, nt, k2, X, th, cp, sp, spi, acc, acci);
#pragma unroll
    for (int i = 0; i < SD; i++) X[i] = prod_sum_axpy(dt, prod_sum_start(half, k2[i]), x[i]);
    df_rhs<SD, OUTLINE>(tid, nt, k3, X, th, cp, sp, spi, acc, acci);
#pragma unroll
    for (int i = 0; i < SD; i++) X[i] = prod_sum_axpy(dt, prod_sum{k3[i].hi, k3[i].lo}, x[i]);
    df_rhs<SD, OUTLINE>(tid, nt, k4, X, t + dt, cp, sp, spi, acc, acci);
#pragma unroll
    for (int i = 0; i < SD; i++) {
        prod_sum s = prod_sum_start(dfloat(1.0 / 6.0), k1[i]);
        prod_sum_add(s, dfloat(1.0 / 3.0), k2[i]);
        prod_sum_add(s, dfloat(1.0 / 3.0), k3[i]);
        prod_sum_add(s, dfloat(1.0 / 6.0), k4[i]);
        xn[i] = prod_sum_axpy(dt, s, x[i]);
        if ((__float_as_uint(xn[i].hi) & 0x7f800000u) == 0x7f800000u) finite = 0;
    }
}

template <int SD>
__device__ __forceinline__ void control_rkck45_df(const DfOptions& o, dfloat dt, const dfloat* x, const dfloat* xn,
                                                  const float* err, const dfloat* rtol, const dfloat* atol,
                                                  int& update, int& finite, int& terminate, dfloat& new_dt,
                                                  int& status)
{
    float lr = INFINITY;
#pragma unroll
    for (int i = 0; i < SD; i++) {
        const float tol = fmaxf(rtol[i].hi * fmaxf(fabsf(xn[i].hi), fabsf(x[i].hi)), atol[i].hi);
        update = update && (err[i] < tol);
        lr = fminf(lr, __log2f(tol) - __log2f(err[i]));
    }
    const float expo = (update == 1) ? 0.2f : 0.25f;
    float q = 0.9f * exp2f(fminf(fmaxf(lr * expo, -120.0f), 120.0f));
    if (finite == 0) {
        q      = o.shrink;
        update = 0;
        if (dt < o.min_dt_guard) {
            terminate = 1;
            status |= MPGOS_INSTANCE_NONFINITE;
        }
    } else if (dt < o.min_dt_guard) {
        update = 1;
        status |= MPGOS_INSTANCE_MINIMUM_STEP;
    }
    q      = fminf(q, o.grow);
    q      = fmaxf(q, o.shrink);
    new_dt = df::mul_f(dt, q);
    new_dt = df::fmin(new_dt, o.max_dt);
    new_dt = df::fmax(new_dt, o.min_dt);
}

template <int SD>
__device__ __forceinline__ void dense_store_df(long long i, long long nt, int store, int& didx, int ndo,
                                               double* dtime, double* dstate, dfloat t, const dfloat* x,
                                               int& skipped, dfloat& dense_next, dfloat dense_min_dt, dfloat upper)
{
    if (store == 1) {
        if (didx < ndo) {
            dtime[i + static_cast<long long>(didx) * nt] = static_cast<double>(t);
            long long idx = i + static_cast<long long>(didx) * nt * SD;
#pragma unroll
            for (int c = 0; c < SD; c++) {
                dstate[idx] = static_cast<double>(x[c]);
                idx += nt;
            }
            didx++;
        }
        skipped    = 0;
        dense_next = df::fmin(t + dense_min_dt, upper);
    } else {
        skipped++;
    }
}

template <class S, int MODE, int ALG = MPGOS_RKCK45>
struct DfSolver {
    static constexpr int SD = S::SD, NCP = S::NCP, NE = S::NE, NA = S::NA, NIA = S::NIA;
    static constexpr bool RK4 = (ALG == MPGOS_RK4);
    static constexpr bool PERSISTENT = (MODE & MPGOS_MODE_PERSISTENT) != 0;
    static constexpr bool RECORD = (MODE & MODE_RECORD) != 0;
    static constexpr bool OUTLINE = (MODE & MODE_OUTLINE_RHS) != 0;
    using Inst = DfInstance<S>;

    // MPGOS_INSTANCE_RANGE when a value the instance starts from (time domain,
    // time, state, control parameters, accessories, tolerances, event
    // tolerances) lies outside float's exponent range, which double-float
    // arithmetic keeps: there it would overflow or lose its low part.
    __device__ MPGOS_STEP_INLINE static int range_status(long long i, const Args<double>& a)
    {
        const long long nt = a.nt;
        bool ok = df::in_float_range(a.t[i]);
#pragma unroll
        for (int k = 0; k < 2; k++) ok = ok && df::in_float_range(a.td[i + k * nt]);
#pragma unroll
        for (int k = 0; k < SD; k++)
            ok = ok && df::in_float_range(a.x[i + k * nt]) && df::in_float_range(a.rtol[k]) &&
                 df::in_float_range(a.atol[k]);
#pragma unroll
        for (int k = 0; k < NCP; k++) ok = ok && df::in_float_range(a.cp[i + k * nt]);
#pragma unroll
        for (int k = 0; k < NA; k++) ok = ok && df::in_float_range(a.acc[i + k * nt]);
#pragma unroll
        for (int k = 0; k < NE; k++) ok = ok && df::in_float_range(a.etol[k]);
        return ok ? 0 : MPGOS_INSTANCE_RANGE;
    }

    __device__ MPGOS_STEP_INLINE static void begin(Inst& s, long long i, const Args<double>& a, const DfStaged<S>& g,
                                 const DfOptions& o)
    {
        const long long nt = a.nt;
        s.i = i;
#pragma unroll
        for (int k = 0; k < 2; k++) {
            s.td64[k] = a.td[i + k * nt];
            s.td[k]   = dfloat(s.td64[k]);
        }
#pragma unroll
        for (int k = 0; k < SD; k++) s.x[k] = dfloat(a.x[i + k * nt]);
#pragma unroll
        for (int k = 0; k < NCP; k++) s.cp[k] = dfloat(a.cp[i + k * nt]);
#pragma unroll
        for (int k = 0; k < NA; k++) s.acc[k] = dfloat(a.acc[i + k * nt]);
#pragma unroll
        for (int k = 0; k < NIA; k++) s.acci[k] = a.acci[i + k * nt];
        s.t          = dfloat(a.t[i]);
        s.dt         = o.initial_dt;
        s.new_dt     = o.initial_dt;
        s.didx       = a.didx[i];
        s.skipped    = 0;
        s.terminate  = 0;
        s.udt        = 0;
        s.status     = range_status(i, a);
        s.nacc       = 0;
        s.nrej       = 0;
        s.attempts   = 0;
        s.dense_next = s.t;
        const int ti = static_cast<int>(i), nti = static_cast<int>(nt);
        PerThread_Initialization(ti, nti, s.didx, s.t, s.dt, s.td, s.x, s.cp, g.sp, g.spi, s.acc, s.acci);
        if constexpr (RK4) s.t64 = df_to_double(s.t, (s.t == s.td[0]) ? s.td64[0] : a.t[i]);
        if (NE > 0)
            PerThread_EventFunction(ti, nti, s.ga, s.t, s.dt, s.td, s.x, s.cp, g.sp, g.spi, s.acc, s.acci);
        if (o.ndo > 0)
            dense_store_df<SD>(i, nt, 1, s.didx, o.ndo, a.dtime, a.dstate, s.t, s.x, s.skipped, s.dense_next,
                               o.dense_min_dt, s.td[1]);
        if constexpr (RECORD) {
            // checkpoint 0: the state the first step starts from
            a.tape.ckpt_t[i] = RK4 ? s.t64 : static_cast<double>(s.t);
#pragma unroll
            for (int d = 0; d < SD; d++) a.tape.ckpt_x[d * nt + i] = static_cast<double>(s.x[d]);
        }
    }

    __device__ MPGOS_STEP_INLINE static void attempt(Inst& s, const Args<double>& a, const DfStaged<S>& g, const DfOptions& o)
    {
        if (s.attempts >= o.max_attempts) {
            s.status |= MPGOS_INSTANCE_ATTEMPT_LIMIT;
            s.terminate = 1;
            return;
        }
        s.attempts++;
        const int ti = static_cast<int>(s.i), nti = static_cast<int>(a.nt);
        int update = 1, finite = 1, end_reached = 0;
        dfloat xn[SD];
        double dt64 = 0.0;
        if constexpr (RK4) {
            // fixed step on the FP64 time grid of the reference (step counts and
            // the clamped end step match it exactly); stages in double-float
            dt64 = o.initial_dt64;
            const double rem64 = s.td64[1] - s.t64;
            if (dt64 > rem64) {
                dt64        = rem64;
                end_reached = 1;
            }
            s.dt = dfloat(dt64);
            step_rk4_df<SD, OUTLINE>(ti, nti, s.t, s.dt, s.x, xn, finite, s.cp, g.sp, g.spi, s.acc, s.acci);
            if (finite == 0) {
                s.terminate = 1;
                s.status |= MPGOS_INSTANCE_NONFINITE;
            }
            s.new_dt = o.initial_dt;
        } else {
            float err[SD];
            s.dt = s.new_dt;
            const dfloat rem = s.td[1] - s.t;
            if (s.dt > rem) {
                s.dt        = rem;
                end_reached = 1;
            }
            step_rkck45_df<SD, OUTLINE>(ti, nti, s.t, s.dt, s.x, xn, err, finite, s.cp, g.sp, g.spi, s.acc, s.acci);
            control_rkck45_df<SD>(o, s.dt, s.x, xn, err, g.rtol, g.atol, update, finite, s.terminate, s.new_dt,
                                  s.status);
        }

        dfloat gn[AtLeastOne<NE>::value];
        if (NE > 0) {
            PerThread_EventFunction(ti, nti, gn, s.t + s.dt, s.dt, s.td, xn, s.cp, g.sp, g.spi, s.acc, s.acci);
            event_step_control<NE, dfloat>(update, s.terminate, s.ga, gn, g.etol, g.edir, s.dt, s.new_dt, o.min_dt,
                                           s.status);
        }

        if (update == 1) {
            s.nacc++;
            if constexpr (RK4) {
                s.t64 += dt64;
                s.t = dfloat(s.t64);
            } else {
                s.t = (end_reached == 1) ? s.td[1] : s.t + s.dt;
            }
#pragma unroll
            for (int k = 0; k < SD; k++) s.x[k] = xn[k];
            PerThread_ActionAfterSuccessfulTimeStep(ti, nti, s.udt, s.t, s.dt, s.td, s.x, s.cp, g.sp, g.spi,
                                                    s.acc, s.acci);
            if constexpr (RK4) {
                if (!(s.t == dfloat(s.t64))) s.t64 = static_cast<double>(s.t);  // a hook moved the time
            }
            if (NE > 0) {
                for (int e = 0; e < NE; e++) {
                    if (event_detected<dfloat>(s.ga[e], gn[e], g.etol[e], g.edir[e]))
                        PerThread_ActionAfterEventDetection(ti, nti, e, s.udt, s.t, s.dt, s.td, s.x, s.cp, g.sp,
                                                            g.spi, s.acc, s.acci);
                }
                PerThread_EventFunction(ti, nti, gn, s.t, s.dt, s.td, s.x, s.cp, g.sp, g.spi, s.acc, s.acci);
#pragma unroll
                for (int e = 0; e < NE; e++) s.ga[e] = gn[e];
            }
            if (o.ndo > 0) {
                const int store = dense_condition<dfloat>(s.t, s.dense_next, s.didx, s.skipped, end_reached, s.udt,
                                                          o.ndo, o.dense_freq);
                dense_store_df<SD>(s.i, a.nt, store, s.didx, o.ndo, a.dtime, a.dstate, s.t, s.x, s.skipped,
                                   s.dense_next, o.dense_min_dt, s.td[1]);
            }
            if constexpr (RECORD) {
                // frozen step size of accepted step nacc, checkpoint every seg steps
                const int k = s.nacc - 1;
                if (k < a.tape.max_steps) {
                    // RK4: the FP64 step and time themselves
                    a.tape.dt[static_cast<long long>(k) * a.nt + s.i] = RK4 ? dt64 : static_cast<double>(s.dt);
                    if (s.nacc % a.tape.seg == 0) {
                        const long long c = s.nacc / a.tape.seg;
                        a.tape.ckpt_t[c * a.nt + s.i] = RK4 ? s.t64 : static_cast<double>(s.t);
#pragma unroll
                        for (int d = 0; d < SD; d++)
                            a.tape.ckpt_x[(c * SD + d) * a.nt + s.i] = static_cast<double>(s.x[d]);
                    }
                } else {
                    s.status |= MPGOS_INSTANCE_TAPE_OVERFLOW;
                }
            }
            if ((end_reached == 1) || (s.udt == 1)) s.terminate = 1;
        } else {
            s.nrej++;
        }
    }

    __device__ MPGOS_STEP_INLINE static void end(Inst& s, const Args<double>& a, const DfStaged<S>& g)
    {
        const long long i = s.i, nt = a.nt;
        const int ti = static_cast<int>(i), nti = static_cast<int>(nt);
        PerThread_Finalization(ti, nti, s.didx, s.t, s.dt, s.td, s.x, s.cp, g.sp, g.spi, s.acc, s.acci);
#pragma unroll
        for (int k = 0; k < 2; k++) a.td[i + k * nt] = df_to_double(s.td[k], s.td64[k]);
        // values the run left unchanged keep their FP64 bits (df_to_double)
#pragma unroll
        for (int k = 0; k < SD; k++) a.x[i + k * nt] = df_to_double(s.x[k], a.x[i + k * nt]);
#pragma unroll
        for (int k = 0; k < NCP; k++) a.cp[i + k * nt] = df_to_double(s.cp[k], a.cp[i + k * nt]);
#pragma unroll
        for (int k = 0; k < NA; k++) a.acc[i + k * nt] = df_to_double(s.acc[k], a.acc[i + k * nt]);
#pragma unroll
        for (int k = 0; k < NIA; k++) a.acci[i + k * nt] = s.acci[k];
        if constexpr (RK4) a.t[i] = s.t64;  // the FP64 time grid
        else a.t[i] = df_to_double(s.t, s.td64[1]);  // ends exactly on the FP64 upper bound
        a.didx[i] = s.didx;
        if (a.status) a.status[i] = s.status;
        if (a.n_acc) a.n_acc[i] = s.nacc;
        if (a.n_rej) a.n_rej[i] = s.nrej;
        if constexpr (RECORD) a.tape.n_steps[i] = s.nacc;
    }
};

// A plugin may define MPGOS_DF_MIN_BLOCKS, the minimum resident blocks of
// MPGOS_MAX_BLOCK threads the DF_STAGE kernels are compiled for (a register
// cap: 65536 / (MPGOS_MAX_BLOCK x this)); left undefined, ptxas chooses.
#ifdef MPGOS_DF_MIN_BLOCKS
#define MPGOS_DF_BOUNDS __launch_bounds__(MPGOS_MAX_BLOCK, MPGOS_DF_MIN_BLOCKS)
#else
#define MPGOS_DF_BOUNDS __launch_bounds__(MPGOS_MAX_BLOCK)
#endif

// DF_STAGE kernel: same launch contract as perthread_kernel<S, ALG, double, *>.
template <class S, int MODE, int ALG = MPGOS_RKCK45>
__global__ void MPGOS_DF_BOUNDS perthread_df_kernel(Args<double> a)
{
    using Sv = DfSolver<S, MODE, ALG>;
    constexpr int SD = S::SD, NSP = S::NSP, NISP = S::NISP, NE = S::NE;
    extern __shared__ __align__(16) unsigned char mpgos_dyn_smem[];
    __shared__ dfloat s_rtol[SD];
    __shared__ dfloat s_atol[SD];
    __shared__ dfloat s_etol[AtLeastOne<NE>::value];
    __shared__ int s_edir[AtLeastOne<NE>::value];
    __shared__ dfloat s_sp[AtLeastOne<NSP>::value];
    int* dyn_spi = reinterpret_cast<int*>(mpgos_dyn_smem + sizeof(double) * NSP);

    for (int k = threadIdx.x; k < SD; k += blockDim.x) {
        s_rtol[k] = dfloat(a.rtol[k]);
        s_atol[k] = dfloat(a.atol[k]);
    }
    for (int k = threadIdx.x; k < NE; k += blockDim.x) {
        s_etol[k] = dfloat(a.etol[k]);
        s_edir[k] = a.edir[k];
    }
    for (int k = threadIdx.x; k < NSP; k += blockDim.x) s_sp[k] = dfloat(a.sp[k]);
    if (a.prefer_shared)
        for (int k = threadIdx.x; k < NISP; k += blockDim.x) dyn_spi[k] = a.spi[k];
    __syncthreads();

    DfStaged<S> g;
    g.sp   = s_sp;
    g.spi  = a.prefer_shared ? dyn_spi : const_cast<int*>(a.spi);
    g.rtol = s_rtol;
    g.atol = s_atol;
    g.etol = s_etol;
    g.edir = s_edir;

    DfOptions o;
    o.initial_dt   = dfloat(a.o.initial_dt);
    o.initial_dt64 = a.o.initial_dt;
    o.max_dt       = dfloat(a.o.max_dt);
    o.min_dt       = dfloat(a.o.min_dt);
    o.min_dt_guard = dfloat(a.o.min_dt_guard);
    o.dense_min_dt = dfloat(a.o.dense_min_dt);
    o.grow         = static_cast<float>(a.o.grow);
    o.shrink       = static_cast<float>(a.o.shrink);
    o.ndo          = a.o.ndo;
    o.dense_freq   = a.o.dense_freq;
    o.max_attempts = a.o.max_attempts;

    const long long total = static_cast<long long>(gridDim.x) * blockDim.x;
    long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    using Next = Solver<S, MPGOS_RKCK45, double, MODE & ~(MODE_RECONVERGE | MODE_OUTLINE_RHS)>;
    if constexpr ((MODE & MODE_RECONVERGE) != 0) {
        // one ballot over the integrating lanes per iteration reconverges the
        // warp once per step attempt (as in perthread_kernel)
        unsigned live = __ballot_sync(__activemask(), i < a.n_active);
        if (i >= a.n_active) return;
        // one call site each of begin, attempt and end (all inlined: an
        // out-of-line call would put the instance in local memory)
        typename Sv::Inst s;
        bool loaded = false;
        while (true) {
            bool stop = false;
            if (!loaded || s.terminate) {
                if (loaded) {
                    Sv::end(s, a, g);
                    i = Next::next_index(a, total, i);
                }
                loaded = true;
                if (i >= a.n_active) stop = true;
                else Sv::begin(s, instance_at(a, i), a, g, o);
            }
            if (!stop) Sv::attempt(s, a, g, o);
            live = __ballot_sync(live, !stop);
            if (stop) break;
        }
    } else {
        if (i >= a.n_active) return;
        typename Sv::Inst s;
        bool loaded = false;
        while (true) {
            if (!loaded || s.terminate) {
                if (loaded) {
                    Sv::end(s, a, g);
                    i = Next::next_index(a, total, i);
                    if (i >= a.n_active) break;
                }
                loaded = true;
                Sv::begin(s, instance_at(a, i), a, g, o);
            }
            Sv::attempt(s, a, g, o);
        }
    }
}

}  // namespace pt
}  // namespace mpgos

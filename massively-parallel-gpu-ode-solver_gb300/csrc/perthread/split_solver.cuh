// Per-thread solver in the precision split (SPLIT mode).
//
// The right-hand side and the stage sums run in double-float (dfloat.cuh:
// ~48 significant bits on the FP32 pipe); everything else of the reference
// scheme runs in FP64:
//   * the state x, the time t, the step dt and the time domain are FP64
//     registers, advanced in FP64: x_new = x + dt * sum_j b_j k_j
//     (one FP64 fused multiply-add on the stage sum rounded to FP64) and
//     t += dt, as in SingleSystem_PerThread_Solver.cuh:338-339 and
//     SingleSystem_PerThread_ExplicitRungeKutta_Steppers.cuh:275-278;
//   * the error estimate dt |sum_j e_j k_j| + 1e-18 (Steppers.cuh:280-285),
//     the tolerances max(rtol max(|x_new|, |x|), atol), the accept test and
//     the minimum ratio R = min(1e30, min_i tol_i/err_i) are FP64 quantities;
//     comparisons of these non-negative doubles run exactly on their bit
//     patterns or, outside a narrow band where FP32 log2 estimates decide
//     them, as FP64 products (control_rkck45_split); the FP64 values are
//     formed only where a decision or the factor needs them (the estimate of
//     log2 err comes from the double-float error sum directly);
//   * the step factor 0.9 R^(1/5) (0.9 R^(1/4) after a rejection,
//     ErrorControllers.cuh:44-53) is evaluated to FP64 accuracy (a few ulp):
//     an FP32 estimate corrected in FP64 by a second-order binomial series
//     (df::root_refine); where the clamp to [shrink, grow] decides the factor
//     alone the estimate suffices;
//   * the new step dt * q, its clamps, the end-of-domain clamp, the event
//     functions, the secant step toward an event
//     (SingleSystem_PerThread_EventHandling.cuh:5-44), event detection, dense
//     output and every user hook other than the right-hand side run in FP64 on
//     the FP64 state (the hooks instantiated for double).
// The right-hand side (PerThread_OdeFunction instantiated for dfloat) sees
// double-float copies of the state, time, control parameters, shared
// parameters and accessories; the state copy is refreshed after every
// accepted step, the others after the hooks that change them. Conversions
// between the formats run on the integer pipe (df_convert.cuh).
//
// Why: on GB300 an FP64 operation costs ~60 FP32 operations of issue
// throughput. The reference step spends ~270 FP64 instructions per attempt on
// the Lorenz system; here ~30 remain in FP64 and the ~100 stage operations
// move to the FP32 pipe, where the double-float arithmetic overlaps the FP64
// pipe.
//
// Range: the right-hand side computes with float's exponent range. Instances
// whose state, time, parameters or accessories leave it (|v| >= 2^128 or
// 0 < |v| < 2^-126) get MPGOS_INSTANCE_RANGE and keep integrating with those
// values converted as far as the format allows.
#pragma once

#include "df_convert.cuh"
#include "ck_tableau.cuh"

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

template <class S>
struct SplitInstance {
    static constexpr int SD = S::SD;
    long long i;
    double td[2];
    double x[SD];
    dfloat xd[SD];
    double cp[AtLeastOne<S::NCP>::value];
    dfloat cpd[AtLeastOne<S::NCP>::value];
    double acc[AtLeastOne<S::NA>::value];
    dfloat accd[AtLeastOne<S::NA>::value];
    int acci[AtLeastOne<S::NIA>::value];
    double ga[AtLeastOne<S::NE>::value];
    double t, dt, new_dt, dense_next, rem;
    dfloat tdf;
    int didx, skipped, terminate, udt, status, nacc, nrej;
    long long attempts;
};

template <class S>
struct SplitStaged {
    double* sp;     // FP64 shared parameters (shared memory or global) for the FP64 hooks
    dfloat* spd;    // double-float copy for the right-hand side
    int* spi;
    const double* rtol;
    const double* atol;
    const float* lrtol;   // log2 of the tolerances
    const float* latol;
    const double* etol;
    const int* edir;
    float shrink_f, grow_f;   // step-factor limits as floats
};

// double -> double-float with the range guard
__device__ __forceinline__ bool finite_float(float f) { return (__float_as_uint(f) & 0x7f800000u) != 0x7f800000u; }

__device__ __forceinline__ dfloat split_guarded(double v, int& status)
{
    if (!df::in_float_range(v)) status |= MPGOS_INSTANCE_RANGE;
    return df::split(v);
}

// Cash-Karp 4(5) step of the split: stage sums and right-hand sides in
// double-float (the sums and their order as step_rkck45_df), then the FP64
// update and error estimate from the two sums rounded to FP64.
template <int SD, bool OUTLINE>
__device__ __forceinline__ void step_rkck45_split(int tid, int nt, dfloat t, double dt, dfloat dtd, const double* x,
                                                  dfloat* xd, double* xn, df::prod_sum* esum, int& finite,
                                                  dfloat* cp, dfloat* sp, int* spi, dfloat* acc, int* acci)
{
    using df::fma;
    using df::prod_sum;
    using df::prod_sum_add;
    using df::prod_sum_axpy;
    using df::prod_sum_start;
    dfloat X[SD];
    dfloat k1[SD], k2[SD], k3[SD], k4[SD], k5[SD], k6[SD];

    df_rhs<SD, OUTLINE>(tid, nt, k1, xd, t, cp, sp, spi, acc, acci);

#pragma unroll
    for (int i = 0; i < SD; i++) X[i] = prod_sum_axpy(dtd, prod_sum_start(dfloat(1.0 / 5.0), k1[i]), xd[i]);
    df_rhs<SD, OUTLINE>(tid, nt, k2, X, fma(dtd, dfloat(1.0 / 5.0), t), cp, sp, spi, acc, acci);

#pragma unroll
    for (int i = 0; i < SD; i++) {
        prod_sum s = prod_sum_start(dfloat(3.0 / 40.0), k1[i]);
        prod_sum_add(s, dfloat(9.0 / 40.0), k2[i]);
        X[i] = prod_sum_axpy(dtd, s, xd[i]);
    }
    df_rhs<SD, OUTLINE>(tid, nt, k3, X, fma(dtd, dfloat(3.0 / 10.0), t), cp, sp, spi, acc, acci);

#pragma unroll
    for (int i = 0; i < SD; i++) {
        prod_sum s = prod_sum_start(dfloat(3.0 / 10.0), k1[i]);
        prod_sum_add(s, dfloat(-9.0 / 10.0), k2[i]);
        prod_sum_add(s, dfloat(6.0 / 5.0), k3[i]);
        X[i] = prod_sum_axpy(dtd, s, xd[i]);
    }
    df_rhs<SD, OUTLINE>(tid, nt, k4, X, fma(dtd, dfloat(3.0 / 5.0), t), cp, sp, spi, acc, acci);

#pragma unroll
    for (int i = 0; i < SD; i++) {
        prod_sum s = prod_sum_start(dfloat(-11.0 / 54.0), k1[i]);
        prod_sum_add(s, dfloat(5.0 / 2.0), k2[i]);
        prod_sum_add(s, dfloat(-70.0 / 27.0), k3[i]);
        prod_sum_add(s, dfloat(35.0 / 27.0), k4[i]);
        X[i] = prod_sum_axpy(dtd, s, xd[i]);
    }
    df_rhs<SD, OUTLINE>(tid, nt, k5, X, t + dtd, cp, sp, spi, acc, acci);

#pragma unroll
    for (int i = 0; i < SD; i++) {
        prod_sum s = prod_sum_start(dfloat(1631.0 / 55296.0), k1[i]);
        prod_sum_add(s, dfloat(175.0 / 512.0), k2[i]);
        prod_sum_add(s, dfloat(575.0 / 13824.0), k3[i]);
        prod_sum_add(s, dfloat(44275.0 / 110592.0), k4[i]);
        prod_sum_add(s, dfloat(253.0 / 4096.0), k5[i]);
        X[i] = prod_sum_axpy(dtd, s, xd[i]);
    }
    df_rhs<SD, OUTLINE>(tid, nt, k6, X, fma(dtd, dfloat(7.0 / 8.0), t), cp, sp, spi, acc, acci);

#pragma unroll
    for (int i = 0; i < SD; i++) {
        prod_sum s = prod_sum_start(dfloat(37.0 / 378.0), k1[i]);
        prod_sum_add(s, dfloat(250.0 / 621.0), k3[i]);
        prod_sum_add(s, dfloat(125.0 / 594.0), k4[i]);
        prod_sum_add(s, dfloat(512.0 / 1771.0), k6[i]);
        prod_sum e = prod_sum_start(dfloat(37.0 / 378.0 - 2825.0 / 27648.0), k1[i]);
        prod_sum_add(e, dfloat(250.0 / 621.0 - 18575.0 / 48384.0), k3[i]);
        prod_sum_add(e, dfloat(125.0 / 594.0 - 13525.0 / 55296.0), k4[i]);
        prod_sum_add(e, dfloat(0.0 - 277.0 / 14336.0), k5[i]);
        prod_sum_add(e, dfloat(512.0 / 1771.0 - 1.0 / 4.0), k6[i]);
        // the unnormalised sum h + l rounded once to FP64; the error sum is
        // kept as its pair (its FP64 estimate dt |h + l| + 1e-18 is formed
        // by the controller where a decision needs it)
        const double sb = df::widen(s.h) + df::widen(s.l);
        xn[i]   = __fma_rn(dt, sb, x[i]);
        esum[i] = e;
        if (!finite_bits(xn[i]) || !finite_float(e.h) || !finite_float(e.l)) finite = 0;
    }
}

// The same step with the six stages as one loop (weights from constant
// memory, the right-hand side inlined once instead of six times); every
// stage input, the solution sum and the error sum accumulate their terms in
// the order above (term j added when k_j is known), so the values are those
// of the straight-line form. A plugin selects it with MPGOS_SPLIT_STAGE_LOOP.
template <int SD, bool OUTLINE>
__device__ __forceinline__ void step_rkck45_split_loop(int tid, int nt, dfloat t, double dt, dfloat dtd,
                                                       const double* x, dfloat* xd, double* xn, df::prod_sum* esum,
                                                       int& finite, dfloat* cp, dfloat* sp, int* spi, dfloat* acc,
                                                       int* acci)
{
    using df::prod_sum;
    using df::prod_sum_add;
    using df::prod_sum_axpy;
    prod_sum in[5][SD], sb[SD], se[SD];
#pragma unroll
    for (int i = 0; i < SD; i++) {
#pragma unroll
        for (int r = 0; r < 5; r++) in[r][i] = prod_sum{0.0f, 0.0f};
        sb[i] = prod_sum{0.0f, 0.0f};
        se[i] = prod_sum{0.0f, 0.0f};
    }
#pragma unroll 1
    for (int st = 0; st < 6; st++) {
        dfloat X[SD], k[SD];
#pragma unroll
        for (int i = 0; i < SD; i++) {
            prod_sum a = in[0][i];
#pragma unroll
            for (int r = 1; r < 5; r++)
                if (st == r + 1) a = in[r][i];
            X[i] = st == 0 ? xd[i] : prod_sum_axpy(dtd, a, xd[i]);
        }
        const float2 c = CK_C[st];
        const dfloat T = st == 0 ? t : (st == 4 ? t + dtd : df::fma(dtd, dfloat(c.x, c.y), t));
        df_rhs<SD, OUTLINE>(tid, nt, k, X, T, cp, sp, spi, acc, acci);
#pragma unroll
        for (int r = 0; r < 5; r++) {
            if (r + 1 > st) {
                const float2 a = CK_A[r + 1][st];
#pragma unroll
                for (int i = 0; i < SD; i++) prod_sum_add(in[r][i], dfloat(a.x, a.y), k[i]);
            }
        }
        const float2 b = CK_B[st], e = CK_E[st];
        if (b.x != 0.0f) {
#pragma unroll
            for (int i = 0; i < SD; i++) prod_sum_add(sb[i], dfloat(b.x, b.y), k[i]);
        }
        if (e.x != 0.0f) {
#pragma unroll
            for (int i = 0; i < SD; i++) prod_sum_add(se[i], dfloat(e.x, e.y), k[i]);
        }
    }
#pragma unroll
    for (int i = 0; i < SD; i++) {
        const double b = df::widen(sb[i].h) + df::widen(sb[i].l);
        xn[i]   = __fma_rn(dt, b, x[i]);
        esum[i] = se[i];
        if (!finite_bits(xn[i]) || !finite_float(se[i].h) || !finite_float(se[i].l)) finite = 0;
    }
}

// Classic RK4 step of the split (Steppers.cuh:6-117): stages in
// double-float, x_new = x + (dt/6) (k1 + 2 k2 + 2 k3 + k4) in FP64 with
// dt/6 formed as the reference forms it.
template <int SD, bool OUTLINE>
__device__ __forceinline__ void step_rk4_split(int tid, int nt, dfloat t, double dt, dfloat dtd, const double* x,
                                               dfloat* xd, double* xn, int& finite, dfloat* cp, dfloat* sp, int* spi,
                                               dfloat* acc, int* acci)
{
    using df::prod_sum;
    using df::prod_sum_add;
    using df::prod_sum_axpy;
    using df::prod_sum_start;
    dfloat X[SD], k1[SD], k2[SD], k3[SD], k4[SD];
    const dfloat half(0.5);
    const dfloat th = df::fma(dtd, half, t);
    df_rhs<SD, OUTLINE>(tid, nt, k1, xd, t, cp, sp, spi, acc, acci);
#pragma unroll
    for (int i = 0; i < SD; i++) X[i] = prod_sum_axpy(dtd, prod_sum_start(half, k1[i]), xd[i]);
    df_rhs<SD, OUTLINE>(tid, nt, k2, X, th, cp, sp, spi, acc, acci);
#pragma unroll
    for (int i = 0; i < SD; i++) X[i] = prod_sum_axpy(dtd, prod_sum_start(half, k2[i]), xd[i]);
    df_rhs<SD, OUTLINE>(tid, nt, k3, X, th, cp, sp, spi, acc, acci);
#pragma unroll
    for (int i = 0; i < SD; i++) X[i] = prod_sum_axpy(dtd, prod_sum{k3[i].hi, k3[i].lo}, xd[i]);
    df_rhs<SD, OUTLINE>(tid, nt, k4, X, t + dtd, cp, sp, spi, acc, acci);
    const double sixth = static_cast<double>(1.0 / 6.0) * dt;
#pragma unroll
    for (int i = 0; i < SD; i++) {
        prod_sum s = prod_sum_start(dfloat(1.0), k1[i]);
        prod_sum_add(s, dfloat(2.0), k2[i]);
        prod_sum_add(s, dfloat(2.0), k3[i]);
        prod_sum_add(s, dfloat(1.0), k4[i]);
        xn[i] = __fma_rn(sixth, df::widen(s.h) + df::widen(s.l), x[i]);
        if (!finite_bits(xn[i])) finite = 0;
    }
}

// Width (log2 units) of the band around a decision inside which the FP32
// log2 estimates (good to ~4e-6) do not decide and the exact FP64 comparison
// runs instead.
constexpr float SPLIT_BAND = 1e-4f;

// The FP64 error estimate dt |sum_j e_j k_j| + 1e-18 of Steppers.cuh:280-285
// from the double-float error sum h + l (rounded once to FP64).
__device__ __forceinline__ double split_error(double dt, float h, float l)
{
    return __fma_rn(dt, fabs(df::widen(h) + df::widen(l)), 1e-18);
}

// FP32 estimate of log2 of that error from the float sum of the pair
// (correctly rounded) and the leading float of dt (within 2^-23 of it):
// relative error below 2^-21, far inside the 1e-4 decision band
__device__ __forceinline__ float split_log2_error(float dt_hi, float h, float l)
{
    return __log2f(fmaf(dt_hi, fabsf(h + l), 1e-18f));
}

// The exact FP64 forms behind the estimates, out of line: they run only
// inside the band (a rare branch, not predicated into every attempt).
static __device__ __noinline__ double split_tolerance(double rtol, double atol, long long mag_bits)
{
    return from_bits(max_bits(bits_of(rtol * from_bits(mag_bits)), bits_of(atol)));
}

static __device__ __noinline__ int split_accepts(double rtol, double atol, long long mag_bits, double dt, float h,
                                                 float l)
{
    return bits_of(split_error(dt, h, l)) < bits_of(split_tolerance(rtol, atol, mag_bits));
}

// tol_a / err_a < tol_b / err_b for positive values, by cross multiplication
static __device__ __noinline__ bool split_ratio_less(double tol_a, double err_a, double tol_b, double err_b)
{
    return tol_a * err_b < tol_b * err_a;
}

// log2(1e30): the reference starts the minimum ratio at 1e30
// (ErrorControllers.cuh:38), so R = min(1e30, min_i tol_i / err_i)
constexpr float SPLIT_LOG2_RATIO_CAP = 99.65784f;

// Step-size control of the split (ErrorControllers.cuh:23-85) on FP64 values
// with exact decisions and an FP64-accurate factor:
//   accept iff err_i < tol_i = max(rtol_i max(|xn_i|, |x_i|), atol_i) for
//   every i, err_i = dt |h_i + l_i| + 1e-18 the FP64 error estimate of the
//   double-float error sum: decided by d_i = log2 tol_i - log2 err_i (FP32
//   estimates, with log2 tol_i = max(log2 rtol_i + log2 m_i, log2 atol_i) and
//   log2 err_i from the float sum of the pair) outside a 1e-4 band, by the
//   FP64 comparison inside it;
//   R = min(1e30, min_i tol_i / err_i): the component of the smallest d_i,
//   ties inside the band settled by cross-multiplied FP64 products; tol and
//   err formed in FP64 for that component only;
//   q = 0.9 R^(1/5) (1/4 after a rejection) to FP64 accuracy
//   (df::root_refine), where the clamp to [shrink, grow] does not decide it
//   from the estimate alone; new step dt q clamped to [min_dt, max_dt].
// lrtol / latol: log2 of the tolerances (per block, FP32); shrink_f /
// grow_f: the limits as floats; dt_hi: the leading float of dt.
template <int SD>
__device__ __forceinline__ void control_rkck45_split(const Options<double>& o, float shrink_f, float grow_f,
                                                     double dt, float dt_hi, const double* x, const double* xn,
                                                     const df::prod_sum* esum, const double* rtol,
                                                     const double* atol, const float* lrtol, const float* latol,
                                                     int& update, int& finite, int& terminate, double& new_dt,
                                                     int& status)
{
    float dmin = INFINITY;
    long long mag_m = 0;
    float eh_m = 0.0f, el_m = 0.0f;
    double err_m = 1.0, rtol_m = 0.0, atol_m = 0.0, tol_m = 0.0;
    bool exact_known = false;   // tol_m and err_m already formed (a tie was settled)
#pragma unroll
    for (int i = 0; i < SD; i++) {
        const long long mag = max_bits(abs_bits(xn[i]), abs_bits(x[i]));
        const float lt = fmaxf(lrtol[i] + df::log2_estimate(from_bits(mag)), latol[i]);
        const float d  = lt - split_log2_error(dt_hi, esum[i].h, esum[i].l);
        int accept_i;
        if (d > SPLIT_BAND) accept_i = 1;
        else if (d < -SPLIT_BAND) accept_i = 0;
        else accept_i = split_accepts(rtol[i], atol[i], mag, dt, esum[i].h, esum[i].l);
        update = update && accept_i;
        bool take, settled = false;
        if (i == 0 || d < dmin - SPLIT_BAND) {
            take = true;
        } else if (d > dmin + SPLIT_BAND) {
            take = false;
        } else {
            // a tie within the estimates' error: compare the ratios exactly;
            // tol_m and err_m are then those of whichever component wins
            const double tol_i = split_tolerance(rtol[i], atol[i], mag);
            const double err_i = split_error(dt, esum[i].h, esum[i].l);
            if (!exact_known) {
                tol_m = split_tolerance(rtol_m, atol_m, mag_m);
                err_m = split_error(dt, eh_m, el_m);
            }
            take    = split_ratio_less(tol_i, err_i, tol_m, err_m);
            settled = true;
            if (take) {
                tol_m = tol_i;
                err_m = err_i;
            }
        }
        exact_known = settled || (!take && exact_known);
        if (take) {
            dmin   = d;
            mag_m  = mag;
            eh_m   = esum[i].h;
            el_m   = esum[i].l;
            rtol_m = rtol[i];
            atol_m = atol[i];
        }
    }
    if (!exact_known) {
        tol_m = from_bits(max_bits(bits_of(rtol_m * from_bits(mag_m)), bits_of(atol_m)));
        err_m = split_error(dt, eh_m, el_m);
    }
    // the reference's initial ratio 1e30 caps R
    if (dmin > SPLIT_LOG2_RATIO_CAP + SPLIT_BAND ||
        (!(dmin < SPLIT_LOG2_RATIO_CAP - SPLIT_BAND) && !split_ratio_less(tol_m, err_m, 1e30, 1.0))) {
        dmin  = SPLIT_LOG2_RATIO_CAP;
        tol_m = 1e30;
        err_m = 1.0;
    }

    const bool fifth = (update == 1);
    const float y0   = df::root_estimate(dmin, fifth);
    const float qf   = 0.9f * y0;
    double q;
    if (qf > shrink_f * (1.0f - 1e-5f) && qf < grow_f * (1.0f + 1e-5f))
        q = 0.9 * df::root_refine(y0, tol_m, err_m, fifth);
    else
        q = df::widen(qf);   // outside the limits by more than the estimate's error: the clamp decides

    const long long dtb    = bits_of(dt);
    const long long guardb = bits_of(o.min_dt_guard);
    if (finite == 0) {
        q      = o.shrink;
        update = 0;
        if (dtb < guardb) {
            terminate = 1;
            status |= MPGOS_INSTANCE_NONFINITE;
        }
    } else if (dtb < guardb) {
        update = 1;
        status |= MPGOS_INSTANCE_MINIMUM_STEP;
    }
    long long qb = min_bits(bits_of(q), bits_of(o.grow));
    qb = max_bits(qb, bits_of(o.shrink));
    const double nd = dt * from_bits(qb);
    new_dt = from_bits(max_bits(min_bits(bits_of(nd), bits_of(o.max_dt)), bits_of(o.min_dt)));
}

template <class S, int MODE, int ALG = MPGOS_RKCK45>
struct SplitSolver {
    static constexpr int SD = S::SD, NCP = S::NCP, NE = S::NE, NA = S::NA, NIA = S::NIA;
    static constexpr bool RK4 = (ALG == MPGOS_RK4);
    static constexpr bool OUTLINE = (MODE & MODE_OUTLINE_RHS) != 0;
    static constexpr bool RECORD = (MODE & MODE_RECORD) != 0;
    using Inst = SplitInstance<S>;

    // double-float copies the right-hand side reads: all of them when an
    // instance is loaded
    __device__ MPGOS_STEP_INLINE static void refresh(Inst& s)
    {
#pragma unroll
        for (int k = 0; k < SD; k++) s.xd[k] = split_guarded(s.x[k], s.status);
#pragma unroll
        for (int k = 0; k < NCP; k++) s.cpd[k] = split_guarded(s.cp[k], s.status);
#pragma unroll
        for (int k = 0; k < NA; k++) s.accd[k] = split_guarded(s.acc[k], s.status);
        s.tdf = split_guarded(s.t, s.status);
        s.rem = s.td[1] - s.t;
    }

    // after an attempt: the parameters and accessories the FP64 hooks
    // changed (compared with their values when the attempt began; where the
    // hooks never write them the compiler removes the test)
    __device__ MPGOS_STEP_INLINE static void refresh_changed(Inst& s, const double* cp0, const double* acc0)
    {
#pragma unroll
        for (int k = 0; k < NCP; k++)
            if (bits_of(s.cp[k]) != bits_of(cp0[k])) s.cpd[k] = split_guarded(s.cp[k], s.status);
#pragma unroll
        for (int k = 0; k < NA; k++)
            if (bits_of(s.acc[k]) != bits_of(acc0[k])) s.accd[k] = split_guarded(s.acc[k], s.status);
    }

    __device__ MPGOS_STEP_INLINE static void begin(Inst& s, long long i, const Args<double>& a, const SplitStaged<S>& g)
    {
        const long long nt = a.nt;
        s.i = i;
#pragma unroll
        for (int k = 0; k < 2; k++) s.td[k] = a.td[i + k * nt];
#pragma unroll
        for (int k = 0; k < SD; k++) s.x[k] = a.x[i + k * nt];
#pragma unroll
        for (int k = 0; k < NCP; k++) s.cp[k] = a.cp[i + k * nt];
#pragma unroll
        for (int k = 0; k < NA; k++) s.acc[k] = a.acc[i + k * nt];
#pragma unroll
        for (int k = 0; k < NIA; k++) s.acci[k] = a.acci[i + k * nt];
        s.t          = a.t[i];
        s.dt         = a.o.initial_dt;
        s.new_dt     = a.o.initial_dt;
        s.didx       = a.didx[i];
        s.skipped    = 0;
        s.terminate  = 0;
        s.udt        = 0;
        s.status     = 0;
        s.nacc       = 0;
        s.nrej       = 0;
        s.attempts   = 0;
        s.dense_next = s.t;
#pragma unroll
        for (int k = 0; k < S::NSP; k++)   // the shared parameters' double-float copies
            if (!df::in_float_range(g.sp[k])) s.status |= MPGOS_INSTANCE_RANGE;
        const int ti = static_cast<int>(i), nti = static_cast<int>(nt);
        PerThread_Initialization(ti, nti, s.didx, s.t, s.dt, s.td, s.x, s.cp, g.sp, g.spi, s.acc, s.acci);
        if (NE > 0)
            PerThread_EventFunction(ti, nti, s.ga, s.t, s.dt, s.td, s.x, s.cp, g.sp, g.spi, s.acc, s.acci);
        if (a.o.ndo > 0)
            dense_store<SD, double>(i, nt, 1, s.didx, a.o.ndo, a.dtime, a.dstate, s.t, s.x, s.skipped, s.dense_next,
                                    a.o.dense_min_dt, s.td[1]);
        refresh(s);
        if constexpr (RECORD) {
            // checkpoint 0: the state the first step starts from
            a.tape.ckpt_t[i] = s.t;
#pragma unroll
            for (int d = 0; d < SD; d++) a.tape.ckpt_x[d * nt + i] = s.x[d];
        }
    }

    __device__ MPGOS_STEP_INLINE static void attempt(Inst& s, const Args<double>& a, const SplitStaged<S>& g)
    {
        const Options<double>& o = a.o;
        if (s.attempts >= o.max_attempts) {
            s.status |= MPGOS_INSTANCE_ATTEMPT_LIMIT;
            s.terminate = 1;
            return;
        }
        s.attempts++;
        const int ti = static_cast<int>(s.i), nti = static_cast<int>(a.nt);
        int update = 1, finite = 1, end_reached = 0;
        double xn[SD];
        double cp0[AtLeastOne<NCP>::value], acc0[AtLeastOne<NA>::value];
#pragma unroll
        for (int k = 0; k < NCP; k++) cp0[k] = s.cp[k];
#pragma unroll
        for (int k = 0; k < NA; k++) acc0[k] = s.acc[k];
        s.dt = s.new_dt;
        // end of the time domain; positive steps compare with the remainder
        // exactly as int64 bit patterns (also when the remainder is negative)
        if (bits_of(s.dt) > bits_of(s.rem)) {
            s.dt        = s.rem;
            end_reached = 1;
        }
        const dfloat dtd = df::split(s.dt);
        if constexpr (RK4) {
            step_rk4_split<SD, OUTLINE>(ti, nti, s.tdf, s.dt, dtd, s.x, s.xd, xn, finite, s.cpd, g.spd, g.spi,
                                        s.accd, s.acci);
            control_rk4<double>(o, finite, s.terminate, s.new_dt, s.status);
        } else {
            df::prod_sum esum[SD];
#ifdef MPGOS_SPLIT_STAGE_LOOP
            step_rkck45_split_loop<SD, OUTLINE>(ti, nti, s.tdf, s.dt, dtd, s.x, s.xd, xn, esum, finite, s.cpd,
                                                g.spd, g.spi, s.accd, s.acci);
#else
            step_rkck45_split<SD, OUTLINE>(ti, nti, s.tdf, s.dt, dtd, s.x, s.xd, xn, esum, finite, s.cpd, g.spd,
                                           g.spi, s.accd, s.acci);
#endif
            control_rkck45_split<SD>(o, g.shrink_f, g.grow_f, s.dt, dtd.hi, s.x, xn, esum, g.rtol, g.atol, g.lrtol,
                                     g.latol, update, finite, s.terminate, s.new_dt, s.status);
        }

        double gn[AtLeastOne<NE>::value];
        if (NE > 0) {
            PerThread_EventFunction(ti, nti, gn, s.t + s.dt, s.dt, s.td, xn, s.cp, g.sp, g.spi, s.acc, s.acci);
            event_step_control<NE, double>(update, s.terminate, s.ga, gn, g.etol, g.edir, s.dt, s.new_dt, o.min_dt,
                                           s.status);
        }

        if (update == 1) {
            s.nacc++;
            s.t += s.dt;
#pragma unroll
            for (int k = 0; k < SD; k++) s.x[k] = xn[k];
            PerThread_ActionAfterSuccessfulTimeStep(ti, nti, s.udt, s.t, s.dt, s.td, s.x, s.cp, g.sp, g.spi, s.acc,
                                                    s.acci);
            if (NE > 0) {
                for (int e = 0; e < NE; e++) {
                    if (event_detected<double>(s.ga[e], gn[e], g.etol[e], g.edir[e]))
                        PerThread_ActionAfterEventDetection(ti, nti, e, s.udt, s.t, s.dt, s.td, s.x, s.cp, g.sp,
                                                            g.spi, s.acc, s.acci);
                }
                PerThread_EventFunction(ti, nti, gn, s.t, s.dt, s.td, s.x, s.cp, g.sp, g.spi, s.acc, s.acci);
#pragma unroll
                for (int e = 0; e < NE; e++) s.ga[e] = gn[e];
            }
            if (o.ndo > 0) {
                const int store = dense_condition<double>(s.t, s.dense_next, s.didx, s.skipped, end_reached, s.udt,
                                                          o.ndo, o.dense_freq);
                dense_store<SD, double>(s.i, a.nt, store, s.didx, o.ndo, a.dtime, a.dstate, s.t, s.x, s.skipped,
                                        s.dense_next, o.dense_min_dt, s.td[1]);
            }
#pragma unroll
            for (int k = 0; k < SD; k++) s.xd[k] = split_guarded(s.x[k], s.status);
            s.tdf = split_guarded(s.t, s.status);
            s.rem = s.td[1] - s.t;
            if constexpr (RECORD) {
                // frozen step size of accepted step nacc, checkpoint every seg steps
                const int k = s.nacc - 1;
                if (k < a.tape.max_steps) {
                    a.tape.dt[static_cast<long long>(k) * a.nt + s.i] = s.dt;
                    if (s.nacc % a.tape.seg == 0) {
                        const long long c = s.nacc / a.tape.seg;
                        a.tape.ckpt_t[c * a.nt + s.i] = s.t;
#pragma unroll
                        for (int d = 0; d < SD; d++) a.tape.ckpt_x[(c * SD + d) * a.nt + s.i] = s.x[d];
                    }
                } else {
                    s.status |= MPGOS_INSTANCE_TAPE_OVERFLOW;
                }
            }
            if ((end_reached == 1) || (s.udt == 1)) s.terminate = 1;
        } else {
            s.nrej++;
        }
        refresh_changed(s, cp0, acc0);
    }

    __device__ MPGOS_STEP_INLINE static void end(Inst& s, const Args<double>& a, const SplitStaged<S>& g)
    {
        const long long i = s.i, nt = a.nt;
        const int ti = static_cast<int>(i), nti = static_cast<int>(nt);
        PerThread_Finalization(ti, nti, s.didx, s.t, s.dt, s.td, s.x, s.cp, g.sp, g.spi, s.acc, s.acci);
#pragma unroll
        for (int k = 0; k < 2; k++) a.td[i + k * nt] = s.td[k];
#pragma unroll
        for (int k = 0; k < SD; k++) a.x[i + k * nt] = s.x[k];
#pragma unroll
        for (int k = 0; k < NCP; k++) a.cp[i + k * nt] = s.cp[k];
#pragma unroll
        for (int k = 0; k < NA; k++) a.acc[i + k * nt] = s.acc[k];
#pragma unroll
        for (int k = 0; k < NIA; k++) a.acci[i + k * nt] = s.acci[k];
        a.t[i]    = s.t;
        a.didx[i] = s.didx;
        if (a.status) a.status[i] = s.status;
        if (a.n_acc) a.n_acc[i] = s.nacc;
        if (a.n_rej) a.n_rej[i] = s.nrej;
        if constexpr (RECORD) a.tape.n_steps[i] = s.nacc;
    }
};

// A plugin may define MPGOS_SPLIT_MIN_BLOCKS, the minimum resident blocks of
// MPGOS_MAX_BLOCK threads the SPLIT kernels are compiled for (a register cap:
// 65536 / (MPGOS_MAX_BLOCK x this)). Left undefined, ptxas chooses: stating 1
// explicitly lets it use more registers (119 instead of 94 on Lorenz, two
// fewer resident blocks of 64, 5 % slower).
#ifdef MPGOS_SPLIT_MIN_BLOCKS
#define MPGOS_SPLIT_BOUNDS __launch_bounds__(MPGOS_MAX_BLOCK, MPGOS_SPLIT_MIN_BLOCKS)
#else
#define MPGOS_SPLIT_BOUNDS __launch_bounds__(MPGOS_MAX_BLOCK)
#endif

// SPLIT kernel: same launch contract as perthread_kernel<S, ALG, double, *>.
template <class S, int MODE, int ALG = MPGOS_RKCK45>
__global__ void MPGOS_SPLIT_BOUNDS perthread_split_kernel(Args<double> a)
{
    using Sv = SplitSolver<S, MODE, ALG>;
    constexpr int SD = S::SD, NSP = S::NSP, NISP = S::NISP, NE = S::NE;
    extern __shared__ __align__(16) unsigned char mpgos_dyn_smem[];
    __shared__ double s_rtol[SD];
    __shared__ double s_atol[SD];
    __shared__ float s_lrtol[SD];
    __shared__ float s_latol[SD];
    __shared__ double s_etol[AtLeastOne<NE>::value];
    __shared__ int s_edir[AtLeastOne<NE>::value];
    __shared__ dfloat s_spd[AtLeastOne<NSP>::value];
    double* dyn_sp = reinterpret_cast<double*>(mpgos_dyn_smem);
    int* dyn_spi   = reinterpret_cast<int*>(mpgos_dyn_smem + sizeof(double) * NSP);

    for (int k = threadIdx.x; k < SD; k += blockDim.x) {
        s_rtol[k]  = a.rtol[k];
        s_atol[k]  = a.atol[k];
        s_lrtol[k] = df::log2_estimate(a.rtol[k]);
        s_latol[k] = df::log2_estimate(a.atol[k]);
    }
    for (int k = threadIdx.x; k < NE; k += blockDim.x) {
        s_etol[k] = a.etol[k];
        s_edir[k] = a.edir[k];
    }
    for (int k = threadIdx.x; k < NSP; k += blockDim.x) s_spd[k] = df::split(a.sp[k]);
    if (a.prefer_shared) {
        for (int k = threadIdx.x; k < NSP; k += blockDim.x) dyn_sp[k] = a.sp[k];
        for (int k = threadIdx.x; k < NISP; k += blockDim.x) dyn_spi[k] = a.spi[k];
    }
    __syncthreads();

    SplitStaged<S> g;
    g.sp       = a.prefer_shared ? dyn_sp : const_cast<double*>(a.sp);
    g.spd      = s_spd;
    g.spi      = a.prefer_shared ? dyn_spi : const_cast<int*>(a.spi);
    g.rtol     = s_rtol;
    g.atol     = s_atol;
    g.lrtol    = s_lrtol;
    g.latol    = s_latol;
    g.etol     = s_etol;
    g.edir     = s_edir;
    g.shrink_f = static_cast<float>(a.o.shrink);
    g.grow_f   = static_cast<float>(a.o.grow);

    const long long total = static_cast<long long>(gridDim.x) * blockDim.x;
    long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    using Next = Solver<S, MPGOS_RKCK45, double, MODE & MPGOS_MODE_PERSISTENT>;
    if constexpr ((MODE & MODE_RECONVERGE) != 0) {
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
                else Sv::begin(s, instance_at(a, i), a, g);
            }
            if (!stop) Sv::attempt(s, a, g);
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
                Sv::begin(s, instance_at(a, i), a, g);
            }
            Sv::attempt(s, a, g);
        }
    }
}

}  // namespace pt
}  // namespace mpgos

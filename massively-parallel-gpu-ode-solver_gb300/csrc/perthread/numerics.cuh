// Numerical building blocks of the per-thread solver: Runge-Kutta steppers,
// step-size controllers, event step control and dense-output storage.
//
// Each block states the reference routine whose behaviour it reproduces. The
// stage sums keep the reference's grouping and operand order (and the
// static_cast<Precision>(a/b) coefficient form) on purpose: with the same
// compiler the PLAIN kernel then rounds exactly as the reference kernel does,
// which is what makes bit-level parity checks possible.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#if __has_include("mpgos.h")
#include "mpgos.h"
#else
#include "../../../include/mpgos.h"
#endif

namespace mpgos {
namespace pt {

template <int N> struct AtLeastOne { static constexpr int value = N > 0 ? N : 1; };

// Device-side view of the adjoint tape (mpgos_pt_tape in mpgos.h).
struct Tape {
    int seg;
    int max_steps;
    double* dt;      // [max_steps][NT]
    double* ckpt_x;  // [max_steps/seg + 1][SD][NT]
    double* ckpt_t;  // [max_steps/seg + 1][NT]
    int* n_steps;    // [NT]
};

// Kernel-internal mode bit: the forward launch records the adjoint tape.
constexpr int MODE_RECORD = 8;
// Internal mode bit of the per-thread kernels (MPGOS_WARP_RECONVERGE): the
// integrating lanes of a warp reconverge once per step attempt.
constexpr int MODE_RECONVERGE = 32;
// Internal mode bit of the double-float kernels (MPGOS_OUTLINE_RHS): the
// right-hand side is one out-of-line function instead of inlined per stage.
constexpr int MODE_OUTLINE_RHS = 64;

// Solver options in the kernel's precision (Struct_SolverOptions of
// SingleSystem_PerThread_Interface.cuh:105-115 plus the extensions).
template <class P>
struct Options {
    P initial_dt, max_dt, min_dt, grow, shrink, dense_min_dt;
    P min_dt_guard;        // MinimumTimeStep * 1.01, the threshold of the controllers
    int dense_freq;
    int ndo;
    long long max_attempts;
};

// ---------------------------------------------------------------------------
// Bit-level helpers for FP64 values. On GB300 the FP64 pipe is the scarce
// resource (about 1/64 of the FP32 rate), so the FAST_CONTROL path moves
// comparisons, absolute values, maxima and the step-factor arithmetic to the
// integer and FP32 pipes. For non-negative finite doubles the IEEE bit
// patterns order like signed 64-bit integers, which makes these exact.
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long bits_of(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ double from_bits(long long b) { return __longlong_as_double(b); }
__device__ __forceinline__ long long abs_bits(double x) { return bits_of(x) & 0x7FFFFFFFFFFFFFFFLL; }
__device__ __forceinline__ bool finite_bits(double x) {
    return (__double2hiint(x) & 0x7FF00000) != 0x7FF00000;
}
__device__ __forceinline__ long long max_bits(long long a, long long b) { return a > b ? a : b; }
__device__ __forceinline__ long long min_bits(long long a, long long b) { return a < b ? a : b; }

// log2 of a non-negative double to FP32 accuracy: exponent from the bit
// pattern, top 20 mantissa bits through the FP32 log2 unit. Zero and
// subnormals give -inf (the controller then shrinks), inf/NaN a large value
// (such steps are already flagged non-finite by the stepper).
__device__ __forceinline__ float log2_nonneg(double x) {
    const int hi = __double2hiint(x);
    const int e  = (hi >> 20) & 0x7FF;
    const float m = __int_as_float(0x3F800000 | ((hi & 0x000FFFFF) << 3));
    const float l = static_cast<float>(e - 1023) + __log2f(m);
    return e == 0 ? -INFINITY : l;
}

// ---------------------------------------------------------------------------
// Steppers. Interface: x (current state), xn (next state), err (error
// estimate, RKCK45 only), finite flag; the hook arguments are forwarded.
// ---------------------------------------------------------------------------

// Classic RK4: SingleSystem_PerThread_ExplicitRungeKutta_Steppers.cuh:6-117.
// xn doubles as the k-accumulator exactly as the reference does.
template <int SD, class P>
__device__ __forceinline__ void step_rk4(int tid, int nt, P t, P dt, P* x, P* xn, int& finite,
                                         P* cp, P* sp, int* spi, P* acc, int* acci)
{
    P X[SD];
    P k[SD];
    const P half  = static_cast<P>(0.5) * dt;
    const P sixth = static_cast<P>(1.0 / 6.0) * dt;

    PerThread_OdeFunction(tid, nt, xn, x, t, cp, sp, spi, acc, acci);

    P T = t + half;
#pragma unroll
    for (int i = 0; i < SD; i++) X[i] = x[i] + xn[i] * half;
    PerThread_OdeFunction(tid, nt, k, X, T, cp, sp, spi, acc, acci);

#pragma unroll
    for (int i = 0; i < SD; i++) {
        xn[i] = xn[i] + static_cast<P>(2.0) * k[i];
        X[i]  = x[i] + k[i] * half;
    }
    PerThread_OdeFunction(tid, nt, k, X, T, cp, sp, spi, acc, acci);

    T = t + dt;
#pragma unroll
    for (int i = 0; i < SD; i++) {
        xn[i] = xn[i] + static_cast<P>(2.0) * k[i];
        X[i]  = x[i] + k[i] * dt;
    }
    PerThread_OdeFunction(tid, nt, k, X, T, cp, sp, spi, acc, acci);

#pragma unroll
    for (int i = 0; i < SD; i++) {
        xn[i] = x[i] + sixth * (xn[i] + k[i]);
        if (isfinite(xn[i]) == 0) finite = 0;
    }
}

// Cash-Karp 4(5): SingleSystem_PerThread_ExplicitRungeKutta_Steppers.cuh:121-289.
// Fifth-order solution, embedded error |sum (b - b*) k| * dt + 1e-18.
template <int SD, class P, bool BITCHECK>
__device__ __forceinline__ void step_rkck45(int tid, int nt, P t, P dt, P* x, P* xn, P* err,
                                            int& finite, P* cp, P* sp, int* spi, P* acc, int* acci)
{
    P X[SD];
    P k1[SD], k2[SD], k3[SD], k4[SD], k5[SD], k6[SD];
    P T;

    PerThread_OdeFunction(tid, nt, k1, x, t, cp, sp, spi, acc, acci);

    T = t + dt * static_cast<P>(1.0 / 5.0);
#pragma unroll
    for (int i = 0; i < SD; i++) X[i] = x[i] + dt * (static_cast<P>(1.0 / 5.0) * k1[i]);
    PerThread_OdeFunction(tid, nt, k2, X, T, cp, sp, spi, acc, acci);

    T = t + dt * static_cast<P>(3.0 / 10.0);
#pragma unroll
    for (int i = 0; i < SD; i++)
        X[i] = x[i] + dt * (static_cast<P>(3.0 / 40.0) * k1[i] +
                            static_cast<P>(9.0 / 40.0) * k2[i]);
    PerThread_OdeFunction(tid, nt, k3, X, T, cp, sp, spi, acc, acci);

    T = t + dt * static_cast<P>(3.0 / 5.0);
#pragma unroll
    for (int i = 0; i < SD; i++)
        X[i] = x[i] + dt * (static_cast<P>(3.0 / 10.0) * k1[i] +
                            static_cast<P>(-9.0 / 10.0) * k2[i] +
                            static_cast<P>(6.0 / 5.0) * k3[i]);
    PerThread_OdeFunction(tid, nt, k4, X, T, cp, sp, spi, acc, acci);

    T = t + dt;
#pragma unroll
    for (int i = 0; i < SD; i++)
        X[i] = x[i] + dt * (static_cast<P>(-11.0 / 54.0) * k1[i] +
                            static_cast<P>(5.0 / 2.0) * k2[i] +
                            static_cast<P>(-70.0 / 27.0) * k3[i] +
                            static_cast<P>(35.0 / 27.0) * k4[i]);
    PerThread_OdeFunction(tid, nt, k5, X, T, cp, sp, spi, acc, acci);

    T = t + dt * static_cast<P>(7.0 / 8.0);
#pragma unroll
    for (int i = 0; i < SD; i++)
        X[i] = x[i] + dt * (static_cast<P>(1631.0 / 55296.0) * k1[i] +
                            static_cast<P>(175.0 / 512.0) * k2[i] +
                            static_cast<P>(575.0 / 13824.0) * k3[i] +
                            static_cast<P>(44275.0 / 110592.0) * k4[i] +
                            static_cast<P>(253.0 / 4096.0) * k5[i]);
    PerThread_OdeFunction(tid, nt, k6, X, T, cp, sp, spi, acc, acci);

#pragma unroll
    for (int i = 0; i < SD; i++) {
        xn[i] = x[i] + dt * (static_cast<P>(37.0 / 378.0) * k1[i] +
                             static_cast<P>(250.0 / 621.0) * k3[i] +
                             static_cast<P>(125.0 / 594.0) * k4[i] +
                             static_cast<P>(512.0 / 1771.0) * k6[i]);
        P e = static_cast<P>(37.0 / 378.0 - 2825.0 / 27648.0) * k1[i] +
              static_cast<P>(250.0 / 621.0 - 18575.0 / 48384.0) * k3[i] +
              static_cast<P>(125.0 / 594.0 - 13525.0 / 55296.0) * k4[i] +
              static_cast<P>(0.0 - 277.0 / 14336.0) * k5[i] +
              static_cast<P>(512.0 / 1771.0 - 1.0 / 4.0) * k6[i];
        err[i] = dt * abs(e) + 1e-18;
        if constexpr (BITCHECK) {
            if (!finite_bits(xn[i]) || !finite_bits(err[i])) finite = 0;
        } else {
            if ((isfinite(xn[i]) == 0) || (isfinite(err[i]) == 0)) finite = 0;
        }
    }
}

// Cash-Karp 4(5) with FP32 stages (extension, FP32_STAGE mode): the user
// right-hand side is instantiated for float and every stage sum runs in FP32;
// the state update x + dt * (sum b k) and the embedded error sum run in FP64 on
// the FP32 stage derivatives.
template <int SD, int NCP, int NA>
__device__ __forceinline__ void step_rkck45_f32stage(int tid, int nt, double t, double dt,
                                                     double* x, double* xn, double* err, int& finite,
                                                     float* cpf, float* spf, int* spi, float* accf,
                                                     int* acci)
{
    float xf[SD], X[SD];
    float k1[SD], k2[SD], k3[SD], k4[SD], k5[SD], k6[SD];
    const float h = static_cast<float>(dt);
#pragma unroll
    for (int i = 0; i < SD; i++) xf[i] = static_cast<float>(x[i]);

    PerThread_OdeFunction(tid, nt, k1, xf, static_cast<float>(t), cpf, spf, spi, accf, acci);

#pragma unroll
    for (int i = 0; i < SD; i++) X[i] = xf[i] + h * (0.2f * k1[i]);
    PerThread_OdeFunction(tid, nt, k2, X, static_cast<float>(t + dt * 0.2), cpf, spf, spi, accf, acci);

#pragma unroll
    for (int i = 0; i < SD; i++)
        X[i] = xf[i] + h * (static_cast<float>(3.0 / 40.0) * k1[i] + static_cast<float>(9.0 / 40.0) * k2[i]);
    PerThread_OdeFunction(tid, nt, k3, X, static_cast<float>(t + dt * 0.3), cpf, spf, spi, accf, acci);

#pragma unroll
    for (int i = 0; i < SD; i++)
        X[i] = xf[i] + h * (0.3f * k1[i] - 0.9f * k2[i] + 1.2f * k3[i]);
    PerThread_OdeFunction(tid, nt, k4, X, static_cast<float>(t + dt * 0.6), cpf, spf, spi, accf, acci);

#pragma unroll
    for (int i = 0; i < SD; i++)
        X[i] = xf[i] + h * (static_cast<float>(-11.0 / 54.0) * k1[i] + 2.5f * k2[i] +
                            static_cast<float>(-70.0 / 27.0) * k3[i] + static_cast<float>(35.0 / 27.0) * k4[i]);
    PerThread_OdeFunction(tid, nt, k5, X, static_cast<float>(t + dt), cpf, spf, spi, accf, acci);

#pragma unroll
    for (int i = 0; i < SD; i++)
        X[i] = xf[i] + h * (static_cast<float>(1631.0 / 55296.0) * k1[i] + static_cast<float>(175.0 / 512.0) * k2[i] +
                            static_cast<float>(575.0 / 13824.0) * k3[i] +
                            static_cast<float>(44275.0 / 110592.0) * k4[i] +
                            static_cast<float>(253.0 / 4096.0) * k5[i]);
    PerThread_OdeFunction(tid, nt, k6, X, static_cast<float>(t + dt * 0.875), cpf, spf, spi, accf, acci);

#pragma unroll
    for (int i = 0; i < SD; i++) {
        const float incr = static_cast<float>(37.0 / 378.0) * k1[i] + static_cast<float>(250.0 / 621.0) * k3[i] +
                           static_cast<float>(125.0 / 594.0) * k4[i] + static_cast<float>(512.0 / 1771.0) * k6[i];
        xn[i] = x[i] + dt * static_cast<double>(incr);
        const double e = (37.0 / 378.0 - 2825.0 / 27648.0) * static_cast<double>(k1[i]) +
                         (250.0 / 621.0 - 18575.0 / 48384.0) * static_cast<double>(k3[i]) +
                         (125.0 / 594.0 - 13525.0 / 55296.0) * static_cast<double>(k4[i]) +
                         (0.0 - 277.0 / 14336.0) * static_cast<double>(k5[i]) +
                         (512.0 / 1771.0 - 1.0 / 4.0) * static_cast<double>(k6[i]);
        err[i] = dt * fabs(e) + 1e-18;
        if (!finite_bits(xn[i]) || !finite_bits(err[i])) finite = 0;
    }
}

// ---------------------------------------------------------------------------
// Controllers.
// ---------------------------------------------------------------------------

// Fixed step: SingleSystem_PerThread_ExplicitRungeKutta_ErrorControllers.cuh:5-20.
// A non-finite state stops the instance; the next step is InitialTimeStep.
template <class P>
__device__ __forceinline__ void control_rk4(const Options<P>& o, int finite, int& terminate,
                                            P& new_dt, int& status)
{
    if (finite == 0) {
        terminate = 1;
        status |= MPGOS_INSTANCE_NONFINITE;
    }
    new_dt = o.initial_dt;
}

// Adaptive step, reference arithmetic:
// SingleSystem_PerThread_ExplicitRungeKutta_ErrorControllers.cuh:23-85.
template <int SD, class P>
__device__ __forceinline__ void control_rkck45_plain(const Options<P>& o, P dt, const P* x, const P* xn,
                                                     const P* err, const P* rtol, const P* atol,
                                                     int& update, int& finite, int& terminate,
                                                     P& new_dt, int& status)
{
    P ratio = 1e30;
    for (int i = 0; i < SD; i++) {
        const P tol = fmax(rtol[i] * fmax(fabs(xn[i]), fabs(x[i])), atol[i]);
        update = update && (err[i] < tol);
        ratio  = fmin(ratio, tol / err[i]);
    }
    P q;
    if (update == 1)
        q = static_cast<P>(0.9) * pow(ratio, static_cast<P>(1.0 / 5.0));
    else
        q = static_cast<P>(0.9) * pow(ratio, static_cast<P>(1.0 / 4.0));
    if (isfinite(q) == 0) finite = 0;

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
    q      = fmin(q, o.grow);
    q      = fmax(q, o.shrink);
    new_dt = dt * q;
    new_dt = fmin(new_dt, o.max_dt);
    new_dt = fmax(new_dt, o.min_dt);
}

// Adaptive step, FAST_CONTROL (FP64 values only). Same accept/reject rule as
// the reference (err_i < max(rtol_i * max(|xn_i|, |x_i|), atol_i) for every
// component), decided without FP64 arithmetic in the common case: the test
// is made on d_i = log2(tol_i) - log2(err_i) in FP32, where log2 tol_i is
// max(log2 rtol_i + log2 m_i, log2 atol_i) from the exponent bits and the FP32
// log2 unit. The FP32 estimate is good to better than 3e-4 (log2 units) over
// the whole double range, so only when |d_i| < FAST_BAND (2e-3, a 0.14% band
// around err = tol) is the exact FP64 product formed and compared; the
// decision is therefore always the one of the FP64 rule.
// The factor 0.9 R^(1/5) (0.9 R^(1/4) after a rejection), R = min_i tol_i/err_i,
// becomes 0.9 * exp2(min_i d_i / 5) in FP32; it is clamped to [shrink, grow]
// afterwards, so its FP32 rounding moves the next step size by ~1e-6 relative.
// Requires non-negative tolerances and options (checked on the host).
// lrtol / latol: log2 of the tolerances (per block, FP32).
constexpr float FAST_BAND = 2e-3f;

template <int SD>
__device__ __forceinline__ void control_rkck45_fast(const Options<double>& o, double dt, const double* x,
                                                    const double* xn, const double* err,
                                                    const double* rtol, const double* atol, const float* lrtol,
                                                    const float* latol, int& update, int& finite, int& terminate,
                                                    double& new_dt, int& status)
{
    float lr = INFINITY;
#pragma unroll
    for (int i = 0; i < SD; i++) {
        const long long mb = max_bits(abs_bits(xn[i]), abs_bits(x[i]));
        const float lt = fmaxf(lrtol[i] + log2_nonneg(from_bits(mb)), latol[i]);
        const float d  = lt - log2_nonneg(err[i]);
        int accept_i;
        if (d > FAST_BAND) {
            accept_i = 1;
        } else if (d < -FAST_BAND) {
            accept_i = 0;
        } else {
            const long long tb = max_bits(bits_of(rtol[i] * from_bits(mb)), bits_of(atol[i]));
            accept_i = bits_of(err[i]) < tb;
        }
        update = update && accept_i;
        lr = fminf(lr, d);
    }
    const float expo = (update == 1) ? 0.2f : 0.25f;
    float qf = 0.9f * exp2f(fminf(fmaxf(lr * expo, -120.0f), 120.0f));

    const long long dtb    = bits_of(dt);
    const long long guardb = bits_of(o.min_dt_guard);
    long long qb;
    if (finite == 0) {
        qb     = bits_of(o.shrink);
        update = 0;
        if (dtb < guardb) {
            terminate = 1;
            status |= MPGOS_INSTANCE_NONFINITE;
        }
    } else {
        qb = bits_of(static_cast<double>(qf));
        if (dtb < guardb) {
            update = 1;
            status |= MPGOS_INSTANCE_MINIMUM_STEP;
        }
    }
    qb = min_bits(qb, bits_of(o.grow));
    qb = max_bits(qb, bits_of(o.shrink));
    // A negative double (sign bit set) is a negative int64 and so orders below
    // the positive limits, like the FP64 compare; only a NaN step (unreachable
    // with finite options) would order differently.
    const double nd = dt * from_bits(qb);
    new_dt = from_bits(max_bits(min_bits(bits_of(nd), bits_of(o.max_dt)), bits_of(o.min_dt)));
}

// ---------------------------------------------------------------------------
// Events.
// ---------------------------------------------------------------------------

// Step rejection toward an event: SingleSystem_PerThread_EventHandling.cuh:5-44.
// A crossing of the +-tolerance band in an allowed direction rejects the step
// and proposes the secant step -g_a/(g_n - g_a) * dt; repeated over successive
// attempts this refines the root until the step lands inside the band.
template <int NE, class P>
__device__ __forceinline__ void event_step_control(int& update, int terminate, const P* ga, const P* gn,
                                                   const P* etol, const int* edir, P dt, P& new_dt,
                                                   P min_dt, int& status)
{
    P event_dt   = dt;
    int corrected = 0;
    if ((update == 1) && (terminate == 0)) {
        for (int i = 0; i < NE; i++) {
            if (((ga[i] > etol[i]) && (gn[i] < -etol[i]) && (edir[i] <= 0)) ||
                ((ga[i] < -etol[i]) && (gn[i] > etol[i]) && (edir[i] >= 0))) {
                event_dt  = fmin(event_dt, -ga[i] / (gn[i] - ga[i]) * dt);
                corrected = 1;
            }
        }
    }
    if (corrected == 1) {
        if (event_dt < min_dt) {
            status |= MPGOS_INSTANCE_EVENT_OMITTED;
        } else {
            new_dt = event_dt;
            update = 0;
        }
    }
}

// Detection on an accepted step: the value moved from outside the band into
// it, in an allowed direction (SingleSystem_PerThread_Solver.cuh:327-328).
template <class P>
__device__ __forceinline__ bool event_detected(P ga, P gn, P tol, int dir)
{
    return ((ga > tol) && (abs(gn) < tol) && (dir <= 0)) ||
           ((ga < -tol) && (abs(gn) < tol) && (dir >= 0));
}

// ---------------------------------------------------------------------------
// Dense output: SingleSystem_PerThread_DenseOutput.cuh:5-58.
// Layout: time [slot][NT], state [slot][component][NT].
// ---------------------------------------------------------------------------
template <class P>
__device__ __forceinline__ int dense_condition(P t, P dense_next, int didx, int skipped, int end_reached,
                                               int udt, int ndo, int freq)
{
    int store = ((didx < ndo) && (dense_next < t) && (skipped >= (freq - 1))) ? 1 : 0;
    if ((didx < ndo) && ((end_reached == 1) || (udt == 1))) store = 1;
    return store;
}

template <int SD, class P>
__device__ __forceinline__ void dense_store(long long i, long long nt, int store, int& didx, int ndo,
                                            P* dtime, P* dstate, P t, const P* x, int& skipped,
                                            P& dense_next, P dense_min_dt, P upper)
{
    if (store == 1) {
        if (didx < ndo) {
            dtime[i + static_cast<long long>(didx) * nt] = t;
            long long idx = i + static_cast<long long>(didx) * nt * SD;
#pragma unroll
            for (int c = 0; c < SD; c++) {
                dstate[idx] = x[c];
                idx += nt;
            }
            didx++;
        }
        skipped    = 0;
        dense_next = fmin(t + dense_min_dt, upper);
    } else {
        skipped++;
    }
}

}  // namespace pt
}  // namespace mpgos

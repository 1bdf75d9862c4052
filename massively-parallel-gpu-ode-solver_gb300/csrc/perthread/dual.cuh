// Forward-mode dual numbers for differentiating user hooks unchanged.
//
// The reference's hooks are templates on Precision
// (Tutorials_SingleSystem_PerThread/T1_Reference/Reference_SystemDefinition.cuh:5-13).
// Instantiating PerThread_OdeFunction with Precision = Dual<N> evaluates the
// right-hand side and, in the same pass, its derivatives along N seeded
// directions: with the state components and the control parameters seeded
// as unit directions this yields the full Jacobian [df/dx | df/dp], from which
// the adjoint kernel forms vector-Jacobian products.
//
// Arithmetic, comparisons and the math functions the hooks use (cos, sin,
// pow, sqrt, exp, log, fabs/abs, sincospi) are overloaded and found by
// argument-dependent lookup. Values come from CUDA's own functions, except
// sin/cos (double-float on the FP32 pipe, see below); derivative parts use
// the analytic derivative identities. A dual whose
// derivative part is identically zero (the time argument, shared parameters)
// skips the derivative evaluation of transcendental functions.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include <type_traits>

#include "dfloat.cuh"

namespace mpgos {
namespace ad {

// a*b + c and a*b + c*d in the value type: contracted FP64 expressions, or
// the fused double-float forms (fewer FP32 operations than separate ops).
__host__ __device__ __forceinline__ double mad(double a, double b, double c) { return a * b + c; }
__host__ __device__ __forceinline__ double mad2(double a, double b, double c, double d) { return a * b + c * d; }
__device__ __forceinline__ df::dfloat mad(df::dfloat a, df::dfloat b, df::dfloat c) { return df::fma(a, b, c); }
__device__ __forceinline__ df::dfloat mad2(df::dfloat a, df::dfloat b, df::dfloat c, df::dfloat d)
{
    return df::dot2(a, b, c, d);
}

template <int N, class T = double>
struct Dual {
    T v;
    T d[N];

    __host__ __device__ Dual() : v(0.0) {
#pragma unroll
        for (int i = 0; i < N; i++) d[i] = T(0.0);
    }
    __host__ __device__ Dual(T x) : v(x) {  // NOLINT: implicit, hooks write static_cast<Precision>(c)
#pragma unroll
        for (int i = 0; i < N; i++) d[i] = T(0.0);
    }
    template <class U = T, class = typename std::enable_if<!std::is_same<U, double>::value>::type>
    __host__ __device__ Dual(double x) : Dual(T(x)) {}  // NOLINT: literals and FP64 values for a double-float T
    __host__ __device__ explicit operator double() const { return static_cast<double>(v); }

    // True when every derivative is +-0 (tested on the bit patterns, which
    // keeps the floating-point pipes free).
    __device__ bool constant() const {
        if constexpr (std::is_same<T, double>::value) {
            long long z = 0;
#pragma unroll
            for (int i = 0; i < N; i++) z |= (__double_as_longlong(d[i]) << 1);
            return z == 0;
        } else {
            int z = 0;
#pragma unroll
            for (int i = 0; i < N; i++) z |= (__float_as_int(d[i].hi) << 1);  // a zero double-float has lo == 0
            return z == 0;
        }
    }

    __device__ Dual& operator+=(const Dual& b) { v += b.v; for (int i = 0; i < N; i++) d[i] += b.d[i]; return *this; }
    __device__ Dual& operator-=(const Dual& b) { v -= b.v; for (int i = 0; i < N; i++) d[i] -= b.d[i]; return *this; }
    __device__ Dual& operator*=(const Dual& b) { *this = *this * b; return *this; }
    __device__ Dual& operator/=(const Dual& b) { *this = *this / b; return *this; }
    __device__ Dual& operator++() { v += T(1.0); return *this; }

    // chain rule helper: f(v) with derivative f'(v)
    __device__ Dual chain(T fv, T dfv) const {
        Dual r;
        r.v = fv;
#pragma unroll
        for (int i = 0; i < N; i++) r.d[i] = dfv * d[i];
        return r;
    }

    friend __device__ Dual operator-(const Dual& a) { Dual r; r.v = -a.v; for (int i = 0; i < N; i++) r.d[i] = -a.d[i]; return r; }
    friend __device__ Dual operator+(const Dual& a) { return a; }
    friend __device__ Dual operator+(const Dual& a, const Dual& b) { Dual r; r.v = a.v + b.v; for (int i = 0; i < N; i++) r.d[i] = a.d[i] + b.d[i]; return r; }
    friend __device__ Dual operator-(const Dual& a, const Dual& b) { Dual r; r.v = a.v - b.v; for (int i = 0; i < N; i++) r.d[i] = a.d[i] - b.d[i]; return r; }
    friend __device__ Dual operator*(const Dual& a, const Dual& b) {
        Dual r;
        r.v = a.v * b.v;
#pragma unroll
        for (int i = 0; i < N; i++) r.d[i] = mad2(a.d[i], b.v, a.v, b.d[i]);
        return r;
    }
    friend __device__ Dual operator/(const Dual& a, const Dual& b) {
        Dual r;
        const T inv = T(1.0) / b.v;
        r.v = a.v * inv;
#pragma unroll
        for (int i = 0; i < N; i++) r.d[i] = (a.d[i] - r.v * b.d[i]) * inv;
        return r;
    }
    friend __device__ Dual operator+(const Dual& a, double b) { Dual r = a; r.v += T(b); return r; }
    friend __device__ Dual operator+(double a, const Dual& b) { Dual r = b; r.v += T(a); return r; }
    friend __device__ Dual operator-(const Dual& a, double b) { Dual r = a; r.v -= T(b); return r; }
    friend __device__ Dual operator-(double a, const Dual& b) { Dual r = -b; r.v += T(a); return r; }
    friend __device__ Dual operator*(const Dual& a, double b) { const T bb(b); Dual r; r.v = a.v * bb; for (int i = 0; i < N; i++) r.d[i] = a.d[i] * bb; return r; }
    friend __device__ Dual operator*(double a, const Dual& b) { return b * a; }
    friend __device__ Dual operator/(const Dual& a, double b) { return a * (1.0 / b); }
    friend __device__ Dual operator/(double a, const Dual& b) { return Dual(T(a)) / b; }

    friend __device__ bool operator<(const Dual& a, const Dual& b) { return a.v < b.v; }
    friend __device__ bool operator>(const Dual& a, const Dual& b) { return a.v > b.v; }
    friend __device__ bool operator<=(const Dual& a, const Dual& b) { return a.v <= b.v; }
    friend __device__ bool operator>=(const Dual& a, const Dual& b) { return a.v >= b.v; }
    friend __device__ bool operator==(const Dual& a, const Dual& b) { return a.v == b.v; }
    friend __device__ bool operator!=(const Dual& a, const Dual& b) { return a.v != b.v; }

    // ---- math functions (found by ADL from the hooks) ----
    // sin and cos run on the FP32 pipe in double-float (dfloat.cuh: error
    // ~1e-15 + |x| 2^-48): a dual evaluation only feeds Jacobians and
    // replayed stage values, where that is far below the tolerance, and an
    // FP64 sin/cos would cost more FP64-pipe time than the rest of a stage.
    __device__ static void sincos_value(double x, double* s, double* c) {
        df::dfloat sd, cd;
        df::sincos(df::dfloat(x), &sd, &cd);
        *s = static_cast<double>(sd);
        *c = static_cast<double>(cd);
    }
    __device__ static void sincos_value(df::dfloat x, df::dfloat* s, df::dfloat* c) { df::sincos(x, s, c); }
    friend __device__ Dual cos(const Dual& a) {
        T s, c;
        sincos_value(a.v, &s, &c);
        if (a.constant()) return Dual(c);
        return a.chain(c, -s);
    }
    friend __device__ Dual sin(const Dual& a) {
        T s, c;
        sincos_value(a.v, &s, &c);
        if (a.constant()) return Dual(s);
        return a.chain(s, c);
    }
    friend __device__ Dual exp(const Dual& a) { const T e = exp(a.v); return a.chain(e, e); }
    friend __device__ Dual log(const Dual& a) { return a.chain(log(a.v), T(1.0) / a.v); }
    friend __device__ Dual sqrt(const Dual& a) { const T s = sqrt(a.v); return a.chain(s, T(0.5) / s); }
    friend __device__ Dual fabs(const Dual& a) { return a.v < T(0.0) ? -a : a; }
    friend __device__ Dual abs(const Dual& a) { return a.v < T(0.0) ? -a : a; }
    friend __device__ Dual pow(const Dual& a, double e) {
        const T p = pow(a.v, e);
        return a.chain(p, T(e) * pow(a.v, e - 1.0));
    }
    friend __device__ Dual pow(const Dual& a, const Dual& b) {
        // d(a^b) = b a^(b-1) da + a^b ln(a) db
        const T p = pow(a.v, b.v);
        Dual r;
        r.v = p;
        const T da = b.v * pow(a.v, b.v - T(1.0));
        const bool bconst = b.constant();
        const T db = bconst ? T(0.0) : p * log(a.v);
#pragma unroll
        for (int i = 0; i < N; i++) r.d[i] = da * a.d[i] + db * b.d[i];
        return r;
    }
    friend __device__ void sincospi(const Dual& a, Dual* s, Dual* c) {
        T sv, cv;
        sincos_value(a.v * T(3.14159265358979323846), &sv, &cv);
        const T w(3.14159265358979323846);
        *s = a.chain(sv, w * cv);
        *c = a.chain(cv, -w * sv);
    }
};

}  // namespace ad
}  // namespace mpgos

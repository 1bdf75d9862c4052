// Coupled per-block ensemble solver for sm_103a: one warp per system.
//
// The reference integrates a system of UPS coupled units with one thread per
// unit inside a block (four kernel variants by launch shape,
// SourceCodes/CoupledSystmes_PerBlock_Solver.cuh:10,786,1507,2214, chosen in
// CoupledSystems_PerBlock_Interface.cuh:1949-1966), system-scope variables in
// shared memory, per-system reductions through shared-memory atomics
// (atomicAnd, a CAS-loop atomicFMIN) and a __syncthreads between every phase
// of a step. Here one warp owns one system:
//
//  * units are spread over the 32 lanes (UPL = ceil(UPS/32) units per lane),
//    their state, stages and parameters live in registers;
//  * system-scope variables (time domain, time, step, dense index, user
//    termination flag, system parameters and accessories) live in a per-warp
//    slot of shared memory, because the hooks take them by reference exactly
//    as in the reference;
//  * the coupling matrix is staged once per CTA in shared memory (all four
//    storages of the reference: full, banded, circular-banded, full circular)
//    and the coupling matrix-vector product of every stage reads the coupling
//    terms as shared-memory broadcasts;
//  * accept/reject, the error ratio and the event step are warp reductions
//    (__all_sync, shuffles) and the phases are separated by __syncwarp only,
//    so systems never wait for each other; in PERSISTENT mode a warp pulls
//    the next system from a device counter when its system finishes.
//
// Arithmetic (stage sums, coupling accumulation, controller with safety
// factor 0.8, event secant step) keeps the reference's operation order
// (CoupledSystems_PerBlock_ExplicitRungeKutta_Steppers.cuh:1483-2014,
// ..._ErrorControllers.cuh:320-423, CoupledSystems_PerBlock_EventHandling.cuh:149-214).
//
// The user hooks (CoupledSystems_PerBlock_OdeFunction, _EventFunction,
// _ActionAfterEventDetection, _ActionAfterSuccessfulTimeStep,
// _Initialization, _Finalization) must be declared before this header.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "../perthread/numerics.cuh"
#include "../perthread/dfloat.cuh"
#include "../perthread/df_convert.cuh"
#include "../perthread/ck_tableau.cuh"

#ifndef MPGOS_CB_MAX_BLOCK
#define MPGOS_CB_MAX_BLOCK 256
#endif

namespace mpgos {
namespace cb {

using df::dfloat;
using pt::AtLeastOne;
using pt::Options;

// Compute precision P and the precision of the arrays in HBM: DF_STAGE
// integrates in double-float (dfloat.cuh) on FP64 arrays.
template <class P>
struct StorageOf {
    using type = P;
};
template <>
struct StorageOf<dfloat> {
    using type = double;
};
template <class P>
constexpr bool IS_DF = std::is_same<P, dfloat>::value;

template <int UPS_, int UD_, int NC_, int CBW_, int CCI_, int NUP_, int NSP_, int NGP_, int NIGP_, int NUA_,
          int NIUA_, int NSA_, int NISA_, int NE_>
struct Shape {
    static constexpr int UPS = UPS_, UD = UD_, NC = NC_, CBW = CBW_, CCI = CCI_, NUP = NUP_, NSP = NSP_;
    static constexpr int NGP = NGP_, NIGP = NIGP_, NUA = NUA_, NIUA = NIUA_, NSA = NSA_, NISA = NISA_, NE = NE_;
    static constexpr int UPL = (UPS + 31) / 32;  // units per lane
    // entries of one stored coupling matrix (CoupledSystems_PerBlock_Interface.cuh:426-438)
    static constexpr int MAT = (CCI == 0 && CBW == 0)  ? UPS * UPS
                               : (CCI == 0 && CBW > 0) ? UPS * (2 * CBW + 1)
                               : (CCI == 1 && CBW > 0) ? (2 * CBW + 1)
                                                       : UPS;
};

template <class P>
struct Args {
    long long ns, n_active;
    // system scope [field][NS]
    P* td;
    P* t;
    P* sp;
    P* sacc;
    int* isacc;
    P* cstr;
    int* didx;
    P* dtime;
    // unit scope [field][NS*UPS], unit u of system s at s*UPS + u
    P* x;
    P* up;
    P* uacc;
    int* iuacc;
    P* dstate;
    // global scope
    const P* gp;
    const int* igp;
    const P* cmat;
    const int* cidx;
    const P* rtol;
    const P* atol;
    const P* etol;
    const int* edir;
    // per system, this launch
    int* status;
    int* n_acc;
    int* n_rej;
    unsigned int* work;
    int shared_global;
    int shared_coupling;
    const void* cmat_df;  // DF_STAGE, matrices in global memory: their double-float copy
    Options<P> o;
    // adjoint tape of a recording launch (MODE_RECORD): dt [max_steps][NS],
    // ckpt_x [max_steps/seg + 1][UD][NS*UPS], ckpt_t [max_steps/seg + 1][NS],
    // n_steps [NS]
    pt::Tape tape;
};

// Kernel-internal mode bit: the forward launch records the adjoint tape.
constexpr int MODE_RECORD = pt::MODE_RECORD;

// Per-warp (per-system) shared-memory slot.
template <class S, class P>
struct WarpSlot {
    P td[2];
    typename StorageOf<P>::type td_in[2];  // the time domain as loaded from HBM
    P t, dt, newdt, dense_next, evdt, ratio;
    P sp[AtLeastOne<S::NSP>::value];
    P sacc[AtLeastOne<S::NSA>::value];
    P cstr[AtLeastOne<S::NC>::value];
    P cpt[S::UPS][AtLeastOne<S::NC>::value];
    int isacc[AtLeastOne<S::NISA>::value];
    int didx, udt, skipped, update;
};

// SPLIT: the slot of the FP64 solver with the coupling strengths and the
// coupling terms, which only the right-hand side reads, held as double-float
// in the same bytes (the size and the offsets of WarpSlot<S, double>).
template <class S>
struct WarpSlotSplit {
    double td[2];
    double td_in[2];
    double t, dt, newdt, dense_next, evdt, ratio;
    double sp[AtLeastOne<S::NSP>::value];
    double sacc[AtLeastOne<S::NSA>::value];
    dfloat cstr[AtLeastOne<S::NC>::value];
    dfloat cpt[S::UPS][AtLeastOne<S::NC>::value];
    int isacc[AtLeastOne<S::NISA>::value];
    int didx, udt, skipped, update;
};

template <class S, class P>
__host__ __device__ constexpr size_t block_smem_bytes()
{
    return 0;
}

// Coupling value of coupling i for unit `unit`: ComputeCouplingValue of
// CoupledSystems_PerBlock_ExplicitRungeKutta_Steppers.cuh:2552-2633.
// Double-float dot product term: s + m * c accumulated as an unnormalised
// pair (sum of leading floats by two_sum, every rounding error and the
// cross products into the trailing float); normalised once at the end.
__device__ __forceinline__ void df_dot_acc(float& sh, float& sl, dfloat m, dfloat c)
{
    const dfloat p = df::two_prod(m.hi, c.hi);
    const dfloat t = df::two_sum(sh, p.hi);
    sh = t.hi;
    sl = df::f_add(sl, df::f_add(t.lo, df::f_fma(m.hi, c.lo, df::f_fma(m.lo, c.hi, p.lo))));
}

// Unroll factor of the dense coupling loop (64 or more terms per unit and
// stage): the whole loop unrolled is hundreds of instructions per copy, and a
// step inlines one copy per unit of the lane and per stage.
#ifndef MPGOS_CB_COUPLING_UNROLL
#define MPGOS_CB_COUPLING_UNROLL 4
#endif
#define MPGOS_CB_PRAGMA(x) _Pragma(#x)
#define MPGOS_CB_UNROLL(n) MPGOS_CB_PRAGMA(unroll n)

template <class S, class P, class W>
__device__ __forceinline__ P coupling_value(const P* M, const W& w, int unit, int i)
{
    constexpr int UPS = S::UPS, CBW = S::CBW, CCI = S::CCI;
    if constexpr (IS_DF<P> && CCI == 0 && CBW == 0) {
        const int shift = i * UPS * UPS;
        float sh = 0.0f, sl = 0.0f;
        MPGOS_CB_UNROLL(MPGOS_CB_COUPLING_UNROLL)
        for (int col = 0; col < UPS; col++) df_dot_acc(sh, sl, M[unit + col * UPS + shift], w.cpt[col][i]);
        return df::two_sum(sh, sl);
    }
    P v = 0;
    if (CCI == 0 && CBW == 0) {
        const int shift = i * UPS * UPS;
        MPGOS_CB_UNROLL(MPGOS_CB_COUPLING_UNROLL)
        for (int col = 0; col < UPS; col++) v += M[unit + col * UPS + shift] * w.cpt[col][i];
    } else if (CCI == 0 && CBW > 0) {
        const int shift = i * UPS * (2 * CBW + 1);
        for (int dg = 0; dg < 2 * CBW + 1; dg++) {
            int su = unit + dg - CBW;
            if (su >= UPS) su -= UPS;
            if (su < 0) su += UPS;
            v += M[unit + dg * UPS + shift] * w.cpt[su][i];
        }
    } else if (CCI == 1 && CBW > 0) {
        const int shift = i * (2 * CBW + 1);
        for (int dg = 0; dg < 2 * CBW + 1; dg++) {
            int su = unit + dg - CBW;
            if (su >= UPS) su -= UPS;
            if (su < 0) su += UPS;
            v += M[dg + shift] * w.cpt[su][i];
        }
    } else {
        const int shift = i * UPS;
        for (int dg = 0; dg < UPS; dg++) {
            int su = unit + dg - CBW;
            if (su >= UPS) su -= UPS;
            if (su < 0) su += UPS;
            v += M[dg + shift] * w.cpt[su][i];
        }
    }
    return v;
}

__device__ __forceinline__ bool warp_all(bool p) { return __all_sync(0xffffffffu, p); }
__device__ __forceinline__ bool warp_any(bool p) { return __any_sync(0xffffffffu, p); }
template <class P>
__device__ __forceinline__ P warp_min(P v)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, off));
    return v;
}
__device__ __forceinline__ dfloat warp_min(dfloat v)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const dfloat o(__shfl_xor_sync(0xffffffffu, v.hi, off), __shfl_xor_sync(0xffffffffu, v.lo, off));
        v = df::fmin(v, o);
    }
    return v;
}
__device__ __forceinline__ float warp_minf(float v)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, off));
    return v;
}

// ---- SPLIT helpers -----------------------------------------------------------------
// The stage loop of the split stepper reads its Cash-Karp weights from
// constant memory: CK_A, CK_B, CK_E, CK_C (ck_tableau.cuh).
// Width (log2 units) of the band around a decision inside which the FP32
// log2 estimates (good to ~4e-6) do not decide and the exact FP64 comparison
// runs instead; log2(1e30), the cap of the minimum ratio
// (CoupledSystems_PerBlock_ExplicitRungeKutta_ErrorControllers.cuh starts it
// at 1e30).
constexpr float SPLIT_BAND = 1e-4f;
constexpr float SPLIT_LOG2_RATIO_CAP = 99.65784f;

__device__ __forceinline__ long long bits_of(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ double from_bits(long long b) { return __longlong_as_double(b); }
__device__ __forceinline__ long long abs_bits(double x) { return bits_of(x) & 0x7FFFFFFFFFFFFFFFLL; }
__device__ __forceinline__ long long max_bits(long long a, long long b) { return a > b ? a : b; }
__device__ __forceinline__ long long min_bits(long long a, long long b) { return a < b ? a : b; }
__device__ __forceinline__ bool finite_bits(double x) { return abs_bits(x) < 0x7FF0000000000000LL; }

// double-float copy of an FP64 value the right-hand side reads; `range` set
// when the value leaves float's exponent range
__device__ __forceinline__ dfloat split_checked(double v, int& range)
{
    if (!df::in_float_range(v)) range = 1;
    return df::split(v);
}

// The exact FP64 forms behind the estimates, out of line: they run only
// inside the band.
static __device__ __noinline__ double split_tolerance(double rtol, double atol, long long mag_bits)
{
    return from_bits(max_bits(bits_of(rtol * from_bits(mag_bits)), bits_of(atol)));
}
// The FP64 error estimate dt |sum_j e_j k_j| + 1e-18 from the double-float
// error sum h + l, and the FP32 estimate of its log2 (float sum of the pair,
// the leading float of dt: relative error below 2^-21)
__device__ __forceinline__ double split_error(double dt, float h, float l)
{
    return __fma_rn(dt, fabs(df::widen(h) + df::widen(l)), 1e-18);
}
__device__ __forceinline__ float split_log2_error(float dt_hi, float h, float l)
{
    return __log2f(fmaf(dt_hi, fabsf(h + l), 1e-18f));
}
__device__ __forceinline__ bool finite_float(float f) { return (__float_as_uint(f) & 0x7f800000u) != 0x7f800000u; }
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

template <class S, int ALG, class P, int MODE>
struct Solver {
    static constexpr int UPS = S::UPS, UD = S::UD, NC = S::NC, NUP = S::NUP, NUA = S::NUA, NIUA = S::NIUA;
    static constexpr int NE = S::NE, UPL = S::UPL, NSP = S::NSP, NSA = S::NSA, NISA = S::NISA;
    static constexpr bool PERSISTENT = (MODE & MPGOS_MODE_PERSISTENT) != 0;
    // the tape is FP64 for both arithmetics (a double-float value is a double exactly)
    static constexpr bool RECORD = (MODE & MODE_RECORD) != 0;
    // SPLIT: the right-hand side, the coupling and the stage sums in
    // double-float; state, time, step, error estimate and norm, control,
    // events and every other hook in FP64 (P = double)
    static constexpr bool SPLIT = (MODE & MPGOS_MODE_SPLIT) != 0;
    static_assert(!SPLIT || std::is_same<P, double>::value, "the split integrates an FP64 state");
    using Slot = typename std::conditional<SPLIT, WarpSlotSplit<S>, WarpSlot<S, P>>::type;
    using SP   = typename StorageOf<P>::type;  // precision of the arrays in HBM

    // Registers of the lane's units.
    struct Units {
        P x[UPL][UD];
        P up[UPL][AtLeastOne<NUP>::value];
        P uacc[UPL][AtLeastOne<NUA>::value];
        int iuacc[UPL][AtLeastOne<NIUA>::value];
        P ga[UPL][AtLeastOne<NE>::value];
        P cpf[UPL][AtLeastOne<NC>::value];
        // SPLIT: double-float copies of what the right-hand side reads (the
        // lane's units and, per lane, the system's parameters and
        // accessories), the coupling factors it writes, and whether a copied
        // value left float's exponent range
        dfloat xd[UPL][UD];
        dfloat upd[UPL][AtLeastOne<NUP>::value];
        dfloat uaccd[UPL][AtLeastOne<NUA>::value];
        dfloat cpfd[UPL][AtLeastOne<NC>::value];
        dfloat spd[AtLeastOne<NSP>::value];
        dfloat saccd[AtLeastOne<NSA>::value];
        int range;
    };

    __device__ static bool has(int lane, int j) { return lane + 32 * j < UPS; }
    __device__ static int unit_of(int lane, int j) { return lane + 32 * j; }

    // One right-hand side for all of the lane's units at stage point X, then
    // the coupling term added (the stepper stage of
    // CoupledSystems_PerBlock_ExplicitRungeKutta_Steppers.cuh:1733-1762).
    __device__ static void stage_rhs(long long s, int lane, Slot& w, Units& u, const P* gp, const int* igp, const P* M,
                                     const int* cidx, P T, P (&X)[UPL][UD], P (&F)[UPL][UD])
    {
        const int sid = static_cast<int>(s);
#pragma unroll
        for (int j = 0; j < UPL; j++) {
            if (has(lane, j)) {
                const int uid = unit_of(lane, j);
                CoupledSystems_PerBlock_OdeFunction<P>(sid, uid, F[j], X[j], T, u.up[j], w.sp, const_cast<P*>(gp),
                                                       const_cast<int*>(igp), u.uacc[j], u.iuacc[j], w.sacc, w.isacc,
                                                       w.cpt[uid], u.cpf[j]);
            }
        }
        __syncwarp();
#pragma unroll
        for (int j = 0; j < UPL; j++) {
            if (has(lane, j)) {
                const int uid = unit_of(lane, j);
#pragma unroll
                for (int i = 0; i < NC; i++) {
                    const P value = coupling_value<S, P>(M, w, uid, i);
                    // the component by a compile-time loop: a run-time index
                    // would put the stage array in local memory
                    const int c = cidx[i];  // validated on the host; out of range adds nothing
                    const P term = w.cstr[i] * u.cpf[j][i] * value;
#pragma unroll
                    for (int d = 0; d < UD; d++)
                        if (d == c) F[j][d] += term;
                }
            }
        }
        __syncwarp();
    }

    // RK4 step: CoupledSystems_PerBlock_ExplicitRungeKutta_Steppers.cuh:1483-1692.
    __device__ static void step_rk4(long long s, int lane, Slot& w, Units& u, const P* gp, const int* igp, const P* M,
                                    const int* cidx, P t, P dt, P (&xn)[UPL][UD], int& finite)
    {
        P X[UPL][UD], k[UPL][UD];
        stage_rhs(s, lane, w, u, gp, igp, M, cidx, t, u.x, xn);
        P T = t + static_cast<P>(0.5) * dt;
#pragma unroll
        for (int j = 0; j < UPL; j++)
#pragma unroll
            for (int d = 0; d < UD; d++) X[j][d] = u.x[j][d] + xn[j][d] * static_cast<P>(0.5) * dt;
        stage_rhs(s, lane, w, u, gp, igp, M, cidx, T, X, k);
#pragma unroll
        for (int j = 0; j < UPL; j++)
#pragma unroll
            for (int d = 0; d < UD; d++) {
                xn[j][d] += 2 * k[j][d];
                X[j][d] = u.x[j][d] + k[j][d] * static_cast<P>(0.5) * dt;
            }
        stage_rhs(s, lane, w, u, gp, igp, M, cidx, T, X, k);
        T = t + dt;
#pragma unroll
        for (int j = 0; j < UPL; j++)
#pragma unroll
            for (int d = 0; d < UD; d++) {
                xn[j][d] += static_cast<P>(2.0) * k[j][d];
                X[j][d] = u.x[j][d] + k[j][d] * dt;
            }
        stage_rhs(s, lane, w, u, gp, igp, M, cidx, T, X, k);
#pragma unroll
        for (int j = 0; j < UPL; j++)
#pragma unroll
            for (int d = 0; d < UD; d++) {
                xn[j][d] = u.x[j][d] + dt * (xn[j][d] + k[j][d]) * static_cast<P>(1.0 / 6.0);
                if (has(lane, j) && isfinite(xn[j][d]) == 0) finite = 0;
            }
    }

    // Cash-Karp 4(5) step: CoupledSystems_PerBlock_ExplicitRungeKutta_Steppers.cuh:1695-2014.
    __device__ static void step_rkck45(long long s, int lane, Slot& w, Units& u, const P* gp, const int* igp,
                                       const P* M, const int* cidx, P t, P dt, P (&xn)[UPL][UD],
                                       P (&err)[UPL][UD], int& finite)
    {
        P X[UPL][UD];
        P k1[UPL][UD], k2[UPL][UD], k3[UPL][UD], k4[UPL][UD], k5[UPL][UD], k6[UPL][UD];
        stage_rhs(s, lane, w, u, gp, igp, M, cidx, t, u.x, k1);
#pragma unroll
        for (int j = 0; j < UPL; j++)
#pragma unroll
            for (int d = 0; d < UD; d++) X[j][d] = u.x[j][d] + (k1[j][d] * static_cast<P>(1.0 / 5.0)) * dt;
        stage_rhs(s, lane, w, u, gp, igp, M, cidx, t + static_cast<P>(1.0 / 5.0) * dt, X, k2);
#pragma unroll
        for (int j = 0; j < UPL; j++)
#pragma unroll
            for (int d = 0; d < UD; d++)
                X[j][d] = u.x[j][d] + (k1[j][d] * static_cast<P>(3.0 / 40.0) + k2[j][d] * static_cast<P>(9.0 / 40.0)) * dt;
        stage_rhs(s, lane, w, u, gp, igp, M, cidx, t + static_cast<P>(3.0 / 10.0) * dt, X, k3);
#pragma unroll
        for (int j = 0; j < UPL; j++)
#pragma unroll
            for (int d = 0; d < UD; d++)
                X[j][d] = u.x[j][d] + (k1[j][d] * static_cast<P>(3.0 / 10.0) + k2[j][d] * static_cast<P>(-9.0 / 10.0) +
                                       k3[j][d] * static_cast<P>(6.0 / 5.0)) * dt;
        stage_rhs(s, lane, w, u, gp, igp, M, cidx, t + static_cast<P>(3.0 / 5.0) * dt, X, k4);
#pragma unroll
        for (int j = 0; j < UPL; j++)
#pragma unroll
            for (int d = 0; d < UD; d++)
                X[j][d] = u.x[j][d] + (k1[j][d] * static_cast<P>(-11.0 / 54.0) + k2[j][d] * static_cast<P>(5.0 / 2.0) +
                                       k3[j][d] * static_cast<P>(-70.0 / 27.0) +
                                       k4[j][d] * static_cast<P>(35.0 / 27.0)) * dt;
        stage_rhs(s, lane, w, u, gp, igp, M, cidx, t + dt, X, k5);
#pragma unroll
        for (int j = 0; j < UPL; j++)
#pragma unroll
            for (int d = 0; d < UD; d++)
                X[j][d] = u.x[j][d] + (k1[j][d] * static_cast<P>(1631.0 / 55296.0) +
                                       k2[j][d] * static_cast<P>(175.0 / 512.0) +
                                       k3[j][d] * static_cast<P>(575.0 / 13824.0) +
                                       k4[j][d] * static_cast<P>(44275.0 / 110592.0) +
                                       k5[j][d] * static_cast<P>(253.0 / 4096.0)) * dt;
        stage_rhs(s, lane, w, u, gp, igp, M, cidx, t + static_cast<P>(7.0 / 8.0) * dt, X, k6);
#pragma unroll
        for (int j = 0; j < UPL; j++)
#pragma unroll
            for (int d = 0; d < UD; d++) {
                xn[j][d] = u.x[j][d] + (k1[j][d] * static_cast<P>(37.0 / 378.0) +
                                        k3[j][d] * static_cast<P>(250.0 / 621.0) +
                                        k4[j][d] * static_cast<P>(125.0 / 594.0) +
                                        k6[j][d] * static_cast<P>(512.0 / 1771.0)) * dt;
                P e = k1[j][d] * (static_cast<P>(37.0 / 378.0 - 2825.0 / 27648.0)) +
                      k3[j][d] * (static_cast<P>(250.0 / 621.0 - 18575.0 / 48384.0)) +
                      k4[j][d] * (static_cast<P>(125.0 / 594.0 - 13525.0 / 55296.0)) +
                      k5[j][d] * (static_cast<P>(0.0 - 277.0 / 14336.0)) +
                      k6[j][d] * (static_cast<P>(512.0 / 1771.0 - 1.0 / 4.0));
                err[j][d] = dt * abs(e) + static_cast<P>(1e-18);
                if (has(lane, j) && ((isfinite(xn[j][d]) == 0) || (isfinite(err[j][d]) == 0))) finite = 0;
            }
    }

    // ---- SPLIT ---------------------------------------------------------------------
    // double-float copies of the lane's unit states
    __device__ static void split_refresh_state(int lane, Units& u)
    {
#pragma unroll
        for (int j = 0; j < UPL; j++)
            if (has(lane, j))
#pragma unroll
                for (int d = 0; d < UD; d++) u.xd[j][d] = split_checked(u.x[j][d], u.range);
    }

    // double-float copies of the parameters and accessories (after the hooks
    // that may change them)
    __device__ static void split_refresh_params(int lane, const Slot& w, Units& u)
    {
#pragma unroll
        for (int k = 0; k < NSP; k++) u.spd[k] = split_checked(w.sp[k], u.range);
#pragma unroll
        for (int k = 0; k < NSA; k++) u.saccd[k] = split_checked(w.sacc[k], u.range);
#pragma unroll
        for (int j = 0; j < UPL; j++) {
            if (!has(lane, j)) continue;
#pragma unroll
            for (int k = 0; k < NUP; k++) u.upd[j][k] = split_checked(u.up[j][k], u.range);
#pragma unroll
            for (int k = 0; k < NUA; k++) u.uaccd[j][k] = split_checked(u.uacc[j][k], u.range);
        }
    }

    // stage_rhs of the split: the hook instantiated for dfloat on the
    // double-float copies, the coupling value and term in double-float
    __device__ static void stage_rhs_split(long long s, int lane, Slot& w, Units& u, const dfloat* gpd,
                                           const int* igp, const dfloat* Md, const int* cidx, dfloat T,
                                           dfloat (&X)[UPL][UD], dfloat (&F)[UPL][UD])
    {
        const int sid = static_cast<int>(s);
#pragma unroll
        for (int j = 0; j < UPL; j++) {
            if (has(lane, j)) {
                const int uid = unit_of(lane, j);
                CoupledSystems_PerBlock_OdeFunction<dfloat>(sid, uid, F[j], X[j], T, u.upd[j], u.spd,
                                                            const_cast<dfloat*>(gpd), const_cast<int*>(igp),
                                                            u.uaccd[j], u.iuacc[j], u.saccd, w.isacc, w.cpt[uid],
                                                            u.cpfd[j]);
            }
        }
        __syncwarp();
#pragma unroll
        for (int j = 0; j < UPL; j++) {
            if (has(lane, j)) {
                const int uid = unit_of(lane, j);
#pragma unroll
                for (int i = 0; i < NC; i++) {
                    const dfloat value = coupling_value<S, dfloat>(Md, w, uid, i);
                    const int c = cidx[i];
                    const dfloat term = w.cstr[i] * u.cpfd[j][i] * value;
#pragma unroll
                    for (int d = 0; d < UD; d++)
                        if (d == c) F[j][d] += term;
                }
            }
        }
        __syncwarp();
    }

    // RK4 step of the split: stages in double-float, then
    // x + dt (k1 + 2 k2 + 2 k3 + k4) / 6 in FP64 from the stage sum rounded
    // to FP64 (the reference's grouping, Steppers.cuh:1483-1692)
    __device__ static void step_rk4_split(long long s, int lane, Slot& w, Units& u, const dfloat* gpd, const int* igp,
                                          const dfloat* Md, const int* cidx, double t, double dt,
                                          double (&xn)[UPL][UD], int& finite)
    {
        using df::prod_sum;
        using df::prod_sum_add;
        using df::prod_sum_axpy;
        using df::prod_sum_start;
        const dfloat td = df::split(t), dtd = df::split(dt), half(0.5f);
        const dfloat th = df::fma(dtd, half, td);
        dfloat X[UPL][UD], k1[UPL][UD], k2[UPL][UD], k3[UPL][UD], k4[UPL][UD];
        stage_rhs_split(s, lane, w, u, gpd, igp, Md, cidx, td, u.xd, k1);
#pragma unroll
        for (int j = 0; j < UPL; j++)
#pragma unroll
            for (int d = 0; d < UD; d++) X[j][d] = prod_sum_axpy(dtd, prod_sum_start(half, k1[j][d]), u.xd[j][d]);
        stage_rhs_split(s, lane, w, u, gpd, igp, Md, cidx, th, X, k2);
#pragma unroll
        for (int j = 0; j < UPL; j++)
#pragma unroll
            for (int d = 0; d < UD; d++) X[j][d] = prod_sum_axpy(dtd, prod_sum_start(half, k2[j][d]), u.xd[j][d]);
        stage_rhs_split(s, lane, w, u, gpd, igp, Md, cidx, th, X, k3);
#pragma unroll
        for (int j = 0; j < UPL; j++)
#pragma unroll
            for (int d = 0; d < UD; d++) X[j][d] = prod_sum_axpy(dtd, prod_sum{k3[j][d].hi, k3[j][d].lo}, u.xd[j][d]);
        stage_rhs_split(s, lane, w, u, gpd, igp, Md, cidx, td + dtd, X, k4);
        const double sixth = dt * static_cast<double>(1.0 / 6.0);
#pragma unroll
        for (int j = 0; j < UPL; j++)
#pragma unroll
            for (int d = 0; d < UD; d++) {
                prod_sum sm = prod_sum_start(dfloat(1.0f), k1[j][d]);
                prod_sum_add(sm, dfloat(2.0f), k2[j][d]);
                prod_sum_add(sm, dfloat(2.0f), k3[j][d]);
                prod_sum_add(sm, dfloat(1.0f), k4[j][d]);
                xn[j][d] = __fma_rn(sixth, df::widen(sm.h) + df::widen(sm.l), u.x[j][d]);
                if (has(lane, j) && !finite_bits(xn[j][d])) finite = 0;
            }
    }

    // Cash-Karp 4(5) step of the split: stages and stage sums in
    // double-float, the update x + dt sum b k in FP64, the error sum kept as
    // its pair. The six stages run as one loop (the unit right-hand sides
    // and the coupling dot products inlined once instead of six times: the
    // instruction cache holds the step) whose weights come from the
    // constant tables above; every stage input, the solution sum and the
    // error sum accumulate their terms in the order of the per-thread split
    // (term j added when k_j is known), so the values are those of the
    // straight-line form.
    __device__ static void step_rkck45_split(long long s, int lane, Slot& w, Units& u, const dfloat* gpd,
                                             const int* igp, const dfloat* Md, const int* cidx, double t, double dt,
                                             double (&xn)[UPL][UD], df::prod_sum (&esum)[UPL][UD], int& finite)
    {
        using df::prod_sum;
        using df::prod_sum_add;
        using df::prod_sum_axpy;
        const dfloat td = df::split(t), dtd = df::split(dt);
        prod_sum acc[5][UPL][UD], sb[UPL][UD], se[UPL][UD];
#pragma unroll
        for (int j = 0; j < UPL; j++)
#pragma unroll
            for (int d = 0; d < UD; d++) {
#pragma unroll
                for (int r = 0; r < 5; r++) acc[r][j][d] = prod_sum{0.0f, 0.0f};
                sb[j][d] = prod_sum{0.0f, 0.0f};
                se[j][d] = prod_sum{0.0f, 0.0f};
            }
#pragma unroll 1
        for (int st = 0; st < 6; st++) {
            dfloat X[UPL][UD], k[UPL][UD];
            // stage input x + dt (sum_j a_st,j k_j): the accumulator of stage st
#pragma unroll
            for (int j = 0; j < UPL; j++)
#pragma unroll
                for (int d = 0; d < UD; d++) {
                    prod_sum a = acc[0][j][d];
#pragma unroll
                    for (int r = 1; r < 5; r++)
                        if (st == r + 1) a = acc[r][j][d];
                    X[j][d] = st == 0 ? u.xd[j][d] : prod_sum_axpy(dtd, a, u.xd[j][d]);
                }
            const float2 c = CK_C[st];
            const dfloat T = st == 0 ? td : (st == 4 ? td + dtd : df::fma(dtd, dfloat(c.x, c.y), td));
            stage_rhs_split(s, lane, w, u, gpd, igp, Md, cidx, T, X, k);
            // k_st into the inputs of the later stages and into the two sums
#pragma unroll
            for (int r = 0; r < 5; r++) {
                if (r + 1 > st) {
                    const float2 a = CK_A[r + 1][st];
                    const dfloat ad(a.x, a.y);
#pragma unroll
                    for (int j = 0; j < UPL; j++)
#pragma unroll
                        for (int d = 0; d < UD; d++) prod_sum_add(acc[r][j][d], ad, k[j][d]);
                }
            }
            const float2 b = CK_B[st], e = CK_E[st];
            if (b.x != 0.0f) {
#pragma unroll
                for (int j = 0; j < UPL; j++)
#pragma unroll
                    for (int d = 0; d < UD; d++) prod_sum_add(sb[j][d], dfloat(b.x, b.y), k[j][d]);
            }
            if (e.x != 0.0f) {
#pragma unroll
                for (int j = 0; j < UPL; j++)
#pragma unroll
                    for (int d = 0; d < UD; d++) prod_sum_add(se[j][d], dfloat(e.x, e.y), k[j][d]);
            }
        }
#pragma unroll
        for (int j = 0; j < UPL; j++)
#pragma unroll
            for (int d = 0; d < UD; d++) {
                // the unnormalised sum h + l rounded once to FP64; the error
                // sum kept as its pair (the controller forms its FP64
                // estimate where a decision or the factor needs it)
                const double b = df::widen(sb[j][d].h) + df::widen(sb[j][d].l);
                xn[j][d]   = __fma_rn(dt, b, u.x[j][d]);
                esum[j][d] = se[j][d];
                if (has(lane, j) && (!finite_bits(xn[j][d]) || !finite_float(se[j][d].h) ||
                                     !finite_float(se[j][d].l)))
                    finite = 0;
            }
    }

    // Step-size control of the split over the warp (the reference's coupled
    // controller, ErrorControllers.cuh:320-423, safety factor 0.8) on FP64
    // values with exact decisions and an FP64-accurate factor: every lane
    // scans its components with FP32 log2 estimates of
    // d = log2 tol - log2 err (err = dt |h + l| + 1e-18 of the double-float
    // error sum), deciding the accept test and its smallest ratio exactly in
    // FP64 inside a 1e-4 band; the warp takes the smallest estimate and, where
    // lanes tie within the band, the exact minimum of their ratios by
    // cross-multiplied FP64 products; the FP64 tolerance and error are formed
    // only for the lanes' candidates; then q = 0.8 R^(1/5) (1/4 after a
    // rejection) to FP64 accuracy where the clamp to [shrink, grow] does not
    // decide it alone.
    __device__ static void control_split(int lane, const Options<double>& o, float shrink_f, float grow_f, double dt,
                                         float dt_hi, const Units& u, const double (&xn)[UPL][UD],
                                         const df::prod_sum (&esum)[UPL][UD], const double* rtol,
                                         const double* atol, const float* lrtol, const float* latol, int& update,
                                         int& finite, int& terminate, double& new_dt, int& status)
    {
        float dmin = INFINITY;
        long long mag_m = 0;
        float eh_m = 0.0f, el_m = 0.0f;
        double err_m = 1.0, rtol_m = 0.0, atol_m = 0.0, tol_m = 0.0;
        bool tol_known = false, any = false;   // tol_known: tol_m and err_m formed
        int lane_update = 1;
#pragma unroll
        for (int j = 0; j < UPL; j++) {
            if (!has(lane, j)) continue;
#pragma unroll
            for (int d = 0; d < UD; d++) {
                const long long mag = max_bits(abs_bits(xn[j][d]), abs_bits(u.x[j][d]));
                const float lt = fmaxf(lrtol[d] + df::log2_estimate(from_bits(mag)), latol[d]);
                const float eh = esum[j][d].h, el = esum[j][d].l;
                const float di = lt - split_log2_error(dt_hi, eh, el);
                int accept_i;
                if (di > SPLIT_BAND) accept_i = 1;
                else if (di < -SPLIT_BAND) accept_i = 0;
                else accept_i = split_accepts(rtol[d], atol[d], mag, dt, eh, el);
                lane_update = lane_update & accept_i;
                bool take, settled = false;
                if (!any || di < dmin - SPLIT_BAND) {
                    take = true;
                } else if (di > dmin + SPLIT_BAND) {
                    take = false;
                } else {
                    const double tol_i = split_tolerance(rtol[d], atol[d], mag);
                    const double err_i = split_error(dt, eh, el);
                    if (!tol_known) {
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
                tol_known = settled || (!take && tol_known);
                if (take) {
                    dmin   = di;
                    mag_m  = mag;
                    eh_m   = eh;
                    el_m   = el;
                    rtol_m = rtol[d];
                    atol_m = atol[d];
                }
                any = true;
            }
        }
        update = warp_all(lane_update != 0) ? 1 : 0;
        // the warp's smallest ratio: the lanes within the band of the
        // smallest estimate, their ratios compared exactly where several are
        const float wmin = warp_minf(dmin);
        const bool cand = any && !(dmin > wmin + SPLIT_BAND);
        const unsigned cmask = __ballot_sync(0xffffffffu, cand);
        if (cand && !tol_known) {
            tol_m = from_bits(max_bits(bits_of(rtol_m * from_bits(mag_m)), bits_of(atol_m)));
            err_m = split_error(dt, eh_m, el_m);
        }
        int src = __ffs(cmask) - 1;
        double tol_w = __shfl_sync(0xffffffffu, tol_m, src);
        double err_w = __shfl_sync(0xffffffffu, err_m, src);
        float d_w = __shfl_sync(0xffffffffu, dmin, src);
        for (unsigned rest = cmask & (cmask - 1); rest != 0; rest &= rest - 1) {
            src = __ffs(rest) - 1;
            const double tol_o = __shfl_sync(0xffffffffu, tol_m, src);
            const double err_o = __shfl_sync(0xffffffffu, err_m, src);
            const float d_o = __shfl_sync(0xffffffffu, dmin, src);
            if (split_ratio_less(tol_o, err_o, tol_w, err_w)) {
                tol_w = tol_o;
                err_w = err_o;
                d_w = d_o;
            }
        }
        // the reference's initial ratio 1e30 caps R
        if (d_w > SPLIT_LOG2_RATIO_CAP + SPLIT_BAND ||
            (!(d_w < SPLIT_LOG2_RATIO_CAP - SPLIT_BAND) && !split_ratio_less(tol_w, err_w, 1e30, 1.0))) {
            d_w   = SPLIT_LOG2_RATIO_CAP;
            tol_w = 1e30;
            err_w = 1.0;
        }
        const bool fifth = (update == 1);
        const float y0 = df::root_estimate(d_w, fifth);
        const float qf = 0.8f * y0;
        double q;
        if (qf > shrink_f * (1.0f - 1e-5f) && qf < grow_f * (1.0f + 1e-5f))
            q = 0.8 * df::root_refine(y0, tol_w, err_w, fifth);
        else
            q = df::widen(qf);   // outside the limits by more than the estimate's error: the clamp decides
        if (!finite_bits(q)) finite = 0;
        const long long dtb = bits_of(dt), guardb = bits_of(o.min_dt_guard);
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

    // Integrate system s with the calling warp: the body of the reference's
    // MultipleSystems_SingleBlockLaunch kernel for one system
    // (CoupledSystmes_PerBlock_Solver.cuh:1575-2211).
    // SPLIT: gpd / Md the double-float global parameters and matrices the
    // right-hand side reads, lrtol / latol the log2 of the tolerances.
    __device__ static void system(long long s, int lane, Slot& w, const Args<SP>& a, const Options<P>& o,
                                  const P* gp, const int* igp, const P* M, const int* cidx, const P* rtol,
                                  const P* atol, const P* etol, const int* edir, const dfloat* gpd = nullptr,
                                  const dfloat* Md = nullptr, const float* lrtol = nullptr,
                                  const float* latol = nullptr)
    {
        const long long ns = a.ns, nu = a.ns * UPS;
        const int sid = static_cast<int>(s);
        Units u;
        // ---- load: system scope into the slot, unit scope into registers
        if (lane == 0) {
            w.td_in[0] = a.td[s];
            w.td_in[1] = a.td[s + ns];
            w.td[0] = P(w.td_in[0]);
            w.td[1] = P(w.td_in[1]);
            w.t = P(a.t[s]);
            w.dt = o.initial_dt;
            w.newdt = o.initial_dt;
            w.didx = a.didx[s];
            w.udt = 0;
            w.skipped = 0;
            w.dense_next = w.t;
        }
        for (int k = lane; k < NSP; k += 32) w.sp[k] = P(a.sp[s + k * ns]);
        for (int k = lane; k < NSA; k += 32) w.sacc[k] = P(a.sacc[s + k * ns]);
        for (int k = lane; k < NISA; k += 32) w.isacc[k] = a.isacc[s + k * ns];
        for (int k = lane; k < NC; k += 32) w.cstr[k] = P(a.cstr[s + k * ns]);
#pragma unroll
        for (int j = 0; j < UPL; j++) {
            if (!has(lane, j)) continue;
            const long long g = s * UPS + unit_of(lane, j);
#pragma unroll
            for (int d = 0; d < UD; d++) u.x[j][d] = P(a.x[g + d * nu]);
#pragma unroll
            for (int k = 0; k < NUP; k++) u.up[j][k] = P(a.up[g + k * nu]);
#pragma unroll
            for (int k = 0; k < NUA; k++) u.uacc[j][k] = P(a.uacc[g + k * nu]);
#pragma unroll
            for (int k = 0; k < NIUA; k++) u.iuacc[j][k] = a.iuacc[g + k * nu];
        }
        __syncwarp();

        P* gpm = const_cast<P*>(gp);
        int* igpm = const_cast<int*>(igp);
#pragma unroll
        for (int j = 0; j < UPL; j++)
            if (has(lane, j))
                CoupledSystems_PerBlock_Initialization<P>(sid, unit_of(lane, j), w.didx, w.t, w.dt, w.td, u.x[j],
                                                          u.up[j], w.sp, gpm, igpm, u.uacc[j], u.iuacc[j], w.sacc,
                                                          w.isacc);
        __syncwarp();
        if (NE > 0) {
#pragma unroll
            for (int j = 0; j < UPL; j++)
                if (has(lane, j))
                    CoupledSystems_PerBlock_EventFunction<P>(sid, unit_of(lane, j), u.ga[j], w.t, w.dt, w.td, u.x[j],
                                                             u.up[j], w.sp, gpm, igpm, u.uacc[j], u.iuacc[j], w.sacc,
                                                             w.isacc);
            __syncwarp();
        }
        if (o.ndo > 0) dense_store(s, lane, w, u, a, o, 1, 1);
        if constexpr (RECORD) record_checkpoint(s, lane, w, u, a, 0);
        float shrink_f = 0.0f, grow_f = 0.0f;
        if constexpr (SPLIT) {
            u.range = 0;
            split_refresh_state(lane, u);
            split_refresh_params(lane, w, u);
            shrink_f = static_cast<float>(o.shrink);
            grow_f = static_cast<float>(o.grow);
        }

        int status = 0, nacc = 0, nrej = 0, terminate = 0;
        long long attempts = 0;
        while (!terminate) {
            if (attempts >= o.max_attempts) {
                status |= MPGOS_INSTANCE_ATTEMPT_LIMIT;
                break;
            }
            attempts++;
            // ---- time stepping (CoupledSystmes_PerBlock_Solver.cuh:1839-1858)
            int update = 1, finite = 1, end_reached = 0;
            P dt = w.newdt;
            const P t = w.t;
            if (dt > (w.td[1] - t)) {
                dt = w.td[1] - t;
                end_reached = 1;
            }
            __syncwarp();
            if (lane == 0) w.dt = dt;
            __syncwarp();

            // ---- stepper
            P xn[UPL][UD], err[UPL][UD];
            df::prod_sum esum[UPL][UD];   // SPLIT: the double-float error sums
            if constexpr (SPLIT) {
                if (ALG == MPGOS_RK4) step_rk4_split(s, lane, w, u, gpd, igp, Md, cidx, t, dt, xn, finite);
                else step_rkck45_split(s, lane, w, u, gpd, igp, Md, cidx, t, dt, xn, esum, finite);
            } else if (ALG == MPGOS_RK4) {
                step_rk4(s, lane, w, u, gp, igp, M, cidx, t, dt, xn, finite);
            } else {
                step_rkck45(s, lane, w, u, gp, igp, M, cidx, t, dt, xn, err, finite);
            }
            finite = warp_all(finite != 0) ? 1 : 0;

            // ---- controller (..._ErrorControllers.cuh:320-423 for RKCK45, safety factor 0.8)
            P newdt;
            if (ALG == MPGOS_RK4) {
                // ..._ErrorControllers.cuh:286-316: a non-finite step stops
                // the system without being accepted
                if (finite == 0) {
                    terminate = 1;
                    update = 0;
                    status |= MPGOS_INSTANCE_NONFINITE;
                }
                newdt = o.initial_dt;
            } else if constexpr (SPLIT) {
                control_split(lane, o, shrink_f, grow_f, dt, df::split(dt).hi, u, xn, esum, rtol, atol, lrtol, latol,
                              update, finite, terminate, newdt, status);
            } else if constexpr (IS_DF<P>) {
                // DF_STAGE: exact double-float accept test, step factor
                // 0.8 * (min tol/err)^(1/5 or 1/4) from FP32 logarithms of the
                // leading floats (relative error ~1e-7), as in the per-thread
                // DF_STAGE controller.
                float lr = INFINITY;
                int lane_update = 1;
#pragma unroll
                for (int j = 0; j < UPL; j++) {
                    if (!has(lane, j)) continue;
                    for (int d = 0; d < UD; d++) {
                        const P tol = fmax(rtol[d] * fmax(fabs(xn[j][d]), fabs(u.x[j][d])), atol[d]);
                        lane_update = lane_update & (err[j][d] < tol);
                        lr = fminf(lr, __log2f(tol.hi) - __log2f(err[j][d].hi));
                    }
                }
                update = warp_all(lane_update != 0) ? 1 : 0;
                lr = warp_minf(lr);
                float q = 0.8f * exp2f(fminf(fmaxf(lr * ((update == 1) ? 0.2f : 0.25f), -120.0f), 120.0f));
                if (finite == 0) {
                    q = o.shrink.hi;
                    update = 0;
                    if (dt < o.min_dt_guard) {
                        terminate = 1;
                        status |= MPGOS_INSTANCE_NONFINITE;
                    }
                } else if (dt < o.min_dt_guard) {
                    update = 1;
                    status |= MPGOS_INSTANCE_MINIMUM_STEP;
                }
                q = fminf(fmaxf(q, o.shrink.hi), o.grow.hi);
                newdt = fmax(fmin(df::mul_f(dt, q), o.max_dt), o.min_dt);
            } else {
                P ratio = 1e30;
                int lane_update = 1;
#pragma unroll
                for (int j = 0; j < UPL; j++) {
                    if (!has(lane, j)) continue;
                    for (int d = 0; d < UD; d++) {
                        const P tol = fmax(rtol[d] * fmax(fabs(xn[j][d]), fabs(u.x[j][d])), atol[d]);
                        lane_update = lane_update & (err[j][d] < tol);
                        ratio = fmin(ratio, tol / err[j][d]);
                    }
                }
                update = warp_all(lane_update != 0) ? 1 : 0;
                ratio = warp_min(ratio);
                P q = (update == 1) ? static_cast<P>(0.8) * pow(ratio, static_cast<P>(1.0 / 5.0))
                                    : static_cast<P>(0.8) * pow(ratio, static_cast<P>(1.0 / 4.0));
                if (isfinite(q) == 0) finite = 0;
                if (finite == 0) {
                    q = o.shrink;
                    update = 0;
                    if (dt < o.min_dt_guard) {
                        terminate = 1;
                        status |= MPGOS_INSTANCE_NONFINITE;
                    }
                } else if (dt < o.min_dt_guard) {
                    update = 1;
                    status |= MPGOS_INSTANCE_MINIMUM_STEP;
                }
                q = fmin(q, o.grow);
                q = fmax(q, o.shrink);
                newdt = dt * q;
                newdt = fmin(newdt, o.max_dt);
                newdt = fmax(newdt, o.min_dt);
            }
            if (lane == 0) w.newdt = newdt;
            __syncwarp();

            // ---- events (CoupledSystems_PerBlock_EventHandling.cuh:149-214)
            P gn[UPL][AtLeastOne<NE>::value];
            if (NE > 0) {
#pragma unroll
                for (int j = 0; j < UPL; j++)
                    if (has(lane, j))
                        CoupledSystems_PerBlock_EventFunction<P>(sid, unit_of(lane, j), gn[j], t + dt, w.newdt, w.td,
                                                                 xn[j], u.up[j], w.sp, gpm, igpm, u.uacc[j],
                                                                 u.iuacc[j], w.sacc, w.isacc);
                __syncwarp();
                P evdt = dt;
                int corrected = 0;
                if (update == 1 && terminate == 0) {
#pragma unroll
                    for (int j = 0; j < UPL; j++) {
                        if (!has(lane, j)) continue;
                        for (int e = 0; e < NE; e++) {
                            if (((u.ga[j][e] > etol[e]) && (gn[j][e] < -etol[e]) && (edir[e] <= 0)) ||
                                ((u.ga[j][e] < -etol[e]) && (gn[j][e] > etol[e]) && (edir[e] >= 0))) {
                                evdt = fmin(evdt, -u.ga[j][e] / (gn[j][e] - u.ga[j][e]) * dt);
                                corrected = 1;
                            }
                        }
                    }
                }
                corrected = warp_any(corrected != 0) ? 1 : 0;
                evdt = warp_min(evdt);
                if (corrected == 1) {
                    if (evdt < o.min_dt) {
                        status |= MPGOS_INSTANCE_EVENT_OMITTED;
                    } else {
                        newdt = evdt;
                        update = 0;
                        if (lane == 0) w.newdt = newdt;
                    }
                }
                __syncwarp();
            }

            // ---- accept (CoupledSystmes_PerBlock_Solver.cuh:1975-2075)
            if (update == 1) {
                nacc++;
                if (lane == 0) {
                    if constexpr (IS_DF<P>) w.t = (end_reached == 1) ? w.td[1] : w.t + dt;
                    else w.t += dt;
                }
#pragma unroll
                for (int j = 0; j < UPL; j++)
#pragma unroll
                    for (int d = 0; d < UD; d++) u.x[j][d] = xn[j][d];
                __syncwarp();
#pragma unroll
                for (int j = 0; j < UPL; j++)
                    if (has(lane, j))
                        CoupledSystems_PerBlock_ActionAfterSuccessfulTimeStep<P>(
                            sid, unit_of(lane, j), w.udt, w.t, w.dt, w.td, u.x[j], u.up[j], w.sp, gpm, igpm,
                            u.uacc[j], u.iuacc[j], w.sacc, w.isacc);
                __syncwarp();
                if (NE > 0) {
#pragma unroll
                    for (int j = 0; j < UPL; j++) {
                        if (!has(lane, j)) continue;
                        for (int e = 0; e < NE; e++) {
                            if (pt::event_detected<P>(u.ga[j][e], gn[j][e], etol[e], edir[e]))
                                CoupledSystems_PerBlock_ActionAfterEventDetection<P>(
                                    sid, unit_of(lane, j), e, w.udt, w.t, w.dt, w.td, u.x[j], u.up[j], w.sp, gpm,
                                    igpm, u.uacc[j], u.iuacc[j], w.sacc, w.isacc);
                        }
                    }
                    __syncwarp();
#pragma unroll
                    for (int j = 0; j < UPL; j++)
                        if (has(lane, j))
                            CoupledSystems_PerBlock_EventFunction<P>(sid, unit_of(lane, j), gn[j], w.t, w.newdt,
                                                                     w.td, u.x[j], u.up[j], w.sp, gpm, igpm,
                                                                     u.uacc[j], u.iuacc[j], w.sacc, w.isacc);
                    __syncwarp();
#pragma unroll
                    for (int j = 0; j < UPL; j++)
#pragma unroll
                        for (int e = 0; e < NE; e++) u.ga[j][e] = gn[j][e];
                }
                if constexpr (SPLIT) {
                    // the accepted state and whatever the hooks changed
                    split_refresh_state(lane, u);
                    split_refresh_params(lane, w, u);
                }
                if constexpr (RECORD) {
                    // frozen step size of accepted step nacc, checkpoint every seg steps
                    const int k = nacc - 1;
                    if (k < a.tape.max_steps) {
                        if (lane == 0) a.tape.dt[static_cast<long long>(k) * ns + s] = static_cast<double>(dt);
                        if (nacc % a.tape.seg == 0) record_checkpoint(s, lane, w, u, a, nacc / a.tape.seg);
                    } else {
                        status |= MPGOS_INSTANCE_TAPE_OVERFLOW;
                    }
                }
            } else {
                nrej++;
            }
            if (o.ndo > 0) dense_store(s, lane, w, u, a, o, update, 0, end_reached);
            __syncwarp();
            if (update == 1 && ((end_reached == 1) || (w.udt == 1))) terminate = 1;
            __syncwarp();
        }

        // ---- finalisation and write back (CoupledSystmes_PerBlock_Solver.cuh:2128-2210)
#pragma unroll
        for (int j = 0; j < UPL; j++)
            if (has(lane, j))
                CoupledSystems_PerBlock_Finalization<P>(sid, unit_of(lane, j), w.didx, w.t, w.dt, w.td, u.x[j],
                                                        u.up[j], w.sp, gpm, igpm, u.uacc[j], u.iuacc[j], w.sacc,
                                                        w.isacc);
        __syncwarp();
        if constexpr (SPLIT) {
            if (warp_any(u.range != 0)) status |= MPGOS_INSTANCE_RANGE;
        }
#pragma unroll
        for (int j = 0; j < UPL; j++) {
            if (!has(lane, j)) continue;
            const long long g = s * UPS + unit_of(lane, j);
#pragma unroll
            for (int d = 0; d < UD; d++) a.x[g + d * nu] = stored(u.x[j][d], a.x[g + d * nu]);
#pragma unroll
            for (int k = 0; k < NUA; k++) a.uacc[g + k * nu] = stored(u.uacc[j][k], a.uacc[g + k * nu]);
#pragma unroll
            for (int k = 0; k < NIUA; k++) a.iuacc[g + k * nu] = u.iuacc[j][k];
        }
        if (lane == 0) {
            // DF_STAGE: values the run left equal to a time-domain bound are
            // written as the FP64 bound itself (a double-float holds 48 of its
            // 53 bits, so the round trip alone would move it)
            a.t[s] = (w.t == P(w.td_in[1])) ? w.td_in[1] : static_cast<SP>(w.t);
            a.td[s] = (w.td[0] == P(w.td_in[0])) ? w.td_in[0] : static_cast<SP>(w.td[0]);
            a.td[s + ns] = (w.td[1] == P(w.td_in[1])) ? w.td_in[1] : static_cast<SP>(w.td[1]);
            a.didx[s] = w.didx;
            if (a.status) a.status[s] = status;
            if (a.n_acc) a.n_acc[s] = nacc;
            if (a.n_rej) a.n_rej[s] = nrej;
            if constexpr (RECORD) a.tape.n_steps[s] = nacc;
        }
        for (int k = lane; k < NSA; k += 32) a.sacc[s + k * ns] = stored(w.sacc[k], a.sacc[s + k * ns]);
        for (int k = lane; k < NISA; k += 32) a.isacc[s + k * ns] = w.isacc[k];
        __syncwarp();
    }

    // Value to write back over `orig`, the FP64 value the launch loaded: in
    // DF_STAGE `orig` itself while the double-float still equals its
    // conversion (the round trip alone would move the last 5 bits of data the
    // run never changed), else the double-float's value.
    __device__ static SP stored(P v, SP orig)
    {
        if constexpr (IS_DF<P>) return (v == P(orig)) ? orig : static_cast<SP>(v);
        else return v;
    }

    // Checkpoint c of the adjoint tape: time and every unit's state.
    __device__ static void record_checkpoint(long long s, int lane, const Slot& w, const Units& u, const Args<SP>& a,
                                             int c)
    {
        const long long ns = a.ns, nu = a.ns * UPS;
        if (lane == 0) a.tape.ckpt_t[static_cast<long long>(c) * ns + s] = static_cast<double>(w.t);
#pragma unroll
        for (int j = 0; j < UPL; j++) {
            if (!has(lane, j)) continue;
            const long long g = s * UPS + unit_of(lane, j);
#pragma unroll
            for (int d = 0; d < UD; d++)
                a.tape.ckpt_x[(static_cast<long long>(c) * UD + d) * nu + g] = static_cast<double>(u.x[j][d]);
        }
    }

    // Dense output of one system (CoupledSystems_PerBlock_DenseOutput.cuh:210-312).
    // initial = 1: the unconditional store before the loop.
    __device__ static void dense_store(long long s, int lane, Slot& w, const Units& u, const Args<SP>& a,
                                       const Options<P>& o, int update, int initial, int end_reached = 0)
    {
        int store;
        if (initial) {
            store = 1;
        } else if (update == 1) {
            store = ((w.didx < o.ndo) && (w.dense_next < w.t) && (w.skipped >= (o.dense_freq - 1))) ? 1 : 0;
            if ((w.didx < o.ndo) && ((end_reached == 1) || (w.udt == 1))) store = 1;
        } else {
            store = 0;
        }
        const long long nu = a.ns * UPS;
        if (store == 1 && w.didx < o.ndo) {
#pragma unroll
            for (int j = 0; j < UPL; j++) {
                if (!has(lane, j)) continue;
                const long long g = s * UPS + unit_of(lane, j);
#pragma unroll
                for (int d = 0; d < UD; d++)
                    a.dstate[g + d * nu + static_cast<long long>(w.didx) * nu * UD] = static_cast<SP>(u.x[j][d]);
            }
            if (lane == 0) a.dtime[s + static_cast<long long>(w.didx) * a.ns] = static_cast<SP>(w.t);
        }
        __syncwarp();
        if (lane == 0) {
            if (store == 1) {
                if (w.didx < o.ndo) w.didx++;
                w.skipped = 0;
                w.dense_next = fmin(w.t + o.dense_min_dt, w.td[1]);
            }
            if (store == 0 && update == 1) w.skipped++;
        }
        __syncwarp();
    }
};

// Dynamic shared memory: [global parameters NGP][coupling matrices NC*MAT]
// [integer global parameters NIGP], padded to 16 bytes, then one WarpSlot per
// warp.
template <class S, class P>
__host__ __device__ constexpr size_t block_part_bytes(int shared_global, int shared_coupling)
{
    const size_t b = sizeof(P) * ((shared_global ? S::NGP : 0) + (shared_coupling ? S::NC * S::MAT : 0)) +
                     sizeof(int) * (shared_global ? S::NIGP : 0);
    return (b + 15) / 16 * 16;
}

template <class S, class P>
__host__ __device__ constexpr size_t dynamic_smem_bytes(int warps, int shared_global, int shared_coupling)
{
    return block_part_bytes<S, P>(shared_global, shared_coupling) + static_cast<size_t>(warps) * sizeof(WarpSlot<S, P>);
}

template <class S, int ALG, class P, int MODE>
__global__ void __launch_bounds__(MPGOS_CB_MAX_BLOCK) coupled_kernel(Args<typename StorageOf<P>::type> a)
{
    using Sv = Solver<S, ALG, P, MODE>;
    constexpr int UD = S::UD, NE = S::NE, NC = S::NC, NGP = S::NGP, NIGP = S::NIGP;
    constexpr bool ADAPTIVE = (ALG == MPGOS_RKCK45);
    constexpr bool SPLIT = Sv::SPLIT;
    // precision of the staged global parameters and matrices (those the
    // right-hand side reads)
    using RP = typename std::conditional<SPLIT, dfloat, P>::type;
    extern __shared__ __align__(16) unsigned char mpgos_cb_smem[];
    __shared__ P s_rtol[ADAPTIVE ? UD : 1];
    __shared__ P s_atol[ADAPTIVE ? UD : 1];
    __shared__ float s_lrtol[(ADAPTIVE && SPLIT) ? UD : 1];
    __shared__ float s_latol[(ADAPTIVE && SPLIT) ? UD : 1];
    __shared__ P s_etol[AtLeastOne<NE>::value];
    __shared__ int s_edir[AtLeastOne<NE>::value];
    __shared__ int s_cidx[AtLeastOne<NC>::value];

    // DF_STAGE converts every FP64 array it reads more than once into shared
    // memory: its layout always holds the global parameters and, where they
    // fit MPGOS_CB_DF_SHARED_MATRIX_BYTES, the coupling matrices; larger
    // matrices are read from the double-float copy the runtime keeps in global
    // memory. Both are compile-time facts of the shape (the runtime applies
    // the same rule), so the matrix loads are shared-memory loads whenever
    // the matrices sit there. SPLIT stages the same double-float copies for
    // its right-hand side; its FP64 hooks read the global parameters in HBM.
    constexpr bool CONVERT = IS_DF<P> || SPLIT;
    constexpr bool DF_SHARED_MATRIX =
        static_cast<size_t>(NC) * S::MAT * sizeof(dfloat) <= static_cast<size_t>(MPGOS_CB_DF_SHARED_MATRIX_BYTES);
    const int sg = CONVERT ? 1 : a.shared_global;
    const int sc = CONVERT ? (DF_SHARED_MATRIX ? 1 : 0) : a.shared_coupling;
    static_assert(sizeof(RP) == sizeof(P), "the staged layout is sized by the FP64 element");
    RP* dyn_gp = reinterpret_cast<RP*>(mpgos_cb_smem);
    RP* dyn_m = dyn_gp + (sg ? NGP : 0);
    int* dyn_igp = reinterpret_cast<int*>(dyn_m + (sc ? NC * S::MAT : 0));
    using Slot = typename Sv::Slot;
    static_assert(sizeof(Slot) == sizeof(WarpSlot<S, P>), "one slot size for every arithmetic");
    Slot* slots = reinterpret_cast<Slot*>(mpgos_cb_smem + block_part_bytes<S, P>(sg, sc));

    for (int k = threadIdx.x; k < UD; k += blockDim.x) {
        if (ADAPTIVE) {
            s_rtol[k] = P(a.rtol[k]);
            s_atol[k] = P(a.atol[k]);
            if constexpr (SPLIT) {
                s_lrtol[k] = df::log2_estimate(a.rtol[k]);
                s_latol[k] = df::log2_estimate(a.atol[k]);
            }
        }
    }
    for (int k = threadIdx.x; k < NE; k += blockDim.x) {
        s_etol[k] = P(a.etol[k]);
        s_edir[k] = a.edir[k];
    }
    for (int k = threadIdx.x; k < NC; k += blockDim.x) s_cidx[k] = a.cidx[k];
    if (sg) {
        for (int k = threadIdx.x; k < NGP; k += blockDim.x) dyn_gp[k] = RP(a.gp[k]);
        for (int k = threadIdx.x; k < NIGP; k += blockDim.x) dyn_igp[k] = a.igp[k];
    }
    if (sc)
        for (int k = threadIdx.x; k < NC * S::MAT; k += blockDim.x) dyn_m[k] = RP(a.cmat[k]);
    __syncthreads();

    const P* gp;
    const int* igp;
    const P* M;
    const dfloat* gpd = nullptr;
    const dfloat* Md = nullptr;
    if constexpr (SPLIT) {
        gp = reinterpret_cast<const P*>(a.gp);
        igp = dyn_igp;
        M = reinterpret_cast<const P*>(a.cmat);
        gpd = dyn_gp;
        Md = sc ? dyn_m : static_cast<const dfloat*>(a.cmat_df);
    } else if constexpr (CONVERT) {
        gp = dyn_gp;
        igp = dyn_igp;
        M = sc ? dyn_m : static_cast<const P*>(a.cmat_df);
    } else {
        gp = sg ? dyn_gp : reinterpret_cast<const P*>(a.gp);
        igp = sg ? dyn_igp : a.igp;
        M = sc ? dyn_m : reinterpret_cast<const P*>(a.cmat);
    }
    Options<P> o;
    o.initial_dt   = P(a.o.initial_dt);
    o.max_dt       = P(a.o.max_dt);
    o.min_dt       = P(a.o.min_dt);
    o.grow         = P(a.o.grow);
    o.shrink       = P(a.o.shrink);
    o.dense_min_dt = P(a.o.dense_min_dt);
    o.min_dt_guard = P(a.o.min_dt_guard);
    o.dense_freq   = a.o.dense_freq;
    o.ndo          = a.o.ndo;
    o.max_attempts = a.o.max_attempts;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int warps = blockDim.x >> 5;
    Slot& w = slots[warp];

    long long s = static_cast<long long>(blockIdx.x) * warps + warp;
    const long long total = static_cast<long long>(gridDim.x) * warps;
    while (s < a.n_active) {
        Sv::system(s, lane, w, a, o, gp, igp, M, s_cidx, s_rtol, s_atol, s_etol, s_edir, gpd, Md, s_lrtol, s_latol);
        if (!Sv::PERSISTENT) break;
        unsigned next = 0;
        if (lane == 0) next = atomicAdd(a.work, 1u);
        next = __shfl_sync(0xffffffffu, next, 0);
        s = total + static_cast<long long>(next);
    }
}

// ---- launch table --------------------------------------------------------------
template <class P>
Args<P> make_args(const mpgos_cb_launch& L)
{
    Args<P> a;
    a.ns = L.ns;
    a.n_active = L.n_active;
    a.td = static_cast<P*>(L.time_domain);
    a.t = static_cast<P*>(L.actual_time);
    a.sp = static_cast<P*>(L.system_parameters);
    a.sacc = static_cast<P*>(L.system_accessories);
    a.isacc = L.integer_system_accessories;
    a.cstr = static_cast<P*>(L.coupling_strength);
    a.didx = L.dense_index;
    a.dtime = static_cast<P*>(L.dense_time);
    a.x = static_cast<P*>(L.actual_state);
    a.up = static_cast<P*>(L.unit_parameters);
    a.uacc = static_cast<P*>(L.unit_accessories);
    a.iuacc = L.integer_unit_accessories;
    a.dstate = static_cast<P*>(L.dense_state);
    a.gp = static_cast<const P*>(L.global_parameters);
    a.igp = L.integer_global_parameters;
    a.cmat = static_cast<const P*>(L.coupling_matrix);
    a.cidx = L.coupling_index;
    a.rtol = static_cast<const P*>(L.relative_tolerance);
    a.atol = static_cast<const P*>(L.absolute_tolerance);
    a.etol = static_cast<const P*>(L.event_tolerance);
    a.edir = L.event_direction;
    a.status = L.status;
    a.n_acc = L.accepted_steps;
    a.n_rej = L.rejected_steps;
    a.work = L.work_counter;
    a.shared_global = L.shared_global;
    a.shared_coupling = L.shared_coupling;
    a.cmat_df = L.coupling_matrix_df;
    a.o.initial_dt = static_cast<P>(L.initial_dt);
    a.o.max_dt = static_cast<P>(L.max_dt);
    a.o.min_dt = static_cast<P>(L.min_dt);
    a.o.grow = static_cast<P>(L.grow_limit);
    a.o.shrink = static_cast<P>(L.shrink_limit);
    a.o.dense_min_dt = static_cast<P>(L.dense_min_dt);
    a.o.min_dt_guard = a.o.min_dt * static_cast<P>(1.01);
    a.o.dense_freq = L.dense_save_frequency;
    a.o.ndo = L.ndo;
    a.o.max_attempts = L.max_attempts;
    return a;
}

template <class S, int ALG, class P>
struct KernelTable {
    static constexpr bool HAS_DF = std::is_same<P, double>::value;

    static void* kernel_for(int mode)
    {
        if constexpr (HAS_DF) {
            if (mode & MPGOS_MODE_DF_STAGE)
                return (mode & MPGOS_MODE_PERSISTENT)
                           ? reinterpret_cast<void*>(&coupled_kernel<S, ALG, dfloat, MPGOS_MODE_PERSISTENT>)
                           : reinterpret_cast<void*>(&coupled_kernel<S, ALG, dfloat, 0>);
            if (mode & MPGOS_MODE_SPLIT)
                return (mode & MPGOS_MODE_PERSISTENT)
                           ? reinterpret_cast<void*>(
                                 &coupled_kernel<S, ALG, double, MPGOS_MODE_SPLIT | MPGOS_MODE_PERSISTENT>)
                           : reinterpret_cast<void*>(&coupled_kernel<S, ALG, double, MPGOS_MODE_SPLIT>);
        }
        return (mode & MPGOS_MODE_PERSISTENT) ? reinterpret_cast<void*>(&coupled_kernel<S, ALG, P, MPGOS_MODE_PERSISTENT>)
                                              : reinterpret_cast<void*>(&coupled_kernel<S, ALG, P, 0>);
    }
    static int launch(const mpgos_cb_launch* L, int grid, int block, size_t smem, void* stream)
    {
        Args<P> a = make_args<P>(*L);
        void* params[] = {&a};
        void* fn = kernel_for(L->mode);
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
            if (e != cudaSuccess) return static_cast<int>(e);
        }
        return static_cast<int>(cudaLaunchKernel(fn, dim3(grid), dim3(block), params, smem,
                                                 static_cast<cudaStream_t>(stream)));
    }
    static int occupancy(int32_t mode, int block, size_t smem, int* blocks)
    {
        void* fn = kernel_for(mode);
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
            if (e != cudaSuccess) return static_cast<int>(e);
        }
        return static_cast<int>(cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, fn, block, smem));
    }
    static size_t smem(int warps, int shared_global, int shared_coupling)
    {
        return dynamic_smem_bytes<S, P>(warps, shared_global, shared_coupling);
    }
    using RecordFn  = int (*)(const mpgos_cb_launch*, const mpgos_pt_tape*, int, int, size_t, void*);
    using AdjointFn = int (*)(const mpgos_cb_launch*, const mpgos_pt_tape*, const double*, double*, double*, int, int,
                              size_t, void*);
    using AdjSmemFn = size_t (*)(int, int32_t);
    using AdjOccFn  = int (*)(int32_t, int, size_t, int*);

    static const mpgos_cb_kernels* get(const char* name, RecordFn record = nullptr, AdjointFn adjoint = nullptr,
                                       AdjSmemFn adjoint_smem = nullptr, AdjOccFn adjoint_occupancy = nullptr)
    {
        static mpgos_cb_kernels table = {
            MPGOS_ABI_VERSION,
            {S::UPS, S::UD, S::NC, S::CBW, S::CCI, S::NUP, S::NSP, S::NGP, S::NIGP, S::NUA, S::NIUA, S::NSA, S::NISA,
             S::NE, ALG, static_cast<int32_t>(sizeof(P)), S::MAT},
            name,
            &launch,
            &occupancy,
            &smem,
            record,
            adjoint,
            adjoint_smem,
            adjoint_occupancy};
        return &table;
    }
};

}  // namespace cb
}  // namespace mpgos

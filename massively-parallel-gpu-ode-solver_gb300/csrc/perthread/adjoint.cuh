// Discrete adjoint of the per-thread explicit Runge-Kutta integration
// (extension: the reference has no differentiation).
//
// Forward (recording) pass: the ordinary solver kernel compiled with
// MODE_RECORD (kernel.cuh) stores, per instance, every accepted step size (the
// frozen step sequence, including event-refined and end-clamped steps) and a
// checkpoint of time and state every SEG accepted steps.
//
// Reverse pass (this file, one instance per thread): for each segment, last
// first, the states at every step of the segment are recomputed from the
// checkpoint with the recorded step sizes (bit-identical to the forward pass:
// the same stepper code), then the adjoint is propagated backwards through the
// Runge-Kutta stages of every step:
//     kappa_i = dt b_i lambda + sum_{j>i} dt a_ji xi_j,   xi_i = J_x(X_i)^T kappa_i,
//     mu     += J_p(X_i)^T kappa_i,                        lambda <- lambda + sum_i xi_i,
// where J = [df/dx | df/dp] at the stage points comes from one evaluation of
// the user's PerThread_OdeFunction instantiated with dual numbers. The result
// is the exact gradient of the discrete map with the step sequence frozen,
// d L / d x(t0) and d L / d cPAR, for a terminal loss whose gradient
// d L / d x(T) the caller supplies.
//
// Scope: the control parameters are the differentiated parameters; hooks
// that change the state outside the right-hand side (event actions, step
// actions, Initialization) are not differentiated.
#pragma once

#include "dual.cuh"
#include "kernel.cuh"

namespace mpgos {
namespace pt {

// Butcher tableaux of the two schemes (mathematical coefficients; the
// reference's RK4 accumulates k1 + 2k2 + 2k3 + k4, which is this tableau).
template <int ALG> struct Tableau;
template <> struct Tableau<MPGOS_RKCK45> {
    static constexpr int S = 6;
    __device__ static double a(int i, int j) {
        const double A[6][5] = {{0, 0, 0, 0, 0},
                                {1.0 / 5.0, 0, 0, 0, 0},
                                {3.0 / 40.0, 9.0 / 40.0, 0, 0, 0},
                                {3.0 / 10.0, -9.0 / 10.0, 6.0 / 5.0, 0, 0},
                                {-11.0 / 54.0, 5.0 / 2.0, -70.0 / 27.0, 35.0 / 27.0, 0},
                                {1631.0 / 55296.0, 175.0 / 512.0, 575.0 / 13824.0, 44275.0 / 110592.0, 253.0 / 4096.0}};
        return A[i][j];
    }
    __device__ static double b(int i) {
        const double B[6] = {37.0 / 378.0, 0.0, 250.0 / 621.0, 125.0 / 594.0, 0.0, 512.0 / 1771.0};
        return B[i];
    }
    __device__ static double c(int i) {
        const double Cc[6] = {0.0, 1.0 / 5.0, 3.0 / 10.0, 3.0 / 5.0, 1.0, 7.0 / 8.0};
        return Cc[i];
    }
};
template <> struct Tableau<MPGOS_RK4> {
    static constexpr int S = 4;
    __device__ static double a(int i, int j) {
        const double A[4][3] = {{0, 0, 0}, {0.5, 0, 0}, {0, 0.5, 0}, {0, 0, 1.0}};
        return A[i][j];
    }
    __device__ static double b(int i) {
        const double B[4] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};
        return B[i];
    }
    __device__ static double c(int i) {
        const double Cc[4] = {0.0, 0.5, 0.5, 1.0};
        return Cc[i];
    }
};

// The tableau in the arithmetic type T of a reverse pass (double, or
// double-float for DF_STAGE), staged once per CTA in shared memory so that no
// per-use conversion is needed.
template <class T, int ST>
struct TableauT {
    T a[ST][ST];
    T b[ST];
    T c[ST];
};

// Coefficient access: FP64 passes use the compile-time constants directly
// (immediate operands after unrolling), double-float passes the staged pairs.
template <class TB, class T>
__device__ __forceinline__ T tab_a(const TableauT<T, TB::S>& tb, int i, int j)
{
    if constexpr (std::is_same<T, double>::value) return TB::a(i, j);
    else return tb.a[i][j];
}
template <class TB, class T>
__device__ __forceinline__ T tab_b(const TableauT<T, TB::S>& tb, int i)
{
    if constexpr (std::is_same<T, double>::value) return TB::b(i);
    else return tb.b[i];
}
template <class TB, class T>
__device__ __forceinline__ T tab_c(const TableauT<T, TB::S>& tb, int i)
{
    if constexpr (std::is_same<T, double>::value) return TB::c(i);
    else return tb.c[i];
}

template <class TB, class T>
__device__ void stage_tableau(TableauT<T, TB::S>& tb)
{
    for (int k = threadIdx.x; k < TB::S * TB::S; k += blockDim.x) {
        const int i = k / TB::S, j = k % TB::S;
        tb.a[i][j] = T(j < i ? TB::a(i, j) : 0.0);
    }
    for (int k = threadIdx.x; k < TB::S; k += blockDim.x) {
        tb.b[k] = T(TB::b(k));
        tb.c[k] = T(TB::c(k));
    }
}

// Maximum segment length compiled into the reverse kernel (local-memory
// buffer of the replayed states).
constexpr int MAX_SEG = 64;

// Local-memory budget (8-byte values) for keeping a whole segment's stage
// Jacobians; 0 always takes the replay-and-re-evaluate form.
#ifndef MPGOS_ADJOINT_JBUF_VALUES
#define MPGOS_ADJOINT_JBUF_VALUES 4096
#endif
constexpr int JBUF_DOUBLES = MPGOS_ADJOINT_JBUF_VALUES;

// Launch shape of the reverse pass: fixed block, and the resident blocks per
// SM the register allocation is held to: FP64 passes (FP64-pipe bound, local
// Jacobian buffer) take occupancy, double-float passes registers (the
// segment-tangent form keeps every stage's dual values in registers).
#ifndef MPGOS_ADJOINT_MIN_BLOCKS
#define MPGOS_ADJOINT_MIN_BLOCKS 12
#endif
#ifndef MPGOS_ADJOINT_MIN_BLOCKS_DF
#define MPGOS_ADJOINT_MIN_BLOCKS_DF 4
#endif
constexpr int ADJOINT_BLOCK = 64;
template <class T>
struct AdjointMinBlocks {
    static constexpr int value = std::is_same<T, double>::value ? MPGOS_ADJOINT_MIN_BLOCKS : MPGOS_ADJOINT_MIN_BLOCKS_DF;
};

// Largest SD x (SD + NCP + 1) (dual values of the state) for which a
// double-float reverse pass takes the segment-tangent form; 0 disables it.
#ifndef MPGOS_ADJOINT_TANGENT_MAX
#define MPGOS_ADJOINT_TANGENT_MAX 16
#endif
constexpr int ADJOINT_TANGENT_MAX = MPGOS_ADJOINT_TANGENT_MAX;
constexpr int ADJOINT_MIN_BLOCKS = MPGOS_ADJOINT_MIN_BLOCKS;

// Stage values K and Jacobians J = [df/dx | df/dp] of one step from (x, t)
// with step dt, by dual-number evaluation of the user's right-hand side at
// the stage points X_st = x + dt * sum_j a_st,j K_j.
template <class TB, int ST, int SD, int N, class D, class T>
__device__ __forceinline__ void dual_stages(const TableauT<T, ST>& tb, int ti, int nti, const T* x, T t, T dt, D* cpd,
                                            D* spd, int* spi, D* accd, int* acci, T (&K)[ST][SD],
                                            T (&J)[ST][SD][N])
{
    for (int st = 0; st < ST; st++) {
        D Xd[SD];
        D Fd[SD];
#pragma unroll
        for (int d = 0; d < SD; d++) {
            T sum(0.0);
            for (int j = 0; j < st; j++) sum += tab_a<TB>(tb, st, j) * K[j][d];
            Xd[d] = D(x[d] + dt * sum);
            Xd[d].d[d] = T(1.0);
        }
        const D Td(t + tab_c<TB>(tb, st) * dt);
        PerThread_OdeFunction(ti, nti, Fd, Xd, Td, cpd, spd, spi, accd, acci);
#pragma unroll
        for (int d = 0; d < SD; d++) {
            K[st][d] = Fd[d].v;
#pragma unroll
            for (int q = 0; q < N; q++) J[st][d][q] = Fd[d].d[q];
        }
    }
}

// Adjoint of one Runge-Kutta step with frozen dt: lambda <- lambda + sum_i xi_i,
// mu += sum_i J_p,i^T kappa_i (see the header comment).
template <class TB, int ST, int SD, int N, int NCP, class T>
__device__ __forceinline__ void reverse_step(const TableauT<T, ST>& tb, const T (&J)[ST][SD][N], T dt, T* lam, T* mu)
{
    T kap[ST][SD];
    for (int st = 0; st < ST; st++)
#pragma unroll
        for (int d = 0; d < SD; d++) kap[st][d] = dt * tab_b<TB>(tb, st) * lam[d];
    T dlam[SD];
#pragma unroll
    for (int d = 0; d < SD; d++) dlam[d] = T(0.0);
    for (int st = ST - 1; st >= 0; st--) {
        T xi[SD];
#pragma unroll
        for (int r = 0; r < SD; r++) {
            T v(0.0);
#pragma unroll
            for (int d = 0; d < SD; d++) v += J[st][d][r] * kap[st][d];
            xi[r] = v;
        }
#pragma unroll
        for (int q = 0; q < NCP; q++) {
            T v(0.0);
#pragma unroll
            for (int d = 0; d < SD; d++) v += J[st][d][SD + q] * kap[st][d];
            mu[q] += v;
        }
        for (int j = 0; j < st; j++) {
            if (TB::a(st, j) != 0.0) {
                const T w = dt * tab_a<TB>(tb, st, j);
#pragma unroll
                for (int d = 0; d < SD; d++) kap[j][d] += w * xi[d];
            }
        }
#pragma unroll
        for (int d = 0; d < SD; d++) dlam[d] += xi[d];
    }
#pragma unroll
    for (int d = 0; d < SD; d++) lam[d] += dlam[d];
}

// y += a x for dual numbers and a plain coefficient a.
template <int N, class T>
__device__ __forceinline__ void dual_axpy(ad::Dual<N, T>& y, T a, const ad::Dual<N, T>& x)
{
    y.v = ad::mad(a, x.v, y.v);
#pragma unroll
    for (int q = 0; q < N; q++) y.d[q] = ad::mad(a, x.d[q], y.d[q]);
}
// x + sum_j h_j K_j for double-float duals, every component accumulated as
// an unnormalised product sum (df::prod_sum, 12 FP32 operations per term)
// and normalised once.
template <int N>
struct DualSum {
    df::prod_sum v;
    df::prod_sum d[N];
};
template <int N>
__device__ __forceinline__ DualSum<N> dual_sum_from(const ad::Dual<N, dfloat>& x)
{
    DualSum<N> s;
    s.v = df::prod_sum{x.v.hi, x.v.lo};
#pragma unroll
    for (int q = 0; q < N; q++) s.d[q] = df::prod_sum{x.d[q].hi, x.d[q].lo};
    return s;
}
template <int N>
__device__ __forceinline__ void dual_sum_add(DualSum<N>& s, dfloat h, const ad::Dual<N, dfloat>& k)
{
    df::prod_sum_add(s.v, h, k.v);
#pragma unroll
    for (int q = 0; q < N; q++) df::prod_sum_add(s.d[q], h, k.d[q]);
}
template <int N>
__device__ __forceinline__ ad::Dual<N, dfloat> dual_sum_value(const DualSum<N>& s)
{
    ad::Dual<N, dfloat> r;
    r.v = df::prod_sum_value(s.v);
#pragma unroll
    for (int q = 0; q < N; q++) r.d[q] = df::prod_sum_value(s.d[q]);
    return r;
}

// One Runge-Kutta step with frozen dt carried out entirely in dual numbers:
// x holds the state and its tangents d x / d (segment start state, control
// parameters); on return, the state and tangents one step later.
template <class TB, int ST, int SD, int N, class D, class T>
__device__ __forceinline__ void tangent_step(const TableauT<T, ST>& tb, int ti, int nti, D* x, T t, T dt, D* cpd,
                                             D* spd, int* spi, D* accd, int* acci)
{
    // stage sums with the step folded into the coefficients: X_st = x + sum_j (dt a_st,j) K_j
    constexpr bool DF = std::is_same<T, dfloat>::value;
    D K[ST][SD];
#pragma unroll
    for (int st = 0; st < ST; st++) {
        D Xd[SD];
        if constexpr (DF) {
#pragma unroll
            for (int d = 0; d < SD; d++) {
                DualSum<N> acc = dual_sum_from(x[d]);
#pragma unroll
                for (int j = 0; j < st; j++)
                    if (TB::a(st, j) != 0.0) dual_sum_add(acc, dt * tab_a<TB>(tb, st, j), K[j][d]);
                Xd[d] = dual_sum_value(acc);
            }
        } else {
#pragma unroll
            for (int d = 0; d < SD; d++) Xd[d] = x[d];
#pragma unroll
            for (int j = 0; j < st; j++) {
                if (TB::a(st, j) != 0.0) {
                    const T h = dt * tab_a<TB>(tb, st, j);
#pragma unroll
                    for (int d = 0; d < SD; d++) dual_axpy(Xd[d], h, K[j][d]);
                }
            }
        }
        const D Td(ad::mad(tab_c<TB>(tb, st), dt, t));
        PerThread_OdeFunction(ti, nti, K[st], Xd, Td, cpd, spd, spi, accd, acci);
    }
    if constexpr (DF) {
#pragma unroll
        for (int d = 0; d < SD; d++) {
            DualSum<N> acc = dual_sum_from(x[d]);
#pragma unroll
            for (int st = 0; st < ST; st++)
                if (TB::b(st) != 0.0) dual_sum_add(acc, dt * tab_b<TB>(tb, st), K[st][d]);
            x[d] = dual_sum_value(acc);
        }
    } else {
#pragma unroll
        for (int st = 0; st < ST; st++) {
            if (TB::b(st) != 0.0) {
                const T h = dt * tab_b<TB>(tb, st);
#pragma unroll
                for (int d = 0; d < SD; d++) dual_axpy(x[d], h, K[st][d]);
            }
        }
    }
}

// T is the arithmetic type of the reverse pass: double, or double-float
// (dfloat, ~48-bit significand on the FP32 pipe) for DF_STAGE solvers. The
// tape is FP64 either way; a DF forward pass records its double-float steps
// and checkpoints exactly (hi + lo of a normalised pair fits a double).
template <class S, int ALG, class T>
__global__ void __launch_bounds__(ADJOINT_BLOCK, AdjointMinBlocks<T>::value) adjoint_kernel(Args<double> a, Tape tp, const double* dLdxT,
                                                                  double* dLdx0, double* dLdp)
{
    constexpr int SD = S::SD, NCP = S::NCP, NSP = S::NSP, NISP = S::NISP, NA = S::NA, NIA = S::NIA;
    constexpr int N = SD + NCP;  // dual directions: state, then control parameters
    using D = ad::Dual<N, T>;
    using TB = Tableau<ALG>;
    constexpr int ST = TB::S;
    static_assert(sizeof(T) == sizeof(double), "shared parameter layout assumes 8-byte values");
    // Keep a segment's stage Jacobians when they fit the local-memory budget;
    // otherwise replay the states and re-evaluate the dual stages per step.
    constexpr bool STORE_J = MAX_SEG * ST * SD * N <= JBUF_DOUBLES;
    // Double-float reverse passes of small systems propagate tangents through
    // each segment instead (no per-step storage; see below).
    constexpr bool TANGENT = !std::is_same<T, double>::value && SD * (N + 1) <= ADJOINT_TANGENT_MAX;

    extern __shared__ __align__(16) unsigned char mpgos_dyn_smem[];
    __shared__ TableauT<T, ST> tb;
    T* sp    = reinterpret_cast<T*>(mpgos_dyn_smem);
    int* spi = reinterpret_cast<int*>(mpgos_dyn_smem + sizeof(T) * NSP);
    for (int k = threadIdx.x; k < NSP; k += blockDim.x) sp[k] = T(a.sp[k]);
    for (int k = threadIdx.x; k < NISP; k += blockDim.x) spi[k] = a.spi[k];
    stage_tableau<TB>(tb);
    __syncthreads();

    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= a.n_active) return;
    const long long nt = a.nt;
    const int ti = static_cast<int>(i), nti = static_cast<int>(nt);

    T cp[AtLeastOne<NCP>::value];
    T acc[AtLeastOne<NA>::value];
    int acci[AtLeastOne<NIA>::value];
#pragma unroll
    for (int k = 0; k < NCP; k++) cp[k] = T(a.cp[i + k * nt]);
#pragma unroll
    for (int k = 0; k < NA; k++) acc[k] = T(a.acc[i + k * nt]);
#pragma unroll
    for (int k = 0; k < NIA; k++) acci[k] = a.acci[i + k * nt];

    // dual copies of the constant inputs
    D cpd[AtLeastOne<NCP>::value];
    D spd[AtLeastOne<NSP>::value];
    D accd[AtLeastOne<NA>::value];
#pragma unroll
    for (int k = 0; k < NCP; k++) {
        cpd[k] = D(cp[k]);
        cpd[k].d[SD + k] = T(1.0);
    }
    for (int k = 0; k < NSP; k++) spd[k] = D(sp[k]);
#pragma unroll
    for (int k = 0; k < NA; k++) accd[k] = D(acc[k]);

    T lam[SD];
    T mu[AtLeastOne<NCP>::value];
#pragma unroll
    for (int d = 0; d < SD; d++) lam[d] = T(dLdxT[d * nt + i]);
#pragma unroll
    for (int k = 0; k < NCP; k++) mu[k] = T(0.0);

    const int n = tp.n_steps[i];
    int status = a.status ? a.status[i] : 0;
    if (n > tp.max_steps) status |= MPGOS_INSTANCE_TAPE_OVERFLOW;

    const int seg = tp.seg;

    if constexpr (TANGENT) {
        // Segment by segment, last first: replay the segment from its
        // checkpoint with every value a dual number seeded with the identity
        // on the state (the control parameters are seeded in cpd), so that
        // at the segment end the duals hold the segment's Jacobians
        // Phi = d x_end / d x_start and Psi = d x_end / d cPAR. Then
        //     mu += Psi^T lambda,   lambda <- Phi^T lambda.
        // This is the same discrete gradient as the per-step reverse sweep
        // (the chain rule through the same frozen steps, multiplied in another
        // order); it trades the stored stage Jacobians for SD x N more
        // arithmetic per stage sum, which pays where the Jacobian buffer would
        // go to DRAM and the arithmetic runs on the FP32 pipe.
        if (!(status & MPGOS_INSTANCE_TAPE_OVERFLOW) && n > 0) {
            for (int sgm = (n - 1) / seg; sgm >= 0; sgm--) {
                const int k0 = sgm * seg;
                const int k1 = min(n, k0 + seg);
                D xd[SD];
                T t(tp.ckpt_t[static_cast<long long>(sgm) * nt + i]);
#pragma unroll
                for (int d = 0; d < SD; d++) {
                    xd[d] = D(T(tp.ckpt_x[(static_cast<long long>(sgm) * SD + d) * nt + i]));
                    xd[d].d[d] = T(1.0);
                }
                for (int k = k0; k < k1; k++) {
                    const T dt(tp.dt[static_cast<long long>(k) * nt + i]);
                    tangent_step<TB, ST, SD, N>(tb, ti, nti, xd, t, dt, cpd, spd, spi, accd, acci);
                    t += dt;
                }
#pragma unroll
                for (int q = 0; q < NCP; q++) {
#pragma unroll
                    for (int d = 0; d < SD; d++) mu[q] += xd[d].d[SD + q] * lam[d];
                }
                T ln[SD];
#pragma unroll
                for (int r = 0; r < SD; r++) {
                    T v(0.0);
#pragma unroll
                    for (int d = 0; d < SD; d++) v += xd[d].d[r] * lam[d];
                    ln[r] = v;
                }
#pragma unroll
                for (int d = 0; d < SD; d++) lam[d] = ln[d];
            }
        }
    } else if constexpr (STORE_J) {
        // One forward pass per segment with dual-number stages: the stage
        // values advance the state (tableau form of the step), the stage
        // Jacobians are kept in local memory, then the segment is swept
        // backwards with algebra only. One right-hand-side evaluation per
        // stage and step in the whole reverse pass.
        T Jseg[MAX_SEG][ST][SD][N];
        if (!(status & MPGOS_INSTANCE_TAPE_OVERFLOW) && n > 0) {
            for (int sgm = (n - 1) / seg; sgm >= 0; sgm--) {
                const int k0 = sgm * seg;
                const int k1 = min(n, k0 + seg);
                T x[SD];
                T t(tp.ckpt_t[static_cast<long long>(sgm) * nt + i]);
#pragma unroll
                for (int d = 0; d < SD; d++) x[d] = T(tp.ckpt_x[(static_cast<long long>(sgm) * SD + d) * nt + i]);
                for (int k = k0; k < k1; k++) {
                    const T dt(tp.dt[static_cast<long long>(k) * nt + i]);
                    T K[ST][SD];
                    dual_stages<TB, ST, SD, N>(tb, ti, nti, x, t, dt, cpd, spd, spi, accd, acci, K, Jseg[k - k0]);
                    if (k + 1 < k1) {
#pragma unroll
                        for (int d = 0; d < SD; d++) {
                            T sum(0.0);
                            for (int st = 0; st < ST; st++) sum += tab_b<TB>(tb, st) * K[st][d];
                            x[d] = x[d] + dt * sum;
                        }
                        t += dt;
                    }
                }
                for (int k = k1 - 1; k >= k0; k--)
                    reverse_step<TB, ST, SD, N, NCP>(tb, Jseg[k - k0], T(tp.dt[static_cast<long long>(k) * nt + i]),
                                                     lam, mu);
            }
        }
    } else {
    T xs[MAX_SEG][SD];
    T ts[MAX_SEG];
    if (!(status & MPGOS_INSTANCE_TAPE_OVERFLOW) && n > 0) {
        for (int sgm = (n - 1) / seg; sgm >= 0; sgm--) {
            const int k0 = sgm * seg;
            const int k1 = min(n, k0 + seg);
            // replay the segment with the recorded steps
            T x[SD];
            T t(tp.ckpt_t[static_cast<long long>(sgm) * nt + i]);
#pragma unroll
            for (int d = 0; d < SD; d++) x[d] = T(tp.ckpt_x[(static_cast<long long>(sgm) * SD + d) * nt + i]);
            for (int k = k0; k < k1; k++) {
                const T dt(tp.dt[static_cast<long long>(k) * nt + i]);
#pragma unroll
                for (int d = 0; d < SD; d++) xs[k - k0][d] = x[d];
                ts[k - k0] = t;
                if (k + 1 < k1) {
                    T xn[SD], err[SD];
                    int finite = 1;
                    if (ALG == MPGOS_RK4)
                        step_rk4<SD, T>(ti, nti, t, dt, x, xn, finite, cp, sp, spi, acc, acci);
                    else
                        step_rkck45<SD, T, false>(ti, nti, t, dt, x, xn, err, finite, cp, sp, spi, acc, acci);
#pragma unroll
                    for (int d = 0; d < SD; d++) x[d] = xn[d];
                    t += dt;
                }
            }
            // reverse through the segment, re-evaluating the dual stages
            for (int k = k1 - 1; k >= k0; k--) {
                const T dt(tp.dt[static_cast<long long>(k) * nt + i]);
                T K[ST][SD];
                T J[ST][SD][N];
                dual_stages<TB, ST, SD, N>(tb, ti, nti, xs[k - k0], ts[k - k0], dt, cpd, spd, spi, accd, acci, K, J);
                reverse_step<TB, ST, SD, N, NCP>(tb, J, dt, lam, mu);
            }
        }
    }
    }
#pragma unroll
    for (int d = 0; d < SD; d++) dLdx0[d * nt + i] = static_cast<double>(lam[d]);
#pragma unroll
    for (int q = 0; q < NCP; q++) dLdp[q * nt + i] = static_cast<double>(mu[q]);
    if (a.status) a.status[i] = status;
}

}  // namespace pt
}  // namespace mpgos

namespace mpgos {
namespace pt {

// Launch side of the adjoint (mpgos_pt_kernels::launch_record / launch_adjoint).
template <class S, int ALG>
struct AdjointTable {
    static Tape tape_of(const mpgos_pt_tape& t)
    {
        return Tape{t.segment, t.max_steps, t.dt, t.ckpt_x, t.ckpt_t, t.n_steps};
    }

    static int launch_record(const mpgos_pt_launch* L, const mpgos_pt_tape* tape, int grid, int block, size_t smem,
                             void* stream)
    {
        if (tape == nullptr || tape->segment < 1 || tape->segment > MAX_SEG) return static_cast<int>(cudaErrorInvalidValue);
        void* fn = nullptr;
        const int arith = L->mode & (MPGOS_MODE_DF_STAGE | MPGOS_MODE_SPLIT);
        if (arith == MPGOS_MODE_DF_STAGE || arith == MPGOS_MODE_SPLIT) {
            fn = double_float_kernel<S, ALG>(arith, MODE_RECORD | (L->mode & MPGOS_MODE_PERSISTENT));
        } else {
            switch (L->mode & (MPGOS_MODE_FAST_CONTROL | MPGOS_MODE_PERSISTENT)) {
                case 0: fn = reinterpret_cast<void*>(&perthread_kernel<S, ALG, double, MODE_RECORD>); break;
                case 1: fn = reinterpret_cast<void*>(&perthread_kernel<S, ALG, double, MODE_RECORD | 1>); break;
                case 2: fn = reinterpret_cast<void*>(&perthread_kernel<S, ALG, double, MODE_RECORD | 2>); break;
                default: fn = reinterpret_cast<void*>(&perthread_kernel<S, ALG, double, MODE_RECORD | 3>); break;
            }
        }
        Args<double> a = make_args<double>(*L);
        a.tape = tape_of(*tape);
        void* params[] = {&a};
        return static_cast<int>(cudaLaunchKernel(fn, dim3(grid), dim3(block), params, smem,
                                                 static_cast<cudaStream_t>(stream)));
    }

    static int launch_adjoint(const mpgos_pt_launch* L, const mpgos_pt_tape* tape, const double* dLdxT,
                              double* dLdx0, double* dLdp, int grid, int block, size_t smem, void* stream)
    {
        if (tape == nullptr || tape->segment < 1 || tape->segment > MAX_SEG) return static_cast<int>(cudaErrorInvalidValue);
        Args<double> a = make_args<double>(*L);
        Tape t = tape_of(*tape);
        void* params[] = {&a, &t, &dLdxT, &dLdx0, &dLdp};
        // DF_STAGE and SPLIT solvers (double-float stages) differentiate in
        // double-float as well
        void* fn = (L->mode & (MPGOS_MODE_DF_STAGE | MPGOS_MODE_SPLIT))
                       ? reinterpret_cast<void*>(&adjoint_kernel<S, ALG, dfloat>)
                       : reinterpret_cast<void*>(&adjoint_kernel<S, ALG, double>);
        return static_cast<int>(cudaLaunchKernel(fn, dim3(grid), dim3(block), params, smem,
                                                 static_cast<cudaStream_t>(stream)));
    }
};

}  // namespace pt
}  // namespace mpgos

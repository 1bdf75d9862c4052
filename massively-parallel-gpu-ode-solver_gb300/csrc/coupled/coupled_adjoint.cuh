// Discrete adjoint of the coupled per-block integration (extension: the
// reference has no differentiation). One warp per system, in FP64 or, for
// DF_STAGE solvers, in double-float (T = dfloat; the tape stays FP64).
//
// Forward (recording) pass: the coupled kernel compiled with MODE_RECORD
// (coupled_kernel.cuh) stores, per system, every accepted step size and a
// checkpoint of the time and of every unit's state every SEG accepted steps.
//
// Reverse pass (this file): for each segment, last first, the states of every
// step of the segment are recomputed from the checkpoint with the recorded
// step sizes by the forward stepper itself (bit-identical to the forward
// pass). Each step is then differentiated through its Runge-Kutta stages:
// the stage points are re-evaluated with the user's
// CoupledSystems_PerBlock_OdeFunction instantiated with dual numbers, seeded
// along the unit's own state components and the system parameters, which
// gives per unit and stage the local Jacobian of the uncoupled right-hand
// side, the derivatives of the coupling term CPT and of the coupling factor
// CPF, and their values. With K_i = f(X_i) the stage derivatives and
//   f_u = F_u(X_u) + e_{CouplingIndex_c} cstr_c CPF_{u,c}(X_u) sum_j C_c[u][j] CPT_{j,c}(X_j),
// the stage Jacobian-transpose product J_i^T kappa is, for unit j,
//   dF_j^T kappa_j                                           (local part)
// + sum_c w_{j,c} dCPT_{j,c}    with w_c = C_c^T z_c,  z_{u,c} = cstr_c CPF_{u,c} kappa_u[CouplingIndex_c]
// + sum_c cstr_c V_{j,c} kappa_j[CouplingIndex_c] dCPF_{j,c},   V_c = C_c CPT_c,
// one transposed coupling matrix-vector product per stage and coupling (the
// transposed matrix is staged in shared memory for the full storage). The
// Runge-Kutta recursion is the per-thread one (csrc/perthread/adjoint.cuh):
//   kappa_i = dt b_i lambda + sum_{l>i} dt a_li xi_l,  xi_i = J_i^T kappa_i,
//   lambda <- lambda + sum_i xi_i,  mu += sum_i (df/dp)_i^T kappa_i,
// the gradient of the discrete map with the step sequence frozen: d L / d x(t0)
// for every unit and d L / d sPAR for every system, given d L / d x(T).
//
// Scope: the system parameters are the differentiated parameters; hooks that
// change the state outside the right-hand side are not differentiated.
#pragma once

#include "../perthread/adjoint.cuh"
#include "coupled_kernel.cuh"

namespace mpgos {
namespace cb {

// Per-warp shared slot of the reverse pass: the forward slot (system scope,
// coupling terms) plus the transposed-product inputs z.
template <class S, class T>
struct AdjSlot {
    WarpSlot<S, T> w;
    T z[S::UPS][AtLeastOne<S::NC>::value];
};

// Dynamic shared memory of the reverse kernel: [global parameters NGP]
// [coupling matrices NC*MAT][transposed full matrices NC*UPS*UPS if full
// storage][integer global parameters NIGP], padded to 16 bytes, then one
// AdjSlot per warp.
template <class S, class T>
__host__ __device__ constexpr size_t adjoint_block_part_bytes()
{
    constexpr bool FULL = (S::CCI == 0 && S::CBW == 0);
    const size_t b = sizeof(T) * (S::NGP + S::NC * S::MAT + (FULL ? S::NC * S::UPS * S::UPS : 0)) +
                     sizeof(int) * S::NIGP;
    return (b + 15) / 16 * 16;
}

template <class S, class T>
__host__ __device__ constexpr size_t adjoint_smem_bytes(int warps)
{
    return adjoint_block_part_bytes<S, T>() + static_cast<size_t>(warps) * sizeof(AdjSlot<S, T>);
}

// w_{j,c} = sum_u C_c[u][j] z_{u,c} for unit j, in each of the four storages
// of the coupling matrix (the transposes of coupling_value).
template <class S, class T>
__device__ __forceinline__ T transposed_coupling_value(const T* M, const T* MT, const AdjSlot<S, T>& sl, int j, int c)
{
    constexpr int UPS = S::UPS, CBW = S::CBW, CCI = S::CCI;
    if constexpr (IS_DF<T> && CCI == 0 && CBW == 0) {
        // compensated double-float dot product, as in the forward product
        const int shift = c * UPS * UPS;
        float sh = 0.0f, sl_ = 0.0f;
        for (int u = 0; u < UPS; u++) df_dot_acc(sh, sl_, MT[j + u * UPS + shift], sl.z[u][c]);
        return df::two_sum(sh, sl_);
    }
    T v(0.0);
    if (CCI == 0 && CBW == 0) {
        const int shift = c * UPS * UPS;
        for (int u = 0; u < UPS; u++) v += MT[j + u * UPS + shift] * sl.z[u][c];
    } else {
        const int width = (CBW > 0) ? 2 * CBW + 1 : UPS;
        for (int dg = 0; dg < width; dg++) {
            int u = j - dg + CBW;  // the row whose shifted diagonal dg holds column j
            if (u >= UPS) u -= UPS;
            if (u < 0) u += UPS;
            const int idx = (CCI == 0) ? u + dg * UPS + c * UPS * width : dg + c * width;
            v += M[idx] * sl.z[u][c];
        }
    }
    return v;
}

template <class S, int ALG, class T>
struct CoupledAdjoint {
    static constexpr int UPS = S::UPS, UD = S::UD, NC = S::NC, NUP = S::NUP, NSP = S::NSP, NUA = S::NUA;
    static constexpr int NIUA = S::NIUA, NSA = S::NSA, NISA = S::NISA, UPL = S::UPL;
    static constexpr int N = UD + NSP;  // dual directions: the unit's state, then the system parameters
    using D = ad::Dual<N, T>;
    using TB = pt::Tableau<ALG>;
    static constexpr int ST = TB::S;
    using Tab = pt::TableauT<T, ST>;
    using Fwd = Solver<S, ALG, T, 0>;
    using Units = typename Fwd::Units;
    static constexpr int NCP1 = AtLeastOne<NC>::value;

    // Stage data of one step, per unit of the lane.
    struct StepData {
        T K[ST][UPL][UD];         // stage derivatives (with coupling)
        T L[ST][UPL][UD][N];      // d(uncoupled F)/d(X_u, sPAR)
        T G[ST][UPL][NCP1][N];    // d(CPT)/d(X_u, sPAR)
        T CF[ST][UPL][NCP1];      // CPF value
        T CFD[ST][UPL][NCP1][N];  // d(CPF)/d(X_u, sPAR)
        T V[ST][UPL][NCP1];       // coupling value sum_j C[u][j] CPT_j
    };

    __device__ static bool has(int lane, int j) { return lane + 32 * j < UPS; }
    __device__ static int unit_of(int lane, int j) { return lane + 32 * j; }

    // Stages of one step from (x, t) with step dt, dual-evaluated.
    __device__ static void stages(const Tab& tb, long long s, int lane, AdjSlot<S, T>& sl, const Units& u,
                                  const T* gp, const int* igp, const T* M, const int* cidx, const T (&x)[UPL][UD],
                                  T t, T dt, StepData& sd)
    {
        WarpSlot<S, T>& w = sl.w;
        const int sid = static_cast<int>(s);
        D spd[AtLeastOne<NSP>::value];
#pragma unroll
        for (int k = 0; k < NSP; k++) {
            spd[k] = D(w.sp[k]);
            spd[k].d[UD + k] = T(1.0);
        }
        D gpd[AtLeastOne<S::NGP>::value];
#pragma unroll
        for (int k = 0; k < S::NGP; k++) gpd[k] = D(gp[k]);
        D saccd[AtLeastOne<NSA>::value];
#pragma unroll
        for (int k = 0; k < NSA; k++) saccd[k] = D(w.sacc[k]);
        int isacc[AtLeastOne<NISA>::value];
#pragma unroll
        for (int k = 0; k < NISA; k++) isacc[k] = w.isacc[k];

        for (int st = 0; st < ST; st++) {
            const D Td(t + pt::tab_c<TB>(tb, st) * dt);
#pragma unroll
            for (int j = 0; j < UPL; j++) {
                if (!has(lane, j)) continue;
                const int uid = unit_of(lane, j);
                D Xd[UD], Fd[UD], cptd[NCP1], cpfd[NCP1];
#pragma unroll
                for (int d = 0; d < UD; d++) {
                    T sum(0.0);
                    for (int q = 0; q < st; q++) sum = ad::mad(pt::tab_a<TB>(tb, st, q), sd.K[q][j][d], sum);
                    Xd[d] = D(ad::mad(dt, sum, x[j][d]));
                    Xd[d].d[d] = T(1.0);
                }
                D upd[AtLeastOne<NUP>::value], uaccd[AtLeastOne<NUA>::value];
#pragma unroll
                for (int k = 0; k < NUP; k++) upd[k] = D(u.up[j][k]);
#pragma unroll
                for (int k = 0; k < NUA; k++) uaccd[k] = D(u.uacc[j][k]);
                int iuacc[AtLeastOne<NIUA>::value];
#pragma unroll
                for (int k = 0; k < NIUA; k++) iuacc[k] = u.iuacc[j][k];
                CoupledSystems_PerBlock_OdeFunction<D>(sid, uid, Fd, Xd, Td, upd, spd, gpd, const_cast<int*>(igp),
                                                       uaccd, iuacc, saccd, isacc, cptd, cpfd);
#pragma unroll
                for (int d = 0; d < UD; d++) {
                    sd.K[st][j][d] = Fd[d].v;
#pragma unroll
                    for (int q = 0; q < N; q++) sd.L[st][j][d][q] = Fd[d].d[q];
                }
                for (int c = 0; c < NC; c++) {
                    w.cpt[uid][c] = cptd[c].v;
                    sd.CF[st][j][c] = cpfd[c].v;
#pragma unroll
                    for (int q = 0; q < N; q++) {
                        sd.G[st][j][c][q] = cptd[c].d[q];
                        sd.CFD[st][j][c][q] = cpfd[c].d[q];
                    }
                }
            }
            __syncwarp();
#pragma unroll
            for (int j = 0; j < UPL; j++) {
                if (!has(lane, j)) continue;
                const int uid = unit_of(lane, j);
                for (int c = 0; c < NC; c++) {
                    const T v = coupling_value<S, T>(M, w, uid, c);
                    sd.V[st][j][c] = v;
                    const int ci = cidx[c];
                    if (ci >= 0 && ci < UD) sd.K[st][j][ci] += w.cstr[c] * sd.CF[st][j][c] * v;
                }
            }
            __syncwarp();
        }
    }

    // Adjoint of one step (see the file comment).
    __device__ static void reverse_step(const Tab& tb, int lane, AdjSlot<S, T>& sl, const T* M, const T* MT,
                                        const int* cidx, const StepData& sd, T dt, T (&lam)[UPL][UD],
                                        T (&mu)[AtLeastOne<NSP>::value])
    {
        WarpSlot<S, T>& w = sl.w;
        T kap[ST][UPL][UD];
        T dlam[UPL][UD];
        for (int st = 0; st < ST; st++) {
            const T hb = dt * pt::tab_b<TB>(tb, st);
#pragma unroll
            for (int j = 0; j < UPL; j++)
#pragma unroll
                for (int d = 0; d < UD; d++) kap[st][j][d] = hb * lam[j][d];
        }
#pragma unroll
        for (int j = 0; j < UPL; j++)
#pragma unroll
            for (int d = 0; d < UD; d++) dlam[j][d] = T(0.0);

        for (int st = ST - 1; st >= 0; st--) {
            T xi[UPL][UD];
#pragma unroll
            for (int j = 0; j < UPL; j++) {
#pragma unroll
                for (int r = 0; r < UD; r++) {
                    T v(0.0);
#pragma unroll
                    for (int d = 0; d < UD; d++) v = ad::mad(sd.L[st][j][d][r], kap[st][j][d], v);
                    xi[j][r] = v;
                }
                if (!has(lane, j)) continue;
#pragma unroll
                for (int q = 0; q < NSP; q++) {
                    T v(0.0);
#pragma unroll
                    for (int d = 0; d < UD; d++) v = ad::mad(sd.L[st][j][d][UD + q], kap[st][j][d], v);
                    mu[q] += v;
                }
            }
            for (int c = 0; c < NC; c++) {
                const int ci = cidx[c];
                const bool ok = ci >= 0 && ci < UD;
#pragma unroll
                for (int j = 0; j < UPL; j++)
                    if (has(lane, j)) sl.z[unit_of(lane, j)][c] = ok ? w.cstr[c] * sd.CF[st][j][c] * kap[st][j][ci] : T(0.0);
                __syncwarp();
#pragma unroll
                for (int j = 0; j < UPL; j++) {
                    if (!has(lane, j)) continue;
                    const T wv = transposed_coupling_value<S, T>(M, MT, sl, unit_of(lane, j), c);
                    const T coef = ok ? w.cstr[c] * sd.V[st][j][c] * kap[st][j][ci] : T(0.0);
#pragma unroll
                    for (int r = 0; r < UD; r++) xi[j][r] += ad::mad2(wv, sd.G[st][j][c][r], coef, sd.CFD[st][j][c][r]);
#pragma unroll
                    for (int q = 0; q < NSP; q++)
                        mu[q] += ad::mad2(wv, sd.G[st][j][c][UD + q], coef, sd.CFD[st][j][c][UD + q]);
                }
                __syncwarp();
            }
            for (int q = 0; q < st; q++) {
                if (TB::a(st, q) != 0.0) {
                    const T a = dt * pt::tab_a<TB>(tb, st, q);
#pragma unroll
                    for (int j = 0; j < UPL; j++)
#pragma unroll
                        for (int d = 0; d < UD; d++) kap[q][j][d] = ad::mad(a, xi[j][d], kap[q][j][d]);
                }
            }
#pragma unroll
            for (int j = 0; j < UPL; j++)
#pragma unroll
                for (int d = 0; d < UD; d++) dlam[j][d] += xi[j][d];
        }
#pragma unroll
        for (int j = 0; j < UPL; j++)
#pragma unroll
            for (int d = 0; d < UD; d++) lam[j][d] += dlam[j][d];
    }
};

// Sum over the warp's lanes (all lanes hold a value).
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}
__device__ __forceinline__ dfloat warp_sum(dfloat v)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
        v = v + dfloat(__shfl_xor_sync(0xffffffffu, v.hi, off), __shfl_xor_sync(0xffffffffu, v.lo, off));
    return v;
}

// Launch shape of the reverse pass: up to CB_ADJOINT_BLOCK threads (one warp
// per system; the runtime picks the warps per block that keep the most warps
// resident, shared memory and registers both counted).
#ifndef MPGOS_CB_ADJOINT_MIN_BLOCKS
#define MPGOS_CB_ADJOINT_MIN_BLOCKS 1
#endif
constexpr int CB_ADJOINT_BLOCK = 256;

template <class S, int ALG, class T>
__global__ void __launch_bounds__(CB_ADJOINT_BLOCK, MPGOS_CB_ADJOINT_MIN_BLOCKS) coupled_adjoint_kernel(Args<double> a, pt::Tape tp,
                                                                            const double* dLdxT, double* dLdx0,
                                                                            double* dLdsp)
{
    using Adj = CoupledAdjoint<S, ALG, T>;
    using Fwd = typename Adj::Fwd;
    using Units = typename Adj::Units;
    using TB = typename Adj::TB;
    constexpr int UPS = S::UPS, UD = S::UD, NC = S::NC, NSP = S::NSP, NSA = S::NSA, NISA = S::NISA, UPL = S::UPL;
    constexpr int NGP = S::NGP, NIGP = S::NIGP, NUP = S::NUP, NUA = S::NUA, NIUA = S::NIUA;
    constexpr bool FULL = (S::CCI == 0 && S::CBW == 0);
    constexpr int MAXSEG = pt::MAX_SEG;
    extern __shared__ __align__(16) unsigned char mpgos_cb_adj_smem[];
    __shared__ int s_cidx[AtLeastOne<NC>::value];
    __shared__ typename Adj::Tab tb;

    T* gp = reinterpret_cast<T*>(mpgos_cb_adj_smem);
    T* M = gp + NGP;
    T* MT = M + NC * S::MAT;
    int* igp = reinterpret_cast<int*>(MT + (FULL ? NC * UPS * UPS : 0));
    AdjSlot<S, T>* slots = reinterpret_cast<AdjSlot<S, T>*>(mpgos_cb_adj_smem + adjoint_block_part_bytes<S, T>());

    for (int k = threadIdx.x; k < NGP; k += blockDim.x) gp[k] = T(a.gp[k]);
    for (int k = threadIdx.x; k < NIGP; k += blockDim.x) igp[k] = a.igp[k];
    for (int k = threadIdx.x; k < NC * S::MAT; k += blockDim.x) M[k] = T(a.cmat[k]);
    if (FULL) {
        for (int k = threadIdx.x; k < NC * UPS * UPS; k += blockDim.x) {
            const int c = k / (UPS * UPS), r = k % (UPS * UPS);
            const int jj = r % UPS, u = r / UPS;  // MT[j + u*UPS] = M[u + j*UPS]
            MT[k] = T(a.cmat[c * UPS * UPS + u + jj * UPS]);
        }
    }
    for (int k = threadIdx.x; k < NC; k += blockDim.x) s_cidx[k] = a.cidx[k];
    pt::stage_tableau<TB>(tb);
    __syncthreads();

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
    const long long s = static_cast<long long>(blockIdx.x) * warps + warp;
    if (s >= a.n_active) return;
    AdjSlot<S, T>& sl = slots[warp];
    WarpSlot<S, T>& w = sl.w;
    const long long ns = a.ns, nu = a.ns * UPS;

    // system and unit scope inputs the hooks read
    for (int k = lane; k < NSP; k += 32) w.sp[k] = T(a.sp[s + k * ns]);
    for (int k = lane; k < NSA; k += 32) w.sacc[k] = T(a.sacc[s + k * ns]);
    for (int k = lane; k < NISA; k += 32) w.isacc[k] = a.isacc[s + k * ns];
    for (int k = lane; k < NC; k += 32) w.cstr[k] = T(a.cstr[s + k * ns]);
    if (lane == 0) {
        w.td[0] = T(a.td[s]);
        w.td[1] = T(a.td[s + ns]);
    }
    Units u;
    T lam[UPL][UD];
#pragma unroll
    for (int j = 0; j < UPL; j++) {
        const bool h = Adj::has(lane, j);
        const long long g = s * UPS + Adj::unit_of(lane, j);
#pragma unroll
        for (int k = 0; k < NUP; k++) u.up[j][k] = h ? T(a.up[g + k * nu]) : T(0.0);
#pragma unroll
        for (int k = 0; k < NUA; k++) u.uacc[j][k] = h ? T(a.uacc[g + k * nu]) : T(0.0);
#pragma unroll
        for (int k = 0; k < NIUA; k++) u.iuacc[j][k] = h ? a.iuacc[g + k * nu] : 0;
#pragma unroll
        for (int d = 0; d < UD; d++) lam[j][d] = h ? T(dLdxT[g + d * nu]) : T(0.0);
    }
    T mu[AtLeastOne<NSP>::value];
#pragma unroll
    for (int q = 0; q < NSP; q++) mu[q] = T(0.0);
    __syncwarp();

    const int n = tp.n_steps[s];
    int status = a.status ? a.status[s] : 0;
    if (n > tp.max_steps) status |= MPGOS_INSTANCE_TAPE_OVERFLOW;
    const int seg = tp.seg;

    if (!(status & MPGOS_INSTANCE_TAPE_OVERFLOW) && n > 0) {
        T xs[MAXSEG][UPL][UD];
        T ts[MAXSEG];
        typename Adj::StepData sd;
        for (int sgm = (n - 1) / seg; sgm >= 0; sgm--) {
            const int k0 = sgm * seg;
            const int k1 = min(n, k0 + seg);
            T t(tp.ckpt_t[static_cast<long long>(sgm) * ns + s]);
#pragma unroll
            for (int j = 0; j < UPL; j++) {
                const long long g = s * UPS + Adj::unit_of(lane, j);
#pragma unroll
                for (int d = 0; d < UD; d++)
                    u.x[j][d] = Adj::has(lane, j) ? T(tp.ckpt_x[(static_cast<long long>(sgm) * UD + d) * nu + g])
                                                  : T(0.0);
            }
            // replay the segment with the recorded steps (the forward stepper)
            for (int k = k0; k < k1; k++) {
                const T dt(tp.dt[static_cast<long long>(k) * ns + s]);
#pragma unroll
                for (int j = 0; j < UPL; j++)
#pragma unroll
                    for (int d = 0; d < UD; d++) xs[k - k0][j][d] = u.x[j][d];
                ts[k - k0] = t;
                if (k + 1 < k1) {
                    T xn[UPL][UD], err[UPL][UD];
                    int finite = 1;
                    if (ALG == MPGOS_RK4)
                        Fwd::step_rk4(s, lane, w, u, gp, igp, M, s_cidx, t, dt, xn, finite);
                    else
                        Fwd::step_rkck45(s, lane, w, u, gp, igp, M, s_cidx, t, dt, xn, err, finite);
#pragma unroll
                    for (int j = 0; j < UPL; j++)
#pragma unroll
                        for (int d = 0; d < UD; d++) u.x[j][d] = xn[j][d];
                    t += dt;
                }
            }
            // reverse through the segment
            for (int k = k1 - 1; k >= k0; k--) {
                const T dt(tp.dt[static_cast<long long>(k) * ns + s]);
                Adj::stages(tb, s, lane, sl, u, gp, igp, M, s_cidx, xs[k - k0], ts[k - k0], dt, sd);
                Adj::reverse_step(tb, lane, sl, M, MT, s_cidx, sd, dt, lam, mu);
            }
        }
    }
#pragma unroll
    for (int j = 0; j < UPL; j++) {
        if (!Adj::has(lane, j)) continue;
        const long long g = s * UPS + Adj::unit_of(lane, j);
#pragma unroll
        for (int d = 0; d < UD; d++) dLdx0[g + d * nu] = static_cast<double>(lam[j][d]);
    }
#pragma unroll
    for (int q = 0; q < NSP; q++) {
        const T v = warp_sum(mu[q]);
        if (lane == 0) dLdsp[s + q * ns] = static_cast<double>(v);
    }
    if (lane == 0 && a.status) a.status[s] = status;
}

// Launch side of the coupled adjoint (mpgos_cb_kernels::launch_record / launch_adjoint).
template <class S, int ALG>
struct CoupledAdjointTable {
    static pt::Tape tape_of(const mpgos_pt_tape& t)
    {
        return pt::Tape{t.segment, t.max_steps, t.dt, t.ckpt_x, t.ckpt_t, t.n_steps};
    }

    static int launch_record(const mpgos_cb_launch* L, const mpgos_pt_tape* tape, int grid, int block, size_t smem,
                             void* stream)
    {
        if (tape == nullptr || tape->segment < 1 || tape->segment > pt::MAX_SEG)
            return static_cast<int>(cudaErrorInvalidValue);
        const bool pers = (L->mode & MPGOS_MODE_PERSISTENT) != 0;
        void* fn = nullptr;
        if (L->mode & MPGOS_MODE_DF_STAGE)
            fn = pers ? reinterpret_cast<void*>(&coupled_kernel<S, ALG, dfloat, MODE_RECORD | MPGOS_MODE_PERSISTENT>)
                      : reinterpret_cast<void*>(&coupled_kernel<S, ALG, dfloat, MODE_RECORD>);
        else if (L->mode & MPGOS_MODE_SPLIT)
            fn = pers ? reinterpret_cast<void*>(
                            &coupled_kernel<S, ALG, double, MODE_RECORD | MPGOS_MODE_SPLIT | MPGOS_MODE_PERSISTENT>)
                      : reinterpret_cast<void*>(&coupled_kernel<S, ALG, double, MODE_RECORD | MPGOS_MODE_SPLIT>);
        else
            fn = pers ? reinterpret_cast<void*>(&coupled_kernel<S, ALG, double, MODE_RECORD | MPGOS_MODE_PERSISTENT>)
                      : reinterpret_cast<void*>(&coupled_kernel<S, ALG, double, MODE_RECORD>);
        Args<double> a = make_args<double>(*L);
        a.tape = tape_of(*tape);
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
            if (e != cudaSuccess) return static_cast<int>(e);
        }
        void* params[] = {&a};
        return static_cast<int>(cudaLaunchKernel(fn, dim3(grid), dim3(block), params, smem,
                                                 static_cast<cudaStream_t>(stream)));
    }

    static int launch_adjoint(const mpgos_cb_launch* L, const mpgos_pt_tape* tape, const double* dLdxT,
                              double* dLdx0, double* dLdsp, int grid, int block, size_t smem, void* stream)
    {
        if (tape == nullptr || tape->segment < 1 || tape->segment > pt::MAX_SEG)
            return static_cast<int>(cudaErrorInvalidValue);
        // a DF_STAGE or SPLIT solver differentiates in double-float
        void* fn = adjoint_fn(L->mode);
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
            if (e != cudaSuccess) return static_cast<int>(e);
        }
        Args<double> a = make_args<double>(*L);
        pt::Tape t = tape_of(*tape);
        void* params[] = {&a, &t, &dLdxT, &dLdx0, &dLdsp};
        return static_cast<int>(cudaLaunchKernel(fn, dim3(grid), dim3(block), params, smem,
                                                 static_cast<cudaStream_t>(stream)));
    }

    static void* adjoint_fn(int32_t mode)
    {
        return (mode & (MPGOS_MODE_DF_STAGE | MPGOS_MODE_SPLIT))
                   ? reinterpret_cast<void*>(&coupled_adjoint_kernel<S, ALG, dfloat>)
                   : reinterpret_cast<void*>(&coupled_adjoint_kernel<S, ALG, double>);
    }

    static int occupancy(int32_t mode, int block, size_t smem, int* blocks)
    {
        void* fn = adjoint_fn(mode);
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
            if (e != cudaSuccess) return static_cast<int>(e);
        }
        return static_cast<int>(cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, fn, block, smem));
    }

    static size_t smem(int warps, int32_t mode)
    {
        return (mode & (MPGOS_MODE_DF_STAGE | MPGOS_MODE_SPLIT)) ? adjoint_smem_bytes<S, dfloat>(warps)
                                                                 : adjoint_smem_bytes<S, double>(warps);
    }
};

}  // namespace cb
}  // namespace mpgos

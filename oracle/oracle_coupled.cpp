// CPU oracle of the coupled per-block ensemble solver.
//
// TEST INFRASTRUCTURE ONLY. This is the oracle the GPU coupled kernels are
// compared against (tests, smoke test, the bench's CPU baseline); the product
// never links or calls it.
//
// A plain restatement of the reference algorithm, one system at a time, the
// units of a system in a loop (the reference runs one thread per unit and
// reduces over units through shared memory):
//   loop order        SourceCodes/CoupledSystmes_PerBlock_Solver.cuh:1575-2211
//                     (MultipleSystems_SingleBlockLaunch)
//   RK4 stepper       SourceCodes/CoupledSystems_PerBlock_ExplicitRungeKutta_Steppers.cuh:1483-1692
//   RKCK45 stepper    SourceCodes/CoupledSystems_PerBlock_ExplicitRungeKutta_Steppers.cuh:1695-2014
//   coupling value    SourceCodes/CoupledSystems_PerBlock_ExplicitRungeKutta_Steppers.cuh:2552-2633
//   controllers       SourceCodes/CoupledSystems_PerBlock_ExplicitRungeKutta_ErrorControllers.cuh:286-423
//                     (safety factor 0.8, minimum over units of tol/err)
//   event control     SourceCodes/CoupledSystems_PerBlock_EventHandling.cuh:149-214
//   dense output      SourceCodes/CoupledSystems_PerBlock_DenseOutput.cuh:213-312
// with the same grouping of every floating-point expression; built with
// -ffp-contract=off it differs from a GPU build only where the GPU fuses
// multiply-adds or its math library rounds differently.
//
// Two deliberate differences, both only for inputs where the reference
// writes out of bounds: a dense-output store with a full buffer is skipped,
// and every system stops after max_attempts step attempts (status flag 8).
//
// Compiled once per coupled system: -DMPGOS_SYSTEM_HEADER="<hooks>.cuh"
// (with MPGOS_SYS_UPS / _CBW / _CCI defined on the command line).
#include "host_shim.hpp"

#include MPGOS_SYSTEM_HEADER

#include <cstdint>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int UPS = MPGOS_SYS_UPS, UD = MPGOS_SYS_UD, NC = MPGOS_SYS_NC, CBW = MPGOS_SYS_CBW, CCI = MPGOS_SYS_CCI;
constexpr int NUP = MPGOS_SYS_NUP, NSP = MPGOS_SYS_NSP, NGP = MPGOS_SYS_NGP, NIGP = MPGOS_SYS_NIGP;
constexpr int NUA = MPGOS_SYS_NUA, NIUA = MPGOS_SYS_NIUA, NSA = MPGOS_SYS_NSA, NISA = MPGOS_SYS_NISA;
constexpr int NE = MPGOS_SYS_NE;
template <int N> constexpr int one_at_least() { return N > 0 ? N : 1; }
constexpr int MAT = (CCI == 0 && CBW == 0)  ? UPS * UPS
                    : (CCI == 0 && CBW > 0) ? UPS * (2 * CBW + 1)
                    : (CCI == 1 && CBW > 0) ? (2 * CBW + 1)
                                            : UPS;

struct Opts {
    double initial_dt, max_dt, min_dt, grow, shrink, dense_min_dt;
    int dense_freq, ndo;
    long long max_attempts;
};

struct Arrays {
    long long ns;
    double *td, *t, *sp, *sacc, *cstr, *dtime, *x, *up, *uacc, *dstate;
    int *isacc, *didx, *iuacc;
    const double *gp, *cmat, *rtol, *atol, *etol;
    const int *igp, *cidx, *edir;
    int *status, *nacc, *nrej;
};

// One system: system scope by value, unit scope as [unit][field].
struct System {
    double td[2], t, dt, newdt, dense_next;
    double sp[one_at_least<NSP>()], sacc[one_at_least<NSA>()], cstr[one_at_least<NC>()];
    int isacc[one_at_least<NISA>()], didx, udt, skipped;
    double x[UPS][UD], up[UPS][one_at_least<NUP>()], uacc[UPS][one_at_least<NUA>()];
    int iuacc[UPS][one_at_least<NIUA>()];
    double cpt[UPS][one_at_least<NC>()], cpf[UPS][one_at_least<NC>()];
    double ga[UPS][one_at_least<NE>()], gn[UPS][one_at_least<NE>()];
};

double coupling_value(const double* M, const System& s, int unit, int i)
{
    double v = 0;
    if (CCI == 0 && CBW == 0) {
        for (int col = 0; col < UPS; col++) v += M[unit + col * UPS + i * UPS * UPS] * s.cpt[col][i];
    } else {
        const int width = (CBW > 0) ? 2 * CBW + 1 : UPS;
        for (int dg = 0; dg < width; dg++) {
            int su = unit + dg - CBW;
            if (su >= UPS) su -= UPS;
            if (su < 0) su += UPS;
            const int idx = (CCI == 0) ? unit + dg * UPS + i * UPS * width : dg + i * width;
            v += M[idx] * s.cpt[su][i];
        }
    }
    return v;
}

// Right-hand side of every unit at stage point X (time T), then the coupling.
void stage(int sid, System& s, double* gp, int* igp, const double* M, const int* cidx, double T,
           const double (&X)[UPS][UD], double (&F)[UPS][UD])
{
    for (int u = 0; u < UPS; u++) {
        double xu[UD];
        for (int d = 0; d < UD; d++) xu[d] = X[u][d];
        CoupledSystems_PerBlock_OdeFunction<double>(sid, u, F[u], xu, T, s.up[u], s.sp, gp, igp, s.uacc[u], s.iuacc[u],
                                                    s.sacc, s.isacc, s.cpt[u], s.cpf[u]);
    }
    for (int u = 0; u < UPS; u++)
        for (int i = 0; i < NC; i++) {
            const double value = coupling_value(M, s, u, i);
            F[u][cidx[i]] += s.cstr[i] * s.cpf[u][i] * value;
        }
}

void rk4(int sid, System& s, double* gp, int* igp, const double* M, const int* cidx, double t, double dt,
         double (&xn)[UPS][UD], int& finite)
{
    double X[UPS][UD], k[UPS][UD];
    stage(sid, s, gp, igp, M, cidx, t, s.x, xn);
    double T = t + 0.5 * dt;
    for (int u = 0; u < UPS; u++)
        for (int d = 0; d < UD; d++) X[u][d] = s.x[u][d] + xn[u][d] * 0.5 * dt;
    stage(sid, s, gp, igp, M, cidx, T, X, k);
    for (int u = 0; u < UPS; u++)
        for (int d = 0; d < UD; d++) {
            xn[u][d] += 2 * k[u][d];
            X[u][d] = s.x[u][d] + k[u][d] * 0.5 * dt;
        }
    stage(sid, s, gp, igp, M, cidx, T, X, k);
    T = t + dt;
    for (int u = 0; u < UPS; u++)
        for (int d = 0; d < UD; d++) {
            xn[u][d] += 2.0 * k[u][d];
            X[u][d] = s.x[u][d] + k[u][d] * dt;
        }
    stage(sid, s, gp, igp, M, cidx, T, X, k);
    for (int u = 0; u < UPS; u++)
        for (int d = 0; d < UD; d++) {
            xn[u][d] = s.x[u][d] + dt * (xn[u][d] + k[u][d]) * (1.0 / 6.0);
            if (!std::isfinite(xn[u][d])) finite = 0;
        }
}

void rkck45(int sid, System& s, double* gp, int* igp, const double* M, const int* cidx, double t, double dt,
            double (&xn)[UPS][UD], double (&err)[UPS][UD], int& finite)
{
    static thread_local double X[UPS][UD], k1[UPS][UD], k2[UPS][UD], k3[UPS][UD], k4[UPS][UD], k5[UPS][UD],
        k6[UPS][UD];
    stage(sid, s, gp, igp, M, cidx, t, s.x, k1);
    for (int u = 0; u < UPS; u++)
        for (int d = 0; d < UD; d++) X[u][d] = s.x[u][d] + (k1[u][d] * (1.0 / 5.0)) * dt;
    stage(sid, s, gp, igp, M, cidx, t + (1.0 / 5.0) * dt, X, k2);
    for (int u = 0; u < UPS; u++)
        for (int d = 0; d < UD; d++)
            X[u][d] = s.x[u][d] + (k1[u][d] * (3.0 / 40.0) + k2[u][d] * (9.0 / 40.0)) * dt;
    stage(sid, s, gp, igp, M, cidx, t + (3.0 / 10.0) * dt, X, k3);
    for (int u = 0; u < UPS; u++)
        for (int d = 0; d < UD; d++)
            X[u][d] = s.x[u][d] + (k1[u][d] * (3.0 / 10.0) + k2[u][d] * (-9.0 / 10.0) + k3[u][d] * (6.0 / 5.0)) * dt;
    stage(sid, s, gp, igp, M, cidx, t + (3.0 / 5.0) * dt, X, k4);
    for (int u = 0; u < UPS; u++)
        for (int d = 0; d < UD; d++)
            X[u][d] = s.x[u][d] + (k1[u][d] * (-11.0 / 54.0) + k2[u][d] * (5.0 / 2.0) + k3[u][d] * (-70.0 / 27.0) +
                                   k4[u][d] * (35.0 / 27.0)) * dt;
    stage(sid, s, gp, igp, M, cidx, t + dt, X, k5);
    for (int u = 0; u < UPS; u++)
        for (int d = 0; d < UD; d++)
            X[u][d] = s.x[u][d] + (k1[u][d] * (1631.0 / 55296.0) + k2[u][d] * (175.0 / 512.0) +
                                   k3[u][d] * (575.0 / 13824.0) + k4[u][d] * (44275.0 / 110592.0) +
                                   k5[u][d] * (253.0 / 4096.0)) * dt;
    stage(sid, s, gp, igp, M, cidx, t + (7.0 / 8.0) * dt, X, k6);
    for (int u = 0; u < UPS; u++)
        for (int d = 0; d < UD; d++) {
            xn[u][d] = s.x[u][d] + (k1[u][d] * (37.0 / 378.0) + k3[u][d] * (250.0 / 621.0) +
                                    k4[u][d] * (125.0 / 594.0) + k6[u][d] * (512.0 / 1771.0)) * dt;
            double e = k1[u][d] * (37.0 / 378.0 - 2825.0 / 27648.0) + k3[u][d] * (250.0 / 621.0 - 18575.0 / 48384.0) +
                       k4[u][d] * (125.0 / 594.0 - 13525.0 / 55296.0) + k5[u][d] * (0.0 - 277.0 / 14336.0) +
                       k6[u][d] * (512.0 / 1771.0 - 1.0 / 4.0);
            err[u][d] = dt * std::fabs(e) + 1e-18;
            if (!std::isfinite(xn[u][d]) || !std::isfinite(err[u][d])) finite = 0;
        }
}

void dense_store(long long sidx, System& s, const Arrays& a, const Opts& o, int update, int initial,
                 int end_reached)
{
    int store;
    if (initial) {
        store = 1;
    } else if (update == 1) {
        store = (s.didx < o.ndo && s.dense_next < s.t && s.skipped >= o.dense_freq - 1) ? 1 : 0;
        if (s.didx < o.ndo && (end_reached == 1 || s.udt == 1)) store = 1;
    } else {
        store = 0;
    }
    const long long nu = a.ns * UPS;
    if (store == 1 && s.didx < o.ndo) {
        for (int u = 0; u < UPS; u++)
            for (int d = 0; d < UD; d++)
                a.dstate[sidx * UPS + u + d * nu + static_cast<long long>(s.didx) * nu * UD] = s.x[u][d];
        a.dtime[sidx + static_cast<long long>(s.didx) * a.ns] = s.t;
    }
    if (store == 1) {
        if (s.didx < o.ndo) s.didx++;
        s.skipped = 0;
        s.dense_next = std::fmin(s.t + o.dense_min_dt, s.td[1]);
    }
    if (store == 0 && update == 1) s.skipped++;
}

void solve_system(long long sidx, const Arrays& a, const Opts& o, int algorithm)
{
    const long long ns = a.ns, nu = ns * UPS;
    const int sid = static_cast<int>(sidx);
    System* sp_ = new System();
    System& s = *sp_;
    s.td[0] = a.td[sidx];
    s.td[1] = a.td[sidx + ns];
    s.t = a.t[sidx];
    s.dt = o.initial_dt;
    s.newdt = o.initial_dt;
    s.didx = a.didx[sidx];
    s.udt = 0;
    s.skipped = 0;
    s.dense_next = s.t;
    for (int k = 0; k < NSP; k++) s.sp[k] = a.sp[sidx + k * ns];
    for (int k = 0; k < NSA; k++) s.sacc[k] = a.sacc[sidx + k * ns];
    for (int k = 0; k < NISA; k++) s.isacc[k] = a.isacc[sidx + k * ns];
    for (int k = 0; k < NC; k++) s.cstr[k] = a.cstr[sidx + k * ns];
    for (int u = 0; u < UPS; u++) {
        const long long g = sidx * UPS + u;
        for (int d = 0; d < UD; d++) s.x[u][d] = a.x[g + d * nu];
        for (int k = 0; k < NUP; k++) s.up[u][k] = a.up[g + k * nu];
        for (int k = 0; k < NUA; k++) s.uacc[u][k] = a.uacc[g + k * nu];
        for (int k = 0; k < NIUA; k++) s.iuacc[u][k] = a.iuacc[g + k * nu];
    }
    double gp[one_at_least<NGP>()];
    int igp[one_at_least<NIGP>()];
    for (int k = 0; k < NGP; k++) gp[k] = a.gp[k];
    for (int k = 0; k < NIGP; k++) igp[k] = a.igp[k];
    const double* M = a.cmat;

    for (int u = 0; u < UPS; u++)
        CoupledSystems_PerBlock_Initialization<double>(sid, u, s.didx, s.t, s.dt, s.td, s.x[u], s.up[u], s.sp, gp, igp,
                                                       s.uacc[u], s.iuacc[u], s.sacc, s.isacc);
    if (NE > 0)
        for (int u = 0; u < UPS; u++)
            CoupledSystems_PerBlock_EventFunction<double>(sid, u, s.ga[u], s.t, s.dt, s.td, s.x[u], s.up[u], s.sp, gp,
                                                          igp, s.uacc[u], s.iuacc[u], s.sacc, s.isacc);
    if (o.ndo > 0) dense_store(sidx, s, a, o, 1, 1, 0);

    int status = 0, nacc = 0, nrej = 0, terminate = 0;
    long long attempts = 0;
    static thread_local double xn[UPS][UD], err[UPS][UD];
    while (!terminate) {
        if (attempts >= o.max_attempts) {
            status |= 8;
            break;
        }
        attempts++;
        int update = 1, finite = 1, end_reached = 0;
        double dt = s.newdt;
        const double t = s.t;
        if (dt > (s.td[1] - t)) {
            dt = s.td[1] - t;
            end_reached = 1;
        }
        s.dt = dt;
        double newdt;
        if (algorithm == 0) {
            rk4(sid, s, gp, igp, M, a.cidx, t, dt, xn, finite);
            if (finite == 0) {
                terminate = 1;
                update = 0;
                status |= 1;
            }
            newdt = o.initial_dt;
        } else {
            rkck45(sid, s, gp, igp, M, a.cidx, t, dt, xn, err, finite);
            double ratio = 1e30;
            int upd = 1;
            for (int u = 0; u < UPS; u++)
                for (int d = 0; d < UD; d++) {
                    const double tol = std::fmax(a.rtol[d] * std::fmax(std::fabs(xn[u][d]), std::fabs(s.x[u][d])),
                                                 a.atol[d]);
                    upd = upd & (err[u][d] < tol);
                    ratio = std::fmin(ratio, tol / err[u][d]);
                }
            update = upd;
            double q = (update == 1) ? 0.8 * std::pow(ratio, 1.0 / 5.0) : 0.8 * std::pow(ratio, 1.0 / 4.0);
            if (!std::isfinite(q)) finite = 0;
            const double guard = o.min_dt * 1.01;
            if (finite == 0) {
                q = o.shrink;
                update = 0;
                if (dt < guard) {
                    terminate = 1;
                    status |= 1;
                }
            } else if (dt < guard) {
                update = 1;
                status |= 2;
            }
            q = std::fmin(q, o.grow);
            q = std::fmax(q, o.shrink);
            newdt = dt * q;
            newdt = std::fmin(newdt, o.max_dt);
            newdt = std::fmax(newdt, o.min_dt);
        }
        s.newdt = newdt;

        if (NE > 0 && terminate == 0) {
            for (int u = 0; u < UPS; u++) {
                double xu[UD];
                for (int d = 0; d < UD; d++) xu[d] = xn[u][d];
                CoupledSystems_PerBlock_EventFunction<double>(sid, u, s.gn[u], t + dt, s.newdt, s.td, xu, s.up[u],
                                                              s.sp, gp, igp, s.uacc[u], s.iuacc[u], s.sacc, s.isacc);
            }
            double evdt = dt;
            int corrected = 0;
            if (update == 1) {
                for (int u = 0; u < UPS; u++)
                    for (int e = 0; e < NE; e++) {
                        const double ga = s.ga[u][e], gn = s.gn[u][e], tol = a.etol[e];
                        const int dir = a.edir[e];
                        if (((ga > tol) && (gn < -tol) && (dir <= 0)) || ((ga < -tol) && (gn > tol) && (dir >= 0))) {
                            evdt = std::fmin(evdt, -ga / (gn - ga) * dt);
                            corrected = 1;
                        }
                    }
            }
            if (corrected == 1) {
                if (evdt < o.min_dt) {
                    status |= 4;
                } else {
                    s.newdt = evdt;
                    update = 0;
                }
            }
        }

        if (update == 1) {
            nacc++;
            s.t += dt;
            for (int u = 0; u < UPS; u++)
                for (int d = 0; d < UD; d++) s.x[u][d] = xn[u][d];
            for (int u = 0; u < UPS; u++)
                CoupledSystems_PerBlock_ActionAfterSuccessfulTimeStep<double>(sid, u, s.udt, s.t, s.dt, s.td, s.x[u],
                                                                              s.up[u], s.sp, gp, igp, s.uacc[u],
                                                                              s.iuacc[u], s.sacc, s.isacc);
            if (NE > 0) {
                for (int u = 0; u < UPS; u++)
                    for (int e = 0; e < NE; e++) {
                        const double ga = s.ga[u][e], gn = s.gn[u][e], tol = a.etol[e];
                        const int dir = a.edir[e];
                        if (((ga > tol) && (std::fabs(gn) < tol) && (dir <= 0)) ||
                            ((ga < -tol) && (std::fabs(gn) < tol) && (dir >= 0)))
                            CoupledSystems_PerBlock_ActionAfterEventDetection<double>(
                                sid, u, e, s.udt, s.t, s.dt, s.td, s.x[u], s.up[u], s.sp, gp, igp, s.uacc[u],
                                s.iuacc[u], s.sacc, s.isacc);
                    }
                for (int u = 0; u < UPS; u++)
                    CoupledSystems_PerBlock_EventFunction<double>(sid, u, s.gn[u], s.t, s.newdt, s.td, s.x[u], s.up[u],
                                                                  s.sp, gp, igp, s.uacc[u], s.iuacc[u], s.sacc,
                                                                  s.isacc);
                for (int u = 0; u < UPS; u++)
                    for (int e = 0; e < NE; e++) s.ga[u][e] = s.gn[u][e];
            }
        } else {
            nrej++;
        }
        if (o.ndo > 0) dense_store(sidx, s, a, o, update, 0, end_reached);
        if (update == 1 && (end_reached == 1 || s.udt == 1)) terminate = 1;
    }

    for (int u = 0; u < UPS; u++)
        CoupledSystems_PerBlock_Finalization<double>(sid, u, s.didx, s.t, s.dt, s.td, s.x[u], s.up[u], s.sp, gp, igp,
                                                     s.uacc[u], s.iuacc[u], s.sacc, s.isacc);
    for (int u = 0; u < UPS; u++) {
        const long long g = sidx * UPS + u;
        for (int d = 0; d < UD; d++) a.x[g + d * nu] = s.x[u][d];
        for (int k = 0; k < NUA; k++) a.uacc[g + k * nu] = s.uacc[u][k];
        for (int k = 0; k < NIUA; k++) a.iuacc[g + k * nu] = s.iuacc[u][k];
    }
    a.t[sidx] = s.t;
    a.td[sidx] = s.td[0];
    a.td[sidx + ns] = s.td[1];
    a.didx[sidx] = s.didx;
    for (int k = 0; k < NSA; k++) a.sacc[sidx + k * ns] = s.sacc[k];
    for (int k = 0; k < NISA; k++) a.isacc[sidx + k * ns] = s.isacc[k];
    if (a.status) a.status[sidx] = status;
    if (a.nacc) a.nacc[sidx] = nacc;
    if (a.nrej) a.nrej[sidx] = nrej;
    delete sp_;
}

}  // namespace

extern "C" {

// {UPS, UD, NC, CBW, CCI, NUP, NSP, NGP, NIGP, NUA, NIUA, NSA, NISA, NE, MAT}
__attribute__((visibility("default"))) void oracle_cb_shape(int* out)
{
    const int v[] = {UPS, UD, NC, CBW, CCI, NUP, NSP, NGP, NIGP, NUA, NIUA, NSA, NISA, NE, MAT};
    for (int i = 0; i < 15; i++) out[i] = v[i];
}

// Integrate systems [first, first + count) of the ensemble; threads <= 0:
// all available.
__attribute__((visibility("default"))) int oracle_cb_solve(const Arrays* a, const Opts* o, int algorithm,
                                                           long long first, long long count, int threads)
{
    if (!a || !o || first < 0 || count < 0 || first + count > a->ns) return 1;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (long long i = first; i < first + count; i++) solve_system(i, *a, *o, algorithm);
    return 0;
}

// Replay of systems [first, first + count) with a frozen step sequence
// (dt [max_steps][NS], n_steps [NS]): the stepper only, no controller, events
// or actions; x, t and sp as given. The discrete map the adjoint
// differentiates, for finite-difference checks.
__attribute__((visibility("default"))) int oracle_cb_replay(const Arrays* a, const Opts* o, int algorithm,
                                                            const double* dt, const int* n_steps, int max_steps,
                                                            long long first, long long count, int threads)
{
    if (!a || !o || !dt || !n_steps || first < 0 || count < 0 || first + count > a->ns) return 1;
    (void)o;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (long long sidx = first; sidx < first + count; sidx++) {
        const long long ns = a->ns, nu = ns * UPS;
        const int sid = static_cast<int>(sidx);
        System* sp_ = new System();
        System& sy = *sp_;
        for (int k = 0; k < NSP; k++) sy.sp[k] = a->sp[sidx + k * ns];
        for (int k = 0; k < NSA; k++) sy.sacc[k] = a->sacc[sidx + k * ns];
        for (int k = 0; k < NISA; k++) sy.isacc[k] = a->isacc[sidx + k * ns];
        for (int k = 0; k < NC; k++) sy.cstr[k] = a->cstr[sidx + k * ns];
        for (int u = 0; u < UPS; u++) {
            const long long g = sidx * UPS + u;
            for (int d = 0; d < UD; d++) sy.x[u][d] = a->x[g + d * nu];
            for (int k = 0; k < NUP; k++) sy.up[u][k] = a->up[g + k * nu];
            for (int k = 0; k < NUA; k++) sy.uacc[u][k] = a->uacc[g + k * nu];
            for (int k = 0; k < NIUA; k++) sy.iuacc[u][k] = a->iuacc[g + k * nu];
        }
        double gp[one_at_least<NGP>()];
        int igp[one_at_least<NIGP>()];
        for (int k = 0; k < NGP; k++) gp[k] = a->gp[k];
        for (int k = 0; k < NIGP; k++) igp[k] = a->igp[k];
        double t = a->t[sidx];
        const int n = n_steps[sidx] < max_steps ? n_steps[sidx] : max_steps;
        static thread_local double xn[UPS][UD], err[UPS][UD];
        for (int k = 0; k < n; k++) {
            const double h = dt[static_cast<long long>(k) * ns + sidx];
            int finite = 1;
            if (algorithm == 0)
                rk4(sid, sy, gp, igp, a->cmat, a->cidx, t, h, xn, finite);
            else
                rkck45(sid, sy, gp, igp, a->cmat, a->cidx, t, h, xn, err, finite);
            for (int u = 0; u < UPS; u++)
                for (int d = 0; d < UD; d++) sy.x[u][d] = xn[u][d];
            t += h;
        }
        for (int u = 0; u < UPS; u++)
            for (int d = 0; d < UD; d++) a->x[sidx * UPS + u + d * nu] = sy.x[u][d];
        a->t[sidx] = t;
        delete sp_;
    }
    return 0;
}

}  // extern "C"

// CPU oracle of the per-thread ensemble solver.
//
// TEST INFRASTRUCTURE ONLY. This is the oracle the GPU kernels are compared
// against (tests, smoke test, the bench's CPU baseline); the product never
// links or calls it.
//
// A plain restatement of the reference algorithm, one instance at a time:
//   loop order        SourceCodes/SingleSystem_PerThread_Solver.cuh:117-435
//   RK4 stepper       SourceCodes/SingleSystem_PerThread_ExplicitRungeKutta_Steppers.cuh:6-117
//   RKCK45 stepper    SourceCodes/SingleSystem_PerThread_ExplicitRungeKutta_Steppers.cuh:121-289
//   controllers       SourceCodes/SingleSystem_PerThread_ExplicitRungeKutta_ErrorControllers.cuh:5-85
//   event control     SourceCodes/SingleSystem_PerThread_EventHandling.cuh:5-44
//   event detection   SourceCodes/SingleSystem_PerThread_Solver.cuh:323-363
//   dense output      SourceCodes/SingleSystem_PerThread_DenseOutput.cuh:5-58
// with the same grouping of every floating-point expression, so that built
// with the same flags it agrees bit for bit with the reference's own code
// compiled for the CPU (oracle/_ref, see oracle/build_oracle.py).
//
// Two deliberate differences, both only for inputs the reference handles
// with undefined behaviour: a dense-output store with a full buffer is
// skipped instead of written out of bounds, and every instance stops after
// max_attempts step attempts (status flag 8).
//
// Compiled once per system: -DMPGOS_SYSTEM_HEADER="<hooks>.cuh".
#include "host_shim.hpp"

#include MPGOS_SYSTEM_HEADER

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int SD = MPGOS_SYS_SD, NCP = MPGOS_SYS_NCP, NSP = MPGOS_SYS_NSP, NISP = MPGOS_SYS_NISP;
constexpr int NE = MPGOS_SYS_NE, NA = MPGOS_SYS_NA, NIA = MPGOS_SYS_NIA;
template <int N> constexpr int one_at_least() { return N > 0 ? N : 1; }

struct Opts {
    double initial_dt, max_dt, min_dt, grow, shrink, dense_min_dt;
    int dense_freq, ndo;
    long long max_attempts;
};

struct Arrays {
    long long nt;
    double *td, *x, *t, *cp, *acc, *dtime, *dstate;
    const double *sp, *rtol, *atol, *etol;
    const int *spi, *edir;
    int *acci, *didx, *status, *nacc, *nrej;
};

// RK4, reference Steppers.cuh:6-117.
void rk4(int tid, int nt, double t, double dt, double* x, double* xn, int& finite, double* cp, double* sp,
         int* spi, double* acc, int* acci)
{
    double X[SD], k[SD];
    const double h2 = 0.5 * dt;
    const double h6 = (1.0 / 6.0) * dt;
    PerThread_OdeFunction(tid, nt, xn, x, t, cp, sp, spi, acc, acci);
    double T = t + h2;
    for (int i = 0; i < SD; i++) X[i] = x[i] + xn[i] * h2;
    PerThread_OdeFunction(tid, nt, k, X, T, cp, sp, spi, acc, acci);
    for (int i = 0; i < SD; i++) {
        xn[i] = xn[i] + 2.0 * k[i];
        X[i]  = x[i] + k[i] * h2;
    }
    PerThread_OdeFunction(tid, nt, k, X, T, cp, sp, spi, acc, acci);
    T = t + dt;
    for (int i = 0; i < SD; i++) {
        xn[i] = xn[i] + 2.0 * k[i];
        X[i]  = x[i] + k[i] * dt;
    }
    PerThread_OdeFunction(tid, nt, k, X, T, cp, sp, spi, acc, acci);
    for (int i = 0; i < SD; i++) {
        xn[i] = x[i] + h6 * (xn[i] + k[i]);
        if (!std::isfinite(xn[i])) finite = 0;
    }
}

// Cash-Karp 4(5), reference Steppers.cuh:121-289.
void rkck45(int tid, int nt, double t, double dt, double* x, double* xn, double* err, int& finite, double* cp,
            double* sp, int* spi, double* acc, int* acci)
{
    double X[SD], k1[SD], k2[SD], k3[SD], k4[SD], k5[SD], k6[SD];
    PerThread_OdeFunction(tid, nt, k1, x, t, cp, sp, spi, acc, acci);
    double T = t + dt * (1.0 / 5.0);
    for (int i = 0; i < SD; i++) X[i] = x[i] + dt * ((1.0 / 5.0) * k1[i]);
    PerThread_OdeFunction(tid, nt, k2, X, T, cp, sp, spi, acc, acci);
    T = t + dt * (3.0 / 10.0);
    for (int i = 0; i < SD; i++) X[i] = x[i] + dt * ((3.0 / 40.0) * k1[i] + (9.0 / 40.0) * k2[i]);
    PerThread_OdeFunction(tid, nt, k3, X, T, cp, sp, spi, acc, acci);
    T = t + dt * (3.0 / 5.0);
    for (int i = 0; i < SD; i++)
        X[i] = x[i] + dt * ((3.0 / 10.0) * k1[i] + (-9.0 / 10.0) * k2[i] + (6.0 / 5.0) * k3[i]);
    PerThread_OdeFunction(tid, nt, k4, X, T, cp, sp, spi, acc, acci);
    T = t + dt;
    for (int i = 0; i < SD; i++)
        X[i] = x[i] + dt * ((-11.0 / 54.0) * k1[i] + (5.0 / 2.0) * k2[i] + (-70.0 / 27.0) * k3[i] +
                            (35.0 / 27.0) * k4[i]);
    PerThread_OdeFunction(tid, nt, k5, X, T, cp, sp, spi, acc, acci);
    T = t + dt * (7.0 / 8.0);
    for (int i = 0; i < SD; i++)
        X[i] = x[i] + dt * ((1631.0 / 55296.0) * k1[i] + (175.0 / 512.0) * k2[i] + (575.0 / 13824.0) * k3[i] +
                            (44275.0 / 110592.0) * k4[i] + (253.0 / 4096.0) * k5[i]);
    PerThread_OdeFunction(tid, nt, k6, X, T, cp, sp, spi, acc, acci);
    for (int i = 0; i < SD; i++) {
        xn[i] = x[i] + dt * ((37.0 / 378.0) * k1[i] + (250.0 / 621.0) * k3[i] + (125.0 / 594.0) * k4[i] +
                             (512.0 / 1771.0) * k6[i]);
        double e = (37.0 / 378.0 - 2825.0 / 27648.0) * k1[i] + (250.0 / 621.0 - 18575.0 / 48384.0) * k3[i] +
                   (125.0 / 594.0 - 13525.0 / 55296.0) * k4[i] + (0.0 - 277.0 / 14336.0) * k5[i] +
                   (512.0 / 1771.0 - 1.0 / 4.0) * k6[i];
        err[i] = dt * std::fabs(e) + 1e-18;
        if (!std::isfinite(xn[i]) || !std::isfinite(err[i])) finite = 0;
    }
}

// Adaptive controller, reference ErrorControllers.cuh:23-85.
void control_rkck45(const Opts& o, double dt, const double* x, const double* xn, const double* err,
                    const double* rtol, const double* atol, int& update, int& finite, int& terminate,
                    double& new_dt, int& status)
{
    double ratio = 1e30;
    for (int i = 0; i < SD; i++) {
        const double tol = std::fmax(rtol[i] * std::fmax(std::fabs(xn[i]), std::fabs(x[i])), atol[i]);
        update = update && (err[i] < tol);
        ratio = std::fmin(ratio, tol / err[i]);
    }
    double q = update == 1 ? 0.9 * std::pow(ratio, 1.0 / 5.0) : 0.9 * std::pow(ratio, 1.0 / 4.0);
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
    new_dt = dt * q;
    new_dt = std::fmin(new_dt, o.max_dt);
    new_dt = std::fmax(new_dt, o.min_dt);
}

void dense_store(long long i, long long nt, int store, int& didx, int ndo, double* dtime, double* dstate, double t,
                 const double* x, int& skipped, double& dense_next, double dense_min_dt, double upper)
{
    if (store == 1) {
        if (didx < ndo) {
            dtime[i + (long long)didx * nt] = t;
            for (int c = 0; c < SD; c++) dstate[i + (long long)didx * nt * SD + c * nt] = x[c];
            didx++;
        }
        skipped = 0;
        dense_next = std::fmin(t + dense_min_dt, upper);
    } else {
        skipped++;
    }
}

void integrate_instance(long long i, int algorithm, const Arrays& a, const Opts& o, double* sp, int* spi)
{
    const long long nt = a.nt;
    const int ti = (int)i, nti = (int)nt;
    double td[2], x[SD], xn[SD], err[SD];
    double cp[one_at_least<NCP>()], acc[one_at_least<NA>()], ga[one_at_least<NE>()], gn[one_at_least<NE>()];
    int acci[one_at_least<NIA>()];
    for (int k = 0; k < 2; k++) td[k] = a.td[i + k * nt];
    for (int k = 0; k < SD; k++) x[k] = a.x[i + k * nt];
    for (int k = 0; k < NCP; k++) cp[k] = a.cp[i + k * nt];
    for (int k = 0; k < NA; k++) acc[k] = a.acc[i + k * nt];
    for (int k = 0; k < NIA; k++) acci[k] = a.acci[i + k * nt];
    double t = a.t[i];
    double dt = o.initial_dt, new_dt = o.initial_dt;
    int didx = a.didx[i];
    int skipped = 0, terminate = 0, udt = 0, status = 0, nacc = 0, nrej = 0;
    double dense_next = t;
    long long attempts = 0;

    PerThread_Initialization(ti, nti, didx, t, dt, td, x, cp, sp, spi, acc, acci);
    if (NE > 0) PerThread_EventFunction(ti, nti, ga, t, dt, td, x, cp, sp, spi, acc, acci);
    if (o.ndo > 0)
        dense_store(i, nt, 1, didx, o.ndo, a.dtime, a.dstate, t, x, skipped, dense_next, o.dense_min_dt, td[1]);

    while (terminate == 0) {
        if (attempts >= o.max_attempts) {
            status |= 8;
            break;
        }
        attempts++;
        int update = 1, finite = 1, end_reached = 0;
        dt = new_dt;
        if (dt > (td[1] - t)) {
            dt = td[1] - t;
            end_reached = 1;
        }
        if (algorithm == 0) {
            rk4(ti, nti, t, dt, x, xn, finite, cp, sp, spi, acc, acci);
            if (finite == 0) {
                terminate = 1;
                status |= 1;
            }
            new_dt = o.initial_dt;
        } else {
            rkck45(ti, nti, t, dt, x, xn, err, finite, cp, sp, spi, acc, acci);
            control_rkck45(o, dt, x, xn, err, a.rtol, a.atol, update, finite, terminate, new_dt, status);
        }
        if (NE > 0) {
            PerThread_EventFunction(ti, nti, gn, t + dt, dt, td, xn, cp, sp, spi, acc, acci);
            double event_dt = dt;
            int corrected = 0;
            if (update == 1 && terminate == 0) {
                for (int e = 0; e < NE; e++) {
                    if (((ga[e] > a.etol[e]) && (gn[e] < -a.etol[e]) && (a.edir[e] <= 0)) ||
                        ((ga[e] < -a.etol[e]) && (gn[e] > a.etol[e]) && (a.edir[e] >= 0))) {
                        event_dt = std::fmin(event_dt, -ga[e] / (gn[e] - ga[e]) * dt);
                        corrected = 1;
                    }
                }
            }
            if (corrected == 1) {
                if (event_dt < o.min_dt) {
                    status |= 4;
                } else {
                    new_dt = event_dt;
                    update = 0;
                }
            }
        }
        if (update == 1) {
            nacc++;
            t += dt;
            for (int k = 0; k < SD; k++) x[k] = xn[k];
            PerThread_ActionAfterSuccessfulTimeStep(ti, nti, udt, t, dt, td, x, cp, sp, spi, acc, acci);
            if (NE > 0) {
                for (int e = 0; e < NE; e++) {
                    const double tol = a.etol[e];
                    const int dir = a.edir[e];
                    if (((ga[e] > tol) && (std::fabs(gn[e]) < tol) && (dir <= 0)) ||
                        ((ga[e] < -tol) && (std::fabs(gn[e]) < tol) && (dir >= 0)))
                        PerThread_ActionAfterEventDetection(ti, nti, e, udt, t, dt, td, x, cp, sp, spi, acc, acci);
                }
                PerThread_EventFunction(ti, nti, gn, t, dt, td, x, cp, sp, spi, acc, acci);
                for (int e = 0; e < NE; e++) ga[e] = gn[e];
            }
            if (o.ndo > 0) {
                int store = ((didx < o.ndo) && (dense_next < t) && (skipped >= (o.dense_freq - 1))) ? 1 : 0;
                if ((didx < o.ndo) && ((end_reached == 1) || (udt == 1))) store = 1;
                dense_store(i, nt, store, didx, o.ndo, a.dtime, a.dstate, t, x, skipped, dense_next, o.dense_min_dt,
                            td[1]);
            }
            if ((end_reached == 1) || (udt == 1)) terminate = 1;
        } else {
            nrej++;
        }
    }
    PerThread_Finalization(ti, nti, didx, t, dt, td, x, cp, sp, spi, acc, acci);
    for (int k = 0; k < 2; k++) a.td[i + k * nt] = td[k];
    for (int k = 0; k < SD; k++) a.x[i + k * nt] = x[k];
    for (int k = 0; k < NCP; k++) a.cp[i + k * nt] = cp[k];
    for (int k = 0; k < NA; k++) a.acc[i + k * nt] = acc[k];
    for (int k = 0; k < NIA; k++) a.acci[i + k * nt] = acci[k];
    a.t[i] = t;
    a.didx[i] = didx;
    if (a.status) a.status[i] = status;
    if (a.nacc) a.nacc[i] = nacc;
    if (a.nrej) a.nrej[i] = nrej;
}

}  // namespace

extern "C" {

int oracle_pt_shape(int* out7)
{
    const int s[7] = {SD, NCP, NSP, NISP, NE, NA, NIA};
    for (int i = 0; i < 7; i++) out7[i] = s[i];
    return 0;
}

// Integrate instances [first, first+count) of an ensemble of nt instances
// (arrays in the reference's SoA layout). threads <= 0: all OpenMP threads.
int oracle_pt_solve(int algorithm, long long nt, long long first, long long count, int ndo, double* td, double* x,
                    double* t, double* cp, const double* sp, const int* spi, double* acc, int* acci,
                    const double* rtol, const double* atol, const double* etol, const int* edir, int* didx,
                    double* dtime, double* dstate, int* status, int* nacc, int* nrej, const double* opt6,
                    int dense_freq, long long max_attempts, int threads)
{
    if (nt < 1 || first < 0 || count < 0 || first + count > nt || (algorithm != 0 && algorithm != 1)) return 1;
    Arrays a{nt, td, x, t, cp, acc, dtime, dstate, sp, rtol, atol, etol, spi, edir, acci, didx, status, nacc, nrej};
    Opts o{opt6[0], opt6[1], opt6[2], opt6[3], opt6[4], opt6[5], dense_freq, ndo, max_attempts};
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel
#endif
    {
        // Hooks take non-const pointers; each thread works on its own copy.
        std::vector<double> spc(sp, sp + NSP);
        std::vector<int> spic(spi, spi + NISP);
        spc.push_back(0.0);
        spic.push_back(0);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 64)
#endif
        for (long long i = first; i < first + count; i++) integrate_instance(i, algorithm, a, o, spc.data(), spic.data());
    }
    return 0;
}

// Integrate instances [first, first+count) with a given step sequence:
// dt[k*nt + i] for k < n_steps[i] (the frozen step sizes of a recorded GPU
// forward pass), no step-size control, no events. x, t are updated in place.
// This is the discrete map whose derivative the GPU adjoint computes, so
// central differences of it check the adjoint without step-selection noise.
int oracle_pt_replay(int algorithm, long long nt, long long first, long long count, double* x, double* t,
                     const double* cp, const double* sp, const int* spi, const double* acc, const int* acci,
                     const double* dt, const int* n_steps, int threads)
{
    if (nt < 1 || first < 0 || count < 0 || first + count > nt || (algorithm != 0 && algorithm != 1)) return 1;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel
#endif
    {
        std::vector<double> spc(sp, sp + NSP);
        std::vector<int> spic(spi, spi + NISP);
        spc.push_back(0.0);
        spic.push_back(0);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 64)
#endif
        for (long long i = first; i < first + count; i++) {
            double xi[SD], xn[SD], err[SD], cpi[one_at_least<NCP>()], acci_d[one_at_least<NA>()];
            int accii[one_at_least<NIA>()];
            for (int k = 0; k < SD; k++) xi[k] = x[i + k * nt];
            for (int k = 0; k < NCP; k++) cpi[k] = cp[i + k * nt];
            for (int k = 0; k < NA; k++) acci_d[k] = acc[i + k * nt];
            for (int k = 0; k < NIA; k++) accii[k] = acci[i + k * nt];
            double ti = t[i];
            for (int s = 0; s < n_steps[i]; s++) {
                const double h = dt[(long long)s * nt + i];
                int finite = 1;
                if (algorithm == 0)
                    rk4((int)i, (int)nt, ti, h, xi, xn, finite, cpi, spc.data(), spic.data(), acci_d, accii);
                else
                    rkck45((int)i, (int)nt, ti, h, xi, xn, err, finite, cpi, spc.data(), spic.data(), acci_d, accii);
                for (int k = 0; k < SD; k++) xi[k] = xn[k];
                ti += h;
            }
            for (int k = 0; k < SD; k++) x[i + k * nt] = xi[k];
            t[i] = ti;
        }
    }
    return 0;
}

// Dense-output interpolation, the CPU statement of the GPU extension
// (csrc/perthread/dense_interp.cuh): for every instance and requested time
// tau, the cubic Hermite polynomial through the stored points (t_k, x_k),
// (t_k+1, x_k+1) bracketing tau, slopes f(t_k, x_k) and f(t_k+1, x_k+1) from
// the hooks; NaN outside [t_0, t_last]; tau equal to the last stored time or
// a repeated time stamp gives the later stored state. out [n_times][SD][nt].
int oracle_pt_dense_interpolate(long long nt, int ndo, const int* didx, const double* dtime, const double* dstate,
                                const double* cp, const double* sp, const int* spi, const double* acc,
                                const int* acci, const double* times, int n_times, double* out)
{
    if (nt < 1 || ndo < 0 || n_times < 0) return 1;
    std::vector<double> spc(sp, sp + NSP);
    std::vector<int> spic(spi, spi + NISP);
    spc.push_back(0.0);
    spic.push_back(0);
    const long long step = nt * SD;
    for (long long i = 0; i < nt; i++) {
        double cpi[one_at_least<NCP>()], acci_d[one_at_least<NA>()];
        int accii[one_at_least<NIA>()];
        for (int k = 0; k < NCP; k++) cpi[k] = cp[i + k * nt];
        for (int k = 0; k < NA; k++) acci_d[k] = acc[i + k * nt];
        for (int k = 0; k < NIA; k++) accii[k] = acci[i + k * nt];
        const int n = std::min(didx[i], ndo);
        for (int j = 0; j < n_times; j++) {
            const double tau = times[j];
            double* o = out + (long long)j * step + i;
            int k = -1;
            for (int m = 0; m < n; m++)
                if (dtime[i + (long long)m * nt] <= tau) k = m;
            const bool inside = k >= 0 && (k < n - 1 || dtime[i + (long long)k * nt] == tau);
            if (!inside) {
                for (int c = 0; c < SD; c++) o[c * nt] = std::nan("");
                continue;
            }
            if (k == n - 1) {
                for (int c = 0; c < SD; c++) o[c * nt] = dstate[i + c * nt + k * step];
                continue;
            }
            const double t0 = dtime[i + (long long)k * nt], t1 = dtime[i + (long long)(k + 1) * nt];
            double x0[SD], x1[SD], f0[SD], f1[SD];
            for (int c = 0; c < SD; c++) {
                x0[c] = dstate[i + c * nt + k * step];
                x1[c] = dstate[i + c * nt + (k + 1) * step];
            }
            const double h = t1 - t0;
            if (!(h > 0.0)) {
                for (int c = 0; c < SD; c++) o[c * nt] = x1[c];
                continue;
            }
            PerThread_OdeFunction((int)i, (int)nt, f0, x0, t0, cpi, spc.data(), spic.data(), acci_d, accii);
            PerThread_OdeFunction((int)i, (int)nt, f1, x1, t1, cpi, spc.data(), spic.data(), acci_d, accii);
            const double s = (tau - t0) / h, r = 1.0 - s;
            const double h00 = (1.0 + 2.0 * s) * r * r, h10 = s * r * r * h;
            const double h01 = s * s * (3.0 - 2.0 * s), h11 = s * s * (s - 1.0) * h;
            for (int c = 0; c < SD; c++) o[c * nt] = h00 * x0[c] + h10 * f0[c] + h01 * x1[c] + h11 * f1[c];
        }
    }
    return 0;
}

int oracle_pt_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"

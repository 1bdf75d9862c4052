// Keller-Miksis single-bubble radial dynamics in dimensionless form, dual-
// frequency forcing, 21 per-instance control parameters.
//
// Hook file in the reference's user-hook convention. The right-hand side is the
// Keller-Miksis equation with the coefficient layout of
// Tutorials_SingleSystem_PerThread/T4_QuasiperiodicForcing/QuasiperiodicForcing_SystemDefinition.cuh:7-33
// (cPAR[0..12] are the precomputed coefficients, cPAR[13] the reference time,
// cPAR[14] the reference radius, cPAR[15..20] the physical parameters); the
// host-side coefficient formulas live in mpgos_gb300/workloads.py.
//
// Time is normalised by the first forcing period, so one launch over TD = [0, 1]
// is one acoustic period; Initialization resets T to TD0 every launch.
//
//   SD = 2 (R/R_E, dR/dt), NCP = 21, NSP = 0, NISP = 0,
//   NE = 1: EF[0] = x1, detected falling (direction -1) = a radius maximum,
//   NA = 1: largest radius seen at a maximum event in this period
//           (reset to the period's initial radius),
//   NIA = 2: maximum events (cumulative), accepted steps (cumulative).
#ifndef MPGOS_SYSTEM_KELLER_MIKSIS_CUH
#define MPGOS_SYSTEM_KELLER_MIKSIS_CUH

#define MPGOS_SYS_NAME "keller_miksis"
#define MPGOS_SYS_SD   2
#define MPGOS_SYS_NCP  21
#define MPGOS_SYS_NSP  0
#define MPGOS_SYS_NISP 0
#define MPGOS_SYS_NE   1
#define MPGOS_SYS_NA   1
#define MPGOS_SYS_NIA  2

#ifndef MPGOS_KM_PI
#define MPGOS_KM_PI 3.14159265358979323846
#endif

template <class Precision>
__forceinline__ __device__ void PerThread_OdeFunction(
    int tid, int NT,
    Precision* F, Precision* X, Precision T,
    Precision* cPAR, Precision* sPAR, int* sPARi, Precision* ACC, int* ACCi)
{
    const Precision one = static_cast<Precision>(1.0);
    Precision rx1 = one / X[0];
    Precision p   = pow(rx1, cPAR[10]);

    Precision s1;
    Precision c1;
    sincospi(static_cast<Precision>(2.0) * T, &s1, &c1);

    Precision arg = static_cast<Precision>(2.0) * cPAR[11] * static_cast<Precision>(MPGOS_KM_PI) * T + cPAR[12];
    Precision s2  = sin(arg);
    Precision c2  = cos(arg);

    Precision N = (cPAR[0] + cPAR[1] * X[1]) * p
                - cPAR[2] * (one + cPAR[9] * X[1])
                - cPAR[3] * rx1
                - cPAR[4] * X[1] * rx1
                - static_cast<Precision>(1.5) * (one - cPAR[9] * X[1] * static_cast<Precision>(1.0 / 3.0)) * X[1] * X[1]
                - (cPAR[5] * s1 + cPAR[6] * s2) * (one + cPAR[9] * X[1])
                - X[0] * (cPAR[7] * c1 + cPAR[8] * c2);
    Precision D  = X[0] - cPAR[9] * X[0] * X[1] + cPAR[4] * cPAR[9];
    Precision rD = one / D;

    F[0] = X[1];
    F[1] = N * rD;
}

template <class Precision>
__forceinline__ __device__ void PerThread_EventFunction(
    int tid, int NT, Precision* EF,
    Precision T, Precision dT, Precision* TD, Precision* X,
    Precision* cPAR, Precision* sPAR, int* sPARi, Precision* ACC, int* ACCi)
{
    EF[0] = X[1];
}

template <class Precision>
__forceinline__ __device__ void PerThread_ActionAfterEventDetection(
    int tid, int NT, int IDX, int& UDT,
    Precision& T, Precision& dT, Precision* TD, Precision* X,
    Precision* cPAR, Precision* sPAR, int* sPARi, Precision* ACC, int* ACCi)
{
    if (X[0] > ACC[0])
        ACC[0] = X[0];
    ACCi[0]++;
}

template <class Precision>
__forceinline__ __device__ void PerThread_ActionAfterSuccessfulTimeStep(
    int tid, int NT, int& UDT,
    Precision& T, Precision& dT, Precision* TD, Precision* X,
    Precision* cPAR, Precision* sPAR, int* sPARi, Precision* ACC, int* ACCi)
{
    ACCi[1]++;
}

template <class Precision>
__forceinline__ __device__ void PerThread_Initialization(
    int tid, int NT, int& DOIDX,
    Precision& T, Precision& dT, Precision* TD, Precision* X,
    Precision* cPAR, Precision* sPAR, int* sPARi, Precision* ACC, int* ACCi)
{
    T      = TD[0];
    ACC[0] = X[0];
}

template <class Precision>
__forceinline__ __device__ void PerThread_Finalization(
    int tid, int NT, int& DOIDX,
    Precision& T, Precision& dT, Precision* TD, Precision* X,
    Precision* cPAR, Precision* sPAR, int* sPARi, Precision* ACC, int* ACCi)
{
}

#endif

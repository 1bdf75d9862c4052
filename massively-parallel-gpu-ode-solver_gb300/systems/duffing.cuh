// Forced hardening Duffing oscillator x'' + k x' + x + x^3 = B cos(t) as a
// first-order system: x0' = x1, x1' = -k x1 - x0 - x0^3 + B cos(T).
//
// Hook file in the reference's user-hook convention (the six PerThread_* device
// templates of Tutorials_SingleSystem_PerThread/T1_Reference/Reference_SystemDefinition.cuh:6-76;
// the reference tutorial integrates the softening variant x - x^3 there).
//
//   SD = 2, NCP = 1 (k), NSP = 1 (B), NISP = 0, NE = 0,
//   NA = 1 (running maximum of x0 over all accepted steps of all phases),
//   NIA = 1 (accepted-step counter).
//
// Every launch is one forcing period [TD0, TD1]: Initialization resets the
// time to TD0 (as Reference_SystemDefinition.cuh:59 does), so a 1024-period run
// is 1024 launches.
#ifndef MPGOS_SYSTEM_DUFFING_CUH
#define MPGOS_SYSTEM_DUFFING_CUH

#define MPGOS_SYS_NAME "duffing"
#define MPGOS_SYS_SD   2
#define MPGOS_SYS_NCP  1
#define MPGOS_SYS_NSP  1
#define MPGOS_SYS_NISP 0
#define MPGOS_SYS_NE   0
#define MPGOS_SYS_NA   1
#define MPGOS_SYS_NIA  1

template <class Precision>
__forceinline__ __device__ void PerThread_OdeFunction(
    int tid, int NT,
    Precision* F, Precision* X, Precision T,
    Precision* cPAR, Precision* sPAR, int* sPARi, Precision* ACC, int* ACCi)
{
    F[0] = X[1];
    F[1] = -cPAR[0] * X[1] - X[0] - X[0] * X[0] * X[0] + sPAR[0] * cos(T);
}

template <class Precision>
__forceinline__ __device__ void PerThread_EventFunction(
    int tid, int NT, Precision* EF,
    Precision T, Precision dT, Precision* TD, Precision* X,
    Precision* cPAR, Precision* sPAR, int* sPARi, Precision* ACC, int* ACCi)
{
}

template <class Precision>
__forceinline__ __device__ void PerThread_ActionAfterEventDetection(
    int tid, int NT, int IDX, int& UDT,
    Precision& T, Precision& dT, Precision* TD, Precision* X,
    Precision* cPAR, Precision* sPAR, int* sPARi, Precision* ACC, int* ACCi)
{
}

template <class Precision>
__forceinline__ __device__ void PerThread_ActionAfterSuccessfulTimeStep(
    int tid, int NT, int& UDT,
    Precision& T, Precision& dT, Precision* TD, Precision* X,
    Precision* cPAR, Precision* sPAR, int* sPARi, Precision* ACC, int* ACCi)
{
    if (X[0] > ACC[0])
        ACC[0] = X[0];
    ACCi[0]++;
}

template <class Precision>
__forceinline__ __device__ void PerThread_Initialization(
    int tid, int NT, int& DOIDX,
    Precision& T, Precision& dT, Precision* TD, Precision* X,
    Precision* cPAR, Precision* sPAR, int* sPARi, Precision* ACC, int* ACCi)
{
    T = TD[0];
}

template <class Precision>
__forceinline__ __device__ void PerThread_Finalization(
    int tid, int NT, int& DOIDX,
    Precision& T, Precision& dT, Precision* TD, Precision* X,
    Precision* cPAR, Precision* sPAR, int* sPARi, Precision* ACC, int* ACCi)
{
}

#endif

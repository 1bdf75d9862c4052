// Forced hardening Duffing oscillator with both coefficients per instance:
// x0' = x1, x1' = -k x1 - x0 - x0^3 + B cos(T), k = cPAR[0], B = cPAR[1].
//
// Hook file in the reference's user-hook convention
// (Tutorials_SingleSystem_PerThread/T1_Reference/Reference_SystemDefinition.cuh:6-76).
// Used by the discrete-adjoint workload: gradients of a terminal loss with
// respect to (k, B, x0(0), x1(0)) need k and B as per-instance parameters.
//
//   SD = 2, NCP = 2 (k, B), NSP = 0, NISP = 0, NE = 0, NA = 0,
//   NIA = 1 (accepted-step counter).
#ifndef MPGOS_SYSTEM_DUFFING_PARAM_CUH
#define MPGOS_SYSTEM_DUFFING_PARAM_CUH

#define MPGOS_SYS_NAME "duffing_param"
#define MPGOS_SYS_SD   2
#define MPGOS_SYS_NCP  2
#define MPGOS_SYS_NSP  0
#define MPGOS_SYS_NISP 0
#define MPGOS_SYS_NE   0
#define MPGOS_SYS_NA   0
#define MPGOS_SYS_NIA  1

template <class Precision>
__forceinline__ __device__ void PerThread_OdeFunction(
    int tid, int NT,
    Precision* F, Precision* X, Precision T,
    Precision* cPAR, Precision* sPAR, int* sPARi, Precision* ACC, int* ACCi)
{
    F[0] = X[1];
    F[1] = -cPAR[0] * X[1] - X[0] - X[0] * X[0] * X[0] + cPAR[1] * cos(T);
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

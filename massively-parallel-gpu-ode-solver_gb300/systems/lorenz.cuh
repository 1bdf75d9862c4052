// Lorenz ensemble: x' = 10 (y - x), y' = rho x - y - x z, z' = x y - (8/3) z.
//
// Hook file in the reference's user-hook convention (the six PerThread_* device
// templates of Tutorials_SingleSystem_PerThread/T1_Reference/Reference_SystemDefinition.cuh:6-76).
// The same file is compiled by the GB300 solver, by the CPU oracle and by the
// reference solver for the parity checks, so all of them integrate identical
// right-hand sides.
//
//   SD = 3, NCP = 1 (rho), NSP = 0, NISP = 0, NE = 0, NA = 0,
//   NIA = 1 (accepted-step counter, incremented after every accepted step, so
//   step counts are measured the same way by every solver).
//
// Constants are cast to Precision so that a float instantiation (FP32-stage
// mode) stays in FP32 arithmetic; for double the values are the same doubles.
#ifndef MPGOS_SYSTEM_LORENZ_CUH
#define MPGOS_SYSTEM_LORENZ_CUH

#define MPGOS_SYS_NAME "lorenz"
#define MPGOS_SYS_SD   3
#define MPGOS_SYS_NCP  1
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
    F[0] = static_cast<Precision>(10.0) * (X[1] - X[0]);
    F[1] = cPAR[0] * X[0] - X[1] - X[0] * X[2];
    F[2] = X[0] * X[1] - static_cast<Precision>(8.0 / 3.0) * X[2];
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
}

template <class Precision>
__forceinline__ __device__ void PerThread_Finalization(
    int tid, int NT, int& DOIDX,
    Precision& T, Precision& dT, Precision* TD, Precision* X,
    Precision* cPAR, Precision* sPAR, int* sPARi, Precision* ACC, int* ACCi)
{
}

#endif

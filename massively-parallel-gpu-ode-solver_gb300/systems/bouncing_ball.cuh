// Bouncing ball with restitution: x0' = x1, x1' = -g (g = sPAR[0]).
// The impact event EF[1] = x0 (falling) reverses and damps the velocity inside
// ActionAfterEventDetection (x1 <- -r x1, r = cPAR[0]), a state jump of the kind
// Tutorials_SingleSystem_PerThread/T6_ImpactDynamics/ImpactDynamics_SystemDefinition.cuh:41-42
// performs. EF[0] = x1 marks the apex; the instance stops itself
// (user-defined termination) after sPARi[0] impacts.
//
//   SD = 2, NCP = 1 (r), NSP = 1 (g), NISP = 1 (impact budget), NE = 2,
//   NA = 1 (last apex height), NIA = 2 (impacts, accepted steps).
#ifndef MPGOS_SYSTEM_BOUNCING_BALL_CUH
#define MPGOS_SYSTEM_BOUNCING_BALL_CUH

#define MPGOS_SYS_NAME "bouncing_ball"
#define MPGOS_SYS_SD   2
#define MPGOS_SYS_NCP  1
#define MPGOS_SYS_NSP  1
#define MPGOS_SYS_NISP 1
#define MPGOS_SYS_NE   2
#define MPGOS_SYS_NA   1
#define MPGOS_SYS_NIA  2

template <class Precision>
__forceinline__ __device__ void PerThread_OdeFunction(
    int tid, int NT,
    Precision* F, Precision* X, Precision T,
    Precision* cPAR, Precision* sPAR, int* sPARi, Precision* ACC, int* ACCi)
{
    F[0] = X[1];
    F[1] = -sPAR[0];
}

template <class Precision>
__forceinline__ __device__ void PerThread_EventFunction(
    int tid, int NT, Precision* EF,
    Precision T, Precision dT, Precision* TD, Precision* X,
    Precision* cPAR, Precision* sPAR, int* sPARi, Precision* ACC, int* ACCi)
{
    EF[0] = X[1];
    EF[1] = X[0];
}

template <class Precision>
__forceinline__ __device__ void PerThread_ActionAfterEventDetection(
    int tid, int NT, int IDX, int& UDT,
    Precision& T, Precision& dT, Precision* TD, Precision* X,
    Precision* cPAR, Precision* sPAR, int* sPARi, Precision* ACC, int* ACCi)
{
    if (IDX == 0)
        ACC[0] = X[0];
    if (IDX == 1) {
        X[1] = -cPAR[0] * X[1];
        ACCi[0]++;
        if (ACCi[0] >= sPARi[0])
            UDT = 1;
    }
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
}

template <class Precision>
__forceinline__ __device__ void PerThread_Finalization(
    int tid, int NT, int& DOIDX,
    Precision& T, Precision& dT, Precision* TD, Precision* X,
    Precision* cPAR, Precision* sPAR, int* sPARi, Precision* ACC, int* ACCi)
{
}

#endif

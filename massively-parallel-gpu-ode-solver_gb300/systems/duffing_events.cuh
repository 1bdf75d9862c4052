// Forced hardening Duffing oscillator with two event functions, accessories,
// dense output and optional user-defined termination; exercises every hook of
// the reference's per-thread interface.
//
// Hook file in the reference's user-hook convention
// (Tutorials_SingleSystem_PerThread/T1_Reference/Reference_SystemDefinition.cuh:6-76).
//
//   x0' = x1, x1' = -k x1 - x0 - x0^3 + B cos(T), k = cPAR[0], B = sPAR[0].
//   Events: EF[0] = x1 (extrema of x0), EF[1] = x0 (zero crossings).
//   ACC[0]  = largest x0 seen at an event-0 detection in this launch,
//   ACC[1]  = smallest x0 over accepted steps of this launch,
//   ACCi[0] = number of event-1 detections (cumulative),
//   ACCi[1] = accepted-step counter (cumulative).
//   sPARi[0] > 0 stops the instance (user-defined termination) once ACCi[0]
//   reaches sPARi[0].
//   Initialization resets T to TD0, the dense-output index to 0 and the two
//   floating accessories, as Reference_SystemDefinition.cuh:54-67 does.
#ifndef MPGOS_SYSTEM_DUFFING_EVENTS_CUH
#define MPGOS_SYSTEM_DUFFING_EVENTS_CUH

#define MPGOS_SYS_NAME "duffing_events"
#define MPGOS_SYS_SD   2
#define MPGOS_SYS_NCP  1
#define MPGOS_SYS_NSP  1
#define MPGOS_SYS_NISP 1
#define MPGOS_SYS_NE   2
#define MPGOS_SYS_NA   2
#define MPGOS_SYS_NIA  2

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
    EF[0] = X[1];
    EF[1] = X[0];
}

template <class Precision>
__forceinline__ __device__ void PerThread_ActionAfterEventDetection(
    int tid, int NT, int IDX, int& UDT,
    Precision& T, Precision& dT, Precision* TD, Precision* X,
    Precision* cPAR, Precision* sPAR, int* sPARi, Precision* ACC, int* ACCi)
{
    if (IDX == 0) {
        if (X[0] > ACC[0])
            ACC[0] = X[0];
    }
    if (IDX == 1) {
        ACCi[0]++;
        if (sPARi[0] > 0 && ACCi[0] >= sPARi[0])
            UDT = 1;
    }
}

template <class Precision>
__forceinline__ __device__ void PerThread_ActionAfterSuccessfulTimeStep(
    int tid, int NT, int& UDT,
    Precision& T, Precision& dT, Precision* TD, Precision* X,
    Precision* cPAR, Precision* sPAR, int* sPARi, Precision* ACC, int* ACCi)
{
    if (X[0] < ACC[1])
        ACC[1] = X[0];
    ACCi[1]++;
}

template <class Precision>
__forceinline__ __device__ void PerThread_Initialization(
    int tid, int NT, int& DOIDX,
    Precision& T, Precision& dT, Precision* TD, Precision* X,
    Precision* cPAR, Precision* sPAR, int* sPARi, Precision* ACC, int* ACCi)
{
    T      = TD[0];
    DOIDX  = 0;
    ACC[0] = X[0];
    ACC[1] = X[0];
}

template <class Precision>
__forceinline__ __device__ void PerThread_Finalization(
    int tid, int NT, int& DOIDX,
    Precision& T, Precision& dT, Precision* TD, Precision* X,
    Precision* cPAR, Precision* sPAR, int* sPARi, Precision* ACC, int* ACCi)
{
}

#endif

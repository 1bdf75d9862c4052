// Ring of coupled forced Duffing oscillators, one system = UPS units:
//   x_i' = v_i,  v_i' = -k v_i - x_i - x_i^3 + B cos(T) + sum_j C_ij x_j
// (the sum is added by the solver: coupling term CPT[0] = x_i with factor
// CPF[0] = 1 into component 1 through CouplingIndex = 1, strength 1).
//
// Hook file in the reference's coupled-system convention
// (Tutorials_CoupledSystems_PerBlock/T1_RingOfDuffingOscillators/RingOfDuffingOscillators_SystemDefinition.cuh:8-104).
//   UD = 2, NC = 1, NUP = 0, NSP = 1 (B), NGP = 1 (k), NiGP = 0,
//   NUA = 0, NiUA = 1 (zero crossings of x_i, counted by the unit event),
//   NSA = 0, NiSA = 1 (accepted steps of the system, counted by unit 0),
//   NE = 1: EF[0] = x_i, any direction.
// Initialization resets T to TD0 (unit 0), so one launch is one interval.
// The coupling storage (full, banded, circular) is chosen by the plugin
// translation unit through MPGOS_SYS_CBW / MPGOS_SYS_CCI.
#ifndef MPGOS_SYSTEM_RING_DUFFING_CUH
#define MPGOS_SYSTEM_RING_DUFFING_CUH

#ifndef MPGOS_SYS_UPS
#define MPGOS_SYS_UPS  64
#endif
#define MPGOS_SYS_UD   2
#define MPGOS_SYS_NC   1
#define MPGOS_SYS_NUP  0
#define MPGOS_SYS_NSP  1
#define MPGOS_SYS_NGP  1
#define MPGOS_SYS_NIGP 0
#define MPGOS_SYS_NUA  0
#define MPGOS_SYS_NIUA 1
#define MPGOS_SYS_NSA  0
#define MPGOS_SYS_NISA 1
#define MPGOS_SYS_NE   1

template <class Precision>
__forceinline__ __device__ void CoupledSystems_PerBlock_OdeFunction(
    int sid, int uid,
    Precision* F, Precision* X, Precision T,
    Precision* uPAR, Precision* sPAR, Precision* gPAR, int* igPAR,
    Precision* uACC, int* iuACC, Precision* sACC, int* isACC,
    Precision* CPT, Precision* CPF)
{
    F[0] = X[1];
    F[1] = -gPAR[0] * X[1] - X[0] - X[0] * X[0] * X[0] + sPAR[0] * cos(T);
    CPT[0] = X[0];
    CPF[0] = static_cast<Precision>(1.0);
}

template <class Precision>
__forceinline__ __device__ void CoupledSystems_PerBlock_EventFunction(
    int sid, int uid, Precision* EF,
    Precision T, Precision dT, Precision* TD, Precision* X,
    Precision* uPAR, Precision* sPAR, Precision* gPAR, int* igPAR,
    Precision* uACC, int* iuACC, Precision* sACC, int* isACC)
{
    EF[0] = X[0];
}

template <class Precision>
__forceinline__ __device__ void CoupledSystems_PerBlock_ActionAfterEventDetection(
    int sid, int uid, int IDX, int& UDT,
    Precision& T, Precision& dT, Precision* TD, Precision* X,
    Precision* uPAR, Precision* sPAR, Precision* gPAR, int* igPAR,
    Precision* uACC, int* iuACC, Precision* sACC, int* isACC)
{
    iuACC[0]++;
}

template <class Precision>
__forceinline__ __device__ void CoupledSystems_PerBlock_ActionAfterSuccessfulTimeStep(
    int sid, int uid, int& UDT,
    Precision& T, Precision& dT, Precision* TD, Precision* X,
    Precision* uPAR, Precision* sPAR, Precision* gPAR, int* igPAR,
    Precision* uACC, int* iuACC, Precision* sACC, int* isACC)
{
    if (uid == 0)
        isACC[0]++;
}

template <class Precision>
__forceinline__ __device__ void CoupledSystems_PerBlock_Initialization(
    int sid, int uid, int& DOIDX,
    Precision& T, Precision& dT, Precision* TD, Precision* X,
    Precision* uPAR, Precision* sPAR, Precision* gPAR, int* igPAR,
    Precision* uACC, int* iuACC, Precision* sACC, int* isACC)
{
    if (uid == 0)
        T = TD[0];
}

template <class Precision>
__forceinline__ __device__ void CoupledSystems_PerBlock_Finalization(
    int sid, int uid, int& DOIDX,
    Precision& T, Precision& dT, Precision* TD, Precision* X,
    Precision* uPAR, Precision* sPAR, Precision* gPAR, int* igPAR,
    Precision* uACC, int* iuACC, Precision* sACC, int* isACC)
{
}

#endif

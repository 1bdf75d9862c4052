// Forward-sensitivity system of duffing_param.cuh: the Duffing oscillator
// x0' = x1, x1' = -k x1 - x0 - x0^3 + B cos(T) augmented with the sensitivity
// matrix S = d(x0, x1) / d(x0(0), x1(0), k, B), S' = J_x S + J_p, integrated by
// the solver as one 10-dimensional system. It is the independent check of the
// discrete adjoint: the gradient of a terminal loss L is S(T)^T dL/dx(T).
//
// Hook file in the reference's user-hook convention
// (Tutorials_SingleSystem_PerThread/T1_Reference/Reference_SystemDefinition.cuh:6-76).
//   X[0], X[1]          state
//   X[2 + 2 j + r]      dX[r] / dtheta_j, theta = (x0(0), x1(0), k, B)
//   cPAR = (k, B); S(0) is the identity block for the initial states, set by
//   the caller; NIA = 1 accepted-step counter.
#ifndef MPGOS_SYSTEM_DUFFING_PARAM_SENS_CUH
#define MPGOS_SYSTEM_DUFFING_PARAM_SENS_CUH

#define MPGOS_SYS_NAME "duffing_param_sens"
#define MPGOS_SYS_SD   10
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
    const Precision k = cPAR[0], B = cPAR[1];
    const Precision c = cos(T);
    F[0] = X[1];
    F[1] = -k * X[1] - X[0] - X[0] * X[0] * X[0] + B * c;
    // J_x = [[0, 1], [-1 - 3 x0^2, -k]]
    const Precision j10 = -static_cast<Precision>(1.0) - static_cast<Precision>(3.0) * X[0] * X[0];
    for (int j = 0; j < 4; j++) {
        const Precision s0 = X[2 + 2 * j], s1 = X[3 + 2 * j];
        F[2 + 2 * j] = s1;
        F[3 + 2 * j] = j10 * s0 - k * s1;
    }
    // J_p: d F[1] / dk = -x1, d F[1] / dB = cos(T)
    F[3 + 2 * 2] += -X[1];
    F[3 + 2 * 3] += c;
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

// Cash-Karp 4(5) coefficients (SingleSystem_PerThread_ExplicitRungeKutta_Steppers.cuh:121-289)
// as double-float pairs in constant memory, for steppers that run the six
// stages as one loop with a warp-uniform stage index: hi = the float nearest
// the coefficient, lo = the float nearest the rest (the values dfloat(double)
// gives). A[i][j] the weight of k_j in the input of stage i, B the 5th-order
// weights, E the error weights b - b*, C the stage times.
#pragma once

#include <cuda_runtime.h>

namespace mpgos {

constexpr float ck_hi(double d) { return static_cast<float>(d); }
constexpr float ck_lo(double d) { return static_cast<float>(d - static_cast<double>(static_cast<float>(d))); }

#define MPGOS_CK(d) {ck_hi(d), ck_lo(d)}
static __constant__ float2 CK_A[6][5] = {
    {MPGOS_CK(0.0), MPGOS_CK(0.0), MPGOS_CK(0.0), MPGOS_CK(0.0), MPGOS_CK(0.0)},
    {MPGOS_CK(1.0 / 5.0), MPGOS_CK(0.0), MPGOS_CK(0.0), MPGOS_CK(0.0), MPGOS_CK(0.0)},
    {MPGOS_CK(3.0 / 40.0), MPGOS_CK(9.0 / 40.0), MPGOS_CK(0.0), MPGOS_CK(0.0), MPGOS_CK(0.0)},
    {MPGOS_CK(3.0 / 10.0), MPGOS_CK(-9.0 / 10.0), MPGOS_CK(6.0 / 5.0), MPGOS_CK(0.0), MPGOS_CK(0.0)},
    {MPGOS_CK(-11.0 / 54.0), MPGOS_CK(5.0 / 2.0), MPGOS_CK(-70.0 / 27.0), MPGOS_CK(35.0 / 27.0), MPGOS_CK(0.0)},
    {MPGOS_CK(1631.0 / 55296.0), MPGOS_CK(175.0 / 512.0), MPGOS_CK(575.0 / 13824.0), MPGOS_CK(44275.0 / 110592.0),
     MPGOS_CK(253.0 / 4096.0)}};
static __constant__ float2 CK_B[6] = {MPGOS_CK(37.0 / 378.0), MPGOS_CK(0.0), MPGOS_CK(250.0 / 621.0),
                                      MPGOS_CK(125.0 / 594.0), MPGOS_CK(0.0), MPGOS_CK(512.0 / 1771.0)};
static __constant__ float2 CK_E[6] = {MPGOS_CK(37.0 / 378.0 - 2825.0 / 27648.0), MPGOS_CK(0.0),
                                      MPGOS_CK(250.0 / 621.0 - 18575.0 / 48384.0),
                                      MPGOS_CK(125.0 / 594.0 - 13525.0 / 55296.0), MPGOS_CK(0.0 - 277.0 / 14336.0),
                                      MPGOS_CK(512.0 / 1771.0 - 1.0 / 4.0)};
static __constant__ float2 CK_C[6] = {MPGOS_CK(0.0), MPGOS_CK(1.0 / 5.0), MPGOS_CK(3.0 / 10.0),
                                      MPGOS_CK(3.0 / 5.0), MPGOS_CK(1.0), MPGOS_CK(7.0 / 8.0)};
#undef MPGOS_CK

}  // namespace mpgos

// sm_103a build of the reference's own coupled per-block solver kernels, one
// template instantiation per cubin. The variant is the one the reference's
// Solve() launches for the (SPB, UPS, TPB) of the cubin
// (CoupledSystems_PerBlock_Interface.cuh:1953-1965): MultipleBlockLaunches
// when SPB*UPS > TPB, SingleBlockLaunch otherwise; MultipleSystems when
// SPB > 1, SingleSystem when SPB == 1.
//
// TEST INFRASTRUCTURE ONLY. oracle/build_oracle.py compiles this file with
// nvcc -cubin against the reference's unmodified
// SourceCodes/CoupledSystmes_PerBlock_Solver.cuh (and the stepper, controller,
// event and dense-output headers it includes) where it lies in the reference
// checkout, into
// oracle/_ref/ref_gpu_cb_<system>_<alg>_ns<NS>_tpb<TPB>_spb<SPB>_ndo<NDO>.cubin
// (git-ignored; device code only). oracle/ref_gpu.py loads it with the CUDA
// driver API and launches it on the device buffers of a GB300 coupled solver
// object, to check the GB300 coupled kernel against the reference kernel bit
// for bit and to time the reference kernel on the same GPU.
//
// Compile: -DMPGOS_SYSTEM_HEADER="<hooks>.cuh" -DMPGOS_SYS_UPS=<UPS>
//          -DMPGOS_SYS_CBW=<CBW> -DMPGOS_SYS_CCI=<CCI> -DREF_NS=<NS>
//          -DREF_TPB=<TPB> -DREF_SPB=<SPB> -DREF_NDO=<NDO>
//          -DREF_ALG=<RK4|RKCK45> -I<reference>/SourceCodes
#include <cstdio>

#include "ref_types_coupled.hpp"

#include MPGOS_SYSTEM_HEADER

#include "CoupledSystmes_PerBlock_Solver.cuh"

#if (REF_SPB > 1) && (REF_SPB * MPGOS_SYS_UPS > REF_TPB)
#define REF_CB_KERNEL CoupledSystems_PerBlock_MultipleSystems_MultipleBlockLaunches
#elif (REF_SPB == 1) && (MPGOS_SYS_UPS > REF_TPB)
#define REF_CB_KERNEL CoupledSystems_PerBlock_SingleSystem_MultipleBlockLaunches
#elif (REF_SPB > 1)
#define REF_CB_KERNEL CoupledSystems_PerBlock_MultipleSystems_SingleBlockLaunch
#else
#define REF_CB_KERNEL CoupledSystems_PerBlock_SingleSystem_SingleBlockLaunch
#endif

template __global__ void REF_CB_KERNEL<
    REF_NS, MPGOS_SYS_UPS, MPGOS_SYS_UD, REF_TPB, REF_SPB, MPGOS_SYS_NC, MPGOS_SYS_CBW, MPGOS_SYS_CCI, MPGOS_SYS_NUP,
    MPGOS_SYS_NSP, MPGOS_SYS_NGP, MPGOS_SYS_NIGP, MPGOS_SYS_NUA, MPGOS_SYS_NIUA, MPGOS_SYS_NSA, MPGOS_SYS_NISA,
    MPGOS_SYS_NE, REF_NDO, REF_ALG, double>(Struct_ThreadConfiguration, Struct_GlobalVariables<double>,
                                            Struct_SharedMemoryUsage, Struct_SolverOptions<double>);
